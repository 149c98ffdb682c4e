"""CPU: the C ABI library loads, exports every declared symbol, and its
host-only parts (threshold, loaders, spectral certificate) are right."""
import json
import math
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def declared_symbols():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        text = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:int|double|void)\s+(ejoin_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol(ej):
    import ctypes
    lib = ctypes.CDLL(ej.LIB_PATH)
    decl = declared_symbols()
    assert decl == set(ej.EXPORTED) | set(ej.TESTING)
    for name in decl:
        assert hasattr(lib, name), name


def test_threshold_matches_oracle(ej, oracle_mod):
    rng = np.random.default_rng(1)
    for eps in list(rng.random(100)) + [0.0, -0.5, 1e-200, 3e200, float("inf")]:
        assert ej.threshold(eps) == oracle_mod.threshold(eps)
    assert math.isnan(ej.threshold(float("nan")))


@pytest.mark.parametrize("fname", ["loader_comma.txt", "loader_space.txt", "loader_mixed.txt",
                                   "loader_partial.txt", "loader_oneline.txt"])
def test_loader_matches_reference_loader(ej, oracle_mod, fname):
    """Golden rows were produced by the reference's own importDataset."""
    g = json.load(open(os.path.join(GOLDEN, "loader_golden.json")))
    exp = np.array(g["files"][fname]["values"]).reshape(-1, g["dim"])
    path = os.path.join(GOLDEN, fname)
    got = ej.importDataset(path, g["dim"])
    assert got.shape == exp.shape
    assert np.array_equal(got, exp)
    assert np.array_equal(oracle_mod.import_dataset(path, g["dim"]), exp)


def test_loader_sample_files_and_runtime_dim(ej, tmp_path):
    x = np.fromfile(os.path.join(GOLDEN, "test128.f64"), dtype="<f8").reshape(-1, 18)
    p = tmp_path / "t.txt"
    with open(p, "w") as f:
        for r in x:
            f.write(", ".join(f"{v:.17g}" for v in r) + " \n")
    assert np.array_equal(ej.importDataset(str(p), 18), x)
    y = ej.importDataset(str(p), 7)  # run-time dim: rows of 7, trailing partial row dropped
    assert y.shape == (128 * 18 // 7, 7)
    assert np.array_equal(y.ravel(), x.ravel()[: y.size])
    b = tmp_path / "t.f64"
    x.tofile(b)
    assert np.array_equal(ej.import_binary(str(b), 18), x)


def test_loader_missing_file(ej):
    with pytest.raises(ej.EjoinError) as e:
        ej.importDataset("/nonexistent/file.txt", 3)
    assert e.value.status == -7


def test_spectral_certificate_is_an_upper_bound(ej):
    rng = np.random.default_rng(2)
    for k, d in ((1, 5), (8, 64), (16, 1024), (4, 3)):
        P = rng.standard_normal((k, d)).astype(np.float32)
        s = np.linalg.svd(P.astype(np.float64), compute_uv=False)[0]
        b = ej.certify_spectral_norm(P)
        assert b >= s
        assert b <= s * (1 + 2e-3)
    assert ej.certify_spectral_norm(np.zeros((3, 4), np.float32)) == 0.0


def test_no_gpu_raises_instead_of_falling_back(ej):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(ej.EjoinError) as e:
        ej.self_join(np.zeros((4, 3)), 0.1)
    assert e.value.status == -4


def test_projection_file_round_trip(ej, tmp_path):
    rng = np.random.default_rng(5)
    P = rng.standard_normal((8, 64)).astype(np.float32)
    path = str(tmp_path / "p.ejp")
    ej.save_projection(path, P, 0.987654321)
    Q, sig = ej.load_projection(path)
    assert Q.dtype == np.float32 and Q.shape == (8, 64)
    assert np.array_equal(Q.view(np.uint32), P.view(np.uint32))
    assert sig == 0.987654321
    assert os.path.getsize(path) == 40 + 4 * 8 * 64


def test_projection_file_rejects_damage(ej, tmp_path):
    P = np.ones((2, 3), dtype=np.float32)
    path = tmp_path / "p.ejp"
    ej.save_projection(str(path), P, 1.0)
    raw = bytearray(path.read_bytes())
    for pos in (0, 9, 13, 30, len(raw) - 20):
        bad = bytearray(raw)
        bad[pos] ^= 0x40
        path.write_bytes(bytes(bad))
        with pytest.raises(ej.EjoinError) as e:
            ej.load_projection(str(path))
        assert e.value.status == -7
    path.write_bytes(bytes(raw[:-1]))
    with pytest.raises(ej.EjoinError):
        ej.load_projection(str(path))
    with pytest.raises(ej.EjoinError) as e:
        ej.load_projection(str(tmp_path / "missing.ejp"))
    assert e.value.status == -7
    with pytest.raises(ej.EjoinError) as e:
        ej.save_projection(str(tmp_path / "k17.ejp"), np.ones((17, 3), np.float32), 1.0)
    assert e.value.status == -1


def test_binary_loader_reads_in_pieces(ej, tmp_path):
    rng = np.random.default_rng(6)
    x = rng.standard_normal((3001, 7))
    path = tmp_path / "x.f64"
    x.astype("<f8").tofile(path)
    assert np.array_equal(ej.import_binary(str(path), 7), x)
    # a trailing partial row is dropped
    with open(path, "ab") as f:
        f.write(b"\0" * 16)
    assert np.array_equal(ej.import_binary(str(path), 7), x)
