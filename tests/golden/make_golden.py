"""Generate the committed golden fixtures under tests/golden/.

Run in the container that has the reference mounted:
    python tests/golden/make_golden.py <reference-root>

Fixtures written (all small):
  test100.f64, test128.f64  -- the reference's shipped sample inputs
                               (test100.txt / test128.txt, 18 columns) as raw
                               little-endian float64, row-major
  join_golden.json          -- known-answer counts for those files at the
                               eps values of the reference's run log, plus
                               per-point counts; computed here with numpy in
                               FP64 (sqrt(sum((a-b)^2)) <= eps) -- independent
                               of the oracle's C code
  ties.f64 / ties.json      -- adversarial boundary cases (integer grid scaled
                               by a power of two, so many d2 equal eps^2
                               exactly) with counts from a pure-Python exact
                               restatement (rational fma)
  loader_*.txt / loader_golden.json
                            -- text inputs in several layouts and the rows the
                               reference's own importDataset (dataset.cu:10-39,
                               built by oracle/build_ref.sh, dim 90) produced
"""
import json
import os
import subprocess
import tempfile
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def numpy_counts(x, eps):
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    return (np.sqrt(d2) <= eps).sum(1).astype(np.int64)


def main(ref):
    import oracle

    out = {"source": "reference sample inputs test100.txt / test128.txt", "files": {}}
    for name in ("test100", "test128"):
        x = np.loadtxt(os.path.join(ref, name + ".txt"), delimiter=",", usecols=range(18))
        x = np.ascontiguousarray(x, dtype="<f8")
        x.tofile(os.path.join(HERE, name + ".f64"))
        entry = {"n": int(x.shape[0]), "d": int(x.shape[1]), "cases": []}
        for eps in (0.001, 0.01, 0.05, 0.1, 0.2):
            c = numpy_counts(x, eps)
            entry["cases"].append({"eps": eps, "total": int(c.sum()), "counts": c.tolist()})
        out["files"][name] = entry
    with open(os.path.join(HERE, "join_golden.json"), "w") as f:
        json.dump(out, f)

    # adversarial ties: 3-D integer grid 0..4 scaled by 2^-3, plus duplicates
    g = np.stack(np.meshgrid(*[np.arange(5)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x = np.concatenate([g, g[:7]], 0).astype("<f8") * 0.125
    x = np.ascontiguousarray(x)
    x.tofile(os.path.join(HERE, "ties.f64"))
    cases = []
    for eps in (0.0, 0.125, 0.125 * np.sqrt(2.0), 0.25, 0.125 * 3, 0.5):
        c, tot = oracle.py_self_join(x, float(eps))
        cases.append({"eps": float(eps), "total": tot, "counts": c.tolist()})
    with open(os.path.join(HERE, "ties.json"), "w") as f:
        json.dump({"n": int(x.shape[0]), "d": 3, "cases": cases}, f)

    # loader fixtures checked against the reference's own importDataset
    if not oracle.reference_loader_available():
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref])
    rng = np.random.default_rng(7)
    vals = rng.standard_normal((5, 90)) * np.array([1e-3, 1.0, 1e3, 1e-300, 7.5])[:, None]
    layouts = {
        "loader_comma.txt": "\n".join(", ".join(f"{v:.17g}" for v in r) for r in vals) + "\n",
        "loader_space.txt": "\n".join(" ".join(f"{v:.6e}" for v in r) for r in vals),
        "loader_mixed.txt": "\n".join(",".join(f"{v:.9f}" for v in r) + " " for r in vals) + "\n",
        # 3 full rows and a trailing partial row of 40 values (dropped)
        "loader_partial.txt": ", ".join(f"{v:.17g}" for v in vals.ravel()[: 90 * 3 + 40]),
        "loader_oneline.txt": " ".join(f"{v:.17g}" for v in vals.ravel()[:180]) + " ",
    }
    golden = {"dim": 90, "files": {}}
    with tempfile.TemporaryDirectory(dir=HERE) as tmp:
        for fname, text in layouts.items():
            p = os.path.join(HERE, fname)
            with open(p, "w") as f:
                f.write(text)
            rows = oracle.reference_import_dataset(p, os.path.join(tmp, fname + ".bin"))
            golden["files"][fname] = {"rows": int(rows.shape[0]),
                                      "values": [float(v) for v in rows.ravel()]}
    with open(os.path.join(HERE, "loader_golden.json"), "w") as f:
        json.dump(golden, f)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference-root>")
    main(sys.argv[1])
