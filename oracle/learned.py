"""CPU restatement of the learned projection's training arithmetic --
TEST INFRASTRUCTURE ONLY (the oracle of the GPU training kernels).

The learned pruning has no reference counterpart; this file restates, in
FP64 numpy, the loss and gradient the training kernel (k_learn.cu,
train_step_kernel) computes:

    y_p = P v_p,  r_p = |y_p|,  active_p = (t_p > 0) and (r_p < t_p)
    L   = (1/M) sum_active (1 - r_p / t_p)
    dL/dP = -(1/M) sum_active (1 / (t_p r_p)) y_p v_p^T
"""
import numpy as np


def loss_and_grad(V, tgt, P):
    V = np.asarray(V, dtype=np.float64)
    t = np.asarray(tgt, dtype=np.float64)
    P = np.asarray(P, dtype=np.float64)
    M = V.shape[0]
    Y = V @ P.T
    r = np.sqrt((Y * Y).sum(1))
    act = (t > 0) & (r < t)
    loss = float(np.sum(1.0 - r[act] / t[act]) / M)
    coef = np.zeros(M)
    nz = act & (r > 0)
    coef[nz] = -1.0 / (M * t[nz] * r[nz])
    G = (coef[:, None] * Y).T @ V
    return loss, G


def loss_only(V, tgt, P):
    return loss_and_grad(V, tgt, P)[0]


def spectral_norm(P):
    return float(np.linalg.svd(np.asarray(P, dtype=np.float64), compute_uv=False)[0])
