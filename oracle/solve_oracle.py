"""CPU baselines of the static solve -- TEST / BASELINE INFRASTRUCTURE ONLY.

The reference solves K U = F with MKL Pardiso (SOLVE_static.py:31-33), which is not available
here.  Two CPU stand-ins are timed beside the GPU solver by bench.py's CPU-baseline leg:

* ``direct``: scipy's SuperLU factorisation + solve (the direct-solver role Pardiso plays);
* ``bj_pcg``: plain FP64 block-Jacobi preconditioned conjugate gradients with scipy sparse
  products, the CPU form of the GPU's FP64 comparison solver (same preconditioner, same
  stopping rule ||F - K u|| / ||F|| on the recursively updated residual).

Nothing in the product package imports this module.
"""
from __future__ import annotations

import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def direct(K, F):
    """SuperLU factorisation and solve; returns (U, seconds)."""
    t = time.perf_counter()
    lu = spla.splu(sp.csc_matrix(K))
    U = lu.solve(np.asarray(F, dtype=np.float64))
    return U, time.perf_counter() - t


def block_jacobi(K):
    """(N, 3, 3) inverses of the 3x3 diagonal blocks of the 3N x 3N matrix K."""
    K = sp.csr_matrix(K)
    n = K.shape[0] // 3
    D = np.zeros((n, 3, 3))
    for p in range(3):
        for q in range(3):
            D[:, p, q] = K[np.arange(n) * 3 + p, np.arange(n) * 3 + q].A1
    return np.linalg.inv(D)


def bj_pcg(K, F, rtol=1e-10, maxit=100000):
    """FP64 block-Jacobi PCG; returns (U, iterations, seconds excluding the setup)."""
    K = sp.csr_matrix(K)
    Minv = block_jacobi(K)
    F = np.asarray(F, dtype=np.float64)
    apply_m = lambda r: np.einsum("nij,nj->ni", Minv, r.reshape(-1, 3)).reshape(-1)  # noqa: E731
    t = time.perf_counter()
    x = np.zeros_like(F)
    r = F.copy()
    z = apply_m(r)
    p = z.copy()
    rz = r @ z
    tol2 = (rtol * np.linalg.norm(F)) ** 2
    it = 0
    while it < maxit and r @ r > tol2:
        q = K @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        z = apply_m(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it, time.perf_counter() - t


def newton_large_displacement(OM, F, max_errs=1e-4, max_iters=20):
    """The large-displacement iteration of SOLVE_static.py:41-75 with exact (SuperLU) solves:
    KT, KM at U (OracleModel.Get_MatrixKN), RF = KM U - F, stop at ||RF|| / ||F|| <= max_errs
    or after max_iters steps, else U -= KT^-1 RF.  (SOLVE_static.py:72 solves with F; the
    Newton-Raphson step uses RF.)  Returns (U, relative residuals)."""
    F = np.asarray(F, dtype=np.float64)
    U = np.zeros_like(F)
    res = []
    step = 0
    while True:
        KT, KM = OM.Get_MatrixKN(U.reshape(-1, 3))
        RF = KM @ U - F
        err = np.linalg.norm(RF) / np.linalg.norm(F)
        res.append(err)
        if err <= max_errs or step == max_iters:
            break
        U = U - spla.spsolve(sp.csc_matrix(KT), RF)
        step += 1
    return U, res
