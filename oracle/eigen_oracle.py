"""CPU oracle for the block-Lanczos modal solve -- TEST INFRASTRUCTURE ONLY.

Restates in numpy the reference's shift-invert block Lanczos (SOLVE_eigen.py:45-89,
Eigen_solver.Lanczos_solve) for K x = lambda M x: an M-orthonormal block Krylov basis of
K^-1 M built with two passes of full reorthogonalisation per step, the block-tridiagonal
projection T, its eigen-decomposition, and lambda = 1 / eig(T).  The reference factorises K
with MKL Pardiso (SOLVE_eigen.py:30-32); here the solve is a callable (SuperLU in the tests).
The random start block is an argument so that the oracle and the GPU path start from the same
block (the reference draws it unseeded, SOLVE_eigen.py:51).

Only ``tests/`` use this module; the product package never imports it.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sl


def lanczos(K_solve, M, u0, num_eigen, num_block):
    """SOLVE_eigen.py:45-89.  K_solve(X) returns K^-1 X for an (n, b) block; M is (n, n)
    sparse; u0 the (n, b) start block.  Returns (lambda ascending [:num_eigen], vectors)."""
    m = num_eigen * 2
    b = int(num_block)
    n = M.shape[0]
    Q = np.zeros((n, m))
    T = np.zeros((m, m))
    u = np.array(u0, dtype=np.float64)
    v = sl.cholesky(u.T @ (M @ u))                 # upper, u^T M u = v^T v  (:53)
    u = u @ sl.inv(v)                              # (:54)
    Q[:, :b] = u
    steps = int(m / b)
    for i in range(steps):
        w = K_solve(M @ u)                          # (:61)
        T[i * b:(i + 1) * b, i * b:(i + 1) * b] = u.T @ (M @ w)          # (:62)
        w = w - u @ T[i * b:(i + 1) * b, i * b:(i + 1) * b]              # (:63)
        if i >= steps - 1:
            break
        for _ in range(2):                          # two passes (:68-69)
            w = w - Q[:, :i * b + b] @ (Q[:, :i * b + b].T @ (M @ w))
        t = sl.cholesky(w.T @ (M @ w))              # (:71)
        T[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b] = t
        T[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = t.T
        u = w @ sl.inv(t)                           # (:74)
        Q[:, (i + 1) * b:(i + 2) * b] = u
    ev, vec = sl.eigh(T)                            # (:81)
    lam = 1.0 / ev                                  # (:83)
    X = Q @ vec
    order = np.argsort(lam)
    return lam[order][:num_eigen], X[:, order][:, :num_eigen]


def frequencies(lam):
    """SOLVE_eigen.py:36: f = sqrt(lambda) / (2 pi)."""
    return np.sqrt(lam) / 2 / np.pi
