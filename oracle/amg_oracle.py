"""CPU restatement of the smoothed-aggregation multigrid preconditioner -- TEST INFRASTRUCTURE ONLY.

The reference has no multigrid: it factorises K with Pardiso (SOLVE_static.py:31-33).  The
product's preconditioner (fem_amg_setup / fem_amg_vcycle) follows the published method of
Vanek, Mandel and Brezina (Computing 56, 1996); this module restates the same steps in
numpy/scipy so the tests can check the library's hierarchy and V-cycle:

* strength on the block-scaled matrix: with D_i = L_i L_i^T, block (i, j), j != i, is strong
  when |L_i^-1 A_ij L_j^-T|_F^2 > theta^2 b; unaggregated rows whose scaled couplings are all
  below 1e-6 (|.|_F^2 / b < 1e-12) are Dirichlet rows;
* aggregation in node order: (a) free node + all-free strong neighbours; (b) join the
  step-(a) aggregate of the most strongly coupled aggregated neighbour; (c) the rest with
  their free strong neighbours; rows without strong neighbours stay unaggregated;
* tentative prolongator: two-pass modified Gram-Schmidt of each aggregate's near-null-space
  rows (rigid-body modes on level 0, coordinates taken about the mesh centroid), columns
  whose remaining norm is <= 1e-10 of their original norm dropped;
* P = T - omega D^-1 A T (zero rows for Dirichlet nodes) with
  omega = 4 / (3 lambda_max), lambda_max from Lanczos on D^-1 A in the D inner product from
  the same splitmix64 start vector;
* A_c = P^T A P, zero coarse diagonals set to 1, dense inverse on the last level;
* V-cycle: Chebyshev pre-smoothing from 0, residual, restriction, coarse cycle,
  prolongation, Chebyshev post-smoothing restarted from the current iterate; Dirichlet
  nodes hold x = D^-1 b throughout and contribute a zero residual.

Only ``tests/`` import this module; the product package never does.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

KMODES = 6


def _blocks(A: sp.bsr_matrix):
    A = sp.bsr_matrix(A)
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int64), A.data


def rigid_modes(xyz):
    """[n][3][6] translations and rotations e_d x (x - centroid)."""
    x = np.asarray(xyz, dtype=np.float64)
    c = x.mean(axis=0)
    d = x - c
    n = x.shape[0]
    B = np.zeros((n, 3, KMODES))
    B[:, 0, 0] = B[:, 1, 1] = B[:, 2, 2] = 1.0
    B[:, 1, 3], B[:, 2, 3] = -d[:, 2], d[:, 1]
    B[:, 0, 4], B[:, 2, 4] = d[:, 2], -d[:, 0]
    B[:, 0, 5], B[:, 1, 5] = -d[:, 1], d[:, 0]
    return B


def inv_cholesky(A: sp.bsr_matrix):
    """[n][b][b] inverses of the Cholesky factors of the diagonal blocks (diagonal scaling
    1 / sqrt|d_pp| where a block is not numerically SPD)."""
    ptr, col, val = _blocks(A)
    n = len(ptr) - 1
    b = val.shape[1]
    G = np.zeros((n, b, b))
    for i in range(n):
        l = ptr[i] + np.searchsorted(col[ptr[i]:ptr[i + 1]], i)
        D = val[l]
        try:
            Lm = np.linalg.cholesky(D)
            G[i] = np.linalg.inv(Lm)
        except np.linalg.LinAlgError:
            d = np.abs(np.diag(D))
            G[i] = np.diag(np.where(d > 0, 1.0 / np.sqrt(np.where(d > 0, d, 1.0)), 1.0))
    return G


def strength(A: sp.bsr_matrix, theta):
    """(ptr, col, scaled squared couplings per block, strong flags, per-row max coupling / b)."""
    ptr, col, val = _blocks(A)
    n = len(ptr) - 1
    b = val.shape[1]
    row = np.repeat(np.arange(n), np.diff(ptr))
    G = inv_cholesky(A)
    S = np.einsum("lrk,lkc,ldc->lrd", G[row], val, G[col])
    f2 = (S ** 2).sum(axis=(1, 2))
    off = row != col
    strong = off & (f2 > theta * theta * b)
    maxc = np.zeros(n)
    np.maximum.at(maxc, row[off], f2[off] / b)
    return ptr, col, f2, strong, maxc


def aggregate(A: sp.bsr_matrix, theta):
    ptr, col, f2, strong, maxc = strength(A, theta)
    n = len(ptr) - 1
    FREE, ALONE = -1, -2
    agg = np.full(n, FREE, dtype=np.int64)
    for i in range(n):
        if not strong[ptr[i]:ptr[i + 1]].any():
            agg[i] = ALONE
    na = 0
    for i in range(n):
        if agg[i] != FREE:
            continue
        nb = col[ptr[i]:ptr[i + 1]][strong[ptr[i]:ptr[i + 1]]]
        if np.all(agg[nb] == FREE):
            agg[i] = na
            agg[nb] = na
            na += 1
    first = agg.copy()
    for i in range(n):
        if agg[i] != FREE:
            continue
        best, bs = -1, -1.0
        for l in range(ptr[i], ptr[i + 1]):
            if strong[l] and first[col[l]] >= 0 and f2[l] > bs:
                bs, best = f2[l], first[col[l]]
        if best >= 0:
            agg[i] = best
    for i in range(n):
        if agg[i] != FREE:
            continue
        agg[i] = na
        for l in range(ptr[i], ptr[i + 1]):
            if strong[l] and agg[col[l]] == FREE:
                agg[col[l]] = na
        na += 1
    agg[agg == ALONE] = -1
    dirichlet = (agg < 0) & (maxc < 1e-12)
    return agg, na, dirichlet


def tentative(agg, na, B):
    """T (n*b x na*6 sparse) and Bc [na][6][6] from the near-null space B [n][b][6]."""
    n, b, k = B.shape
    rows, cols, vals = [], [], []
    Bc = np.zeros((na, k, k))
    for a in range(na):
        mem = np.flatnonzero(agg == a)
        Q = B[mem].reshape(-1, k).copy()
        Rr = np.zeros((k, k))
        for c in range(k):
            n0 = np.linalg.norm(Q[:, c])
            for _ in range(2):
                for c2 in range(c):
                    d = Q[:, c2] @ Q[:, c]
                    Q[:, c] -= d * Q[:, c2]
                    Rr[c2, c] += d
            nr = np.linalg.norm(Q[:, c])
            if nr > 1e-10 * n0 and nr > 0:
                Q[:, c] /= nr
                Rr[c, c] = nr
            else:
                Q[:, c] = 0.0
                Rr[c, c] = 0.0
        for s_, i in enumerate(mem):
            for cc in range(b):
                for m in range(k):
                    rows.append(i * b + cc)
                    cols.append(a * k + m)
                    vals.append(Q[s_ * b + cc, m])
        Bc[a] = Rr
    T = sp.csr_matrix((vals, (rows, cols)), shape=(n * b, na * k))
    return T, Bc


def block_diag_inverse(A: sp.bsr_matrix, b):
    A = sp.csr_matrix(A)
    n = A.shape[0] // b
    D = np.zeros((n, b, b))
    for p in range(b):
        for q in range(b):
            D[:, p, q] = A[np.arange(n) * b + p, np.arange(n) * b + q].A1
    return D, np.linalg.inv(D)


def _splitmix_start(N):
    i = np.arange(N, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = i + np.uint64(0x9e3779b97f4a7c15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xbf58476d1ce4e5b9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94d049bb133111eb)
        z ^= z >> np.uint64(31)
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def lanczos_lmax(A, D, Dinv, steps):
    """Largest Ritz value of D^-1 A after `steps` Lanczos steps (D inner product)."""
    A = sp.csr_matrix(A)
    n, b, _ = D.shape
    bd = lambda M, x: np.einsum("nij,nj->ni", M, x.reshape(n, b)).reshape(-1)  # noqa: E731
    v = _splitmix_start(n * b)
    v /= np.sqrt(v @ bd(D, v))
    vp = np.zeros_like(v)
    alpha, beta = [], [0.0]
    for j in range(steps):
        u = A @ v
        a = v @ u
        alpha.append(a)
        w = bd(Dinv, u) - a * v - beta[-1] * vp
        bn = np.sqrt(max(0.0, w @ bd(D, w)))
        if not bn > 1e-12 * abs(a) or j + 1 == steps:
            break
        beta.append(bn)
        vp, v = v, w / bn
    m = len(alpha)
    Tm = np.diag(alpha) + np.diag(beta[1:m], 1) + np.diag(beta[1:m], -1)
    return float(np.linalg.eigvalsh(Tm).max())


def chebyshev_coeffs(lmax, degree, upper=1.1, ratio=30.0):
    up = upper * lmax
    lo = up / ratio
    theta, delta = 0.5 * (up + lo), 0.5 * (up - lo)
    sigma = theta / delta
    c1, c2 = [0.0], [1.0 / theta]
    rho = 1.0 / sigma
    for _ in range(1, degree):
        rn = 1.0 / (2 * sigma - rho)
        c1.append(rn * rho)
        c2.append(2 * rn / delta)
        rho = rn
    return c1, c2


def setup(K, xyz, theta=0.08, max_levels=10, max_coarse=512, eig_steps=12, lmax_given=None):
    """Hierarchy as a list of dicts (A, Dinv, P, agg, lmax, omega) + the dense coarse inverse.
    lmax_given: optional per-level lambda_max values to use instead of the oracle's own
    Lanczos estimates (so a comparison isolates the rest of the setup)."""
    A = sp.bsr_matrix(sp.csr_matrix(K), blocksize=(3, 3))
    B = rigid_modes(xyz)
    levels = []
    b = 3
    for l in range(max_levels):
        n = A.shape[0] // b
        D, Dinv = block_diag_inverse(A, b)
        m = n * b
        lv = {"A": sp.csr_matrix(A), "Dinv": Dinv, "b": b, "n": n}
        levels.append(lv)
        if m <= max_coarse or l + 1 >= max_levels:
            break
        agg, na, dirichlet = aggregate(A, theta)
        if na == 0 or na * KMODES >= m:
            break
        lm = lanczos_lmax(A, D, Dinv, eig_steps)
        lv["lmax_oracle"] = lm
        if lmax_given is not None:
            lm = lmax_given[l]
        omega = 4.0 / (3.0 * lm)
        T, Bc = tentative(agg, na, B)
        Dm = sp.block_diag([sp.csr_matrix(Dinv[i]) for i in range(n)], format="csr")
        P = (T - omega * (Dm @ (sp.csr_matrix(A) @ T))).tocsr()
        keep = np.repeat(~dirichlet, b).astype(np.float64)
        P = (sp.diags(keep) @ P).tocsr()
        P.eliminate_zeros()
        Ac = (P.T @ sp.csr_matrix(A) @ P).tocsr()
        Ac = Ac.tolil()
        for d in range(Ac.shape[0]):
            if Ac[d, d] == 0.0:
                Ac[d, d] = 1.0
        lv.update(agg=agg, na=na, lmax=lm, omega=omega, P=P, dirichlet=dirichlet)
        A = sp.bsr_matrix(Ac.tocsr(), blocksize=(KMODES, KMODES))
        B = Bc
        b = KMODES
    coarse = np.linalg.inv(levels[-1]["A"].toarray())
    return levels, coarse


def vcycle(levels, coarse_inv, r, pre=2, post=2, upper=1.1, ratio=30.0, l=0, dirichlet_fix=False):
    """FP64 V-cycle z = M^-1 r on the hierarchy (levels[l] needs A, Dinv, b, and for non-last
    levels P and lmax).  dirichlet_fix: after the level-0 cycle, one block-Jacobi update on the
    Dirichlet rows, x_I += D_I^-1 (r - A x)_I (the symmetric I, F, I order)."""
    if l == len(levels) - 1:
        return coarse_inv @ r
    L = levels[l]
    A, b, n = L["A"], L["b"], L["n"]
    Dinv = L["Dinv"]
    free = np.repeat(~L["dirichlet"], b)
    c1, c2 = chebyshev_coeffs(L["lmax"], max(pre, post), upper, ratio)
    apply_dinv = lambda v: np.einsum("nij,nj->ni", Dinv, v.reshape(n, b)).reshape(-1)  # noqa: E731
    x = np.where(free, c2[0], 1.0) * apply_dinv(r)
    d = x.copy()
    for k in range(1, pre):
        d = c1[k] * d + c2[k] * apply_dinv(r - A @ x)
        x = np.where(free, x + d, x)
    res = np.where(free, r - A @ x, 0.0)
    xc = vcycle(levels, coarse_inv, L["P"].T @ res, pre, post, upper, ratio, l + 1)
    x = x + L["P"] @ xc
    for k in range(post):
        z = apply_dinv(r - A @ x)
        d = c2[k] * z if k == 0 else c1[k] * d + c2[k] * z
        x = np.where(free, x + d, x)
    if dirichlet_fix and l == 0:
        x = np.where(free, x, x + apply_dinv(r - A @ x))
    return x
