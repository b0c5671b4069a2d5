"""GPU block-Lanczos modal solve (SOLVE_eigen.py:45-89) against the numpy restatement of the
same algorithm with exact (SuperLU) solves and the same start block, and against scipy's
shift-invert eigsh for the lowest modes.

Tolerances: eigenvalues 1e-8 relative (the K solves run to 1e-11 relative residual);
eigenvectors M-orthonormal to 1e-8 and parallel to the oracle's (|x_gpu^T M x_ref| within
1e-6 of 1) for the modes below the first near-degenerate pair."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import fem_taichi_gb300 as F
from oracle import eigen_oracle as EO
from tests.fixtures import STEEL

pytestmark = pytest.mark.gpu


def _model(nx=8, ny=5, nz=4, seed=3):
    P = F.hex_block(nx, ny, nz, jitter=0.1, seed=seed, fix="zmin")
    return F.Model("e", P, STEEL)


@pytest.mark.parametrize("precond", ["amg", "bj"])
def test_lanczos_matches_oracle_same_start_block(precond):
    M = _model()
    K, Mm = M.Get_MatrixKL().tocsc(), M.Get_MatrixM().tocsr()
    n = K.shape[0]
    ne, nb = 10, 5
    u0 = np.random.default_rng(11).uniform(size=(n, nb))
    lu = spla.splu(K)
    lam_o, X_o = EO.lanczos(lu.solve, Mm, u0, ne, nb)
    solver = F.Eigen_solver(M)
    lam, X = solver.Solve_gpu(num_eigen=ne, num_block=nb, u0=u0, precond=precond)
    lam, X = lam.cpu().numpy(), X.cpu().numpy()
    assert np.all(np.abs(lam - lam_o) <= 1e-8 * np.abs(lam_o))
    G = X.T @ (Mm @ X)
    assert np.allclose(G, np.eye(ne), atol=1e-8)
    gaps = np.diff(lam_o) / lam_o[1:]
    k = int(np.argmax(gaps < 1e-6)) if np.any(gaps < 1e-6) else ne
    c = np.abs(np.sum(X[:, :k] * (Mm @ X_o[:, :k]), axis=0))
    assert np.all(np.abs(c - 1) <= 1e-6), c


def test_lowest_modes_match_shift_invert_eigsh_and_dropin_frequencies():
    M = _model(10, 6, 4, seed=5)
    K, Mm = M.Get_MatrixKL().tocsc(), M.Get_MatrixM().tocsc()
    w = spla.eigsh(K, k=6, M=Mm, sigma=0.0, which="LM", return_eigenvectors=False)
    ref = np.sort(w)
    # 2 * 40 Krylov vectors: the reference algorithm converges the lowest modes to ~1e-12 here
    freq, vec = F.Eigen_solver(M).Solve_cpu(num_eigen=40, num_block=10)
    lam = (2 * np.pi * freq) ** 2
    assert vec.shape == (K.shape[0], 40) and np.all(np.diff(freq) >= 0)
    assert np.all(np.abs(lam[:6] - ref) <= 1e-8 * ref)


def test_fp64_inner_solves_give_the_same_modes():
    M = _model(6, 4, 3, seed=7)
    u0 = np.random.default_rng(2).uniform(size=(3 * M.Num_Node, 4))
    a, _ = F.Eigen_solver(M).Solve_gpu(num_eigen=8, num_block=4, u0=u0, mixed=True)
    b, _ = F.Eigen_solver(M).Solve_gpu(num_eigen=8, num_block=4, u0=u0, mixed=False)
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.all(np.abs(a - b) <= 1e-8 * np.abs(b))


@pytest.mark.parametrize("n,m,b", [(1, 1, 1), (1000, 7, 5), (65_559, 200, 10), (40_000, 300, 13), (3_001, 64, 40),
                                   (129, 256, 32)])
def test_tall_skinny_products_match_numpy(n, m, b):
    """fem_ts_gemm_tn / fem_ts_gemm_nn (through the modal solver's wrapper) against numpy FP64
    on strided column blocks, with the 256-column and 32-column launch splits; the transposed
    product is deterministic (bitwise equal on a repeat).  Tolerance 1e-13 of |Q|^T |X|."""
    import torch
    from fem_taichi_gb300 import _lib
    from fem_taichi_gb300.eigen import _TallSkinny
    from fem_taichi_gb300.model import _stream
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(n + m + b)
    Qf = rng.standard_normal((n, m + 3))
    X, C, W0 = rng.standard_normal((n, b)), rng.standard_normal((m, b)), rng.standard_normal((n, b + 2))
    Qd = torch.as_tensor(Qf, device=dev)[:, 2:2 + m]                # leading dimension m + 3
    ts = _TallSkinny(_lib.load(), n, dev, _stream(dev))
    Q = Qf[:, 2:2 + m]
    got = ts.tn(Qd, torch.as_tensor(X, device=dev))
    again = ts.tn(Qd, torch.as_tensor(X, device=dev))
    assert torch.equal(got, again)
    scale = np.abs(Q).T @ np.abs(X)
    assert np.all(np.abs(got.cpu().numpy() - Q.T @ X) <= 1e-13 * scale)
    Wd = torch.as_tensor(W0, device=dev)[:, 1:1 + b]
    ts.nn(Qd, torch.as_tensor(C, device=dev), Wd, -0.5, 2.0)
    want = 2.0 * W0[:, 1:1 + b] - 0.5 * (Q @ C)
    scale = 2.0 * np.abs(W0[:, 1:1 + b]) + 0.5 * (np.abs(Q) @ np.abs(C))
    assert np.all(np.abs(Wd.cpu().numpy() - want) <= 1e-13 * scale)
    out = torch.full((n, b), np.nan, dtype=torch.float64, device=dev)  # beta = 0 must not read W
    ts.nn(Qd, torch.as_tensor(C, device=dev), out, 1.0, 0.0)
    assert np.all(np.abs(out.cpu().numpy() - Q @ C) <= 1e-13 * (np.abs(Q) @ np.abs(C)))
