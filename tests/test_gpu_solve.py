"""GPU static solve: BSR SpMV/SpMM, block Jacobi, FP64 PCG, FP32-inner/FP64-refinement,
multi-RHS, CUDA-graph replay, status codes.  Oracle: scipy SuperLU (FP64 direct solve, the
stand-in for the reference's MKL Pardiso).  Solution tolerance: relative error
||U - U*|| / ||U*|| <= 1e-8 for every solve (rtol 1e-12 on the FP64 true residual)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from tests.fixtures import STEEL

pytestmark = pytest.mark.gpu

ERR = 1e-8


def relerr(U, Ur):
    return np.linalg.norm(np.asarray(U) - Ur) / np.linalg.norm(Ur)


@pytest.fixture(scope="module")
def sysm():
    P = F.hex_block(20, 20, 6, size=(20.0, 20.0, 6.0), jitter=0.1, seed=1, fix="zmin", load_face="zmax",
                    load=(0, 0, -1))
    M = F.Model("s", P, STEEL)
    S = F.DeviceSystem(M)
    K = M.Get_MatrixKL()
    Fv = M.Get_VectorF()
    lu = spla.splu(K.tocsc())
    return P, M, S, K, Fv, lu


def test_spmv_f64_f32_and_spmm(sysm):
    P, M, S, K, Fv, lu = sysm
    rng = np.random.default_rng(0)
    x = rng.standard_normal(3 * P.Num_Node)
    scale = np.abs(K) @ np.abs(x)
    y = S.spmv(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.all(np.abs(y - K @ x) <= 1e-14 * scale)
    y32 = S.spmv(torch.from_numpy(x).float().cuda(), fp32=True).double().cpu().numpy()
    assert np.all(np.abs(y32 - K @ x) <= 2e-6 * scale)
    for R in (2, 4, 32):
        X = rng.standard_normal((3 * P.Num_Node, R))
        Y = S.spmv(torch.from_numpy(X).cuda(), nrhs=R).cpu().numpy()
        sc = np.abs(K) @ np.abs(X)
        assert np.all(np.abs(Y - K @ X) <= 1e-14 * sc)


def test_block_jacobi_inverse(sysm):
    P, M, S, K, Fv, lu = sysm
    bj = S.block_jacobi().cpu().numpy().reshape(-1, 3, 3)
    Kd = K.toarray() if K.shape[0] < 4000 else None
    for i in (0, 5, P.Num_Node // 2, P.Num_Node - 1):
        D = K[3 * i:3 * i + 3, 3 * i:3 * i + 3].toarray()
        assert np.allclose(bj[i] @ D, np.eye(3), atol=1e-10)
    assert Kd is None or True


def test_autotune_returns_valid_variant(sysm):
    S = sysm[2]
    for fp32 in (False, True):
        v = S.variant(fp32, 1)
        assert 0 <= v < 8


@pytest.mark.parametrize("mixed", [False, True])
def test_pcg_matches_direct_solve(sysm, mixed):
    P, M, S, K, Fv, lu = sysm
    Ur = lu.solve(Fv)
    U, st = S.solve(rtol=1e-12, mixed=mixed)
    assert st["status"] == 0, st
    assert st["relres"] <= 1e-12
    assert relerr(U.cpu().numpy(), Ur) <= ERR, st
    if mixed:
        assert st["outer"] >= 2


@pytest.mark.parametrize("mixed", [False, True])
def test_multi_rhs(sysm, mixed):
    P, M, S, K, Fv, lu = sysm
    rng = np.random.default_rng(5)
    Fm = np.stack([Fv] + [rng.standard_normal(3 * P.Num_Node) for _ in range(4)], axis=1)   # 5 -> padded 8
    U, st = S.solve(F=torch.from_numpy(Fm).cuda(), rtol=1e-12, mixed=mixed)
    assert st["status"] == 0 and U.shape == (3 * P.Num_Node, 5), st
    U = U.cpu().numpy()
    for k in range(5):
        assert relerr(U[:, k], lu.solve(Fm[:, k])) <= ERR


def test_32_rhs(sysm):
    P, M, S, K, Fv, lu = sysm
    rng = np.random.default_rng(6)
    Fm = rng.standard_normal((3 * P.Num_Node, 32))
    U, st = S.solve(F=torch.from_numpy(Fm).cuda(), rtol=1e-12, mixed=True)
    assert st["status"] == 0, st
    U = U.cpu().numpy()
    Ur = lu.solve(Fm)
    assert max(relerr(U[:, k], Ur[:, k]) for k in range(32)) <= ERR


def test_graph_replay_is_bitwise_identical_to_eager(sysm):
    S = sysm[2]
    U1, s1 = S.solve(rtol=1e-10, mixed=False, use_graph=True, unroll=8)
    U2, s2 = S.solve(rtol=1e-10, mixed=False, use_graph=False, unroll=8)
    U3, s3 = S.solve(rtol=1e-10, mixed=False, use_graph=True, unroll=8)
    assert torch.equal(U1, U2) and torch.equal(U1, U3)
    assert s1["iterations"] == s2["iterations"] == s3["iterations"]


def test_status_codes(sysm):
    P, M, S, K, Fv, lu = sysm
    U, st = S.solve(rtol=1e-12, maxit=5, mixed=False)
    assert st["status"] == _lib.FEM_ERR_MAXITER and st["iterations"] == 5
    Fn = S.F.clone()
    Fn[7] = float("nan")
    U, st = S.solve(F=Fn, rtol=1e-10, mixed=False)
    assert st["status"] == _lib.FEM_ERR_BREAKDOWN
    neg = F.DeviceSystem(M, K=-S.K64, F=S.F)
    U, st = neg.solve(rtol=1e-10, mixed=False, precond=-S.block_jacobi())
    assert st["status"] == _lib.FEM_ERR_NOT_SPD
    Z = torch.zeros_like(S.F)
    U, st = S.solve(F=Z, rtol=1e-10, mixed=True)
    assert st["status"] == 0 and float(U.abs().max()) == 0.0


def test_static_solver_dropin(sysm):
    P, M, S, K, Fv, lu = sysm
    sol = F.Static_solver(M, 0)
    U = sol.Solve_cpu()
    assert U.shape == (3 * P.Num_Node,)
    assert relerr(U, lu.solve(Fv)) <= ERR
    assert sol.last_stats["relres"] <= 1e-12


def test_c1_mixed_and_fp64_against_superlu():
    """40x40x12 (65,559 DOF): both solvers within 1e-8 of the FP64 direct solve."""
    P = F.config_mesh("c1")
    M = F.Model("c1", P, STEEL)
    S = F.DeviceSystem(M)
    K = M.Get_MatrixKL()
    Fv = M.Get_VectorF()
    Ur = spla.spsolve(K.tocsc(), Fv)
    for mixed in (False, True):
        U, st = S.solve(rtol=1e-12, mixed=mixed)
        assert st["status"] == 0, st
        assert relerr(U.cpu().numpy(), Ur) <= ERR, (mixed, st)
