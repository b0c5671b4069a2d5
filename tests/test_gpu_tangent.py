"""Large-displacement tangent / secant matrices (Get_MatrixKN, FEM_model_bsr.py:134-145,
476-592) against the oracle, and the device Newton iteration (SOLVE_static.py:41-75) against
the oracle's with exact solves.

Tolerances: KT, KM per scalar row <= 1e-12 x row max (penalty entries exactly 1e20); Newton
displacements <= 1e-8 relative."""
import numpy as np
import pytest

import fem_taichi_gb300 as F
from oracle import fem_oracle as O
from oracle import solve_oracle as SO
from tests.fixtures import STEEL
from tests.test_gpu_assembly import assert_K_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["block", "twisted"])
def test_tangent_and_secant_match_oracle(name):
    P = {"block": lambda: F.hex_block(5, 4, 3, jitter=0.1, seed=2, fix="zmin"),
         "twisted": lambda: F.hex_block(6, 3, 3, jitter=0.12, twist_deg=35, seed=4, fix="zmin")}[name]()
    M = F.Model("t", P, STEEL)
    U = np.random.default_rng(5).uniform(-0.03, 0.03, size=(P.Num_Node, 3))
    M.LDinit(U.reshape(-1))
    KT, KM = M.Get_MatrixKN()
    KTo, KMo = O.OracleModel(P, STEEL).Get_MatrixKN(U)
    assert_K_close(KT, KTo)
    assert_K_close(KM, KMo)


def test_zero_displacement_gives_the_linear_stiffness():
    P = F.hex_block(4, 3, 3, jitter=0.1, seed=1, fix="zmin")
    M = F.Model("z", P, STEEL)
    M.LDinit(np.zeros(3 * P.Num_Node))
    KT, KM = M.Get_MatrixKN()
    K = M.Get_MatrixKL()
    assert_K_close(KT, K)
    assert_K_close(KM, K)


def test_newton_matches_oracle_on_a_bent_cantilever():
    P = F.hex_block(2, 2, 8, size=(2.0, 2.0, 8.0), jitter=0.05, seed=3, fix="zmin")
    load = F.face_traction_loads(P, "zmax", (60.0, 0.0, 0.0))
    M = F.Model("c", P, STEEL, Omegas=(0, 0, 0), extra_loads=load)
    solver = F.Static_solver(M, Qtype=1)
    U = solver.Solve_cpu(max_errs=1e-9, max_iters=30)
    st = solver.last_stats
    assert st["converged"] and st["steps"] >= 2
    OM = O.OracleModel(P, STEEL, (0, 0, 0))
    Fo = OM.Get_VectorF() + load.reshape(-1)
    Uo, res = SO.newton_large_displacement(OM, Fo, max_errs=1e-9, max_iters=30)
    assert np.linalg.norm(U - Uo) <= 1e-8 * np.linalg.norm(Uo)
    # the nonlinear answer differs from the linear one (the load bends the beam appreciably)
    Ul = np.linalg.solve(M.Get_MatrixKL().toarray(), M.Get_VectorF())
    assert np.linalg.norm(U - Ul) > 1e-3 * np.linalg.norm(Ul)
