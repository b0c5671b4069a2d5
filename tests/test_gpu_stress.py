"""GPU parity of nodal stress recovery against the oracle.

Tolerance: stresses, principal stresses and "VM" within 1e-10 relative -- per node, the
largest deviation over the 10 columns is at most 1e-10 x the largest |value| of that node.
"""
import numpy as np
import pytest

import fem_taichi_gb300 as F
from oracle import c_oracle as C
from oracle import fem_oracle as O
from tests.fixtures import STEEL, mesh2_physics

pytestmark = pytest.mark.gpu

REL = 1e-10


def assert_stress_close(S, So, rel=REL):
    assert S.shape == So.shape
    sc = np.abs(So).max(axis=1, keepdims=True)
    dev = np.abs(S - So)
    assert np.all(dev <= rel * sc), f"max rel dev {np.max(dev / np.maximum(sc, 1e-300))}"


@pytest.mark.parametrize("algo", ["dd", "fp64"])
@pytest.mark.parametrize("mode", ["written", "aliased"])
@pytest.mark.parametrize("name", ["mesh2", "c1", "twisted"])
def test_stress_matches_oracle(name, mode, algo):
    P = {"mesh2": mesh2_physics, "c1": lambda: F.config_mesh("c1"),
         "twisted": lambda: F.hex_block(6, 5, 3, jitter=0.12, twist_deg=40, seed=4)}[name]()
    rng = np.random.default_rng(17)
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3, 1))
    S = F.Post(name, P, STEEL, u, gmat_mode=mode, algo=algo).Get_Stress()
    assert_stress_close(S, O.oracle_stress(P, STEEL, u, gmat_mode=mode))


def test_constant_stress_field_is_reproduced_exactly():
    P = F.hex_block(5, 4, 3, jitter=0.15, seed=1)
    Gd = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -1e-3, 1e-4], [2e-4, 3e-4, 4e-4]])
    u = P.xyz @ Gd.T
    S = F.Post("p", P, STEEL, u).Get_Stress()
    assert np.allclose(S, S[:1], rtol=1e-10, atol=1e-8)


def test_isolated_node_gives_nan_like_reference():
    """A node with no element divides 0 by CoElem = 0 (POST_process.py:186)."""
    xyz = np.vstack([F.hex_block(1, 1, 1).xyz, [[5.0, 5.0, 5.0]]])
    elem = F.hex_block(1, 1, 1).Elem
    P = F.Physics(np.arange(1, 10), xyz, elem, [], [])
    S = F.Post("i", P, STEEL, np.zeros((9, 3))).Get_Stress()
    assert np.all(np.isnan(S[8, :6])) and np.all(np.isfinite(S[:8]))


def test_full_size_c2_stress_against_c_oracle():
    P = F.config_mesh("c2")
    rng = np.random.default_rng(2)
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
    Sc = C.stress(P.xyz, P.conn, P.CoElem, STEEL, u, O.extrapolation_table("aliased"), nthreads=0)
    for algo in ("dd", "fp64"):
        S = F.Post("c2", P, STEEL, u, algo=algo).Get_Stress()
        assert_stress_close(S, Sc)


def test_double_eigenvalues_and_constant_fields():
    """Uniaxial / hydrostatic stress states have repeated principal values, the hard case
    for eigenvalue accuracy."""
    P = F.hex_block(4, 3, 3, jitter=0.1, seed=8)
    n = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    for Gd in (np.diag([1e-3, 0.0, 0.0]), np.eye(3) * 1e-3, np.outer(n, n) * 1e-3,
               np.outer(n, n) * 1e-3 + np.eye(3) * 2e-4):
        u = P.xyz @ Gd.T
        for algo in ("dd", "fp64"):
            S = F.Post("p", P, STEEL, u, algo=algo).Get_Stress()
            assert_stress_close(S, O.oracle_stress(P, STEEL, u))


def test_row_ordered_and_element_ordered_records_agree():
    """FEM_ALGO_DD stress with and without mesh->ne_inv (row-ordered vs element-ordered
    corner records) gives the same bits."""
    import ctypes
    import torch
    P = F.hex_block(9, 7, 4, jitter=0.12, seed=5)
    rng = np.random.default_rng(3)
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
    post = F.Post("r", P, STEEL, u)
    a = post.stress_device().clone()
    c = post.mesh.c
    saved = c.ne_inv
    try:
        c.ne_inv = None
        b = post.stress_device().clone()
    finally:
        c.ne_inv = saved
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(a), torch.nan_to_num(b))
