"""GPU parity pinned to the reference's own execution.

The CUDA path (both arithmetic variants) against ``tests/golden/refexec_*.npz``: outputs of
the reference's unmodified FEM_model_csr.py / FEM_model_bsr.py / POST_process.py, run under
the Taichi 0.6.28 stand-in (see tests/golden/make_refexec.py).

Tolerances (written here as in tests/checks.py): pattern bit-exact; K, KT, KM per scalar row
<= 1e-12 x row max, penalty entries exactly 1e20; M, F <= 1e-12 x max; stresses per node
<= 1e-10 x node max; on the full Mesh/2.cdb, K.v and M.v per entry <= 1e-12 x (|A|.|v|).
"""
import hashlib

import numpy as np
import pytest
import scipy.sparse as sp

import fem_taichi_gb300 as F
from tests.checks import assert_K_close, assert_rows_close, assert_stress_close, assert_vec_close
from tests.fixtures import (REFEXEC_SMALL, probe_vector, refexec, refexec_csr, refexec_materials,
                            refexec_physics)

pytestmark = pytest.mark.gpu

ALGOS = ["fp64", "dd"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


@pytest.fixture(scope="module", params=REFEXEC_SMALL)
def case(request):
    d = refexec(request.param)
    mat, om = refexec_materials(d)
    return request.param, d, refexec_physics(d), mat, om


@pytest.mark.parametrize("algo", ALGOS)
def test_K_M_F_match_reference(case, algo):
    name, d, P, mat, om = case
    M = F.Model(name, P, mat, Omegas=om, algo=algo)
    assert_K_close(M.Get_MatrixKL(), refexec_csr(d, "K"))
    Mg = M.Get_MatrixM()
    assert np.array_equal(Mg.indptr, d["M_indptr"]) and np.array_equal(Mg.indices, d["M_indices"])
    assert_vec_close(Mg.data, d["M_data"])
    assert_vec_close(M.Get_VectorF(), d["F"])


@pytest.mark.parametrize("algo", ALGOS)
def test_bsr_layout_matches_reference_bsr_variant(algo):
    """FEM_model_bsr.Get_MatrixKL (bsr_matrix((ValKT, ReNode, SmNode)).tocsr())."""
    for name in ("block_twist", "block_partial"):
        d = refexec(name)
        mat, om = refexec_materials(d)
        P = refexec_physics(d)
        K, _, _ = F.Model(name, P, mat, Omegas=om, algo=algo).assemble(k_layout="bsr", M=False, F=False)
        n3 = 3 * P.Num_Node
        Kb = sp.bsr_matrix((K.cpu().numpy(), P.ReNode, P.SmNode), shape=(n3, n3)).tocsr()
        assert_K_close(Kb, refexec_csr(d, "Kb"))


def test_device_topology_matches_reference():
    for name in REFEXEC_SMALL:
        d = refexec(name)
        P = refexec_physics(d, topology="gpu")
        assert np.array_equal(np.asarray(P.SmNode, np.int64), d["SmNode"])
        assert np.array_equal(np.asarray(P.ReNode, np.int64), d["ReNode"])
        assert np.array_equal(np.asarray(P.CoElem, np.int64), d["CoElem"])


@pytest.mark.parametrize("algo", ALGOS)
def test_stress_matches_reference(case, algo):
    name, d, P, mat, om = case
    S = F.Post(name, P, mat, d["u"].reshape(-1, 3, 1), algo=algo).Get_Stress()
    if name == "mesh2_isolated":
        # the reference's six averaged components (0/0 = NaN on the node without elements)
        assert_stress_close(S[:, :6], d["S_vector"])
    else:
        assert_stress_close(S, d["S"])


@pytest.mark.parametrize("name", ["block_twist", "block_partial"])
def test_tangent_matches_reference(name):
    d = refexec(name)
    mat, om = refexec_materials(d)
    M = F.Model(name, refexec_physics(d), mat, Omegas=om)
    M.LDinit(d["u_tangent"].reshape(-1))
    KT, KM = M.Get_MatrixKN()
    assert_K_close(KT, refexec_csr(d, "KT", "KT_indices", "KT_indptr"))
    assert_K_close(KM, refexec_csr(d, "KM", "KT_indices", "KT_indptr"))


@pytest.mark.parametrize("algo", ALGOS)
def test_full_mesh2_matches_reference(algo):
    d = refexec("mesh2_full")
    mat, om = refexec_materials(d)
    P = refexec_physics(d)
    M = F.Model("2", P, mat, Omegas=om, algo=algo)
    K, Mm, Fv = M.Get_MatrixKL(), M.Get_MatrixM(), M.Get_VectorF()
    assert _sha(K.indptr) == str(d["K_indptr_sha"]) and _sha(K.indices) == str(d["K_indices_sha"])
    assert _sha(Mm.indptr) == str(d["M_indptr_sha"]) and _sha(Mm.indices) == str(d["M_indices_sha"])
    v = probe_vector(K.shape[0])
    assert_rows_close(K @ v, d["Kv"], d["Kabs_v"])
    pen = d["Kdiag"] >= 1e19
    assert np.array_equal(K.diagonal()[pen], d["Kdiag"][pen])
    assert_rows_close(Mm @ v, d["Mv"], d["Mabs_v"])
    assert_vec_close(Fv, d["F"])
    S = F.Post("2", P, mat, d["u"], algo=algo, mesh=M.mesh).Get_Stress()
    assert_stress_close(S[d["S_nodes"]], d["S_sample"])
