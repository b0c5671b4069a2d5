"""Parity pinned to the reference's own execution (CPU).

``tests/golden/refexec_*.npz`` hold outputs of the reference's unmodified
FEM_model_csr.py (K CSR written in place, M, F; :118-146, 150-243), FEM_model_bsr.py
(Get_MatrixKL via bsr.tocsr(), Get_MatrixKN; :123-145, 163-191) and POST_process.py
(Get_Stress; :72-99, 172-223) on small meshes, produced under the Taichi 0.6.28 stand-in by
tests/golden/make_refexec.py.  These tests check the oracle and this package's host topology
against them; tests/test_gpu_refexec.py checks the CUDA path.

Tolerances: pattern bit-exact; K per scalar row <= 1e-12 x row max (penalty exactly 1e20);
M, F <= 1e-12 x max; stresses per node <= 1e-10 x node max.
"""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import fem_oracle as O
from tests.checks import assert_K_close, assert_rows_close, assert_stress_close, assert_vec_close
from tests.fixtures import (REFEXEC_SMALL, probe_vector, refexec, refexec_csr, refexec_materials,
                            refexec_physics)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _loads(P):
    """Nodal loads as the reference packs them (FEM_model_*.py:75-84, int cast), node-major."""
    fp = O._forces_packed(P)
    out = np.zeros((P.Num_Node, 3))
    if P.Forces:
        np.add.at(out, P.Nind[fp[0].astype(np.int64)], fp[1:].T)
    return out.reshape(-1)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


@pytest.fixture(scope="module", params=REFEXEC_SMALL)
def case(request):
    d = refexec(request.param)
    P = refexec_physics(d)
    mat, om = refexec_materials(d)
    return request.param, d, P, mat, om, O.OracleModel(P, mat, om)


def test_topology_matches_reference_pre_process(case):
    """Read.pre_process (READ_physics.py:42-61) as the reference ran it vs this package's
    native host build and the oracle's restatement: bit-exact."""
    name, d, P, *_ = case
    for got in (P, O.pre_process(P.Node, P.Elem)):
        sm = got.SmNode if hasattr(got, "SmNode") else got["SmNode"]
        re = got.ReNode if hasattr(got, "ReNode") else got["ReNode"]
        co = got.CoElem if hasattr(got, "CoElem") else got["CoElem"]
        assert np.array_equal(np.asarray(sm, np.int64), d["SmNode"])
        assert np.array_equal(np.asarray(re, np.int64), d["ReNode"])
        assert np.array_equal(np.asarray(co, np.int64), d["CoElem"])


def test_oracle_K_matches_reference(case):
    name, d, P, mat, om, OM = case
    Kref = refexec_csr(d, "K")
    assert_K_close(OM.Get_MatrixKL(), Kref)
    if "Kb_data" in d:            # the BSR variant's bsr.tocsr(): same pattern, same values
        Kb = refexec_csr(d, "Kb")
        assert_K_close(Kb, Kref)


def test_oracle_M_and_F_match_reference(case):
    name, d, P, mat, om, OM = case
    Mo = OM.Get_MatrixM()
    assert np.array_equal(Mo.indptr, d["M_indptr"]) and np.array_equal(Mo.indices, d["M_indices"])
    assert_vec_close(Mo.data, d["M_data"])
    Fo = OM.Get_VectorF()
    assert_vec_close(Fo, d["F"])
    # the centrifugal part alone (nodal loads are small integers after the reference's cast)
    loads = _loads(P)
    if np.any(loads):
        assert_vec_close(Fo - loads, d["F"] - loads)


def test_reference_casts_forces_to_int():
    """FEM_model_*.py:78 casts the Forces values to int: (1.7, -2.5, 3.9) adds (1, -2, 3)."""
    d = refexec("block_twist")
    P = refexec_physics(d)
    mat, om = refexec_materials(d)
    cen = O.OracleModel(P, mat, om).Get_VectorF() - _loads(P)
    top = P.Nind[d["forces_ids"]]
    got = (d["F"] - cen).reshape(-1, 3)[top]
    assert np.allclose(got, [1.0, -2.0, 3.0], rtol=0, atol=1e-9)


def test_oracle_stress_matches_reference(case):
    """Post.Get_Stress as the reference computes it: under Taichi 0.6's dense addressing the
    shape-2 GMat field (POST_process.py:145) aliases entry j to j & 1, which is the oracle's
    'aliased' reading; the 'written' reading (eight distinct corners) does not match."""
    name, d, P, mat, om, OM = case
    u = d["u"]
    if name == "mesh2_isolated":
        return
    assert_stress_close(O.oracle_stress(P, mat, u, gmat_mode="aliased"), d["S"])
    Sw = O.oracle_stress(P, mat, u, gmat_mode="written")
    assert np.max(np.abs(Sw - d["S"])) > 1e-3 * np.max(np.abs(d["S"]))


def test_isolated_node_components_are_nan_in_the_reference():
    d = refexec("mesh2_isolated")
    P = refexec_physics(d)
    mat, _ = refexec_materials(d)
    V = d["S_vector"]
    iso = np.nonzero(np.asarray(P.CoElem) == 0)[0]
    assert iso.size == 1 and np.all(np.isnan(V[iso]))
    keep = np.asarray(P.CoElem) > 0
    # the oracle's six components on the other nodes (its eigen step needs finite rows)
    import types
    Q = types.SimpleNamespace(**{k: getattr(P, k) for k in ("Node", "Elem", "Nind", "conn", "CoElem")})
    Q.CoElem = np.where(keep, P.CoElem, 1)
    S6 = O.oracle_stress(Q, mat, d["u"], gmat_mode="aliased")[:, :6]
    assert_stress_close(S6[keep], V[keep])


@pytest.mark.parametrize("name", ["block_twist", "block_partial"])
def test_oracle_tangent_matches_reference(name):
    """FEM_model_bsr.LDinit + Get_MatrixKN (:134-145, 455-598) at a finite displacement."""
    d = refexec(name)
    P = refexec_physics(d)
    mat, om = refexec_materials(d)
    KTo, KMo = O.OracleModel(P, mat, om).Get_MatrixKN(d["u_tangent"])
    assert_K_close(KTo, refexec_csr(d, "KT", "KT_indices", "KT_indptr"))
    assert_K_close(KMo, refexec_csr(d, "KM", "KT_indices", "KT_indptr"))


@pytest.mark.slow
def test_oracle_matches_reference_on_full_mesh2():
    """All of Mesh/2.cdb: pattern digests bit-exact, K.v and M.v per entry within 1e-12 of
    |A|.|v|, F within 1e-12, sampled stresses within 1e-10."""
    d = refexec("mesh2_full")
    P = refexec_physics(d)
    mat, om = refexec_materials(d)
    assert _sha(P.SmNode) == str(d["SmNode_sha"]) and _sha(P.ReNode) == str(d["ReNode_sha"])
    assert np.array_equal(np.asarray(P.CoElem), d["CoElem"])
    OM = O.OracleModel(P, mat, om)
    K, M = OM.Get_MatrixKL(), OM.Get_MatrixM()
    assert _sha(K.indptr) == str(d["K_indptr_sha"]) and _sha(K.indices) == str(d["K_indices_sha"])
    assert _sha(M.indptr) == str(d["M_indptr_sha"]) and _sha(M.indices) == str(d["M_indices_sha"])
    v = probe_vector(K.shape[0])
    assert_rows_close(K @ v, d["Kv"], d["Kabs_v"])
    assert np.array_equal(K.diagonal()[d["Kdiag"] >= 1e19], d["Kdiag"][d["Kdiag"] >= 1e19])
    assert_rows_close(M @ v, d["Mv"], d["Mabs_v"])
    assert_vec_close(OM.Get_VectorF(), d["F"])
    S = O.oracle_stress(P, mat, d["u"], gmat_mode="aliased")
    assert_stress_close(S[d["S_nodes"]], d["S_sample"])


def test_fixtures_reproduce_from_the_reference():
    """Re-runs the reference's own code (unmodified, Taichi stand-in) on two small cases and
    requires the committed fixtures back bit for bit.  Needs a reference checkout, named by
    FEM_TAICHI_REFERENCE (default /root/reference); skipped without one."""
    ref = os.environ.get("FEM_TAICHI_REFERENCE", "/root/reference")
    if not os.path.isfile(os.path.join(ref, "FEM_model_csr.py")):
        pytest.skip("no reference checkout")
    r = subprocess.run([sys.executable, "-W", "ignore", os.path.join(ROOT, "tests", "golden", "make_refexec.py"),
                        ref, "--check", "block_nobc", "block_partial"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
