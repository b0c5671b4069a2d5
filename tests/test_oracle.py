"""CPU tests of the oracle: golden fixtures, the two independent restatements against each
other, and analytic known-answer properties of the reference's element formulas."""
import hashlib

import numpy as np
import pytest

from oracle import c_oracle as C
from oracle import fem_oracle as O
from tests.fixtures import STEEL, golden, mesh2_physics

import fem_taichi_gb300 as F


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def m2():
    P = mesh2_physics()
    OM = O.OracleModel(P, STEEL, (0, 0, 100))
    return P, OM, OM.Get_MatrixKL(), OM.Get_MatrixM(), OM.Get_VectorF()


def test_golden_pattern(m2):
    P, *_ = m2
    g = golden()
    topo = O.pre_process(P.Node, P.Elem)
    assert _sha(topo["SmNode"]) == str(g["smnode_sha"])
    assert _sha(topo["ReNode"]) == str(g["renode_sha"])
    assert _sha(topo["CoElem"]) == str(g["coelem_sha"])
    assert int(topo["SmNode"][-1]) == int(g["nnzb"]) == 188100


def test_golden_values(m2):
    P, OM, K, M, Fv = m2
    g = golden()
    assert _sha(K.indptr) == str(g["k_indptr_sha"]) and _sha(K.indices) == str(g["k_indices_sha"])
    kv = np.asarray(K[g["k_row"], g["k_col"]]).ravel()
    scale = np.abs(np.where(K.data < 1e19, K.data, 0)).max()
    assert np.max(np.abs(kv - g["k_val"])) <= 1e-13 * scale
    assert np.max(np.abs(M.data[g["m_idx"]] - g["m_val"])) <= 1e-13 * np.abs(M.data).max()
    assert np.max(np.abs(Fv - g["f"])) <= 1e-13 * np.abs(Fv).max()
    assert int(np.sum(K.data == 1e20)) == int(g["n_penalty"])
    rng = np.random.default_rng(int(g["u_seed"]))
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
    for mode, key in (("written", "s_val"), ("aliased", "s_alias_val")):
        S = O.oracle_stress(P, STEEL, u, gmat_mode=mode)[g["s_nodes"]]
        sc = np.abs(g[key]).max(axis=1, keepdims=True)
        assert np.all(np.abs(S - g[key]) <= 1e-11 * sc)


def test_bsr_equals_csr_direct(m2):
    """FEM_model_bsr's bsr.tocsr() and FEM_model_csr's in-place CSR give the same matrix."""
    P, OM, K, *_ = m2
    Kd = O.csr_direct_K(P, OM.ValKT())
    assert np.array_equal(K.indptr, Kd.indptr) and np.array_equal(K.indices, Kd.indices)
    assert np.array_equal(K.data, Kd.data)


def _c_args(P):
    bn = np.concatenate([P.Nind[np.asarray(b[0])] for b in P.Bounds]) if P.Bounds else np.zeros(0, int)
    bc = (np.concatenate([np.repeat(np.array(b[1], float)[None], len(b[0]), 0) for b in P.Bounds])
          if P.Bounds else np.zeros((0, 3)))
    fn = np.concatenate([P.Nind[np.asarray(f[0])] for f in P.Forces]) if P.Forces else np.zeros(0, int)
    fv = (np.concatenate([np.repeat(np.array(f[1], dtype=np.int64).astype(float)[None], len(f[0]), 0)
                          for f in P.Forces]) if P.Forces else np.zeros((0, 3)))
    return bn, bc, fn, fv


@pytest.mark.parametrize("nthreads", [1, 4])
def test_c_vs_numpy_restatement(m2, nthreads):
    P, OM, K, M, Fv = m2
    Kc, Mc, Fc = C.assemble(P.xyz, P.conn, P.SmNode, P.ReNode, STEEL, (0, 0, 100), *_c_args(P),
                            nthreads=nthreads)
    Kn = OM.ValKT()
    pen = Kn >= 1e19
    assert np.array_equal(Kc[pen], Kn[pen])
    scale = np.abs(np.where(pen, 0, Kn)).max()
    assert np.abs(np.where(pen, 0, Kc - Kn)).max() <= 1e-13 * scale
    assert np.abs(Mc - OM.ValMB()).max() <= 1e-13 * np.abs(Mc).max()
    assert np.abs(Fc.reshape(-1) - Fv).max() <= 1e-13 * np.abs(Fv).max()


def test_c_vs_numpy_stress(m2):
    P = m2[0]
    rng = np.random.default_rng(3)
    u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
    for mode in ("written", "aliased"):
        S = O.oracle_stress(P, STEEL, u, gmat_mode=mode)
        Sc = C.stress(P.xyz, P.conn, P.CoElem, STEEL, u, O.extrapolation_table(mode), nthreads=2)
        sc = np.abs(S).max(axis=1, keepdims=True)
        assert np.all(np.abs(Sc - S) <= 1e-12 * sc)


# ---- analytic known-answer tests of the restated formulas ---------------------------------
@pytest.fixture(scope="module")
def small():
    P = F.hex_block(5, 4, 3, size=(5.0, 4.0, 3.0), jitter=0.15, seed=11, fix=None)
    OM = O.OracleModel(P, STEEL, (0, 0, 0))
    return P, OM


def _rigid_modes(xyz):
    n = xyz.shape[0]
    modes = []
    for d in range(3):
        v = np.zeros((n, 3))
        v[:, d] = 1
        modes.append(v.ravel())
    for a, b in ((0, 1), (1, 2), (0, 2)):
        v = np.zeros((n, 3))
        v[:, a] = -xyz[:, b]
        v[:, b] = xyz[:, a]
        modes.append(v.ravel())
    return modes


def test_kat_rigid_body_null_space(small):
    P, OM = small
    V = OM.ValKT()
    # remove the auto-added penalty on node Nind[0] (reference behaviour with no bounds)
    n3 = 3 * P.Num_Node
    import scipy.sparse as sp
    K = sp.bsr_matrix((V, P.ReNode, P.SmNode), shape=(n3, n3)).tocsr()
    d = K.diagonal()
    d[d >= 1e19] = 0
    K.setdiag(d)
    i0 = P.Nind[0]
    Kd = O.OracleModel(P, STEEL, (0, 0, 0)).element_K(0, P.Num_Elem)
    kii = sum(Kd[e, a, a] for e in range(P.Num_Elem) for a in range(8) if P.conn[e, a] == i0)
    for j in range(3):
        K[3 * i0 + j, 3 * i0 + j] = kii[j, j]
    scale = np.abs(K.data).max()
    for r in _rigid_modes(P.xyz):
        assert np.abs(K @ r).max() <= 1e-9 * scale * np.abs(r).max()
    assert abs(K - K.T).max() <= 1e-12 * scale


def test_kat_mass_volume_and_centrifugal(small):
    P, OM = small
    mb = OM.ValMB()
    C_, _ = O._coords(P)
    vol = sum(O.det3(C_ @ O.DNR[g]).sum() for g in range(8))        # sum_g detJ = volume
    assert abs(vol - 5 * 4 * 3) <= 1e-12 * 60
    assert abs(mb.sum() - STEEL['DE'] * vol) <= 1e-13 * STEEL['DE'] * vol
    om = np.array([0.0, 0.0, 100.0])
    OMw = O.OracleModel(P, STEEL, om)
    Fn = OMw.ValF()
    # resultant = rho w^2 int (x, y, 0) dV; for the jittered block use the GP quadrature itself
    mom = np.zeros(3)
    for g in range(8):
        J = C_ @ O.DNR[g]
        X = C_ @ O.NR[g]
        mom += (O.det3(J)[:, None] * X).sum(axis=0)
    expect = STEEL['DE'] * 100.0 ** 2 * np.array([mom[0], mom[1], 0.0])
    assert np.allclose(Fn.sum(axis=0), expect, rtol=1e-12, atol=1e-18)


def test_kat_constant_stress_patch(small):
    """A linear displacement field gives the same constant stress at every node, for both
    extrapolation tables (each row of W sums to one)."""
    P, _ = small
    Gd = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -1e-3, 1e-4], [2e-4, 3e-4, 4e-4]])
    u = P.xyz @ Gd.T
    D0, D1 = O.dmats(STEEL['EX'], STEEL['PO'])
    eps_n = np.diag(Gd)
    sig_n = D0 @ eps_n
    mu = D1[0, 0]
    sig_s = mu * np.array([Gd[0, 1] + Gd[1, 0], Gd[1, 2] + Gd[2, 1], Gd[0, 2] + Gd[2, 0]])
    for mode in ("written", "aliased"):
        S = O.oracle_stress(P, STEEL, u, gmat_mode=mode)
        assert np.allclose(S[:, :3], sig_n[None], rtol=1e-10, atol=1e-9)
        assert np.allclose(S[:, 3:6], sig_s[None], rtol=1e-10, atol=1e-9)
        for mode_w in ("written", "aliased"):
            assert np.allclose(O.extrapolation_table(mode_w).sum(axis=1), 1.0, rtol=0, atol=1e-14)


def test_penalty_and_auto_bound(small):
    """No Bounds: the reference packs one zero column and so fixes node Nind[0]."""
    P, OM = small
    V = OM.ValKT()
    i0 = P.Nind[0]
    s = P.SmNode[i0] + np.nonzero(P.ReNode[P.SmNode[i0]:P.SmNode[i0 + 1]] == i0)[0][0]
    assert all(V[s, j, j] == 1e20 for j in range(3))
    assert np.sum(V == 1e20) == 3


def test_force_int_cast():
    """Load values are truncated to int before use (FEM_model_bsr.py:82)."""
    P = F.hex_block(2, 2, 1, jitter=0.0, fix="zmin", load_face="zmax", load=(0.7, -1.9, 2.5))
    OM = O.OracleModel(P, STEEL, (0, 0, 0))
    Fv = OM.ValF()
    top = P.Nind[P.Forces[0][0]]
    assert np.allclose(Fv[top], [[0.0, -1.0, 2.0]] * len(top))
