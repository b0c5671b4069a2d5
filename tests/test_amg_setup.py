"""Multigrid hierarchy built by the library on the host (fem_amg_setup, no GPU involved)
against the numpy restatement in oracle/amg_oracle.py.

Checked per level: the aggregates and Dirichlet rows (bit-exact), the inverse diagonal blocks, the prolongator
P, the restriction R = P^T and the coarse operator A_c = P^T A P (all within 1e-12 of the
largest entry: same arithmetic, different summation order), the Lanczos estimate of
lambda_max(D^-1 A) (1e-9 relative), and the dense inverse of the last level (1e-10).
The oracle uses the library's lambda_max so that the rest of the comparison is not
blurred by the estimate.  Also: the hierarchy is the same for 1 and for all host threads,
and bad inputs are refused before any work."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.sparse as sp

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.solve import AmgHierarchy
from oracle import amg_oracle as AO
from oracle import c_oracle as C
from tests.fixtures import STEEL

REL = 1e-12
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def host_system(P, omega=(0, 0, 100)):
    bn = P.Nind[P.Bounds[0][0]] if P.Bounds else np.zeros(0, dtype=np.int64)
    K, _, _ = C.assemble(P.xyz, P.conn, P.SmNode, P.ReNode, STEEL, omega, bn, np.zeros((bn.size, 3)), nthreads=0)
    n = P.Num_Node
    Kb = sp.bsr_matrix((K, np.asarray(P.ReNode), np.asarray(P.SmNode)), shape=(3 * n, 3 * n))
    Kb.sort_indices()
    return Kb


CASES = {
    "jittered_block": lambda: F.hex_block(8, 6, 5, size=(8.0, 3.0, 2.0), jitter=0.1, seed=3, fix="xmin",
                                          load_face="xmax", load=(0, 0, -1.0)),
    "twisted_slab": lambda: F.hex_block(16, 4, 3, size=(16.0, 2.0, 1.0), jitter=0.05, twist_deg=60, seed=5,
                                        fix="xmin", load_face="xmax", load=(0, 1.0, 0)),
}


def bsr_dense(ptr, col, blk, rows, cols):
    return sp.bsr_matrix((blk, col, ptr), shape=(rows, cols)).toarray()


@pytest.fixture(scope="module", params=sorted(CASES))
def built(request):
    P = CASES[request.param]()
    Kb = host_system(P)
    L = _lib.load()
    H = AmgHierarchy(L, P.Num_Node, Kb.indptr, Kb.indices, Kb.data, P.xyz, None, max_coarse=100)
    info = H.levels()
    levels, cinv = AO.setup(Kb, P.xyz, max_coarse=100, lmax_given=[lv["lmax"] for lv in info])
    return P, Kb, H, info, levels, cinv


def test_level_sizes_and_lmax(built):
    P, Kb, H, info, levels, cinv = built
    assert len(info) == len(levels) >= 2
    for l, lv in enumerate(levels):
        assert info[l]["n"] == lv["n"] and info[l]["b"] == lv["b"]
        if "lmax_oracle" in lv:
            assert abs(info[l]["lmax"] - lv["lmax_oracle"]) <= 1e-9 * lv["lmax_oracle"]
            assert info[l]["omega"] == pytest.approx(4.0 / (3.0 * info[l]["lmax"]), rel=1e-15)


def test_aggregates_prolongator_and_coarse_operator(built):
    P, Kb, H, info, levels, cinv = built
    for l, lv in enumerate(levels[:-1]):
        assert np.array_equal(H.export(l, 4), lv["agg"])
        assert np.array_equal(H.export(l, 6).astype(bool), lv["dirichlet"])
        b, n, na = lv["b"], lv["n"], lv["na"]
        Pl = bsr_dense(*H.export(l, 1), n * b, na * 6)
        Po = lv["P"].toarray()
        assert np.abs(Pl - Po).max() <= REL * np.abs(Po).max()
        Rl = bsr_dense(*H.export(l, 2), na * 6, n * b)
        assert np.array_equal(Rl, Pl.T)
        di = H.export(l, 3).reshape(-1, b, b)
        assert np.abs(di - lv["Dinv"]).max() <= REL * np.abs(lv["Dinv"]).max()
    for l in range(1, len(levels)):
        lv = levels[l]
        Al = bsr_dense(*H.export(l, 0), lv["n"] * 6, lv["n"] * 6)
        Ao = lv["A"].toarray()
        assert np.abs(Al - Ao).max() <= REL * np.abs(Ao).max()
        assert np.array_equal(Al, Al.T) or np.abs(Al - Al.T).max() <= REL * np.abs(Al).max()


def test_coarse_inverse(built):
    P, Kb, H, info, levels, cinv = built
    ci = H.export(len(levels) - 1, 5).reshape(cinv.shape)
    assert np.abs(ci - cinv).max() <= 1e-10 * np.abs(cinv).max()


def test_oracle_vcycle_is_a_good_preconditioner(built):
    """The restated cycle (FP64) on the library's hierarchy: symmetric, and CG with it needs
    far fewer iterations than with block Jacobi."""
    P, Kb, H, info, levels, cinv = built
    A = sp.csr_matrix(Kb)
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal((2, A.shape[0]))
    vx, vy = AO.vcycle(levels, cinv, x), AO.vcycle(levels, cinv, y)
    assert abs(y @ vx - x @ vy) <= 1e-10 * np.linalg.norm(vx) * np.linalg.norm(y)
    assert x @ vx > 0

    def pcg(apply, b, rtol=1e-8):
        u = np.zeros_like(b)
        r = b.copy()
        z = apply(r)
        p = z.copy()
        rz = r @ z
        for it in range(5000):
            q = A @ p
            a = rz / (p @ q)
            u += a * p
            r -= a * q
            if np.linalg.norm(r) <= rtol * np.linalg.norm(b):
                return it + 1
            z = apply(r)
            rzn = r @ z
            p = z + rzn / rz * p
            rz = rzn
        return 5000

    b = rng.standard_normal(A.shape[0])
    n = P.Num_Node
    Dinv = levels[0]["Dinv"]
    it_amg = pcg(lambda r: AO.vcycle(levels, cinv, r), b)
    it_bj = pcg(lambda r: np.einsum("nij,nj->ni", Dinv, r.reshape(n, 3)).reshape(-1), b)
    assert it_amg * 3 < it_bj, (it_amg, it_bj)


def _dump_hierarchy(threads):
    code = f"""
import os, sys, hashlib
sys.path.insert(0, {ROOT!r})
import numpy as np
from tests.test_amg_setup import CASES, host_system
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.solve import AmgHierarchy
P = CASES['twisted_slab']()
Kb = host_system(P)
H = AmgHierarchy(_lib.load(), P.Num_Node, Kb.indptr, Kb.indices, Kb.data, P.xyz, None, max_coarse=100)
h = hashlib.sha256()
for l in range(len(H.levels()) - 1):
    for what in (1, 2):
        for a in H.export(l, what):
            h.update(np.ascontiguousarray(a).tobytes())
print(h.hexdigest())
"""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return out.stdout.strip().splitlines()[-1]


def test_hierarchy_independent_of_thread_count():
    assert _dump_hierarchy(1) == _dump_hierarchy(max(2, os.cpu_count() or 2))


def test_bad_inputs_refused():
    L = _lib.load()
    o = _lib.FemAmgOpts()
    L.fem_amg_default_opts(ctypes.byref(o))
    h = ctypes.c_void_p()
    ip = np.array([0, 2, 3], dtype=np.int32)
    ix = np.array([1, 0, 1], dtype=np.int32)  # row 0 not ascending
    va = np.ones(27)
    xy = np.zeros(6)
    rc = L.fem_amg_setup(2, ip.ctypes.data, ix.ctypes.data, va.ctypes.data, xy.ctypes.data, ctypes.byref(o),
                         ctypes.byref(h))
    assert rc == _lib.FEM_ERR_INVALID and not h.value
    rc = L.fem_amg_setup(2, ip.ctypes.data, None, va.ctypes.data, xy.ctypes.data, ctypes.byref(o), ctypes.byref(h))
    assert rc == _lib.FEM_ERR_INVALID
    o.pre_degree = 0
    ix = np.array([0, 1, 1], dtype=np.int32)
    rc = L.fem_amg_setup(2, ip.ctypes.data, ix.ctypes.data, va.ctypes.data, xy.ctypes.data, ctypes.byref(o),
                         ctypes.byref(h))
    assert rc == _lib.FEM_ERR_INVALID


def _setup(Kb, xyz, **opts):
    return AmgHierarchy(_lib.load(), Kb.shape[0] // 3, Kb.indptr, Kb.indices, Kb.data, xyz, None, **opts)


def test_single_dense_level_when_small():
    """A system at most max_coarse DOF is one dense level: its inverse is K^-1."""
    P = F.hex_block(3, 2, 2, jitter=0.1, seed=9, fix="zmin")
    Kb = host_system(P)
    H = _setup(Kb, P.xyz, max_coarse=10000)
    assert len(H.levels()) == 1
    inv = H.export(0, 5).reshape(Kb.shape)
    Kd = Kb.toarray()
    assert np.abs(inv @ Kd - np.eye(Kd.shape[0])).max() <= 1e-8


def test_all_penalised_nodes_give_no_aggregates():
    """Every diagonal entry penalised (1e20): no strong couplings, no aggregates, all rows
    Dirichlet on the dense level; the setup still succeeds."""
    P = F.hex_block(4, 3, 3, jitter=0.1, seed=2, fix=None)
    Kb = host_system(P)
    Kb = sp.bsr_matrix(Kb.tocsr() + sp.identity(Kb.shape[0]) * 1e20, blocksize=(3, 3))
    Kb.sort_indices()
    H = _setup(Kb, P.xyz, max_coarse=10)
    lv = H.levels()
    assert len(lv) == 1 and lv[0]["n"] == P.Num_Node


def test_theta_zero_and_one_level_cap():
    P = F.hex_block(6, 4, 3, jitter=0.1, seed=4, fix="xmin")
    Kb = host_system(P)
    H = _setup(Kb, P.xyz, theta=0.0, max_coarse=60)
    lv = H.levels()
    assert len(lv) >= 2 and lv[1]["n"] < lv[0]["n"]
    H1 = _setup(Kb, P.xyz, max_levels=1)
    assert len(H1.levels()) == 1


def test_uncoarsenable_large_level_is_refused():
    """A level that is too large for the dense solve and cannot be coarsened (a purely
    diagonal system: no couplings) is refused with FEM_ERR_INVALID, not run."""
    n = 3000
    Kb = sp.bsr_matrix(sp.identity(3 * n, format="csr") * 2.0, blocksize=(3, 3))
    Kb.sort_indices()
    xyz = np.random.default_rng(0).uniform(size=(n, 3))
    with pytest.raises(_lib.FemError) as e:
        _setup(Kb, xyz, max_coarse=100)
    assert e.value.code == _lib.FEM_ERR_INVALID


def test_set_smoother_checks_its_arguments(built):
    """fem_amg_set_smoother (per-level smoother weights): accepted on every level but the dense
    last one, within 1 <= upper <= 4 and 1 < ratio <= 1e4; refused otherwise."""
    H = built[2]
    n = len(H.levels())
    L = H.lib
    for l in range(n - 1):
        assert L.fem_amg_set_smoother(H.h, l, 1.2, 20.0) == 0
    assert L.fem_amg_set_smoother(H.h, n - 1, 1.2, 20.0) == _lib.FEM_ERR_INVALID
    assert L.fem_amg_set_smoother(H.h, -1, 1.2, 20.0) == _lib.FEM_ERR_INVALID
    assert L.fem_amg_set_smoother(H.h, 0, 0.9, 20.0) == _lib.FEM_ERR_INVALID
    assert L.fem_amg_set_smoother(H.h, 0, 1.2, 1.0) == _lib.FEM_ERR_INVALID
    assert L.fem_amg_set_smoother(H.h, 0, 1.1, 30.0) == 0   # back to the defaults
