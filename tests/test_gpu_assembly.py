"""GPU parity of K / M / F assembly against the oracle.

Tolerances (stated by the hot-path contract): block pattern (indptr / indices) bit-exact;
K, M, F values within 1e-12 relative -- per scalar row of K the largest deviation is at
most 1e-12 x the largest |entry| of that row (penalty entries must equal 1e20 exactly);
M and F within 1e-12 x their largest |entry|.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import fem_taichi_gb300 as F
from oracle import c_oracle as C
from oracle import fem_oracle as O
from tests.fixtures import STEEL, mesh2_physics

pytestmark = pytest.mark.gpu

REL = 1e-12


def assert_K_close(Kg, Ko, rel=REL):
    assert Kg.shape == Ko.shape
    assert Kg.indptr.dtype == np.int32 and Kg.indices.dtype == np.int32
    assert np.array_equal(Kg.indptr, Ko.indptr), "row pointers differ"
    assert np.array_equal(Kg.indices, Ko.indices), "column indices differ"
    pen = Ko.data >= 1e19
    assert np.array_equal(Kg.data[pen], Ko.data[pen])
    assert np.all(Kg.data[Kg.data >= 1e19] == 1e20)
    a = np.where(pen, 0.0, Kg.data)
    b = np.where(pen, 0.0, Ko.data)
    rows = np.repeat(np.arange(Ko.shape[0]), np.diff(Ko.indptr))
    rmax = np.zeros(Ko.shape[0])
    np.maximum.at(rmax, rows, np.abs(b))
    dev = np.abs(a - b)
    assert np.all(dev <= rel * rmax[rows]), f"max rel dev {np.max(dev / np.maximum(rmax[rows], 1e-300))}"


@pytest.fixture(scope="module")
def c2_oracle():
    P = F.config_mesh("c2")
    bn = P.Nind[P.Bounds[0][0]]
    bc = np.zeros((bn.size, 3))
    Kc, Mc, Fc = C.assemble(P.xyz, P.conn, P.SmNode, P.ReNode, STEEL, (0, 0, 100), bn, bc, nthreads=0)
    return P, Kc, Mc, Fc


def assert_vec_close(x, y, rel=REL):
    s = np.abs(y).max()
    assert np.abs(np.asarray(x) - np.asarray(y)).max() <= rel * s


CASES = {
    "mesh2": lambda: (mesh2_physics(), (0, 0, 100)),
    "c1": lambda: (F.config_mesh("c1"), (0, 0, 100)),
    "twisted_omega": lambda: (F.hex_block(9, 5, 4, size=(9.0, 3.0, 2.0), jitter=0.1, twist_deg=45, seed=7,
                                          fix="xmin", load_face="zmax", load=(1.7, 0, -2.2)), (30.0, -20.0, 80.0)),
    "no_bounds": lambda: (F.hex_block(3, 2, 2, jitter=0.1, seed=9, fix=None), (0, 0, 100)),
    "single_element": lambda: (F.hex_block(1, 1, 1, jitter=0.0, fix=None), (5.0, 0, 0)),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    P, om = CASES[request.param]()
    OM = O.OracleModel(P, STEEL, om)
    return request.param, P, om, OM


ALGOS = ["dd", "fp64"]


@pytest.mark.parametrize("algo", ALGOS)
def test_K_matches_oracle(case, algo):
    name, P, om, OM = case
    M = F.Model(name, P, STEEL, Omegas=om, algo=algo)
    assert_K_close(M.Get_MatrixKL(), OM.Get_MatrixKL())
    assert M.Get_MatrixK is not None


@pytest.mark.parametrize("algo", ALGOS)
def test_M_matches_oracle(case, algo):
    name, P, om, OM = case
    M = F.Model(name, P, STEEL, Omegas=om, algo=algo)
    Mg, Mo = M.Get_MatrixM(), OM.Get_MatrixM()
    assert np.array_equal(Mg.indptr, Mo.indptr) and np.array_equal(Mg.indices, Mo.indices)
    assert_vec_close(Mg.data, Mo.data)


@pytest.mark.parametrize("algo", ALGOS)
def test_F_matches_oracle(case, algo):
    name, P, om, OM = case
    M = F.Model(name, P, STEEL, Omegas=om, algo=algo)
    Fg = M.Get_VectorF()
    assert Fg.shape == (3 * P.Num_Node,)
    assert_vec_close(Fg, OM.Get_VectorF())


@pytest.mark.parametrize("algo", ALGOS)
def test_bsr_layout_equals_csr_and_is_deterministic(algo):
    P = mesh2_physics()
    M = F.Model("2", P, STEEL, algo=algo)
    K1, M1, F1 = M.assemble(k_layout="bsr", m_layout="bsr")
    K2, M2, F2 = M.assemble(k_layout="bsr", m_layout="bsr")
    torch.cuda.synchronize()
    assert torch.equal(K1, K2) and torch.equal(M1, M2) and torch.equal(F1, F2)   # bitwise
    n3 = 3 * P.Num_Node
    Kb = sp.bsr_matrix((K1.cpu().numpy(), P.ReNode, P.SmNode), shape=(n3, n3)).tocsr()
    Kc = M.Get_MatrixKL()
    assert np.array_equal(Kb.indptr, Kc.indptr) and np.array_equal(Kb.indices, Kc.indices)
    assert np.array_equal(Kb.data, Kc.data)
    # repeated getters return identical results (idempotent)
    assert np.array_equal(M.Get_MatrixKL().data, Kc.data)


def test_extra_float_loads_bypass_int_cast():
    P = F.hex_block(4, 4, 2, jitter=0.05, seed=3, fix="zmin", load_face="zmax", load=(0.0, 0.0, -1.0))
    extra = F.face_traction_loads(P, "zmax", (0.0, 0.0, -0.37))
    M = F.Model("t", P, STEEL, extra_loads=extra)
    Fo = O.OracleModel(P, STEEL, (0, 0, 100)).ValF() + extra
    assert_vec_close(M.Get_VectorF(), Fo.reshape(-1))


def test_degenerate_element_with_repeated_corner():
    """A wedge-like element listing one node twice: every block the reference adds
    (both corner copies) must be summed, in both arithmetic variants."""
    xyz = np.random.default_rng(4).random((12, 3)) * 0.2 + np.array(
        [[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)] + [[2, 0, 0], [2, 1, 0], [2, 0, 1], [2, 1, 1]])
    e0 = [3, 2, 0, 1, 7, 6, 4, 5]                      # corner order (+,+,-),(-,+,-),... of the unit cube
    e1 = [9, 3, 1, 8, 11, 7, 5, 11]                     # last corner repeats node 11
    P = F.Physics(np.arange(1, 13), xyz, np.array([e0, e1]).T, [[np.array([0, 1]), [0, 0, 0]]], [])
    OM = O.OracleModel(P, STEEL, (0, 0, 100))
    for algo in ALGOS:
        M = F.Model("d", P, STEEL, algo=algo)
        assert_K_close(M.Get_MatrixKL(), OM.Get_MatrixKL())
        assert_vec_close(M.Get_MatrixM().data, OM.Get_MatrixM().data)


def test_many_incident_entries_and_unaligned_slot_map():
    """Nodes with more than 8 incident (element, corner) entries -- every element listed twice,
    so interior nodes have 16 -- take the FP64 gather's later chunks of 8 entries; both
    arithmetic variants against the oracle.  A slot_map that does not start on an 8-byte
    boundary (an offset view a C-ABI caller may pass) takes the byte-wise loads and gives the
    same K, M, F bit for bit, on the device and through the host pipeline."""
    P1 = F.hex_block(5, 4, 3, jitter=0.1, seed=11, fix="zmin")
    P = F.Physics(P1.Node[0], P1.xyz, np.concatenate([P1.conn, P1.conn]).T, P1.Bounds, [])
    assert np.diff(np.asarray(P.ne_ptr)).max() > 8
    OM = O.OracleModel(P, STEEL, (0, 0, 100))
    for algo in ALGOS:
        M = F.Model("dup", P, STEEL, algo=algo)
        assert_K_close(M.Get_MatrixKL(), OM.Get_MatrixKL())
        assert_vec_close(M.Get_MatrixM().data, OM.Get_MatrixM().data)
        assert_vec_close(M.Get_VectorF(), OM.Get_VectorF())
    M = F.Model("dup", P, STEEL, algo="fp64")
    Kd, Md, Fd = M.assemble(k_layout="csr", m_layout="csr")
    Kh, Mh, Fh = M.assemble_host(3)
    sm = M.mesh.slot_map
    buf = torch.zeros(sm.numel() + 16, dtype=torch.uint8, device=sm.device)
    buf[3:3 + sm.numel()].copy_(sm)
    saved = M.mesh.c.slot_map
    M.mesh.c.slot_map = buf.data_ptr() + 3
    try:
        Ku, Mu, Fu = M.assemble(k_layout="csr", m_layout="csr")
        Khu, Mhu, Fhu = M.assemble_host(3)
    finally:
        M.mesh.c.slot_map = saved
    torch.cuda.synchronize()
    assert torch.equal(Ku, Kd) and torch.equal(Mu, Md) and torch.equal(Fu, Fd)
    assert np.array_equal(Khu, Kh) and np.array_equal(Mhu, Mh) and np.array_equal(Fhu, Fh)
    assert np.array_equal(Kh, Kd.cpu().numpy())


@pytest.mark.parametrize("algo", ALGOS)
def test_full_size_c2_against_c_oracle(algo, c2_oracle):
    """200x200x24 (960,000 elements): the whole BSR K, M and F against the threaded C
    restatement; pattern bit-exact, values at the 1e-12 bar."""
    P, Kc, Mc, Fc = c2_oracle
    M = F.Model("c2", P, STEEL, algo=algo)
    Kd, Md, Fd = M.assemble(k_layout="bsr", m_layout="bsr")
    Kg = Kd.cpu().numpy()
    pen = Kc >= 1e19
    assert np.array_equal(Kg[pen], Kc[pen])
    # per block-row scale
    rows = np.repeat(np.arange(P.Num_Node), np.diff(P.SmNode))
    blk = np.abs(np.where(pen, 0, Kc)).reshape(-1, 9).max(axis=1)
    rmax = np.zeros(P.Num_Node)
    np.maximum.at(rmax, rows, blk)
    dev = np.abs(np.where(pen, 0, Kg - Kc)).reshape(-1, 9).max(axis=1)
    assert np.all(dev <= REL * rmax[rows])
    assert_vec_close(Md.cpu().numpy(), Mc)
    assert_vec_close(Fd.cpu().numpy(), Fc)
    # total mass = rho * volume (sum_g detJ), a size-independent invariant
    assert abs(Md.sum().item() - STEEL['DE'] * 200 * 200 * 24) <= 1e-10 * STEEL['DE'] * 200 * 200 * 24


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("order", ["natural", "shuffled"])
def test_host_pipeline_equals_device_assembly(algo, order):
    """fem_assemble_host (parts of block rows, copies overlapping later parts) returns the
    device assembly bit for bit, for any number of parts, into page-locked or pageable
    host memory."""
    import ctypes
    from fem_taichi_gb300 import _lib
    from fem_taichi_gb300.model import _dptr, _stream
    P = F.hex_block(13, 9, 5, jitter=0.1, seed=6, fix="zmin")
    if order == "shuffled":
        perm = np.random.default_rng(2).permutation(P.Num_Elem)
        P = F.Physics(P.Node[0], P.xyz, P.conn[perm].T, P.Bounds, [])
    M = F.Model("h", P, STEEL, algo=algo)
    Kd, Md, Fd = M.assemble(k_layout="csr", m_layout="csr")
    torch.cuda.synchronize()
    Kd, Md, Fd = Kd.cpu().numpy(), Md.cpu().numpy(), Fd.cpu().numpy().reshape(-1)
    for parts in (1, 3, 8, 50):
        Kh, Mh, Fh = M.assemble_host(parts)
        assert np.array_equal(Kh, Kd) and np.array_equal(Mh, Md) and np.array_equal(Fh, Fd)
    # pageable destination (plain numpy arrays)
    L = _lib.load()
    nnzb = M.mesh.nnzb
    Kt = torch.empty(9 * nnzb, dtype=torch.float64, device="cuda")
    Mt = torch.empty(3 * nnzb, dtype=torch.float64, device="cuda")
    Ft = torch.empty(3 * P.Num_Node, dtype=torch.float64, device="cuda")
    Kp, Mp, Fp = np.full(9 * nnzb, np.nan), np.full(3 * nnzb, np.nan), np.full(3 * P.Num_Node, np.nan)
    o = _lib.FemAssemblyOut(_lib.LAYOUT_CSR, _lib.LAYOUT_CSR, Kt.data_ptr(), Mt.data_ptr(), Ft.data_ptr(),
                            M.fixed.data_ptr(), M.loads.data_ptr(), _lib.ALGO_DD if algo == "dd" else _lib.ALGO_FP64)
    rs, es, bs = M.pipeline_plan(4)
    ws = M.workspace()
    _lib.check(L.fem_assemble_host(ctypes.byref(M.mesh.c), ctypes.byref(M.mat), ctypes.byref(o), rs.ctypes.data,
                                   es.ctypes.data, bs.ctypes.data, 4, Kp.ctypes.data, Mp.ctypes.data, Fp.ctypes.data,
                                   _dptr(ws), ws.numel(), _stream(M.device)))
    torch.cuda.synchronize()
    assert np.array_equal(Kp, Kd) and np.array_equal(Mp, Md) and np.array_equal(Fp, Fd)


@pytest.mark.parametrize("algo", ALGOS)
def test_staged_host_pipeline_equals_device_assembly(algo):
    """fem_assemble_host_staged (M over the link as one value per block, written in the
    reference CSR order on the host part by part) returns the device assembly's CSR K, M, F bit
    for bit, into pageable numpy buffers, for 1 and 5 parts."""
    import ctypes
    from fem_taichi_gb300 import _lib
    from fem_taichi_gb300.model import _dptr, _stream
    P = F.hex_block(11, 7, 6, jitter=0.1, seed=9, fix="zmin", load_face="zmax", load=(1.0, 0, -2.0))
    M = F.Model("s", P, STEEL, algo=algo)
    Kd, Md, Fd = M.assemble(k_layout="csr", m_layout="csr")
    torch.cuda.synchronize()
    Kd, Md, Fd = Kd.cpu().numpy(), Md.cpu().numpy(), Fd.cpu().numpy().reshape(-1)
    L = _lib.load()
    nnzb = M.mesh.nnzb
    ind = np.ascontiguousarray(P.SmNode, dtype=np.int32)
    for parts in (1, 5):
        Kt = torch.empty(9 * nnzb, dtype=torch.float64, device="cuda")
        Mt = torch.empty(3 * nnzb, dtype=torch.float64, device="cuda")
        Ft = torch.empty(3 * P.Num_Node, dtype=torch.float64, device="cuda")
        Kp, Mp, Fp = np.full(9 * nnzb, np.nan), np.full(3 * nnzb, np.nan), np.full(3 * P.Num_Node, np.nan)
        stage = np.full(nnzb, np.nan)
        o = _lib.FemAssemblyOut(_lib.LAYOUT_CSR, _lib.LAYOUT_CSR, Kt.data_ptr(), Mt.data_ptr(), Ft.data_ptr(),
                                M.fixed.data_ptr(), M.loads.data_ptr(),
                                _lib.ALGO_DD if algo == "dd" else _lib.ALGO_FP64)
        rs, es, bs = M.pipeline_plan(parts)
        ws = M.workspace()
        _lib.check(L.fem_assemble_host_staged(ctypes.byref(M.mesh.c), ctypes.byref(M.mat), ctypes.byref(o),
                                              rs.ctypes.data, es.ctypes.data, bs.ctypes.data, parts, ind.ctypes.data,
                                              Kp.ctypes.data, Mp.ctypes.data, Fp.ctypes.data, stage.ctypes.data,
                                              _dptr(ws), ws.numel(), _stream(M.device)), "fem_assemble_host_staged")
        torch.cuda.synchronize()
        assert np.array_equal(Kp, Kd) and np.array_equal(Mp, Md) and np.array_equal(Fp, Fd), parts


def test_host_pipeline_rejects_bad_plan():
    import ctypes
    from fem_taichi_gb300 import _lib
    from fem_taichi_gb300.model import _dptr, _stream
    P = F.hex_block(3, 3, 2)
    M = F.Model("b", P, STEEL)
    rs, es, bs = (a.copy() for a in M.pipeline_plan(2))
    rs[1], rs[2] = rs[2], rs[1]          # not monotone
    Kt = torch.empty(9 * M.mesh.nnzb, dtype=torch.float64, device="cuda")
    o = _lib.FemAssemblyOut(_lib.LAYOUT_CSR, _lib.LAYOUT_CSR, Kt.data_ptr(), None, None, None, None, _lib.ALGO_DD)
    Kh = np.zeros(9 * M.mesh.nnzb)
    ws = M.workspace()
    L = _lib.load()
    rc = L.fem_assemble_host(ctypes.byref(M.mesh.c), ctypes.byref(M.mat), ctypes.byref(o), rs.ctypes.data,
                             es.ctypes.data, bs.ctypes.data, 2, Kh.ctypes.data, None, None, _dptr(ws), ws.numel(),
                             _stream(M.device))
    assert rc == _lib.FEM_ERR_INVALID
