"""Native pattern / incidence (host code of libfemgb.so) against the reference's scipy
SpGEMM construction (READ_physics.py:42-61): bit-exact, including edge cases."""
import ctypes

import numpy as np
import pytest

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.mesh import build_incidence, build_pattern
from oracle import fem_oracle as O
from tests.fixtures import mesh2_physics


def _check(P):
    T = O.pre_process(P.Node, P.Elem)
    assert np.array_equal(T["SmNode"], P.SmNode)
    assert np.array_equal(T["ReNode"], P.ReNode)
    assert np.array_equal(T["CoNode"], P.CoNode)
    assert np.array_equal(T["CoElem"], P.CoElem)
    assert np.array_equal(T["Nind"], P.Nind)


def test_mesh2_pattern():
    _check(mesh2_physics())


@pytest.mark.parametrize("cfg", ["c1"])
def test_config_pattern(cfg):
    _check(F.config_mesh(cfg))


def test_twisted_and_random_order():
    P = F.hex_block(7, 3, 2, jitter=0.05, twist_deg=30, seed=2)
    _check(P)
    # shuffled element order and non-contiguous node ids
    rng = np.random.default_rng(5)
    perm = rng.permutation(P.Num_Elem)
    ids = P.Node[0].astype(np.int64) * 3 + 7
    elem = (ids[P.conn[perm]] - 1).T
    Q = F.Physics(ids, P.xyz, elem, [], [])
    _check(Q)


def test_isolated_nodes_and_degenerate_element():
    xyz = np.random.default_rng(0).random((13, 3))
    elem = np.array([[0, 1, 2, 3, 4, 5, 6, 7], [4, 5, 6, 7, 8, 9, 10, 10]]).T   # node 10 repeated
    Q = F.Physics(np.arange(1, 14), xyz, elem, [], [])                           # nodes 11, 12 isolated
    _check(Q)
    assert Q.CoNode[11] == 0 and Q.CoElem[12] == 0
    ne_ptr, ne_list, co = build_incidence(Q.conn, Q.Num_Node)
    assert ne_ptr[11] - ne_ptr[10] == 2 and co[10] == 1          # two corners, one element


def test_incidence_order():
    P = F.hex_block(4, 3, 2, seed=1)
    ptr, lst, co = build_incidence(P.conn, P.Num_Node)
    for i in range(P.Num_Node):
        ent = lst[ptr[i]:ptr[i + 1]]
        assert np.all(np.diff(ent) > 0)
        assert np.all(P.conn[ent >> 3, ent & 7] == i)
    assert ptr[-1] == 8 * P.Num_Elem


def test_empty_mesh():
    ip, ind = build_pattern(np.zeros((0, 8), np.int32), 3)
    assert np.array_equal(ip, [0, 0, 0, 0]) and ind.size == 0


def test_out_of_range_connectivity_is_rejected():
    conn = np.zeros((1, 8), np.int32)
    conn[0, 3] = 9
    with pytest.raises(_lib.FemError) as ei:
        build_pattern(conn, 4)
    assert ei.value.code == _lib.FEM_ERR_INVALID
    conn[0, 3] = -1
    with pytest.raises(_lib.FemError):
        build_incidence(conn, 4)


def test_gather_map_matches_search():
    """ne_inv inverts ne_list; slot_map[8k+b] is the position of corner b's node in the row of
    the entry's node (the reference's linear search, FEM_model_bsr.py:171-175)."""
    P = mesh2_physics()
    k = np.arange(P.ne_list.size)
    assert np.array_equal(P.ne_inv[P.ne_list], k)
    ent = P.ne_list
    e, a = ent >> 3, ent & 7
    rows = P.conn[e, a]
    for b in range(8):
        cols = P.conn[e, b]
        s = P.slot_map.reshape(-1, 8)[k, b].astype(np.int64)
        assert np.array_equal(P.ReNode[P.SmNode[rows] + s], cols)


def _plan(P, parts):
    L = _lib.load()
    ind = np.ascontiguousarray(P.SmNode, dtype=np.int32)
    nep = np.ascontiguousarray(P.ne_ptr, dtype=np.int32)
    nel = np.ascontiguousarray(P.ne_list, dtype=np.int32)
    rs, es, bs = (np.zeros(parts + 1, dtype=np.int64) for _ in range(3))
    _lib.check(L.fem_pipeline_plan(P.Num_Node, P.Num_Elem, ind.ctypes.data, nep.ctypes.data, nel.ctypes.data,
                                   parts, rs.ctypes.data, es.ctypes.data, bs.ctypes.data))
    return rs, es, bs


@pytest.mark.parametrize("parts", [1, 2, 8, 37])
@pytest.mark.parametrize("order", ["natural", "shuffled"])
def test_pipeline_plan(parts, order):
    """Every row of part q only needs elements below elem_split[q+1]; splits span the mesh
    monotonically; block_split = indptr[row_split]; parts hold about nnzb / parts blocks."""
    P = F.hex_block(9, 7, 5, jitter=0.1, seed=3)
    if order == "shuffled":
        perm = np.random.default_rng(1).permutation(P.Num_Elem)
        P = F.Physics(P.Node[0], P.xyz, P.conn[perm].T, [], [])
    rs, es, bs = _plan(P, parts)
    assert rs[0] == 0 and rs[-1] == P.Num_Node and es[0] == 0 and es[-1] == P.Num_Elem
    assert np.all(np.diff(rs) >= 0) and np.all(np.diff(es) >= 0) and np.all(np.diff(bs) >= 0)
    assert np.array_equal(bs, P.SmNode[rs])
    for q in range(parts):
        for r in range(rs[q], rs[q + 1]):
            inc = P.ne_list[P.ne_ptr[r]:P.ne_ptr[r + 1]] >> 3
            assert inc.size == 0 or inc.max() < es[q + 1]
    nnzb = int(P.SmNode[-1])
    maxrow = int(np.diff(P.SmNode).max())
    assert np.all(np.abs(np.diff(bs) - nnzb / parts) <= maxrow + 1)


def test_pipeline_plan_rejects_bad_parts():
    P = F.hex_block(2, 2, 2)
    with pytest.raises(_lib.FemError):
        _plan(P, 0)


def test_rsoa4_row_pointers():
    """Padded row-SoA row pointers: every row rounded up to a multiple of 4 blocks."""
    P = F.hex_block(5, 4, 3, jitter=0.1, seed=1)
    ind = np.ascontiguousarray(P.SmNode, dtype=np.int32)
    ind4 = np.zeros_like(ind)
    _lib.check(_lib.load().fem_rsoa4_indptr(P.Num_Node, ind.ctypes.data, ind4.ctypes.data))
    L = np.diff(ind)
    assert np.array_equal(np.diff(ind4), (L + 3) // 4 * 4) and ind4[0] == 0


def test_tecplot_ascii_output(tmp_path):
    """POST_process.py:101-135 layout: header lines, node rows (x y z + fields per step,
    '%10.5e', NaN empty), element rows with 1-based node numbers."""
    from fem_taichi_gb300.post import write_tecplot_ascii
    P = F.hex_block(3, 2, 2, jitter=0.1, seed=1)
    rng = np.random.default_rng(0)
    Fld = rng.standard_normal((P.Num_Node, 4, 2))
    Fld[1, 2, 0] = np.nan
    out = tmp_path / "s.dat"
    write_tecplot_ascii(str(out), "blk", P, Fld, ["u", "v", "w", "s"])
    lines = out.read_text().splitlines()
    assert lines[0] == 'TITLE = "blk.data"'
    assert lines[1] == 'VARIABLES = "X [ m ]","Y [ m ]","Z [m]"' + "".join(
        f'," {n}{s}"' for s in (1, 2) for n in "uvws")
    assert lines[2] == f"ZONE  I={P.Num_Node}, J={P.Num_Elem}, F=FEPOINT, ET=BRICK"
    rows = lines[3:3 + P.Num_Node]
    assert rows[1].split(" ")[3 + 2] == ""            # NaN written empty
    vals = np.array([float(x) for x in rows[0].split(" ")])
    ref = np.concatenate([P.xyz[0], Fld[0].T.reshape(-1)])
    assert np.allclose(vals, ref, rtol=1e-5)
    conn = np.array([[int(x) for x in r.split(" ")] for r in lines[3 + P.Num_Node:]])
    assert np.array_equal(conn, P.conn + 1)


def test_tecplot_ascii_rows_and_nan_fields(tmp_path):
    """Node rows: x y z then every field of every step, '%10.5e' each, space separated, NaN
    as an empty field (POST_process.py:101-135)."""
    from fem_taichi_gb300.post import write_tecplot_ascii
    P = F.hex_block(3, 2, 2, jitter=0.1, seed=1, fix="zmin")
    N = P.Num_Node
    Fld = np.random.default_rng(0).standard_normal((N, 2, 2))
    Fld[1, 0, 1] = np.nan
    Fld[4, :, :] = np.nan
    out = tmp_path / "t.dat"
    write_tecplot_ascii(str(out), "t", P, Fld, ["a", "b"])
    lines = out.read_text().splitlines()
    body = lines[3:3 + N]
    data = np.concatenate((P.Node[-3:].T, Fld.transpose(0, 2, 1).reshape(N, -1)), axis=-1)
    for i in (0, 1, 4, N - 1):
        want = " ".join("" if np.isnan(v) else "%10.5e" % v for v in data[i])
        assert body[i] == want
    assert len(lines) == 3 + N + P.Num_Elem
