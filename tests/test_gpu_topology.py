"""Device build of the topology (incidence, block pattern, gather map) against the host build:
every array bit-exact (READ_physics.py:42-61 pattern, ascending columns; FEM_model_bsr.py:171-175
slot map)."""
import numpy as np
import pytest

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.mesh import build_topology_gpu
from tests.fixtures import mesh2_physics

pytestmark = pytest.mark.gpu


def _check(P):
    t = {k: v.cpu().numpy() for k, v in build_topology_gpu(P.conn, P.Num_Node).items()}
    assert np.array_equal(t["indptr"], P.SmNode.astype(np.int32))
    assert np.array_equal(t["indices"], P.ReNode.astype(np.int32))
    assert np.array_equal(t["ne_ptr"], P.ne_ptr)
    assert np.array_equal(t["ne_list"], P.ne_list)
    assert np.array_equal(t["co_elem"], P.CoElem.astype(np.int32))
    assert np.array_equal(t["ne_inv"], P.ne_inv)
    assert np.array_equal(t["slot_map"], P.slot_map)


@pytest.mark.parametrize("name", ["mesh2", "c1", "twisted", "c2s"])
def test_device_topology_matches_host(name):
    P = {"mesh2": mesh2_physics, "c1": lambda: F.config_mesh("c1"),
         "twisted": lambda: F.hex_block(7, 5, 3, jitter=0.12, twist_deg=40, seed=4),
         "c2s": lambda: F.config_mesh("c2s")}[name]()
    _check(P)


def test_shuffled_elements_isolated_node_and_repeated_corner():
    Q = F.hex_block(6, 5, 3, jitter=0.1, seed=2)
    perm = np.random.default_rng(8).permutation(Q.Num_Elem)
    conn = Q.conn[perm].copy()
    conn[3, 5] = conn[3, 4]                       # degenerate element (repeated corner)
    ids = Q.Node[0].astype(np.int64) * 2 + 5      # non-contiguous ids
    xyz = np.vstack([Q.xyz, [[9.0, 9.0, 9.0]]])   # one isolated node
    ids = np.concatenate([ids, [ids.max() + 3]])
    P = F.Physics(ids, xyz, (ids[conn] - 1).T, [], [])
    _check(P)
    Pg = F.Physics(ids, xyz, (ids[conn] - 1).T, [], [], topology="gpu")
    assert np.array_equal(Pg.ReNode, P.ReNode) and np.array_equal(Pg.slot_map, P.slot_map)


def test_node_valence_limit_is_reported():
    """129 elements sharing one node exceed the device build's per-row limit: an error, not
    a wrong pattern."""
    rng = np.random.default_rng(0)
    n_node = 2000
    conn = np.zeros((129, 8), dtype=np.int32)
    for e in range(129):
        conn[e, 0] = 0
        conn[e, 1:] = rng.choice(np.arange(1, n_node), size=7, replace=False)
    with pytest.raises(_lib.FemError) as ei:
        build_topology_gpu(conn, n_node)
    assert ei.value.code == _lib.FEM_ERR_INVALID


def test_out_of_range_connectivity_is_rejected():
    conn = np.array([[0, 1, 2, 3, 4, 5, 6, 99]], dtype=np.int32)
    with pytest.raises(_lib.FemError):
        build_topology_gpu(conn, 8)
