"""Shared test inputs: the reference's Mesh/2.cdb fixture (committed as tests/golden/mesh2.npz)
and small seeded synthetic blocks."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STEEL = {'DE': 7.8e-9, 'EX': 200000.0, 'PO': 0.3}


def mesh2_arrays():
    d = np.load(os.path.join(GOLDEN, "mesh2.npz"))
    return {k: d[k] for k in d.files}


def mesh2_physics():
    from fem_taichi_gb300.mesh import Physics
    d = mesh2_arrays()
    bounds = [[d["bot_in"].astype(np.int64) - 1, [0, 0, 0]], [d["bot_out"].astype(np.int64) - 1, [0, 0, 0]]]
    return Physics(d["node_ids"], d["xyz"], d["elem"].astype(np.int64), bounds, [], name="2")


def golden():
    d = np.load(os.path.join(GOLDEN, "mesh2_golden.npz"))
    return {k: d[k] for k in d.files}
