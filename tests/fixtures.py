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


# ---------------------------------------------------------------------------------------
# Reference-executed fixtures (tests/golden/refexec_*.npz, made by make_refexec.py): the
# reference's own FEM_model_csr / FEM_model_bsr / POST_process code run on these inputs.
# ---------------------------------------------------------------------------------------
REFEXEC_SMALL = ("block_twist", "block_partial", "block_nobc", "mesh2_slice", "mesh2_isolated")


def refexec(name):
    d = np.load(os.path.join(GOLDEN, "refexec_%s.npz" % name))
    return {k: d[k] for k in d.files}


def _groups(ids, ptr, vals):
    return [[ids[ptr[g]:ptr[g + 1]], list(vals[g])] for g in range(len(ptr) - 1)]


def refexec_materials(d):
    de, ex, po = (float(x) for x in d["materials"])
    return {'DE': de, 'EX': ex, 'PO': po}, tuple(float(x) for x in d["omegas"])


def refexec_physics(d, topology="host"):
    """The fixture's inputs as a Physics object (pattern built by this package)."""
    from fem_taichi_gb300.mesh import Physics
    bounds = _groups(d["bounds_ids"], d["bounds_ptr"], d["bounds_codes"])
    forces = _groups(d["forces_ids"], d["forces_ptr"], d["forces_vals"])
    return Physics(d["node_ids"], d["xyz"], d["elem"], bounds, forces, name="fixture", topology=topology)


def refexec_csr(d, prefix, indices=None, indptr=None):
    import scipy.sparse as sp
    n = 3 * d["node_ids"].size
    ind = d[indices or prefix + "_indices"]
    ptr = d[indptr or prefix + "_indptr"]
    return sp.csr_matrix((d[prefix + "_data"], ind, ptr), shape=(n, n))


def probe_vector(n):
    """Deterministic vector in [-0.5, 0.5) by integer hashing (the one make_refexec.py uses)."""
    i = np.arange(n, dtype=np.uint64)
    h = (i * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(1 << 32)
    return h.astype(np.float64) / float(1 << 32) - 0.5
