"""Mesh and boundary data in the layout of the reference's ``Read`` object.

``Physics`` carries the attributes ``Model`` and ``Post`` consume (READ_physics.py:42-61):

    Node     (6, N) float64   row 0 = 1-based node id, rows 3..5 = x, y, z
    Elem     (k, E) int64     last 8 rows = node ids - 1, in the reference's corner order
    Nind     (Num_MaxN,)      node id - 1  ->  node index
    SmNode   (N+1,) int32     block-row pointer of the K pattern
    ReNode   (nnzb,) int32    block column indices, ascending per row, self included
    CoNode   (N,)             blocks per row
    CoElem   (N,)             elements per node
    Bounds   list of [ids - 1, [c0, c1, c2]]   (code != -1 => DOF fixed)
    Forces   list of [ids - 1, [fx, fy, fz]]   (values are int-cast by Model, as the reference does)

The pattern and the node->element incidence are built by the native topology code in
``libfemgb.so``; ``conn`` (E, 8) int32 node indices and the incidence arrays are kept on
the object for ``Model`` / ``Post``.

Corner order of a hexahedron (FEM_model_bsr.py:371-382), natural-coordinate signs:
    0:(+,+,-) 1:(-,+,-) 2:(-,-,-) 3:(+,-,-) 4:(+,+,+) 5:(-,+,+) 6:(-,-,+) 7:(+,-,+)
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import _lib

CORNER_SIGNS = np.array([[1, 1, -1], [-1, 1, -1], [-1, -1, -1], [1, -1, -1],
                         [1, 1, 1], [-1, 1, 1], [-1, -1, 1], [1, -1, 1]], dtype=np.int64)

STEEL = {'DE': 7.8e-9, 'EX': 200000.0, 'PO': 0.3}


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def build_pattern(conn: np.ndarray, n_node: int):
    """(indptr, indices) of the block pattern via the native topology code."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    L = _lib.load()
    indptr = np.empty(n_node + 1, dtype=np.int32)
    nnzb = ctypes.c_int64(0)
    _lib.check(L.fem_pattern_count(n_node, conn.shape[0], _ptr(conn), _ptr(indptr), ctypes.byref(nnzb)),
               "fem_pattern_count")
    indices = np.empty(nnzb.value, dtype=np.int32)
    _lib.check(L.fem_pattern_fill(n_node, conn.shape[0], _ptr(conn), _ptr(indptr), _ptr(indices)),
               "fem_pattern_fill")
    return indptr, indices


def build_gather_map(conn, indptr, indices, ne_ptr, ne_list, n_node: int):
    """(ne_inv, slot_map) element-to-block map of the gather via the native topology code."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    L = _lib.load()
    E = conn.shape[0]
    ne_inv = np.empty(8 * E, dtype=np.int32)
    slot_map = np.empty(64 * E, dtype=np.uint8)
    _lib.check(L.fem_gather_map(n_node, E, _ptr(conn), _ptr(np.ascontiguousarray(indptr, dtype=np.int32)),
                                _ptr(np.ascontiguousarray(indices, dtype=np.int32)),
                                _ptr(np.ascontiguousarray(ne_ptr, dtype=np.int32)),
                                _ptr(np.ascontiguousarray(ne_list, dtype=np.int32)), _ptr(ne_inv), _ptr(slot_map)),
               "fem_gather_map")
    return ne_inv, slot_map


def build_incidence(conn: np.ndarray, n_node: int):
    """(ne_ptr, ne_list, co_elem) via the native topology code."""
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    L = _lib.load()
    ne_ptr = np.empty(n_node + 1, dtype=np.int32)
    ne_list = np.empty(8 * conn.shape[0], dtype=np.int32)
    co_elem = np.empty(n_node, dtype=np.int32)
    _lib.check(L.fem_incidence_build(n_node, conn.shape[0], _ptr(conn), _ptr(ne_ptr), _ptr(ne_list),
                                     _ptr(co_elem)), "fem_incidence_build")
    return ne_ptr, ne_list, co_elem


def build_topology_gpu(conn, n_node: int, device="cuda"):
    """Incidence, block pattern and gather map built on the device (fem_topology_*_gpu), the
    same arrays as build_incidence + build_pattern + build_gather_map.  Returns a dict of
    device int32 / uint8 tensors: ne_ptr, ne_list, co_elem, indptr, indices, ne_inv, slot_map."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("build_topology_gpu needs a CUDA device")
    d = torch.device(device)
    c = torch.as_tensor(np.ascontiguousarray(conn, dtype=np.int32)).to(d)
    E = int(c.shape[0])
    L = _lib.load()
    st = ctypes.c_void_p(torch.cuda.current_stream(d).cuda_stream)
    ws = torch.empty(max(int(L.fem_topology_workspace_bytes(n_node, E)), 16), dtype=torch.uint8, device=d)
    t = {"ne_ptr": torch.empty(n_node + 1, dtype=torch.int32, device=d),
         "ne_list": torch.empty(max(8 * E, 1), dtype=torch.int32, device=d),
         "co_elem": torch.empty(max(n_node, 1), dtype=torch.int32, device=d),
         "indptr": torch.empty(n_node + 1, dtype=torch.int32, device=d)}
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    nnzb = ctypes.c_int64(0)
    _lib.check(L.fem_topology_count_gpu(n_node, E, p(c), p(t["ne_ptr"]), p(t["ne_list"]), p(t["co_elem"]),
                                        p(t["indptr"]), ctypes.byref(nnzb), p(ws), ws.numel(), st),
               "fem_topology_count_gpu")
    t["indices"] = torch.empty(max(nnzb.value, 1), dtype=torch.int32, device=d)
    t["ne_inv"] = torch.empty(max(8 * E, 1), dtype=torch.int32, device=d)
    t["slot_map"] = torch.empty(max(64 * E, 1), dtype=torch.uint8, device=d)
    _lib.check(L.fem_topology_fill_gpu(n_node, E, p(c), p(t["ne_ptr"]), p(t["ne_list"]), p(t["indptr"]),
                                       p(t["indices"]), p(t["ne_inv"]), p(t["slot_map"]), p(ws), ws.numel(), st),
               "fem_topology_fill_gpu")
    t["indices"] = t["indices"][:nnzb.value]
    t["ne_list"] = t["ne_list"][:8 * E]
    t["ne_inv"] = t["ne_inv"][:8 * E]
    t["slot_map"] = t["slot_map"][:64 * E]
    t["co_elem"] = t["co_elem"][:n_node]
    return t


class Physics:
    """Reference ``Read`` duck type built from in-memory arrays.  topology='gpu' builds the
    pattern, incidence and gather map on the device (same arrays, host copies kept)."""

    def __init__(self, node_ids, xyz, elem_ids, Bounds=None, Forces=None, name="mesh", topology="host"):
        if topology not in ("host", "gpu"):
            raise ValueError("topology must be 'host' or 'gpu'")
        self.topology = topology
        node_ids = np.asarray(node_ids, dtype=np.int64)
        xyz = np.asarray(xyz, dtype=np.float64)
        N = node_ids.size
        self.name = name
        self.Node = np.zeros((6, N), dtype=np.float64)
        self.Node[0] = node_ids
        self.Node[3:] = xyz.T
        self.Elem = np.asarray(elem_ids, dtype=np.int64)          # (k, E): ids - 1
        self.Bounds = list(Bounds or [])
        self.Forces = list(Forces or [])
        self.pre_process()

    def pre_process(self):
        """READ_physics.py:42-61, with the pattern built natively."""
        self.Num_Node = self.Node.shape[-1]
        self.Num_Elem = self.Elem.shape[-1]
        self.Num_MaxN = int(self.Node[0, :].max())
        self.Nind = np.zeros((self.Num_MaxN,), dtype=np.int64)
        self.Nind[self.Node[0, :].astype(np.int64) - 1] = np.arange(self.Num_Node, dtype=np.int64)
        self.conn = np.ascontiguousarray(self.Nind[self.Elem[-8:]].T, dtype=np.int32)   # (E, 8)
        if getattr(self, "topology", "host") == "gpu":
            t = build_topology_gpu(self.conn, self.Num_Node)
            h = {k: v.cpu().numpy() for k, v in t.items()}
            self.SmNode, self.ReNode = h["indptr"], h["indices"]
            self.ne_ptr, self.ne_list, self.CoElem = h["ne_ptr"], h["ne_list"], h["co_elem"]
            self.ne_inv, self.slot_map = h["ne_inv"], h["slot_map"]
        else:
            self.SmNode, self.ReNode = build_pattern(self.conn, self.Num_Node)
            self.ne_ptr, self.ne_list, self.CoElem = build_incidence(self.conn, self.Num_Node)
            self.ne_inv, self.slot_map = build_gather_map(self.conn, self.SmNode, self.ReNode, self.ne_ptr,
                                                          self.ne_list, self.Num_Node)
        self.CoNode = np.diff(self.SmNode)

    @property
    def xyz(self) -> np.ndarray:
        return np.ascontiguousarray(self.Node[-3:].T)

    def node_index(self, ids_minus_one) -> np.ndarray:
        return self.Nind[np.asarray(ids_minus_one, dtype=np.int64)]


# ---------------------------------------------------------------------------------------
# Synthetic structured hexahedral blocks (seeded)
# ---------------------------------------------------------------------------------------
def block_arrays(nx, ny, nz, size=None, jitter=0.0, seed=0, twist_deg=0.0, origin=(0.0, 0.0, 0.0),
                 center_yz=False, fix="zmin", load_face=None, load=(0.0, 0.0, 0.0)):
    """Arrays of a structured nx*ny*nz hex block with seeded interior-node jitter (numpy only).

    size: (Lx, Ly, Lz) extents (default one unit per element).  jitter: amplitude as a
    fraction of the element size in each direction, applied to nodes strictly inside the
    block so that the boundary faces stay planar.  twist_deg: linear twist about the x
    axis (through the y-z centre) from 0 at x = 0 to twist_deg at x = Lx.  fix / load_face:
    face name ('xmin','xmax','ymin','ymax','zmin','zmax' or None) whose nodes go to Bounds
    (all DOFs) / Forces (value ``load``).  Node ids are 1-based, x fastest.

    Returns a dict: ids (N,), xyz (N, 3), elem (8, E) node ids - 1, bounds, forces (the
    reference's [ids - 1, [3 values]] groups), grid_index (ix, iy, iz), h.
    """
    size = size or (float(nx), float(ny), float(nz))
    h = np.array([size[0] / nx, size[1] / ny, size[2] / nz])
    ix, iy, iz = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    ix, iy, iz = (a.transpose(2, 1, 0).ravel() for a in (ix, iy, iz))          # x fastest
    xyz = np.stack([ix * h[0], iy * h[1], iz * h[2]], axis=1).astype(np.float64)
    if jitter:
        rng = np.random.default_rng(seed)
        inner = (ix > 0) & (ix < nx) & (iy > 0) & (iy < ny) & (iz > 0) & (iz < nz)
        d = rng.uniform(-1.0, 1.0, size=(int(inner.sum()), 3)) * (jitter * h)
        xyz[inner] += d
    if center_yz:
        xyz[:, 1] -= size[1] / 2
        xyz[:, 2] -= size[2] / 2
    if twist_deg:
        th = np.deg2rad(twist_deg) * (xyz[:, 0] / size[0])
        c, s = np.cos(th), np.sin(th)
        y, z = xyz[:, 1].copy(), xyz[:, 2].copy()
        xyz[:, 1] = c * y - s * z
        xyz[:, 2] = s * y + c * z
    xyz += np.asarray(origin, dtype=np.float64)
    ids = np.arange(1, xyz.shape[0] + 1, dtype=np.int64)
    ex, ey, ez = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ex, ey, ez = (a.transpose(2, 1, 0).ravel() for a in (ex, ey, ez))
    corner = CORNER_SIGNS > 0
    nid = ((ex[:, None] + corner[None, :, 0]) + (nx + 1) * ((ey[:, None] + corner[None, :, 1])
           + (ny + 1) * (ez[:, None] + corner[None, :, 2])))                 # (E, 8) 0-based index
    elem = nid.T.astype(np.int64)                                            # ids - 1 == index

    def face(name_):
        if name_ is None:
            return np.zeros(0, dtype=np.int64)
        sel = {"xmin": ix == 0, "xmax": ix == nx, "ymin": iy == 0, "ymax": iy == ny,
               "zmin": iz == 0, "zmax": iz == nz}[name_]
        return np.nonzero(sel)[0].astype(np.int64)

    bounds = [[face(fix), [0, 0, 0]]] if fix else []
    forces = [[face(load_face), list(load)]] if load_face else []
    return {"ids": ids, "xyz": xyz, "elem": elem, "bounds": bounds, "forces": forces,
            "grid_index": (ix, iy, iz), "h": h}


def hex_block(nx, ny, nz, size=None, jitter=0.0, seed=0, twist_deg=0.0, origin=(0.0, 0.0, 0.0),
              center_yz=False, fix="zmin", load_face=None, load=(0.0, 0.0, 0.0), name="block"):
    """Structured nx*ny*nz hex block (see ``block_arrays``) as a Physics object."""
    b = block_arrays(nx, ny, nz, size=size, jitter=jitter, seed=seed, twist_deg=twist_deg, origin=origin,
                     center_yz=center_yz, fix=fix, load_face=load_face, load=load)
    P = Physics(b["ids"], b["xyz"], b["elem"], b["bounds"], b["forces"], name=name)
    P.grid = (nx, ny, nz)
    P.grid_index = b["grid_index"]
    P.h = b["h"]
    return P


def face_traction_loads(P: Physics, face: str, traction) -> np.ndarray:
    """Consistent nodal loads (N, 3) of a uniform traction on a planar structured face.

    Each bilinear quad of the face contributes traction * area / 4 to its corners.
    """
    nx, ny, nz = P.grid
    ix, iy, iz = P.grid_index
    xyz = P.xyz
    t = np.asarray(traction, dtype=np.float64)
    F = np.zeros((P.Num_Node, 3))
    if face not in ("zmin", "zmax"):
        raise ValueError("only z faces are supported")
    k = 0 if face == "zmin" else nz
    idx = lambda i, j: i + (nx + 1) * (j + (ny + 1) * k)  # noqa: E731
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    i, j = i.ravel(), j.ravel()
    c = [idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)]
    p = [xyz[q] for q in c]
    area = 0.5 * np.linalg.norm(np.cross(p[2] - p[0], p[3] - p[1]), axis=1)
    for q in c:
        np.add.at(F, q, (area / 4.0)[:, None] * t[None, :])
    return F


CONFIGS = {
    # 40x40x12, h = 1 mm, jitter +-0.1 mm, z = 0 fixed, z = max nodes carry (0, 0, -1) N
    "c1": dict(nx=40, ny=40, nz=12, size=(40.0, 40.0, 12.0), jitter=0.1, seed=1, fix="zmin",
               load_face="zmax", load=(0, 0, -1)),
    # 200x200x24, jitter +-0.1 h, z = 0 fixed
    "c2": dict(nx=200, ny=200, nz=24, size=(200.0, 200.0, 24.0), jitter=0.1, seed=2, fix="zmin"),
    # profiling-size member of the c2 family (100x100x24, 240,000 elements)
    "c2s": dict(nx=100, ny=100, nz=24, size=(100.0, 100.0, 24.0), jitter=0.1, seed=2, fix="zmin"),
    # 100x100x20 stretched 4:1 in z, jitter +-0.1 h, bottom fixed, top traction (host loads)
    "c3": dict(nx=100, ny=100, nz=20, size=(100.0, 100.0, 80.0), jitter=0.1, seed=3, fix="zmin"),
    # evaluation block of the learned-preconditioner study
    "c4": dict(nx=160, ny=160, nz=20, size=(160.0, 160.0, 20.0), jitter=0.1, seed=4, fix="zmin"),
    # twisted slab 1200x120x15 over 1000x60x8 mm, root (x = 500) fixed
    "c5": dict(nx=1200, ny=120, nz=15, size=(1000.0, 60.0, 8.0), jitter=0.05, seed=5, twist_deg=60.0,
               center_yz=True, origin=(500.0, 0.0, 0.0), fix="xmin"),
}


def config_mesh(name: str, **override) -> Physics:
    kw = dict(CONFIGS[name])
    kw.update(override)
    return hex_block(name=name, **kw)


# ---------------------------------------------------------------------------------------
# ANSYS .cdb / node-list .lis reader (READ_physics.py:64-154)
# ---------------------------------------------------------------------------------------
def read_cdb(path: str):
    """Fixed-width NBLOCK (3i9,6e20.13) / EBLOCK (19i8) parser.

    Returns (node_ids, xyz, elem) with elem = (18, E) int64 holding the non-blank EBLOCK
    fields minus one, as READ_physics.py:85-96 produces (last 8 rows = corner ids - 1).
    """
    with open(path, "r", errors="replace") as f:
        lines = f.read().splitlines()
    i = next(k for k, s in enumerate(lines) if "NBLOCK" in s) + 2
    ids, xyz = [], []
    while i < len(lines) and not lines[i].startswith("N,R5"):
        s = lines[i]
        if s.strip() == "" or s.strip() == "-1":
            break
        ids.append(int(s[0:9]))
        vals = [float(s[27 + 20 * k: 47 + 20 * k]) for k in range(3)]
        xyz.append(vals)
        i += 1
    j = next(k for k, s in enumerate(lines) if "EBLOCK" in s) + 2
    rows = []
    while j < len(lines) and lines[j].strip() != "-1":
        s = lines[j]
        fields = [s[8 * k: 8 * k + 8] for k in range((len(s) + 7) // 8)]
        toks = [int(x) for x in fields if x.strip() != ""]
        rows.append(toks)
        j += 1
    width = max(len(r) for r in rows)
    elem = np.array([r for r in rows if len(r) == width], dtype=np.int64)
    return np.array(ids, dtype=np.int64), np.array(xyz, dtype=np.float64), elem.T - 1


def read_lis(path: str) -> np.ndarray:
    """Node ids of an ANSYS node-list file (READ_physics.py:106-114): the first non-blank
    line is a header, lines naming NAME/NODE/LIST are dropped, every other token is an id."""
    with open(path, "r", errors="replace") as f:
        lines = [s for s in f.read().splitlines() if s.strip() != ""]
    out = []
    for s in lines[1:]:
        if re.search("NAME|NODE|LIST", s):
            continue
        out.extend(int(t) for t in s.split())
    return np.array(out, dtype=np.int64)


class Read(Physics):
    """Drop-in for ``READ_physics.Read`` (READ_physics.py:7-154)."""

    def __init__(self, name, bounds_file=("bot", "lis"), forces_file=("top", "lis"), mesh_path="Mesh",
                 bounds_path="Boundary", forces_path="Boundary"):
        self.name = str(name)
        cdb = os.path.join(mesh_path, self.name + ".cdb")
        if os.path.exists(cdb):
            ids, xyz, elem = read_cdb(cdb)
        else:
            node = np.loadtxt(os.path.join(mesh_path, self.name + "_node.txt"), skiprows=1)
            el = np.loadtxt(os.path.join(mesh_path, self.name + "_element.txt"), skiprows=1, dtype=np.int64)
            ids, xyz, elem = node[:, 0].astype(np.int64), node[:, -3:], el.T - 1
        bounds = [[read_lis(f) - 1, [0, 0, 0]] for f in self._files(bounds_path, bounds_file)]
        forces = [[read_lis(f) - 1, [0, 0, 0]] for f in self._files(forces_path, forces_file)]
        Physics.__init__(self, ids, xyz, elem, bounds, forces, name=self.name)

    def _files(self, path, spec):
        prefix, ext = spec
        if not os.path.isdir(path):
            return []
        out = []
        for fn in sorted(os.listdir(path)):
            full = os.path.join(path, fn)
            if os.path.isfile(full) and os.path.splitext(fn)[1][1:] in ext and self.name + "_" + prefix in full:
                out.append(full)
        return out
