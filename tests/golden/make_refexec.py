"""Generates the reference-executed golden fixtures ``tests/golden/refexec_*.npz``.

The reference's own ``FEM_model_csr.py``, ``FEM_model_bsr.py`` and ``POST_process.py``
(tianshao1992/FEM_taichi) are imported unmodified and run on the CPU under the Taichi 0.6.28
stand-in of ``oracle/refexec`` (see ``oracle/refexec/reference_runner.py``); their topology
comes from the reference's own ``Read.pre_process`` (READ_physics.py:42-61).  Each fixture
holds the inputs (nodes, elements, Bounds / Forces groups, materials, Omegas, displacement
fields) next to the reference's outputs, so tests rebuild every case without the reference
tree:

  block_twist     4x3x3 twisted, jittered block; Omegas off-axis; float Forces (int-cast by
                  the reference); K (CSR and BSR variants), M, F, stresses, and the
                  large-displacement KT / KM at a finite displacement field
  block_partial   3x3x2 block, one edge-collapsed (degenerate) element, a Bounds group that
                  fixes only y (codes [-1, 0, -1]), two overlapping Forces groups
  block_nobc      2x2x2 block with no Bounds / Forces files (the reference packs one zero
                  column: node Nind[0] fixed, zero load)
  mesh2_slice     the 250 elements of the reference's Mesh/2.cdb nearest to a fixed node of
                  Boundary/2_bot_in.lis, original (gapped) node ids, both bot files
  mesh2_isolated  40 elements of Mesh/2.cdb plus one node that no element uses: the averaged
                  nodal stress components (the reference divides 0/0 there; its Get_Stress
                  then raises in numpy's eigh, so the six components are stored)
  mesh2_full      all of Mesh/2.cdb (9,468 nodes, 5,856 elements, both bot files): pattern
                  digests, K.v, |K|.|v|, diag K, M.v, F, and the stresses of 2,048 nodes

Usage:  python tests/golden/make_refexec.py REFERENCE_ROOT [case ...]
        python tests/golden/make_refexec.py REFERENCE_ROOT --check block_nobc
(--check re-runs the reference on the named cases and compares with the committed files.)
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

STEEL = {'DE': 7.8e-9, 'EX': 200000.0, 'PO': 0.3}
ALUMINIUM = {'DE': 2.7e-9, 'EX': 70000.0, 'PO': 0.33}


def probe_vector(n: int) -> np.ndarray:
    """Deterministic test vector in [-0.5, 0.5) from integer hashing (exact on any machine)."""
    i = np.arange(n, dtype=np.uint64)
    h = (i * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(1 << 32)
    return h.astype(np.float64) / float(1 << 32) - 0.5


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def pack_groups(groups):
    ids = [np.asarray(g[0], dtype=np.int64) for g in groups]
    ptr = np.zeros(len(groups) + 1, dtype=np.int64)
    ptr[1:] = np.cumsum([len(x) for x in ids])
    vals = np.array([list(map(float, g[1])) for g in groups], dtype=np.float64).reshape(-1, 3)
    return (np.concatenate(ids) if ids else np.zeros(0, np.int64)), ptr, vals


def unpack_groups(ids, ptr, vals):
    """Inverse of pack_groups: [[ids - 1, [c0, c1, c2]], ...] with the stored values."""
    return [[ids[ptr[g]:ptr[g + 1]], list(vals[g])] for g in range(len(ptr) - 1)]


def _block(nx, ny, nz, size, jitter, seed, twist_deg=0.0):
    from fem_taichi_gb300.mesh import CORNER_SIGNS
    h = np.array([size[0] / nx, size[1] / ny, size[2] / nz])
    iz, iy, ix = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()                      # x fastest
    xyz = np.stack([ix * h[0], iy * h[1], iz * h[2]], axis=1).astype(np.float64)
    rng = np.random.default_rng(seed)
    inner = (ix > 0) & (ix < nx) & (iy > 0) & (iy < ny) & (iz > 0) & (iz < nz)
    xyz[inner] += rng.uniform(-1.0, 1.0, size=(int(inner.sum()), 3)) * (jitter * h)
    if twist_deg:
        th = np.deg2rad(twist_deg) * xyz[:, 0] / size[0]
        y, z = xyz[:, 1] - size[1] / 2, xyz[:, 2] - size[2] / 2
        xyz[:, 1], xyz[:, 2] = np.cos(th) * y - np.sin(th) * z, np.sin(th) * y + np.cos(th) * z
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
    c = CORNER_SIGNS > 0
    nid = (ex[:, None] + c[None, :, 0]) + (nx + 1) * ((ey[:, None] + c[None, :, 1]) + (ny + 1) * (ez[:, None] + c[None, :, 2]))
    ids = np.arange(1, xyz.shape[0] + 1, dtype=np.int64)
    face = {"zmin": np.nonzero(iz == 0)[0], "zmax": np.nonzero(iz == nz)[0], "xmax": np.nonzero(ix == nx)[0],
            "ymin": np.nonzero(iy == 0)[0]}
    return ids, xyz, nid.T.astype(np.int64), face


def case_inputs(name):
    """(node_ids, xyz, elem (8,E) ids-1, bounds, forces, materials, omegas, u_stress, u_tangent)."""
    if name == "block_twist":
        ids, xyz, elem, face = _block(4, 3, 3, (4.0, 3.0, 3.0), 0.15, 11, twist_deg=30.0)
        bounds = [[face["zmin"], [0, 0, 0]]]
        forces = [[face["zmax"], [1.7, -2.5, 3.9]]]
        mat, om = ALUMINIUM, (30.0, -40.0, 100.0)
    elif name == "block_partial":
        ids, xyz, elem, face = _block(3, 3, 2, (3.0, 3.0, 2.0), 0.1, 12)
        elem[5, 0] = elem[6, 0]        # element 0: corner 5 collapsed onto corner 6 (edge collapse)
        bounds = [[face["zmin"], [0, 0, 0]], [face["xmax"], [-1, 0, -1]]]
        forces = [[face["ymin"], [0.0, 2.0, -1.0]], [face["zmax"], [-3.0, 0.0, 1.0]]]
        mat, om = STEEL, (0.0, 0.0, 100.0)
    elif name == "block_nobc":
        ids, xyz, elem, face = _block(2, 2, 2, (2.0, 2.0, 2.0), 0.1, 13)
        bounds, forces = [], []
        mat, om = STEEL, (0.0, 0.0, 100.0)
    elif name.startswith("mesh2"):
        d = np.load(os.path.join(HERE, "mesh2.npz"))
        nid_all, xyz_all, elem_all = d["node_ids"].astype(np.int64), d["xyz"], d["elem"].astype(np.int64)
        bot_in, bot_out = d["bot_in"].astype(np.int64), d["bot_out"].astype(np.int64)
        pos = np.zeros(nid_all.max() + 1, dtype=np.int64)
        pos[nid_all] = np.arange(nid_all.size)
        if name == "mesh2_full":
            sel = np.arange(elem_all.shape[1])
        else:
            cen = xyz_all[pos[elem_all + 1]].mean(axis=0)                    # (E, 3)
            anchor = xyz_all[pos[bot_in[len(bot_in) // 2]]]
            order = np.argsort(np.linalg.norm(cen - anchor, axis=1), kind="stable")
            sel = np.sort(order[:250 if name == "mesh2_slice" else 40])
        elem = elem_all[:, sel]
        used = np.unique(elem + 1)
        if name == "mesh2_isolated":
            spare = np.setdiff1d(nid_all, used)
            used = np.sort(np.append(used, spare[len(spare) // 2]))
        ids = used
        xyz = xyz_all[pos[ids]]
        present = set(ids.tolist())
        bounds = []
        for lis in (bot_in, bot_out):
            b = np.array([i for i in lis if i in present], dtype=np.int64)
            if b.size:
                bounds.append([b - 1, [0, 0, 0]])
        forces = []
        mat, om = STEEL, (0.0, 0.0, 100.0)
    else:
        raise KeyError(name)
    rng = np.random.default_rng(sum(map(ord, name)))
    u = rng.uniform(-1e-3, 1e-3, size=(len(ids), 3))
    ut = rng.uniform(-0.05, 0.05, size=(len(ids), 3))
    return ids, xyz, elem, bounds, forces, mat, om, u, ut


CASES = ("block_twist", "block_partial", "block_nobc", "mesh2_slice", "mesh2_isolated", "mesh2_full")


def run_case(mods, name):
    from oracle.refexec import reference_runner as RR
    ids, xyz, elem, bounds, forces, mat, om, u, ut = case_inputs(name)
    R = RR.physics(mods, ids, xyz, elem, bounds, forces)
    bi, bp, bv = pack_groups(bounds)
    fi, fp, fv = pack_groups(forces)
    out = dict(node_ids=ids.astype(np.int64), xyz=xyz, elem=elem.astype(np.int64), bounds_ids=bi, bounds_ptr=bp,
               bounds_codes=bv, forces_ids=fi, forces_ptr=fp, forces_vals=fv,
               materials=np.array([mat['DE'], mat['EX'], mat['PO']]), omegas=np.asarray(om, dtype=np.float64),
               u=u)
    t0 = time.time()
    K, M, F = RR.model_csr(mods, R, mat, om)
    if name == "mesh2_full":
        v = probe_vector(K.shape[0])
        absK = abs(K)
        out.update(SmNode_sha=sha(R.SmNode), ReNode_sha=sha(R.ReNode), CoElem=R.CoElem.astype(np.int32),
                   nnzb=int(R.SmNode[-1]), K_indptr_sha=sha(K.indptr), K_indices_sha=sha(K.indices),
                   M_indptr_sha=sha(M.indptr), M_indices_sha=sha(M.indices), Kv=K @ v, Kabs_v=(absK @ np.abs(v)).astype(np.float32),
                   Kdiag=K.diagonal(), Mv=M @ v, Mabs_v=(abs(M) @ np.abs(v)).astype(np.float32), F=F)
        S = RR.post_stress(mods, R, mat, u)
        nodes = np.sort(np.random.default_rng(7).choice(len(ids), size=2048, replace=False))
        out.update(S_nodes=nodes.astype(np.int64), S_sample=S[nodes], S_colsum=S.sum(axis=0))
    else:
        out.update(SmNode=R.SmNode.astype(np.int32), ReNode=R.ReNode.astype(np.int32),
                   CoElem=R.CoElem.astype(np.int32),
                   K_data=K.data, K_indices=K.indices.astype(np.int32), K_indptr=K.indptr.astype(np.int32),
                   M_data=M.data, M_indices=M.indices.astype(np.int32), M_indptr=M.indptr.astype(np.int32), F=F)
        if name == "mesh2_isolated":
            out.update(S_vector=RR.post_nodal_vector(mods, R, mat, u))
        else:
            out.update(S=RR.post_stress(mods, R, mat, u))
        if name in ("block_twist", "block_partial"):
            Kb = RR.model_bsr_K(mods, R, mat, om)
            out.update(Kb_data=Kb.data, Kb_indices=Kb.indices.astype(np.int32), Kb_indptr=Kb.indptr.astype(np.int32))
        if name in ("block_twist", "block_partial"):
            KT, KM = RR.model_bsr_tangent(mods, R, mat, om, ut)
            out.update(u_tangent=ut, KT_data=KT.data, KM_data=KM.data, KT_indices=KT.indices.astype(np.int32),
                       KT_indptr=KT.indptr.astype(np.int32))
    print("%-15s N=%d E=%d nnzb=%d  %.1f s" % (name, len(ids), elem.shape[1], int(R.SmNode[-1]), time.time() - t0),
          flush=True)
    return out


def main(argv):
    if not argv:
        print(__doc__)
        return 2
    ref_root, rest = argv[0], argv[1:]
    check = "--check" in rest
    names = [a for a in rest if a != "--check"] or list(CASES)
    from oracle.refexec import reference_runner as RR
    mods = RR.load(ref_root)
    bad = 0
    for name in names:
        out = run_case(mods, name)
        path = os.path.join(HERE, "refexec_%s.npz" % name)
        if not check:
            np.savez_compressed(path, **out)
            continue
        old = np.load(path)
        for k, v in out.items():
            a, b = np.asarray(v), old[k]
            same = (a.shape == b.shape and np.array_equal(a, b, equal_nan=True)) if a.dtype.kind != "f" else \
                (a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b)))))
            if not same:
                print("MISMATCH %s.%s" % (name, k))
                bad += 1
    if check:
        print("check: %d mismatching arrays" % bad)
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
