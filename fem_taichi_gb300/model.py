"""GPU drop-in for the reference ``Model`` (FEM_model_csr.py:7-146 / FEM_model_bsr.py:6-161).

``Model(name, Physics, Materials, Omegas=(0,0,100), Largedisp=False)`` keeps the
reference's constructor and getters:

    Get_MatrixKL() / Get_MatrixK()  -> scipy.sparse.csr_matrix (3N x 3N, float64, int32 indices)
    Get_MatrixM()                   -> scipy.sparse.csr_matrix (3 entries per block)
    Get_VectorF()                   -> ndarray (3N,), node-major

All arithmetic runs in the sm_103a kernels of ``libfemgb.so``; mesh, pattern and outputs
live in HBM (torch tensors used as raw device buffers).  The getters share one assembly pass
(``fem_assemble_host``) whose device->host copies of each part of the block rows overlap the
kernels of the next part.  Getters are idempotent: the reference's Taichi fields accumulate
across repeated calls (FEM_model_bsr.py:174; values match the reference's first call).

Extensions beyond the reference surface (for the solver and the benchmark):
    assemble(k_layout, m_layout)  -> device tensors (K, M, F) without host copies
    extra_loads                   -> float nodal loads added after the int-cast Forces
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from ._lib import FemAssemblyOut, FemMaterial, FemMesh, LAYOUT_BSR, LAYOUT_CSR


def _require_cuda(device):
    if not torch.cuda.is_available():
        raise RuntimeError("fem_taichi_gb300 needs a CUDA device (sm_103a); no CPU fallback exists")
    return torch.device(device)


def _dptr(t: torch.Tensor | None):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class DeviceMesh:
    """Device copies of the mesh, pattern and incidence; builds the C ``fem_mesh``."""

    def __init__(self, Physics, device="cuda"):
        self.device = _require_cuda(device)
        d = self.device
        P = Physics
        self.n_node = int(P.Num_Node)
        self.n_elem = int(P.Num_Elem)
        self.nnzb = int(P.SmNode[-1])
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=d, dtype=dt)  # noqa: E731
        self.xyz = t(P.xyz, torch.float64)
        self.conn = t(P.conn, torch.int32)
        self.indptr = t(P.SmNode.astype(np.int32), torch.int32)
        self.indices = t(P.ReNode.astype(np.int32), torch.int32)
        self.ne_ptr = t(P.ne_ptr, torch.int32)
        self.ne_list = t(P.ne_list, torch.int32)
        self.co_elem = t(P.CoElem.astype(np.int32), torch.int32)
        self.ne_inv = t(P.ne_inv, torch.int32)
        self.slot_map = t(P.slot_map, torch.uint8)
        self.c = FemMesh(self.n_node, self.n_elem, self.nnzb, self.xyz.data_ptr(), self.conn.data_ptr(),
                         self.indptr.data_ptr(), self.indices.data_ptr(), self.ne_ptr.data_ptr(),
                         self.ne_list.data_ptr(), self.ne_inv.data_ptr(), self.slot_map.data_ptr())

    def set_coordinates(self, xyz) -> None:
        """Replace node coordinates in place (host array or device tensor, (N, 3))."""
        src = torch.as_tensor(xyz, dtype=torch.float64)
        self.xyz.copy_(src.reshape(self.n_node, 3), non_blocking=True)


def material(Materials, Omegas) -> FemMaterial:
    om = np.asarray(Omegas, dtype=np.float64)
    return FemMaterial(float(Materials['DE']), float(Materials['EX']), float(Materials['PO']),
                       (ctypes.c_double * 3)(*om.tolist()))


def bounds_mask(Physics) -> np.ndarray:
    """Per-node DOF bit mask from Physics.Bounds (FEM_model_bsr.py:68-77, 248-259).

    With no bounds the reference packs one all-zero column, which fixes node Nind[0]."""
    mask = np.zeros(int(Physics.Num_Node), dtype=np.uint8)
    groups = list(Physics.Bounds) or [[np.zeros(1, dtype=np.int64), [0, 0, 0]]]
    for ids, codes in groups:
        nodes = Physics.Nind[np.asarray(ids, dtype=np.float64).astype(np.int64)]
        bits = 0
        for j in range(3):
            if float(codes[j]) != -1:
                bits |= 1 << j
        np.bitwise_or.at(mask, nodes, np.uint8(bits))
    return mask


def nodal_loads(Physics) -> np.ndarray:
    """Per-node loads from Physics.Forces with the reference's int cast (FEM_model_bsr.py:79-88,
    220-226); groups are summed in order."""
    F = np.zeros((int(Physics.Num_Node), 3))
    for ids, vals in Physics.Forces:
        v = np.array(vals, dtype=np.int64).astype(np.float64)
        nodes = Physics.Nind[np.asarray(ids, dtype=np.float64).astype(np.int64)]
        np.add.at(F, nodes, v[None, :])
    return F


class Model:
    """Drop-in GPU replacement of the reference FE model (linear part)."""

    def __init__(self, name, Physics, Materials, Omegas=(0, 0, 100), Largedisp=False, device="cuda",
                 extra_loads=None, algo="fp64"):
        self.name = name
        self.DE, self.EX, self.PO = Materials['DE'], Materials['EX'], Materials['PO']
        self.OM = np.array(Omegas, dtype=np.float64)
        self.Physics = Physics
        self.Largedisp = Largedisp
        self.Num_Node = int(Physics.Num_Node)
        self.Num_Elem = int(Physics.Num_Elem)
        self.Num_MaxN = int(Physics.Num_MaxN)
        self.Num_Free = self.Num_Node * 3
        self.nnz_K, self.nnz_M = int(Physics.SmNode[-1]) * 9, int(Physics.SmNode[-1]) * 3
        self.lib = _lib.load()
        self.mesh = DeviceMesh(Physics, device)
        self.device = self.mesh.device
        self.mat = material(Materials, Omegas)
        self.fixed_host = bounds_mask(Physics)
        self.fixed = torch.from_numpy(self.fixed_host).to(self.device)
        loads = nodal_loads(Physics)
        if extra_loads is not None:
            loads = loads + np.asarray(extra_loads, dtype=np.float64).reshape(-1, 3)
        self.loads_host = loads
        self.loads = torch.from_numpy(np.ascontiguousarray(loads)).to(self.device)
        self._ws = None
        self._csr_index = None
        self._version = 0          # bumped whenever an assembly input changes
        self._cache = None         # (version, {"K", "M", "F"} host arrays not yet handed out)
        self._plan = None
        self.U = None              # large-displacement state (LDinit)
        self.pipeline_parts = 16   # parts of fem_assemble_host (copies overlap the next part)
        self.m_staging = True      # M leaves the device as one value per block (fem_assemble_host_staged)
        if algo not in ("dd", "fp64"):
            raise ValueError("algo must be 'dd' or 'fp64'")
        self.algo = algo

    # -- device-level API --------------------------------------------------------------
    def workspace(self) -> torch.Tensor:
        nbytes = int(self.lib.fem_assemble_workspace_bytes(self.Num_Elem))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=self.device)
        return self._ws

    def assemble(self, K=True, M=True, F=True, k_layout="bsr", m_layout="bsr", out=None, algo=None):
        """Run the assembly kernels; returns (K, M, F) device tensors (None where skipped).

        k_layout 'bsr' -> K (nnzb, 3, 3); 'csr' -> K (9*nnzb,) in the reference CSR order.
        m_layout 'bsr' -> M (nnzb,);       'csr' -> M (3*nnzb,) reference CSR order.
        algo: 'fp64' (FP64 arithmetic, default) or 'dd' (double-float pairs on the FP32 pipes,
        about 48-bit significands).
        """
        algo = self.algo if algo is None else algo
        d = self.device
        nnzb = self.mesh.nnzb
        out = out or {}
        Kt = out.get("K") if K else None
        Mt = out.get("M") if M else None
        Ft = out.get("F") if F else None
        if K and Kt is None:
            Kt = torch.empty((nnzb, 3, 3) if k_layout == "bsr" else (9 * nnzb,), dtype=torch.float64, device=d)
        if M and Mt is None:
            Mt = torch.empty((nnzb,) if m_layout == "bsr" else (3 * nnzb,), dtype=torch.float64, device=d)
        if F and Ft is None:
            Ft = torch.empty((self.Num_Node, 3), dtype=torch.float64, device=d)
        ws = self.workspace()
        o = FemAssemblyOut(LAYOUT_BSR if k_layout == "bsr" else LAYOUT_CSR,
                           LAYOUT_BSR if m_layout == "bsr" else LAYOUT_CSR,
                           Kt.data_ptr() if Kt is not None else None,
                           Mt.data_ptr() if Mt is not None else None,
                           Ft.data_ptr() if Ft is not None else None,
                           self.fixed.data_ptr(), self.loads.data_ptr(),
                           _lib.ALGO_DD if algo == "dd" else _lib.ALGO_FP64)
        _lib.check(self.lib.fem_assemble(ctypes.byref(self.mesh.c), ctypes.byref(self.mat), ctypes.byref(o),
                                         _dptr(ws), ws.numel(), _stream(d)), "fem_assemble")
        return Kt, Mt, Ft

    def csr_index(self):
        """Host (rowK, colK, rowM, colM) int32 arrays of the reference CSR layout (cached)."""
        if self._csr_index is None:
            d = self.device
            n3 = 3 * self.Num_Node + 1
            nnzb = self.mesh.nnzb
            rowK = torch.empty(n3, dtype=torch.int32, device=d)
            colK = torch.empty(9 * nnzb, dtype=torch.int32, device=d)
            rowM = torch.empty(n3, dtype=torch.int32, device=d)
            colM = torch.empty(3 * nnzb, dtype=torch.int32, device=d)
            _lib.check(self.lib.fem_csr_index(ctypes.byref(self.mesh.c), _dptr(rowK), _dptr(colK), _dptr(rowM),
                                              _dptr(colM), _stream(d)), "fem_csr_index")
            self._csr_index = tuple(t.cpu().numpy() for t in (rowK, colK, rowM, colM))
        return self._csr_index

    def pipeline_plan(self, n_parts=None):
        """(row_split, elem_split, block_split) int64 host arrays of fem_assemble_host (cached)."""
        n_parts = self.pipeline_parts if n_parts is None else int(n_parts)
        if self._plan is None or self._plan[0] != n_parts:
            P = self.Physics
            ind = np.ascontiguousarray(P.SmNode, dtype=np.int32)
            nep = np.ascontiguousarray(P.ne_ptr, dtype=np.int32)
            nel = np.ascontiguousarray(P.ne_list, dtype=np.int32)
            rs, es, bs = (np.zeros(n_parts + 1, dtype=np.int64) for _ in range(3))
            _lib.check(self.lib.fem_pipeline_plan(self.Num_Node, self.Num_Elem, ind.ctypes.data, nep.ctypes.data,
                                                  nel.ctypes.data, n_parts, rs.ctypes.data, es.ctypes.data,
                                                  bs.ctypes.data), "fem_pipeline_plan")
            self._plan = (n_parts, rs, es, bs)
        return self._plan[1:]

    def assemble_host(self, n_parts=None):
        """One assembly pass delivered to page-locked host arrays: K (9*nnzb,) and M (3*nnzb,)
        in the reference CSR orders, F (3N,).  The device->host copies of each part of the
        block rows overlap the kernels of the next part; M leaves the device as one value per
        block and is written in the CSR order on the host while later parts are copied
        (fem_assemble_host_staged)."""
        d = self.device
        nnzb = self.mesh.nnzb
        Kd = torch.empty(9 * nnzb, dtype=torch.float64, device=d)
        Md = torch.empty(3 * nnzb, dtype=torch.float64, device=d)
        Fd = torch.empty((self.Num_Node, 3), dtype=torch.float64, device=d)
        Kh = torch.empty(9 * nnzb, dtype=torch.float64, pin_memory=True)
        Mh = torch.empty(3 * nnzb, dtype=torch.float64, pin_memory=True)
        Fh = torch.empty(3 * self.Num_Node, dtype=torch.float64, pin_memory=True)
        ws = self.workspace()
        o = FemAssemblyOut(LAYOUT_CSR, LAYOUT_CSR, Kd.data_ptr(), Md.data_ptr(), Fd.data_ptr(),
                           self.fixed.data_ptr(), self.loads.data_ptr(),
                           _lib.ALGO_DD if self.algo == "dd" else _lib.ALGO_FP64)
        rs, es, bs = self.pipeline_plan(n_parts)
        if not self.m_staging:
            _lib.check(self.lib.fem_assemble_host(ctypes.byref(self.mesh.c), ctypes.byref(self.mat), ctypes.byref(o),
                                                  rs.ctypes.data, es.ctypes.data, bs.ctypes.data, len(rs) - 1,
                                                  Kh.data_ptr(), Mh.data_ptr(), Fh.data_ptr(), _dptr(ws), ws.numel(),
                                                  _stream(d)), "fem_assemble_host")
            torch.cuda.current_stream(d).synchronize()
            return Kh.numpy(), Mh.numpy(), Fh.numpy()
        Ms = torch.empty(nnzb, dtype=torch.float64, pin_memory=True)   # M, one value per block
        ind = self._indptr_host()
        _lib.check(self.lib.fem_assemble_host_staged(ctypes.byref(self.mesh.c), ctypes.byref(self.mat),
                                                     ctypes.byref(o), rs.ctypes.data, es.ctypes.data, bs.ctypes.data,
                                                     len(rs) - 1, ind.ctypes.data, Kh.data_ptr(), Mh.data_ptr(),
                                                     Fh.data_ptr(), Ms.data_ptr(), _dptr(ws), ws.numel(), _stream(d)),
                   "fem_assemble_host_staged")
        torch.cuda.current_stream(d).synchronize()
        return Kh.numpy(), Mh.numpy(), Fh.numpy()

    def _indptr_host(self):
        if getattr(self, "_indptr_h", None) is None:
            self._indptr_h = np.ascontiguousarray(self.Physics.SmNode, dtype=np.int32)
        return self._indptr_h

    def set_coordinates(self, xyz) -> None:
        """Move the nodes (same topology); the next getter re-assembles."""
        self.mesh.set_coordinates(xyz)
        self._version += 1

    def _take(self, key):
        """Host result `key` of the current inputs.  One assembly pass serves K, M and F;
        each array is handed out once (a repeated getter call runs a new pass, so callers
        never share a buffer)."""
        if self._cache is None or self._cache[0] != self._version or key not in self._cache[1]:
            K, M, F = self.assemble_host()
            self._cache = (self._version, {"K": K, "M": M, "F": F})
        return self._cache[1].pop(key)

    # -- reference getters -------------------------------------------------------------
    def Get_MatrixKL(self):
        """FEM_model_csr.py:118-127: K as scipy CSR (penalty applied)."""
        K = self._take("K")
        rowK, colK, _, _ = self.csr_index()
        n = self.Num_Free
        return sp.csr_matrix((K, colK, rowK), shape=(n, n), dtype=np.float64, copy=False)

    Get_MatrixK = Get_MatrixKL

    def Get_MatrixM(self):
        """FEM_model_csr.py:129-137 / FEM_model_bsr.py:147-155."""
        M = self._take("M")
        _, _, rowM, colM = self.csr_index()
        n = self.Num_Free
        return sp.csr_matrix((M, colM, rowM), shape=(n, n), dtype=np.float64, copy=False)

    def Get_VectorF(self):
        """FEM_model_csr.py:141-146: element centrifugal loads + nodal loads, node-major (3N,)."""
        return self._take("F")

    # -- large displacement (FEM_model_bsr.py:134-145, 476-598) ----------------------------
    def LDinit(self, displace):
        """FEM_model_bsr.py:595-598: set the nodal displacements (3N,) the tangent is taken at."""
        self.U = torch.as_tensor(np.asarray(displace, dtype=np.float64).reshape(-1, 3)).to(self.device).contiguous()

    def assemble_tangent(self, k_layout="bsr"):
        """Device (KT, KM) at the displacements of LDinit: (nnzb, 3, 3) BSR or (9 nnzb,) CSR order."""
        if getattr(self, "U", None) is None:
            self.LDinit(np.zeros(self.Num_Free))
        d = self.device
        nnzb = self.mesh.nnzb
        shape = (nnzb, 3, 3) if k_layout == "bsr" else (9 * nnzb,)
        KT = torch.empty(shape, dtype=torch.float64, device=d)
        KM = torch.empty(shape, dtype=torch.float64, device=d)
        nbytes = max(int(self.lib.fem_tangent_workspace_bytes(self.Num_Elem)), 16)
        if getattr(self, "_tws", None) is None or self._tws.numel() < nbytes:
            self._tws = torch.empty(nbytes, dtype=torch.uint8, device=d)
        _lib.check(self.lib.fem_assemble_tangent(ctypes.byref(self.mesh.c), ctypes.byref(self.mat), _dptr(self.U),
                                                 LAYOUT_BSR if k_layout == "bsr" else LAYOUT_CSR, _dptr(KT),
                                                 _dptr(KM), _dptr(self.fixed), _dptr(self._tws),
                                                 self._tws.numel(), _stream(d)), "fem_assemble_tangent")
        return KT, KM

    def Get_MatrixKN(self):
        """FEM_model_bsr.py:134-145: (KT, KM) as scipy CSR at the displacements of LDinit."""
        KT, KM = self.assemble_tangent(k_layout="csr")
        rowK, colK, _, _ = self.csr_index()
        n = self.Num_Free
        mk = lambda V: sp.csr_matrix((V.cpu().numpy(), colK, rowK), shape=(n, n), dtype=np.float64)  # noqa: E731
        return mk(KT), mk(KM)
