"""GPU static solve: drop-in for ``SOLVE_static.Static_solver`` (SOLVE_static.py:6-77).

The reference factorises K with MKL Pardiso (``pardisoSolver(KL, mtype=2)``,
SOLVE_static.py:31-33).  Here K stays in HBM as 3x3-block BSR and the system is solved by
the block-preconditioned CG of ``libfemgb.so`` (``fem_pcg_solve``):

* ``mixed=False``: FP64 PCG with block-Jacobi (inverse 3x3 diagonal blocks);
* ``mixed=True``: FP32 SpMV / FP32 preconditioner inner PCG inside FP64 iterative
  refinement (true residual r = F - K u in FP64);
* up to 32 right-hand sides in one solve (lockstep PCG, BSR SpMM);
* iterations replayed as CUDA graphs; SpMV launch shape chosen by the autotuner;
* ``precond="amg"``: a smoothed-aggregation multigrid V-cycle (rigid-body modes, Chebyshev
  smoothing, FP32) preconditions the solve, for meshes where block-diagonal preconditioners
  stall (``fem_amg_setup`` / ``fem_pcg_solve_amg``).  ``mixed=True`` runs it inside the FP32
  inner solve of the refinement loop; ``mixed=False`` runs FP64 flexible CG (FP64 products
  with K) around the FP32 cycle, which also converges when the condition number is beyond
  FP32 refinement (kappa >~ 1e7, e.g. slender cantilevers); a mixed solve that stalls is
  repeated that way.

``Static_solver(Model, Qtype=0).Solve_cpu(max_errs, max_iters)`` keeps the reference's
signature and return value (U, (3N,) float64) but runs the GPU solve to a tight tolerance
(there is no CPU path).  ``Solve_gpu(...)`` exposes the options.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import FemAmgLevelInfo, FemAmgOpts, FemBsr, FemPcgOpts, FemPcgStats, FEM_F32, FEM_F64
from .model import _dptr, _stream

SUPPORTED_NRHS = (1, 2, 4, 8, 16, 32)

_STATUS = {0: "converged", _lib.FEM_ERR_MAXITER: "max iterations", _lib.FEM_ERR_NOT_CONVERGED: "stalled",
           _lib.FEM_ERR_NOT_SPD: "non-positive curvature", _lib.FEM_ERR_BREAKDOWN: "NaN/Inf breakdown"}


def padded_nrhs(r: int) -> int:
    for s in SUPPORTED_NRHS:
        if r <= s:
            return s
    raise ValueError("at most 32 right-hand sides per solve")


class AmgHierarchy:
    """Owner of a ``fem_amg`` hierarchy for one matrix.

    ``AmgHierarchy(lib, n, indptr, indices, vals, xyz, stream)`` sets it up on the host from
    HOST copies of the FP64 BSR matrix and the node coordinates (``fem_amg_setup``), then
    uploads it; ``AmgHierarchy.on_device(system)`` sets it up on the device from the
    system's FP64 matrix (``fem_amg_setup_device``).  ``opts`` overrides fields of
    ``fem_amg_default_opts``."""

    @staticmethod
    def _options(lib, opts):
        o = FemAmgOpts()
        lib.fem_amg_default_opts(ctypes.byref(o))
        for k, v in opts.items():
            if not hasattr(o, k):
                raise ValueError(f"unknown AMG option {k}")
            setattr(o, k, v)
        return o

    def __init__(self, lib, n, indptr, indices, vals, xyz, stream=None, **opts):
        import time
        self.lib = lib
        self.where = "host"
        o = self.opts = self._options(lib, opts)
        ip = np.ascontiguousarray(indptr, dtype=np.int32)
        ix = np.ascontiguousarray(indices, dtype=np.int32)
        va = np.ascontiguousarray(vals, dtype=np.float64)
        xy = np.ascontiguousarray(xyz, dtype=np.float64).reshape(n, 3)
        h = ctypes.c_void_p()
        t0 = time.perf_counter()
        _lib.check(lib.fem_amg_setup(n, ip.ctypes.data, ix.ctypes.data, va.ctypes.data, xy.ctypes.data,
                                     ctypes.byref(o), ctypes.byref(h)), "fem_amg_setup")
        self.h = h
        self.setup_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        if stream is not None:
            _lib.check(lib.fem_amg_upload(self.h, stream), "fem_amg_upload")
        self.upload_s = time.perf_counter() - t0

    @classmethod
    def on_device(cls, system, host_pattern=True, **opts):
        """Set up from ``system.A64`` and the model's device coordinates; the host pattern of
        the model (``Physics.SmNode`` / ``ReNode``) saves downloading it (host_pattern=False:
        the setup downloads it)."""
        import time
        self = cls.__new__(cls)
        self.lib = system.lib
        self.where = "device"
        o = self.opts = cls._options(system.lib, opts)
        xyz = system.model.mesh.xyz.to(torch.float64).contiguous()
        P = system.model.Physics
        ip = np.ascontiguousarray(P.SmNode, dtype=np.int32)
        ix = np.ascontiguousarray(P.ReNode, dtype=np.int32)
        if not host_pattern or ip.shape[0] != system.n + 1 or ix.shape[0] != system.nnzb:
            ip = ix = None
        h = ctypes.c_void_p()
        torch.cuda.synchronize(system.device)
        t0 = time.perf_counter()
        _lib.check(system.lib.fem_amg_setup_device(ctypes.byref(system.A64), xyz.data_ptr(),
                                                   None if ip is None else ip.ctypes.data,
                                                   None if ix is None else ix.ctypes.data, ctypes.byref(o),
                                                   system.stream, ctypes.byref(h)), "fem_amg_setup_device")
        self.h = h
        self.setup_s = time.perf_counter() - t0
        self.upload_s = 0.0
        return self

    def levels(self):
        out = []
        for l in range(int(self.lib.fem_amg_num_levels(self.h))):
            info = FemAmgLevelInfo()
            _lib.check(self.lib.fem_amg_get_level(self.h, l, ctypes.byref(info)), "fem_amg_get_level")
            out.append({"n": info.n, "b": info.b, "nnzb_A": info.nnzb_A, "nnzb_P": info.nnzb_P,
                        "lmax": info.lmax, "omega": info.omega, "setup_s": info.setup_s})
        return out

    def setup_phases(self):
        """Host seconds per setup phase (summed over levels)."""
        t = (ctypes.c_double * 6)()
        _lib.check(self.lib.fem_amg_setup_phases(self.h, t), "fem_amg_setup_phases")
        return dict(zip(("strength_aggregation", "tentative", "lanczos", "smoothing", "galerkin", "coarse_inverse"),
                        (round(v, 3) for v in t)))

    def export(self, level, what):
        """Host copy of one level's array (see fem_amg_export): a scipy BSR-like triple
        (indptr, indices, blocks) for what in 0..2, else the value / index array."""
        dims = (ctypes.c_int64 * 4)()
        _lib.check(self.lib.fem_amg_export(self.h, level, what, dims, None, None, None), "fem_amg_export")
        rows, nnz, br, bc = (int(d) for d in dims)
        if what <= 2:
            ptr = np.zeros(rows + 1, dtype=np.int64)
            col = np.zeros(max(nnz, 1), dtype=np.int32)
            val = np.zeros(max(nnz, 1) * br * bc, dtype=np.float64)
            _lib.check(self.lib.fem_amg_export(self.h, level, what, dims, ptr.ctypes.data, col.ctypes.data,
                                               val.ctypes.data), "fem_amg_export")
            return ptr, col[:nnz], val[:nnz * br * bc].reshape(nnz, br, bc)
        if what in (4, 6):
            idx = np.zeros(max(nnz, 1), dtype=np.int32)
            _lib.check(self.lib.fem_amg_export(self.h, level, what, dims, None, idx.ctypes.data, None),
                       "fem_amg_export")
            return idx[:nnz]
        val = np.zeros(max(nnz, 1), dtype=np.float64)
        _lib.check(self.lib.fem_amg_export(self.h, level, what, dims, None, None, val.ctypes.data),
                   "fem_amg_export")
        return val[:nnz]

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fem_amg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceSystem:
    """K (FP64 BSR, and its FP32 copy on demand) plus F of a ``Model`` on the device."""

    def __init__(self, model, K=None, F=None):
        self.model = model
        self.lib = _lib.load()
        self.device = model.device
        if K is None or F is None:
            K, _, F = model.assemble(K=True, M=False, F=True, k_layout="bsr")
        self.K64 = K
        self.F = F.reshape(-1)
        self.n = model.Num_Node
        self.nnzb = model.mesh.nnzb
        self.A64 = FemBsr(self.n, self.nnzb, model.mesh.indptr.data_ptr(), model.mesh.indices.data_ptr(),
                          self.K64.data_ptr(), FEM_F64, _lib.LAYOUT_BSR)
        self._K32 = None
        self._A32 = None
        self._bj = None
        self._variant = {}
        self._ws = None
        self._amg = None

    @property
    def stream(self):
        return _stream(self.device)

    def K32(self):
        """FP32 copy of K in the padded row-SoA layout (rows rounded up to 4 blocks, so the
        SpMV reads 4 slots of a value with one 16-byte load)."""
        if self._K32 is None:
            P = self.model.Physics
            ind = np.ascontiguousarray(P.SmNode, dtype=np.int32)
            ind4 = np.zeros(self.n + 1, dtype=np.int32)
            _lib.check(self.lib.fem_rsoa4_indptr(self.n, ind.ctypes.data, ind4.ctypes.data), "fem_rsoa4_indptr")
            nnzb4 = int(ind4[-1])
            self._indptr4 = torch.from_numpy(ind4).to(self.device)
            self._indices4 = torch.empty(max(nnzb4, 4), dtype=torch.int32, device=self.device)
            self._K32 = torch.empty(9 * max(nnzb4, 4), dtype=torch.float32, device=self.device)
            _lib.check(self.lib.fem_bsr_to_rsoa4_f32(ctypes.byref(self.A64), _dptr(self._indptr4),
                                                     _dptr(self._indices4), _dptr(self._K32), self.stream),
                       "fem_bsr_to_rsoa4_f32")
            self._A32 = FemBsr(self.n, nnzb4, self._indptr4.data_ptr(), self._indices4.data_ptr(),
                               self._K32.data_ptr(), FEM_F32, _lib.LAYOUT_RSOA4)
        return self._K32

    def block_jacobi(self) -> torch.Tensor:
        """(N, 9) FP64 inverses of the diagonal blocks."""
        if self._bj is None:
            bj = torch.empty((self.n, 9), dtype=torch.float64, device=self.device)
            bad = torch.zeros(1, dtype=torch.int32, device=self.device)
            _lib.check(self.lib.fem_block_jacobi(ctypes.byref(self.A64), _dptr(bj), None, _dptr(bad), self.stream),
                       "fem_block_jacobi")
            if int(bad.item()):
                raise _lib.FemError(_lib.FEM_ERR_NOT_SPD, f"{int(bad.item())} singular diagonal blocks")
            self._bj = bj
        return self._bj

    def amg(self, setup="device", **opts) -> AmgHierarchy:
        """Smoothed-aggregation multigrid hierarchy of K (built once; ``opts`` as
        ``fem_amg_opts``).  setup: "device" (``fem_amg_setup_device``, from the FP64 matrix in
        HBM) or "host" (``fem_amg_setup`` on a host copy of K, then uploaded)."""
        if self._amg is None or opts or self._amg.where != setup:
            if self._amg is not None:
                self._amg.close()
            self._amg = self.amg_variant(setup=setup, **opts)
        return self._amg

    def amg_variant(self, setup="device", **opts) -> AmgHierarchy:
        """A separate multigrid hierarchy of K built with ``opts`` (not cached; pass it to
        ``solve(precond=...)`` and close it when done)."""
        if setup == "device":
            return AmgHierarchy.on_device(self, **opts)
        if setup != "host":
            raise ValueError("setup must be 'device' or 'host'")
        xyz = self.model.mesh.xyz.cpu().numpy()
        K = self.K64.reshape(-1).cpu().numpy()
        P = self.model.Physics
        return AmgHierarchy(self.lib, self.n, P.SmNode, P.ReNode, K, xyz, self.stream, **opts)

    def spmv(self, x: torch.Tensor, fp32=False, nrhs=1) -> torch.Tensor:
        A = self._A32 if fp32 else self.A64
        if fp32:
            self.K32()
            A = self._A32
        y = torch.empty_like(x)
        _lib.check(self.lib.fem_bsr_spmv(ctypes.byref(A), nrhs, _dptr(x), _dptr(y),
                                         self.variant(fp32, nrhs), self.stream), "fem_bsr_spmv")
        return y

    def variant(self, fp32: bool, nrhs: int) -> int:
        """Autotuned SpMV launch variant for (precision, nrhs), tuned once on this matrix."""
        key = (fp32, nrhs)
        if key not in self._variant:
            if nrhs != 1:
                self._variant[key] = 0
            else:
                if fp32:
                    self.K32()
                A = self._A32 if fp32 else self.A64
                dt = torch.float32 if fp32 else torch.float64
                x = torch.ones(3 * self.n, dtype=dt, device=self.device)
                y = torch.empty_like(x)
                best = ctypes.c_int(0)
                ms = ctypes.c_float(0)
                _lib.check(self.lib.fem_spmv_autotune(ctypes.byref(A), 1, _dptr(x), _dptr(y), 5, ctypes.byref(best),
                                                      ctypes.byref(ms), self.stream), "fem_spmv_autotune")
                self._variant[key] = best.value
                self.variant_ms = getattr(self, "variant_ms", {})
                self.variant_ms[key] = ms.value
        return self._variant[key]

    def solve(self, F=None, rtol=1e-10, maxit=50000, mixed=True, precond=None, use_graph=True, unroll=16,
              inner_rtol=1e-4, inner_maxit=20000, max_outer=40, residual="fp64", stall_window=0):
        """Solve K U = F.  F: device/host array (3N,) or (3N, R) (default: the assembled F).

        precond: (N, 9) FP64 blocks (default block Jacobi), "amg" (multigrid V-cycle; with
        mixed=True inside the FP32 inner solve, falling back to the FP64 flexible-CG form when
        the refinement stalls) or an AmgHierarchy of this matrix (amg_variant).  residual: "fp64" or "extra" -- how the true residual F - K U
        that decides convergence and drives the refinement is formed ("extra": compensated,
        as accurate as twice-FP64 arithmetic).  Returns (U (3N,) or (3N, R) device tensor,
        stats dict).  stall_window > 0 ends a solve whose worst relative residual has not
        halved in that many iterations (status FEM_ERR_NOT_CONVERGED).  stats["status"] is 0 only when ||F - K U|| / ||F|| <= rtol for every
        right-hand side, and stats["floor"] is the residual that rounding U to FP64 alone
        leaves (2^-53 || |F| + |K||U| || / ||F||, max over RHS)."""
        if residual not in ("fp64", "extra"):
            raise ValueError("residual must be 'fp64' or 'extra'")
        if F is None:
            F = self.F
        F = torch.as_tensor(F, dtype=torch.float64, device=self.device)
        squeeze = F.dim() == 1
        F2 = F.reshape(3 * self.n, -1)
        R = F2.shape[1]
        Rp = padded_nrhs(R)
        if Rp != R:
            F2 = torch.cat([F2, torch.zeros((3 * self.n, Rp - R), dtype=torch.float64, device=self.device)], 1)
        F2 = F2.contiguous()
        U = torch.empty_like(F2)
        use_amg = isinstance(precond, AmgHierarchy) or (isinstance(precond, str) and precond == "amg")
        if use_amg:
            amg = precond if isinstance(precond, AmgHierarchy) else self.amg()
            self.K32()
            P = None
        else:
            P = self.block_jacobi() if precond is None else torch.as_tensor(precond, dtype=torch.float64,
                                                                             device=self.device).reshape(self.n, 9)
            P = P.contiguous()
        if mixed:
            self.K32()
        nbytes = int(self.lib.fem_pcg_workspace_bytes(self.n, Rp, int(mixed)))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        opts = FemPcgOpts(Rp, int(mixed), float(rtol), int(maxit), float(inner_rtol), int(inner_maxit),
                          int(max_outer), int(use_graph), int(unroll), self.variant(False, Rp),
                          self.variant(True, Rp) if mixed else 0,
                          _lib.RESIDUAL_EXTRA if residual == "extra" else _lib.RESIDUAL_FP64, int(stall_window))
        st = FemPcgStats()
        A32 = ctypes.byref(self._A32) if (mixed or use_amg) else None
        if use_amg:
            _lib.check(self.lib.fem_pcg_solve_amg(ctypes.byref(self.A64), A32, amg.h, _dptr(F2), _dptr(U),
                                                  ctypes.byref(opts), ctypes.byref(st), _dptr(self._ws),
                                                  self._ws.numel(), self.stream), "fem_pcg_solve_amg")
        else:
            _lib.check(self.lib.fem_pcg_solve(ctypes.byref(self.A64), A32, _dptr(P), _dptr(F2), _dptr(U),
                                              ctypes.byref(opts), ctypes.byref(st), _dptr(self._ws),
                                              self._ws.numel(), self.stream), "fem_pcg_solve")
        stats = {"status": st.status, "status_text": _STATUS.get(st.status, str(st.status)),
                 "iterations": st.iterations, "outer": st.outer, "relres": st.relres, "time_ms": st.time_ms,
                 "floor": st.floor, "nrhs": R, "mixed": bool(mixed), "precond": "amg" if use_amg else "block",
                 "residual": residual, "stall_window": int(stall_window)}
        if use_amg and mixed and st.status == _lib.FEM_ERR_NOT_CONVERGED:
            # FP32 refinement stalled (condition number beyond FP32): FP64 flexible CG instead
            U2, st2 = self.solve(F=F if squeeze else F2[:, :R], rtol=rtol, maxit=maxit, mixed=False, precond=precond,
                                 use_graph=use_graph, unroll=unroll, max_outer=max_outer, residual=residual)
            st2["fallback_from"] = stats
            return U2, st2
        U = U[:, :R]
        return (U.reshape(-1) if squeeze else U), stats


class Static_solver:
    """Drop-in for SOLVE_static.Static_solver (linear part, Qtype=0)."""

    def __init__(self, Model, Qtype=0):
        self.Qtype = Qtype
        self.Model = Model
        self.system = None
        self.last_stats = None

    def _system(self):
        if self.system is None:
            self.system = DeviceSystem(self.Model)
        return self.system

    def Solve_nonlinear(self, max_errs=1e-4, max_iters=20, rtol=1e-10, mixed=True):
        """Large-displacement Newton iteration of SOLVE_static.py:41-75 on the device.  Each
        step: tangent KT and secant KM at U (Model.assemble_tangent), residual RF = KM U - F,
        stop when ||RF|| / ||F|| <= max_errs or after max_iters steps, else KT dU = RF by PCG
        and U -= dU.  (The reference solves KT dU = F at SOLVE_static.py:72, which does not
        converge; this is the Newton-Raphson step that line stands for.)  Returns U (3N,) numpy;
        self.last_stats["residuals"] holds the relative residual of every step."""
        M = self.Model
        dev = M.device
        F = torch.as_tensor(M.Get_VectorF(), dtype=torch.float64).to(dev)
        fn = float(torch.linalg.norm(F))
        U = torch.zeros_like(F)
        res, its = [], 0
        step = 0
        while True:
            M.LDinit(U.cpu().numpy())
            KT, KM = M.assemble_tangent(k_layout="bsr")
            A = FemBsr(M.Num_Node, M.mesh.nnzb, M.mesh.indptr.data_ptr(), M.mesh.indices.data_ptr(),
                       KM.data_ptr(), FEM_F64, _lib.LAYOUT_BSR)
            KU = torch.empty_like(U)
            _lib.check(M.lib.fem_bsr_spmv(ctypes.byref(A), 1, _dptr(U), _dptr(KU), 0,
                                          ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)), "KM U")
            RF = KU - F
            err = float(torch.linalg.norm(RF)) / fn if fn > 0 else 0.0
            res.append(err)
            if err <= max_errs or step == max_iters:
                break
            S = DeviceSystem(M, K=KT, F=RF)
            dU, st = S.solve(F=RF, rtol=rtol, mixed=mixed)
            if st["status"] != 0:
                raise _lib.FemError(st["status"], f"Newton step {step}: {st['status_text']}")
            its += st["iterations"]
            U = U - dU
            step += 1
        self.last_stats = {"residuals": res, "steps": step, "pcg_iterations": its,
                           "converged": res[-1] <= max_errs}
        return U.cpu().numpy()

    def Solve_gpu(self, rtol=1e-10, F=None, mixed=True, precond="bj", maxit=50000, stall_window=None, **kw):
        """GPU solve; returns U as numpy ((3N,) or (3N, R)).  precond: 'bj', 'amg' (multigrid
        V-cycle), 'learned' (uses ``self.Model.learned_precond`` (N, 9) if set) or an (N, 9)
        array.  The learned solve runs with a stall detector: when its worst relative residual
        has not halved within ``stall_window`` iterations (default 256; or it fails otherwise)
        the solve switches to plain block Jacobi from the start; ``last_stats["fallback_from"]``
        then holds the abandoned attempt.  For the other preconditioners ``stall_window`` (default
        off) ends a stalling solve with FEM_ERR_NOT_CONVERGED."""
        if self.Qtype != 0:
            raise ValueError("Solve_gpu is the linear solve; Qtype=1 uses Solve_cpu / Solve_nonlinear")
        S = self._system()
        P = None
        fallback = False
        if isinstance(precond, str):
            if precond == "learned":
                P = getattr(self.Model, "learned_precond", None)
                if P is None:
                    raise ValueError("no learned preconditioner attached to the model (Model.learned_precond)")
                fallback = True
            elif precond == "amg":
                P = "amg"
            elif precond != "bj":
                raise ValueError("precond must be 'bj', 'amg', 'learned' or an (N, 9) array")
        else:
            P = precond
        if stall_window is None:
            stall_window = 256 if fallback else 0
        U, st = S.solve(F=F, rtol=rtol, maxit=maxit, mixed=mixed, precond=P, stall_window=stall_window, **kw)
        if fallback and st["status"] != 0:
            U, st2 = S.solve(F=F, rtol=rtol, maxit=maxit, mixed=mixed, precond=None, **kw)
            st2["fallback_from"] = st
            st = st2
        self.last_stats = st
        return U.cpu().numpy()

    def Solve_cpu(self, max_errs=1e-4, max_iters=20):
        """SOLVE_static.py:12-75 signature: returns U (3N,).  Qtype 0 runs the GPU linear solve
        to a relative residual of 1e-12 (the reference used a direct factorisation, which
        always returns a solution): mixed block-Jacobi PCG first (capped at 20,000
        iterations, and abandoned once its residual has not halved in 1,000), and when that does
        not converge (slender or stretched meshes) the FP64 multigrid solve with compensated
        residuals to 1e-12 or as far as FP64 allows;
        ``last_stats["fallback_from"]`` then holds the first attempt.  When the fallback also
        stops above 1e-12, a RuntimeWarning gives its residual and the FP64 floor
        (``last_stats["floor"]``): the displacement is then as accurate as FP64 storage permits
        when the two are close.  Qtype 1 runs the large-displacement Newton iteration
        (Solve_nonlinear)."""
        if self.Qtype == 1:
            return self.Solve_nonlinear(max_errs=max_errs, max_iters=max_iters)
        U = self.Solve_gpu(rtol=1e-12, mixed=True, maxit=20000, stall_window=1000)
        if self.last_stats["status"] != 0:
            first = self.last_stats
            U = self.Solve_gpu(rtol=1e-12, mixed=False, precond="amg", residual="extra", max_outer=8)
            self.last_stats["fallback_from"] = first
            st = self.last_stats
            if st["status"] != 0:
                import warnings
                warnings.warn(f"static solve stopped at relative residual {st['relres']:.3e} > 1e-12 "
                              f"({st['status_text']}); FP64 floor of this system {st['floor']:.3e}",
                              RuntimeWarning, stacklevel=2)
        return U
