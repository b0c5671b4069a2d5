"""GPU modal solve: drop-in for ``SOLVE_eigen.Eigen_solver`` (SOLVE_eigen.py:9-89).

The reference runs a shift-invert block Lanczos for K x = lambda M x on the CPU: Pardiso
factorises K once (SOLVE_eigen.py:30-32) and every step applies K^-1 M to a block of
``num_block`` vectors, with two passes of full M-orthogonal reorthogonalisation, then the
block-tridiagonal projection is diagonalised (lambda = 1 / eig(T)) and the frequencies are
sqrt(lambda) / 2 pi.

Here every vector lives in HBM: M is applied as a BSR SpMM (the scalar-per-block mass matrix
expanded to diagonal 3x3 blocks), each K^-1 M u is one multi-right-hand-side PCG solve of the
whole block (FP32 inner solves inside FP64 refinement, ``fem_pcg_solve`` with the block padded
to the next supported count; preconditioned by the multigrid V-cycle by default, or block
Jacobi), and the reorthogonalisation products are tall-skinny FP64 kernels on the device
(fem_ts_gemm_tn / fem_ts_gemm_nn).  Only the (2 num_eigen)^2 projection T is diagonalised on the host.

``Eigen_solver(Model).Solve_cpu(num_eigen, num_block)`` keeps the reference's signature and
returns (freq (num_eigen,), vectors (3N, num_eigen)); it runs the GPU path (there is no CPU
path).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import FemBsr, FEM_F64
from .model import _dptr
from .solve import DeviceSystem, padded_nrhs


class _TallSkinny:
    """FP64 products of a tall block Q (n x m, unit column stride) on the device through
    fem_ts_gemm_tn / fem_ts_gemm_nn: Q^T X and W = beta W + alpha Q C, split into launches of
    at most 256 columns of Q and 32 columns of X / W.  The FP64 pipe bounds them; they
    replace library GEMMs whose tall-skinny shapes ran far below it."""

    def __init__(self, lib, n: int, device, stream):
        self.lib, self.stream = lib, stream
        self.ws_bytes = int(lib.fem_ts_gemm_tn_workspace_bytes(n, 256, 32))
        self.ws = torch.empty(self.ws_bytes // 8 + 1, dtype=torch.float64, device=device)

    @staticmethod
    def _rows(A: torch.Tensor) -> torch.Tensor:
        return A if A.stride(1) == 1 else A.contiguous()

    def tn(self, Q: torch.Tensor, X: torch.Tensor) -> torch.Tensor:
        Q, X = self._rows(Q), self._rows(X)
        n, m = Q.shape
        b = X.shape[1]
        C = torch.empty((m, b), dtype=torch.float64, device=Q.device)
        for j0 in range(0, m, 256):
            for c0 in range(0, b, 32):
                _lib.check(self.lib.fem_ts_gemm_tn(n, min(256, m - j0), min(32, b - c0), Q.data_ptr() + 8 * j0,
                                                   Q.stride(0), X.data_ptr() + 8 * c0, X.stride(0),
                                                   C.data_ptr() + 8 * (j0 * b + c0), b, _dptr(self.ws),
                                                   self.ws_bytes, self.stream), "fem_ts_gemm_tn")
        return C

    def nn(self, Q: torch.Tensor, C: torch.Tensor, W: torch.Tensor, alpha: float, beta: float) -> torch.Tensor:
        """W = beta W + alpha Q C in place (W must have unit column stride)."""
        Q, C = self._rows(Q), self._rows(C)
        if W.stride(1) != 1:
            raise ValueError("W needs unit column stride")
        n, m = Q.shape
        b = C.shape[1]
        for c0 in range(0, b, 32):
            for j0 in range(0, m, 256):
                _lib.check(self.lib.fem_ts_gemm_nn(n, min(256, m - j0), min(32, b - c0), Q.data_ptr() + 8 * j0,
                                                   Q.stride(0), C.data_ptr() + 8 * (j0 * C.stride(0) + c0),
                                                   C.stride(0), alpha, beta if j0 == 0 else 1.0,
                                                   W.data_ptr() + 8 * c0, W.stride(0), self.stream),
                           "fem_ts_gemm_nn")
        return W


class _PhaseTimes:
    """Accumulates device time per phase with CUDA events on the launch stream (read once at
    the end of the solve) and host time for host-side phases."""

    def __init__(self, device):
        self.device = device
        self.pairs = {}
        self.host = {}

    def device_phase(self, name):
        t = self

        class _Ctx:
            def __enter__(self_):
                s = torch.cuda.current_stream(t.device)
                self_.e0 = torch.cuda.Event(enable_timing=True)
                self_.e1 = torch.cuda.Event(enable_timing=True)
                self_.e0.record(s)

            def __exit__(self_, *a):
                self_.e1.record(torch.cuda.current_stream(t.device))
                t.pairs.setdefault(name, []).append((self_.e0, self_.e1))
        return _Ctx()

    def host_phase(self, name):
        import time
        t = self

        class _Ctx:
            def __enter__(self_):
                self_.t0 = time.perf_counter()

            def __exit__(self_, *a):
                t.host[name] = t.host.get(name, 0.0) + time.perf_counter() - self_.t0
        return _Ctx()

    def result_ms(self):
        torch.cuda.synchronize(self.device)
        out = {k: sum(a.elapsed_time(b) for a, b in v) for k, v in self.pairs.items()}
        out.update({k: 1e3 * v for k, v in self.host.items()})
        return out


class Eigen_solver:
    """Drop-in for SOLVE_eigen.Eigen_solver (Qtype 0)."""

    def __init__(self, Model, Qtype=0):
        self.Qtype = Qtype
        self.Model = Model
        self.system = None
        self.last_stats = None
        self._Mb = None

    def _system(self) -> DeviceSystem:
        if self.system is None:
            self.system = DeviceSystem(self.Model)
        return self.system

    def _mass_operator(self):
        """M as FP64 BSR with diagonal 3x3 blocks m_ij I (same pattern as K)."""
        if self._Mb is None:
            S = self._system()
            _, M, _ = self.Model.assemble(K=False, M=True, F=False, m_layout="bsr")
            Mb = torch.zeros((S.nnzb, 3, 3), dtype=torch.float64, device=S.device)
            for i in range(3):
                Mb[:, i, i] = M
            self._Mb = Mb
            self._AM = FemBsr(S.n, S.nnzb, self.Model.mesh.indptr.data_ptr(), self.Model.mesh.indices.data_ptr(),
                              Mb.data_ptr(), FEM_F64, _lib.LAYOUT_BSR)
        return self._AM

    def _apply_M(self, X: torch.Tensor) -> torch.Tensor:
        """M X for an (n, b) block (b padded to a supported right-hand-side count; blocks wider
        than 32 columns are applied 32 at a time)."""
        if X.shape[1] > 32:
            return torch.cat([self._apply_M(X[:, j:j + 32]) for j in range(0, X.shape[1], 32)], 1)
        S = self._system()
        A = self._mass_operator()
        b = X.shape[1]
        R = padded_nrhs(b)
        Xp = X if R == b else torch.cat([X, X.new_zeros((X.shape[0], R - b))], 1)
        Xp = Xp.contiguous()
        Y = torch.empty_like(Xp)
        _lib.check(S.lib.fem_bsr_spmv(ctypes.byref(A), R, _dptr(Xp), _dptr(Y), 0, S.stream), "fem_bsr_spmv (M)")
        return Y[:, :b]

    def Solve_gpu(self, num_eigen=100, num_block=10, rtol=1e-11, seed=0, u0=None, mixed=True, precond="amg"):
        """Block Lanczos (SOLVE_eigen.py:45-89) on the device.  Returns (lambda (num_eigen,),
        vectors (3N, num_eigen)) as device tensors, lambda ascending.  precond: "amg"
        (multigrid V-cycle, built once per solver) or "bj" (block Jacobi) for the K solves."""
        if precond not in ("amg", "bj"):
            raise ValueError("precond must be 'amg' or 'bj'")
        pc = "amg" if precond == "amg" else None
        if self.Qtype != 0:
            raise NotImplementedError("only the linear modal problem (Qtype 0) is built")
        S = self._system()
        n = 3 * S.n
        b = int(num_block)
        m = 2 * int(num_eigen)
        steps = int(m / b)
        if b < 1 or b > 32 or steps < 1:
            raise ValueError("need 1 <= num_block <= 32 and 2*num_eigen >= num_block")
        dev = S.device
        if u0 is None:
            u0 = np.random.default_rng(seed).uniform(size=(n, b))
        u = torch.as_tensor(np.asarray(u0, dtype=np.float64), device=dev).reshape(n, b)
        Q = torch.zeros((n, m), dtype=torch.float64, device=dev)
        T = np.zeros((m, m))
        ts = _TallSkinny(S.lib, n, dev, S.stream)
        ph = _PhaseTimes(dev)
        with ph.device_phase("m_products"):
            Mu = self._apply_M(u)
        with ph.device_phase("cholesky"):
            v = torch.linalg.cholesky(ts.tn(u, Mu)).T                  # upper, u^T M u = v^T v
            u = torch.linalg.solve_triangular(v, u, upper=True, left=False)
        Q[:, :b] = u
        iters = 0
        for i in range(steps):
            Qs = Q[:, i * b:(i + 1) * b]                                # = u
            with ph.device_phase("m_products"):
                Mu = self._apply_M(Qs)
            with ph.device_phase("k_solves"):
                w, st = S.solve(F=Mu, rtol=rtol, mixed=mixed, precond=pc)
            if st["status"] != 0:
                raise _lib.FemError(st["status"], f"K solve of Lanczos step {i}: {st['status_text']}")
            iters += st["iterations"]
            w = w.reshape(n, b).contiguous()
            with ph.device_phase("m_products"):
                Mw = self._apply_M(w)
            with ph.device_phase("reorth_gemms"):
                Tii = ts.tn(Qs, Mw)
                ts.nn(Qs, Tii, w, -1.0, 1.0)                            # w -= u Tii
            with ph.host_phase("host_copies_eigh"):
                T[i * b:(i + 1) * b, i * b:(i + 1) * b] = Tii.cpu().numpy()
            if i >= steps - 1:
                break
            Qi = Q[:, :(i + 1) * b]
            for _ in range(2):
                with ph.device_phase("m_products"):
                    Mw = self._apply_M(w)
                with ph.device_phase("reorth_gemms"):
                    ts.nn(Qi, ts.tn(Qi, Mw), w, -1.0, 1.0)              # w -= Qi (Qi^T M w)
            with ph.device_phase("m_products"):
                Mw = self._apply_M(w)
            with ph.device_phase("cholesky"):
                t = torch.linalg.cholesky(ts.tn(w, Mw)).T
                u = torch.linalg.solve_triangular(t, w, upper=True, left=False)
            with ph.host_phase("host_copies_eigh"):
                tn = t.cpu().numpy()
            T[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b] = tn
            T[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = tn.T
            Q[:, (i + 1) * b:(i + 2) * b] = u
        with ph.host_phase("host_copies_eigh"):
            ev, vec = np.linalg.eigh(T)
        lam = 1.0 / ev
        order = np.argsort(lam)[:num_eigen]
        with ph.device_phase("reorth_gemms"):
            V = torch.as_tensor(np.ascontiguousarray(vec[:, order]), device=dev)
            X = ts.nn(Q, V, torch.empty((n, num_eigen), dtype=torch.float64, device=dev), 1.0, 0.0)
        self.last_stats = {"steps": steps, "solve_iterations": iters, "phase_ms": ph.result_ms()}
        return torch.as_tensor(lam[order], device=dev), X

    def Solve_cpu(self, num_eigen=100, num_block=10):
        """SOLVE_eigen.py:14-43 signature: returns (freq (num_eigen,), vectors (3N, num_eigen))
        as numpy arrays, freq = sqrt(lambda) / 2 pi (SOLVE_eigen.py:36)."""
        lam, X = self.Solve_gpu(num_eigen=num_eigen, num_block=num_block)
        freq = torch.sqrt(lam) / 2 / np.pi
        return freq.cpu().numpy(), X.cpu().numpy()
