"""Learned correction of the block-Jacobi preconditioner, trained on the GPU.

For every node i with diagonal block D_i = G_i G_i^T, a per-node MLP (16 -> 64 -> 64 -> 6,
SiLU, BF16 weights, FP32 accumulation on the tensor cores) maps scale-free node features
to the Cholesky factor L_i of an SPD 3x3 matrix C_i, and the PCG preconditioner block is
P_i = G_i^{-T} L_i L_i^T G_i^{-1}.  With the last layer at zero, C_i = I and P_i is the
block-Jacobi inverse D_i^{-1} exactly, which is where training starts.

Training data are Gaussian probe vectors zhat ~ N(0, I) and their products
yhat = G^{-1} K G^{-T} zhat generated by the assembled operator itself (BSR SpMM); the loss
is mean_{i,r} |C_i yhat_ir - zhat_ir|^2, i.e. C should act as the inverse of the
block-scaled operator on the probes.  Forward: ``fem_mlp_forward`` (tcgen05); backward:
``fem_mlp_backward_tc`` (tcgen05, BF16 operands, FP32 accumulation; ``backward(...,
tensor_cores=False)`` runs the FP32 CUDA-core kernel ``fem_mlp_backward``); both reduce their
per-CTA partials in a fixed order (deterministic); optimiser: Adam on FP32 masters.

``LearnedSmoother`` is the second learned form, not block-diagonal: per-level Chebyshev
smoother weights of the multigrid V-cycle fitted on the same training family.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import FemMlp
from .model import _dptr, _stream

N_IN, N_HID, N_OUT = 16, 64, 16
N_PARAMS = N_HID * N_IN + N_HID + N_HID * N_HID + N_HID + N_OUT * N_HID + N_OUT


def _bf16_bits(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).view(torch.int16)


class NodeData:
    """Features and probe pairs of one assembled system (all on the device)."""

    def __init__(self, system, n_probes=8, seed=0, with_probes=True):
        L = _lib.load()
        m = system.model
        dev = system.device
        st = _stream(dev)
        n = system.n
        self.n = n
        self.ginv = torch.empty((n, 9), dtype=torch.float64, device=dev)
        bad = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.check(L.fem_precond_cholesky(ctypes.byref(system.A64), _dptr(self.ginv), _dptr(bad), st),
                   "fem_precond_cholesky")
        if int(bad.item()):
            raise _lib.FemError(_lib.FEM_ERR_NOT_SPD, f"{int(bad.item())} diagonal blocks are not SPD")
        xyz = m.mesh.xyz
        lo = xyz.min(0).values.double().cpu().numpy().copy()
        hi = xyz.max(0).values.double().cpu().numpy().copy()
        self.X = torch.empty((n, N_IN), dtype=torch.int16, device=dev)
        _lib.check(L.fem_precond_features(ctypes.byref(system.A64), _dptr(self.ginv), _dptr(xyz), _dptr(m.fixed),
                                          lo.ctypes.data_as(ctypes.c_void_p), hi.ctypes.data_as(ctypes.c_void_p),
                                          _dptr(self.X), None, st), "fem_precond_features")
        self.R = n_probes
        self.yhat = self.zhat = None
        if with_probes:
            g = torch.Generator(device=dev)
            g.manual_seed(seed)
            z = torch.randn((n, 3, n_probes), dtype=torch.float64, device=dev, generator=g)
            w = torch.empty_like(z)
            y = torch.empty_like(z)
            self.yhat = torch.empty((n, 3, n_probes), dtype=torch.float32, device=dev)
            _lib.check(L.fem_probe_products(ctypes.byref(system.A64), n_probes, _dptr(self.ginv), _dptr(z), _dptr(w),
                                            _dptr(y), _dptr(self.yhat), st), "fem_probe_products")
            self.zhat = z.float()


class LearnedPreconditioner:
    """Per-node MLP producing SPD corrections of the block-Jacobi inverse."""

    def __init__(self, device="cuda", seed=0):
        self.lib = _lib.load()
        self.device = torch.device(device)
        g = np.random.default_rng(seed)
        p = np.zeros(N_PARAMS, dtype=np.float32)
        o = 0
        p[o:o + N_HID * N_IN] = g.standard_normal(N_HID * N_IN) * np.sqrt(1.0 / N_IN); o += N_HID * N_IN + N_HID
        p[o:o + N_HID * N_HID] = g.standard_normal(N_HID * N_HID) * np.sqrt(1.0 / N_HID); o += N_HID * N_HID + N_HID
        # last layer zero: C = I, i.e. plain block Jacobi
        self.params = torch.from_numpy(p).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self._bf16 = None
        self._refresh_bf16()

    # -- weights --------------------------------------------------------------------------
    def _views(self, t):
        o = 0
        out = []
        for shape in ((N_HID, N_IN), (N_HID,), (N_HID, N_HID), (N_HID,), (N_OUT, N_HID), (N_OUT,)):
            k = int(np.prod(shape))
            out.append(t[o:o + k].view(shape))
            o += k
        return out

    def _refresh_bf16(self):
        W1, b1, W2, b2, W3, b3 = self._views(self.params)
        self._bf16 = [_bf16_bits(W1).contiguous(), _bf16_bits(W2).contiguous(), _bf16_bits(W3).contiguous()]

    def net(self) -> FemMlp:
        W1, b1, W2, b2, W3, b3 = self._views(self.params)
        return FemMlp(self._bf16[0].data_ptr(), b1.data_ptr(), self._bf16[1].data_ptr(), b2.data_ptr(),
                      self._bf16[2].data_ptr(), b3.data_ptr())

    def state_dict(self):
        return {"params": self.params.cpu().numpy().copy(), "step": self.step}

    def load_state_dict(self, d):
        self.params.copy_(torch.as_tensor(d["params"], dtype=torch.float32))
        self.step = int(d.get("step", 0))
        self._refresh_bf16()

    def save(self, path):
        np.savez(path, **self.state_dict())

    def load(self, path):
        d = np.load(path)
        self.load_state_dict({k: d[k] for k in d.files})

    # -- kernels ----------------------------------------------------------------------------
    def forward(self, X: torch.Tensor, save=False):
        n = X.shape[0]
        out = torch.empty((n, N_OUT), dtype=torch.float32, device=self.device)
        z1 = torch.empty((n, N_HID), dtype=torch.float32, device=self.device) if save else None
        z2 = torch.empty((n, N_HID), dtype=torch.float32, device=self.device) if save else None
        err = torch.zeros(1, dtype=torch.int32, device=self.device)
        net = self.net()
        _lib.check(self.lib.fem_mlp_forward(ctypes.byref(net), _dptr(X), n, _dptr(out), _dptr(z1), _dptr(z2),
                                            _dptr(err), _stream(self.device)), "fem_mlp_forward")
        if int(err.item()):
            raise _lib.FemError(_lib.FEM_ERR_CUDA, "tensor-core forward timed out waiting on its mbarrier")
        return out, z1, z2

    def loss_and_grad(self, data: NodeData, out):
        n = data.n
        dout = torch.empty_like(out)
        part = torch.empty(1024, dtype=torch.float64, device=self.device)
        npart = ctypes.c_int(0)
        _lib.check(self.lib.fem_mlp_loss_grad(_dptr(out), _dptr(data.yhat), _dptr(data.zhat), data.R, n, _dptr(dout),
                                              _dptr(part), ctypes.byref(npart), _stream(self.device)),
                   "fem_mlp_loss_grad")
        loss = part[:npart.value].sum() / (n * data.R)
        return loss, dout

    def backward(self, X, z1, z2, dout, tensor_cores=True):
        n = X.shape[0]
        grad = torch.empty(N_PARAMS, dtype=torch.float32, device=self.device)
        if tensor_cores:
            nb = int(self.lib.fem_mlp_backward_tc_workspace_bytes(n))
            ws = torch.empty(nb, dtype=torch.uint8, device=self.device)
            err = torch.zeros(1, dtype=torch.int32, device=self.device)
            _lib.check(self.lib.fem_mlp_backward_tc(_dptr(self.params), _dptr(X), _dptr(z1), _dptr(z2), _dptr(dout),
                                                    n, _dptr(grad), _dptr(ws), nb, _dptr(err), _stream(self.device)),
                       "fem_mlp_backward_tc")
            if int(err.item()):
                raise _lib.FemError(_lib.FEM_ERR_CUDA, "tensor-core backward timed out waiting on its mbarrier")
            return grad
        nb = int(self.lib.fem_mlp_backward_workspace_bytes(n))
        ws = torch.empty(nb, dtype=torch.uint8, device=self.device)
        _lib.check(self.lib.fem_mlp_backward(_dptr(self.params), _dptr(X), _dptr(z1), _dptr(z2), _dptr(dout), n,
                                             _dptr(grad), _dptr(ws), nb, _stream(self.device)), "fem_mlp_backward")
        return grad

    def adam(self, grad, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        _lib.check(self.lib.fem_mlp_adam(_dptr(self.params), _dptr(grad), _dptr(self.m), _dptr(self.v), self.step,
                                         lr, beta1, beta2, eps, _dptr(self._bf16[0]), _dptr(self._bf16[1]),
                                         _dptr(self._bf16[2]), _stream(self.device)), "fem_mlp_adam")

    def train(self, datasets, steps=300, lr=2e-3, log_every=50):
        """Full-batch Adam over the concatenated nodes of ``datasets`` (list of NodeData);
        returns the loss history (one entry per step)."""
        hist = []
        for it in range(steps):
            grads = None
            total = 0.0
            for d in datasets:
                out, z1, z2 = self.forward(d.X, save=True)
                loss, dout = self.loss_and_grad(d, out)
                w = d.n / sum(x.n for x in datasets)
                g = self.backward(d.X, z1, z2, dout * w)
                grads = g if grads is None else grads + g
                total += float(loss) * w
            self.adam(grads, lr=lr)
            hist.append(total)
        return hist

    def evaluate_loss(self, datasets):
        tot, cnt = 0.0, 0
        for d in datasets:
            out, _, _ = self.forward(d.X)
            loss, _ = self.loss_and_grad(d, out)
            tot += float(loss) * d.n
            cnt += d.n
        return tot / cnt

    def blocks(self, system, data: NodeData | None = None) -> torch.Tensor:
        """(N, 9) FP64 preconditioner blocks for ``system`` (a DeviceSystem)."""
        data = data or NodeData(system, with_probes=False)
        out, _, _ = self.forward(data.X)
        P = torch.empty((data.n, 9), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.fem_learned_blocks(data.n, _dptr(out), _dptr(data.ginv), _dptr(P), _stream(self.device)),
                   "fem_learned_blocks")
        return P


class LearnedSmoother:
    """Learned smoother weights of the multigrid V-cycle: a non-block-diagonal learned
    preconditioner.

    The V-cycle smooths with a Chebyshev polynomial in D^-1 A on [upper lmax / ratio,
    upper lmax] on every level (``fem_amg_opts``: one (upper, ratio) for all levels).  Here
    the first ``levels`` level indices have their own (upper_l, ratio_l) (the default, 2:
    the fine level and one pair shared by every coarser level, which keeps the weights from
    fitting the depth of the training hierarchies), learned on a family of training systems
    by minimising the mean log10 of the relative residual that the FP64 multigrid-preconditioned
    CG reaches after ``iters`` iterations on a seeded random right-hand side (a convergence
    factor, smooth in the weights).  The search is a coordinate search in log space with
    shrinking steps over the 2 x ``levels`` weights, started from the default smoother, so
    the training loss never ends above the default's.  Levels deeper than ``levels`` reuse the
    last level's weights.  ``apply(hierarchy)`` writes the weights into a hierarchy
    (``fem_amg_set_smoother``); the preconditioner stays a symmetric V-cycle (the same
    polynomial before and after the coarse correction), with upper >= 1 so the smoother does
    not amplify the top of the spectrum.
    """

    def __init__(self, levels=2, upper=1.1, ratio=30.0):
        self.upper = [float(upper)] * levels
        self.ratio = [float(ratio)] * levels
        self.history = []

    def weights(self, level):
        k = min(level, len(self.upper) - 1)
        return self.upper[k], self.ratio[k]

    def apply(self, hierarchy):
        lib = hierarchy.lib
        for l in range(int(lib.fem_amg_num_levels(hierarchy.h)) - 1):
            u, r = self.weights(l)
            _lib.check(lib.fem_amg_set_smoother(hierarchy.h, l, u, r), "fem_amg_set_smoother")
        return hierarchy

    def loss(self, cases, iters=12):
        """Mean log10 relative residual after `iters` FP64 multigrid-PCG iterations over the
        (system, hierarchy, right-hand side) cases."""
        tot = 0.0
        for S, H, F in cases:
            self.apply(H)
            _, st = S.solve(F=F, rtol=1e-30, maxit=iters, mixed=False, precond=H, max_outer=1)
            tot += float(np.log10(max(st["relres"], 1e-300)))
        return tot / len(cases)

    def fit(self, cases, iters=12, steps=(1.6, 1.25, 1.1), upper_bounds=(1.0, 1.6), ratio_bounds=(6.0, 120.0)):
        """Coordinate search from the current weights; returns (loss at start, loss at end)."""
        best = self.loss(cases, iters)
        start = best
        self.history = [best]
        for f in steps:
            for l in range(len(self.upper)):
                for name, lo, hi in (("ratio",) + tuple(ratio_bounds), ("upper",) + tuple(upper_bounds)):
                    vals = getattr(self, name)
                    cur = vals[l]
                    for cand in (min(hi, cur * f), max(lo, cur / f)):
                        if cand == cur:
                            continue
                        vals[l] = cand
                        v = self.loss(cases, iters)
                        if v < best - 1e-9:
                            best, cur = v, cand
                        else:
                            vals[l] = cur
                    self.history.append(best)
        for S, H, F in cases:
            self.apply(H)
        return start, best

    def state_dict(self):
        return {"upper": list(self.upper), "ratio": list(self.ratio)}

    def load_state_dict(self, d):
        self.upper = [float(x) for x in d["upper"]]
        self.ratio = [float(x) for x in d["ratio"]]
