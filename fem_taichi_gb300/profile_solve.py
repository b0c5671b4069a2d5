"""One warm multigrid-preconditioned static solve bracketed by cudaProfilerStart/Stop, for
launch-list captures with ``ncu --profile-from-start off`` (the summary under profiles/ names
the exact command).  ``python -m fem_taichi_gb300.profile_solve c3 [nrhs]``."""
from __future__ import annotations

import sys

import torch

from . import mesh as _mesh
from . import study
from .model import Model
from .solve import DeviceSystem


def main(cfg="c3", nrhs=1):
    P = _mesh.config_mesh(cfg)
    extra = _mesh.face_traction_loads(P, "zmax", (0.0, 0.0, -1.0))
    S = DeviceSystem(Model(cfg, P, study.STEEL, extra_loads=extra))
    S.amg()
    F = S.F if nrhs == 1 else S.F.reshape(-1, 1).repeat(1, nrhs).contiguous()
    U, st = S.solve(F=F, rtol=1e-10, mixed=False, precond="amg")
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    U, st = S.solve(F=F, rtol=1e-10, mixed=False, precond="amg")
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print({k: st[k] for k in ("status", "iterations", "relres", "time_ms")})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "c3", int(sys.argv[2]) if len(sys.argv) > 2 else 1)
