"""GPU drop-in for the reference ``Post`` stress recovery (POST_process.py:14-99).

``Post(name, Physics, Materials, Solutions).Get_Stress()`` returns the (N, 10) float64
table [xx, yy, zz, xy, yz, xz, p1, p2, p3, VM] exactly as the reference lays it out
(POST_process.py:79-95), with the reference's extrapolation convention and "VM" formula.

Extrapolation table.  get_NdSol (POST_process.py:172-181) weights Gauss point k's stress
for element corner j by shapefunc_GS(GMat[j])[k].  GMat is assigned eight corner points
(POST_process.py:310-317) but declared with two entries (POST_process.py:145).  Taichi 0.6
(the reference's pinned runtime) lowers a dense-field index to its low bits, without a bounds
check, so entry j reads entry j & 1, which holds the last value written to it: (1, 1, -1) for
even j and (1, 1, 1) for odd j.  ``gmat_mode='aliased'`` (default) is that reading, the one
the reference's own code produces when executed; ``gmat_mode='written'`` uses the eight
assigned points (what the source appears to intend).

Arithmetic.  ``algo='fp64'`` (default) computes on the FP64 pipe; ``algo='dd'`` uses
double-float pairs on the FP32 pipes (about 48-bit significands; faster, not FP64).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _lib
from .mesh import Physics  # noqa: F401  (type reference)
from .model import DeviceMesh, _dptr, _stream, material

GS1 = 0.57735026918962
_GMAT_WRITTEN = np.array([[-1, -1, -1], [-1, -1, 1], [-1, 1, -1], [-1, 1, 1],
                          [1, -1, -1], [1, -1, 1], [1, 1, -1], [1, 1, 1]], dtype=np.float64)


def extrapolation_table(gmat_mode: str = "aliased") -> np.ndarray:
    """W[j, k] = shapefunc_GS(GMat[j])[k] (POST_process.py:212-223)."""
    if gmat_mode == "written":
        g = _GMAT_WRITTEN
    elif gmat_mode == "aliased":
        g = np.array([_GMAT_WRITTEN[6 + (j & 1)] for j in range(8)])
    else:
        raise ValueError("gmat_mode must be 'written' or 'aliased'")
    W = np.empty((8, 8))
    for j in range(8):
        a, b, c = g[j, 0] / GS1, g[j, 1] / GS1, g[j, 2] / GS1
        W[j] = [0.125 * (1 + a) * (1 + b) * (1 - c), 0.125 * (1 - a) * (1 + b) * (1 - c),
                0.125 * (1 - a) * (1 - b) * (1 - c), 0.125 * (1 + a) * (1 - b) * (1 - c),
                0.125 * (1 + a) * (1 + b) * (1 + c), 0.125 * (1 - a) * (1 + b) * (1 + c),
                0.125 * (1 - a) * (1 - b) * (1 + c), 0.125 * (1 + a) * (1 - b) * (1 + c)]
    return W


def write_tecplot_ascii(output_file, title, Physics, Fields, Field_names):
    """Tecplot ASCII FE-point file, as POST_process.py:101-135 (Output_field_ASC) writes it:
    a TITLE line, the VARIABLES line (x, y, z, then every field name per step, numbered from 1),
    the ZONE line (I = nodes, J = elements, FEPOINT, BRICK), one row per node (x y z and the
    fields of every step, '%10.5e', space separated, NaN written empty) and one row per element
    (its 8 nodes, 1-based).  Fields: (N, n_fields, n_steps)."""
    Fields = np.asarray(Fields, dtype=np.float64)
    Node = Physics.Node[-3:]
    N = Node.shape[-1]
    if Fields.ndim != 3 or Fields.shape[0] != N:
        raise ValueError("Fields must be (N, n_fields, n_steps)")
    data = np.concatenate((Node.T, Fields.transpose(0, 2, 1).reshape(N, -1)), axis=-1)
    conn = Physics.Nind[np.asarray(Physics.Elem[-8:], dtype=np.int64)].T + 1
    head = ['TITLE = "' + title + '.data"\n', 'VARIABLES = "X [ m ]","Y [ m ]","Z [m]"']
    for step in range(Fields.shape[-1]):
        for name in Field_names:
            head.append(',"' + " " + str(name) + str(step + 1) + '"')  # ("%s " % ',"') + name + step + '"'
    head.append("\n")
    head.append("ZONE  I=" + str(N) + ", J=" + str(conn.shape[0]) + ", F=FEPOINT, ET=BRICK\n")
    # one format string per row; rows holding NaN (written as empty fields) go value by value
    fmt = " ".join(["%10.5e"] * data.shape[1])
    nan_rows = np.isnan(data).any(axis=1)
    rows = data.tolist()
    lines = [(" ".join("" if v != v else "%10.5e" % v for v in r) if bad else fmt % tuple(r))
             for r, bad in zip(rows, nan_rows.tolist())]
    with open(output_file, "w") as f:
        f.write("".join(head))
        f.write("\n".join(lines))
        f.write("\n")
        f.write("\n".join(" ".join(map(str, r)) for r in conn.tolist()))
        f.write("\n")


class Post:
    """Drop-in for POST_process.Post (stress part)."""

    def __init__(self, name, Physics, Materials, Solutions, gmat_mode="aliased", device="cuda", mesh=None,
                 algo="fp64"):
        self.name = name
        self.DE, self.EX, self.PO = Materials['DE'], Materials['EX'], Materials['PO']
        self.Physics = Physics
        self.Num_Node = int(Physics.Node.shape[-1])
        self.Num_Elem = int(Physics.Elem.shape[-1])
        self.lib = _lib.load()
        self.mesh = mesh if mesh is not None else DeviceMesh(Physics, device)
        self.device = self.mesh.device
        self.mat = material(Materials, (0.0, 0.0, 0.0))
        self.W = np.ascontiguousarray(extrapolation_table(gmat_mode))
        if algo not in ("dd", "fp64"):
            raise ValueError("algo must be 'dd' or 'fp64'")
        self.algo = _lib.ALGO_DD if algo == "dd" else _lib.ALGO_FP64
        self.set_solution(Solutions)
        self._ws = None

    def set_solution(self, Solutions) -> None:
        """Solutions: (N, 3[, 1]) host array or device tensor (POST_process.py:28: squeeze().T)."""
        u = torch.as_tensor(Solutions).reshape(self.Num_Node, 3)
        self.u = u.to(device=self.device, dtype=torch.float64).contiguous()

    def stress_device(self, out: torch.Tensor | None = None) -> torch.Tensor:
        nbytes = int(self.lib.fem_stress_workspace_bytes(self.Num_Elem))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=self.device)
        if out is None:
            out = torch.empty((self.Num_Node, 10), dtype=torch.float64, device=self.device)
        W = self.W.ctypes.data_as(ctypes.c_void_p)
        _lib.check(self.lib.fem_stress_ex(ctypes.byref(self.mesh.c), ctypes.byref(self.mat), _dptr(self.u),
                                          _dptr(self.mesh.co_elem), W, _dptr(out), _dptr(self._ws),
                                          self._ws.numel(), self.algo, _stream(self.device)), "fem_stress_ex")
        return out

    def Get_Stress(self) -> np.ndarray:
        """POST_process.py:72-99."""
        return self.stress_device().cpu().numpy()

    @property
    def path(self) -> str:
        """Results directory of the reference (POST_process.py:20, "Results/<name>/")."""
        return os.path.join("Results", self.name) + os.sep

    def Output_field_ASC(self, file_name, Fields, Field_names):
        """POST_process.py:101-135: Tecplot ASCII file <path><file_name>.dat (the directory is
        created on the first write instead of in the constructor)."""
        os.makedirs(self.path, exist_ok=True)
        write_tecplot_ascii(self.path + file_name + ".dat", self.name, self.Physics, Fields, Field_names)

    def Output_field_BIN(self, file_name, Fields, Field_names):
        """POST_process.py:32-69 writes through the Windows TecIO library; not available."""
        raise NotImplementedError("binary Tecplot output needs the closed TecIO library; use Output_field_ASC")
