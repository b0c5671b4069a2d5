"""Runs the reference's own FE code (tianshao1992/FEM_taichi) unmodified on the CPU --
TEST INFRASTRUCTURE ONLY.

``load(ref_root)`` imports ``READ_physics.py``, ``FEM_model_csr.py``, ``FEM_model_bsr.py`` and
``POST_process.py`` from a reference checkout, with

* the Taichi 0.6.28 stand-in (``oracle/refexec/taichi``) and a pandas import stub
  (``oracle/refexec/pandas``) first on ``sys.path``;
* ``numpy.int`` restored as an alias of ``int`` (numpy 2 removed it; the reference uses it at
  READ_physics.py:48-51 and FEM_model_*.py:78);
* ``ctypes.cdll.LoadLibrary`` replaced, only while ``POST_process`` is imported, by a loader
  that returns a placeholder: POST_process.py:11-12 loads a Windows Tecplot DLL at import
  time.  The placeholder loads nothing and raises if the binary-output path is called.

The other functions drive the reference classes the way ``run_main.py:26-45`` does:
``Read.pre_process`` (READ_physics.py:42-61) builds the topology from arrays (the pandas file
readers are not used), ``Model.Get_MatrixKL / Get_MatrixM / Get_VectorF`` assemble,
``Model(FEM_model_bsr).LDinit + Get_MatrixKN`` builds the large-displacement matrices, and
``Post.Get_Stress`` recovers nodal stresses.  This module is used only to generate the golden
fixtures under ``tests/golden/`` and by the CPU test that re-checks one of them.
"""
from __future__ import annotations

import contextlib
import ctypes
import importlib
import io
import os
import sys
import tempfile

import numpy as np

STANDIN = os.path.dirname(os.path.abspath(__file__))
MODULES = ("READ_physics", "FEM_model_csr", "FEM_model_bsr", "POST_process")


class _NoLibrary:
    def __init__(self, path):
        self._path = path

    def __getattr__(self, name):
        raise RuntimeError("the reference's native Tecplot DLL (%s) is not available" % self._path)


def load(ref_root: str) -> dict:
    """Imports the reference modules from ``ref_root`` (unmodified) and returns them by name."""
    ref_root = os.path.abspath(ref_root)
    for p in (ref_root, STANDIN):
        if p in sys.path:
            sys.path.remove(p)
        sys.path.insert(0, p)
    if not hasattr(np, "int"):
        np.int = int
    import taichi
    if not getattr(taichi, "__version__", "").endswith("standin"):
        raise RuntimeError("a real taichi is importable; the stand-in must be the one loaded")
    mods = {}
    orig = ctypes.cdll.__dict__.get("LoadLibrary")
    ctypes.cdll.LoadLibrary = _NoLibrary
    try:
        with contextlib.redirect_stdout(io.StringIO()):
            for name in MODULES:
                mods[name] = importlib.import_module(name)
    finally:
        if orig is None:
            del ctypes.cdll.LoadLibrary
        else:
            ctypes.cdll.LoadLibrary = orig
    for name in MODULES:
        f = os.path.abspath(mods[name].__file__)
        if os.path.dirname(f) != ref_root:
            raise RuntimeError("%s was imported from %s, not from the reference tree" % (name, f))
    return mods


def physics(mods, node_ids, xyz, elem, bounds=(), forces=()):
    """A reference ``Read`` object whose topology comes from its own ``pre_process``.

    node_ids: (N,) 1-based ids; xyz: (N, 3); elem: (8, E) node ids - 1 in corner order (the
    reader's ``Elem`` rows, READ_physics.py:96); bounds / forces: lists of [ids - 1, [3 values]]
    as the reader builds them (READ_physics.py:114, 134)."""
    Read = mods["READ_physics"].Read
    R = Read.__new__(Read)
    node = np.zeros((6, len(node_ids)), dtype=np.float64)
    node[0] = np.asarray(node_ids, dtype=np.float64)
    node[3:] = np.asarray(xyz, dtype=np.float64).T
    R.name = "fixture"
    R.Node = node
    R.Elem = np.asarray(elem, dtype=np.int64)
    with contextlib.redirect_stdout(io.StringIO()):
        R.pre_process()
    R.Bounds = [[np.asarray(ids, dtype=np.int64), list(c)] for ids, c in bounds]
    R.Forces = [[np.asarray(ids, dtype=np.int64), list(v)] for ids, v in forces]
    return R


def model_csr(mods, R, materials, omegas):
    """FEM_model_csr.Model: K (CSR written in place), M, F -- first calls, as run_main.py does."""
    with contextlib.redirect_stdout(io.StringIO()):
        m = mods["FEM_model_csr"].Model("fixture", R, materials, Omegas=omegas, Largedisp=False)
        K = m.Get_MatrixKL()
        M = m.Get_MatrixM()
        F = m.Get_VectorF()
    return K, M, F


def model_bsr_K(mods, R, materials, omegas):
    """FEM_model_bsr.Model.Get_MatrixKL: the BSR assembly converted with bsr.tocsr()."""
    with contextlib.redirect_stdout(io.StringIO()):
        m = mods["FEM_model_bsr"].Model("fixture", R, materials, Omegas=omegas, Largedisp=False)
        return m.Get_MatrixKL()


def model_bsr_tangent(mods, R, materials, omegas, u):
    """FEM_model_bsr.Model: LDinit(u) then Get_MatrixKN() -> (KT, KM) CSR."""
    with contextlib.redirect_stdout(io.StringIO()):
        m = mods["FEM_model_bsr"].Model("fixture", R, materials, Omegas=omegas, Largedisp=True)
        m.LDinit(np.asarray(u, dtype=np.float64).reshape(-1))
        return m.Get_MatrixKN()


@contextlib.contextmanager
def _scratch_cwd():
    # Post.__init__ creates "Results\<name>\" under the working directory (POST_process.py:20-22)
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            yield
        finally:
            os.chdir(old)


def post_stress(mods, R, materials, u):
    """POST_process.Post(...).Get_Stress() -> (N, 10); u is (N, 3) node-major."""
    sol = np.asarray(u, dtype=np.float64).reshape(-1, 3, 1)
    with _scratch_cwd(), contextlib.redirect_stdout(io.StringIO()):
        p = mods["POST_process"].Post("fixture", R, materials, sol)
        return p.Get_Stress()


def post_nodal_vector(mods, R, materials, u):
    """The six averaged nodal components before the eigen-decomposition: the reference's own
    get_NdSol + get_NdAve kernels (POST_process.py:172-187) and the reshaping of
    Get_Stress (:79).  Used where Get_Stress itself raises (a node with no element gives 0/0,
    and numpy's eigh rejects the NaN tensor)."""
    sol = np.asarray(u, dtype=np.float64).reshape(-1, 3, 1)
    with _scratch_cwd(), contextlib.redirect_stdout(io.StringIO()):
        p = mods["POST_process"].Post("fixture", R, materials, sol)
        p.get_NdSol(p.Num_Elem)
        p.get_NdAve(p.Num_Node)
        return p.Stress.to_numpy().transpose((1, 0, 2)).reshape((-1, 6))
