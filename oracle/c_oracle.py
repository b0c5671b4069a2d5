"""ctypes binding of the C restatement (oracle/fem_oracle.c) -- test infrastructure only.

Used by tests (cross-check of the numpy oracle) and by bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libfem_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(
            os.path.join(_HERE, "fem_oracle.c")):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        D = ctypes.c_double
        L.oracle_assemble.argtypes = [I64, I64, P, P, P, P, D, D, D, P, I64, P, P, I64, P, P, P, P, P,
                                      ctypes.c_int]
        L.oracle_assemble.restype = ctypes.c_int
        L.oracle_stress.argtypes = [I64, I64, P, P, P, D, D, P, P, P, ctypes.c_int]
        L.oracle_stress.restype = ctypes.c_int
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def assemble(xyz, conn, indptr, indices, mat, omega, bound_node=None, bound_code=None,
             force_node=None, force_val=None, nthreads=1, out=None):
    """Returns (K [nnzb,3,3], M [nnzb], F [N,3]) from the C restatement (``out`` may hold
    preallocated (K, M, F) arrays to reuse)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    indptr = np.ascontiguousarray(indptr, dtype=np.int32)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    N, E = xyz.shape[0], conn.shape[0]
    nnzb = int(indptr[-1])
    bn = np.ascontiguousarray(bound_node if bound_node is not None else np.zeros(0), dtype=np.int32)
    bc = np.ascontiguousarray(bound_code if bound_code is not None else np.zeros((0, 3)), dtype=np.float64)
    fn = np.ascontiguousarray(force_node if force_node is not None else np.zeros(0), dtype=np.int32)
    fv = np.ascontiguousarray(force_val if force_val is not None else np.zeros((0, 3)), dtype=np.float64)
    om = np.ascontiguousarray(omega, dtype=np.float64)
    K, M, F = out if out is not None else (np.empty((nnzb, 3, 3)), np.empty(nnzb), np.empty((N, 3)))
    rc = lib().oracle_assemble(N, E, _p(xyz), _p(conn), _p(indptr), _p(indices),
                               mat['DE'], mat['EX'], mat['PO'], _p(om),
                               bn.size, _p(bn), _p(bc), fn.size, _p(fn), _p(fv),
                               _p(K), _p(M), _p(F), int(nthreads))
    if rc != 0:
        raise ValueError("oracle_assemble: element node pair missing from pattern")
    return K, M, F


def stress(xyz, conn, co_elem, mat, u, W, nthreads=1):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    co = np.ascontiguousarray(co_elem, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
    W = np.ascontiguousarray(W, dtype=np.float64)
    out = np.empty((xyz.shape[0], 10))
    rc = lib().oracle_stress(xyz.shape[0], conn.shape[0], _p(xyz), _p(conn), _p(co), mat['EX'],
                             mat['PO'], _p(u), _p(W), _p(out), int(nthreads))
    if rc != 0:
        raise MemoryError("oracle_stress")
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())
