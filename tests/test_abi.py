"""The C-ABI library loads and exports every entry point declared in include/*.h; argument
validation happens on the host before any device work (no GPU needed here)."""
import ctypes
import glob
import os
import re

import pytest

from fem_taichi_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(fem_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_loads_and_exports_all_declared_symbols():
    L = _lib.load()
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/ but not exported"
        assert n in _lib.SIGNATURES, f"{n} has no ctypes signature"
    assert L.fem_abi_version() >= 1


def test_workspace_sizes():
    L = _lib.load()
    assert L.fem_assemble_workspace_bytes(0) == 0
    assert L.fem_assemble_workspace_bytes(1000) == 1000 * 8 * 672
    assert L.fem_stress_workspace_bytes(10) == 10 * 48 * 8


def test_invalid_arguments_return_status():
    L = _lib.load()
    rc = L.fem_assemble(None, None, None, None, 0, None)
    assert rc == _lib.FEM_ERR_INVALID
    assert b"NULL" in L.fem_last_error()
    m = _lib.FemMesh(10, 1, 5, 0, 0, 0, 0, 0, 0)
    rc = L.fem_assemble(ctypes.byref(m), None, None, None, 0, None)
    assert rc == _lib.FEM_ERR_INVALID
    with pytest.raises(_lib.FemError):
        _lib.check(rc, "probe")
