"""fem_stress_noalloc: stress recovery for callers that may not allocate device memory.

Such callers (a plug-in inside a host program that owns every device buffer, or a loop in
which cudaMalloc/cudaFree are not allowed because they synchronise the device) pass only
their inputs and outputs; the per-element scratch comes from an array built into the
library.  This file checks, through the C ABI, that two calls in a row give the same
stresses as the workspace-taking fem_stress (same tolerance as the other stress tests:
per node, deviation <= 1e-10 x the node's largest |value|), and that meshes beyond the
built-in limit are refused.  It is named so that pytest collects it last.
"""
import ctypes
import re
import os

import numpy as np
import pytest
import torch

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.model import DeviceMesh, material
from fem_taichi_gb300.post import extrapolation_table
from tests.fixtures import STEEL, mesh2_physics

REL = 1e-10
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def max_elems_from_header():
    src = open(os.path.join(ROOT, "include", "fem_gb300.h")).read()
    return int(re.search(r"#define FEM_STRESS_NOALLOC_MAX_ELEMS (\d+)", src).group(1))


def _stress_pair(P, u, L):
    mesh = DeviceMesh(P)
    mat = material(STEEL, (0.0, 0.0, 0.0))
    W = np.ascontiguousarray(extrapolation_table("written"))
    Wp = W.ctypes.data_as(ctypes.c_void_p)
    ud = torch.from_numpy(u).cuda()
    out_ref = torch.empty((P.Num_Node, 10), dtype=torch.float64, device="cuda")
    out_na = torch.full((P.Num_Node, 10), float("nan"), dtype=torch.float64, device="cuda")
    nb = int(L.fem_stress_workspace_bytes(P.Num_Elem))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.fem_stress(ctypes.byref(mesh.c), ctypes.byref(mat), ctypes.c_void_p(ud.data_ptr()),
                      ctypes.c_void_p(mesh.co_elem.data_ptr()), Wp, ctypes.c_void_p(out_ref.data_ptr()),
                      ctypes.c_void_p(ws.data_ptr()), nb, s)
    assert rc == 0, L.fem_last_error()
    rc = L.fem_stress_noalloc(ctypes.byref(mesh.c), ctypes.byref(mat), ctypes.c_void_p(ud.data_ptr()),
                              ctypes.c_void_p(mesh.co_elem.data_ptr()), Wp, ctypes.c_void_p(out_na.data_ptr()), s)
    assert rc == 0, L.fem_last_error()
    torch.cuda.synchronize()
    return out_ref.cpu().numpy(), out_na.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_workspace_entry_point_on_two_calls_in_a_row():
    L = _lib.load()
    rng = np.random.default_rng(11)
    # first call: the reference's mesh fixture; second call: a larger block, so the shared
    # scratch still holds the first call's records when the second call starts
    for P in (mesh2_physics(), F.hex_block(30, 24, 10, jitter=0.1, seed=3, fix="zmin")):
        assert P.Num_Elem <= max_elems_from_header()
        u = rng.uniform(-1e-3, 1e-3, size=(P.Num_Node, 3))
        ref, na = _stress_pair(P, u, L)
        scale = np.abs(ref).max(axis=1, keepdims=True)
        assert np.all(np.abs(na - ref) <= REL * scale)


@pytest.mark.gpu
def test_noalloc_rejects_meshes_above_the_limit():
    L = _lib.load()
    limit = max_elems_from_header()
    m = _lib.FemMesh(8, limit + 1, 8, 0, 0, 0, 0, 0, 0)
    mat = material(STEEL, (0.0, 0.0, 0.0))
    rc = L.fem_stress_noalloc(ctypes.byref(m), ctypes.byref(mat), None, None, None, None, None)
    assert rc == _lib.FEM_ERR_WORKSPACE
    assert b"limit" in L.fem_last_error()
