"""ctypes binding of ``libfemgb.so`` (the C ABI declared in ``include/fem_gb300.h``).

The library is required: importing a GPU entry point without it raises.  There is no
CPU fallback for any kernel.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

c_int64 = ctypes.c_int64
c_int = ctypes.c_int
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_size_t = ctypes.c_size_t

FEM_OK = 0
FEM_ERR_INVALID = -1
FEM_ERR_CUDA = -2
FEM_ERR_PATTERN = -3
FEM_ERR_NOT_CONVERGED = -4
FEM_ERR_MAXITER = -5
FEM_ERR_NOT_SPD = -6
FEM_ERR_WORKSPACE = -7
FEM_ERR_BREAKDOWN = -8
RESIDUAL_FP64 = 0
RESIDUAL_EXTRA = 1

LAYOUT_BSR = 0
LAYOUT_CSR = 1
LAYOUT_RSOA = 2
LAYOUT_RSOA4 = 3
ALGO_DD = 0
ALGO_FP64 = 1
FEM_F64 = 0
FEM_F32 = 1

_NAMES = {FEM_ERR_INVALID: "FEM_ERR_INVALID", FEM_ERR_CUDA: "FEM_ERR_CUDA",
          FEM_ERR_PATTERN: "FEM_ERR_PATTERN", FEM_ERR_NOT_CONVERGED: "FEM_ERR_NOT_CONVERGED",
          FEM_ERR_MAXITER: "FEM_ERR_MAXITER", FEM_ERR_NOT_SPD: "FEM_ERR_NOT_SPD",
          FEM_ERR_WORKSPACE: "FEM_ERR_WORKSPACE", FEM_ERR_BREAKDOWN: "FEM_ERR_BREAKDOWN"}


class FemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_NAMES.get(code, code)}: {msg}")
        self.code = code


class FemMesh(ctypes.Structure):
    _fields_ = [("n_node", c_int64), ("n_elem", c_int64), ("nnzb", c_int64),
                ("xyz", c_void_p), ("conn", c_void_p), ("indptr", c_void_p), ("indices", c_void_p),
                ("ne_ptr", c_void_p), ("ne_list", c_void_p), ("ne_inv", c_void_p), ("slot_map", c_void_p)]


class FemMaterial(ctypes.Structure):
    _fields_ = [("DE", c_double), ("EX", c_double), ("PO", c_double), ("omega", c_double * 3)]


class FemAssemblyOut(ctypes.Structure):
    _fields_ = [("k_layout", c_int), ("m_layout", c_int), ("K", c_void_p), ("M", c_void_p),
                ("F", c_void_p), ("fixed", c_void_p), ("loads", c_void_p), ("algo", c_int)]


class FemBsr(ctypes.Structure):
    _fields_ = [("n_brow", c_int64), ("nnzb", c_int64), ("indptr", c_void_p), ("indices", c_void_p),
                ("vals", c_void_p), ("dtype", c_int), ("layout", c_int)]


class FemPcgOpts(ctypes.Structure):
    _fields_ = [("nrhs", c_int), ("mixed", c_int), ("rtol", c_double), ("maxit", c_int), ("inner_rtol", c_double),
                ("inner_maxit", c_int), ("max_outer", c_int), ("use_graph", c_int), ("unroll", c_int),
                ("spmv_variant", c_int), ("spmv_variant32", c_int), ("residual", c_int), ("stall_window", c_int)]


class FemPcgStats(ctypes.Structure):
    _fields_ = [("status", c_int), ("iterations", c_int), ("outer", c_int), ("relres", c_double),
                ("time_ms", c_double), ("floor", c_double)]


class FemAmgOpts(ctypes.Structure):
    _fields_ = [("theta", c_double), ("max_levels", c_int), ("max_coarse", c_int), ("smooth", c_int),
                ("eig_steps", c_int), ("pre_degree", c_int), ("post_degree", c_int), ("cheb_upper", c_double),
                ("cheb_ratio", c_double)]


class FemAmgLevelInfo(ctypes.Structure):
    _fields_ = [("n", c_int64), ("b", c_int), ("nnzb_A", c_int64), ("nnzb_P", c_int64), ("lmax", c_double),
                ("omega", c_double), ("setup_s", c_double)]


class FemMlp(ctypes.Structure):
    _fields_ = [("W1", c_void_p), ("b1", c_void_p), ("W2", c_void_p), ("b2", c_void_p), ("W3", c_void_p),
                ("b3", c_void_p)]


# name -> (restype, argtypes); every exported symbol of include/fem_gb300.h
SIGNATURES = {
    "fem_last_error": (ctypes.c_char_p, []),
    "fem_abi_version": (c_int, []),
    "fem_pattern_count": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p]),
    "fem_pattern_fill": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p]),
    "fem_incidence_build": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_gather_map": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p]),
    "fem_assemble_workspace_bytes": (c_size_t, [c_int64]),
    "fem_assemble": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial),
                             ctypes.POINTER(FemAssemblyOut), c_void_p, c_size_t, c_void_p]),
    "fem_assemble_elements": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), c_int, c_void_p,
                                      c_size_t, c_void_p]),
    "fem_assemble_gather": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemAssemblyOut), c_void_p, c_size_t,
                                    c_void_p]),
    "fem_assemble_host_staged": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial),
                                         ctypes.POINTER(FemAssemblyOut), c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                         c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "fem_assemble_host": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), ctypes.POINTER(FemAssemblyOut),
                                  c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_size_t, c_void_p]),
    "fem_rsoa4_indptr": (c_int, [c_int64, c_void_p, c_void_p]),
    "fem_bsr_to_rsoa4_f32": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_topology_workspace_bytes": (c_size_t, [c_int64, c_int64]),
    "fem_topology_count_gpu": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       ctypes.POINTER(c_int64), c_void_p, c_size_t, c_void_p]),
    "fem_topology_fill_gpu": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_size_t, c_void_p]),
    "fem_tangent_workspace_bytes": (c_size_t, [c_int64]),
    "fem_assemble_tangent": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), c_void_p, c_int, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
    "fem_pipeline_plan": (c_int, [c_int64, c_int64, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p,
                                  c_void_p]),
    "fem_csr_index": (c_int, [ctypes.POINTER(FemMesh), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_bsr_spmv": (c_int, [ctypes.POINTER(FemBsr), c_int, c_void_p, c_void_p, c_int, c_void_p]),
    "fem_spmv_autotune": (c_int, [ctypes.POINTER(FemBsr), c_int, c_void_p, c_void_p, c_int, ctypes.POINTER(c_int),
                                  ctypes.POINTER(ctypes.c_float), c_void_p]),
    "fem_convert_f64_to_f32": (c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    "fem_bsr_to_rsoa_f32": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p]),
    "fem_block_jacobi": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_pcg_workspace_bytes": (c_size_t, [c_int64, c_int, c_int]),
    "fem_pcg_solve": (c_int, [ctypes.POINTER(FemBsr), ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p,
                              ctypes.POINTER(FemPcgOpts), ctypes.POINTER(FemPcgStats), c_void_p, c_size_t, c_void_p]),
    "fem_amg_default_opts": (None, [ctypes.POINTER(FemAmgOpts)]),
    "fem_amg_setup": (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p, ctypes.POINTER(FemAmgOpts),
                              ctypes.POINTER(c_void_p)]),
    "fem_amg_setup_device": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p, ctypes.POINTER(FemAmgOpts),
                                     c_void_p, ctypes.POINTER(c_void_p)]),
    "fem_amg_upload": (c_int, [c_void_p, c_void_p]),
    "fem_amg_destroy": (None, [c_void_p]),
    "fem_amg_num_levels": (c_int, [c_void_p]),
    "fem_amg_set_smoother": (c_int, [c_void_p, c_int, ctypes.c_double, ctypes.c_double]),
    "fem_amg_setup_phases": (c_int, [c_void_p, c_void_p]),
    "fem_amg_get_level": (c_int, [c_void_p, c_int, ctypes.POINTER(FemAmgLevelInfo)]),
    "fem_amg_export": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_amg_vcycle": (c_int, [c_void_p, ctypes.POINTER(FemBsr), c_int, c_void_p, c_void_p, c_int, c_void_p]),
    "fem_pcg_solve_amg": (c_int, [ctypes.POINTER(FemBsr), ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p,
                                  ctypes.POINTER(FemPcgOpts), ctypes.POINTER(FemPcgStats), c_void_p, c_size_t,
                                  c_void_p]),
    "fem_mlp_nparams": (c_int, []),
    "fem_precond_cholesky": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p]),
    "fem_precond_features": (c_int, [ctypes.POINTER(FemBsr), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p]),
    "fem_probe_products": (c_int, [ctypes.POINTER(FemBsr), c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]),
    "fem_mlp_forward": (c_int, [ctypes.POINTER(FemMlp), c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
    "fem_mlp_loss_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int64, c_void_p, c_void_p,
                                  ctypes.POINTER(c_int), c_void_p]),
    "fem_ts_gemm_tn_workspace_bytes": (c_size_t, [c_int64, c_int, c_int]),
    "fem_ts_gemm_tn": (c_int, [c_int64, c_int, c_int, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                               c_void_p, c_size_t, c_void_p]),
    "fem_ts_gemm_nn": (c_int, [c_int64, c_int, c_int, c_void_p, c_int64, c_void_p, c_int64, ctypes.c_double,
                               ctypes.c_double, c_void_p, c_int64, c_void_p]),
    "fem_mlp_backward_tc_workspace_bytes": (c_size_t, [c_int64]),
    "fem_mlp_backward_tc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                    c_size_t, c_void_p, c_void_p]),
    "fem_mlp_backward_workspace_bytes": (c_size_t, [c_int64]),
    "fem_mlp_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                 c_size_t, c_void_p]),
    "fem_mlp_adam": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_learned_blocks": (c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_stress_ex": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_size_t, c_int, c_void_p]),
    "fem_stress_noalloc": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_void_p]),
    "fem_stress_workspace_bytes": (c_size_t, [c_int64]),
    "fem_stress": (c_int, [ctypes.POINTER(FemMesh), ctypes.POINTER(FemMaterial), c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_size_t, c_void_p]),
}

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building in-tree first if needed) and type the library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"libfemgb.so not found at {_build.LIB}; run fem_taichi_gb300.build.build()")
        L = ctypes.CDLL(_build.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(rc: int, what: str = "") -> None:
    if rc != FEM_OK:
        msg = load().fem_last_error().decode(errors="replace")
        raise FemError(rc, f"{what}: {msg}" if what else msg)
