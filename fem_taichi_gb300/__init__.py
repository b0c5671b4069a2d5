"""GB300 (sm_103a) hex8 finite-element hot path with the FEM_taichi Python surface.

    from fem_taichi_gb300 import Read, Model, Post, Static_solver, Eigen_solver

``Model`` / ``Post`` / ``Static_solver`` / ``Eigen_solver`` keep the reference's constructors and getters;
all arithmetic runs in hand-written CUDA kernels behind the C ABI of ``libfemgb.so``.
"""
from .mesh import CONFIGS, STEEL, Physics, Read, config_mesh, face_traction_loads, hex_block  # noqa: F401
from .model import Model  # noqa: F401
from .post import Post, extrapolation_table  # noqa: F401
from .solve import DeviceSystem, Static_solver  # noqa: F401
from .eigen import Eigen_solver  # noqa: F401

__all__ = ["Read", "Physics", "Model", "Post", "hex_block", "config_mesh", "CONFIGS", "STEEL",
           "face_traction_loads", "extrapolation_table", "Static_solver", "DeviceSystem", "Eigen_solver"]
