"""Builds the sm_103a shared library ``libfemgb.so`` in-tree with nvcc.

Every CUDA/C++ translation unit under ``csrc/`` is compiled in parallel to an object
under ``_build/`` and linked into ``_build/libfemgb.so`` (static CUDA runtime, OpenMP for
the host-side topology code).  A rebuild happens only when a source or header is newer
than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfemgb.so")
# measurement-only library of the benchmark (arithmetic-rate probes), not part of the product
PROBE_SRC = os.path.join(HERE, "probe", "fp64_rate.cu")
PROBE_LIB = os.path.join(OUT, "libfemprobe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-fopenmp,-O2", "-I", INCLUDE] + ARCH


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libfemgb.so")
    return path


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps() + [__file__])


# The two multigrid setups must round alike (the device hierarchy is bit-identical to the host
# one): no contraction of a multiply and an add into an FMA in either translation unit.
PER_FILE_FLAGS = {
    "amg_device.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "amg_setup.cpp": ["-Xcompiler", "-ffp-contract=off"],
}


def _compile(src: str, extra) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + NVCC_FLAGS + PER_FILE_FLAGS.get(os.path.basename(src), []) + list(extra)
    subprocess.run(cmd, check=True)
    return obj


def build_probe(force: bool = False) -> str:
    """Compile the benchmark's rate probes into libfemprobe.so; returns its path."""
    if not force and os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= os.path.getmtime(PROBE_SRC):
        return PROBE_LIB
    os.makedirs(OUT, exist_ok=True)
    tmp = PROBE_LIB + ".tmp"
    subprocess.run([nvcc(), "-shared", "-o", tmp, PROBE_SRC, "-O3", "-Xcompiler", "-fPIC"] + ARCH, check=True)
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile and link; returns the library path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"],
                   check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
