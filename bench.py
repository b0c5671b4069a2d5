#!/usr/bin/env python
"""Benchmark: hex8 K+M(+F) assembly throughput on one GB300 (Melem/s).

Workload (default): the 200x200x24-element seeded jittered steel block (1,010,025 nodes,
960,000 elements, 26,367,673 3x3 blocks), FP64 K and M in BSR layout plus F with the
centrifugal term for Omegas=(0,0,100), bottom face penalised.  A step is one pass of the
path over that mesh: the element-integral kernel and the deterministic gather kernel.

  value  : device-resident throughput of the FP64 kernels (the reference computes in f64
           throughout; FEM_model_csr.py:33), inputs already in HBM, CUDA events on the
           launch stream, W warm-up steps then K timed steps, max over ranks.
  e2e    : the same metric through the public Python API with host buffers: per step the
           node coordinates are copied host->device from pinned memory, then
           Model.Get_MatrixKL(), Get_MatrixM() and Get_VectorF() return scipy/numpy objects
           (device->host copies included), FP64 kernels.
  roofline: algorithmic bytes of one assembly (24N + 32E + 80 nnzb + 24N + 4 nnzb + 4(N+1))
           / measured time, against the measured HBM copy bandwidth; and, because the FP64
           element kernel is bound by the FP64 pipe, its FP64 operation rate against the
           FP64 FMA rate measured on the same device ("binding": "fp64").
  double_float: the same assembly with the double-float kernels (pairs of FP32 on the FP32
           pipes, about 48-bit significands) -- faster, reported separately, not FP64.
  cpu_baseline / --impl reference: the C restatement of the reference algorithm (element
           loop, per-element scratch, linear-search slot lookup, atomic scatter, penalty)
           on all host cores, on the same 200x200x24 mesh, its pattern built by the oracle's
           restatement of Read.pre_process (scipy); the product library is not loaded.

Multi-GPU (torchrun): every rank assembles its own replica of the workload (weak scaling,
no data-path collective); value = all ranks' elements / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "K+M assembly Melem/s"
UNIT = "Melem/s"

# FP64 operations of one element's integrals (FMA = 2), counted from k_hex8_element:
# W x and element-local coordinates 8 x (15 + 3); trilinear coefficients 24 x 15;
# per Gauss point J 27 FMA, adjugate 27, det 5, reciprocal ~10, R 24 x 5, R/det 24;
# 8 diagonal pairs x (8 x 6 FMA + 16); 28 off-diagonal pairs x (8 x 9 FMA + 30); the mass by
# sum factorisation 12 x 3 + 18 x 3 + 27 x 4; F = M W x 8 x 24 FMA.  ELEM_FP64_INSTR counts
# instructions (FMA = 1) the same way.
ELEM_FP64_FLOPS = (8 * 18 + 24 * 15 + 8 * (54 + 27 + 5 + 10 + 120 + 24) + 8 * (96 + 16) + 28 * (144 + 30)
                   + (12 * 3 + 18 * 3 + 27 * 4) + 8 * 48)
ELEM_FP64_INSTR = (8 * 12 + 24 * 8 + 8 * (27 + 18 + 3 + 5 + 72 + 24) + 8 * (48 + 14) + 28 * (72 + 21)
                   + (12 * 2 + 18 * 2 + 27 * 3) + 8 * 24)
# FP64 operations of one element of the stress element kernel (k_stress_element): corner 0
# subtracted 48; trilinear coefficients of x and u 24 x 2 x (7 FMA + 1); per Gauss point J
# and the displacement gradient 2 x 27 FMA, adjugate 27, det 5, reciprocal ~10, H 9 x 6,
# stresses 18; extrapolation to the corners 6 x 8 FMA for each distinct row of the table (2 for
# the reference's aliased GMat, the default).
STRESS_ELEM_FP64_FLOPS = 48 + 24 * 2 * 15 + 8 * (2 * 54 + 27 + 5 + 10 + 54 + 18) + 2 * 2 * 6 * 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2")
    ap.add_argument("--no-dd", action="store_true", help="skip the double-float assembly line")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-solve", action="store_true", help="skip the static-solve studies")
    ap.add_argument("--no-c5", action="store_true", help="skip the 32-RHS twisted-slab (c5) solve study")
    return ap.parse_args()


def algorithmic_bytes(N, E, nnzb):
    """Minimum HBM bytes of one K+M+F assembly (coords, conn, K, M, F, pattern)."""
    return 24 * N + 32 * E + 72 * nnzb + 8 * nnzb + 24 * N + 4 * nnzb + 4 * (N + 1)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fma_rate_tflops(fp64: bool, stream_handle) -> float:
    """FMA throughput of this device (TFLOP/s) from the benchmark's probe library."""
    from fem_taichi_gb300 import build as B
    L = ctypes.CDLL(B.build_probe())
    L.fem_probe_fma_tflops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    L.fem_probe_fma_tflops.restype = ctypes.c_int
    r = ctypes.c_double(0)
    rc = L.fem_probe_fma_tflops(1 if fp64 else 0, ctypes.byref(r), stream_handle)
    if rc != 0:
        raise RuntimeError(f"FMA rate probe failed (CUDA error {rc})")
    return r.value


def native_libraries():
    """Shared libraries of this repository mapped into the process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for ln in f:
                p = ln.split()[-1] if ln.strip() else ""
                if p.startswith(ROOT) and ".so" in p:
                    out.add(os.path.relpath(p, ROOT))
    except OSError:
        pass
    return sorted(out)


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(backend):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank, local


def max_over_ranks(x, device="cpu"):
    """Largest x over all ranks of the process group (x itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world_size, units_per_rank, seconds):
    """Units processed by all ranks per second (in millions), timed by the slowest rank."""
    return world_size * units_per_rank / seconds / 1e6


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def workload_name(cfg, grid, N, E, nnzb):
    return (f"{cfg}: hex8 K+M+F assembly, {grid[0]}x{grid[1]}x{grid[2]} elements ({N:,} nodes, "
            f"{E:,} elements, nnzb {nnzb:,}), FP64, BSR")


# ---------------------------------------------------------------------------------------------
# CPU side: the reference algorithm's C restatement on the same mesh
# ---------------------------------------------------------------------------------------------
def reference_mesh(cfg):
    """The workload's mesh with its pattern built by the oracle's restatement of
    Read.pre_process (READ_physics.py:42-61, scipy): no product library is loaded."""
    from fem_taichi_gb300.mesh import CONFIGS, block_arrays
    from oracle import fem_oracle as O
    kw = CONFIGS[cfg]
    b = block_arrays(**kw)
    N = b["ids"].size
    Node = np.zeros((6, N))
    Node[0] = b["ids"]
    Node[3:] = b["xyz"].T
    topo = O.pre_process(Node, b["elem"])
    nind = topo["Nind"]
    conn = np.ascontiguousarray(nind[b["elem"]].T, dtype=np.int32)
    bn = np.concatenate([nind[np.asarray(g[0])] for g in b["bounds"]]) if b["bounds"] else np.zeros(0, np.int64)
    return {"xyz": np.ascontiguousarray(b["xyz"]), "conn": conn, "SmNode": topo["SmNode"].astype(np.int32),
            "ReNode": topo["ReNode"].astype(np.int32), "CoElem": topo["CoElem"].astype(np.int32), "N": N,
            "E": conn.shape[0], "nnzb": int(topo["SmNode"][-1]), "bn": bn, "bc": np.zeros((bn.size, 3)),
            "grid": (kw["nx"], kw["ny"], kw["nz"])}


def time_cpu_port(R, mat, om, steps, warmup, threads):
    """Times the C restatement of the reference algorithm (all threads); returns s/step."""
    from oracle import c_oracle as C
    out = (np.zeros((R["nnzb"], 3, 3)), np.zeros(R["nnzb"]), np.zeros((R["N"], 3)))
    args = (R["xyz"], R["conn"], R["SmNode"], R["ReNode"], mat, om, R["bn"], R["bc"])
    for _ in range(warmup):
        C.assemble(*args, nthreads=threads, out=out)
    t0 = time.perf_counter()
    for _ in range(steps):
        C.assemble(*args, nthreads=threads, out=out)
    return (time.perf_counter() - t0) / max(steps, 1)


def reference_arm(a):
    ws, rank, _ = dist_setup("gloo")
    if rank != 0:
        return
    from fem_taichi_gb300.mesh import STEEL
    R = reference_mesh(a.config)
    thr = cpu_threads()
    t = time_cpu_port(R, STEEL, (0, 0, 100), a.steps, a.warmup, thr)
    v = R["E"] / t / 1e6
    name = workload_name(a.config, R["grid"], R["N"], R["E"], R["nnzb"])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered hex block, steel, Omegas=(0,0,100))",
            "config": {"workload": name, "threads": thr, "same_config": True},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": f"the full {a.config} mesh ({R['E']:,} elements, K+M+F) per step, "
                                       f"{a.steps} steps after {a.warmup} warm-up"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "native_so_loaded": native_libraries(),
            "note": ("reference (Python/Taichi 0.6.28 + MKL Pardiso) cannot run at this size here: taichi is not "
                     "installed; timed: C restatement of its algorithm (oracle/fem_oracle.c, OpenMP atomics, all "
                     "host cores), whose numpy twin is pinned to the reference's own outputs")}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------------------
def time_assembly(L, _lib, model, algo, steps, warmup, dev, clocks=None, ws=1):
    """Times `steps` device-resident assemblies (element + gather kernels) with CUDA events
    on the launch stream; returns (total_ms over ranks, mean element ms, mean gather ms, clocks)."""
    import torch
    from fem_taichi_gb300.model import _dptr, _stream
    N, nnzb = model.Num_Node, model.mesh.nnzb
    Kt = torch.empty((nnzb, 3, 3), dtype=torch.float64, device=dev)
    Mt = torch.empty((nnzb,), dtype=torch.float64, device=dev)
    Ft = torch.empty((N, 3), dtype=torch.float64, device=dev)
    wsb = model.workspace()
    code = _lib.ALGO_DD if algo == "dd" else _lib.ALGO_FP64
    out = _lib.FemAssemblyOut(_lib.LAYOUT_BSR, _lib.LAYOUT_BSR, Kt.data_ptr(), Mt.data_ptr(), Ft.data_ptr(),
                              model.fixed.data_ptr(), model.loads.data_ptr(), code)
    st = _stream(dev)
    stream = torch.cuda.current_stream(dev)
    mesh_c, mat_c = ctypes.byref(model.mesh.c), ctypes.byref(model.mat)

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        _lib.check(L.fem_assemble_elements(mesh_c, mat_c, code, _dptr(wsb), wsb.numel(), st), "elements")
        if ev is not None:
            ev[1].record(stream)
        _lib.check(L.fem_assemble_gather(mesh_c, ctypes.byref(out), _dptr(wsb), wsb.numel(), st), "gather")
        if ev is not None:
            ev[2].record(stream)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    if clocks is not None:
        clocks.start()
        time.sleep(0.25)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(steps):
        step(evs[k])
    t1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop() if clocks is not None else None
    total_ms = max_over_ranks(t0.elapsed_time(t1), dev)
    el_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
    ga_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
    del Kt, Mt, Ft
    return total_ms, el_ms, ga_ms, clk


def time_stress(post, N, dev, reps=5):
    import torch
    Sout = torch.empty((N, 10), dtype=torch.float64, device=dev)
    for _ in range(2):
        post.stress_device(Sout)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(reps):
        post.stress_device(Sout)
    s1.record(stream)
    torch.cuda.synchronize()
    return s0.elapsed_time(s1) / reps


def traffic_record(kind):
    """DRAM bytes per assembly of the given kernels from the committed ncu summary."""
    tf = os.path.join(ROOT, "profiles", "assembly_c2_traffic.json")
    if not os.path.exists(tf):
        return None
    with open(tf) as f:
        d = json.load(f)
    r = d.get(kind)
    return r.get("dram_bytes_per_assembly") if isinstance(r, dict) else None


def main():
    t_start = time.perf_counter()
    a = parse()
    if a.impl == "reference":
        return reference_arm(a)
    import torch
    ws, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import fem_taichi_gb300 as F
    from fem_taichi_gb300 import _lib
    from fem_taichi_gb300.model import _stream
    L = _lib.load()
    mat, om = F.STEEL, (0, 0, 100)
    t_mesh = time.perf_counter()
    P = F.config_mesh(a.config)
    t_mesh = time.perf_counter() - t_mesh
    N, E, nnzb = P.Num_Node, P.Num_Elem, int(P.SmNode[-1])
    model = F.Model(a.config, P, mat, Omegas=om, device=dev, algo="fp64")
    st = _stream(dev)
    smi = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
    clocks = ClockSampler(int(smi) if smi.isdigit() else local)

    # -- headline: FP64 kernels -----------------------------------------------------------------
    total_ms, el_ms, ga_ms, clk = time_assembly(L, _lib, model, "fp64", a.steps, a.warmup, dev, clocks, ws)
    ms_step = total_ms / a.steps
    value = whole_job_rate(ws, E * a.steps, total_ms * 1e-3)

    # -- roofline -----------------------------------------------------------------------------
    peak, peak_kind = measured_peaks()
    ab = algorithmic_bytes(N, E, nnzb)
    achieved = ab / (ms_step * 1e-3) / 1e9
    fp64_peak = fma_rate_tflops(True, st)
    fp32_peak = fma_rate_tflops(False, st)
    fp64_ach = E * ELEM_FP64_FLOPS / (el_ms * 1e-3) / 1e12
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded jittered hex block, steel, Omegas=(0,0,100))",
            "config": {"workload": workload_name(a.config, P.grid, N, E, nnzb), "n_node": N, "n_elem": E,
                       "nnzb": nnzb, "arith": "FP64 (FP64 pipe)",
                       "layout": "BSR K [nnzb][3][3], M [nnzb], F [N][3]",
                       "l2": "inputs+outputs+workspace ~5 GB per step >> 129 MB L2 (no flush needed)",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic_record("fp64"), "peak_kind": peak_kind,
                         "kernel": "fem_assemble = k_hex8_element + k_gather (one assembly, FP64)",
                         "algorithmic_bytes": ab,
                         "binding": "fp64",
                         "fp64": {"kernel": "k_hex8_element", "flops_per_elem": ELEM_FP64_FLOPS,
                                  "achieved_tflops": fp64_ach, "peak_tflops": fp64_peak,
                                  "peak_kind": "measured FP64 FMA rate of this device (fem_probe_fma_tflops)",
                                  "frac_fp64": fp64_ach / fp64_peak,
                                  "instr_per_elem": ELEM_FP64_INSTR,
                                  "frac_fp64_instr": E * ELEM_FP64_INSTR / (el_ms * 1e-3) / (fp64_peak * 1e12 / 2),
                                  "element_share": el_ms / (el_ms + ga_ms)}},
            "kernels": {"k_hex8_element_ms": el_ms, "k_gather_ms": ga_ms,
                        "share_element": el_ms / (el_ms + ga_ms), "share_gather": ga_ms / (el_ms + ga_ms)},
            "gpu_launches": 2 * a.steps, "clocks": clk}

    # -- the double-float kernels, separately ------------------------------------------------
    if not a.no_dd:
        t_dd, el_dd, ga_dd, _ = time_assembly(L, _lib, model, "dd", a.steps, a.warmup, dev, None, ws)
        ms_dd = t_dd / a.steps
        line["double_float"] = {
            "arith": "double-float (48-bit): FP32 pairs on the FP32 pipes", "value": whole_job_rate(ws, E * a.steps,
                                                                                                    t_dd * 1e-3),
            "unit": UNIT, "ms_per_step": ms_dd, "k_hex8_element_dd_ms": el_dd, "k_gather_dd_ms": ga_dd,
            "hbm_frac": algorithmic_bytes(N, E, nnzb) / (ms_dd * 1e-3) / 1e9 / peak,
            "traffic": traffic_record("dd"),
            "fp64_equivalent_tflops": E * ELEM_FP64_FLOPS / (el_dd * 1e-3) / 1e12,
            "fp32_fma_peak_tflops": fp32_peak, "gpu_launches": 2 * a.steps}

    # -- e2e through the public API (FP64 kernels) ----------------------------------------------
    if not a.no_e2e:
        ne = a.e2e_steps or max(3, min(a.steps, 10))
        xyz_h = torch.from_numpy(P.xyz.copy()).pin_memory()

        def e2e_step():
            model.set_coordinates(xyz_h)
            K = model.Get_MatrixKL()
            M = model.Get_MatrixM()
            Fv = model.Get_VectorF()
            return K, M, Fv

        for _ in range(2):
            r = e2e_step()
        del r
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for _ in range(ne):
            r = e2e_step()
            del r
        torch.cuda.synchronize()
        w1 = max_over_ranks(time.perf_counter() - w0, dev)
        staged = getattr(model, "m_staging", True)
        line["e2e"] = {"value": whole_job_rate(ws, E * ne, w1), "unit": UNIT, "h2d_bytes_per_step": 24 * N,
                       # K (9 per block) + M (1 per block when staged, else the 3 of the CSR) + F
                       "d2h_bytes_per_step": 72 * nnzb + (8 if staged else 24) * nnzb + 24 * N, "steps": ne,
                       "host_writes_per_step": 72 * nnzb + 24 * nnzb + 24 * N,
                       "parts": model.pipeline_parts,
                       "ms_per_step": w1 / ne * 1e3, "arith": "FP64",
                       "path": "Model.set_coordinates(pinned) + Get_MatrixKL + Get_MatrixM + Get_VectorF",
                       "gpu_launches": 2 * ne * model.pipeline_parts}

    # -- extras: stress recovery on the same mesh -------------------------------------------------
    if not a.no_extras:
        u = np.random.default_rng(2).uniform(-1e-3, 1e-3, size=(N, 3))
        sbytes = 24 * N + 24 * N + 32 * E + 80 * N + 4 * (N + 1) + 32 * E + 4 * N
        post = F.Post(a.config, P, mat, u, mesh=model.mesh, algo="fp64")
        sms = time_stress(post, N, dev)
        st_ach = E * STRESS_ELEM_FP64_FLOPS / (sms * 1e-3) / 1e12
        line["stress"] = {"ms": sms, "arith": "FP64", "algorithmic_bytes": sbytes,
                          "gbs": sbytes / (sms * 1e-3) / 1e9, "frac_hbm": sbytes / (sms * 1e-3) / 1e9 / peak,
                          "Mnodes_per_s": N / sms / 1e3, "binding": "fp64",
                          "fp64": {"flops_per_elem": STRESS_ELEM_FP64_FLOPS, "achieved_tflops": st_ach,
                                   "frac_fp64": st_ach / fp64_peak,
                                   "note": "element-kernel operations over the time of both stress kernels"},
                          "gpu_launches": 2 * 5}
        post_dd = F.Post(a.config, P, mat, u, mesh=model.mesh, algo="dd")
        sdd = time_stress(post_dd, N, dev)
        line["stress"]["double_float"] = {"ms": sdd, "gbs": sbytes / (sdd * 1e-3) / 1e9,
                                          "Mnodes_per_s": N / sdd / 1e3}
        del post, post_dd
        line["host_setup_s"] = {"mesh_and_pattern": t_mesh}
        # topology (incidence + block pattern + gather map): host C++ build vs device build
        from fem_taichi_gb300 import mesh as M_
        t0 = time.perf_counter()
        ind, _ = M_.build_pattern(P.conn, N)
        nep, nel, _ = M_.build_incidence(P.conn, N)
        M_.build_gather_map(P.conn, ind, P.ReNode, nep, nel, N)
        t_host = time.perf_counter() - t0
        M_.build_topology_gpu(P.conn, N, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            M_.build_topology_gpu(P.conn, N, device=dev)
        torch.cuda.synchronize()
        t_gpu = (time.perf_counter() - t0) / 3
        line["topology"] = {"host_threads": cpu_threads(), "host_s": t_host, "gpu_s": t_gpu,
                            "note": "incidence + block pattern + gather map; gpu includes the conn upload and two "
                                    "host syncs (nnzb read back)"}

    # -- static solve studies (seconds to 1e-8 relative error vs an FP64 reference) ---------------
    if not a.no_solve and rank == 0:
        import bench_solve as study

        def brief(r):
            keep = ("label", "wall_s", "iterations", "outer", "rtol", "relres", "floor", "at_floor", "relerr",
                    "meets_1e-8", "status_text", "ms_per_iteration", "gb_per_iteration", "gbs", "nrhs", "setup_s")
            out = {"reference": r["reference"], "solves": [{k: x[k] for k in keep if k in x} for x in r["solves"]]}
            if "amg" in r:
                out["amg_setup"] = r["amg"]
            return out

        phases = {}

        def timed(name, fn):
            t = time.perf_counter()
            r = fn()
            phases[name] = round(time.perf_counter() - t, 1)
            print(f"[bench] {name}: {phases[name]} s", file=sys.stderr, flush=True)
            return r

        r3 = timed("c3_study", lambda: study.c3_study(device=dev, peak_gbs=peak))
        sol = {"c3": brief(r3)}
        sol["c3"]["spmv"] = r3["spmv"]
        r4, net = timed("c4_study", lambda: study.c4_study(device=dev))
        sol["c4"] = brief(r4)
        for k in ("training", "smoother_training", "inference_s", "mlp", "gain"):
            if k in r4:
                sol["c4"][k] = r4[k]
        if not a.no_c5:
            r5 = timed("c5_study", lambda: study.c5_study(net, device=dev, include_fp64=False, maxit=1000))
            sol["c5"] = brief(r5)
            sol["c5"]["workload"] = r5["workload"]
        sol["modal_c1"] = timed("modal_c1", lambda: study.modal_study("c1", num_eigen=100, num_block=10, device=dev))
        sol["bench_phases_s"] = phases
        line["solve"] = sol

    # -- CPU baseline (rank 0, N = 1): the reference algorithm's C port on the same mesh ---------
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        thr = cpu_threads()
        R = reference_mesh(a.config)
        ns = 8
        t = time_cpu_port(R, mat, om, ns, 1, thr)
        line["cpu_baseline"] = {"value": R["E"] / t / 1e6, "unit": UNIT, "cores": thr, "kind": "port",
                                "sample": f"{ns} assemblies (K+M+F) of the full {a.config} mesh ({R['E']:,} "
                                          f"elements) with oracle/fem_oracle.c on {thr} threads, {t:.2f} s each"}
        if not a.no_extras:
            from oracle import c_oracle as C
            from oracle import fem_oracle as O
            us = np.random.default_rng(2).uniform(-1e-3, 1e-3, size=(R["N"], 3))
            W = O.extrapolation_table("aliased")
            C.stress(R["xyz"], R["conn"], R["CoElem"], mat, us, W, nthreads=thr)
            t0 = time.perf_counter()
            C.stress(R["xyz"], R["conn"], R["CoElem"], mat, us, W, nthreads=thr)
            ts = time.perf_counter() - t0
            line["cpu_baseline"]["stress"] = {"Mnodes_per_s": R["N"] / ts / 1e6, "s": ts, "cores": thr,
                                              "sample": f"all {R['N']:,} nodes of the same mesh"}
        if not a.no_solve:
            # static solve: FP64 block-Jacobi PCG with scipy products (1 thread) on the c3
            # system, a bounded sample of iterations scaled to the GPU FP64 solver's count
            from oracle import solve_oracle as SO
            P3 = F.config_mesh("c3")
            M3 = F.Model("c3", P3, mat, extra_loads=F.face_traction_loads(P3, "zmax", (0.0, 0.0, -1.0)),
                         device=dev)
            K3, F3 = M3.Get_MatrixKL(), M3.Get_VectorF()
            _, it, tsol = SO.bj_pcg(K3, F3, rtol=1e-10, maxit=30)
            gpu_it = next((r["iterations"] for r in line.get("solve", {}).get("c3", {}).get("solves", [])
                           if r["label"] == "fp64_bj"), None)
            est = tsol / it * gpu_it if gpu_it else None
            line["cpu_baseline"]["solve"] = {
                "kind": "port", "cores": 1, "s_per_iteration": tsol / it,
                "c3_fp64_bj_estimated_s": est,
                "sample": f"{it} FP64 block-Jacobi PCG iterations on c3 (214,221 nodes) with scipy products, "
                          f"scaled to the {gpu_it} iterations the same method takes to 1e-10; Pardiso "
                          "(the reference's solver) is not available"}
    line["native_so_loaded"] = native_libraries()
    if rank == 0:
        print(json.dumps(line), flush=True)
        print(f"[bench] total: {time.perf_counter() - t_start:.1f} s", file=sys.stderr, flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
