"""Solve studies on the synthetic workloads (used by bench.py).

* ``c3``: 100x100x20 block stretched 4:1 in z, bottom fixed, uniform top traction: FP64
  block-Jacobi PCG vs FP32-inner / FP64-refinement PCG to a relative residual of 1e-10.
* ``c4``: learned preconditioner.  Training set: 50 jittered blocks whose element counts
  are drawn uniformly to give 20k-200k nodes, element aspect ratio (z stretch) uniform in
  [1, 8], EX uniform in [7e4, 2.1e5], PO uniform in [0.25, 0.35]; probes z ~ N(0, I).
  Evaluation: the unseen 160x160x20 block.
* ``c5``: 1200x120x15 slab over 1000x60x8 mm twisted 60 degrees, root fixed, 32
  right-hand sides (centrifugal load + 31 seeded random tip-face nodal tractions).

Every solution is compared with an FP64 reference solve of the same system (FP32-inner /
FP64-refinement PCG driven to a relative residual of 1e-13; its own error is estimated by a
second solve at 1e-12), standing in for the reference's MKL Pardiso.  The reference solve
uses block Jacobi on c3 / c4 and the multigrid preconditioner on c5, where block-diagonal
preconditioners do not converge.  ``mixed_amg`` rows add the multigrid preconditioner
(host setup time reported separately as ``amg_setup_s``).
"""
from __future__ import annotations

import time

import numpy as np
import torch

from fem_taichi_gb300 import mesh as _mesh
from fem_taichi_gb300.learned import LearnedPreconditioner, LearnedSmoother, NodeData
from fem_taichi_gb300.model import Model
from fem_taichi_gb300.solve import DeviceSystem

STEEL = _mesh.STEEL


def training_meshes(count=50, seed=0, min_nodes=20_000, max_nodes=200_000):
    """Seeded training blocks (see module docstring); yields (Physics, Materials)."""
    rng = np.random.default_rng(seed)
    for k in range(count):
        target = rng.uniform(min_nodes, max_nodes)
        aspect = rng.uniform(1.0, 8.0)
        mat = {'DE': 7.8e-9, 'EX': float(rng.uniform(7e4, 2.1e5)), 'PO': float(rng.uniform(0.25, 0.35))}
        nz = max(4, int(round((target / 16.0) ** (1.0 / 3.0))))
        nx = max(4, int(round(np.sqrt(target / (nz + 1)) - 1)))
        ny = max(4, int(round(target / ((nx + 1) * (nz + 1)) - 1)))
        P = _mesh.hex_block(nx, ny, nz, size=(float(nx), float(ny), float(nz) * aspect), jitter=0.1,
                            seed=1000 * seed + k, fix="zmin", name=f"train{k}")
        yield P, mat


def concat(datasets):
    """One NodeData-like batch from many (features and probe pairs are per node)."""
    class Batch:
        pass
    b = Batch()
    b.X = torch.cat([d.X for d in datasets])
    b.yhat = torch.cat([d.yhat for d in datasets])
    b.zhat = torch.cat([d.zhat for d in datasets])
    b.n = int(b.X.shape[0])
    b.R = datasets[0].R
    return b


def train_c4(count=50, steps=300, lr=3e-3, n_probes=8, seed=0, device="cuda", min_nodes=20_000,
             max_nodes=200_000):
    t0 = time.perf_counter()
    data = []
    nodes = 0
    for P, mat in training_meshes(count, seed, min_nodes=min_nodes, max_nodes=max_nodes):
        S = DeviceSystem(Model(P.name, P, mat, device=device))
        data.append(NodeData(S, n_probes=n_probes, seed=len(data)))
        nodes += P.Num_Node
        del S
    batch = concat(data)
    del data
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = LearnedPreconditioner(device=device, seed=seed)
    l0 = net.evaluate_loss([batch])
    t1 = time.perf_counter()
    hist = net.train([batch], steps=steps, lr=lr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    return net, {"meshes": count, "nodes": nodes, "probes": n_probes, "steps": steps, "loss_start": l0,
                 "loss_end": hist[-1], "data_s": t_data, "train_s": t_train}


def smoother_cases(count=8, seed=0, device="cuda", min_nodes=20_000, max_nodes=200_000):
    """Training cases of the learned smoother: (system, device multigrid hierarchy, seeded
    random right-hand side) on blocks of the c4 training family."""
    cases = []
    for k, (P, mat) in enumerate(training_meshes(count, seed, min_nodes=min_nodes, max_nodes=max_nodes)):
        S = DeviceSystem(Model(P.name, P, mat, device=device))
        H = S.amg_variant()
        g = torch.Generator(device=S.device).manual_seed(100 + k)
        F = torch.randn(S.F.shape, generator=g, device=S.device, dtype=torch.float64)
        cases.append((S, H, F))
    return cases


def train_smoother(count=10, seed=0, device="cuda", iters=12, **kw):
    """Learned per-level Chebyshev smoother weights (learned.py:LearnedSmoother) fitted on
    the c4 training family; returns (smoother, info)."""
    t0 = time.perf_counter()
    cases = smoother_cases(count, seed, device, **kw)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    sm = LearnedSmoother(levels=2)
    t1 = time.perf_counter()
    l0, l1 = sm.fit(cases, iters=iters)
    t_train = time.perf_counter() - t1
    for _, H, _ in cases:
        H.close()
    return sm, {"meshes": count, "nodes": int(sum(S.n for S, _, _ in cases)), "iters": iters,
                "loss_start": l0, "loss_end": l1, "evaluations": len(sm.history), "data_s": t_data,
                "train_s": t_train, "weights": sm.state_dict()}


def reference_solution(S: DeviceSystem, F=None, precond="amg", check=None, check_cols=None, check_name=None):
    """FP64 reference solution standing in for the reference's Pardiso (SOLVE_static.py:31-33):
    FP64 PCG followed by residual-replacement refinement on compensated (twice-FP64-accurate)
    residuals, until the true residual stops falling -- the FP64 floor of the system, where
    U is as accurate as FP64 storage allows.  Its forward error is estimated by the relative
    difference to a second reference computed the same way with another preconditioner
    ``check`` (block Jacobi when None; on the columns ``check_cols`` of F when given)."""
    kw = dict(mixed=False, maxit=400000, max_outer=10, residual="extra", rtol=1e-15)
    t = time.perf_counter()
    U1, s1 = S.solve(F=F, precond=precond, **kw)
    torch.cuda.synchronize()
    out = {"method": "FP64 PCG (%s) + refinement on compensated residuals, to the FP64 floor"
                     % ("multigrid" if precond is not None else "block Jacobi"),
           "relres": s1["relres"], "floor": s1["floor"], "status_text": s1["status_text"],
           "iterations": s1["iterations"], "outer": s1["outer"], "wall_s": time.perf_counter() - t}
    Fc = F if (F is None or check_cols is None) else F[:, check_cols].contiguous()
    U2, s2 = S.solve(F=Fc, precond=check, **kw)
    U1c = U1 if check_cols is None else U1[:, check_cols]
    out["check"] = {"precond": check_name or ("block Jacobi" if check is None else "multigrid"),
                    "relres": s2["relres"], "floor": s2["floor"], "iterations": s2["iterations"],
                    "columns": "all" if check_cols is None else list(check_cols)}
    out["est_err"] = relerr(U2, U1c)
    return U1, out


def _levels(H):
    return [(l["n"], l["b"], l["nnzb_A"] or None) for l in H.levels()]


def amg_setup(S: DeviceSystem, compare_host=False, **opts):
    """Builds the multigrid hierarchy of S on the device and reports its cost; with
    compare_host, also the cost of the host setup of the same hierarchy (copy of K to the
    host, setup, upload)."""
    torch.cuda.synchronize()
    t = time.perf_counter()
    H = S.amg(**opts)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t
    lv = H.levels()
    out = {"where": H.where, "setup_s": H.setup_s, "upload_s": H.upload_s, "wall_s": wall,
           "phases_s": H.setup_phases(), "levels": _levels(H),
           "operator_complexity": (S.nnzb * 9 + sum(l["nnzb_A"] * 36 for l in lv[1:])) / (S.nnzb * 9)}
    if compare_host:
        torch.cuda.synchronize()
        t = time.perf_counter()
        Hh = S.amg_variant(setup="host", **opts)
        torch.cuda.synchronize()
        hw = time.perf_counter() - t
        ld, lh = H.levels(), Hh.levels()
        out["host_setup"] = {"wall_s": hw, "setup_s": Hh.setup_s, "upload_s": Hh.upload_s,
                             "phases_s": Hh.setup_phases(), "levels": _levels(Hh),
                             "same_levels": _levels(Hh) == out["levels"],
                             "same_lmax": [a["lmax"] for a in ld] == [b["lmax"] for b in lh],
                             "same_aggregates": all(np.array_equal(H.export(l, 4), Hh.export(l, 4))
                                                    for l in range(len(ld) - 1)),
                             "same_coarsest_inverse": bool(np.array_equal(H.export(len(ld) - 1, 5),
                                                                         Hh.export(len(lh) - 1, 5)))}
        Hh.close()
    return out


def relerr(U, Ur):
    if U.dim() == 1:
        return float(torch.linalg.norm(U - Ur) / torch.linalg.norm(Ur))
    return float(((U - Ur).norm(dim=0) / Ur.norm(dim=0)).max())


def timed_solve(S, label, reps=None, **kw):
    """Warm solve, then the best of `reps` timed solves (default: 2 when a solve takes under
    1 s, which absorbs an occasional host-side stall of a single short measurement, else 1)."""
    U, st = S.solve(**kw)          # warm (graphs, autotune, FP32 copy)
    best = None
    k = 0
    while True:
        torch.cuda.synchronize()
        t = time.perf_counter()
        U, st = S.solve(**kw)
        torch.cuda.synchronize()
        w = time.perf_counter() - t
        best = w if best is None else min(best, w)
        k += 1
        if k >= (reps if reps is not None else (2 if w < 1.0 else 1)):
            break
    st = dict(st)
    st["wall_s"] = best
    st["label"] = label
    return U, st


def compare(S: DeviceSystem, Ur, variants, F=None, target=1e-8, amg=None):
    """Each variant: (label, kwargs).  Adds the relative error vs Ur and whether it meets the
    error target; multigrid rows carry the hierarchy's setup time (``setup_s``, not in
    wall_s).  ``status_text`` is the solver's own verdict on its true residual: "converged"
    only when it is <= rtol; "not converged" rows show where they stopped (``relres``) and
    the FP64 floor of the system (``floor``)."""
    rows = []
    for label, kw in variants:
        U, st = timed_solve(S, label, F=F, **kw)
        st["relerr"] = relerr(U, Ur)
        st["rtol"] = kw.get("rtol")
        st["at_floor"] = bool(st["relres"] <= 16 * st["floor"])
        st["meets_1e-8"] = bool(st["relerr"] <= target)
        if amg is not None and (kw.get("precond") == "amg"):
            st["setup_s"] = amg["wall_s"]
        rows.append(st)
    return rows


def spmv_bytes(n, nnzb, value_bytes, nrhs=1):
    """Algorithmic HBM bytes of one BSR product: values, column indices, row pointers, x, y."""
    return 9 * value_bytes * nnzb + 4 * nnzb + 4 * (n + 1) + 2 * 3 * n * value_bytes * nrhs


def pcg_iteration_bytes(n, nnzb, value_bytes):
    """Algorithmic HBM bytes of one block-Jacobi PCG iteration: the product with K, the
    block-diagonal apply (9 values per node) and ~10 passes over the 3N-vectors."""
    return spmv_bytes(n, nnzb, value_bytes) + 9 * value_bytes * n + 10 * 3 * n * value_bytes


def bf16_peak_tflops():
    import json
    import os
    f = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(f) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def mlp_rates(net, S: DeviceSystem, reps=10):
    """CUDA-event times of the MLP forward (tcgen05) and of its tensor-core backward on the
    nodes of S; FLOPs of the padded 16 -> 64 -> 64 -> 16 layers the tensor cores compute."""
    from fem_taichi_gb300.learned import N_HID, N_IN, N_OUT
    X = NodeData(S, with_probes=False).X
    n = int(X.shape[0])
    out, z1, z2 = net.forward(X, save=True)
    dout = torch.randn(out.shape, device=out.device, dtype=out.dtype) * 1e-3
    stream = torch.cuda.current_stream(S.device)
    res = {}
    for name, fn in (("forward", lambda: net.forward(X)), ("backward", lambda: net.backward(X, z1, z2, dout))):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        res[name + "_ms"] = e0.elapsed_time(e1) / reps
    peak, kind = bf16_peak_tflops()
    fl = 2.0 * n * (N_IN * N_HID + N_HID * N_HID + N_HID * N_OUT)
    tf = fl / (res["forward_ms"] * 1e-3) / 1e12
    res.update({"nodes": n, "forward_flops": fl, "forward_tflops": tf, "bf16_peak_tflops": peak, "peak_kind": kind,
                "frac_bf16": tf / peak,
                "backward_weight_gradient_flops": fl,
                "note": "per-node MLP: small matrices (K = 16 / 64), a memory- and latency-bound use of the "
                        "tensor cores; a small share of the solve"})
    return res


def spmv_rates(S: DeviceSystem, reps=20, peak_gbs=None):
    """CUDA-event time of the autotuned FP64 and FP32 (row-SoA) SpMV on this system's K."""
    out = {}
    stream = torch.cuda.current_stream(S.device)
    for fp32, name, vb in ((False, "fp64", 8), (True, "fp32", 4)):
        x = torch.ones(3 * S.n, dtype=torch.float32 if fp32 else torch.float64, device=S.device)
        for _ in range(3):
            S.spmv(x, fp32=fp32)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            S.spmv(x, fp32=fp32)
        e1.record(stream)
        torch.cuda.synchronize(S.device)
        ms = e0.elapsed_time(e1) / reps
        b = spmv_bytes(S.n, S.nnzb, vb)
        out[name] = {"variant": S.variant(fp32, 1), "ms": ms, "algorithmic_bytes": b, "gbs": b / (ms * 1e-3) / 1e9}
        if peak_gbs:
            out[name]["frac_hbm"] = out[name]["gbs"] / peak_gbs
    return out


def spmm_rates(S: DeviceSystem, nrhs_list=(2, 4, 8, 16, 32), reps=10, peak_gbs=None):
    """CUDA-event time of the multi-right-hand-side products (FP64 BSR and the FP32 copy)."""
    out = {}
    stream = torch.cuda.current_stream(S.device)
    for fp32, name, vb in ((False, "fp64", 8), (True, "fp32", 4)):
        for R in nrhs_list:
            x = torch.ones((3 * S.n, R), dtype=torch.float32 if fp32 else torch.float64, device=S.device)
            for _ in range(2):
                S.spmv(x, fp32=fp32, nrhs=R)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                S.spmv(x, fp32=fp32, nrhs=R)
            e1.record(stream)
            torch.cuda.synchronize(S.device)
            ms = e0.elapsed_time(e1) / reps
            b = spmv_bytes(S.n, S.nnzb, vb, R)
            out[f"{name}_r{R}"] = {"ms": ms, "gbs": b / (ms * 1e-3) / 1e9, "ms_per_rhs": ms / R}
            if peak_gbs:
                out[f"{name}_r{R}"]["frac_hbm"] = out[f"{name}_r{R}"]["gbs"] / peak_gbs
    return out


def c3_study(device="cuda", rtol=1e-10, peak_gbs=None):
    P = _mesh.config_mesh("c3")
    extra = _mesh.face_traction_loads(P, "zmax", (0.0, 0.0, -1.0))
    S = DeviceSystem(Model("c3", P, STEEL, device=device, extra_loads=extra))
    amg = amg_setup(S)
    Ur, ref = reference_solution(S)
    rows = compare(S, Ur, [("fp64_bj", dict(rtol=rtol, mixed=False)),
                           ("mixed_bj", dict(rtol=rtol, mixed=True)),
                           ("mixed_amg", dict(rtol=rtol, mixed=True, precond="amg")),
                           ("fp64_amg", dict(rtol=rtol, mixed=False, precond="amg"))], amg=amg)
    for r in rows:
        r["ms_per_iteration"] = 1e3 * r["wall_s"] / max(r["iterations"], 1)
        if r["label"].endswith("_bj"):
            b = pcg_iteration_bytes(S.n, S.nnzb, 4 if r["label"].startswith("mixed") else 8)
            r["gb_per_iteration"] = b / 1e9
            r["gbs"] = b / (r["ms_per_iteration"] * 1e-3) / 1e9
    return {"workload": "c3 100x100x20 (4:1), 214,221 nodes", "reference": ref, "solves": rows,
            "amg": amg, "spmv": spmv_rates(S, peak_gbs=peak_gbs)}


def face_rhs(S: DeviceSystem, P, F0, nrhs, face, seed):
    """nrhs right-hand sides: F0 and nrhs - 1 seeded random nodal loads N(0, 1) N on a face."""
    nx, ny, nz = P.grid
    ix, iy, iz = P.grid_index
    sel = {"xmax": ix == nx, "zmax": iz == nz}[face]
    nodes = np.nonzero(sel)[0]
    rng = np.random.default_rng(seed)
    Fm = torch.zeros((3 * P.Num_Node, nrhs), dtype=torch.float64, device=S.device)
    Fm[:, 0] = F0
    for k in range(1, nrhs):
        f = np.zeros((P.Num_Node, 3))
        f[nodes] = rng.standard_normal((nodes.size, 3))
        Fm[:, k] = torch.from_numpy(f.reshape(-1)).to(S.device)
    return Fm


def c4_study(net=None, device="cuda", rtol=1e-10, train_kw=None, nrhs=32, smoother=None):
    """Learned preconditioner on the unseen 160x160x20 block: 1 and 32 right-hand sides
    (the top traction plus 31 seeded random top-face loads), learned vs plain block Jacobi,
    against the FP64 reference."""
    info = {}
    if net is None:
        net, info = train_c4(device=device, **(train_kw or {}))
    P = _mesh.config_mesh("c4", fix="zmin", load_face=None)
    extra = _mesh.face_traction_loads(P, "zmax", (0.0, 0.0, -1.0))
    M = Model("c4", P, STEEL, device=device, extra_loads=extra)
    S = DeviceSystem(M)
    t = time.perf_counter()
    Pl = net.blocks(S)
    torch.cuda.synchronize()
    t_inf = time.perf_counter() - t
    mlp = mlp_rates(net, S)
    amg = amg_setup(S)
    Fm = face_rhs(S, P, S.F, nrhs, "zmax", seed=4)
    Urm, ref = reference_solution(S, F=Fm, check_cols=[0, 1, 2, 3])
    Ur = Urm[:, 0].contiguous()
    F1 = Fm[:, 0].contiguous()
    rows = compare(S, Ur, [("fp64_bj", dict(rtol=rtol, mixed=False)),
                           ("mixed_bj", dict(rtol=rtol, mixed=True)),
                           ("mixed_learned", dict(rtol=rtol, mixed=True, precond=Pl)),
                           ("fp64_learned", dict(rtol=rtol, mixed=False, precond=Pl)),
                           ("mixed_amg", dict(rtol=rtol, mixed=True, precond="amg")),
                           ("fp64_amg", dict(rtol=rtol, mixed=False, precond="amg"))], F=F1, amg=amg)
    rows += compare(S, Urm, [("fp64_bj_32rhs", dict(rtol=rtol, mixed=False)),
                             ("mixed_bj_32rhs", dict(rtol=rtol, mixed=True)),
                             ("mixed_learned_32rhs", dict(rtol=rtol, mixed=True, precond=Pl)),
                             ("mixed_amg_32rhs", dict(rtol=rtol, mixed=True, precond="amg")),
                             ("fp64_amg_32rhs", dict(rtol=rtol, mixed=False, precond="amg"))], F=Fm, amg=amg)
    # learned smoother weights (trained on the same family) in a second hierarchy of K
    sm_info = {}
    if smoother is None:
        smoother, sm_info = train_smoother(device=device)
    Hl = smoother.apply(S.amg_variant())
    for F_, Ur_, suffix in ((F1, Ur, ""), (Fm, Urm, "_32rhs")):
        r = compare(S, Ur_, [("fp64_amg_learned_smoother" + suffix, dict(rtol=rtol, mixed=False, precond=Hl))],
                    F=F_)[0]
        r["setup_s"] = amg["wall_s"]
        rows.append(r)
    Hl.close()
    by = {r["label"]: r for r in rows}
    gain = {}
    for suffix in ("", "_32rhs"):
        lb, bj, fb = by["mixed_learned" + suffix], by["mixed_bj" + suffix], by["fp64_bj" + suffix]
        gain["learned_vs_mixed_bj" + suffix] = {"iterations": lb["iterations"] / max(bj["iterations"], 1),
                                               "wall": lb["wall_s"] / bj["wall_s"]}
        gain["learned_mixed_vs_fp64_bj" + suffix] = {"wall": lb["wall_s"] / fb["wall_s"]}
        ls, da = by["fp64_amg_learned_smoother" + suffix], by["fp64_amg" + suffix]
        gain["learned_smoother_vs_amg" + suffix] = {"iterations": ls["iterations"] / max(da["iterations"], 1),
                                                   "wall": ls["wall_s"] / da["wall_s"]}
    return {"workload": "c4 eval 160x160x20, 544,341 nodes, 1 and %d RHS" % nrhs, "training": info,
            "smoother_training": sm_info, "inference_s": t_inf, "mlp": mlp, "reference": ref, "solves": rows,
            "amg": amg,
            "gain": gain}, net


def c5_system(device="cuda", nrhs=32, seed=5):
    P = _mesh.config_mesh("c5")
    M = Model("c5", P, STEEL, device=device)
    S = DeviceSystem(M)
    return S, face_rhs(S, P, S.F, nrhs, "xmax", seed)


def c5_independent_check(device="cuda", maxit=150_000, rtol=1e-12):
    """An oracle for c5 that shares nothing with the multigrid path: FP64 block-Jacobi PCG on
    the first right-hand side (the tip traction), refined on compensated residuals, under an
    iteration cap; its solution against the multigrid reference of ``c5_study``.  Minutes of
    GPU time, so not part of the default bench: ``python bench_solve.py --c5-check``."""
    S, Fm = c5_system(device, 1)
    F1 = Fm[:, 0].contiguous()
    t = time.perf_counter()
    Ua, sa = S.solve(F=F1, precond="amg", mixed=False, maxit=400000, max_outer=10, residual="extra", rtol=1e-15)
    torch.cuda.synchronize()
    ta = time.perf_counter() - t
    t = time.perf_counter()
    Ub, sb = S.solve(F=F1, mixed=False, maxit=maxit, max_outer=4, residual="extra", rtol=rtol)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t
    return {"workload": "c5, 1 RHS (tip traction)",
            "multigrid_reference": {"relres": sa["relres"], "floor": sa["floor"], "iterations": sa["iterations"],
                                    "outer": sa["outer"], "wall_s": ta},
            "block_jacobi": {"relres": sb["relres"], "floor": sb["floor"], "iterations": sb["iterations"],
                             "outer": sb["outer"], "status_text": sb["status_text"], "wall_s": tb, "maxit": maxit},
            "relative_difference": relerr(Ub, Ua)}


def c5_study(net=None, device="cuda", rtol=1e-10, nrhs=32, include_fp64=True, maxit=1000, block_variants=True):
    """32 right-hand sides on the slender twisted slab (condition number far beyond FP32
    refinement).  The reference is the FP64 multigrid solve refined on compensated residuals
    to the FP64 floor, cross-checked on 2 columns by the same procedure with a different
    preconditioner (degree-3 instead of degree-2 Chebyshev smoothing).  Rows: the FP64
    multigrid solve with compensated residuals (``fp64_amg_extra_residual``, 32 and 1 RHS; the
    residual of this system floors near 5e-8, and only refinement on compensated residuals
    brings the error below 1e-8) and with plain FP64 residuals (``fp64_amg``, which stops at
    the floor with an error above 1e-8).  Block-diagonal preconditioners are run
    on the first right-hand side with an iteration cap and reported with the error they
    reach ("not converged in `maxit` iterations")."""
    S, Fm = c5_system(device, nrhs)
    amg = amg_setup(S, compare_host=True)
    H2 = S.amg_variant(pre_degree=3, post_degree=3)
    Ur, ref = reference_solution(S, F=Fm, precond="amg", check=H2, check_cols=[0, 1],
                                 check_name="multigrid with degree-3 Chebyshev smoothing")
    H2.close()
    variants = [("fp64_amg_extra_residual", dict(rtol=rtol, mixed=False, precond="amg", residual="extra")),
                ("fp64_amg", dict(rtol=rtol, mixed=False, precond="amg")),
                ("fp64_amg_extra_residual_1rhs", dict(F=Fm[:, 0].contiguous(), rtol=rtol, mixed=False, precond="amg",
                                                      residual="extra")),
                ("fp64_amg_1rhs", dict(F=Fm[:, 0].contiguous(), rtol=rtol, mixed=False, precond="amg"))]
    rows = []
    for label, kw in variants:
        F_ = kw.pop("F", Fm)
        U, st = timed_solve(S, label, F=F_, **kw)
        st["relerr"] = relerr(U, Ur if F_.dim() == 2 else Ur[:, 0])
        st["rtol"] = rtol
        st["at_floor"] = bool(st["relres"] <= 16 * st["floor"])
        st["meets_1e-8"] = bool(st["relerr"] <= 1e-8)
        st["setup_s"] = amg["wall_s"]
        rows.append(st)
    if block_variants:
        F1, U1r = Fm[:, 0].contiguous(), Ur[:, 0].contiguous()
        bv = [("fp64_bj_1rhs_capped", dict(rtol=rtol, mixed=False, maxit=maxit))]
        if net is not None:
            bv.append(("fp64_learned_1rhs_capped", dict(rtol=rtol, mixed=False, precond=net.blocks(S), maxit=maxit)))
        if include_fp64:
            bv.append(("mixed_bj_1rhs_capped", dict(rtol=rtol, mixed=True, maxit=maxit, inner_maxit=maxit)))
        rows += compare(S, U1r, bv, F=F1)
    return {"workload": f"c5 twisted slab 1200x120x15, 2,325,136 nodes, {nrhs} RHS", "reference": ref,
            "amg": amg, "solves": rows}


def modal_study(cfg="c1", num_eigen=100, num_block=10, device="cuda", precond="amg"):
    """Block-Lanczos modal solve (SOLVE_eigen.py:45-89, the reference driver's num_eigen=100)
    on a config mesh: wall time of a warm solve and the lowest frequencies."""
    from fem_taichi_gb300.eigen import Eigen_solver
    P = _mesh.config_mesh(cfg)
    M = Model(cfg, P, STEEL, device=device)
    solver = Eigen_solver(M)
    solver.Solve_gpu(num_eigen=min(num_eigen, 10), num_block=min(num_block, 5), precond=precond)  # warm
    torch.cuda.synchronize()
    t = time.perf_counter()
    lam, X = solver.Solve_gpu(num_eigen=num_eigen, num_block=num_block, precond=precond)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t
    freq = (torch.sqrt(lam) / 2 / np.pi).cpu().numpy()
    G = X.T @ solver._apply_M(X)
    orth = float((G - torch.eye(num_eigen, dtype=G.dtype, device=G.device)).abs().max())
    return {"workload": f"{cfg}: {P.Num_Node:,} nodes, {num_eigen} modes, block {num_block}", "precond": precond,
            "wall_s": wall,
            "steps": solver.last_stats["steps"], "solve_iterations": solver.last_stats["solve_iterations"],
            "phase_ms": solver.last_stats["phase_ms"],
            "lowest_freq_hz": [float(f) for f in freq[:5]], "M_orthonormality_err": orth}


def profile_setup(cfg="c5"):
    """One device multigrid setup (after a warm one) bracketed by cudaProfilerStart/Stop, for
    launch-list captures with ``ncu --profile-from-start off``:
    ``python bench_solve.py --profile-setup c5``."""
    P = _mesh.config_mesh(cfg)
    S = DeviceSystem(Model(cfg, P, STEEL))
    S.amg_variant().close()
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t = time.perf_counter()
    H = S.amg_variant()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t
    torch.cuda.profiler.stop()
    print({"setup_s": wall, "phases_s": H.setup_phases(), "levels": _levels(H)})
    H.close()


def profile_solve(cfg="c3", nrhs=1):
    """One warm multigrid-preconditioned FP64 static solve bracketed by cudaProfilerStart/Stop,
    for launch-list captures with ``ncu --profile-from-start off``:
    ``python bench_solve.py --profile c3 1``."""
    P = _mesh.config_mesh(cfg)
    extra = _mesh.face_traction_loads(P, "zmax", (0.0, 0.0, -1.0))
    S = DeviceSystem(Model(cfg, P, STEEL, extra_loads=extra))
    S.amg()
    F = S.F if nrhs == 1 else S.F.reshape(-1, 1).repeat(1, nrhs).contiguous()
    S.solve(F=F, rtol=1e-10, mixed=False, precond="amg")
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    U, st = S.solve(F=F, rtol=1e-10, mixed=False, precond="amg")
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print({k: st[k] for k in ("status", "iterations", "relres", "time_ms")})


if __name__ == "__main__":
    import sys
    if len(sys.argv) >= 2 and sys.argv[1] == "--profile":
        profile_solve(sys.argv[2] if len(sys.argv) > 2 else "c3", int(sys.argv[3]) if len(sys.argv) > 3 else 1)
    elif len(sys.argv) >= 2 and sys.argv[1] == "--profile-setup":
        profile_setup(sys.argv[2] if len(sys.argv) > 2 else "c5")
    elif len(sys.argv) >= 2 and sys.argv[1] == "--c5-check":
        import json
        print(json.dumps(c5_independent_check(maxit=int(sys.argv[2]) if len(sys.argv) > 2 else 150_000)))
