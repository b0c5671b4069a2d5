"""GPU checks of the learned preconditioner: the tensor-core forward and backward passes and
the FP32 CUDA-core backward against the numpy oracle (same BF16 rounding points), the identity
start (zero last layer == block Jacobi), a train-then-solve run checked against the FP64 direct
solve, the stall detector's fallback to block Jacobi, and what the trained network changes
against block Jacobi on a held-out mesh (1 and 32 right-hand sides)."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

import fem_taichi_gb300 as F
from fem_taichi_gb300 import _lib
from fem_taichi_gb300.learned import LearnedPreconditioner, NodeData
from oracle import mlp_oracle as MO
from tests.fixtures import STEEL

pytestmark = pytest.mark.gpu


def _random_net(seed=0):
    net = LearnedPreconditioner(seed=seed)
    g = np.random.default_rng(seed + 100)
    p = (g.standard_normal(MO.unpack(np.zeros(6288))[0].size * 0 + 6288) * 0.15).astype(np.float32)
    p[1024 + 64 + 4096 + 64 + 6 * 64:1024 + 64 + 4096 + 64 + 16 * 64] = 0        # unused output rows
    p[-10:] = 0
    net.load_state_dict({"params": p, "step": 0})
    return net, p.astype(np.float64)


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 70001])
def test_tensor_core_forward_matches_oracle(n):
    net, p = _random_net(1)
    g = np.random.default_rng(n)
    Xf = MO.bf16_round(g.standard_normal((n, 16)).astype(np.float32))
    X = torch.from_numpy(MO.bf16_bits(Xf).view(np.int16)).cuda()
    out, z1, z2 = net.forward(X, save=True)
    o_ref, z1_ref, z2_ref, _, _ = MO.forward(p, Xf)
    z1g = z1.cpu().numpy()
    # layer 1 pre-activations: exact BF16 products, FP32 accumulation of 16 terms
    assert np.max(np.abs(z1g - z1_ref)) <= 1e-5 * max(1.0, np.abs(z1_ref).max())
    og = out.cpu().numpy()
    err = np.abs(og - o_ref)
    scale = np.abs(o_ref[:, :6]).max()
    # rare BF16 rounding-boundary flips of hidden activations move outputs by ~2^-8 relative
    assert np.max(err[:, :6]) <= 2e-2 * scale
    assert np.median(err[:, :6]) <= 1e-5 * scale
    assert np.all(og[:, 6:] == 0.0)


def _backward_case(n, seed):
    net, p = _random_net(2)
    g = np.random.default_rng(seed)
    Xf = MO.bf16_round(g.standard_normal((n, 16)).astype(np.float32))
    X = torch.from_numpy(MO.bf16_bits(Xf).view(np.int16)).cuda()
    out, z1, z2 = net.forward(X, save=True)
    dout = g.standard_normal((n, 16)).astype(np.float32)
    dout[:, 6:] = 0
    z1d, z2d = z1.double().cpu().numpy(), z2.double().cpu().numpy()
    return net, p, X, Xf, z1, z2, z1d, z2d, dout


def test_backward_matches_oracle():
    """CUDA-core FP32 backward: within 1e-4 (norm) of the FP64 oracle."""
    net, p, X, Xf, z1, z2, z1d, z2d, dout = _backward_case(5000, 7)
    grad = net.backward(X, z1, z2, torch.from_numpy(dout).cuda(), tensor_cores=False).cpu().numpy()
    ref = MO.backward(p, Xf, z1d, z2d, dout.astype(np.float64))
    assert np.linalg.norm(grad - ref) <= 1e-4 * np.linalg.norm(ref)


@pytest.mark.parametrize("n", [127, 5000, 70001])
def test_tensor_core_backward_matches_oracle(n):
    """tcgen05 backward (BF16 operands, FP32 accumulation in TMEM): within 5e-4 (norm) of the
    oracle with the same BF16 rounding points, every parameter block checked; within 2e-2 of
    the full-precision gradient.  n = 127 is one partial tile, 70001 gives several tiles per
    CTA (accumulation across tiles in TMEM)."""
    net, p, X, Xf, z1, z2, z1d, z2d, dout = _backward_case(n, 11)
    grad = net.backward(X, z1, z2, torch.from_numpy(dout).cuda(), tensor_cores=True).cpu().numpy()
    ref = MO.backward_bf16(p, Xf, z1d, z2d, dout.astype(np.float64))
    assert np.linalg.norm(grad - ref) <= 5e-4 * np.linalg.norm(ref)
    o = 0
    for size in (1024, 64, 4096, 64, 1024, 16):        # W1 b1 W2 b2 W3 b3
        a, b = grad[o:o + size], ref[o:o + size]
        assert np.linalg.norm(a - b) <= 2e-3 * max(np.linalg.norm(b), 1e-30) + 1e-7, (o, size)
        o += size
    full = MO.backward(p, Xf, z1d, z2d, dout.astype(np.float64))
    assert np.linalg.norm(grad - full) <= 2e-2 * np.linalg.norm(full)
    again = net.backward(X, z1, z2, torch.from_numpy(dout).cuda(), tensor_cores=True).cpu().numpy()
    assert np.array_equal(grad, again)                  # deterministic


def test_loss_grad_kernel_matches_oracle():
    net, p = _random_net(3)
    P = F.hex_block(6, 5, 4, jitter=0.1, seed=2, fix="zmin")
    S = F.DeviceSystem(F.Model("l", P, STEEL))
    d = NodeData(S, n_probes=4, seed=1)
    out, _, _ = net.forward(d.X)
    loss, dout = net.loss_and_grad(d, out)
    l_ref, d_ref = MO.loss_grad(out.double().cpu().numpy(), d.yhat.double().cpu().numpy(),
                                d.zhat.double().cpu().numpy())
    assert abs(float(loss) - l_ref) <= 1e-5 * l_ref
    assert np.abs(dout.cpu().numpy() - d_ref).max() <= 1e-4 * np.abs(d_ref).max()


def test_identity_start_equals_block_jacobi():
    P = F.hex_block(5, 4, 3, jitter=0.1, seed=5, fix="zmin")
    S = F.DeviceSystem(F.Model("i", P, STEEL))
    net = LearnedPreconditioner(seed=0)                 # last layer zero -> C = I
    B = net.blocks(S).cpu().numpy()
    bj = S.block_jacobi().cpu().numpy()
    assert np.abs(B - bj).max() <= 1e-12 * np.abs(bj).max()


def test_train_reduces_loss_and_learned_solve_is_exact():
    train = [F.DeviceSystem(F.Model("t%d" % k, F.hex_block(10 + 2 * k, 8, 4 + k, size=(10.0 + 2 * k, 8.0, 4.0 * (1 + k)),
                                                              jitter=0.1, seed=10 + k, fix="zmin"),
                                    {'DE': 7.8e-9, 'EX': 1e5 * (1 + 0.5 * k), 'PO': 0.25 + 0.04 * k}))
             for k in range(3)]
    data = [NodeData(S, n_probes=8, seed=k) for k, S in enumerate(train)]
    net = LearnedPreconditioner(seed=0)
    l0 = net.evaluate_loss(data)
    hist = net.train(data, steps=150, lr=3e-3)
    assert hist[-1] < 0.9 * l0, (l0, hist[-1])
    P = F.hex_block(14, 12, 6, size=(14.0, 12.0, 12.0), jitter=0.1, seed=99, fix="zmin", load_face="zmax",
                    load=(0, 0, -1))
    M = F.Model("e", P, STEEL)
    S = F.DeviceSystem(M)
    M.learned_precond = net.blocks(S)
    sol = F.Static_solver(M)
    U = sol.Solve_gpu(rtol=1e-12, precond="learned", mixed=True)
    K = M.Get_MatrixKL()
    Ur = spla.spsolve(K.tocsc(), M.Get_VectorF())
    assert np.linalg.norm(U - Ur) / np.linalg.norm(Ur) <= 1e-8, sol.last_stats


def test_stalled_learned_solve_switches_to_block_jacobi():
    """Solve_gpu(precond='learned') watches the learned solve: an SPD preconditioner whose
    blocks are block Jacobi scaled by factors spanning 16 decades stagnates; the solve is
    abandoned once its residual stops halving (long before the iteration cap) and plain
    block Jacobi takes over, reaching the direct solution."""
    P = F.hex_block(12, 10, 5, size=(12.0, 10.0, 5.0), jitter=0.1, seed=5, fix="zmin", load_face="zmax",
                    load=(0, 0, -1))
    M = F.Model("stall", P, STEEL)
    S = F.DeviceSystem(M)
    scale = 10.0 ** np.random.default_rng(1).uniform(-8, 8, size=P.Num_Node)
    M.learned_precond = S.block_jacobi() * torch.from_numpy(scale).to(S.device)[:, None]
    sol = F.Static_solver(M)
    U = sol.Solve_gpu(rtol=1e-12, precond="learned", mixed=False, maxit=20000, stall_window=64)
    st = sol.last_stats
    first = st.get("fallback_from")
    assert first is not None and first["status"] == _lib.FEM_ERR_NOT_CONVERGED, st
    assert first["iterations"] < 2000, first
    assert st["status"] == 0 and st["precond"] == "block", st
    K = M.Get_MatrixKL()
    Ur = spla.spsolve(K.tocsc(), M.Get_VectorF())
    assert np.linalg.norm(U - Ur) / np.linalg.norm(Ur) <= 1e-8, st
    print("stall detected after", first["iterations"], "iterations; block Jacobi:", st["iterations"])


def _held_out_system():
    """A block of the training family that no training set contains (aspect 3, seed 321)."""
    P = F.hex_block(96, 96, 12, size=(96.0, 96.0, 36.0), jitter=0.1, seed=321, fix="zmin")
    M = F.Model("held_out", P, {'DE': 7.8e-9, 'EX': 1.3e5, 'PO': 0.29},
                extra_loads=F.face_traction_loads(P, "zmax", (0.0, 0.0, -1.0)))
    return F.DeviceSystem(M)


def _held_out_rhs(S, nrhs):
    """The top traction, plus nrhs - 1 seeded random loads, and the FP64 reference solution."""
    Fm = S.F.reshape(-1, 1).repeat(1, nrhs).contiguous()
    if nrhs > 1:
        g = torch.Generator(device=S.device).manual_seed(7)
        Fm[:, 1:] = torch.randn(Fm[:, 1:].shape, generator=g, device=S.device, dtype=torch.float64) * 1e-3
    Ur, _ = S.solve(F=Fm, rtol=1e-13, mixed=False, precond="amg", residual="extra", max_outer=8)
    return Fm, Ur


def _timed_rows(S, Fm, Ur, variants):
    import time
    rows = {}
    for label, kw in variants:
        S.solve(F=Fm, rtol=1e-10, **kw)                      # warm: graphs, autotune, FP32 copy
        wall = None
        for _ in range(2):                                    # best of two timed solves
            torch.cuda.synchronize()
            t = time.perf_counter()
            U, st = S.solve(F=Fm, rtol=1e-10, **kw)
            torch.cuda.synchronize()
            wall = min(wall or 1e30, time.perf_counter() - t)
        err = float(((U - Ur).norm(dim=0) / Ur.norm(dim=0)).max())
        rows[label] = dict(wall=wall, it=st["iterations"], outer=st["outer"], status=st["status"], err=err)
    return rows


def _held_out_gain(net, nrhs):
    """Learned mixed PCG vs the same method without the network (mixed block Jacobi) and vs
    plain FP64 block Jacobi on a held-out block of the training family, 1 or `nrhs` RHS."""
    S = _held_out_system()
    Pl = net.blocks(S)
    Fm, Ur = _held_out_rhs(S, nrhs)
    return _timed_rows(S, Fm, Ur, (("mixed_learned", dict(mixed=True, precond=Pl)), ("mixed_bj", dict(mixed=True)),
                                   ("fp64_bj", dict(mixed=False))))


def test_learned_preconditioner_gain_on_a_held_out_mesh(capsys):
    """Trains on blocks of the c4 family (aspect 1-8, EX 7e4-2.1e5, PO 0.25-0.35) and prints,
    on an unseen block, what the network changes against block Jacobi: iterations and wall
    time of the learned mixed solve over mixed block Jacobi (the same solver without the
    network) and over plain FP64 block Jacobi, for 1 and 32 right-hand sides.  Asserted: every
    solve reaches 1e-8 against the FP64 reference, and the network costs at most 1.6x the
    iterations of block Jacobi (the block-diagonal correction has measured no gain over block
    Jacobi on this family: the ratio is printed, not assumed)."""
    import bench_solve
    net, info = bench_solve.train_c4(count=8, steps=120, min_nodes=8_000, max_nodes=40_000, seed=3)
    out = {}
    for nrhs in (1, 32):
        rows = _held_out_gain(net, nrhs)
        out[nrhs] = {"iterations_vs_mixed_bj": rows["mixed_learned"]["it"] / rows["mixed_bj"]["it"],
                     "wall_vs_mixed_bj": rows["mixed_learned"]["wall"] / rows["mixed_bj"]["wall"],
                     "iterations_vs_fp64_bj": rows["mixed_learned"]["it"] / rows["fp64_bj"]["it"],
                     "wall_vs_fp64_bj": rows["mixed_learned"]["wall"] / rows["fp64_bj"]["wall"], "rows": rows}
    with capsys.disabled():
        print("\nlearned preconditioner on the held-out block (training loss",
              f"{info['loss_start']:.4g} -> {info['loss_end']:.4g}):", out)
    for nrhs, o in out.items():
        for r in o["rows"].values():
            assert r["status"] == 0 and r["err"] <= 1e-8, (nrhs, o)
        assert o["iterations_vs_mixed_bj"] <= 1.6, (nrhs, o)


def test_learned_smoother_gain_on_a_held_out_mesh(capsys):
    """The non-block-diagonal learned form: per-level Chebyshev smoother weights of the
    multigrid V-cycle (fine level, and one pair for the coarser levels), learned on 6 blocks of
    the c4 family (learned.py:LearnedSmoother).
    Prints, on the held-out block, the FP64 multigrid solve's iterations and wall time with the
    learned weights over the default smoother, for 1 and 32 right-hand sides.  Asserted: the
    training loss does not end above the default's, every solve reaches 1e-8 against the FP64
    reference, and the learned weights cost at most 1.1x the default's iterations."""
    import bench_solve
    sm, info = bench_solve.train_smoother(count=6, seed=3, min_nodes=20_000, max_nodes=100_000)
    assert info["loss_end"] <= info["loss_start"]
    S = _held_out_system()
    Hd, Hl = S.amg_variant(), sm.apply(S.amg_variant())
    out = {}
    for nrhs in (1, 32):
        Fm, Ur = _held_out_rhs(S, nrhs)
        rows = _timed_rows(S, Fm, Ur, (("amg_learned_smoother", dict(mixed=False, precond=Hl)),
                                       ("amg_default", dict(mixed=False, precond=Hd))))
        out[nrhs] = {"iterations_vs_default": rows["amg_learned_smoother"]["it"] / rows["amg_default"]["it"],
                     "wall_vs_default": rows["amg_learned_smoother"]["wall"] / rows["amg_default"]["wall"],
                     "rows": rows}
    Hd.close()
    Hl.close()
    with capsys.disabled():
        print("\nlearned smoother on the held-out block (training loss",
              f"{info['loss_start']:.4g} -> {info['loss_end']:.4g}, weights {info['weights']}):", out)
    for nrhs, o in out.items():
        for r in o["rows"].values():
            assert r["status"] == 0 and r["err"] <= 1e-8, (nrhs, o)
        assert o["iterations_vs_default"] <= 1.1, (nrhs, o)
