"""CPU checks of the MLP oracle itself: BF16 rounding and analytic gradients against
central finite differences (the oracle then checks the GPU kernels)."""
import numpy as np

from oracle import mlp_oracle as MO


def test_bf16_round_matches_bit_truncation_rules():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-30, 0.0], dtype=np.float32)
    r = MO.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even (0x3F808000 -> 0x3F80)
    assert r[2] == 1.0078125                    # above the tie rounds up
    assert abs(r[3] - (-3.140625)) < 1e-12
    assert np.array_equal(MO.bits_to_float(MO.bf16_bits(x)), r)


def _setup(seed=0, n=37, R=3):
    g = np.random.default_rng(seed)
    p = g.standard_normal(6288) * 0.2
    X = MO.bf16_round(g.standard_normal((n, 16)))
    yh = g.standard_normal((n, 3, R))
    zh = g.standard_normal((n, 3, R))
    return p, X, yh, zh


def test_loss_gradient_finite_differences():
    p, X, yh, zh = _setup()
    out = np.random.default_rng(1).standard_normal((X.shape[0], 16)) * 0.3
    loss, d = MO.loss_grad(out, yh, zh)
    for (i, k) in [(0, 0), (3, 1), (5, 2), (7, 3), (11, 4), (13, 5)]:
        e = 1e-6
        o1 = out.copy(); o1[i, k] += e
        o2 = out.copy(); o2[i, k] -= e
        fd = (MO.loss_grad(o1, yh, zh)[0] - MO.loss_grad(o2, yh, zh)[0]) / (2 * e)
        assert abs(fd - d[i, k]) <= 1e-6 * max(1.0, abs(fd))
    assert np.all(d[:, 6:] == 0)


def test_backward_matches_directional_derivative():
    """Exact chain rule of the BF16-pinned network: with activations frozen at their BF16
    values the network is smooth in z, so compare against the linearised forward."""
    p, X, yh, zh = _setup(2)
    out, z1, z2, h1, h2 = MO.forward(p, X)
    dout = np.random.default_rng(3).standard_normal(out.shape)
    dout[:, 6:] = 0
    g = MO.backward(p, X, z1, z2, dout)
    W1, b1, W2, b2, W3, b3 = MO.unpack(p)
    # last-layer gradients are exact products
    gW3 = g[1024 + 64 + 4096 + 64:][:16 * 64].reshape(16, 64)
    assert np.allclose(gW3[:6], dout[:, :6].T @ h2, rtol=1e-12, atol=1e-12)
    assert np.allclose(gW3[6:], 0)
    # first-layer bias gradient: chain through SiLU derivatives
    dz2 = (dout[:, :6] @ MO.bf16_round(W3[:6])) * MO.silu_grad(z2)
    dz1 = (dz2 @ MO.bf16_round(W2)) * MO.silu_grad(z1)
    assert np.allclose(g[1024:1088], dz1.sum(0), rtol=1e-12, atol=1e-12)
