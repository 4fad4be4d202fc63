"""The U-Net oracle's backward pass against finite differences (CPU).

The GPU network is checked against this oracle (tests/test_unet_gpu.py), so
the oracle's own gradient is pinned here: float64 mode, central differences
on sampled parameters of every layer, and the adjoint identities of the pool
and up-sampling operators.
"""
import numpy as np

from oracle import unet_oracle as uo


def test_pool_and_up_adjoints():
    rng = np.random.default_rng(0)
    for H in (17, 9, 5):
        x = rng.normal(size=(H, H, 3))
        yc = rng.normal(size=((H - 1) // 2 + 1, (H - 1) // 2 + 1, 3))
        assert np.isclose(np.sum(uo.pool(x) * yc), np.sum(x * uo.pool_bwd(yc, H, H)))
        xc = rng.normal(size=((H - 1) // 2 + 1, (H - 1) // 2 + 1, 3))
        y = rng.normal(size=(H, H, 3))
        assert np.isclose(np.sum(uo.up(xc) * y), np.sum(xc * uo.up_bwd(y)))


def test_bf16_rounding():
    # BF16 keeps 7 fraction bits: the spacing at 1 is 2^-7
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, 1.0 + 3 * 2.0 ** -9, -2.5e-3],
                 dtype=np.float32)
    r = uo.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                            # tie, kept bit even: down
    assert r[2] == np.float32(1.0 + 2.0 ** -6)    # tie, kept bit odd: up to even
    assert r[3] == 1.0                            # below the tie
    assert r[4] == np.float32(1.0 + 2.0 ** -7)    # above the tie
    assert abs(r[5] - x[5]) <= abs(x[5]) * 2.0 ** -8


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    H = W = 17
    theta = rng.normal(size=uo.num_params()) * 0.2
    x = rng.normal(size=(H, W, 5))
    target = rng.normal(size=(H, W))
    net = uo.UNet(theta, bf16_mode=False)
    loss, _, g = net.loss_grad(x, target)
    # a few parameters of each layer
    offs, off = [], 0
    for ci, co, _ in uo.layer_shapes():
        n = 9 * co * ci + co
        offs += list(off + rng.choice(n, 3, replace=False))
        off += n
    eps = 1e-6
    for i in offs:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += eps
        tm[i] -= eps
        lp = uo.UNet(tp, bf16_mode=False).loss_grad(x, target)[0]
        lm = uo.UNet(tm, bf16_mode=False).loss_grad(x, target)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[i])
