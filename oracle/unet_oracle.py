"""CPU oracle of the warm-start U-Net (test infrastructure only).

The reference has no learned component; this module restates, in numpy, the
network that ``qdeqcycle_fdm_gb300/csrc/unet.cu`` runs on the tensor cores,
so that its forward pass, loss and every parameter gradient can be checked.
With ``bf16=True`` it rounds to BF16 at the points where the GPU stores BF16
(activations, their gradients, weights as the tensor cores read them) and
accumulates in float64; with ``bf16=False`` it is plain float64 throughout,
which is what the finite-difference check of the backward pass uses.

Layout: arrays are (H, W, C).  A 3x3 convolution with weights w[9, cout, cin]
(tap t = 3*(dy+1) + (dx+1)) and bias b[cout] computes
    y[h, w, co] = b[co] + sum_t sum_ci x[h+dy, w+dx, ci] * w[t, co, ci]
with zeros outside the grid.  pool: mean of the in-grid nodes of the 2x2
block (2i..2i+1, 2j..2j+1); up: bilinear with the multigrid prolongation
weights.  The parameter vector is, per layer in order, w.ravel() then b.
"""
from __future__ import annotations

import numpy as np

TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def layer_shapes():
    """(cin, cout, relu) of the 15 convolutions, in parameter order."""
    enc = [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128)]
    dec = [(128, 64), (64, 64), (64, 32), (32, 32), (32, 16), (16, 16)]
    return [(ci, co, 1) for ci, co in enc] + [(ci, co, 1) for ci, co in dec] + [(16, 16, 0)]


def num_params():
    return sum(9 * co * ci + co for ci, co, _ in layer_shapes())


def unpack(theta):
    out, off = [], 0
    for ci, co, _ in layer_shapes():
        w = theta[off:off + 9 * co * ci].reshape(9, co, ci)
        off += 9 * co * ci
        b = theta[off:off + co]
        off += co
        out.append((w, b))
    return out


def pack(pairs):
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in pairs])


def _shift(x, dy, dx):
    """x[h+dy, w+dx] with zeros outside."""
    H, W = x.shape[:2]
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[yd, xd] = x[ys, xs]
    return out


def conv(x, w, b):
    y = np.zeros(x.shape[:2] + (w.shape[1],), dtype=np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        y += _shift(x, dy, dx).astype(np.float64) @ w[t].T.astype(np.float64)
    return y + b


def conv_bwd(x, w, g):
    """(dx, dw, db) of conv for output gradient g."""
    gw = np.zeros(w.shape, dtype=np.float64)
    gx = np.zeros(x.shape, dtype=np.float64)
    H, W = x.shape[:2]
    g2 = g.reshape(-1, g.shape[2]).astype(np.float64)
    for t, (dy, dx) in enumerate(TAPS):
        gw[t] = g2.T @ _shift(x, dy, dx).reshape(-1, x.shape[2]).astype(np.float64)
        gx += _shift(g, -dy, -dx).astype(np.float64) @ w[t].astype(np.float64)
    return gx, gw, g2.sum(axis=0)


def pool(x):
    H, W, C = x.shape
    Hc, Wc = (H - 1) // 2 + 1, (W - 1) // 2 + 1
    s = np.zeros((Hc, Wc, C))
    n = np.zeros((Hc, Wc, 1))
    for a in (0, 1):
        for b_ in (0, 1):
            blk = x[a::2, b_::2]
            s[:blk.shape[0], :blk.shape[1]] += blk
            n[:blk.shape[0], :blk.shape[1]] += 1
    return s / n


def pool_bwd(g, H, W):
    Hc, Wc = g.shape[:2]
    n = np.zeros((Hc, Wc, 1))
    for a in (0, 1):
        for b_ in (0, 1):
            n[:len(range(a, H, 2)), :len(range(b_, W, 2))] += 1
    gc = g / n
    out = np.zeros((H, W, g.shape[2]))
    for a in (0, 1):
        for b_ in (0, 1):
            hh, ww = len(range(a, H, 2)), len(range(b_, W, 2))
            out[a::2, b_::2] = gc[:hh, :ww]
    return out


def up(x):
    Hc, Wc, C = x.shape
    H, W = 2 * Hc - 1, 2 * Wc - 1
    y = np.zeros((H, W, C))
    y[0::2, 0::2] = x
    y[1::2, 0::2] = 0.5 * (x[:-1] + x[1:])
    y[0::2, 1::2] = 0.5 * (x[:, :-1] + x[:, 1:])
    y[1::2, 1::2] = 0.25 * (x[:-1, :-1] + x[1:, :-1] + x[:-1, 1:] + x[1:, 1:])
    return y


def up_bwd(g):
    H, W, C = g.shape
    Hc, Wc = (H + 1) // 2, (W + 1) // 2
    out = np.zeros((Hc, Wc, C))
    out += g[0::2, 0::2]
    out[:-1] += 0.5 * g[1::2, 0::2]
    out[1:] += 0.5 * g[1::2, 0::2]
    out[:, :-1] += 0.5 * g[0::2, 1::2]
    out[:, 1:] += 0.5 * g[0::2, 1::2]
    q = 0.25 * g[1::2, 1::2]
    out[:-1, :-1] += q
    out[1:, :-1] += q
    out[:-1, 1:] += q
    out[1:, 1:] += q
    return out


class UNet:
    """Forward, loss and parameter gradient of the network for x (H, W, 5)."""

    def __init__(self, theta, bf16_mode=True):
        self.q = bf16 if bf16_mode else (lambda a: np.asarray(a, dtype=np.float64))
        self.layers = [(self.q(w) if bf16_mode else w.astype(np.float64), b.astype(np.float64))
                       for w, b in unpack(np.asarray(theta, dtype=np.float64 if not bf16_mode else np.float32))]

    def forward(self, x):
        q = self.q
        H, W = x.shape[:2]
        x0 = np.zeros((H, W, 16))
        x0[..., :x.shape[2]] = x
        x0 = q(x0)
        L = self.layers
        cache = {"x0": x0}

        def cv(i, inp, relu=True):
            y = conv(inp, *L[i])
            return q(np.maximum(y, 0.0) if relu else y)

        e0a = cv(0, x0); e0 = cv(1, e0a)
        p1 = q(pool(e0)); e1a = cv(2, p1); e1 = cv(3, e1a)
        p2 = q(pool(e1)); e2a = cv(4, p2); e2 = cv(5, e2a)
        p3 = q(pool(e2)); e3a = cv(6, p3); e3 = cv(7, e3a)
        u2 = q(up(e3)); d2a = cv(8, u2); d2s = q(d2a + e2); d2 = cv(9, d2s)
        u1 = q(up(d2)); d1a = cv(10, u1); d1s = q(d1a + e1); d1 = cv(11, d1s)
        u0 = q(up(d1)); d0a = cv(12, u0); d0s = q(d0a + e0); d0 = cv(13, d0s)
        out = conv(d0, *L[14])[..., 0]
        cache.update(locals())
        self.cache = cache
        return out

    def loss_grad(self, x, target):
        q = self.q
        out = self.forward(x)
        c = self.cache
        L = self.layers
        n = out.size
        loss = float(np.sum((out - target) ** 2) / n)
        g_head = np.zeros(out.shape + (16,))
        g_head[..., 0] = 2.0 * (out - target) / n
        g_head = q(g_head)
        grads = [None] * 15

        def back(i, inp, y, g, relu=True):
            """gradient into conv i's input for its output gradient g"""
            if relu:
                g = g * (y > 0)
            gx, gw, gb = conv_bwd(inp, L[i][0], g)
            grads[i] = (gw, gb)
            return q(gx)

        g_d0 = back(14, c["d0"], None, g_head, relu=False)
        g_d0s = back(13, c["d0s"], c["d0"], g_d0)
        g_d0a, g_e0 = g_d0s, g_d0s.copy()
        g_u0 = back(12, c["u0"], c["d0a"], g_d0a)
        g_d1 = q(up_bwd(g_u0))
        g_d1s = back(11, c["d1s"], c["d1"], g_d1)
        g_d1a, g_e1 = g_d1s, g_d1s.copy()
        g_u1 = back(10, c["u1"], c["d1a"], g_d1a)
        g_d2 = q(up_bwd(g_u1))
        g_d2s = back(9, c["d2s"], c["d2"], g_d2)
        g_d2a, g_e2 = g_d2s, g_d2s.copy()
        g_u2 = back(8, c["u2"], c["d2a"], g_d2a)
        g_e3 = q(up_bwd(g_u2))
        g_e3a = back(7, c["e3a"], c["e3"], g_e3)
        g_p3 = back(6, c["p3"], c["e3a"], g_e3a)
        g_e2 = q(g_e2 + pool_bwd(g_p3, *c["e2"].shape[:2]))
        g_e2a = back(5, c["e2a"], c["e2"], g_e2)
        g_p2 = back(4, c["p2"], c["e2a"], g_e2a)
        g_e1 = q(g_e1 + pool_bwd(g_p2, *c["e1"].shape[:2]))
        g_e1a = back(3, c["e1a"], c["e1"], g_e1)
        g_p1 = back(2, c["p1"], c["e1a"], g_e1a)
        g_e0 = q(g_e0 + pool_bwd(g_p1, *c["e0"].shape[:2]))
        g_e0a = back(1, c["e0a"], c["e0"], g_e0)
        back(0, c["x0"], c["e0a"], g_e0a)
        return loss, out, pack(grads)
