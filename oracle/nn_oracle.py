"""CPU oracle of the learned-guess network (test infrastructure only).

A numpy restatement of the encoder-decoder that libtracer_gpu.so trains
(include/tracer_nn.h; the kernels are tracer_code_gb300/csrc/k_conv.cu and
k_nn.cu): the same layers, parameter layout, input normalisation, loss and
backward pass, with every value the GPU stores in BF16 rounded to BF16
(round to nearest even) and sums taken in float64.  The GPU sums in FP32,
so values that land on a BF16 rounding boundary can differ by one BF16 ulp;
the tests compare with tolerances that cover that.

There is no reference counterpart: tracer_code has no learned component.
"""
from __future__ import annotations

import numpy as np

# (cin, cout, level) of the 14 3x3 convolutions, as in k_nn.cu
CONV = [(3, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 128, 2), (128, 128, 2), (128, 128, 3),
        (128, 128, 3), (256, 128, 2), (128, 128, 2), (192, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0)]
HEAD_C = 32


def bf16(a):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32).reshape(a.shape)


def param_layout():
    """[(w_off, b_off, cout, cin)] per conv layer and the head offset; total count."""
    off, out = 0, []
    for cin, cout, _ in CONV:
        w = off
        off += cout * 9 * cin
        out.append((w, off, cout, cin))
        off += cout
    head = off
    off += HEAD_C + 1
    return out, head, off


def unpack(params):
    lay, head, n = param_layout()
    assert params.size == n
    Ws, bs = [], []
    for (w, b, cout, cin) in lay:
        Ws.append(params[w:w + cout * 9 * cin].reshape(cout, 9, cin).astype(np.float64))
        bs.append(params[b:b + cout].astype(np.float64))
    return Ws, bs, params[head:head + HEAD_C].astype(np.float64), float(params[head + HEAD_C])


def _shift(x, dy, dx):
    """x[n, y+dy, x+dx, c] with zeros outside (NHWC)."""
    n, H, W, c = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv3x3(x, Wt, b, relu=True):
    """BF16-rounded output of conv (bias, optional ReLU); x BF16 values NHWC."""
    Wb = bf16(Wt).astype(np.float64)
    acc = np.zeros(x.shape[:3] + (Wt.shape[0],))
    for t in range(9):
        acc += _shift(x.astype(np.float64), t // 3 - 1, t % 3 - 1) @ Wb[:, t, :].T
    acc += b
    if relu:
        acc = np.maximum(acc, 0.0)
    return bf16(acc)


def conv3x3_bwd(x, Wt, dz):
    """(dW, db, dX) of a conv given dZ (BF16 values); dX BF16-rounded."""
    Wb = bf16(Wt).astype(np.float64)
    dz64 = dz.astype(np.float64)
    x64 = x.astype(np.float64)
    dW = np.zeros(Wt.shape)
    dX = np.zeros(x.shape[:3] + (Wt.shape[2],))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        xs = _shift(x64, dy, dx)
        dW[:, t, :] = np.einsum("nhwo,nhwi->oi", dz64, xs)
        dX += _shift(dz64 @ Wb[:, t, :], -dy, -dx)
    return dW, dz64.sum(axis=(0, 1, 2)), bf16(dX)


def pool(x):
    n, H, W, c = x.shape
    return bf16(np.float32(0.25) * x.reshape(n, H // 2, 2, W // 2, 2, c).sum(axis=(2, 4), dtype=np.float32))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def up_bwd(d):
    n, H, W, c = d.shape
    return bf16(d.reshape(n, H // 2, 2, W // 2, 2, c).sum(axis=(2, 4), dtype=np.float32))


def prepare(raw):
    """raw[n][3][H][W] -> x16 values (NHWC, 3 channels used) and stats."""
    raw = raw.astype(np.float32)
    n, _, H, W = raw.shape
    st = np.zeros((n, 4), np.float32)
    x = np.zeros((n, H, W, 3), np.float32)
    for k in range(n):
        c0, c1, c2 = (raw[k, j].astype(np.float64) for j in range(3))
        mean = c0.mean()
        var = (c0 * c0).mean() - mean * mean
        st[k] = [mean, np.sqrt(max(var, 1e-12)), np.sqrt(max((c1 * c1).mean(), 1e-60)),
                 np.sqrt(max((c2 * c2).mean(), 1e-60))]
        x[k, :, :, 0] = (raw[k, 0] - st[k, 0]) / st[k, 1]
        x[k, :, :, 1] = raw[k, 1] / st[k, 2]
        x[k, :, :, 2] = raw[k, 2] / st[k, 3]
    return bf16(x), st


def forward(params, raw):
    """Output o[n][H][W] and the activations the backward pass needs."""
    Ws, bs, hw, hb = unpack(params)
    x, st = prepare(raw)
    a = {"x": x}
    a["A0"] = conv3x3(x, Ws[0], bs[0])
    a["E0"] = conv3x3(a["A0"], Ws[1], bs[1])
    a["P0"] = pool(a["E0"])
    a["A1"] = conv3x3(a["P0"], Ws[2], bs[2])
    a["E1"] = conv3x3(a["A1"], Ws[3], bs[3])
    a["P1"] = pool(a["E1"])
    a["A2"] = conv3x3(a["P1"], Ws[4], bs[4])
    a["E2"] = conv3x3(a["A2"], Ws[5], bs[5])
    a["P2"] = pool(a["E2"])
    a["A3"] = conv3x3(a["P2"], Ws[6], bs[6])
    a["B3"] = conv3x3(a["A3"], Ws[7], bs[7])
    a["U2"] = np.concatenate([up(a["B3"]), a["E2"]], axis=3)
    a["D2a"] = conv3x3(a["U2"], Ws[8], bs[8])
    a["D2b"] = conv3x3(a["D2a"], Ws[9], bs[9])
    a["U1"] = np.concatenate([up(a["D2b"]), a["E1"]], axis=3)
    a["D1a"] = conv3x3(a["U1"], Ws[10], bs[10])
    a["D1b"] = conv3x3(a["D1a"], Ws[11], bs[11])
    a["U0"] = np.concatenate([up(a["D1b"]), a["E0"]], axis=3)
    a["D0a"] = conv3x3(a["U0"], Ws[12], bs[12])
    a["D0b"] = conv3x3(a["D0a"], Ws[13], bs[13])
    out = a["D0b"].astype(np.float64) @ hw + hb
    return out, a, st


def loss_and_grads(params, raw, sf_new):
    """Masked MSE against (sf_new - sf_prev)/rms(sf_prev) and its gradient."""
    Ws, bs, hw, hb = unpack(params)
    out, a, st = forward(params, raw)
    n, H, W = out.shape
    tgt = (sf_new.astype(np.float32) - raw[:, 2].astype(np.float32)) / st[:, 3][:, None, None]
    mask = np.zeros((H, W))
    mask[1:, 1:] = 1.0
    count = n * (H - 1) * (W - 1)
    d = (out - tgt) * mask
    loss = float((d * d).sum() / count)
    dout = 2.0 * d / count
    g = np.zeros_like(params, dtype=np.float64)
    lay, head, _ = param_layout()
    g[head:head + HEAD_C] = np.einsum("nhw,nhwc->c", dout, a["D0b"].astype(np.float64))
    g[head + HEAD_C] = dout.sum()
    dD0b = bf16((dout[..., None] * hw[None, None, None, :]).astype(np.float32))

    def layer(l, X, Y, dY):
        dz = np.where(Y > 0, dY, 0.0).astype(np.float32)
        dW, db, dX = conv3x3_bwd(X, Ws[l], dz)
        w, b, cout, cin = lay[l]
        g[w:w + cout * 9 * cin] = dW.reshape(-1)
        g[b:b + cout] = db
        return dX

    dD0a = layer(13, a["D0a"], a["D0b"], dD0b)
    dU0 = layer(12, a["U0"], a["D0a"], dD0a)
    dD1b = up_bwd(dU0[..., :64])
    dD1a = layer(11, a["D1a"], a["D1b"], dD1b)
    dU1 = layer(10, a["U1"], a["D1a"], dD1a)
    dD2b = up_bwd(dU1[..., :128])
    dD2a = layer(9, a["D2a"], a["D2b"], dD2b)
    dU2 = layer(8, a["U2"], a["D2a"], dD2a)
    dB3 = up_bwd(dU2[..., :128])
    dA3 = layer(7, a["A3"], a["B3"], dB3)
    dP2 = layer(6, a["P2"], a["A3"], dA3)
    dE2 = bf16(dU2[..., 128:] + np.float32(0.25) * up(dP2))
    dA2 = layer(5, a["A2"], a["E2"], dE2)
    dP1 = layer(4, a["P1"], a["A2"], dA2)
    dE1 = bf16(dU1[..., 128:] + np.float32(0.25) * up(dP1))
    dA1 = layer(3, a["A1"], a["E1"], dE1)
    dP0 = layer(2, a["P0"], a["A1"], dA1)
    dE0 = bf16(dU0[..., 64:] + np.float32(0.25) * up(dP0))
    dA0 = layer(1, a["A0"], a["E0"], dE0)
    layer(0, a["x"], a["A0"], dA0)
    return loss, g, out
