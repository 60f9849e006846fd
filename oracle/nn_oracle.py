"""CPU restatement of the warm-start network (test infrastructure only).

Same architecture, parameter layout and BF16 rounding points as
quantumvortices_gb300/csrc/vk_nn.cu, computed in FP64 with numpy: BF16
weights, BF16 stored activations and gradients, FP32 head output.  Used to
check the tensor-core forward and backward kernels.  The network has no
counterpart in the reference (which has no machine learning).
"""
from __future__ import annotations

import numpy as np


EXACT = False  # True: no BF16 rounding anywhere (for finite-difference checks)


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def layers(base, levels):
    """(cin, cout, relu) per conv in the GPU order."""
    L = [(3, base, True), (base, base, True)]
    for lv in range(1, levels):
        L += [(base << (lv - 1), base << lv, True), (base << lv, base << lv, True)]
    for lv in range(levels - 2, -1, -1):
        L += [(base << (lv + 1), base << lv, True), (base << lv, base << lv, True)]
    L.append((base, 2, False))
    return L


def unpack(params, base, levels):
    out, o = [], 0
    for cin, cout, relu in layers(base, levels):
        w = params[o:o + cout * 9 * cin].reshape(cout, 9, cin)
        o += cout * 9 * cin
        b = params[o:o + cout]
        o += cout
        out.append((w, b, relu))
    return out


TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def shift(x, dy, dx):  # x[y+dy, x+dx] (periodic)
    return np.roll(x, (-dy, -dx), axis=(0, 1))


def conv(x, w, b, relu):
    wb = bf16(w)
    out = np.zeros(x.shape[:2] + (w.shape[0],))
    for t, (dy, dx) in enumerate(TAPS):
        out += shift(x, dy, dx) @ wb[:, t, :].T
    out = out + b
    if relu:
        out = np.maximum(out, 0.0)
    return out


def conv_bwd(x, w, dpre):
    wb = bf16(w)
    dw = np.zeros_like(w)
    for t, (dy, dx) in enumerate(TAPS):
        dw[:, t, :] = np.einsum("hwo,hwi->oi", dpre, shift(x, dy, dx))
    db = dpre.sum(axis=(0, 1))
    dx_ = np.zeros(x.shape[:2] + (w.shape[2],))
    for t, (dy, dx) in enumerate(TAPS):
        dx_ += np.roll(dpre @ wb[:, t, :], (dy, dx), axis=(0, 1))
    return dw, db, dx_


def pool(x):
    return bf16(0.25 * (x[0::2, 0::2] + x[1::2, 0::2] + x[0::2, 1::2] + x[1::2, 1::2]))


def up(x):
    return np.repeat(np.repeat(x, 2, axis=0), 2, axis=1)


def forward(params, inp, base, levels):
    """inp [3][H][W] float; returns (out [2][H][W], cache)."""
    P = unpack(params, base, levels)
    x0 = bf16(np.transpose(inp, (1, 2, 0)))
    cache = {"x0": x0}
    ci = 0
    cur = x0
    a, s, p = [], [], []
    for lv in range(levels):
        w, b, r = P[ci]; ci += 1
        a.append(bf16(conv(cur, w, b, r)))
        w, b, r = P[ci]; ci += 1
        s.append(bf16(conv(a[lv], w, b, r)))
        if lv + 1 < levels:
            p.append(pool(s[lv]))
            cur = p[lv]
    dec = s[levels - 1]
    u, c, e, d = {}, {}, {}, {}
    for lv in range(levels - 2, -1, -1):
        u[lv] = up(dec)
        w, b, r = P[ci]; ci += 1
        c[lv] = bf16(conv(u[lv], w, b, r))
        e[lv] = bf16(c[lv] + s[lv])
        w, b, r = P[ci]; ci += 1
        d[lv] = bf16(conv(e[lv], w, b, r))
        dec = d[lv]
    w, b, r = P[ci]
    out = conv(dec, w, b, r)
    if not EXACT:
        out = out.astype(np.float32).astype(np.float64)
    cache.update(a=a, s=s, p=p, u=u, c=c, e=e, d=d, dec0=dec)
    return np.transpose(out, (2, 0, 1)), cache


def loss_grad(params, inp, target, base, levels):
    """MSE loss and the full parameter gradient (GPU parameter layout)."""
    P = unpack(params, base, levels)
    out, C = forward(params, inp, base, levels)
    H, W = inp.shape[1:]
    n = 2 * H * W
    err = out - target
    loss = float((err ** 2).sum() / n)
    grads = [None] * len(P)
    dout = bf16(np.transpose(2.0 * err / n, (1, 2, 0)))
    k = len(P) - 1

    def back(k, x, y, dpost, need_dx=True):
        w, b, relu = P[k]
        dpre = bf16(dpost * (y > 0)) if relu else dpost
        dw, db, dx = conv_bwd(x, w, dpre)
        grads[k] = (dw, db)
        return bf16(dx) if need_dx else None

    g = back(k, C["dec0"], None, dout)
    k -= 1
    de = {}
    for lv in range(0, levels - 1):
        de[lv] = back(k, C["e"][lv], C["d"][lv], g); k -= 1
        gu = back(k, C["u"][lv], C["c"][lv], de[lv]); k -= 1
        g = bf16(gu[0::2, 0::2] + gu[1::2, 0::2] + gu[0::2, 1::2] + gu[1::2, 1::2])
    for lv in range(levels - 1, -1, -1):
        ds = g
        if lv < levels - 1:
            ds = bf16(bf16(0.25 * up(g)) + de[lv])
        da = back(2 * lv + 1, C["a"][lv], C["s"][lv], ds)
        x_in = C["p"][lv - 1] if lv > 0 else C["x0"]
        g = back(2 * lv, x_in, C["a"][lv], da, need_dx=lv > 0)
    flat = []
    for dw, db in grads:
        flat.append(dw.ravel())
        flat.append(db.ravel())
    return loss, np.concatenate(flat)


def features(h, w, pos, psi, width):
    """[3, h, w] input features (vk_nn_features restated): Re/Im psi and the
    signed vortex-charge density sum_j q_j exp(-|x - x_j|^2 / (2 width^2))
    with periodic distances folded into [-pi, pi), q_j = +1 for the first
    half of pos and -1 for the rest."""
    nv = len(pos)
    x = np.arange(w) * 2 * np.pi / w
    y = np.arange(h) * 2 * np.pi / h
    X, Y = np.meshgrid(x, y)
    q = np.zeros((h, w))
    for j in range(nv):
        dx = (X - pos[j, 0] + np.pi) % (2 * np.pi) - np.pi
        dy = (Y - pos[j, 1] + np.pi) % (2 * np.pi) - np.pi
        q += (1.0 if j < nv // 2 else -1.0) * np.exp(-(dx * dx + dy * dy) / (2 * width * width))
    return np.stack([psi.real, psi.imag, q])
