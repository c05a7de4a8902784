"""FP64 numpy restatement of the warm-start U-Net: forward, masked MSE loss,
backward.  TEST INFRASTRUCTURE ONLY -- the oracle the CUDA training kernels'
outputs and gradients are checked against (no counterpart in the reference,
which has no learned component).

Architecture (levels l = 0..3, widths w = (w0, w1, w2, w3)):
  enc_l : conv3x3(c_in -> w_l) + ReLU, conv3x3(w_l -> w_l) + ReLU   (l = 0, 1, 2)
          skip_l = output; then 2x2 average pool
  bott  : conv3x3(w_2 -> w_3) + ReLU, conv3x3(w_3 -> w_3) + ReLU
  dec_l : nearest 2x upsample, concat [up, skip_l] on channels,
          conv3x3(w_{l+1} + w_l -> w_l) + ReLU, conv3x3(w_l -> w_l) + ReLU  (l = 2, 1, 0)
  head  : conv1x1(w_0 -> c_out), no activation
Tensors are NHWC; conv weights are [c_out][ky][kx][c_in] with bias [c_out],
stored flat in the order of `layer_shapes` (weight then bias per layer).
"""
from __future__ import annotations

import numpy as np


def layer_shapes(c_in, c_out, widths):
    w0, w1, w2, w3 = widths
    convs = []
    c = c_in
    for l, w in enumerate((w0, w1, w2)):
        convs += [(f"enc{l}a", w, 3, c), (f"enc{l}b", w, 3, w)]
        c = w
    convs += [("botta", w3, 3, w2), ("bottb", w3, 3, w3)]
    up = w3
    for l, w in ((2, w2), (1, w1), (0, w0)):
        convs += [(f"dec{l}a", w, 3, up + w), (f"dec{l}b", w, 3, w)]
        up = w
    convs += [("head", c_out, 1, w0)]
    return convs


def param_count(c_in, c_out, widths):
    return sum(co * k * k * ci + co for (_, co, k, ci) in layer_shapes(c_in, c_out, widths))


def unpack(flat, c_in, c_out, widths):
    p = {}
    o = 0
    for (name, co, k, ci) in layer_shapes(c_in, c_out, widths):
        n = co * k * k * ci
        p[name] = (flat[o:o + n].reshape(co, k, k, ci), flat[o + n:o + n + co])
        o += n + co
    return p


def pack(grads, c_in, c_out, widths):
    out = []
    for (name, co, k, ci) in layer_shapes(c_in, c_out, widths):
        gw, gb = grads[name]
        out += [gw.reshape(-1), gb.reshape(-1)]
    return np.concatenate(out)


def conv(x, w, b):
    """x: (N,H,W,Ci), w: (Co,k,k,Ci) -> (N,H,W,Co), zero padding k//2."""
    k = w.shape[1]
    r = k // 2
    N, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (r, r), (r, r), (0, 0)))
    out = np.zeros((N, H, W, w.shape[0]))
    for ky in range(k):
        for kx in range(k):
            out += np.einsum("nhwc,oc->nhwo", xp[:, ky:ky + H, kx:kx + W, :], w[:, ky, kx, :])
    return out + b


def conv_backward(x, w, dy):
    k = w.shape[1]
    r = k // 2
    N, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (r, r), (r, r), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    for ky in range(k):
        for kx in range(k):
            dw[:, ky, kx, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, ky:ky + H, kx:kx + W, :])
            dxp[:, ky:ky + H, kx:kx + W, :] += np.einsum("nhwo,oc->nhwc", dy, w[:, ky, kx, :])
    db = dy.sum(axis=(0, 1, 2))
    return dxp[:, r:r + H, r:r + W, :], dw, db


def pool(x):
    N, H, W, C = x.shape
    return x.reshape(N, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_backward(dy):
    return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) / 4.0


def upsample(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample_backward(dy):
    N, H, W, C = dy.shape
    return dy.reshape(N, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward(flat, x, c_in, c_out, widths):
    p = unpack(flat, c_in, c_out, widths)
    cache = {}
    h = x
    skips = []
    for l in range(3):
        for s in "ab":
            cache[f"enc{l}{s}"] = h
            h = np.maximum(conv(h, *p[f"enc{l}{s}"]), 0.0)
            cache[f"enc{l}{s}_out"] = h
        skips.append(h)
        h = pool(h)
    for s in "ab":
        cache[f"bott{s}"] = h
        h = np.maximum(conv(h, *p[f"bott{s}"]), 0.0)
        cache[f"bott{s}_out"] = h
    for l in (2, 1, 0):
        h = np.concatenate([upsample(h), skips[l]], axis=3)
        for s in "ab":
            cache[f"dec{l}{s}"] = h
            h = np.maximum(conv(h, *p[f"dec{l}{s}"]), 0.0)
            cache[f"dec{l}{s}_out"] = h
    cache["head"] = h
    y = conv(h, *p["head"])
    return y, cache


def loss_and_grads(flat, x, target, c_in, c_out, widths):
    """loss = mean over all output values of (y - target)^2."""
    p = unpack(flat, c_in, c_out, widths)
    y, cache = forward(flat, x, c_in, c_out, widths)
    n = y.size
    loss = float(((y - target) ** 2).sum() / n)
    dy = 2.0 * (y - target) / n
    g = {}
    dh, g["head"] = (lambda r: (r[0], (r[1], r[2])))(conv_backward(cache["head"], p["head"][0], dy))
    dskip = {}
    for l in (0, 1, 2):
        for s in "ba":
            name = f"dec{l}{s}"
            dh = dh * (cache[name + "_out"] > 0)
            dx, dw, db = conv_backward(cache[name], p[name][0], dh)
            g[name] = (dw, db)
            dh = dx
        wl = p[f"enc{l}b"][0].shape[0]
        cu = dh.shape[3] - wl
        dskip[l] = dh[..., cu:]
        dh = upsample_backward(dh[..., :cu])
    for s in "ba":
        name = f"bott{s}"
        dh = dh * (cache[name + "_out"] > 0)
        dx, dw, db = conv_backward(cache[name], p[name][0], dh)
        g[name] = (dw, db)
        dh = dx
    for l in (2, 1, 0):
        dh = pool_backward(dh) + dskip[l]
        for s in "ba":
            name = f"enc{l}{s}"
            dh = dh * (cache[name + "_out"] > 0)
            dx, dw, db = conv_backward(cache[name], p[name][0], dh)
            g[name] = (dw, db)
            dh = dx
    return loss, y, pack(g, c_in, c_out, widths)
