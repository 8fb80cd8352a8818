"""CPU oracle of the learned warm-start MLP (test infrastructure only).

The network has no counterpart in the reference; this restatement fixes what the GPU
kernels must compute: 24 -> 64 -> 64 -> 3 with ReLU, BF16 operands (inputs, weights,
hidden activations, and the back-propagated errors that enter a GEMM) and FP32
accumulation, biases and element-wise math.  `rounding=False` gives the exact FP64
network for finite-difference checks of the gradient formulas.

Parameter layout (as jg_mlp_load): W1[64x24], b1[64], W2[64x64], b2[64], W3[3x64], b3[3],
mean[24], scale[24], oscale[3].
"""
import numpy as np

IN, HID, OUT = 24, 64, 3
SIZES = [("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (OUT, HID)),
         ("b3", (OUT,)), ("mean", (IN,)), ("scale", (IN,)), ("oscale", (OUT,))]
NW = HID * IN + HID + HID * HID + HID + OUT * HID + OUT
NPARAM = NW + IN + IN + OUT


def unpack(p):
    out, o = {}, 0
    for name, shp in SIZES:
        k = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + k]).reshape(shp)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def forward_backward(p, X, T=None, rounding=True):
    """Returns (pred [n,3], loss, grads [NW] or None)."""
    P = unpack(np.asarray(p, np.float64))
    f32 = np.float32 if rounding else np.float64
    rd = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    X = np.asarray(X, f32)
    n = len(X)
    xn = rd((X - P["mean"].astype(f32)) * P["scale"].astype(f32))
    W1, W2, W3 = rd(P["W1"]), rd(P["W2"]), rd(P["W3"])
    b1, b2, b3 = (P[k].astype(f32) for k in ("b1", "b2", "b3"))
    z1 = (xn.astype(np.float64) @ W1.T.astype(np.float64)).astype(f32) + b1
    h1 = rd(np.maximum(z1, 0))
    z2 = (h1.astype(np.float64) @ W2.T.astype(np.float64)).astype(f32) + b2
    h2 = rd(np.maximum(z2, 0))
    y = (h2.astype(np.float64) @ W3.T.astype(np.float64)).astype(f32) + b3
    pred = y * P["oscale"].astype(f32)
    if T is None:
        return pred, None, None
    tn = np.asarray(T, f32) / P["oscale"].astype(f32)
    e = y - tn
    loss = float(np.sum(e.astype(np.float64) ** 2) / (3 * n))
    inv3n = f32(1.0) / (f32(3.0) * f32(n))
    dy = f32(2.0) * e * inv3n
    g = {}
    g["b3"] = dy.astype(np.float64).sum(0)
    g["W3"] = dy.T.astype(np.float64) @ h2.astype(np.float64)
    dyb = rd(dy)
    dh2 = (dyb.astype(np.float64) @ W3.astype(np.float64)).astype(f32)
    dz2 = np.where(h2 > 0, dh2, 0).astype(f32)
    g["b2"] = dz2.astype(np.float64).sum(0)
    dz2b = rd(dz2)
    g["W2"] = dz2b.T.astype(np.float64) @ h1.astype(np.float64)
    dh1 = (dz2b.astype(np.float64) @ W2.astype(np.float64)).astype(f32)
    dz1 = np.where(h1 > 0, dh1, 0).astype(f32)
    g["b1"] = dz1.astype(np.float64).sum(0)
    dz1b = rd(dz1)
    g["W1"] = dz1b.T.astype(np.float64) @ xn.astype(np.float64)
    grads = np.concatenate([np.asarray(g[name]).ravel() for name, _ in SIZES[:6]])
    return pred, loss, grads
