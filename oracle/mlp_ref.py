"""FP64 reference of the surrogate network (TEST INFRASTRUCTURE ONLY).

Restates the forward pass, the Gaussian negative log-likelihood and the
backward pass of the GPU kernels (abc_inference_transcription_gb300/csrc/mlp.cu)
in numpy FP64, rounding to BF16 exactly where the GPU feeds its tensor-core
GEMMs (weights, layer inputs, loss gradient, hidden-layer gradients), so the
GPU gradients can be checked against it at ~1e-3 relative error.
"""
from __future__ import annotations

import numpy as np

IN_PAD, H = 16, 256
LV_MIN, LV_MAX = -9.0, 9.0


def bf16(x: np.ndarray) -> np.ndarray:
    """Round FP32 values to BF16 (round to nearest even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    out[nan] = np.nan
    return out


def dims(in_dim: int, K: int) -> dict:
    out_pad = ((2 * K + 15) // 16) * 16
    d = {"in_dim": in_dim, "K": K, "out_pad": out_pad}
    o = 0
    for name, n in (("w1", IN_PAD * H), ("b1", H), ("w2", H * H), ("b2", H), ("w3", H * H), ("b3", H),
                    ("w4", H * out_pad), ("b4", out_pad)):
        d[name] = (o, o + n)
        o += n
    d["n"] = o
    return d


def unpack(p: np.ndarray, d: dict) -> dict:
    g = lambda k: p[d[k][0]:d[k][1]].astype(np.float64)
    return {"w1": g("w1").reshape(IN_PAD, H), "b1": g("b1"), "w2": g("w2").reshape(H, H), "b2": g("b2"),
            "w3": g("w3").reshape(H, H), "b3": g("b3"), "w4": g("w4").reshape(H, d["out_pad"]), "b4": g("b4")}


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_and_grads(p: np.ndarray, d: dict, theta: np.ndarray, stats: np.ndarray, xm, xs, ym, ys,
                   rounding: bool = True):
    """Loss and flat gradient of one member for the batch (all rows valid).
    rounding=False drops the BF16/FP32 roundings (exact FP64 network, used to
    check this restatement against finite differences)."""
    global bf16
    keep_bf16 = bf16
    if not rounding:
        bf16 = lambda x: np.asarray(x, np.float64)  # noqa: E731
    try:
        return _loss_and_grads(p, d, theta, stats, xm, xs, ym, ys, rounding)
    finally:
        bf16 = keep_bf16


def _loss_and_grads(p, d, theta, stats, xm, xs, ym, ys, rounding):
    f32 = (lambda a: np.asarray(a, np.float32).astype(np.float64)) if rounding else (lambda a: np.asarray(a, np.float64))
    W = unpack(p, d)
    K, N = d["K"], theta.shape[0]
    x = np.zeros((N, IN_PAD))
    x[:, :d["in_dim"]] = f32((theta - xm) / xs)
    x = bf16(x)
    t = f32(np.where(np.isfinite(stats), (stats - ym) / ys, np.nan))
    Wh = {k: bf16(v) if k.startswith("w") else f32(v) for k, v in W.items()}
    z1 = x @ Wh["w1"] + Wh["b1"]
    a1 = bf16(silu(z1))
    z2 = a1 @ Wh["w2"] + Wh["b2"]
    a2 = bf16(silu(z2))
    z3 = a2 @ Wh["w3"] + Wh["b3"]
    a3 = bf16(silu(z3))
    y = a3 @ Wh["w4"] + Wh["b4"]
    mu, lvr = y[:, :K], y[:, K:2 * K]
    lv = np.clip(lvr, LV_MIN, LV_MAX)
    inside = (lvr > LV_MIN) & (lvr < LV_MAX)
    valid = np.isfinite(t)
    tt = np.where(valid, t, 0.0)
    r = tt - mu
    ei = np.exp(-lv)
    inv = 1.0 / (N * K)
    loss = np.sum(np.where(valid, 0.5 * (lv + r * r * ei), 0.0)) * inv
    dy = np.zeros_like(y)
    dy[:, :K] = np.where(valid, -r * ei * inv, 0.0)
    dy[:, K:2 * K] = np.where(valid & inside, 0.5 * (1.0 - r * r * ei) * inv, 0.0)
    dy = bf16(dy)
    g = {}
    g["w4"] = a3.T @ dy
    g["b4"] = dy.sum(0)
    dz3 = bf16((dy @ Wh["w4"].T) * dsilu(z3))
    g["w3"] = a2.T @ dz3
    g["b3"] = dz3.sum(0)
    dz2 = bf16((dz3 @ Wh["w3"].T) * dsilu(z2))
    g["w2"] = a1.T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = bf16((dz2 @ Wh["w2"].T) * dsilu(z1))
    g["w1"] = x.T @ dz1
    g["b1"] = dz1.sum(0)
    flat = np.zeros(d["n"])
    for k, v in g.items():
        flat[d[k][0]:d[k][1]] = v.reshape(-1)
    return loss, flat
