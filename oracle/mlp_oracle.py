"""FP64 numpy restatement of the surrogate MLP (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA training kernels in
spacetime_gb300/csrc/st_surrogate.cu.  Same parameter layout and loss:
    6 -> 256 -> 256 -> 256 -> 256 -> 6, SiLU, flat parameter vector
    [W0(256x6) b0 W1(256x256) b1 W2 b2 W3 b3 W4(6x256) b4]
    loss = mean_b md (0.5 |o[:2]-t[:2]|^2 e^-s + s) + (o3-t3)^2 + mc (o4-t4)^2
    with s = o5 clamped to [-30, 12]; o2 is unused (no gradient).
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 6, 256, 6
SIZES = [("W0", (NH, NIN)), ("b0", (NH,)), ("W1", (NH, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
         ("W3", (NH, NH)), ("b3", (NH,)), ("W4", (NOUT, NH)), ("b4", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(P):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(P[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].ravel() for name, _ in SIZES])


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(P, X):
    w = unpack(P)
    X = np.asarray(X, dtype=np.float64)
    zs, hs = [], []
    z = X @ w["W0"].T + w["b0"]
    zs.append(z)
    hs.append(_silu(z))
    for l in (1, 2, 3):
        z = hs[-1] @ w[f"W{l}"].T + w[f"b{l}"]
        zs.append(z)
        hs.append(_silu(z))
    out = hs[-1] @ w["W4"].T + w["b4"]
    return out, zs, hs


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def forward_bf16(P, X):
    """The forward pass under the tensor-core kernels' arithmetic contract
    (st_surrogate.cu): the edge layers in FP32 parameters, the hidden layers'
    weights and every hidden activation rounded to bf16, sums exact (FP64
    here; the kernels accumulate in FP32).  Returns the (n, 6) outputs."""
    w = unpack(P)
    X = np.asarray(X, dtype=np.float64)
    h = bf16(_silu(X @ w["W0"].T + w["b0"]))
    for l in (1, 2, 3):
        h = bf16(_silu(h @ bf16(w[f"W{l}"]).T + w[f"b{l}"]))
    return h @ w["W4"].T + w["b4"]


def split_bf16(x):
    """(hi, lo) bf16 pair of FP32 values: hi = bf16(x), lo = bf16(x - hi)."""
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    hi = bf16(x)
    return hi, bf16((x - hi).astype(np.float32))


def forward_split(P, X):
    """forward_bf16 with the edge layers as the tensor-core network kernel
    computes them (sur_mlp_tc_kernel): layer 0 as the split-bf16 product
    x_hi.w_hi + x_lo.w_hi + x_hi.w_lo + b_hi + b_lo, layer 4 as
    h.(w_hi + w_lo) + b4 on the bf16 activations.  Returns (outputs, z0)."""
    w = unpack(P)
    xh, xl = split_bf16(X)
    wh, wl = split_bf16(w["W0"])
    bh, bl = split_bf16(w["b0"])
    z0 = xh @ wh.T + xl @ wh.T + xh @ wl.T + bh + bl
    h = bf16(_silu(z0))
    for l in (1, 2, 3):
        h = bf16(_silu(h @ bf16(w[f"W{l}"]).T + w[f"b{l}"]))
    w4h, w4l = split_bf16(w["W4"])
    return h @ (w4h + w4l).T + w["b4"], z0


def loss_grad(P, X, T):
    """(loss4, grad) with loss4 = (total, direction MSE, radius MSE, g MSE)."""
    w = unpack(P)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    B = X.shape[0]
    out, zs, hs = forward(P, X)
    md, mc = T[:, 5], T[:, 6]
    s_raw = out[:, 5]
    s = np.clip(s_raw, -30.0, 12.0)
    es = np.exp(-s)
    e = out[:, :2] - T[:, :2]
    e2 = (e * e).sum(1)
    er = out[:, 3] - T[:, 3]
    eg = out[:, 4] - T[:, 4]
    tot = md * (0.5 * e2 * es + s) + er * er + mc * eg * eg
    loss4 = np.array([tot.mean(), (md * e2).mean(), (er * er).mean(), (mc * eg * eg).mean()])
    d = np.zeros_like(out)
    d[:, :2] = (md * es)[:, None] * e
    inside = (s_raw > -30.0) & (s_raw < 12.0)
    d[:, 5] = np.where(inside, md * (-0.5 * e2 * es + 1.0), 0.0)
    d[:, 3] = 2.0 * er
    d[:, 4] = 2.0 * mc * eg
    d /= B
    g = {}
    g["W4"] = d.T @ hs[3]
    g["b4"] = d.sum(0)
    dz = (d @ w["W4"]) * _dsilu(zs[3])
    for l in (3, 2, 1):
        g[f"W{l}"] = dz.T @ hs[l - 1]
        g[f"b{l}"] = dz.sum(0)
        dz = (dz @ w[f"W{l}"]) * _dsilu(zs[l - 1])
    g["W0"] = dz.T @ X
    g["b0"] = dz.sum(0)
    return loss4, pack(g)
