"""CPU restatement of the far-field surrogate's forward and backward passes.

Test infrastructure only (the gradient oracle of the GPU kernels): the same
model as mpifdtd_gb300/surrogate/model.py in float64 numpy, with values
rounded to BF16 at the points where the GPU stores BF16 (GEMM operands and
BF16 outputs), so that GPU-vs-oracle differences are FP32 summation order and
the occasional tie of a BF16 rounding, not the BF16 format itself.
"""
from __future__ import annotations

import numpy as np

C, NS, Q, NL, H1, NT, NOUT = 64, 1024, 256, 6, 512, 31 * 360, 22336


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def gelu(x):
    k0, k1 = 0.7978845608, 0.044715
    return 0.5 * x * (1 + np.tanh(k0 * (x + k1 * x ** 3)))


def gelu_grad(x):
    k0, k1 = 0.7978845608, 0.044715
    t = np.tanh(k0 * (x + k1 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * k0 * (1 + 3 * k1 * x * x)


def pool_map(maps):
    """[NIN, B, 1024]: per 8 x 8 block the fill fraction and the moments
    mean(e u_x), mean(e u_y), mean(e u_x^2), mean(e u_y^2), u = (p - 3.5) / 4."""
    b = maps.shape[0]
    e = (maps > 0).reshape(b, 32, 8, 32, 8).astype(np.float64)
    u = (np.arange(8) - 3.5) / 4
    ux, uy = u[None, None, :, None, None], u[None, None, None, None, :]
    chans = [e, e * ux, e * uy, e * ux * ux, e * uy * uy]
    return np.stack([c.mean(axis=(2, 4)).reshape(b, NS) for c in chans])


def to_modes(F, B):   # [B*C, 2Q] -> [Q, B, 2C] with [q][b][r*C + c] = F[b*C + c][2q + r]
    return F.reshape(B, C, Q, 2).transpose(2, 0, 3, 1).reshape(Q, B, 2 * C)


def from_modes(Y, B):  # inverse of to_modes
    return Y.reshape(Q, B, 2, C).transpose(1, 3, 0, 2).reshape(B * C, 2 * Q)


HP = 4   # the head's pooling factor (model.HP)


def head_pool(h, B):
    g = 32 // HP
    return h.reshape(B, C, g, HP, g, HP).mean(axis=(3, 5)).reshape(B, C * g * g)


def head_unpool(d, B):
    g = 32 // HP
    return np.repeat(np.repeat(d.reshape(B, C, g, g), HP, axis=2), HP, axis=3).reshape(B, C, NS) / (HP * HP)


def loss_and_grads(p, x, y, D, E, w=None):
    """p: float32 params (model.init_params layout), x [NIN, B, 1024] (pool_map), y [B, NT],
    w [B] row weights of the squared error (None: 1).
    Returns (per-row loss [B], grads dict)."""
    p = {k: np.asarray(v, np.float64) for k, v in p.items()}
    B = x.shape[1]
    Db, Eb = bf16(D), bf16(E)
    Mb = [bf16(p[f"M{l}"]) for l in range(NL)]
    W1b, W2b = bf16(p["W1"]), bf16(p["W2"])
    Wpb = [bf16(p[f"wp{l}"]) for l in range(NL)]   # the point-wise mixing runs in the BF16 GEMM
    h = bf16(np.einsum("ibs,ic->bcs", x, p["wl"]) + p["bl"][None, :, None])
    hs, Fms, zs = [], [], []
    for l in range(NL):
        F = bf16(h.reshape(B * C, NS) @ Db.T)
        Fm = to_modes(F, B)
        Y = bf16(np.einsum("qbk,qnk->qbn", Fm, Mb[l]))
        Hs = from_modes(Y, B) @ Eb.T
        z = Hs.reshape(B, C, NS) + np.einsum("ck,bks->bcs", Wpb[l], h) + p[f"bp{l}"][None, :, None]
        hs.append(h)
        Fms.append(Fm)
        zs.append(z)
        h = bf16(gelu(z) if l < NL - 1 else z)
    flat = bf16(head_pool(h, B))
    pre1 = flat @ W1b.T + p["b1"]
    u = bf16(gelu(pre1))
    out = u @ W2b.T + p["b2"]
    re, im = out[:, :NT], out[:, NT:2 * NT]        # amplitude head: I = re^2 + im^2
    d = (re * re + im * im) - y
    wv = np.ones(B) if w is None else np.asarray(w, np.float64)
    loss = wv * (d * d).mean(axis=1)
    dout = np.zeros((B, NOUT))
    gI = 2 * wv[:, None] * d / (B * NT)
    dout[:, :NT] = 2 * gI * re
    dout[:, NT:2 * NT] = 2 * gI * im
    dout = bf16(dout)
    g = {"W2": dout.T @ u, "b2": dout.sum(0)}
    du = dout @ W2b
    dpre1 = bf16(du * gelu_grad(pre1))
    g["W1"] = dpre1.T @ flat
    g["b1"] = dpre1.sum(0)
    dflat = dpre1 @ W1b
    dh = head_unpool(dflat, B)
    for l in reversed(range(NL)):
        dz = dh * (gelu_grad(zs[l]) if l < NL - 1 else 1.0)
        dzb = bf16(dz)                                # GEMM operand
        g[f"wp{l}"] = np.einsum("bcs,bks->ck", dzb, hs[l])
        g[f"bp{l}"] = dz.sum(axis=(0, 2))
        dYt = bf16(dzb.reshape(B * C, NS) @ Eb)
        dY = to_modes(dYt, B)
        g[f"M{l}"] = np.einsum("qbn,qbk->qnk", dY, Fms[l])
        dFm = bf16(np.einsum("qbn,qnk->qbk", dY, Mb[l]))
        dspec = from_modes(dFm, B) @ Db
        dh = np.einsum("ck,bcs->bks", Wpb[l], dzb) + dspec.reshape(B, C, NS)
    g["wl"] = np.einsum("bcs,ibs->ic", dh, x)
    g["bl"] = dh.sum(axis=(0, 2))
    return loss, g
