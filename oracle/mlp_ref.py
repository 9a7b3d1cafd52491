"""CPU oracle of the learned surrogate (test infrastructure only).

The reference has no learned part, so this is the oracle the library's own
MLP kernels (calypso-gap_gb300/csrc/mlp.cu) are checked against: a float64
numpy statement of the per-atom network, its input gradient, the
energy + descriptor-gradient loss and that loss's weight gradient (double
backpropagation), written out from the formulas rather than through an
autodiff package.  `emulate_bf16=True` rounds to bfloat16 (round to nearest
even) at exactly the points where the CUDA kernels store BF16 operands, so
the GPU result can be compared tightly; `emulate_bf16=False` is the exact
float64 function, checked against finite differences by the CPU tests.

Parameter block layout (one member, one species), flat float vector:
W1[H][D], b1[H], W2[H][H], b2[H], w3[H], b3, then zeros up to a multiple of
8 parameters (the library's block size).
"""
import numpy as np


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _id(x):
    return np.asarray(x, dtype=np.float64)


def layout(D, H):
    W1 = 0
    b1 = W1 + H * D
    W2 = b1 + H
    b2 = W2 + H * H
    w3 = b2 + H
    b3 = w3 + H
    # the library pads each (member, species) block to a multiple of 8
    # parameters (16-byte aligned BF16 weights); the padding is zero
    return dict(W1=W1, b1=b1, W2=W2, b2=b2, w3=w3, b3=b3, P=(b3 + 1 + 7) // 8 * 8)


def unpack(p, D, H):
    L = layout(D, H)
    p = np.asarray(p, dtype=np.float64)
    return (p[L["W1"]:L["b1"]].reshape(H, D), p[L["b1"]:L["W2"]],
            p[L["W2"]:L["b2"]].reshape(H, H), p[L["b2"]:L["w3"]], p[L["w3"]:L["b3"]],
            p[L["b3"]])


def pack(W1, b1, W2, b2, w3, b3):
    p = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])
    P = layout(W1.shape[1], W1.shape[0])["P"]
    return np.concatenate([p, np.zeros(P - p.size)])


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sig(z)


def dsilu(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def d2silu(z):
    s = _sig(z)
    return s * (1.0 - s) * (2.0 + z * (1.0 - 2.0 * s))


def forward(p, x, D, H, emulate_bf16=False, tc=False):
    """y[B] and g = dy/dx [B, D] for standardised inputs x [B, D].  tc adds
    the rounding points of the tensor-core inference kernel (d2 and d1 are
    BF16 GEMM operands there, FP32 in the SIMT kernels)."""
    r = bf16 if emulate_bf16 else _id
    rt = r if tc else _id
    W1, b1, W2, b2, w3, b3 = unpack(p, D, H)
    W1h, W2h = r(W1), r(W2)
    x = r(x)
    z1 = x @ W1h.T + b1
    a1 = r(silu(z1))
    z2 = a1 @ W2h.T + b2
    y = silu(z2) @ w3 + b3
    d2 = w3 * dsilu(z2)
    d1 = dsilu(z1) * (rt(d2) @ W2h)
    g = rt(d1) @ W1h
    return dict(x=x, z1=z1, a1=a1, z2=z2, y=y, d2=d2, d1=d1, g=g, W1h=W1h, W2h=W2h, w3=w3)


def loss_and_grad(p, x, y_lab, t_lab, lam, D, H, emulate_bf16=False):
    """Loss = mean_b (y_b - y*_b)^2 + lam |g_b - t*_b|^2 (normalised units)
    and its gradient with respect to the flat parameter block p."""
    r = bf16 if emulate_bf16 else _id
    B = x.shape[0]
    f = forward(p, x, D, H, emulate_bf16)
    dy = f["y"] - y_lab
    dg = f["g"] - t_lab
    loss = np.mean(dy * dy + lam * (dg * dg).sum(1))
    eps = 2.0 * dy / B
    rv = 2.0 * lam * dg / B
    rh = r(rv)
    z1, z2, a1, x = f["z1"], f["z2"], f["a1"], f["x"]
    W1h, W2h, w3 = f["W1h"], f["W2h"], f["w3"]
    # tangent pass along r
    u1 = rh @ W1h.T
    v1 = r(dsilu(z1) * u1)
    u2 = v1 @ W2h.T
    v2 = dsilu(z2) * u2
    # reverse pass over value and tangent
    zb2 = r(eps[:, None] * w3 * dsilu(z2) + w3 * d2silu(z2) * u2)
    ub2 = r(w3 * dsilu(z2) * np.ones_like(z2))
    gW2 = zb2.T @ a1 + ub2.T @ v1
    gb2 = zb2.sum(0)
    gw3 = (eps[:, None] * silu(z2) + v2).sum(0)
    gb3 = eps.sum()
    ab1 = zb2 @ W2h
    vb1 = ub2 @ W2h
    zb1 = r(ab1 * dsilu(z1) + vb1 * d2silu(z1) * u1)
    ub1 = r(vb1 * dsilu(z1))
    gW1 = zb1.T @ x + ub1.T @ rh
    gb1 = zb1.sum(0)
    return loss, pack(gW1, gb1, gW2, gb2, gw3, gb3)


def numeric_grad(p, x, y_lab, t_lab, lam, D, H, h=1e-6):
    """Central finite differences of the exact float64 loss."""
    p = np.array(p, dtype=np.float64)
    out = np.zeros_like(p)
    for i in range(p.size):
        old = p[i]
        p[i] = old + h
        lp, _ = loss_and_grad(p, x, y_lab, t_lab, lam, D, H)
        p[i] = old - h
        lm, _ = loss_and_grad(p, x, y_lab, t_lab, lam, D, H)
        p[i] = old
        out[i] = (lp - lm) / (2 * h)
    return out


def committee(blocks, x, D, H, e_scale, e_shift, sd, emulate_bf16=False, tc=False):
    """Committee mean energy (eV), std (eV, ddof 1) and mean dE/dG for the
    rows x of one species, from that species' parameter blocks."""
    ys, gs = [], []
    for p in blocks:
        f = forward(p, x, D, H, emulate_bf16, tc)
        ys.append(f["y"])
        gs.append(f["g"])
    ys = np.array(ys)
    gs = np.array(gs)
    e = e_scale * ys.mean(0) + e_shift
    std = e_scale * ys.std(0, ddof=1) if len(blocks) > 1 else np.zeros(x.shape[0])
    dedg = e_scale * gs.mean(0) / sd
    return e, std, dedg
