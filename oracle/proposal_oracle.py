"""CPU FP64 restatement of the learned rotation proposal network.

TEST INFRASTRUCTURE ONLY: the gradient checks of the GPU kernels import it;
the product path never does.

The network, its parameter layout and its precision points are the ones
the C ABI documents (``fftdock_proposal_*`` in include/fftdock.h).  This
module computes the same forward and backward passes in float64 and rounds to
BF16 exactly where the GPU stores BF16 (the weight copies, the occupancy grid,
the ReLU outputs of every layer, the descriptor, and the activation gradients
dzf, dz3, dz2, dz1 that the backward GEMMs read), so a GPU gradient must agree
with it up to FP32 accumulation order.  With ``bf16=False`` everything
stays float64, which the finite-difference check of this module itself uses.

The proposal has no counterpart in the reference; its occupancy grid uses the
scan's rotation arithmetic (p' = R p as ((r0 x0) + r1 x1) + r2 x2,
``include/PRODDL/Geom/transformation.hpp:206-222``).
"""
from __future__ import annotations

import numpy as np

G0, C1, C2, C3 = 16, 16, 32, 64
D1, D2, D3 = 8, 4, 2
NA3 = C3 * D3 ** 3
DESC = 128
NU = NA3 + DESC
HID = 256

SHAPES = [
    ("w1", (C1, 1, 3, 3, 3)), ("b1", (C1,)),
    ("w2", (C2, C1, 3, 3, 3)), ("b2", (C2,)),
    ("w3", (C3, C2, 3, 3, 3)), ("b3", (C3,)),
    ("f1", (NU, HID)), ("fb1", (HID,)),
    ("f2", (HID,)), ("fb2", (1,)),
]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(flat):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def bf16(x):
    """Round to BF16 (via float32, round to nearest even), back to float64."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def half_width(xyz):
    xyz = np.asarray(xyz, dtype=np.float64)
    r = np.sqrt((xyz[:, 0] * xyz[:, 0] + xyz[:, 1] * xyz[:, 1]) + xyz[:, 2] * xyz[:, 2])
    L = float(r.max()) if len(r) else 0.0
    return L if L > 0.0 else 1.0


def occupancy(xyz, L, rot):
    """16^3 atom counts of the rotated ligand, cell floor((p' + L) / (2L/16))."""
    xyz = np.asarray(xyz, dtype=np.float64)
    R = np.asarray(rot, dtype=np.float64).reshape(3, 3)
    cs = (2.0 * L) / float(G0)
    c = []
    for d in range(3):
        q = (R[d, 0] * xyz[:, 0] + R[d, 1] * xyz[:, 1]) + R[d, 2] * xyz[:, 2]
        k = np.floor((q + L) / cs).astype(np.int64)
        c.append(np.clip(k, 0, G0 - 1))
    occ = np.zeros(G0 ** 3)
    np.add.at(occ, (c[0] * G0 + c[1]) * G0 + c[2], 1.0)
    return occ.reshape(1, G0, G0, G0)


def descriptor(xyz, element):
    """Radial element histograms (fftdock_receptor_descriptor)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    out = np.zeros(DESC)
    if len(xyz) == 0:
        return out
    c = 0.5 * (xyz.min(axis=0) + xyz.max(axis=0))
    t = xyz - c
    r = np.sqrt((t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1]) + t[:, 2] * t[:, 2])
    shell = np.minimum(np.floor(r / 1.5).astype(np.int64), 31)
    np.add.at(out, np.asarray(element, dtype=np.int64) * 32 + shell, 1.0)
    return out / float(len(xyz))


def descriptor_oriented(xyz):
    """Scan-frame occupancy, 4^3 cells of all and of outer atoms
    (fftdock_receptor_descriptor_oriented)."""
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(DESC)
    if len(xyz) == 0:
        return out
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    c = 0.5 * (lo + hi)
    L = float((0.5 * (hi - lo)).max())
    L = L if L > 0 else 1.0
    t = xyz - c
    r = np.sqrt((t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1]) + t[:, 2] * t[:, 2])
    k = np.clip(np.floor((xyz - (c - L)) / (0.5 * L)).astype(np.int64), 0, 3)
    cell = (k[:, 0] * 4 + k[:, 1]) * 4 + k[:, 2]
    np.add.at(out, cell, 1.0)
    np.add.at(out, 64 + cell[r > 0.7 * r.max()], 1.0)
    return out / float(len(xyz))


def _taps(x, dout):
    """Patches of a stride-2, pad-1, 3^3 convolution: k -> [C, dout^3]."""
    c, d = x.shape[0], x.shape[1]
    xp = np.zeros((c, d + 2, d + 2, d + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    taps = []
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                taps.append(xp[:, kz:kz + 2 * dout:2, ky:ky + 2 * dout:2, kx:kx + 2 * dout:2].reshape(c, -1))
    return taps


def _conv(x, w, b, dout):
    taps = _taps(x, dout)
    wk = w.reshape(w.shape[0], w.shape[1], 27)
    z = b[:, None] + sum(wk[:, :, k] @ taps[k] for k in range(27))
    return z.reshape(w.shape[0], dout, dout, dout), taps


def _conv_bwd_data(dz, w, din):
    """Gradient of the conv input (shape [CIN, din^3]) from dz [COUT, dout^3]."""
    dout = din // 2
    cin = w.shape[1]
    wk = w.reshape(w.shape[0], cin, 27)
    g = np.zeros((cin, din + 2, din + 2, din + 2))
    dzf = dz.reshape(dz.shape[0], -1)
    k = 0
    for kz in range(3):
        for ky in range(3):
            for kx in range(3):
                g[:, kz:kz + 2 * dout:2, ky:ky + 2 * dout:2, kx:kx + 2 * dout:2] += \
                    (wk[:, :, k].T @ dzf).reshape(cin, dout, dout, dout)
                k += 1
    return g[:, 1:-1, 1:-1, 1:-1]


def forward_backward(params, samples, targets, bf=True):
    """Mean squared error of the samples and its gradient.

    ``samples``: list of (xyz, L, rot, desc).  Returns (loss, grad flat,
    predictions)."""
    P = unpack(params)
    rnd = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    W = {k: rnd(v) for k, v in P.items()}
    G = {k: np.zeros_like(v) for k, v in P.items()}
    B = len(samples)
    preds, loss = [], 0.0
    for (xyz, L, rot, desc), t in zip(samples, targets):
        x0 = rnd(0.25 * occupancy(xyz, L, rot))
        z1, t1 = _conv(x0, W["w1"], W["b1"], D1)
        a1 = rnd(np.maximum(z1, 0.0))
        z2, t2 = _conv(a1, W["w2"], W["b2"], D2)
        a2 = rnd(np.maximum(z2, 0.0))
        z3, t3 = _conv(a2, W["w3"], W["b3"], D3)
        a3 = rnd(np.maximum(z3, 0.0))
        u = np.concatenate([a3.reshape(-1), rnd(np.asarray(desc, dtype=np.float64))])
        zf = W["fb1"] + u @ W["f1"]
        h1 = rnd(np.maximum(zf, 0.0))
        y = W["fb2"][0] + h1 @ W["f2"]
        preds.append(y)
        loss += (y - t) ** 2 / B
        dy = 2.0 * (y - t) / B
        # backward
        G["f2"] += dy * h1
        G["fb2"] += dy
        dzf = rnd(np.where(h1 > 0, dy * W["f2"], 0.0))
        G["f1"] += np.outer(u, dzf)
        G["fb1"] += dzf
        du = W["f1"][:NA3] @ dzf
        dz3 = rnd(np.where(a3.reshape(-1) > 0, du, 0.0)).reshape(C3, -1)
        G["w3"] += np.stack([dz3 @ t3[k].T for k in range(27)], axis=-1).reshape(G["w3"].shape)
        G["b3"] += dz3.sum(axis=1)
        dz2 = rnd(np.where(a2 > 0, _conv_bwd_data(dz3, W["w3"], D2), 0.0)).reshape(C2, -1)
        G["w2"] += np.stack([dz2 @ t2[k].T for k in range(27)], axis=-1).reshape(G["w2"].shape)
        G["b2"] += dz2.sum(axis=1)
        dz1 = rnd(np.where(a1 > 0, _conv_bwd_data(dz2, W["w2"], D1), 0.0)).reshape(C1, -1)
        G["w1"] += np.stack([dz1 @ t1[k].T for k in range(27)], axis=-1).reshape(G["w1"].shape)
        G["b1"] += dz1.sum(axis=1)
    return loss, pack(G), np.array(preds)


def init_params(seed):
    """He-normal weights, zero biases (the distribution, not the GPU's draws)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    P = {}
    for name, shape in SHAPES:
        if name.startswith("b") or name.startswith("fb"):
            P[name] = np.zeros(shape)
        else:
            fan_in = {"w1": 27, "w2": C1 * 27, "w3": C2 * 27, "f1": NU, "f2": HID}[name]
            P[name] = rng.normal(0.0, np.sqrt(2.0 / fan_in), size=shape)
    return pack(P)
