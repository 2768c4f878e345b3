"""CPU reference of the occluder-proposal network (test infrastructure only).

float64 arithmetic with bf16 rounding at the points where the GPU kernels
store bf16 (inputs, weights, hidden activations, output and hidden
gradients), so the GPU loss and gradients can be checked against it; the
remaining differences are fp32-vs-fp64 accumulation and the erf/exp
implementations.
"""
from __future__ import annotations

import math

import numpy as np

IN_USED, IN, H, OUT, OUT_PAD = 45, 48, 128, 3, 16
GATE, GATE_WEIGHT = 3, 0.05


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layout():
    sizes = [H * IN, H, H * H, H, H * H, H, OUT_PAD * H, OUT_PAD]
    shapes = [(H, IN), (H,), (H, H), (H,), (H, H), (H,), (OUT_PAD, H), (OUT_PAD,)]
    off = np.concatenate([[0], np.cumsum(sizes)])
    return sizes, shapes, off


def unpack(params):
    sizes, shapes, off = layout()
    p = np.asarray(params, np.float32)
    return [p[off[i]:off[i + 1]].reshape(shapes[i]) for i in range(8)]


def pack(parts):
    return np.concatenate([np.asarray(x, np.float32).reshape(-1) for x in parts])


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def random_params(seed: int):
    rng = np.random.default_rng(seed)
    parts = []
    for (o, i) in ((H, IN), (H, H), (H, H), (OUT_PAD, H)):
        w = rng.uniform(-1.0, 1.0, (o, i)) / math.sqrt(IN_USED if i == IN else i)
        if i == IN:
            w[:, IN_USED:] = 0.0
        if o == OUT_PAD:
            w[OUT + 1:, :] = 0.0
        b = rng.uniform(-0.1, 0.1, o)
        if o == OUT_PAD:
            b[OUT + 1:] = 0.0
            b[:OUT] += 0.6
        parts += [w, b]
    return pack(parts)


def forward(params, x):
    W1, b1, W2, b2, W3, b3, W4, b4 = [np.asarray(p, np.float64) for p in unpack(params)]
    xb = np.zeros((x.shape[0], IN))
    xb[:, :IN_USED] = bf16(x)
    Ws = [bf16(W) for W in (W1, W2, W3, W4)]
    Z, A = [], [xb]
    for l, b in enumerate((b1, b2, b3)):
        z = A[-1] @ Ws[l].T + b
        Z.append(z)
        A.append(bf16(gelu(z)))
    O = A[-1] @ Ws[3].T + b4
    return O, Z, A, Ws


def loss_and_grad(params, x, t, kind):
    O, Z, A, Ws = forward(params, x)
    M = x.shape[0]
    dO = np.zeros_like(O)
    loss = 0.0
    for i in range(M):
        o = O[i, :OUT]
        if kind[i] == 1:
            best = int(np.argmin(np.abs(o - t[i])))
            for k in range(OUT):
                w = 1.0 if k == best else 0.02
                d = o[k] - t[i]
                loss += w * d * d
                dO[i, k] = 2.0 * w * d
        elif kind[i] == 0:
            for k in range(OUT):
                d = 1.1 - o[k]
                if d > 0:
                    loss += 0.5 * d * d
                    dO[i, k] = -d
        if kind[i] in (0, 1):
            z, y = O[i, GATE], float(kind[i] == 1)
            loss += GATE_WEIGHT * (max(z, 0.0) - y * z + math.log1p(math.exp(-abs(z))))
            dO[i, GATE] = GATE_WEIGHT * (1.0 / (1.0 + math.exp(-z)) - y)
    loss /= M
    dO = bf16(dO / M)
    grads = [None] * 8
    grads[6] = dO.T @ A[3]
    grads[7] = dO.sum(0)
    dA = dO @ Ws[3]
    for l in (2, 1, 0):
        dZ = bf16(dA * gelu_grad(Z[l]))
        grads[2 * l] = dZ.T @ A[l]
        grads[2 * l + 1] = dZ.sum(0)
        dA = dZ @ Ws[l]
    return loss, pack(grads), O[:, :OUT + 1]
