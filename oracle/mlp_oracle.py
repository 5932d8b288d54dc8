"""CPU oracle of the learned warm start's network (test infrastructure only:
imported by the tests, never by the package).

The reference has no learned component; this is the mathematical definition
of the network the GPU kernels train, in numpy, with the kernels' rounding
points made explicit so that their gradients can be checked:

  x  = bf16((features - mean) / std)                      (17 -> padded 32)
  A1 = bf16(relu(x W0 + b0)), A2 = bf16(relu(A1 W1 + b1)),
  A3 = bf16(relu(A2 W2 + b2)),  y = A3 W3 + b3            (first 3 of 16)
  L  = sum over samples and the 3 outputs of (y - t_std)^2 / (3 n)

with BF16 weights and FP32 accumulation.  Backward: dZ3 = bf16(dL/dy),
dW_l = A_{l-1}^T dZ_l, db_l = column sums of dZ_l, dZ_{l-1} =
bf16((dZ_l W_l^T) * [A_{l-1} > 0]).  With ``exact=True`` every rounding is
skipped and the arithmetic is float64, for finite-difference checks.

Parameter layout: for l = 0..3, W_l as [K_l][N_l] row-major then b_l[N_l];
(K, N) = (32, 128), (128, 128), (128, 128), (128, 16).
"""
from __future__ import annotations

import numpy as np

NF, NO, KIN, H, KOUT = 17, 3, 32, 128, 16
SHAPES = [(KIN, H), (H, H), (H, H), (H, KOUT)]


def offsets():
    offs, o = [], 0
    for k, n in SHAPES:
        offs.append((o, o + k * n))
        o += k * n + n
    return offs, o


OFFS, NPARAM = offsets()


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), kept as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((b >> 16) & 1) + np.uint32(0x7FFF)
    return ((b + r) & np.uint32(0xFFFF0000)).view(np.float32)


def unpack(params):
    p = np.asarray(params)
    out = []
    for (k, n), (wo, bo) in zip(SHAPES, OFFS):
        out.append((p[wo:wo + k * n].reshape(k, n), p[bo:bo + n]))
    return out


def pack(layers):
    p = np.zeros(NPARAM, np.float32)
    for (W, b), (wo, bo) in zip(layers, OFFS):
        p[wo:wo + W.size] = W.reshape(-1)
        p[bo:bo + b.size] = b
    return p


def standardise(X, stats):
    return (np.asarray(X, np.float32) - stats[:NF]) / stats[NF:2 * NF]


def forward(params, stats, X, exact=False):
    """Outputs in target units (n x 3) and the activations."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    L = unpack(params)
    x = np.zeros((len(X), KIN), dt)
    x[:, :NF] = standardise(X, stats)
    x = rnd(x)
    acts = [x]
    a = x
    for l in range(3):
        W, b = L[l]
        z = a.astype(dt) @ rnd(W).astype(dt) + b.astype(dt)
        a = rnd(np.maximum(z, 0))
        acts.append(a)
    W, b = L[3]
    y = (a.astype(dt) @ rnd(W).astype(dt) + b.astype(dt))[:, :NO]
    return y, acts


def loss_and_grad(params, stats, X, T, exact=False):
    """Loss (mean squared error on standardised targets) and its gradient
    with respect to every parameter (NPARAM values)."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    n = len(X)
    y, acts = forward(params, stats, X, exact)
    tn = (np.asarray(T, dt) - stats[2 * NF:2 * NF + NO]) / stats[2 * NF + NO:2 * NF + 2 * NO]
    diff = y - tn
    loss = float(np.sum(diff.astype(np.float64) ** 2) / (NO * n))
    dz = np.zeros((n, KOUT), dt)
    dz[:, :NO] = 2.0 * diff / (NO * n)
    dz = rnd(dz)
    L = unpack(params)
    grads = [None] * 4
    for l in (3, 2, 1, 0):
        W, _ = L[l]
        a_prev = acts[l]
        gW = a_prev.astype(dt).T @ dz.astype(dt)
        gb = dz.astype(dt).sum(axis=0)
        grads[l] = (gW, gb)
        if l == 0:
            break
        da = dz.astype(dt) @ rnd(W).astype(dt).T
        dz = rnd(np.where(a_prev > 0, da, 0))
    return loss, pack([(g.astype(np.float32), b.astype(np.float32)) for g, b in grads]) if not exact else \
        _pack64(grads)


def _pack64(grads):
    p = np.zeros(NPARAM, np.float64)
    for (gW, gb), (wo, bo) in zip(grads, OFFS):
        p[wo:wo + gW.size] = gW.reshape(-1)
        p[bo:bo + gb.size] = gb
    return p


def loss_only(params, stats, X, T):
    y, _ = forward(params, stats, X, exact=True)
    tn = (np.asarray(T, np.float64) - stats[2 * NF:2 * NF + NO]) / stats[2 * NF + NO:2 * NF + 2 * NO]
    return float(np.sum((y - tn) ** 2) / (NO * len(X)))
