"""CPU oracle of the learned (sigma_T c_R)max network (TEST INFRASTRUCTURE ONLY).

Restates the arithmetic of hystrath_gb300/csrc/dsmc_mlp.cu in numpy: the
3-64-64-1 SiLU perceptron with bf16-rounded weights and activations and FP32
sums, its mean-squared-error loss on standardised log maxima, and the
gradients its backward kernel produces (dout, dz2 and dz1 in FP32, bf16(dz2)
into the two tensor-core products).  With ``exact=True`` every rounding is
dropped and the sums run in FP64, so the formulas themselves can be checked
against finite differences.

The learned maximum has no reference counterpart (dsmcFoam+ keeps only the
running maximum of noTimeCounter.C:243-246); this oracle pins the kernels to
their own specification.  Only the tests import it.
"""
from __future__ import annotations

import numpy as np

H, IN = 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NPARAM = OFF_B3 + 1


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p, exact=False):
    p = np.asarray(p, dtype=np.float64 if exact else np.float32)
    q = p if exact else bf16(p)
    return (q[OFF_W1:OFF_B1].reshape(H, IN), q[OFF_B1:OFF_W2], q[OFF_W2:OFF_B2].reshape(H, H),
            q[OFF_B2:OFF_W3], q[OFF_W3:OFF_B3], q[OFF_B3])


def _silu(z):
    return z / (1 + np.exp(-z))


def _dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def forward(p, norm, X, exact=False):
    """Returns (out, cache): out is the standardised prediction."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    norm = np.asarray(norm, dtype=dt)
    mu, sd, = norm[0:3], norm[3:6]
    W1, b1, W2, b2, w3, b3 = unpack(p, exact)
    X = np.asarray(X, dtype=dt)
    xn = rnd((X - mu) / sd)
    z1 = (xn @ W1.T.astype(dt) + b1).astype(dt)
    a1 = rnd(_silu(z1).astype(dt))
    z2 = (a1 @ W2.T.astype(dt) + b2).astype(dt)
    a2 = rnd(_silu(z2).astype(dt))
    out = (a2 @ w3.astype(dt) + b3).astype(dt)
    return out, (xn, z1, a1, z2, a2)


def predict(p, norm, X, exact=False):
    """log maximum: ymean + yscale * net(x)."""
    out, _ = forward(p, norm, X, exact)
    return norm[6] + norm[7] * out


def loss_grad(p, norm, X, Y, exact=False):
    """Mean squared error on standardised targets and its gradient."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(dt)) if exact else bf16
    norm = np.asarray(norm, dtype=dt)
    W1, b1, W2, b2, w3, b3 = unpack(p, exact)
    out, (xn, z1, a1, z2, a2) = forward(p, norm, X, exact)
    yn = ((np.asarray(Y, dtype=dt) - norm[6]) / norm[7]).astype(dt)
    e = out - yn
    n = len(Y)
    loss = float(np.mean(e.astype(np.float64) ** 2))
    dout = (2 * e / n).astype(dt)
    g = np.zeros(NPARAM, dtype=np.float64)
    g[OFF_W3:OFF_B3] = a2.T @ dout
    g[OFF_B3] = dout.sum()
    dz2 = (dout[:, None] * w3[None, :] * _dsilu(z2)).astype(dt)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz2b = rnd(dz2)
    g[OFF_W2:OFF_B2] = (dz2b.T @ a1).ravel()
    dh1 = (dz2b @ W2.astype(dt)).astype(dt)
    dz1 = (dh1 * _dsilu(z1)).astype(dt)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (dz1.T @ xn).ravel()
    return loss, g
