"""CPU oracle of the learned sensor's network (test infrastructure only).

Restates, in numpy, the forward pass and the loss gradient that the CUDA
kernels (enlightning_gb300/csrc/enl_mlp.cu, enl_mlp.cuh) compute on the
tensor cores, with BF16 rounding at the same points: inputs and weight
matrices (W1, W2, w3) in BF16, hidden activations rounded to BF16 where they
feed the next layer, back-propagated deltas rounded to BF16 where they feed a
tensor-core product; accumulation in float64 here (FP32 on the GPU), so the
two agree to accumulation-order rounding.

Parameter vector layout: W1[40][64], b1[64], W2[64][64], b2[64], w3[64], b3.
Loss: sum_s w_s * BCE(sigmoid(logit_s), y_s).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

NF, NH = 40, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NF * NH
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAMS = OFF_B3 + 1


ROUND = True  # BF16 rounding points on; off for finite-difference checks in float64


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    if not ROUND:
        return np.asarray(x, dtype=np.float64)
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32)


def unpack(P):
    P = np.asarray(P, dtype=np.float32 if ROUND else np.float64)
    return (P[OFF_W1:OFF_B1].reshape(NF, NH), P[OFF_B1:OFF_W2], P[OFF_W2:OFF_B2].reshape(NH, NH),
            P[OFF_B2:OFF_W3], P[OFF_W3:OFF_B3], P[OFF_B3])


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def forward(P, X):
    W1, b1, W2, b2, w3, b3 = unpack(P)
    Xb = bf16(X).astype(np.float64)
    z1 = Xb @ bf16(W1).astype(np.float64) + b1
    h1 = bf16(gelu(z1)).astype(np.float64)
    z2 = h1 @ bf16(W2).astype(np.float64) + b2
    h2 = bf16(gelu(z2)).astype(np.float64)
    logit = h2 @ bf16(w3).astype(np.float64) + float(b3)
    return logit, (Xb, z1, h1, z2, h2)


def loss_and_grad(P, X, y, w):
    W1, b1, W2, b2, w3, b3 = unpack(P)
    logit, (Xb, z1, h1, z2, h2) = forward(P, X)
    p = 1.0 / (1.0 + np.exp(-logit))
    loss = np.sum(w * (np.maximum(logit, 0) - y * logit + np.log1p(np.exp(-np.abs(logit)))))
    dl = w * (p - y)
    if ROUND:
        dl = dl.astype(np.float32).astype(np.float64)
    w3b = bf16(w3).astype(np.float64)
    dz2 = bf16(dl[:, None] * w3b[None, :] * gelu_grad(z2)).astype(np.float64)
    dh1 = dz2 @ bf16(W2).astype(np.float64).T
    dz1 = bf16(dh1 * gelu_grad(z1)).astype(np.float64)
    g = np.zeros(NPARAMS)
    g[OFF_W1:OFF_B1] = (Xb.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = h2.T @ dl
    g[OFF_B3] = dl.sum()
    return loss, g


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    P = np.zeros(NPARAMS, np.float32)
    P[OFF_W1:OFF_B1] = rng.normal(0, np.sqrt(2.0 / NF), NF * NH)
    P[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2.0 / NH), NH * NH)
    P[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(1.0 / NH), NH)
    return P
