"""CPU restatement of the (s, m) proposer network, for checking the GPU kernels' forward pass
and gradients.  TEST INFRASTRUCTURE ONLY (imported by tests/).

Parameter layout (flat float32): W1[16][64] b1[64] W2[64][64] b2[64] W3[64][51] b3[51], W[i][j]
mapping input i to output j; ReLU after the two hidden layers; logits = 21 for s in 0..20 then
30 for m in 1..30; loss = mean over the batch of CE_s + CE_m.  Computed in float64 so the check
measures the GPU's float32 arithmetic, not the oracle's.
"""
from __future__ import annotations

import numpy as np

IN, H1, H2, OS, OM = 16, 64, 64, 21, 30
OUT = OS + OM
SHAPES = [("W1", (IN, H1)), ("b1", (H1,)), ("W2", (H1, H2)), ("b2", (H2,)), ("W3", (H2, OUT)), ("b3", (OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].astype(np.float64).reshape(shape)
        o += n
    return out


def forward(p: np.ndarray, X: np.ndarray):
    w = unpack(p)
    X = X.astype(np.float64)
    z1 = X @ w["W1"] + w["b1"]
    a1 = np.maximum(z1, 0)
    z2 = a1 @ w["W2"] + w["b2"]
    a2 = np.maximum(z2, 0)
    logits = a2 @ w["W3"] + w["b3"]
    return logits, (X, z1, a1, z2, a2)


def _softmax(l):
    e = np.exp(l - l.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grad(p: np.ndarray, X: np.ndarray, ys: np.ndarray, ym: np.ndarray):
    """Per-row loss and the gradient of the mean loss (flat, float64)."""
    w = unpack(p)
    logits, (X, z1, a1, z2, a2) = forward(p, X)
    B = X.shape[0]
    dl = np.zeros_like(logits)
    loss = np.zeros(B)
    for head, (o0, n, lab) in enumerate(((0, OS, ys), (OS, OM, ym - 1))):
        l = logits[:, o0:o0 + n]
        pr = _softmax(l)
        ok = (lab >= 0) & (lab < n)
        onehot = np.zeros_like(pr)
        onehot[np.arange(B)[ok], lab[ok]] = 1.0
        dl[:, o0:o0 + n] = np.where(ok[:, None], (pr - onehot) / B, 0.0)
        lse = np.log(np.exp(l - l.max(axis=1, keepdims=True)).sum(axis=1)) + l.max(axis=1)
        loss += np.where(ok, lse - l[np.arange(B), np.clip(lab, 0, n - 1)], 0.0)
    g = {"W3": a2.T @ dl, "b3": dl.sum(0)}
    d2 = (dl @ w["W3"].T) * (z2 > 0)
    g["W2"], g["b2"] = a1.T @ d2, d2.sum(0)
    d1 = (d2 @ w["W2"].T) * (z1 > 0)
    g["W1"], g["b1"] = X.T @ d1, d1.sum(0)
    flat = np.concatenate([g[name].ravel() for name, _ in SHAPES])
    return loss, flat
