"""TEST INFRASTRUCTURE ONLY -- CPU oracle for the learned form's network (efanna_gb300's efg_learned).

The product trains and runs the network with its own CUDA kernels (efanna_gb300/csrc/learned.cu);
this numpy restatement is what the tests check those kernels against.  It follows the same
arithmetic: inputs standardised per dimension and rounded to BF16, BF16 weights (rounded from the
FP32 master copy), BF16 copies of the hidden activations as GEMM operands, FP32 accumulation, FP32
gradients.  The loss is the softmax cross-entropy of the cluster logits against the histogram of the
query's 10 neighbour clusters plus the softmax cross-entropy of the rung logits against the label,
averaged over the batch.  With ``exact=True`` every step runs in float64 without rounding (used to
check the backward pass against finite differences).
"""
from __future__ import annotations

import numpy as np

GT_K = 10


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (round to nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def split(w: np.ndarray, din: int, H: int, O: int):
    """[W1 | b1 | W2 | b2 | W3 | b3] -> the six arrays (views)."""
    sizes = [H * din, H, H * H, H, O * H, O]
    out, o = [], 0
    for s in sizes:
        out.append(w[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(H, din), b1, W2.reshape(H, H), b2, W3.reshape(O, H), b3


def loss_and_grad(w, x, mean, istd, tclusters, tlabel, Cn, R, H, exact=False):
    """Loss (mean over rows) and the flat gradient for query rows x (B x din)."""
    din = x.shape[1]
    O = Cn + R
    f = np.float64 if exact else np.float32
    rnd = (lambda a: a.astype(np.float64)) if exact else bf16
    W1, b1, W2, b2, W3, b3 = split(np.asarray(w, f), din, H, O)
    xin = (np.asarray(x, np.float32) - mean.astype(np.float32)) * istd.astype(np.float32)
    xb = rnd(xin).astype(f)
    W1b, W2b, W3b = rnd(W1).astype(f), rnd(W2).astype(f), rnd(W3).astype(f)
    h1 = np.maximum(xb @ W1b.T + b1, 0).astype(f)
    h1b = rnd(h1).astype(f)
    h2 = np.maximum(h1b @ W2b.T + b2, 0).astype(f)
    h2b = rnd(h2).astype(f)
    z = (h2b @ W3b.T + b3).astype(f)
    B = x.shape[0]
    tgt = np.zeros((B, O), f)
    for g in range(GT_K):
        np.add.at(tgt, (np.arange(B), tclusters[:, g]), 1.0 / GT_K)
    tgt[np.arange(B), Cn + tlabel.astype(np.int64)] = 1.0
    dz = np.zeros_like(z)
    loss = 0.0
    for off, ln in ((0, Cn), (Cn, R)):
        zz = z[:, off:off + ln].astype(np.float64)
        lse = zz.max(1, keepdims=True) + np.log(np.exp(zz - zz.max(1, keepdims=True)).sum(1, keepdims=True))
        p = np.exp(zz - lse)
        t = tgt[:, off:off + ln]
        loss -= float((t * (zz - lse)).sum())
        dz[:, off:off + ln] = ((p - t) / B).astype(f)
    gW3 = dz.T @ h2b
    gb3 = dz.sum(0)
    dh2 = (dz @ W3b) * (h2 > 0)
    gW2 = dh2.T @ h1b
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2b) * (h1 > 0)
    gW1 = dh1.T @ xb
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss / B, g
