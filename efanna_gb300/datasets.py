"""Seeded synthetic vector sets that stand in for the benchmark corpora.

SIFT1M/GIST1M are not available offline, so the workloads use seeded generators with the
same shapes and value ranges:

* ``mixture_u8``: an isotropic Gaussian mixture in ``d`` dimensions (Dirichlet(5) component
  weights, gamma(0.8, 25) centres, per-component sigma ~ U(10, 30)), clipped to [0, 255] and
  rounded to integers -- non-negative, heavy-tailed and histogram-like, as SIFT descriptors are.
  Integer-valued data make every squared distance an exact FP32 integer (< 2**24 for d <= 128).
* ``mixture_unit``: a Dirichlet-weighted mixture of non-negative components with values in
  [0, 1] and L1-normalised blocks (GIST-like, for the high-dimensional precision workload).

Base points use ``seed`` and queries ``seed + 1``; the mixture parameters always come from
``seed``, so queries are held-out draws from the same mixture.
"""
from __future__ import annotations

import numpy as np


def _mixture_params(d: int, n_comp: int, seed: int):
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.full(n_comp, 5.0))
    centres = rng.gamma(0.8, 25.0, size=(n_comp, d))
    sigma = rng.uniform(10.0, 30.0, size=n_comp)
    return rng, w, centres, sigma


def mixture_u8(n: int, d: int = 128, n_comp: int = 64, seed: int = 0, queries: bool = False,
               chunk: int = 1 << 18, sample_seed: int | None = None) -> np.ndarray:
    """``n`` x ``d`` float32 integer-valued vectors of the seeded Gaussian mixture.  With
    ``sample_seed`` the draws come from that seed (a further held-out sample of the same mixture,
    e.g. training queries)."""
    prng, w, centres, sigma = _mixture_params(d, n_comp, seed)
    if sample_seed is not None:
        rng = np.random.default_rng(sample_seed)
    else:
        rng = np.random.default_rng(seed + 1) if queries else prng
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        comp = rng.choice(n_comp, size=e - s, p=w)
        x = centres[comp] + rng.standard_normal((e - s, d)) * sigma[comp, None]
        np.rint(np.clip(x, 0.0, 255.0), out=x)
        out[s:e] = x
    return out


def mixture_unit(n: int, d: int = 960, n_comp: int = 32, block: int = 16, seed: int = 0,
                 queries: bool = False, chunk: int = 1 << 16) -> np.ndarray:
    """``n`` x ``d`` float32 vectors in [0, 1], L1-normalised per block of ``block`` dims."""
    assert d % block == 0
    prng = np.random.default_rng(seed)
    w = prng.dirichlet(np.full(n_comp, 5.0))
    alpha = prng.gamma(2.0, 1.0, size=(n_comp, d)) + 0.05
    rng = np.random.default_rng(seed + 1) if queries else prng
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        comp = rng.choice(n_comp, size=e - s, p=w)
        g = rng.gamma(alpha[comp], 1.0)
        g = g.reshape(e - s, d // block, block)
        g /= g.sum(axis=2, keepdims=True)
        out[s:e] = g.reshape(e - s, d)
    return out


def sign_codes(x: np.ndarray, tables: int, bits: int, seed: int = 0, center: np.ndarray | None = None,
               chunk: int = 1 << 16) -> np.ndarray:
    """Binary codes for the hashing-seeded search: per table, ``bits`` seeded random hyperplanes
    through ``center`` (pass the base's mean for base and queries alike); bit b of a code is set
    where the point lies on the positive side of hyperplane b.  Returns tables x n uint64."""
    x = np.asarray(x, dtype=np.float32)
    if center is None:
        center = x.mean(0)
    rng = np.random.default_rng(seed)
    planes = rng.standard_normal((tables, x.shape[1], bits)).astype(np.float32)
    weights = (np.uint64(1) << np.arange(bits, dtype=np.uint64))
    out = np.empty((tables, x.shape[0]), dtype=np.uint64)
    for s in range(0, x.shape[0], chunk):
        xc = x[s:s + chunk] - center
        for t in range(tables):
            side = (xc @ planes[t]) > 0
            out[t, s:s + chunk] = (side.astype(np.uint64) * weights).sum(1, dtype=np.uint64)
    return out
