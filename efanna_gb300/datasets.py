"""Seeded synthetic vector sets that stand in for the benchmark corpora.

SIFT1M/GIST1M are not available offline, so the workloads use seeded generators with the
same shapes and value ranges:

* ``mixture_u8``: an isotropic Gaussian mixture in ``d`` dimensions (Dirichlet(5) component
  weights, gamma(0.8, 25) centres, per-component sigma ~ U(10, 30)), clipped to [0, 255] and
  rounded to integers -- non-negative, heavy-tailed and histogram-like, as SIFT descriptors are.
  Integer-valued data make every squared distance an exact FP32 integer (< 2**24 for d <= 128).
* ``mixture_unit``: a Dirichlet-weighted mixture of non-negative components with values in
  [0, 1] and L1-normalised blocks (GIST-like, for the high-dimensional precision workload).

* ``mixture_unit_device``: the same GIST-like family drawn on the GPU with torch's seeded
  generator (the 1M x 960 workload: numpy's gamma draws would take tens of seconds on the host).
* ``mixture_aniso_device``: a Gaussian mixture with anisotropic covariances -- per component a
  random rotation times a decaying spectrum -- drawn on the GPU (the 10M x 96 workload of the
  learned form).

Base points use ``seed`` and queries ``seed + 1``; the mixture parameters always come from
``seed``, so queries are held-out draws from the same mixture.  The device generators depend on
torch's generator, so their draws are reproducible for a given torch build, not across builds.
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


def mixture_unit_device(n: int, d: int = 960, n_comp: int = 32, block: int = 16, seed: int = 0,
                        queries: bool = False, chunk: int = 1 << 17):
    """``n`` x ``d`` float32 CUDA tensor in [0, 1], L1-normalised per block of ``block`` dims: a
    Dirichlet-weighted mixture of ``n_comp`` gamma-distributed components, drawn on the GPU."""
    import torch
    assert d % block == 0
    g = torch.Generator(device="cuda").manual_seed(seed)
    # component parameters always from `seed`; samples from seed + 1 for queries
    weights = torch._sample_dirichlet(torch.full((n_comp,), 5.0, device="cuda"), generator=g)
    alpha = torch._standard_gamma(torch.full((n_comp, d), 2.0, device="cuda"), generator=g) + 0.05
    gs = torch.Generator(device="cuda").manual_seed(seed + 1) if queries else g
    out = torch.empty((n, d), dtype=torch.float32, device="cuda")
    for s0 in range(0, n, chunk):
        e = min(n, s0 + chunk)
        comp = torch.multinomial(weights, e - s0, replacement=True, generator=gs)
        x = torch._standard_gamma(alpha[comp], generator=gs).view(e - s0, d // block, block)
        x /= x.sum(dim=2, keepdim=True)
        out[s0:e] = x.view(e - s0, d)
    return out


def mixture_aniso_device(n: int, d: int = 96, n_comp: int = 1024, seed: int = 0, queries: bool = False,
                         spread: float = 0.3, decay: float = 0.35, sample_seed: int | None = None):
    """``n`` x ``d`` float32 CUDA tensor from a seeded mixture of ``n_comp`` anisotropic Gaussians:
    centres ~ N(0, spread^2 I); component k draws R_k (s * z) with R_k a random rotation (QR of a
    Gaussian matrix) and the spectrum s_i = (i + 1)^-decay scaled by a per-component U(0.5, 1.5).
    The defaults (spread 0.3, decay 0.35) make overlapping components of high intrinsic dimension:
    at 10M points a K = 32 graph search reaches recall@10 0.95 near a pool of 1,000 and per-query
    difficulty varies widely (as on SIFT-like data).  The difficulty turns sharply with the decay: at
    0.3 the same search levels off near recall 0.944 at 10M, at 0.4 it passes 0.95 at a pool of 400.
    With ``sample_seed`` the draws come from that seed (a further held-out sample, e.g. training
    queries)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    weights = torch._sample_dirichlet(torch.full((n_comp,), 5.0, device="cuda"), generator=g)
    centres = torch.randn((n_comp, d), generator=g, device="cuda") * spread
    q, r = torch.linalg.qr(torch.randn((n_comp, d, d), generator=g, device="cuda"))
    q = q * torch.sign(torch.diagonal(r, dim1=1, dim2=2)).unsqueeze(1)  # uniformly random orthogonal
    spec = (torch.arange(1, d + 1, device="cuda", dtype=torch.float32) ** -decay)
    scale = torch.rand((n_comp, 1), generator=g, device="cuda") + 0.5
    basis = q * (spec.unsqueeze(0) * scale).unsqueeze(1)  # R_k diag(s_k)
    if sample_seed is not None:
        gs = torch.Generator(device="cuda").manual_seed(sample_seed)
    else:
        gs = torch.Generator(device="cuda").manual_seed(seed + 1) if queries else g
    comp = torch.cat([torch.multinomial(weights, min(1 << 20, n - s0), replacement=True, generator=gs)
                      for s0 in range(0, n, 1 << 20)])
    order = torch.argsort(comp, stable=True)
    counts = torch.bincount(comp, minlength=n_comp).tolist()
    z = torch.randn((n, d), generator=gs, device="cuda")  # row i of z belongs to the i-th row in component order
    out = torch.empty((n, d), dtype=torch.float32, device="cuda")
    start = 0
    for k, c in enumerate(counts):  # one rotation per component: a matmul over its rows
        if c:
            out[order[start:start + c]] = centres[k] + z[start:start + c] @ basis[k].T
        start += c
    return out
