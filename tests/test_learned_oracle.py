"""The learned form's CPU network oracle (oracle/mlp_oracle.py): its backward pass against finite
differences, and its BF16 rounding."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import mlp_oracle as M  # noqa: E402


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    din, H, Cn, R, B = 6, 5, 4, 3, 7
    n = H * din + H + H * H + H + (Cn + R) * H + Cn + R
    w = rng.normal(0, 0.5, n)
    x = rng.normal(0, 1, (B, din)).astype(np.float32)
    mean, istd = np.zeros(din, np.float32), np.ones(din, np.float32)
    tc = rng.integers(0, Cn, (B, M.GT_K))
    tl = rng.integers(0, R, B)
    loss, g = M.loss_and_grad(w, x, mean, istd, tc, tl, Cn, R, H, exact=True)
    eps = 1e-6
    num = np.zeros(n)
    for i in range(n):
        wp, wm = w.copy(), w.copy()
        wp[i] += eps
        wm[i] -= eps
        num[i] = (M.loss_and_grad(wp, x, mean, istd, tc, tl, Cn, R, H, exact=True)[0] -
                  M.loss_and_grad(wm, x, mean, istd, tc, tl, Cn, R, H, exact=True)[0]) / (2 * eps)
    assert np.linalg.norm(num - g) / np.linalg.norm(num) < 1e-6
    assert loss > 0


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 255.0, 257.0], np.float32)
    r = M.bf16(v)
    # 8 significant bits: 1 + 2^-8 is a tie -> even (1.0); 1 + 3*2^-8 ties up to 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1 + 2 ** -6) and r[3] == 1.0
    assert r[4] == -2.5 and r[5] == 255.0 and r[6] == 256.0
