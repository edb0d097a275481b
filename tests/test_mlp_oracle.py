"""The network oracle itself (CPU): its gradient against finite differences, BF16 rounding."""
from __future__ import annotations

import numpy as np

from oracle import mlp_oracle as M


def _setup(n_mix, seed=0):
    rng = np.random.default_rng(seed)
    d = M.dims(4, 16, 3, 5, n_mix)
    n_params = sum(d[l + 1] * d[l] + d[l + 1] for l in range(len(d) - 1))
    p = rng.standard_normal(n_params) * 0.3
    x = rng.standard_normal((7, 4))
    t = rng.standard_normal((7, 5))
    mix = rng.uniform(0.2, 1.0, (7, n_mix)) if n_mix else None
    w = rng.uniform(0.5, 2.0, 7)
    return d, p, x, t, mix, w


def test_gradient_matches_finite_differences():
    for n_mix in (0, 2):
        d, p, x, t, mix, w = _setup(n_mix)
        loss, g = M.loss_and_grad(p, d, x, t, mix, w, n_mix, emulate_bf16=False)
        rng = np.random.default_rng(5)
        for k in rng.choice(p.size, 25, replace=False):
            e = np.zeros_like(p)
            e[k] = 1e-6
            lp, _ = M.loss_and_grad(p + e, d, x, t, mix, w, n_mix, emulate_bf16=False)
            lm, _ = M.loss_and_grad(p - e, d, x, t, mix, w, n_mix, emulate_bf16=False)
            fd = (lp - lm) / 2e-6
            assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (n_mix, k, fd, g[k])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-3, 0.0], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even
    assert r[2] == 1.0 + 4 * 2 ** -8        # tie -> even (up)
    assert r[3] == -2.5 and r[5] == 0.0
    assert abs(r[4] - 1e-3) / 1e-3 < 2 ** -8
