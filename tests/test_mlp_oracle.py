"""The FP64 oracle of the radiance-cache network checked against itself:
finite-difference gradients, the encoding's closed form, and that Adam
reduces the loss on a small fitting problem."""
from __future__ import annotations

import numpy as np

from oracle_lib import OracleMlp


def init_weights(n, seed=0):
    rng = np.random.default_rng(seed)
    fan = np.concatenate([np.full(64 * 216, 216), np.full(3 * 64 * 64, 64), np.full(3 * 64, 64)])
    return rng.uniform(-1, 1, n) * np.sqrt(6.0 / fan)


def test_encoding_closed_form(oracle):
    m = OracleMlp(oracle)
    x = np.array([[0.25, 0.5, 0.125, 1.0, 0.0, -0.5, 0.75, -1.0, 0.3]], np.float32)
    e = m.encode(x)[0]
    for i in range(9):
        for k in range(12):
            a = np.pi * (2.0 ** k) * np.float64(x[0, i])
            assert abs(e[(i * 12 + k) * 2] - np.sin(a)) < 1e-12
            assert abs(e[(i * 12 + k) * 2 + 1] - np.cos(a)) < 1e-12


def test_gradient_matches_finite_differences(oracle):
    m = OracleMlp(oracle)
    assert m.n_params == 64 * 216 + 3 * 64 * 64 + 3 * 64
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, (8, 9)).astype(np.float32)
    t = rng.uniform(0, 2, (8, 3)).astype(np.float32)
    w = init_weights(m.n_params)
    loss, g = m.loss_grad(w, x, t)
    # the relative loss treats the denominator as a constant: check against a
    # finite difference of the numerator-only objective with frozen denominators
    y0 = m.forward(w, x)
    den = y0 ** 2 + 0.01

    def obj(wv):
        y = m.forward(wv, x)
        return float(np.sum((y - t) ** 2 / den) / (3 * len(x)))

    assert abs(obj(w) - loss) < 1e-12
    idx = np.concatenate([rng.integers(0, 64 * 216, 12), rng.integers(64 * 216, m.n_params, 12)])
    for i in idx:
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (obj(wp) - obj(wm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_adam_fits_a_smooth_field(oracle):
    m = OracleMlp(oracle)
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 1, (256, 9)).astype(np.float32)
    t = (0.5 + 0.4 * np.sin(3 * x[:, :3])).astype(np.float32)
    w = init_weights(m.n_params, 3)
    mm = np.zeros_like(w)
    vv = np.zeros_like(w)
    first, _ = m.loss_grad(w, x, t)
    for step in range(1, 41):
        loss, g = m.loss_grad(w, x, t)
        m.adam(w, mm, vv, g, step, lr=1e-2)
    assert loss < 0.2 * first
