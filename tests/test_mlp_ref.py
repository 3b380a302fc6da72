"""The CPU check of the learned classifier (oracle/mlp_ref.py) against finite differences, with
the BF16 roundings switched off, so the GPU gradient test compares against correct formulas."""
from __future__ import annotations

import numpy as np


def test_mlp_ref_gradient_matches_finite_differences():
    import mlp_ref

    rng = np.random.default_rng(0)
    p = rng.standard_normal(mlp_ref.N_PARAMS) * 0.5
    x = rng.standard_normal((40, 6)) * 0.5
    y = rng.integers(0, 8, 40)
    with mlp_ref.exact():
        _, g = mlp_ref.loss_and_grad(p, x, y)
        for i in list(range(0, 1379, 37)) + [1376, 1377, 1378]:
            e = 1e-6
            pp = p.copy()
            pp[i] += e
            lp = mlp_ref.loss_and_grad(pp, x, y)[0]
            pp[i] -= 2 * e
            lm = mlp_ref.loss_and_grad(pp, x, y)[0]
            assert abs((lp - lm) / (2 * e) - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), i


def test_mlp_ref_bf16_rounding():
    import mlp_ref

    v = mlp_ref.bf16(np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159, 0.0]))
    np.testing.assert_array_equal(v, [1.0, 1.0, 1.0 + 4 * 2 ** -8, -3.140625, 0.0])


def test_normalised_stencil_range():
    import mlp_ref

    s = mlp_ref.normalise(np.array([[1.0, 2, 3, 4, 5, 6], [2.0, 2, 2, 2, 2, 2]]))
    assert np.allclose(s.max(axis=1) - s.min(axis=1), [1.0, 0.0]) and np.allclose(s.mean(axis=1), 0)
