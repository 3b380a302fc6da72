"""Accuracy figures used by the measurements (hteno/metrics.py)."""
from __future__ import annotations

import numpy as np


def test_shock_shift_and_errors():
    from hteno import metrics

    a = np.zeros((20, 30))
    a[:, 10:] = 1.0
    b = np.zeros((20, 30))
    b[:, 12:] = 1.0
    assert metrics.shock_shift(a, a) == 0 and metrics.shock_shift(b, a) == 2
    c = np.zeros((20, 30))
    c[:, 10:] = 1.0
    c[5, 3] = 0.1  # a weak feature far from the jump does not count
    assert metrics.shock_shift(c, a) == 0
    qa, qb = np.stack([a] * 4), np.stack([b] * 4)
    l1, linf = metrics.density_errors(qb, qa)
    assert l1 == 2 * 20 / 600 and linf == 1.0


def test_shock_shift_beyond_the_first_window():
    """A jump displaced by more than the search window is still measured (the window widens)."""
    from hteno import metrics

    a = np.zeros((8, 64))
    a[:, 20:] = 1.0
    for d in (3, 4, 5, 9, 17, 30):
        b = np.zeros((8, 64))
        b[:, 20 + d:] = 1.0
        assert metrics.shock_shift(b, a) == d, d
