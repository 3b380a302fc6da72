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


def test_canonical_row_order_is_independent_of_arrival_order():
    """learned.canonical_order: the same multiset of harvested rows, appended in any order, comes
    out in one order (what makes the harvest-to-network workflow repeat bit for bit)."""
    import torch

    from hteno import learned

    g = torch.Generator().manual_seed(3)
    x = torch.randint(-3, 3, (5000, 8), dtype=torch.int16, generator=g)
    y = torch.randint(0, 8, (5000,), dtype=torch.uint8, generator=g)
    o = learned.canonical_order(torch, x, y)
    perm = torch.randperm(5000, generator=g)
    xp, yp = x[perm].contiguous(), y[perm].contiguous()
    op = learned.canonical_order(torch, xp, yp)
    assert torch.equal(x[o], xp[op]) and torch.equal(y[o], yp[op])
