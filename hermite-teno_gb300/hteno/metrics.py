"""Accuracy figures of a solution against a reference solution on the same grid."""
from __future__ import annotations

import numpy as np


def density_errors(a, b):
    """(L1, Linf) of the density difference of two conserved states [4][ny][nx]."""
    d = np.abs(np.asarray(a)[0] - np.asarray(b)[0])
    return float(d.mean()), float(d.max())


def _steepest_near(g, p, window):
    """Index of the largest entry of the line g near p: searched within `window` cells of p, the
    window doubled while the largest entry sits on its edge (so a displacement of any size is
    found, not cut off at the window)."""
    n = g.shape[0]
    w = max(1, window)
    while True:
        lo, hi = max(0, p - w), min(n, p + w + 1)
        q = lo + int(np.argmax(g[lo:hi]))
        if abs(q - p) < w or (lo == 0 and hi == n):
            return q
        w *= 2


def shock_shift(rho, rho_ref, frac=0.25, window=4):
    """Largest displacement, in cells, of the steepest density jump between two solutions: along
    every grid line (both directions) whose steepest reference jump exceeds `frac` of the
    largest jump anywhere, the position of the steepest jump of `rho` near the reference's (within
    `window` cells, the window widened while the match sits on its edge) is compared with the
    reference's."""
    worst = 0
    for axis in (0, 1):
        gr = np.abs(np.diff(rho_ref, axis=axis))
        gt = np.abs(np.diff(rho, axis=axis))
        if axis == 0:
            gr, gt = gr.T, gt.T
        big = gr.max() * frac
        for line in np.nonzero(gr.max(axis=1) > big)[0]:
            p = int(np.argmax(gr[line]))
            q = _steepest_near(gt[line], p, window)
            worst = max(worst, abs(q - p))
    return worst
