"""Accuracy figures of a solution against a reference solution on the same grid."""
from __future__ import annotations

import numpy as np


def density_errors(a, b):
    """(L1, Linf) of the density difference of two conserved states [4][ny][nx]."""
    d = np.abs(np.asarray(a)[0] - np.asarray(b)[0])
    return float(d.mean()), float(d.max())


def shock_shift(rho, rho_ref, frac=0.25, window=4):
    """Largest displacement, in cells, of the steepest density jump between two solutions: along
    every grid line (both directions) whose steepest reference jump exceeds `frac` of the
    largest jump anywhere, the position of the steepest jump of `rho` within `window` cells of
    the reference's is compared with the reference's."""
    worst = 0
    for axis in (0, 1):
        gr = np.abs(np.diff(rho_ref, axis=axis))
        gt = np.abs(np.diff(rho, axis=axis))
        if axis == 0:
            gr, gt = gr.T, gt.T
        big = gr.max() * frac
        for line in np.nonzero(gr.max(axis=1) > big)[0]:
            p = int(np.argmax(gr[line]))
            lo, hi = max(0, p - window), min(gr.shape[1], p + window + 1)
            q = lo + int(np.argmax(gt[line, lo:hi]))
            worst = max(worst, abs(q - p))
    return worst
