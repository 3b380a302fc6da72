"""The float cut-off rule of the plain FP64 path (parity_math.cuh: scaled_ratios + cutoff_core),
restated in numpy float32 and checked on the CPU against the reference's own decision (the
cut-off of cutOff(), Schemes_Lagrange.cpp:1141-1149, evaluated in double with pow): wherever the
rule decides (outside its guard band, inside its scaling range) it decides as the reference does.
The device code is checked bit for bit against the oracle by the GPU tests; this test pins the
error analysis behind the guard band on many more cases, including adversarial ones near the
cut-off.  (numpy's float32 reciprocal-and-multiply stands in for __fdividef: both are within
2 ulp.)"""
from __future__ import annotations

import numpy as np

F32 = np.float32
CT, EPSZ, BAND = 5e-4, 1e-40, 2.0 ** -13


def reference_pattern(SI, tau):
    d = SI + EPSZ
    with np.errstate(over="ignore", invalid="ignore"):
        w = np.power(1.0 + tau / d, 6.0)
        s = (w[0] + w[1]) + w[2]
        return sum(np.where(w[k] / s < CT, 0, 1) << k for k in range(3)), np.isfinite(s)


def float_rule(SI, tau):
    """(pattern, decided) of the float path: decided is False where the rule hands the decision on
    (value out of the scaling range, or inside the guard band)."""
    d = SI + EPSZ
    vals = np.vstack([d, tau[None, :]])
    e = ((vals.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    em = e.max(axis=0)
    ok = em < 0x7FF
    for i in range(4):
        zero = (vals[i] == 0) if i == 3 else np.zeros(vals.shape[1], bool)
        ok &= zero | ((e[i] != 0) & (e[i] + 125 >= em))
    with np.errstate(all="ignore"):
        f = np.ldexp(vals, -(em - 1023)[None, :].repeat(4, 0)).astype(F32)
        dmin = np.minimum(np.minimum(f[0], f[1]), f[2])
        x = np.stack([(dmin * (F32(1) / f[k])) * ((f[k] + f[3]) * (F32(1) / (dmin + f[3])))
                      for k in range(3)]).astype(F32)
        x2 = x * x
        a = (x2 * x2) * x2
        lim = F32(CT) * ((a[0] + a[1]) + a[2])
        pat = sum((a[k] >= lim).astype(np.int64) << k for k in range(3))
        near = np.any(np.abs(a - lim) <= F32(BAND) * lim, axis=0)
    return pat, ok & ~near


def test_float_cutoff_rule_decides_as_the_reference():
    rng = np.random.default_rng(11)
    n = 400_000
    decided = 0
    for trial in range(6):
        SI = 10.0 ** rng.uniform(-45, 8, size=(3, n))
        SI[rng.random((3, n)) < 0.05] = 0.0
        if trial % 2:  # one indicator near another: ratios near the cut-off
            SI[1] = SI[0] * 10.0 ** rng.uniform(-2, 2, size=n)
            SI[2] = SI[0] * (1.0 + rng.normal(scale=1e-3, size=n))
        tau = 10.0 ** rng.uniform(-45, 10, size=n)
        tau[rng.random(n) < 0.02] = 0.0
        want, finite = reference_pattern(SI, tau)
        got, ok = float_rule(SI, tau)
        assert not np.any(ok & ~finite)  # in the rule's range the reference's weights are finite
        assert np.array_equal(got[ok], want[ok])
        decided += int(ok.sum())
    assert decided > 0.9 * 6 * n * 0.5  # the rule decides most cases itself
