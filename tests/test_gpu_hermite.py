"""GPU parity of the Hermite solvers (FVHermite::System2D, FVHermite::System1D) against the
oracle and the reference's golden runs.  The plain FP64 path reproduces the oracle's rounding
(tolerance 1e-12 relative L-inf, bitwise expected); the mixed path is checked by its error."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
TOL = 1e-12


def rel_linf(a, b):
    ax = tuple(range(1, a.ndim))
    return (np.abs(a - b).max(axis=ax) / np.maximum(np.abs(b).max(axis=ax), 1e-300)).max()


def run2(h, q, v, w, nsteps, **kw):
    cfg = h.config(dims=2, scheme=h.SCHEME_HERMITE, nx=q.shape[2], ny=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.set_moments(v, w)
        s.step(nsteps)
        t, n, _ = s.time()
        vo, wo = s.get_moments()
        return s.get_state(), vo, wo, t, n


def run1(h, q, v, nsteps, **kw):
    cfg = h.config(dims=1, scheme=h.SCHEME_HERMITE, nx=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.set_moments(v)
        s.step(nsteps)
        t, n, _ = s.time()
        return s.get_state(), s.get_moments(), t, n


def test_hermite2d_matches_reference_golden(hteno_lib, cuda):
    g = np.load(GOLD / "solvers.npz")
    q, v, w, t, n = run2(hteno_lib, g["h2d_q0"], g["h2d_v0"], g["h2d_w0"], int(g["h2d_steps"]))
    assert n == int(g["h2d_steps"])
    for a, b in ((q, g["h2d_q"]), (v, g["h2d_v"]), (w, g["h2d_w"])):
        assert rel_linf(a, b) <= TOL


def test_hermite2d_matches_oracle_bitwise(hteno_lib, cuda, oracle):
    from hteno import ic

    q = ic.four_quadrant(30, 22, 8)
    rng = np.random.default_rng(3)
    v = np.ascontiguousarray(rng.normal(size=q.shape) * 0.3)
    w = np.ascontiguousarray(rng.normal(size=q.shape) * 0.3)
    qo, vo, wo, to, no = oracle.hermite2d_run(q, v, w, 6)
    qg, vg, wg, tg, ng = run2(hteno_lib, q, v, w, 6)
    assert ng == no == 6 and tg == to
    for a, b in ((qg, qo), (vg, vo), (wg, wo)):
        assert rel_linf(a, b) <= TOL
        np.testing.assert_array_equal(a, b)


def test_hermite2d_full_size_matches_oracle(hteno_lib, cuda, oracle):
    """The Hermite benchmark configuration at its stated size: 2048^2, 32 seeded Gaussian density
    blobs on rho = p = 1 with a Mach-2 shock entering from x = 0, moments by face differences,
    Rusanov, plain FP64, 3 steps; against the CPU oracle on the host cores: <= 1e-12 relative
    L-inf per field, and bit for bit."""
    from hteno import ic

    n = 2048
    f = ic.blobs_shock_fn(5)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    q = np.ascontiguousarray(f(X, Y))
    v, w = ic.face_difference_moments(f, n, n, 0.0, 1.0, 0.0, 1.0)
    qo, vo, wo, to, no = oracle.hermite2d_run(q, v, w, 3)
    qg, vg, wg, tg, ng = run2(hteno_lib, q, v, w, 3, flux=hteno_lib.FLUX_RUSANOV)
    assert ng == no == 3 and tg == to
    for a, b in ((qg, qo), (vg, vo), (wg, wo)):
        assert rel_linf(a, b) <= TOL
        np.testing.assert_array_equal(a, b)


def test_hermite2d_limiter_chunks_bitwise(hteno_lib, cuda, oracle):
    """Lines longer than the limiter's shared-memory chunk (64 cells) and line counts that are not
    multiples of its 32-line blocks: the chunked Gauss-Seidel sweep reproduces the oracle's."""
    from hteno import ic

    q = ic.gaussian_blobs_shock(150, 97, 4)
    rng = np.random.default_rng(11)
    v = np.ascontiguousarray(rng.normal(size=q.shape) * 0.2)
    w = np.ascontiguousarray(rng.normal(size=q.shape) * 0.2)
    qo, vo, wo, to, no = oracle.hermite2d_run(q, v, w, 3)
    qg, vg, wg, tg, ng = run2(hteno_lib, q, v, w, 3)
    assert ng == no and tg == to
    for a, b in ((qg, qo), (vg, vo), (wg, wo)):
        np.testing.assert_array_equal(a, b)
    qm, _, _, _, _ = run2(hteno_lib, q, v, w, 3, precision=1)
    assert np.abs(qm[0] - qo[0]).mean() <= 1e-4


def test_hermite2d_mixed_precision_error(hteno_lib, cuda, oracle):
    from hteno import ic

    q = ic.gaussian_blobs_shock(48, 48, 2)
    v = np.zeros_like(q)
    w = np.zeros_like(q)
    qo, _, _, _, _ = oracle.hermite2d_run(q, v, w, 8)
    qg, _, _, _, _ = run2(hteno_lib, q, v, w, 8, precision=1)
    l1 = np.abs(qg[0] - qo[0]).mean()
    assert l1 <= 1e-4, l1


def test_hermite1d_matches_reference_golden(hteno_lib, cuda):
    g = np.load(GOLD / "solvers.npz")
    q, v, t, n = run1(hteno_lib, g["h1d_q0"], g["h1d_v0"], int(g["h1d_steps"]))
    assert n == int(g["h1d_steps"])
    assert rel_linf(q, g["h1d_q"]) <= TOL
    assert rel_linf(v, g["h1d_v"]) <= TOL


def test_hermite1d_matches_oracle_bitwise(hteno_lib, cuda, oracle):
    nx = 200
    x = (np.arange(nx) + 0.5) / nx
    q = np.ascontiguousarray(np.stack([1 + 0.2 * np.sin(2 * np.pi * x) + (x > 0.3) * 0.4 - (x > 0.7) * 0.3,
                                       0.4 * np.ones(nx), 2.5 + 0.5 * (x > 0.5)]))
    v = np.ascontiguousarray(np.gradient(q, 1.0 / nx, axis=1))
    qo, vo, to, no = oracle.hermite1d_run(q, v, 40)
    qg, vg, tg, ng = run1(hteno_lib, q, v, 40)
    assert ng == no == 40 and tg == to
    np.testing.assert_array_equal(qg, qo)
    np.testing.assert_array_equal(vg, vo)


def test_side_stream_same_bits(hteno_lib, cuda):
    """The y-direction kernels beside the x-direction ones on a second stream (the default) give
    the bits of the one-stream order (HTENO_SIDE_STREAM=0): FV 2D FP64, Hermite 2D FP64 and mixed."""
    import os

    from hteno import ic

    h = hteno_lib
    n = 96
    f = ic.blobs_shock_fn(5)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    qh = np.ascontiguousarray(f(X, Y))
    v, w = ic.face_difference_moments(f, n, n, 0.0, 1.0, 0.0, 1.0)
    qf = ic.four_quadrant(n, n, 13)

    def run(kw, q, mom):
        with h.Solver(h.config(dims=2, nx=n, ny=n, **kw)) as s:
            s.set_state(q)
            if mom:
                s.set_moments(*mom)
            s.step(6)
            out = [s.get_state()]
            if mom:
                out += list(s.get_moments())
            return out

    cases = [(dict(flux=1), qf, None), (dict(scheme=1, flux=0), qh, (v, w)),
             (dict(scheme=1, flux=0, precision=1), qh, (v, w))]
    for kw, q, mom in cases:
        two = run(kw, q, mom)
        os.environ["HTENO_SIDE_STREAM"] = "0"
        try:
            one = run(kw, q, mom)
        finally:
            os.environ.pop("HTENO_SIDE_STREAM", None)
        for a, b in zip(two, one):
            np.testing.assert_array_equal(a, b)
