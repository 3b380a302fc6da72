"""Generate the golden fixtures in tests/golden/ from the reference solver itself.

The reference's own sources are compiled unmodified against the project's Eigen-subset header
(oracle/Makefile target `ref` -> oracle/_ref/libhteno_ref.so); this script feeds seeded inputs
through that library and stores inputs and outputs as compressed .npz files.  It needs the
reference tree (it runs where the reference is mounted) and is committed together with its
outputs so the fixtures can be regenerated:

    make -C oracle ref ref_bc && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "hermite-teno_gb300"))
from hteno import ic  # noqa: E402

REF = ctypes.CDLL(str(REPO / "oracle" / "_ref" / "libhteno_ref.so"))
_D = ctypes.POINTER(ctypes.c_double)
GAMMA = 1.4


def p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def c(x):
    return ctypes.c_double(float(x))


def states(rng, n):
    """Random physical conserved states [n][4] (rho, u, v, p as in the four-quadrant data)."""
    rho = rng.uniform(0.1, 1.5, n)
    u = rng.uniform(-1, 1, n)
    v = rng.uniform(-1, 1, n)
    pr = rng.uniform(0.03, 1.5, n)
    return np.ascontiguousarray(ic.conservative2(rho, u, v, pr, GAMMA).T)


def stencils(rng, n, width):
    """Mixture of smooth, step and random stencils (with scale spread), so that every TENO
    cut-off pattern occurs."""
    x = np.arange(width)
    out = np.empty((n, width))
    kind = rng.integers(0, 4, n)
    for k in range(n):
        s = 10.0 ** rng.uniform(-3, 2)
        if kind[k] == 0:    # smooth polynomial
            cf = rng.normal(size=4)
            out[k] = s * (cf[0] + cf[1] * x + cf[2] * x ** 2 / 10 + cf[3] * x ** 3 / 100)
        elif kind[k] == 1:  # step at a random position
            j = rng.integers(1, width)
            out[k] = s * np.where(x < j, rng.normal(), rng.normal())
        elif kind[k] == 2:  # kink
            j = rng.integers(1, width - 1)
            out[k] = s * np.abs(x - j - rng.uniform())
        else:               # noise
            out[k] = s * rng.normal(size=width)
    return np.ascontiguousarray(out)


def pointwise(rng):
    n = 256
    g = {}
    u6 = stencils(rng, n, 6)
    g["lag_u"] = u6
    for name, fn in (("teno5", REF.ref_teno5), ("teno5i", REF.ref_teno5i), ("linear5", REF.ref_linear5)):
        out = np.empty((n, 2))
        fn(p(u6), p(out), ctypes.c_long(n))
        g[f"lag_{name}"] = out
    u5 = stencils(rng, n, 5)
    out = np.empty((n, 3))
    REF.ref_gl3(p(u5), p(out), ctypes.c_long(n))
    g["gl3_u"], g["gl3_out"] = u5, out
    dx = 0.01
    u4 = stencils(rng, n, 4)
    d4 = np.ascontiguousarray(stencils(rng, n, 4) / dx * 0.1)
    g["her_dx"], g["her_u"], g["her_d"] = np.array(dx), u4, d4
    for kind, name in enumerate(("hteno", "htenoi", "hlinear")):
        out = np.empty((n, 4))
        REF.ref_hermite_recon(kind, c(dx), p(u4), p(d4), p(out), ctypes.c_long(n))
        g[f"her_{name}"] = out
    u3 = np.ascontiguousarray(u4[:, :3])
    d3 = np.ascontiguousarray(d4[:, :3])
    out = np.empty(n)
    REF.ref_hermite_limiter(c(dx), p(u3), p(d3), p(out), ctypes.c_long(n))
    g["lim_u"], g["lim_d"], g["lim_out"] = u3, d3, out
    ql, qr = states(rng, n), states(rng, n)
    qa, qb = states(rng, n), states(rng, n)
    dql, dqr = rng.normal(size=(n, 4)), rng.normal(size=(n, 4))
    g.update(flux_ql=ql, flux_qr=qr, flux_qa=qa, flux_qb=qb, flux_dql=dql, flux_dqr=dqr)
    for d in (1, 2):
        out = np.empty((n, 4))
        REF.ref_hllc2d(c(GAMMA), d, p(ql), p(qr), p(out), ctypes.c_long(n))
        g[f"hllc2d_{d}"] = out
        R, L = np.empty((n, 16)), np.empty((n, 16))
        REF.ref_roe2d(c(GAMMA), d, p(qa), p(qb), p(R), p(L), ctypes.c_long(n))
        g[f"roeR_{d}"], g[f"roeL_{d}"] = R, L
        out = np.empty((n, 4))
        REF.ref_rusanov2d(c(GAMMA), d, p(ql), p(qr), p(L), p(R), p(out), ctypes.c_long(n))
        g[f"rusanov2d_{d}"] = out
        out = np.empty((n, 4))
        REF.ref_drusanov2d(c(GAMMA), d, p(ql), p(qr), p(dql), p(dqr), p(L), p(R), p(out), ctypes.c_long(n))
        g[f"drusanov2d_{d}"] = out
    q1l = np.ascontiguousarray(ql[:, [0, 1, 3]])
    q1r = np.ascontiguousarray(qr[:, [0, 1, 3]])
    out = np.empty((n, 3))
    REF.ref_hllc1d(c(GAMMA), p(q1l), p(q1r), p(out), ctypes.c_long(n))
    g["hllc1d_ql"], g["hllc1d_qr"], g["hllc1d_out"] = q1l, q1r, out
    q0, qn, rhs = (rng.normal(size=n) for _ in range(3))
    g["rk_q0"], g["rk_qn"], g["rk_rhs"] = q0, qn, rhs
    for st in (1, 2, 3):
        out = np.empty(n)
        REF.ref_ssprk3(p(q0), p(qn), p(rhs), c(0.013), st, p(out), ctypes.c_long(n))
        g[f"rk_stage{st}"] = out
    np.savez_compressed(HERE / "pointwise.npz", **g)


def solvers():
    g = {}
    # FV::System2D as shipped (TENO5, characteristic Rusanov, zero-gradient), four quadrants
    nx, ny, steps = 24, 20, 10
    q = ic.four_quadrant(nx, ny, 3, GAMMA)
    out = np.empty_like(q)
    t = ctypes.c_double()
    REF.ref_fv2d_run.restype = ctypes.c_int
    n = REF.ref_fv2d_run(nx, ny, c(0), c(1), c(0), c(1), c(0.4), c(GAMMA), c(1e30), steps, p(q), p(out), ctypes.byref(t))
    g.update(fv2d_q0=q, fv2d_q=out, fv2d_t=np.array(t.value), fv2d_steps=np.array(n))
    # FV::System1D as shipped (teno5i, Rusanov) on Sod's problem to t = 0.2
    nx = 100
    x = (np.arange(nx) + 0.5) / nx
    q = np.empty(3 * nx)
    REF.ref_sod_ic(c(GAMMA), p(np.ascontiguousarray(x)), p(q), ctypes.c_long(nx))
    q = np.ascontiguousarray(q.reshape(nx, 3).T)
    out = np.empty_like(q)
    REF.ref_fv1d_run.restype = ctypes.c_int
    n = REF.ref_fv1d_run(nx, c(0), c(1), c(0.5), c(GAMMA), c(0.2), 100000, p(q), p(out), ctypes.byref(t))
    g.update(fv1d_q0=q, fv1d_q=out, fv1d_t=np.array(t.value), fv1d_steps=np.array(n))
    # FVHermite::System2D (HTENO, zero-gradient): four quadrants with seeded moments
    nx, ny, steps = 16, 12, 3
    rng = np.random.default_rng(11)
    q = ic.four_quadrant(nx, ny, 4, GAMMA)
    v = np.ascontiguousarray(rng.normal(size=q.shape) * 0.5)
    w = np.ascontiguousarray(rng.normal(size=q.shape) * 0.5)
    qo, vo, wo = (np.empty_like(q) for _ in range(3))
    REF.ref_hermite2d_run.restype = ctypes.c_int
    n = REF.ref_hermite2d_run(nx, ny, c(0), c(1), c(0), c(1), c(0.4), c(GAMMA), c(1e30), steps,
                              p(q), p(v), p(w), p(qo), p(vo), p(wo), ctypes.byref(t))
    g.update(h2d_q0=q, h2d_v0=v, h2d_w0=w, h2d_q=qo, h2d_v=vo, h2d_w=wo, h2d_t=np.array(t.value),
             h2d_steps=np.array(n))
    # FVHermite::System1D (periodic, LMPE routing)
    nx, steps = 60, 20
    x = (np.arange(nx) + 0.5) / nx
    q = np.ascontiguousarray(np.stack([1 + 0.2 * np.sin(2 * np.pi * x) + (x > 0.5) * 0.5,
                                       0.3 * np.ones(nx), 2.5 * np.ones(nx)]))
    v = np.ascontiguousarray(np.gradient(q, 1.0 / nx, axis=1))
    qo, vo = np.empty_like(q), np.empty_like(q)
    REF.ref_hermite1d_run.restype = ctypes.c_int
    n = REF.ref_hermite1d_run(nx, c(0), c(1), c(0.4), c(GAMMA), c(1e30), steps, p(q), p(v), p(qo),
                              p(vo), ctypes.byref(t))
    g.update(h1d_q0=q, h1d_v0=v, h1d_q=qo, h1d_v=vo, h1d_t=np.array(t.value), h1d_steps=np.array(n))
    np.savez_compressed(HERE / "solvers.npz", **g)


def boundaries():
    """FV::System2D as shipped (TENO5, characteristic Rusanov) with rhs() calling TaylorInstBc()
    resp. doubleMachBc() (oracle/Makefile target `ref_bc`), from the reference's own initial
    data at the cell centres."""
    g = {}
    t = ctypes.c_double()
    for name, lib, icfn, (nx, ny, xl, xr, yb, yt), steps in (
            ("taylor", "libhteno_ref_taylor.so", "ref_taylor_ic", (16, 40, 0.0, 0.25, 0.0, 1.0), 20),
            ("dmach", "libhteno_ref_dmach.so", "ref_double_mach_ic", (64, 16, 0.0, 4.0, 0.0, 1.0), 20)):
        R = ctypes.CDLL(str(REPO / "oracle" / "_ref" / lib))
        X, Y = ic.cell_centres(nx, ny, xl, xr, yb, yt)
        x, y = np.ascontiguousarray(X.ravel()), np.ascontiguousarray(Y.ravel())
        q = np.empty(4 * x.size)
        getattr(R, icfn)(c(GAMMA), p(x), p(y), p(q), ctypes.c_long(x.size))
        q = np.ascontiguousarray(q.reshape(ny, nx, 4).transpose(2, 0, 1))
        out = np.empty_like(q)
        R.ref_fv2d_run.restype = ctypes.c_int
        n = R.ref_fv2d_run(nx, ny, c(xl), c(xr), c(yb), c(yt), c(0.4), c(GAMMA), c(1e30), steps,
                           p(q), p(out), ctypes.byref(t))
        g.update({f"{name}_q0": q, f"{name}_q": out, f"{name}_t": np.array(t.value),
                  f"{name}_steps": np.array(n), f"{name}_box": np.array([xl, xr, yb, yt])})
    np.savez_compressed(HERE / "boundaries.npz", **g)


def alternatives(rng):
    """weno5JS, weno5Z, weno5N, teno5N, teno5a (Schemes_Lagrange.cpp:358-594, 1265-1294) on the
    same kinds of stencils as the pointwise fixtures."""
    n = 256
    u6 = stencils(rng, n, 6)
    g = {"alt_u": u6}
    REF.ref_lagrange_alt.argtypes = [ctypes.c_int, _D, _D, ctypes.c_long]
    for kind in (3, 4, 5, 6, 7):
        out = np.empty((n, 2))
        REF.ref_lagrange_alt(kind, p(u6), p(out), n)
        g[f"alt_{kind}"] = out
    np.savez_compressed(HERE / "alternatives.npz", **g)


if __name__ == "__main__":
    pointwise(np.random.default_rng(20261203))
    solvers()
    alternatives(np.random.default_rng(20261204))
    boundaries()
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
