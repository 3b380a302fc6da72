"""CPU checks of the oracle: golden vectors produced by the reference's own sources, live
comparison with the reference build where it exists, and mathematical invariants of the schemes
(the reference ships no tests; these pins are the project's)."""
from __future__ import annotations

import platform
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
X86 = platform.machine() in ("x86_64", "AMD64")


def same(a, b):
    """Bitwise on x86 (the fixtures were generated there with contraction off); on other hosts
    libm's pow may round differently in the last bit, so allow a few ulp."""
    if X86:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-300)


@pytest.fixture(scope="module")
def pw():
    return dict(np.load(GOLD / "pointwise.npz"))


@pytest.fixture(scope="module")
def sv():
    return dict(np.load(GOLD / "solvers.npz"))


def test_lagrange_golden(oracle, pw):
    for kind, name in enumerate(("teno5", "teno5i", "linear5")):
        same(oracle.lagrange(kind, pw["lag_u"]), pw[f"lag_{name}"])


def test_alternative_reconstructions_golden(oracle):
    """weno5JS, weno5Z, weno5N, teno5N, teno5a: the oracle reproduces the reference's outputs."""
    g = dict(np.load(GOLD / "alternatives.npz"))
    for kind in (3, 4, 5, 6, 7):
        same(oracle.lagrange(kind, g["alt_u"]), g[f"alt_{kind}"])


def test_gl3_golden(oracle, pw):
    same(oracle.gl3(pw["gl3_u"]), pw["gl3_out"])


def test_hermite_golden(oracle, pw):
    dx = float(pw["her_dx"])
    for kind, name in enumerate(("hteno", "htenoi", "hlinear")):
        same(oracle.hermite(kind, dx, pw["her_u"], pw["her_d"]), pw[f"her_{name}"])
    same(oracle.hlimiter(dx, pw["lim_u"], pw["lim_d"]), pw["lim_out"])


def test_fluxes_golden(oracle, pw):
    for d in (1, 2):
        same(oracle.hllc2d(1.4, d, pw["flux_ql"], pw["flux_qr"]), pw[f"hllc2d_{d}"])
        R, L = oracle.roe2d(1.4, d, pw["flux_qa"], pw["flux_qb"])
        same(R, pw[f"roeR_{d}"])
        same(L, pw[f"roeL_{d}"])
        same(oracle.rusanov2d(1.4, d, pw["flux_qa"], pw["flux_qb"], pw["flux_ql"], pw["flux_qr"]),
             pw[f"rusanov2d_{d}"])
        same(oracle.drusanov2d(1.4, d, pw["flux_qa"], pw["flux_qb"], pw["flux_ql"], pw["flux_qr"],
                               pw["flux_dql"], pw["flux_dqr"]), pw[f"drusanov2d_{d}"])
    same(oracle.hllc1d(1.4, pw["hllc1d_ql"], pw["hllc1d_qr"]), pw["hllc1d_out"])


def test_ssprk_golden(oracle, pw):
    for st in (1, 2, 3):
        same(oracle.ssprk3(pw["rk_q0"], pw["rk_qn"], pw["rk_rhs"], 0.013, st), pw[f"rk_stage{st}"])


def test_fv2d_golden(oracle, sv):
    q, t, n = oracle.fv2d_run(sv["fv2d_q0"], int(sv["fv2d_steps"]))
    assert n == int(sv["fv2d_steps"])
    same(q, sv["fv2d_q"])
    same(np.array(t), sv["fv2d_t"])


@pytest.mark.parametrize("name,bc", [("taylor", 2), ("dmach", 3)])
def test_fv2d_boundaries_golden(oracle, name, bc):
    """TaylorInstBc and doubleMachBc (reflective walls, fixed and time-dependent ghost states):
    the oracle against the reference with rhs() switched to those routines, and the project's
    initial data against the reference's."""
    from hteno import ic

    g = np.load(GOLD / "boundaries.npz")
    q0 = g[f"{name}_q0"]
    xl, xr, yb, yt = g[f"{name}_box"]
    fn = ic.rayleigh_taylor if name == "taylor" else ic.double_mach
    np.testing.assert_allclose(fn(q0.shape[2], q0.shape[1]), q0, rtol=1e-15, atol=1e-15)
    q, t, n = oracle.fv2d_run(q0, int(g[f"{name}_steps"]), xl=xl, xr=xr, yb=yb, yt=yt, bc=bc)
    assert n == int(g[f"{name}_steps"])
    same(q, g[f"{name}_q"])
    same(np.array(t), g[f"{name}_t"])


def test_fv1d_golden(oracle, sv):
    q, t, n = oracle.fv1d_run(sv["fv1d_q0"], 100000, t_final=0.2, cfl=0.5, recon=1, flux=0)
    assert n == int(sv["fv1d_steps"])
    same(q, sv["fv1d_q"])
    assert t == pytest.approx(0.2, abs=0)


def test_hermite2d_golden(oracle, sv):
    q, v, w, t, n = oracle.hermite2d_run(sv["h2d_q0"], sv["h2d_v0"], sv["h2d_w0"], int(sv["h2d_steps"]))
    same(q, sv["h2d_q"])
    same(v, sv["h2d_v"])
    same(w, sv["h2d_w"])


def test_hermite1d_golden(oracle, sv):
    q, v, t, n = oracle.hermite1d_run(sv["h1d_q0"], sv["h1d_v0"], int(sv["h1d_steps"]))
    same(q, sv["h1d_q"])
    same(v, sv["h1d_v"])


# ---- invariants ----------------------------------------------------------------------------

def test_linear_reconstruction_exact_on_quartics(oracle):
    """Averages of a degree-4 polynomial are reconstructed exactly at x_{i+1/2} by the linear
    scheme, and TENO5 equals it on such smooth data."""
    rng = np.random.default_rng(0)
    cf = rng.normal(size=(64, 5))
    x = np.arange(6) - 2.0  # cells i-2..i+3, face at x = 0.5 (cell i = [-0.5, 0.5])

    def avg(c, a, b):  # exact cell average of sum c_k x^k over [a, b]
        return sum(c[k] * (b ** (k + 1) - a ** (k + 1)) / (k + 1) for k in range(5)) / (b - a)

    u = np.array([[avg(c, xi - 0.5, xi + 0.5) for xi in x] for c in cf])
    exact = np.array([sum(c[k] * 0.5 ** k for k in range(5)) for c in cf])
    lin = oracle.lagrange(2, u)
    np.testing.assert_allclose(lin[:, 0], exact, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(lin[:, 1], exact, rtol=1e-10, atol=1e-10)
    # on finely resolved smooth data every sub-stencil passes the cut-off: TENO5 == linear
    h = 0.02
    us = np.sin(0.3 + h * (np.arange(6) - 2.0))[None, :] + np.zeros((4, 1))
    us = us * np.array([[1.0], [10.0], [1e-3], [-5.0]])
    np.testing.assert_allclose(oracle.lagrange(0, us), oracle.lagrange(2, us), rtol=1e-13, atol=1e-15)


def test_teno_mirror_identity(oracle):
    rng = np.random.default_rng(1)
    u = rng.normal(size=(500, 6))
    a = oracle.lagrange(0, u)
    b = oracle.lagrange(0, u[:, ::-1].copy())
    np.testing.assert_allclose(a[:, 1], b[:, 0], rtol=1e-12, atol=1e-12)


def test_teno_cuts_discontinuous_substencil(oracle):
    """Across a step the cut-off drops the stencils that straddle it: the left-biased value at a
    face two cells before the jump equals the plateau value."""
    u = np.array([[1.0, 1.0, 1.0, 1.0, 5.0, 5.0]])
    np.testing.assert_allclose(oracle.lagrange(0, u)[0, 0], 1.0, rtol=0, atol=1e-14)


def test_flux_consistency(oracle):
    rng = np.random.default_rng(2)
    rho, u, v, p = rng.uniform(0.2, 1.5, 64), rng.uniform(-1, 1, 64), rng.uniform(-1, 1, 64), rng.uniform(0.1, 1.5, 64)
    q = np.ascontiguousarray(np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)]).T)
    f1 = np.stack([rho * u, rho * u * u + p, rho * u * v, u * (q[:, 3] + p)]).T
    np.testing.assert_allclose(oracle.hllc2d(1.4, 1, q, q), f1, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.rusanov2d(1.4, 1, q, q, q, q), f1, rtol=1e-12, atol=1e-12)


def test_ssprk3_third_order(oracle):
    """SSP-RK3 on du/dt = lam*u is exact through third order: one step gives
    1 + z + z^2/2 + z^3/6 with z = lam*dt."""
    lam, dt = -0.7, 0.1
    q0 = np.ones(1)
    u1 = oracle.ssprk3(q0, q0, lam * q0, dt, 1)
    u2 = oracle.ssprk3(q0, u1, lam * u1, dt, 2)
    u3 = oracle.ssprk3(q0, u2, lam * u2, dt, 3)
    z = lam * dt
    assert u3[0] == pytest.approx(1 + z + z * z / 2 + z ** 3 / 6, rel=1e-15)


def test_fv2d_conserves_with_periodic_bc(oracle):
    from hteno import ic

    q = ic.four_quadrant(16, 16, 9)
    out, t, n = oracle.fv2d_run(q, 3, bc=1)
    np.testing.assert_allclose(out.sum(axis=(1, 2)), q.sum(axis=(1, 2)), rtol=1e-12)


def test_fv2d_transpose_symmetry(oracle):
    """Swapping x and y (and the two momenta) commutes with the 2D scheme."""
    from hteno import ic

    q = ic.four_quadrant(12, 12, 5)
    qt = np.ascontiguousarray(q[[0, 2, 1, 3]].transpose(0, 2, 1))
    a, _, _ = oracle.fv2d_run(q, 2)
    b, _, _ = oracle.fv2d_run(qt, 2)
    np.testing.assert_allclose(a, b[[0, 2, 1, 3]].transpose(0, 2, 1), rtol=1e-12, atol=1e-12)


def test_oracle_matches_reference_live(oracle):
    """Fresh random inputs through the reference build, where it was built here."""
    import ctypes

    ref = oracle.REF_LIB
    if not ref.exists():
        pytest.skip("reference not built on this host")
    R = ctypes.CDLL(str(ref))
    rng = np.random.default_rng(123)
    u = np.ascontiguousarray(rng.normal(size=(2000, 6)) * 10.0 ** rng.uniform(-3, 3, (2000, 1)))
    out = np.empty((2000, 2))
    R.ref_teno5(u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_long(2000))
    same(oracle.lagrange(0, u), out)


def test_fv2d_seeded_quadrants_can_go_nonphysical(oracle):
    """The reference's own arithmetic leaves the physical states on some seeded four-quadrant
    data: TENO5 + HLLC at CFL 0.4 without a positivity limiter (the reference's checks are
    commented out, FV_System2D.cpp:236-250).  Instance 139 of the 256-grid batch configuration
    (374 x 485, seed 1139) has a negative density after one step, so a health flag on such an
    instance reports the scheme, not the precision of the path that flags it."""
    from hteno import ic

    out, t, n = oracle.fv2d_run(ic.four_quadrant(374, 485, 1139), 1)
    assert n == 1 and out[0].min() < 0.0
