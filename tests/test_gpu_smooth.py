"""The reference's smooth accuracy cases with exact solutions, on periodic domains: the 2D
entropy wave and isentropic vortex (FV::System2D), the 1D entropy wave (FV::System1D and
FVHermite::System1D).  The L1 density error (printResult, FV_System2D.cpp:653-666) must fall at
the scheme's order as the grid is refined, on the plain FP64 path and on the mixed path."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def l1_2d(h, q0, exact, t, prec=0, **kw):
    cfg = h.config(dims=2, nx=q0.shape[2], ny=q0.shape[1], bc=1, precision=prec, **kw)
    with h.Solver(cfg) as s:
        s.set_state(q0)
        s.step(1 << 20, t)
        tt, _, _ = s.time()
        assert tt == pytest.approx(t, rel=1e-13)
        return np.abs(s.get_state()[0] - exact[0]).mean()


def orders(errs):
    return [np.log2(a / b) for a, b in zip(errs[:-1], errs[1:])]


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "mixed"])
def test_entropy_wave_2d_convergence(hteno_lib, cuda, prec):
    """FV::System2D entropy wave on [-1,1]^2 (main.cpp's case: CFL 0.6), TENO5 + Rusanov."""
    from hteno import ic

    t = 0.25
    errs = []
    for n in (16, 32, 64):
        kw = dict(xl=-1.0, xr=1.0, yb=-1.0, yt=1.0, cfl=0.6, flux=0)
        errs.append(l1_2d(hteno_lib, ic.entropy_wave_2d(n, n), ic.entropy_wave_2d(n, n, t=t), t, prec, **kw))
    o = orders(errs)
    assert errs[-1] < 1e-4 and min(o) > 2.7, (errs, o)


def test_isentropic_vortex_2d_convergence(hteno_lib, cuda):
    """The vortex on [-5,5]^2 is periodic only to ~1e-5 (its velocity tail at the edges), which
    floors the error near 1e-5; above the floor the error falls at better than second order."""
    from hteno import ic

    t = 1.0
    errs = []
    for n in (32, 64):
        kw = dict(xl=-5.0, xr=5.0, yb=-5.0, yt=5.0, cfl=0.4, flux=0)
        errs.append(l1_2d(hteno_lib, ic.isentropic_vortex_2d(n, n), ic.isentropic_vortex_2d(n, n, t=t), t, **kw))
    o = orders(errs)
    assert errs[-1] < 6e-5 and o[0] > 2.0, (errs, o)


def run_1d(h, q0, t, v0=None, **kw):
    cfg = h.config(dims=1, nx=q0.shape[1], xl=-1.0, xr=1.0, bc=1, **kw)
    with h.Solver(cfg) as s:
        s.set_state(q0)
        if v0 is not None:
            s.set_moments(v0)
        s.step(1 << 20, t)
        return s.get_state()


def test_entropy_wave_1d_fv_convergence(hteno_lib, cuda):
    from hteno import ic

    t = 0.5
    errs = []
    for n in (20, 40, 80, 160):
        got = run_1d(hteno_lib, ic.entropy_wave_1d(n), t, cfl=0.4, recon=0, flux=0)
        errs.append(np.abs(got[0] - ic.entropy_wave_1d(n, t=t)[0]).mean())
    o = orders(errs)
    assert errs[-1] < 1e-5 and o[-1] > 2.7, (errs, o)


def test_entropy_wave_1d_hermite_convergence(hteno_lib, cuda):
    """FVHermite::System1D entropy wave (main.cpp's case: [-1,1], CFL 1.0, t = 0.5) with the
    moments as cell averages of d/dx; dt scales as dx^(5/3), so the error falls faster than RK3."""
    from hteno import ic

    t = 0.5
    errs = []
    for n in (20, 40, 80):
        got = run_1d(hteno_lib, ic.entropy_wave_1d(n), t, v0=ic.entropy_wave_1d(n, derivative=True),
                     scheme=1, cfl=1.0)
        errs.append(np.abs(got[0] - ic.entropy_wave_1d(n, t=t)[0]).mean())
    o = orders(errs)
    assert errs[-1] < 1e-5 and o[-1] > 3.5, (errs, o)
