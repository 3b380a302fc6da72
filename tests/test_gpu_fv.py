"""GPU parity of the FV solvers (FV::System2D, FV::System1D) against the oracle and the reference's
golden runs, plus size-independent properties at full benchmark size.  Called through the C-ABI.

Tolerance (FP64 plain path): relative L-infinity error <= 1e-12 per conserved variable, measured
against max |q_v| of the reference state.  The plain path is built to reproduce the oracle's
rounding exactly, so the tests also report whether the states are bit-identical."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
TOL = 1e-12


def rel_linf(a, b):
    """Relative L-inf error per variable (NaNs, which the reference produces too where its HLLC
    goes non-physical, must sit at the same places and are excluded from the norm)."""
    assert np.array_equal(np.isnan(a), np.isnan(b)), "NaN pattern differs"
    ax = tuple(range(1, a.ndim))
    d = np.where(np.isnan(b), 0.0, np.abs(a - b))
    return (np.nanmax(d, axis=ax) / np.nanmax(np.abs(b), axis=ax)).max()


def gpu_run2d(h, q, nsteps, t_final=1e30, **kw):
    cfg = h.config(dims=2, nx=q.shape[2], ny=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.step(nsteps, t_final)
        t, n, _ = s.time()
        return s.get_state(), t, n


CONFIGS = [
    dict(flux=0, recon=0, bc=0),  # the reference as shipped: TENO5 + characteristic Rusanov
    dict(flux=1, recon=0, bc=0),  # HLLC (the configuration of the 2D benchmark)
    dict(flux=1, recon=1, bc=1),  # teno5i, periodic
    dict(flux=0, recon=2, bc=1),  # linear, periodic (smooth data: linear is unlimited)
]


def smooth_periodic(nx, ny):
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    rho = 1 + 0.2 * np.sin(2 * np.pi * (X + Y))
    return np.ascontiguousarray(ic.conservative2(rho, 0.5 + 0 * X, -0.3 + 0 * X, 1 + 0 * X))


@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: f"flux{c['flux']}-recon{c['recon']}-bc{c['bc']}")
def test_fv2d_matches_oracle(hteno_lib, cuda, oracle, cfg):
    from hteno import ic

    q = ic.four_quadrant(40, 28, 17) if cfg["recon"] != 2 else smooth_periodic(40, 28)
    want, t_o, n_o = oracle.fv2d_run(q, 25, **cfg)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, 25, **cfg)
    assert n_g == n_o == 25
    assert t_g == t_o
    assert rel_linf(got, want) <= TOL
    np.testing.assert_array_equal(got, want)  # the plain path reproduces the oracle's rounding


def test_fv2d_bitwise_200_steps(hteno_lib, cuda, oracle):
    """The benchmark scheme (TENO5 + HLLC) for 200 steps on 256^2: the plain FP64 path reproduces
    the oracle's rounding, so the states agree bit for bit (tolerance kept at 1e-12)."""
    from hteno import ic

    q = ic.four_quadrant(256, 256, 0)
    want, t_o, n_o = oracle.fv2d_run(q, 200, flux=1)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, 200, flux=1)
    assert n_g == n_o == 200 and t_g == t_o
    assert rel_linf(got, want) <= TOL
    np.testing.assert_array_equal(got, want)


def test_fv2d_matches_reference_golden(hteno_lib, cuda):
    g = np.load(GOLD / "solvers.npz")
    got, t, n = gpu_run2d(hteno_lib, g["fv2d_q0"], int(g["fv2d_steps"]))
    assert n == int(g["fv2d_steps"])
    assert rel_linf(got, g["fv2d_q"]) <= TOL


def test_fv2d_residual_matches_oracle(hteno_lib, cuda, oracle):
    from hteno import ic

    q = ic.four_quadrant(33, 21, 2)
    for flux in (0, 1):
        want = oracle.fv2d_rhs(q, flux=flux)
        cfg = hteno_lib.config(dims=2, nx=33, ny=21, flux=flux)
        with hteno_lib.Solver(cfg) as s:
            dq = cuda.from_numpy(q).cuda()
            rhs = cuda.empty_like(dq)
            s.residual(dq, rhs)
            got = rhs.cpu().numpy()
        scale = np.abs(want).max(axis=(1, 2), keepdims=True)
        assert (np.abs(got - want) / scale).max() <= TOL


def test_fv2d_edge_sizes_and_time_clipping(hteno_lib, cuda, oracle):
    """Smallest accepted grid and non-square grids, stopping on t_final mid-run, with both fluxes.
    The reference's HLLC (sound speeds without gamma) drives the 64 x 9 case to negative pressure
    at step 10, to values beyond 1e35 by step 60 and to NaN later; the two sides stay bit-identical
    through the non-physical steps (compared over 25 steps here) and the GPU must flag them."""
    from hteno import ic

    for flux in (0, 1):
        for nx, ny in ((6, 6), (7, 13), (64, 9)):
            q = ic.four_quadrant(nx, ny, nx * 100 + ny)
            if flux == 1 and (nx, ny) == (64, 9):
                want, t_o, n_o = oracle.fv2d_run(q, 25, t_final=0.05, flux=flux)
                got, t_g, n_g = gpu_run2d(hteno_lib, q, 25, t_final=0.05, flux=flux)
                assert n_g == n_o == 25 and t_g == t_o
                np.testing.assert_array_equal(got, want)
                with hteno_lib.Solver(hteno_lib.config(dims=2, nx=nx, ny=ny, flux=flux)) as s:
                    s.set_state(q)
                    s.step(1000, 0.05)
                    assert s.status() != 0
                continue
            want, t_o, n_o = oracle.fv2d_run(q, 1000, t_final=0.05, flux=flux)
            got, t_g, n_g = gpu_run2d(hteno_lib, q, 1000, t_final=0.05, flux=flux)
            assert n_g == n_o and t_g == pytest.approx(0.05, abs=0) and t_o == pytest.approx(0.05, abs=0)
            assert rel_linf(got, want) <= TOL
            np.testing.assert_array_equal(got, want)


def blob_field(nx, ny, scale=1.0, mach=0.3, p_bg=1.0):
    """A dense, high-pressure disc in a uniform stream: most cells sit in bitwise-uniform 7 x 7
    blocks, which the plain path gives a zero residual without computing their faces."""
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    disc = (X - 0.45) ** 2 + (Y - 0.5) ** 2 < 0.12 ** 2
    u = mach * np.sqrt(1.4) + 0 * X
    return np.ascontiguousarray(ic.conservative2(scale * (1.0 + disc), u, -0.2 * u, scale * (p_bg + 2.0 * disc)))


UNIFORM_CASES = {
    "stream": dict(q=lambda: blob_field(96, 72), flux=1, bc=0),
    "stream-rusanov-periodic": dict(q=lambda: blob_field(96, 72), flux=0, bc=1),
    "tiny-density": dict(q=lambda: blob_field(96, 72, scale=1e-22), flux=1, bc=0),  # below 2^-64
    "hypersonic": dict(q=lambda: blob_field(96, 72, mach=12.0), flux=1, bc=0),  # Mach above 8
    "negative-pressure": dict(q=lambda: blob_field(48, 40, p_bg=-1.0), flux=1, bc=0, steps=2),
}


@pytest.mark.parametrize("case", list(UNIFORM_CASES))
def test_fv2d_uniform_regions_exact(hteno_lib, cuda, oracle, case):
    """The plain path skips the faces that only cells of bitwise-uniform, tame 7 x 7 blocks use;
    the result is the full computation's bits, whether or not a case qualifies (states outside
    the tame bounds, and nonphysical ones whose fluxes are NaN, take the full path)."""
    c = dict(UNIFORM_CASES[case])
    q, steps = c.pop("q")(), c.pop("steps", 30)
    want, t_o, n_o = oracle.fv2d_run(q, steps, **c)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, steps, **c)
    assert n_g == n_o and (t_g == t_o or (np.isnan(t_g) and np.isnan(t_o)))
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("name,bc", [("taylor", 2), ("dmach", 3)])
def test_fv2d_boundaries_match_reference_golden(hteno_lib, cuda, name, bc):
    """TaylorInstBc and doubleMachBc (reflective walls, fixed and time-dependent ghost states),
    against the reference with rhs() switched to those routines (scheme as shipped)."""
    g = np.load(GOLD / "boundaries.npz")
    q0 = g[f"{name}_q0"]
    xl, xr, yb, yt = g[f"{name}_box"]
    got, t, n = gpu_run2d(hteno_lib, q0, int(g[f"{name}_steps"]), xl=xl, xr=xr, yb=yb, yt=yt, bc=bc)
    assert n == int(g[f"{name}_steps"]) and t == float(g[f"{name}_t"])
    np.testing.assert_array_equal(got, g[f"{name}_q"])


BOUNDARY_CASES = {
    "rayleigh-taylor-hllc": (2, "rayleigh_taylor", (40, 150), (0.0, 0.25, 0.0, 1.0), 60, dict(flux=1)),
    "double-mach-hllc": (3, "double_mach", (160, 41), (0.0, 4.0, 0.0, 1.0), 60, dict(flux=1)),
    "double-mach-teno5i": (3, "double_mach", (97, 30), (0.0, 4.0, 0.0, 1.0), 40, dict(flux=0, recon=1)),
}


@pytest.mark.parametrize("case", list(BOUNDARY_CASES))
def test_fv2d_boundaries_match_oracle(hteno_lib, cuda, oracle, case):
    """The benchmark scheme (HLLC) and teno5i with the two boundary routines: bit for bit against
    the oracle, on grids that are not multiples of any tile; the uniform-region skipping (on by
    default) is exact with the ghost states too."""
    from hteno import ic

    bc, fn, (nx, ny), (xl, xr, yb, yt), steps, kw = BOUNDARY_CASES[case]
    q = getattr(ic, fn)(nx, ny, xl, xr, yb, yt)
    want, t_o, n_o = oracle.fv2d_run(q, steps, xl=xl, xr=xr, yb=yb, yt=yt, bc=bc, **kw)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, steps, xl=xl, xr=xr, yb=yb, yt=yt, bc=bc, **kw)
    assert n_g == n_o == steps and t_g == t_o
    np.testing.assert_array_equal(got, want)


def test_fv2d_constant_state_is_steady(hteno_lib, cuda):
    q = np.ascontiguousarray(np.broadcast_to(np.array([1.3, 0.2, -0.4, 2.7])[:, None, None], (4, 16, 20)).copy())
    got, _, _ = gpu_run2d(hteno_lib, q, 5, flux=1)
    np.testing.assert_allclose(got, q, rtol=1e-14, atol=1e-14)


def test_fv2d_nonphysical_state_reports_status(hteno_lib, cuda):
    """A negative density is recorded in the health flags; in strict mode the step returns
    HTENO_ERR_NONPHYSICAL (or NAN).  Like the reference, the kernels take sqrt(|rho|) and keep
    running; nothing faults."""
    from hteno import ic, HtenoError

    q = ic.four_quadrant(16, 16, 1)
    q[0, 5, 5] = -0.5
    cfg = hteno_lib.config(dims=2, nx=16, ny=16, flux=1)
    with hteno_lib.Solver(cfg) as s:
        s.set_state(q)
        s.step(1)
        assert s.status() & 2
        s.set_state(q)
        assert s.status() == 0
        s.set_strict(True)
        with pytest.raises(HtenoError) as e:
            s.step(1)
        assert e.value.code in (4, 5)


def periodic_box(nx, ny):
    """A dense, high-pressure square advected diagonally through periodic boundaries: contacts
    and shocks that stay physical (the random four-quadrant data do not under periodic wrap)."""
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    inside = (np.abs(X - 0.5) < 0.25) & (np.abs(Y - 0.5) < 0.25)
    return np.ascontiguousarray(ic.conservative2(1.0 + inside, 0.5 + 0 * X, -0.3 + 0 * X, 1.0 + 1.5 * inside))


def test_fv2d_full_size_matches_oracle(hteno_lib, cuda, oracle):
    """The 2D benchmark configuration exactly as specified: 1024^2 seeded four-quadrant data
    (seed 0), TENO5 + HLLC, CFL 0.4, zero-gradient, 200 steps.  The GPU FP64 state against the
    CPU oracle run on the host cores (OpenMP) inside the test: <= 1e-12 relative L-inf per
    conserved variable, and bit for bit (the plain path reproduces the oracle's rounding).  A
    second GPU run is identical (deterministic) and the density stays positive."""
    from hteno import ic

    q = ic.four_quadrant(1024, 1024, 0)
    a, t1, n1 = gpu_run2d(hteno_lib, q, 200, flux=1)
    want, t_o, n_o = oracle.fv2d_run(q, 200, flux=1)
    assert n1 == n_o == 200 and t1 == t_o
    assert rel_linf(a, want) <= TOL
    np.testing.assert_array_equal(a, want)
    b, t2, n2 = gpu_run2d(hteno_lib, q, 200, flux=1)
    assert n2 == 200 and t1 == t2
    np.testing.assert_array_equal(a, b)
    assert a[0].min() > 0


def test_fv2d_full_size_properties(hteno_lib, cuda):
    """With periodic boundaries the totals of a 1024^2 run are conserved to rounding."""
    p = periodic_box(1024, 1024)
    c, _, _ = gpu_run2d(hteno_lib, p, 50, flux=1, bc=1)
    assert np.isfinite(c).all() and c[0].min() > 0
    tot0, tot = p.sum(axis=(1, 2)), c.sum(axis=(1, 2))
    scale = np.abs(p).sum(axis=(1, 2))
    assert (np.abs(tot - tot0) <= 1e-12 * scale).all(), (tot - tot0) / scale


def test_fv2d_transpose_symmetry_gpu(hteno_lib, cuda):
    """Swapping x and y commutes with the scheme up to rounding: the x and y characteristic sums
    associate the normal and tangential momenta in opposite order (as in the reference), and a
    rounding difference can flip a TENO cut-off in a wave tail, so the bound is 1e-7, not 1e-12.
    The first step is symmetric to rounding."""
    from hteno import ic

    q = ic.four_quadrant(96, 96, 4)
    qt = np.ascontiguousarray(q[[0, 2, 1, 3]].transpose(0, 2, 1))
    a, _, _ = gpu_run2d(hteno_lib, q, 1, flux=1)
    b, _, _ = gpu_run2d(hteno_lib, qt, 1, flux=1)
    assert rel_linf(a, np.ascontiguousarray(b[[0, 2, 1, 3]].transpose(0, 2, 1))) <= 1e-14
    a, _, _ = gpu_run2d(hteno_lib, q, 20, flux=1)
    b, _, _ = gpu_run2d(hteno_lib, qt, 20, flux=1)
    assert rel_linf(a, np.ascontiguousarray(b[[0, 2, 1, 3]].transpose(0, 2, 1))) <= 1e-7


def test_fv2d_mixed_precision_error(hteno_lib, cuda, oracle):
    from hteno import ic

    q = ic.four_quadrant(64, 64, 3)
    want, _, _ = oracle.fv2d_run(q, 40, flux=1)
    got, _, _ = gpu_run2d(hteno_lib, q, 40, flux=1, precision=1)
    l1 = np.abs(got[0] - want[0]).mean()
    assert l1 <= 1e-4, l1


# ---- FV 1D --------------------------------------------------------------------------------

def gpu_run1d(h, q, nsteps, t_final=1e30, **kw):
    cfg = h.config(dims=1, nx=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.step(nsteps, t_final)
        t, n, _ = s.time()
        return s.get_state(), t, n


def test_fv1d_sod_teno5_hllc(hteno_lib, cuda, oracle):
    """The 1D benchmark case: 400 cells, Sod, TENO5 + HLLC, CFL 0.5, t = 0.2."""
    from hteno import ic

    q = ic.sod(400)
    want, t_o, n_o = oracle.fv1d_run(q, 100000, t_final=0.2, cfl=0.5, recon=0, flux=1)
    got, t_g, n_g = gpu_run1d(hteno_lib, q, 100000, t_final=0.2, cfl=0.5, recon=0, flux=1)
    assert n_g == n_o and t_g == pytest.approx(0.2, abs=0)
    assert rel_linf(got, want) <= TOL


def test_fv1d_matches_reference_golden(hteno_lib, cuda):
    g = np.load(GOLD / "solvers.npz")
    got, t, n = gpu_run1d(hteno_lib, g["fv1d_q0"], 100000, t_final=0.2, cfl=0.5, recon=1, flux=0)
    assert n == int(g["fv1d_steps"])
    assert rel_linf(got, g["fv1d_q"]) <= TOL


def test_fv1d_periodic_and_linear(hteno_lib, cuda, oracle):
    x = (np.arange(128) + 0.5) / 128
    rho = 1 + 0.2 * np.sin(2 * np.pi * x)
    q = np.ascontiguousarray(np.stack([rho, rho * 1.0, 1 / 0.4 + 0.5 * rho]))
    for recon in (0, 1, 2):
        want, _, _ = oracle.fv1d_run(q, 30, recon=recon, flux=0, bc=1, cfl=0.5)
        got, _, _ = gpu_run1d(hteno_lib, q, 30, recon=recon, flux=0, bc=1, cfl=0.5)
        assert rel_linf(got, want) <= TOL


def kxrcf_ref(q, dx, bc=0):
    """FV::System1D KXRCF flags (FV_System1D.cpp:166-192) restated in numpy."""
    n = q.shape[1]
    idx = lambda k: np.clip(k, 0, n - 1) if bc == 0 else k % n
    rho = lambda k: q[0, idx(k)]
    i = np.arange(n)
    left = q[1] < 0.0
    h1 = np.where(left, (2.0 * rho(i - 1) + 5.0 * rho(i) - rho(i + 1)) / 6.0,
                  (-rho(i - 1) + 5.0 * rho(i) + 2.0 * rho(i + 1)) / 6.0)
    h2 = np.where(left, (-rho(i - 2) + 5.0 * rho(i - 1) + 2.0 * rho(i)) / 6.0,
                  (2.0 * rho(i) + 5.0 * rho(i + 1) - rho(i + 2)) / 6.0)
    return (np.abs(h1 - h2) / ((dx / 2.0) ** 1.5 * np.abs(rho(i))) > 1.0).astype(np.uint8)


def test_fv1d_kxrcf_sensor(hteno_lib, cuda):
    """The KXRCF sensor flags the Sod tube's discontinuities and agrees with the formula."""
    from hteno import ic

    h = hteno_lib
    with h.Solver(h.config(dims=1, nx=400, flux=1, recon=0, cfl=0.5)) as s:
        s.set_state(ic.sod(400))
        s.step(1 << 20, 0.2)
        q = s.get_state()
        f = cuda.zeros(400, dtype=cuda.uint8, device="cuda")
        s.kxrcf(f)
        got = f.cpu().numpy()
    want = kxrcf_ref(q, 1.0 / 400)
    assert (got != want).sum() <= 2  # threshold ties aside
    assert 3 <= got.sum() <= 80 and got[:80].sum() == 0  # flags sit at the waves only


@pytest.mark.parametrize("recon", [3, 4, 5, 6, 7], ids=["weno5js", "weno5z", "weno5n", "teno5n", "teno5a"])
def test_fv2d_alternative_reconstructions(hteno_lib, cuda, oracle, recon):
    """The reference's other selectable schemes through the same solver: the plain path against
    the oracle (bit for bit; weno5N within 1e-12, its |.|^2.5 going through the device pow), and
    the mixed path within its bound."""
    from hteno import ic

    q = ic.four_quadrant(40, 28, 23)
    want, t_o, n_o = oracle.fv2d_run(q, 15, flux=1, recon=recon)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, 15, flux=1, recon=recon)
    assert n_g == n_o == 15
    if recon == 5:
        assert rel_linf(got, want) <= TOL
    else:
        assert t_g == t_o
        np.testing.assert_array_equal(got, want)
    mixed, _, _ = gpu_run2d(hteno_lib, q, 1000, t_final=t_o, flux=1, recon=recon, precision=1)
    assert np.abs(mixed[0] - want[0]).mean() <= 1e-4


def test_fv2d_4096_matches_oracle(hteno_lib, cuda, oracle):
    """The 4096^2 grid of the learned-routing configuration (four-quadrant data, seed 7, TENO5 +
    HLLC, plain FP64) for 3 steps against the CPU oracle on the host cores: bit for bit."""
    from hteno import ic

    q = ic.four_quadrant(4096, 4096, 7)
    want, t_o, n_o = oracle.fv2d_run(q, 3, flux=1)
    got, t_g, n_g = gpu_run2d(hteno_lib, q, 3, flux=1)
    assert n_g == n_o == 3 and t_g == t_o
    assert rel_linf(got, want) <= TOL
    np.testing.assert_array_equal(got, want)


def gpu_run2d_fused(h, q, nsteps, fused, t_final=1e30, **kw):
    cfg = h.config(dims=2, nx=q.shape[2], ny=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        if fused:
            s.set_fp64_fused(True)
        s.set_state(q)
        s.step(nsteps, t_final)
        t, n, _ = s.time()
        return s.get_state(), t, n, s.counters()["uniform_cells"], s.launches_per_step()


@pytest.mark.parametrize("case", [
    ((96, 80), 40, dict(flux=1, recon=0, bc=0)),    # TENO5 + HLLC, partial tiles
    ((64, 64), 30, dict(flux=0, recon=1, bc=1)),    # teno5i + Rusanov, periodic
    ((100, 37), 30, dict(flux=1, recon=4, bc=0)),   # WENO-Z, both edges partial
    ((40, 150), 30, dict(flux=1, recon=2, bc=1)),   # linear weights, periodic, tall
    ((12, 9), 20, dict(flux=1, recon=0, bc=1)),     # a grid smaller than one tile, periodic
], ids=["teno5-hllc", "teno5i-periodic", "wenoz", "linear-periodic", "tiny-periodic"])
def test_fp64_fused_stage_same_bits(hteno_lib, cuda, case):
    """One fused launch per stage gives the five-launch path's state bit for bit, with the same
    time, step count and uniform-cell count, in five launches per step instead of twenty."""
    from hteno import ic

    (nx, ny), steps, kw = case
    q = ic.four_quadrant(nx, ny, 11)
    a, ta, na, ua, la = gpu_run2d_fused(hteno_lib, q, steps, False, **kw)
    b, tb, nb, ub, lb = gpu_run2d_fused(hteno_lib, q, steps, True, **kw)
    np.testing.assert_array_equal(a, b)
    assert (ta, na, ua) == (tb, nb, ub) and la == 20 and lb == 5


def test_fp64_fused_matches_oracle(hteno_lib, cuda, oracle):
    """The fused stage against the CPU oracle directly (TENO5 + HLLC, 96 x 80, 40 steps)."""
    from hteno import ic

    q = ic.four_quadrant(96, 80, 3)
    got, t, n, _, _ = gpu_run2d_fused(hteno_lib, q, 40, True, flux=1, recon=0, bc=0)
    want, t_o, n_o = oracle.fv2d_run(q, 40, flux=1, recon=0, bc=0)
    assert n == n_o == 40 and t == t_o
    assert rel_linf(got, want) <= TOL
    np.testing.assert_array_equal(got, want)


def test_fp64_fused_full_size_same_bits(hteno_lib, cuda):
    """The headline configuration at its stated size (1024^2 four-quadrant, TENO5 + HLLC, 200
    steps): the fused stage equals the five-launch path bit for bit (which the full-size test
    above pins to the oracle)."""
    from hteno import ic

    q = ic.four_quadrant(1024, 1024, 0)
    a, ta, na, ua, _ = gpu_run2d_fused(hteno_lib, q, 200, False, flux=1, recon=0, bc=0)
    b, tb, nb, ub, _ = gpu_run2d_fused(hteno_lib, q, 200, True, flux=1, recon=0, bc=0)
    assert (ta, na, ua) == (tb, nb, ub)
    np.testing.assert_array_equal(a, b)


def test_fp64_fused_rejects_other_configurations(hteno_lib, cuda):
    h = hteno_lib
    for kw in (dict(bc=2), dict(bc=3), dict(precision=1)):
        with h.Solver(h.config(dims=2, nx=32, ny=32, **kw)) as s:
            with pytest.raises(h.HtenoError) as e:
                s.set_fp64_fused(True)
            assert e.value.code == 7  # HTENO_ERR_UNSUPPORTED


def test_launches_per_step_counts_the_launches(hteno_lib, cuda):
    """hteno_launches_per_step (the bench's gpu_launches per step) equals the kernels a step
    launches: those the per-kernel timing records, plus the step's begin and end kernels."""
    import ctypes

    from hteno import ic

    h = hteno_lib
    lib = h.lib()
    n = 64
    q = ic.four_quadrant(n, n, 5)
    f = ic.blobs_shock_fn(5)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    qh = np.ascontiguousarray(f(X, Y))
    v, w = ic.face_difference_moments(f, n, n, 0.0, 1.0, 0.0, 1.0)
    cases = [(dict(flux=1), q, None, False), (dict(flux=1), q, None, True),
             (dict(flux=1, precision=1), q, None, False),
             (dict(scheme=1, flux=0, precision=1), qh, (v, w), False),
             (dict(scheme=1, flux=0), qh, (v, w), False)]
    for kw, q0, mom, fused in cases:
        with h.Solver(h.config(dims=2, nx=n, ny=n, **kw)) as s:
            if fused:
                s.set_fp64_fused(True)
            s.set_state(q0)
            if mom:
                s.set_moments(*mom)
            lib.hteno_enable_kernel_timing(s.h, 1)
            s.step(3)
            kt = (h.KernelTime * 16)()
            cnt = ctypes.c_int()
            lib.hteno_kernel_timing(s.h, kt, 16, ctypes.byref(cnt))
            traced = sum(kt[k].launches for k in range(cnt.value))
            assert traced % 3 == 0 and traced // 3 + 2 == s.launches_per_step(), (kw, fused, traced)


def test_fp64_fused_uniform_skip_and_user_stream(hteno_lib, cuda):
    """The fused stage computes uniform regions in full with HTENO_UNIFORM_SKIP=0 and gives the same
    bits; on a caller's stream it gives the same bits as on its own."""
    import os

    from hteno import ic

    h = hteno_lib
    q = ic.four_quadrant(160, 96, 21)
    cfg = h.config(dims=2, nx=160, ny=96, flux=1)

    def run(stream=None):
        with h.Solver(cfg) as s:
            if stream is not None:
                s.set_stream(stream.cuda_stream)
            s.set_fp64_fused(True)
            s.set_state(q)
            s.step(30)
            return s.get_state(), s.counters()["uniform_cells"]

    base, uni = run()
    os.environ["HTENO_UNIFORM_SKIP"] = "0"
    try:
        full, uni0 = run()
    finally:
        os.environ.pop("HTENO_UNIFORM_SKIP", None)
    np.testing.assert_array_equal(base, full)
    assert uni > 0 and uni0 == 0
    own, _ = run(cuda.cuda.Stream())
    np.testing.assert_array_equal(base, own)
