"""Mixed-precision FV 2D path (float reconstruction and fluxes, double state and SSP-RK3; one
fused launch per stage): error against the plain FP64 path, which is bit-identical to the CPU
oracle, at the same simulated time; independence of the tile shape; conservation; health flags."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_TOL = 1e-4  # L1 density error bound of the mixed path against FP64


def run(h, q, nsteps, t_final=1e30, **kw):
    cfg = h.config(dims=2, nx=q.shape[2], ny=q.shape[1], **kw)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.step(nsteps, t_final)
        t, n, _ = s.time()
        return s.get_state(), t, n, s.status()


def smooth_periodic(nx, ny):
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    rho = 1 + 0.2 * np.sin(2 * np.pi * (X + Y))
    return np.ascontiguousarray(ic.conservative2(rho, 0.5 + 0 * X, -0.3 + 0 * X, 1 + 0 * X))


def periodic_box(nx, ny):
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    inside = (np.abs(X - 0.5) < 0.25) & (np.abs(Y - 0.5) < 0.25)
    return np.ascontiguousarray(ic.conservative2(1.0 + inside, 0.5 + 0 * X, -0.3 + 0 * X, 1.0 + 1.5 * inside))


CASES = [
    dict(flux=1, recon=0, bc=0), dict(flux=0, recon=0, bc=0), dict(flux=1, recon=1, bc=0),
    dict(flux=0, recon=0, bc=1), dict(flux=1, recon=2, bc=1),
]


@pytest.mark.parametrize("cfg", CASES, ids=lambda c: f"flux{c['flux']}-recon{c['recon']}-bc{c['bc']}")
def test_mixed_error_against_fp64(hteno_lib, cuda, cfg):
    from hteno import ic

    nx, ny = 96, 80
    if cfg["recon"] == 2:
        q = smooth_periodic(nx, ny)
    elif cfg["bc"] == 1:
        q = periodic_box(nx, ny)
    else:
        q = ic.four_quadrant(nx, ny, 11)
    ref, t_ref, _, _ = run(hteno_lib, q, 40, **cfg)
    got, t_got, n_got, st = run(hteno_lib, q, 1000, t_final=t_ref, precision=1, **cfg)
    assert t_got == pytest.approx(t_ref, rel=1e-14, abs=0) and st == 0
    l1 = np.abs(got[0] - ref[0]).mean()
    assert l1 <= L1_TOL, l1
    # each conserved variable, relative to its range
    rng = ref.max(axis=(1, 2)) - ref.min(axis=(1, 2)) + 1e-300
    assert (np.abs(got - ref).mean(axis=(1, 2)) / rng).max() <= 1e-3


def test_mixed_smooth_flow_is_accurate(hteno_lib, cuda):
    """On a smooth periodic flow the mixed path stays within float rounding of FP64."""
    q = smooth_periodic(64, 64)
    ref, t_ref, _, _ = run(hteno_lib, q, 30, flux=1, bc=1)
    got, _, _, _ = run(hteno_lib, q, 1000, t_final=t_ref, flux=1, bc=1, precision=1)
    assert np.abs(got - ref).max() <= 1e-5


@pytest.mark.parametrize("kw", [dict(flux=1), dict(flux=0, recon=1), dict(flux=1, recon=5, bc=1)],
                         ids=["hllc-teno5", "rusanov-teno5i", "hllc-weno5n-periodic"])
def test_mixed_tile_shapes_agree_bitwise(hteno_lib, cuda, kw):
    """Every tile shape computes each face from the same data with the same arithmetic, so the
    results are identical; the grid is not a multiple of any tile."""
    from hteno import ic

    q = ic.four_quadrant(70, 45, 5) if kw.get("bc", 0) == 0 else periodic_box(70, 45)
    outs = []
    try:
        for v in range(8):  # every tile shape and register budget of the tuner
            os.environ["HTENO_FV2D_TILE"] = str(v)
            outs.append(run(hteno_lib, q, 12, precision=1, **kw)[0])
    finally:
        os.environ.pop("HTENO_FV2D_TILE", None)
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


def blob_field(nx, ny, scale=1.0, mach=0.3):
    """A dense, high-pressure disc in a uniform stream: most tiles are uniform."""
    from hteno import ic

    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    disc = (X - 0.45) ** 2 + (Y - 0.5) ** 2 < 0.12 ** 2
    u = mach * np.sqrt(1.4) + 0 * X
    return np.ascontiguousarray(ic.conservative2(scale * (1.0 + disc), u, -0.2 * u, scale * (1.0 + 2.0 * disc)))


def four_quadrant(nx, ny, seed):
    from hteno import ic

    return ic.four_quadrant(nx, ny, seed)


UNIFORM_CASES = {
    "four-quadrant": (lambda: four_quadrant(150, 110, 3), dict(flux=1)),
    "stream-periodic": (lambda: blob_field(160, 96), dict(flux=0, bc=1)),
    "tiny-density": (lambda: blob_field(160, 96, scale=1e-6), dict(flux=1)),  # below 2^-16
    "hypersonic": (lambda: blob_field(160, 96, mach=12.0), dict(flux=1)),  # Mach above 8
}


@pytest.mark.parametrize("case", list(UNIFORM_CASES))
def test_mixed_uniform_tiles_exact(hteno_lib, cuda, case):
    """Tiles whose cells and halo hold one tame float state take their residual (exactly +0)
    without computing faces; HTENO_UNIFORM_SKIP=0 computes them in full: the same bits.  (The
    batch path runs the same tile code; it matches the single-grid path bit for bit.)"""
    make, kw = UNIFORM_CASES[case]
    q = make()
    try:
        os.environ["HTENO_UNIFORM_SKIP"] = "0"
        full, t_full, n_full, _ = run(hteno_lib, q, 40, precision=1, **kw)
    finally:
        os.environ.pop("HTENO_UNIFORM_SKIP", None)
    got, t_got, n_got, _ = run(hteno_lib, q, 40, precision=1, **kw)
    assert n_got == n_full and t_got == t_full
    np.testing.assert_array_equal(got, full)


@pytest.mark.parametrize("nx,ny,bc,tile", [(160, 96, 0, None), (128, 72, 1, "6"), (96, 96, 0, "4"),
                                          (161, 90, 0, None)])
def test_mixed_tma_tiles_same_bits(hteno_lib, cuda, nx, ny, bc, tile):
    """Interior tiles staged by a TMA box copy of the four state planes give the same bits as the
    cell-by-cell loads (HTENO_TMA=0), for several tile shapes and both copy boundaries; a grid with
    an odd nx (row stride not a multiple of 16 bytes) loads every tile cell by cell."""
    from hteno import ic

    q = ic.four_quadrant(nx, ny, 21)
    cfg = hteno_lib.config(dims=2, nx=nx, ny=ny, flux=1, bc=bc, precision=1)

    def go():
        with hteno_lib.Solver(cfg) as s:
            s.set_state(q)
            s.step(30)
            return s.get_state(), s.counters(), s.time()

    try:
        if tile is not None:
            os.environ["HTENO_FV2D_TILE"] = tile
        got, c, t = go()
        os.environ["HTENO_TMA"] = "0"
        want, c0, t0 = go()
    finally:
        os.environ.pop("HTENO_TMA", None)
        os.environ.pop("HTENO_FV2D_TILE", None)
    assert t == t0 and c0["tma_tiles"] == 0
    np.testing.assert_array_equal(got, want)
    if nx % 2:
        assert c["tma_tiles"] == 0
    else:
        assert c["tma_tiles"] > 0


@pytest.mark.parametrize("bc,fn,shape,box", [
    (2, "rayleigh_taylor", (40, 150), (0.0, 0.25, 0.0, 1.0)),
    (3, "double_mach", (160, 41), (0.0, 4.0, 0.0, 1.0))])
def test_mixed_boundaries(hteno_lib, cuda, bc, fn, shape, box):
    """TaylorInstBc / doubleMachBc on the mixed path: close to FP64 at the same time, the same
    bits with and without the uniform-tile skipping, and a batch of the grid reproduces it."""
    from hteno import ic

    xl, xr, yb, yt = box
    q = getattr(ic, fn)(*shape, xl, xr, yb, yt)
    kw = dict(flux=1, bc=bc, xl=xl, xr=xr, yb=yb, yt=yt)
    ref, t_ref, _, _ = run(hteno_lib, q, 40, **kw)
    got, t_got, _, st = run(hteno_lib, q, 1000, t_final=t_ref, precision=1, **kw)
    assert t_got == pytest.approx(t_ref, rel=1e-14, abs=0) and st == 0
    assert np.abs(got[0] - ref[0]).mean() <= 1e-3 * np.abs(ref[0]).mean()
    try:
        os.environ["HTENO_UNIFORM_SKIP"] = "0"
        full, _, _, _ = run(hteno_lib, q, 1000, t_final=t_ref, precision=1, **kw)
    finally:
        os.environ.pop("HTENO_UNIFORM_SKIP", None)
    np.testing.assert_array_equal(got, full)
    cfg = hteno_lib.config(dims=2, nx=shape[0], ny=shape[1], precision=1, **kw)
    with hteno_lib.Batch([cfg]) as b:
        b.set_state(0, q)
        b.step(10)
        single, _, _, _ = run(hteno_lib, q, 10, precision=1, **kw)
        np.testing.assert_array_equal(b.get_state(0), single)


def test_mixed_periodic_conservation(hteno_lib, cuda):
    q = periodic_box(128, 96)
    got, _, _, _ = run(hteno_lib, q, 60, flux=1, bc=1, precision=1)
    tot0, tot = q.sum(axis=(1, 2)), got.sum(axis=(1, 2))
    assert (np.abs(tot - tot0) <= 1e-12 * np.abs(q).sum(axis=(1, 2))).all(), tot - tot0


def test_mixed_residual_close_to_fp64(hteno_lib, cuda):
    from hteno import ic

    q = ic.four_quadrant(80, 64, 21)
    out = {}
    for prec in (0, 1):
        with hteno_lib.Solver(hteno_lib.config(dims=2, nx=80, ny=64, flux=1, precision=prec)) as s:
            dq = cuda.from_numpy(q).cuda()
            r = cuda.empty_like(dq)
            s.residual(dq, r)
            cuda.cuda.synchronize()
            out[prec] = r.cpu().numpy()
    d = np.abs(out[1] - out[0]).mean(axis=(1, 2)) / np.abs(out[0]).mean(axis=(1, 2))
    assert (d <= 1e-3).all(), d


def test_mixed_edge_sizes(hteno_lib, cuda):
    from hteno import ic

    for nx, ny in ((6, 6), (7, 13), (64, 9), (200, 6)):
        q = ic.four_quadrant(nx, ny, nx * 100 + ny)
        ref, t_ref, _, _ = run(hteno_lib, q, 8, flux=0)
        got, t_got, _, _ = run(hteno_lib, q, 1000, t_final=t_ref, flux=0, precision=1)
        assert t_got == pytest.approx(t_ref, rel=1e-14, abs=0) and np.isfinite(got).all()
        assert np.abs(got[0] - ref[0]).mean() <= 1e-3


def test_mixed_constant_state_is_steady(hteno_lib, cuda):
    q = np.ascontiguousarray(np.broadcast_to(np.array([1.3, 0.2, -0.4, 2.7])[:, None, None], (4, 20, 24)).copy())
    got, _, _, st = run(hteno_lib, q, 5, flux=1, precision=1)
    np.testing.assert_allclose(got, q, rtol=1e-6, atol=1e-6)
    assert st == 0


def test_mixed_nonphysical_state_is_flagged(hteno_lib, cuda):
    from hteno import ic

    q = ic.four_quadrant(32, 32, 1)
    q[0, 10, 10] = -0.5
    _, _, _, st = run(hteno_lib, q, 1, flux=1, precision=1)
    assert st != 0
