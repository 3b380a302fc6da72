"""Batched independent 2D grids (hteno_batch_*): every instance evolves exactly as the same grid
run alone through the single-grid mixed path (same tiles arithmetic, same per-instance dt), with
its own time, step count and stop test."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (130, 70), (48, 200), (96, 33), (250, 128), (6, 9)]


def make_batch(h, sizes, seed0=100, **kw):
    from hteno import ic

    cfgs = [h.config(dims=2, nx=nx, ny=ny, flux=1, precision=1, **kw) for nx, ny in sizes]
    states = [ic.four_quadrant(nx, ny, seed0 + k) for k, (nx, ny) in enumerate(sizes)]
    b = h.Batch(cfgs)
    for k, q in enumerate(states):
        b.set_state(k, q)
    return b, cfgs, states


def single(h, cfg, q, nsteps, t_final=float("inf")):
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.step(nsteps, t_final)
        t, n, _ = s.time()
        return s.get_state(), t, n


def test_batch_matches_single_grids(hteno_lib, cuda):
    b, cfgs, states = make_batch(hteno_lib, SIZES)
    with b:
        b.step(15)
        for k, (cfg, q) in enumerate(zip(cfgs, states)):
            want, t_w, n_w = single(hteno_lib, cfg, q, 15)
            t, n, st = b.time(k)
            assert n == n_w == 15 and t == t_w and st == 0
            np.testing.assert_array_equal(b.get_state(k), want)


def test_batch_per_instance_time_and_stop(hteno_lib, cuda):
    """Instances stop independently when they reach t_final; their dts differ."""
    b, cfgs, states = make_batch(hteno_lib, SIZES[:4], seed0=7)
    with b:
        b.step(1000, 0.02)
        counts = set()
        for k, (cfg, q) in enumerate(zip(cfgs, states)):
            want, t_w, n_w = single(hteno_lib, cfg, q, 1000, 0.02)
            t, n, _ = b.time(k)
            assert n == n_w and t == t_w == pytest.approx(0.02, rel=1e-14, abs=0)
            counts.add(n)
            np.testing.assert_array_equal(b.get_state(k), want)
        assert len(counts) > 1


def test_batch_graph_replay_is_resumable(hteno_lib, cuda):
    b1, _, _ = make_batch(hteno_lib, SIZES[:3], seed0=3)
    b2, _, _ = make_batch(hteno_lib, SIZES[:3], seed0=3)
    with b1, b2:
        b1.step(7)
        b2.step(3)
        b2.step(4)
        for k in range(3):
            np.testing.assert_array_equal(b1.get_state(k), b2.get_state(k))
            assert b1.time(k)[:2] == b2.time(k)[:2]


def test_batch_tile_shapes_agree(hteno_lib, cuda):
    outs = []
    try:
        for v in range(8):  # every tile shape and register budget of the tuner
            os.environ["HTENO_FV2D_TILE"] = str(v)
            b, _, _ = make_batch(hteno_lib, SIZES[:3], seed0=9)
            with b:
                assert b.tile()[0] > 0
                b.step(5)
                outs.append([b.get_state(k) for k in range(3)])
    finally:
        os.environ.pop("HTENO_FV2D_TILE", None)
    for o in outs[1:]:
        for a, c in zip(o, outs[0]):
            np.testing.assert_array_equal(a, c)


def test_batch_tuner_picks_a_candidate(hteno_lib, cuda):
    b, _, _ = make_batch(hteno_lib, SIZES[:2])
    with b:
        tx, ty, nt = b.tile()
        assert (tx, ty, nt) in {(32, 16, 256), (32, 8, 256), (16, 16, 256), (64, 8, 256), (32, 32, 512), (16, 8, 128)}


def test_batch_tma_same_bits(hteno_lib, cuda):
    """Interior tiles of the batch's instances staged by TMA box copies (tensor maps in the instance
    records) give the same bits as cell-by-cell loads (HTENO_TMA=0), for three forced tile shapes;
    an instance with an odd nx (row stride not a multiple of 16 bytes) loads cell by cell."""
    sizes = [(250, 128), (130, 70), (96, 96), (64, 64), (161, 90)]
    for v in (0, 4, 6):
        outs = []
        try:
            os.environ["HTENO_FV2D_TILE"] = str(v)
            for tma in ("1", "0"):
                os.environ["HTENO_TMA"] = tma
                b, _, _ = make_batch(hteno_lib, sizes, seed0=31)
                with b:
                    b.step(12)
                    outs.append([b.get_state(k) for k in range(len(sizes))])
                    tiles = b.counters(0)["tma_tiles"]  # the 250 x 128 instance
                    assert (tiles > 0) == (tma == "1"), (v, tma, tiles)
                    assert b.counters(4)["tma_tiles"] == 0
        finally:
            os.environ.pop("HTENO_TMA", None)
            os.environ.pop("HTENO_FV2D_TILE", None)
        for a, c in zip(outs[0], outs[1]):
            np.testing.assert_array_equal(a, c)


def test_batch_256_configuration(hteno_lib, cuda):
    """The batched configuration at its stated size: 256 instances with sides drawn from
    {64, ..., 512} (seeded, non-square), seeded four-quadrant data each, TENO5 + HLLC, mixed
    precision, 100 steps.  Eight sampled instances equal the same grids run alone bit for bit, and
    every instance's density stays within the mixed path's bound of the plain FP64 run at its own
    end time (three sampled instances checked against FP64)."""
    from hteno import ic

    h = hteno_lib
    rng = np.random.default_rng(4)
    sides = rng.integers(64, 513, size=(256, 2))
    cfgs = [h.config(dims=2, nx=int(nx), ny=int(ny), flux=1, precision=1) for nx, ny in sides]
    states = [ic.four_quadrant(int(nx), int(ny), 1000 + k) for k, (nx, ny) in enumerate(sides)]
    with h.Batch(cfgs) as b:
        for k, q in enumerate(states):
            b.set_state(k, q)
        b.step(100)
        picks = [0, 17, 64, 101, 128, 199, 230, 255]
        got = {k: (b.get_state(k), b.time(k)) for k in picks}
    for k in picks:
        state, (t, n, st) = got[k]
        want, t_w, n_w = single(h, cfgs[k], states[k], 100)
        assert n == n_w == 100 and t == t_w
        np.testing.assert_array_equal(state, want)
    for k in picks[:3]:
        state, (t, n, st) = got[k]
        if st:
            continue  # instances whose data go non-physical (as the FP64 solver's do) are flagged
        c64 = h.config(dims=2, nx=int(sides[k][0]), ny=int(sides[k][1]), flux=1)
        ref, t_r, _ = single(h, c64, states[k], 1000, t)
        assert t_r == pytest.approx(t, rel=1e-14, abs=0)
        assert np.abs(state[0] - ref[0]).mean() <= 1e-4


def test_batch_health_flags_follow_plain_fp64(hteno_lib, cuda):
    """Instances of the 256-grid configuration that the batch flags as non-physical are flagged by
    the plain FP64 solver (the reference's arithmetic, bit for bit) in the same steps; a healthy
    one stays unflagged in both.  Instances 0, 35 and 139: (390 x 487, seed 1000), (511 x 481,
    seed 1035), (374 x 485, seed 1139)."""
    from hteno import ic

    h = hteno_lib
    inst = [((390, 487), 1000), ((511, 481), 1035), ((374, 485), 1139)]
    cfgs = [h.config(dims=2, nx=nx, ny=ny, flux=1, precision=1) for (nx, ny), _ in inst]
    states = [ic.four_quadrant(nx, ny, seed) for (nx, ny), seed in inst]
    with h.Batch(cfgs) as b:
        for k, q in enumerate(states):
            b.set_state(k, q)
        b.step(5)
        flags = [b.time(k)[2] for k in range(len(inst))]
    fp64 = []
    for ((nx, ny), _), q in zip(inst, states):
        with h.Solver(h.config(dims=2, nx=nx, ny=ny, flux=1)) as s:
            s.set_state(q)
            s.step(5)
            fp64.append(s.status())
    assert flags[0] == 0 and fp64[0] == 0
    assert flags[1] and flags[2]
    assert all(f64 for f, f64 in zip(flags, fp64) if f)
