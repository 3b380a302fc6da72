"""Learned routing end to end: the plain solver records (stencil, TENO cut-off) rows, the tensor-
core MLP trains on them, and a mixed-precision solver routes confidently smooth stencils to the
linear weights.  Checked: the recorded labels agree with the cut-off decided on the recorded
stencils; a router that routes everything (nothing) reproduces the linear (plain TENO) mixed
solver bit for bit; the audit counts; and what the trained network gains."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def teno5_pattern(v):
    """Cut-off bits of the left-biased TENO5 side (cutOff, Schemes_Lagrange.cpp:1141-1149) for rows
    v [n, >=5], float64 (scale-invariant up to the 1e-40 offset)."""
    c0 = v[:, 2] - 2 * v[:, 3] + v[:, 4]
    b0 = (3 * v[:, 2] - 4 * v[:, 3] + v[:, 4]) / 2
    c1 = v[:, 1] - 2 * v[:, 2] + v[:, 3]
    b1 = (v[:, 1] - v[:, 3]) / 2
    c2 = v[:, 0] - 2 * v[:, 1] + v[:, 2]
    b2 = (v[:, 0] - 4 * v[:, 1] + 3 * v[:, 2]) / 2
    si = np.stack([b * b + 13 / 12 * c * c for b, c in ((b0, c0), (b1, c1), (b2, c2))], axis=1)
    u = v
    b35 = (u[:, 4] * (6908 * u[:, 4] - 51001 * u[:, 3] + 67923 * u[:, 2] - 38947 * u[:, 1] + 8209 * u[:, 0])
           + u[:, 3] * (104963 * u[:, 3] - 299076 * u[:, 2] + 179098 * u[:, 1] - 38947 * u[:, 0])
           + u[:, 2] * (231153 * u[:, 2] - 299076 * u[:, 1] + 67923 * u[:, 0])
           + u[:, 1] * (104963 * u[:, 1] - 51001 * u[:, 0]) + 6908 * u[:, 0] ** 2) / 5040
    tau = np.abs(b35 - (si[:, 0] + si[:, 2] + 4 * si[:, 1]) / 6)
    w = (1 + tau[:, None] / (si + 1e-40)) ** 6
    w = w / w.sum(axis=1, keepdims=True)
    return ((w >= 5e-4) * np.array([1, 2, 4])).sum(axis=1)


def bf16_to_float(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def sorted_rows(x, y):
    a = np.concatenate([x.view(np.uint8).reshape(x.shape[0], -1), y[:, None]], axis=1)
    return a[np.lexsort(a.T[::-1])]


def test_harvest_counts_and_labels(hteno_lib, cuda):
    from hteno import ic

    h = hteno_lib
    nx, ny = 64, 48
    total = ((nx + 1) * ny + (ny + 1) * nx) * 4 * 2
    x = cuda.empty((total + 10, 8), dtype=cuda.int16, device="cuda")
    y = cuda.empty((total + 10,), dtype=cuda.uint8, device="cuda")
    with h.Solver(h.config(dims=2, nx=nx, ny=ny, flux=1)) as s:
        s.set_state(ic.four_quadrant(nx, ny, 3))
        s.step(10)
        n1 = s.harvest(1.0, 1, x, y)  # flat stencils are not recorded
        assert 0.2 * total < n1 <= total
        xa = x[:n1].cpu().numpy().view(np.uint16)
        ya = y[:n1].cpu().numpy()
        n3 = s.harvest(0.3, 2, x, y)
        assert abs(n3 - 0.3 * n1) < 0.05 * n1
        a3 = sorted_rows(x[:n3].cpu().numpy().view(np.uint16), y[:n3].cpu().numpy())
        assert s.harvest(0.3, 2, x, y) == n3  # the same rows (in another order)
        np.testing.assert_array_equal(sorted_rows(x[:n3].cpu().numpy().view(np.uint16), y[:n3].cpu().numpy()), a3)
    assert ya.max() <= 7 and 0.1 < (ya == 7).mean() < 1.0
    v = bf16_to_float(xa[:, :6])
    assert np.abs(v).max() <= 1.0 and (xa[:, 6:] == 0).all()
    # the label is the cut-off of the recorded stencil: normalisation preserves it (up to the
    # 1e-40 offset); rounding the recorded values to BF16 (8 significant bits) moves the
    # near-threshold decisions, about 1 in 20 here
    agree = (teno5_pattern(v) == ya).mean()
    assert agree >= 0.92, agree


def test_harvest_1d(hteno_lib, cuda):
    from hteno import ic

    h = hteno_lib
    x = cuda.empty((401 * 6, 8), dtype=cuda.int16, device="cuda")
    y = cuda.empty((401 * 6,), dtype=cuda.uint8, device="cuda")
    with h.Solver(h.config(dims=1, nx=400, flux=1, recon=0, cfl=0.5)) as s:
        s.set_state(ic.sod(400))
        s.step(20, 0.2)
        n = s.harvest(1.0, 5, x, y)
    assert 0 < n <= 401 * 6
    ya = y[:n].cpu().numpy()
    assert (ya == 7).any() and (ya != 7).any()


def test_harvest_and_training_reproducible(hteno_lib, cuda):
    """The whole learned pipeline is reproducible: the harvest kernels append rows in thread
    order, harvest_runs puts them in a canonical order before its seeded shuffle, and training is
    deterministic, so two runs give the same rows and the same network bit for bit."""
    from hteno import learned

    h = hteno_lib
    nets = []
    for _ in range(2):
        x, y = learned.harvest_runs(h, cuda, seeds=[7], n=128, snapshots=(0, 10), keep=0.5,
                                    sod_snapshots=(0, 50))
        with h.Mlp(seed=3) as m:
            m.train(x, y, epochs=2, batch=4096, lr=3e-3)
            nets.append((x.cpu().numpy(), y.cpu().numpy(), m.params().copy()))
    np.testing.assert_array_equal(nets[0][0], nets[1][0])
    np.testing.assert_array_equal(nets[0][1], nets[1][1])
    np.testing.assert_array_equal(nets[0][2], nets[1][2])


def constant_classifier(h, logit):
    m = h.Mlp()
    p = np.zeros(m.nparams, dtype=np.float32)
    p[1376:1379] = logit  # b3: every stencil gets the same probabilities
    m.set_params(p)
    return m


def run_mixed(h, q, steps, router=None, audit=0, **kw):
    cfg = h.config(dims=2, nx=q.shape[2], ny=q.shape[1], flux=1, precision=1, **kw)
    with h.Solver(cfg) as s:
        if router is not None:
            s.set_router(router, 0.9, audit)
        s.set_state(q)
        s.step(steps)
        st = s.router_stats() if router is not None else None
        return s.get_state(), st


def test_router_all_and_nothing(hteno_lib, cuda):
    """A network that routes nothing reproduces the plain run bit for bit (the same kernel runs).
    One that routes everything it is shown (every stencil that is not flat when the step starts;
    the masks are made once per step and serve its three stages) reconstructs those with the
    linear weights: the audits count them, and the run stays close to the all-linear run."""
    from hteno import ic

    h = hteno_lib
    q = ic.four_quadrant(70, 52, 8)
    with constant_classifier(h, 20.0) as all_smooth, constant_classifier(h, -20.0) as none:
        got_none, st0 = run_mixed(h, q, 6, none, audit=2)
        want_teno, _ = run_mixed(h, q, 6)
        np.testing.assert_array_equal(got_none, want_teno)
        faces = (71 * 52 + 53 * 70) * 8
        assert st0["routed"] == 0 and st0["misrouted"] == 0
        assert st0["audits"] == 3 and st0["seen"] == faces * 3 * 3
        got_all, st = run_mixed(h, q, 6, all_smooth, audit=1)
        want_lin, _ = run_mixed(h, q, 6, recon=2)
        assert st["audits"] == 6 and st["seen"] == faces * 3 * 6 and st["network_rows"] > 0
        assert st["routed"] >= 0.5 * (st["seen"] - st["flat"])
        assert 0 < st["misrouted"] <= st["seen"] - st["smooth"]
        assert np.isfinite(got_all).all()
        assert np.abs(got_all[0] - want_lin[0]).mean() <= 0.1 * np.abs(want_teno[0] - want_lin[0]).mean() + 1e-6


def test_router_schedule(hteno_lib, cuda):
    """Classification every k steps with eroded masks: a network that routes nothing still
    reproduces the plain run bit for bit; one that routes everything routes fewer stencils once
    the masks are eroded (faces near the grid's edge keep no route), and every step is audited."""
    from hteno import ic

    h = hteno_lib
    q = ic.four_quadrant(70, 52, 8)
    want_teno, _ = run_mixed(h, q, 6)

    def run_sched(router, every, margin):
        cfg = h.config(dims=2, nx=70, ny=52, flux=1, precision=1)
        with h.Solver(cfg) as s:
            s.set_router(router, 0.9, 1)
            s.set_router_schedule(every, margin)
            s.set_state(q)
            s.step(6)
            return s.get_state(), s.router_stats()

    with constant_classifier(h, 20.0) as all_smooth, constant_classifier(h, -20.0) as none:
        got, st = run_sched(none, 4, 2)
        np.testing.assert_array_equal(got, want_teno)
        assert st["routed"] == 0 and st["audits"] == 6
        _, st1 = run_sched(all_smooth, 1, 0)
        got3, st3 = run_sched(all_smooth, 3, 2)
        assert st3["audits"] == 6 and 0 < st3["routed"] < st1["routed"]
        assert np.isfinite(got3).all()
    with pytest.raises(h.HtenoError):
        with h.Solver(h.config(dims=2, nx=70, ny=52, flux=1, precision=1)) as s:
            s.set_router_schedule(2, 1)  # no router set


def host_misrouted64(oracle, q, bc):
    """Stencils of every face whose FP64 TENO5 cut-off, computed on the host from the oracle's Roe
    eigenvectors, drops a candidate; and the number of stencils."""
    ny, nx = q.shape[1], q.shape[2]
    bad = total = 0
    for d in (1, 2):
        nf, nt, ns = (nx + 1, ny, nx) if d == 1 else (ny + 1, nx, ny)
        f, t = np.meshgrid(np.arange(nf), np.arange(nt), indexing="ij")
        f, t = f.ravel(), t.ravel()

        def cells(off):
            s = (f - 1 + off) % ns if bc == 1 else np.clip(f - 1 + off, 0, ns - 1)
            return q[:, t, s].T if d == 1 else q[:, s, t].T  # [n, 4]

        _, L = oracle.roe2d(1.4, d, np.ascontiguousarray(cells(0)), np.ascontiguousarray(cells(1)))
        L = L.reshape(-1, 4, 4)
        ch = np.stack([np.einsum("nrv,nv->nr", L, cells(m - 2)) for m in range(6)], axis=2)  # [n, 4, 6]
        for r in range(4):
            bad += int((teno5_pattern(ch[:, r, 0:5]) != 7).sum())
            bad += int((teno5_pattern(ch[:, r, 1:6]) != 7).sum())  # the + side: cells 1..5
        total += 8 * f.size
    return bad, total


def test_router_audit64_matches_host(hteno_lib, cuda, oracle):
    """The FP64 judge of the routing: with every stencil routed on a periodic state without flat
    stencils, it counts every stencil as routed, and the stencils whose plain FP64 cut-off drops a
    candidate agree with a host computation from the oracle's eigenvectors (up to decisions at the
    cut-off threshold, which rounding can move).  A router that routes nothing routes nothing."""
    from hteno import ic

    h = hteno_lib
    q = ic.smooth_waves_2d(48, 40)
    q[0] += 0.05 * (np.arange(48)[None, :] % 7 == 0)  # a few kinks, so that some cut-offs drop
    q = np.ascontiguousarray(q)
    want, total = host_misrouted64(oracle, q, 1)
    cfg = h.config(dims=2, nx=48, ny=40, flux=1, bc=1, precision=1)
    with constant_classifier(h, 20.0) as all_smooth, constant_classifier(h, -20.0) as none:
        with h.Solver(cfg) as s:
            s.set_router(all_smooth, 0.9, 0)
            s.set_state(q)
            got = s.router_audit64()
            s.set_router(none, 0.9, 0)
            got0 = s.router_audit64()
    assert got["routed"] == total
    assert 0 < want < total and abs(got["misrouted64"] - want) <= 0.005 * total + 2, (got, want)
    assert got0["routed"] == 0 and got0["misrouted64"] == 0


@pytest.fixture(scope="module")
def trained(hteno_lib, cuda):
    """A classifier trained on rows the plain FP64 solver records from 256^2 four-quadrant runs
    with fresh seeds (and the Sod tube)."""
    from hteno import learned

    h = hteno_lib
    x, y = learned.harvest_runs(h, cuda, seeds=[41, 42], n=256, snapshots=(0, 15, 30), keep=1.0)
    assert x.shape[0] > 50000
    m = h.Mlp(seed=1)
    loss0 = m.grad(x, y)[1]
    loss = m.train(x, y, epochs=10, batch=8192, lr=3e-3)
    acc, routed, mis = learned.accuracy(m, cuda, x, y, 0.9)
    assert loss < 0.7 * loss0 and acc > 0.85 and mis < 0.05, (loss0, loss, acc, routed, mis)
    yield m
    m.close()


def test_trained_router_accuracy(hteno_lib, cuda, trained):
    """Route a mixed 256^2 four-quadrant run: the density error against FP64 stays within the
    mixed path's bound and no shock moves by more than one cell (routing at every step costs
    some accuracy on this small grid: its L1 error is within 5x of the plain mixed run's).  The
    network routes non-flat stencils; the FP64 judge's counts are consistent (on this data it
    finds about a fifth of the float-resolved routes misrouted; those sit on weak features, as the
    density bound shows)."""
    from hteno import ic, metrics

    h = hteno_lib
    q = ic.four_quadrant(256, 256, 99)
    with h.Solver(h.config(dims=2, nx=256, ny=256, flux=1)) as s:
        s.set_state(q)
        s.step(30)
        t_ref, _, _ = s.time()
        ref = s.get_state()
    with h.Solver(h.config(dims=2, nx=256, ny=256, flux=1, precision=1)) as s:
        s.set_state(q)
        s.step(1000, t_ref)
        plain = s.get_state()
    with h.Solver(h.config(dims=2, nx=256, ny=256, flux=1, precision=1)) as s:
        s.set_router(trained, 0.99, 5)
        s.set_state(q)
        s.step(1000, t_ref)
        st = s.router_stats()
        got = s.get_state()
        a64 = s.router_audit64()
    l1 = np.abs(got[0] - ref[0]).mean()
    assert l1 <= 1e-4, l1  # the accuracy bound of the learned path against FP64
    assert np.abs(plain[0] - ref[0]).mean() <= l1 <= 5 * np.abs(plain[0] - ref[0]).mean()
    assert metrics.shock_shift(got[0], ref[0]) <= 1  # no shock moves by more than one cell
    assert st["routed"] > 0 and st["flat"] > 0, st
    assert 0 < a64["routed_resolved"] <= a64["routed"], a64
    assert a64["misrouted64_resolved"] <= a64["misrouted64"] <= a64["routed"], a64
    assert a64["misrouted64_resolved"] < a64["routed_resolved"], a64


def step_kernels_ms(h, s, steps):
    """Per-step time of the stage kernels (CUDA events around each launch) and of the classifier."""
    import ctypes

    lib = h.lib()
    lib.hteno_enable_kernel_timing(s.h, 1)
    s.step(steps)
    kt = (h.KernelTime * 16)()
    cnt = ctypes.c_int()
    lib.hteno_kernel_timing(s.h, kt, 16, ctypes.byref(cnt))
    lib.hteno_enable_kernel_timing(s.h, 0)
    ms = {kt[k].name.decode(): kt[k].ms / steps for k in range(cnt.value) if kt[k].launches}
    return sum(v for k, v in ms.items() if k.startswith("fused")), ms.get("classify", 0.0)


@pytest.fixture(scope="module")
def trained_1024(hteno_lib, cuda):
    """A classifier trained as the bench trains it, on rows from 1024^2 four-quadrant runs (two
    fresh seeds, four snapshots each) and the Sod tube."""
    from hteno import learned

    h = hteno_lib
    x, y = learned.harvest_runs(h, cuda, seeds=[201, 202], n=1024, snapshots=(0, 20, 40, 60), keep=1.0)
    m = h.Mlp(seed=0)
    m.train(x, y, epochs=10, batch=16384, lr=3e-3)
    del x, y
    yield m
    m.close()


def test_trained_router_gains(hteno_lib, cuda, trained_1024):
    """What the trained network gains over plain TENO, on a fixed case with no flat stencil: a
    smooth periodic flow on 2048^2.  The network routes nearly every stencil to the linear
    weights, the stage kernels skip the nonlinear weights there and run faster than plain TENO's,
    and the solution is the plain mixed solution to float rounding (TENO keeps all three
    candidates on smooth data too).  Classified every 20 steps with masks eroded by 8 faces, the
    classifier's share is small enough that whole steps are faster as well."""
    from hteno import ic

    h = hteno_lib
    trained = trained_1024
    n = 2048
    q = ic.smooth_waves_2d(n, n)
    cfg = h.config(dims=2, nx=n, ny=n, flux=1, bc=1, precision=1)
    with h.Solver(cfg) as s:
        s.set_state(q)
        s.step(5)
        plain_stage, _ = step_kernels_ms(h, s, 40)
        s.set_state(q)
        s.step(45)
        want = s.get_state()
    with h.Solver(cfg) as s:
        s.set_router(trained, 0.99, 0)
        s.set_router_schedule(20, 8)
        s.set_state(q)
        s.step(5)
        routed_stage, classify = step_kernels_ms(h, s, 40)
        s.set_state(q)
        s.step(40)
        st = s.router_audit64()
        s.set_state(q)
        s.step(45)
        got = s.get_state()
    assert st["routed"] >= 0.9 * 8 * 2 * n * (n + 1) and st["misrouted64"] <= 1e-4 * st["routed"], st
    assert np.abs(got[0] - want[0]).max() <= 1e-5 * np.abs(want[0]).max()
    assert routed_stage <= 0.97 * plain_stage, (routed_stage, plain_stage)
    assert routed_stage + classify <= plain_stage, (routed_stage, classify, plain_stage)
