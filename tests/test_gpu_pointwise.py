"""GPU parity of the pointwise batch kernels (one reference function each) against the oracle
and against the reference's own golden vectors.  Called through the C-ABI."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"

# FP64: the kernels perform the oracle's IEEE operations in the oracle's order (compiled without
# contraction), so the results are bit-identical; the scaled error must be exactly zero.
RTOL64 = 0.0


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def close_scaled(got, want, scale, rtol):
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    assert np.nanmax(err) <= rtol, f"max scaled error {np.nanmax(err):.3e}"


def stencils(rng, n, width):
    x = np.arange(width)
    out = rng.normal(size=(n, width)) * 10.0 ** rng.uniform(-3, 3, (n, 1))
    k = n // 3
    out[:k] = np.sin(0.1 + 0.05 * x)[None, :] * rng.uniform(0.5, 2, (k, 1))
    steps = rng.integers(1, width, n - 2 * k)
    out[2 * k:] = np.where(x[None, :] < steps[:, None], 1.0, 4.0) * rng.uniform(0.5, 2, (n - 2 * k, 1))
    return np.ascontiguousarray(out)


@pytest.fixture(scope="module")
def pw():
    return dict(np.load(GOLD / "pointwise.npz"))


def run_lagrange(h, torch, kind, u, prec=0):
    du = dev(torch, u)
    out = torch.empty((u.shape[0], 2), dtype=torch.float64, device="cuda")
    assert h.lib().hteno_lagrange_batch(kind, prec, du.data_ptr(), out.data_ptr(), u.shape[0], None) == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_lagrange_vs_oracle_and_reference(hteno_lib, cuda, oracle, pw):
    rng = np.random.default_rng(5)
    for u in (pw["lag_u"], stencils(rng, 20000, 6)):
        scale = np.abs(u).max(axis=1, keepdims=True)
        for kind in (0, 1, 2):
            got = run_lagrange(hteno_lib, cuda, kind, u)
            close_scaled(got, oracle.lagrange(kind, u), scale, RTOL64)
    for kind, name in enumerate(("teno5", "teno5i", "linear5")):
        u = pw["lag_u"]
        close_scaled(run_lagrange(hteno_lib, cuda, kind, u), pw[f"lag_{name}"],
                     np.abs(u).max(axis=1, keepdims=True), RTOL64)


def test_lagrange_mixed_precision_smooth(hteno_lib, cuda, oracle):
    x = np.arange(6)
    u = np.ascontiguousarray(np.sin(0.2 + 0.03 * x)[None, :] * np.linspace(0.5, 2, 512)[:, None])
    got = run_lagrange(hteno_lib, cuda, 0, u, prec=1)
    np.testing.assert_allclose(got, oracle.lagrange(0, u), rtol=2e-6, atol=1e-6)


def test_gl3(hteno_lib, cuda, oracle, pw):
    rng = np.random.default_rng(6)
    for u in (pw["gl3_u"], stencils(rng, 20000, 5)):
        du = dev(cuda, u)
        out = cuda.empty((u.shape[0], 3), dtype=cuda.float64, device="cuda")
        assert hteno_lib.lib().hteno_gl3_batch(0, du.data_ptr(), out.data_ptr(), u.shape[0], None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), oracle.gl3(u), np.abs(u).max(axis=1, keepdims=True), RTOL64)
    close_scaled(oracle.gl3(pw["gl3_u"]), pw["gl3_out"], 1.0, 0.0)


def test_gl3_bitwise_extreme_scales(hteno_lib, cuda, oracle):
    """The FP64 GL3 divides by shared denominators through one correctly rounded reciprocal and a
    remainder correction, with operands outside [2^-500, 2^501) sent to the division itself.
    Stencils scaled from 1e-300 to 1e300, with zeros, negative zeros, subnormals and lone spikes,
    reproduce the CPU oracle (plain IEEE division) bit for bit."""
    rng = np.random.default_rng(17)
    n = 40000
    u = rng.normal(size=(n, 5)) * 10.0 ** rng.uniform(-300, 300, (n, 1))
    u[:2000] = 0.0
    u[2000:4000] = -0.0
    u[4000:6000, 2] = rng.normal(size=2000) * 1e-310  # subnormal spikes on zero
    u[6000:8000] = rng.normal(size=(2000, 5)) * 5e-324 * rng.integers(1, 50, (2000, 1))
    spikes = rng.integers(0, 5, 4000)
    u[8000:12000] = 0.0
    u[8000 + np.arange(4000), spikes] = 10.0 ** rng.uniform(-200, 200, 4000)
    u[12000:14000] = np.array([1.0, 1.0, 1.0, 1.0, 1.0]) * 10.0 ** rng.uniform(-250, 250, (2000, 1))
    du = dev(cuda, u)
    out = cuda.empty((n, 3), dtype=cuda.float64, device="cuda")
    assert hteno_lib.lib().hteno_gl3_batch(0, du.data_ptr(), out.data_ptr(), n, None) == 0
    cuda.cuda.synchronize()
    got, want = out.cpu().numpy(), oracle.gl3(u)
    np.testing.assert_array_equal(got.view(np.uint64), want.view(np.uint64))


def test_hermite_recon_and_limiter(hteno_lib, cuda, oracle, pw):
    dx = float(pw["her_dx"])
    u, d = pw["her_u"], pw["her_d"]
    du, dd = dev(cuda, u), dev(cuda, d)
    scale = (np.abs(u).max(axis=1) + dx * np.abs(d).max(axis=1))[:, None]
    for kind, name in enumerate(("hteno", "htenoi", "hlinear")):
        out = cuda.empty((u.shape[0], 4), dtype=cuda.float64, device="cuda")
        assert hteno_lib.lib().hteno_hermite_batch(kind, 0, dx, du.data_ptr(), dd.data_ptr(),
                                                   out.data_ptr(), u.shape[0], None) == 0
        cuda.cuda.synchronize()
        got = out.cpu().numpy()
        want = pw[f"her_{name}"]
        close_scaled(got[:, :2], want[:, :2], scale, RTOL64)          # values
        close_scaled(got[:, 2:], want[:, 2:], scale / dx, RTOL64)     # derivatives
    u3, d3 = pw["lim_u"], pw["lim_d"]
    out = cuda.empty(u3.shape[0], dtype=cuda.float64, device="cuda")
    assert hteno_lib.lib().hteno_hlimiter_batch(0, dx, dev(cuda, u3).data_ptr(), dev(cuda, d3).data_ptr(),
                                                out.data_ptr(), u3.shape[0], None) == 0
    cuda.cuda.synchronize()
    lscale = np.abs(u3).max(axis=1) / dx + np.abs(d3).max(axis=1)
    close_scaled(out.cpu().numpy(), pw["lim_out"], lscale, RTOL64)


def test_fluxes(hteno_lib, cuda, oracle, pw):
    L = hteno_lib.lib()
    ql, qr, qa, qb = pw["flux_ql"], pw["flux_qr"], pw["flux_qa"], pw["flux_qb"]
    dql, dqr = pw["flux_dql"], pw["flux_dqr"]
    n = ql.shape[0]
    t = {k: dev(cuda, v) for k, v in dict(ql=ql, qr=qr, qa=qa, qb=qb, dql=dql, dqr=dqr).items()}
    out = cuda.empty((n, 4), dtype=cuda.float64, device="cuda")
    scale = np.maximum(np.abs(ql).max(axis=1), np.abs(qr).max(axis=1))[:, None] * 4
    for d in (1, 2):
        assert L.hteno_hllc2d_batch(0, 1.4, d, t["ql"].data_ptr(), t["qr"].data_ptr(), out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"hllc2d_{d}"], scale, RTOL64)
        assert L.hteno_rusanov2d_batch(0, 1.4, d, t["qa"].data_ptr(), t["qb"].data_ptr(), t["ql"].data_ptr(),
                                       t["qr"].data_ptr(), out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"rusanov2d_{d}"], scale, RTOL64)
        assert L.hteno_drusanov2d_batch(0, 1.4, d, t["qa"].data_ptr(), t["qb"].data_ptr(), t["ql"].data_ptr(),
                                        t["qr"].data_ptr(), t["dql"].data_ptr(), t["dqr"].data_ptr(),
                                        out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"drusanov2d_{d}"], scale * 4, RTOL64)
    a, b = dev(cuda, pw["hllc1d_ql"]), dev(cuda, pw["hllc1d_qr"])
    o3 = cuda.empty((n, 3), dtype=cuda.float64, device="cuda")
    assert L.hteno_hllc1d_batch(0, 1.4, a.data_ptr(), b.data_ptr(), o3.data_ptr(), n, None) == 0
    cuda.cuda.synchronize()
    close_scaled(o3.cpu().numpy(), pw["hllc1d_out"], scale[:, :1], RTOL64)


def test_fluxes_float(hteno_lib, cuda, pw):
    """The float fluxes of the mixed path (reciprocals and square roots on the MUFU) against the
    reference's FP64 values: within float accuracy of the states' magnitude."""
    L = hteno_lib.lib()
    ql, qr, qa, qb = pw["flux_ql"], pw["flux_qr"], pw["flux_qa"], pw["flux_qb"]
    dql, dqr = pw["flux_dql"], pw["flux_dqr"]
    n = ql.shape[0]
    t = {k: dev(cuda, v) for k, v in dict(ql=ql, qr=qr, qa=qa, qb=qb, dql=dql, dqr=dqr).items()}
    out = cuda.empty((n, 4), dtype=cuda.float64, device="cuda")
    scale = np.maximum(np.abs(ql).max(axis=1), np.abs(qr).max(axis=1))[:, None] * 4
    rtol = 2e-5  # float (2^-24) through ~20 dependent operations, approximate reciprocals included
    for d in (1, 2):
        assert L.hteno_hllc2d_batch(1, 1.4, d, t["ql"].data_ptr(), t["qr"].data_ptr(), out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"hllc2d_{d}"], scale, rtol)
        assert L.hteno_rusanov2d_batch(1, 1.4, d, t["qa"].data_ptr(), t["qb"].data_ptr(), t["ql"].data_ptr(),
                                       t["qr"].data_ptr(), out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"rusanov2d_{d}"], scale, rtol)
        assert L.hteno_drusanov2d_batch(1, 1.4, d, t["qa"].data_ptr(), t["qb"].data_ptr(), t["ql"].data_ptr(),
                                        t["qr"].data_ptr(), t["dql"].data_ptr(), t["dqr"].data_ptr(),
                                        out.data_ptr(), n, None) == 0
        cuda.cuda.synchronize()
        close_scaled(out.cpu().numpy(), pw[f"drusanov2d_{d}"], scale * 4, rtol)


def test_ssprk3_bitwise(hteno_lib, cuda, pw):
    """The stage combination is plain IEEE arithmetic in the reference's order: bit-exact."""
    q0, qn, rhs = (dev(cuda, pw[k]) for k in ("rk_q0", "rk_qn", "rk_rhs"))
    out = cuda.empty_like(q0)
    for st in (1, 2, 3):
        assert hteno_lib.lib().hteno_ssprk3_batch(q0.data_ptr(), qn.data_ptr(), rhs.data_ptr(), 0.013, st,
                                                  out.data_ptr(), q0.numel(), None) == 0
        cuda.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), pw[f"rk_stage{st}"])


def test_alternative_reconstructions(hteno_lib, cuda, oracle):
    """weno5JS, weno5Z, teno5N, teno5a bit for bit against the oracle (itself pinned to the
    reference's outputs); weno5N within 1e-14, its |.|^2.5 going through the device pow."""
    from pathlib import Path

    g = dict(np.load(Path(__file__).resolve().parent / "golden" / "alternatives.npz"))
    rng = np.random.default_rng(8)
    for u in (g["alt_u"], stencils(rng, 20000, 6)):
        scale = np.abs(u).max(axis=1, keepdims=True)
        for kind in (3, 4, 5, 6, 7):
            got = run_lagrange(hteno_lib, cuda, kind, u)
            want = oracle.lagrange(kind, u)
            if kind == 5:
                close_scaled(got, want, scale, 1e-14)
            else:
                np.testing.assert_array_equal(got, want)
    for kind in (3, 4, 5, 6, 7):  # float versions: close to double on smooth data
        x = np.arange(6)
        u = np.ascontiguousarray(np.sin(0.2 + 0.03 * x)[None, :] * np.linspace(0.5, 2, 256)[:, None])
        np.testing.assert_allclose(run_lagrange(hteno_lib, cuda, kind, u, prec=1), oracle.lagrange(kind, u),
                                   rtol=5e-6, atol=5e-6)


def test_lagrange_cutoff_edge_cases_vs_oracle(hteno_lib, cuda, oracle):
    """TENO cut-off decisions at the ends of the fast paths' ranges, bit for bit against the
    oracle: constant sub-stencils next to huge jumps (indicator 0, so r = 1 + tau / epsz beyond the
    float scaling's 2^125 and, from |jump| ~ 1e6 on, weights whose pow(r, 6) overflows to inf in
    the reference), tiny and huge magnitudes, and equal indicators."""
    rng = np.random.default_rng(17)
    n = 6000
    rows = []
    for mag in (1e-30, 1e-8, 1.0, 1e3, 1e6, 1e12, 1e20):
        base = rng.uniform(0.5, 2.0, (n, 6))
        const = base.copy()
        const[:, :3] = base[:, :1]  # three equal cells: one indicator exactly 0
        const[:, 3:] *= mag
        rows += [const, const[:, ::-1].copy(), base * mag]
    u = np.ascontiguousarray(np.vstack(rows))
    scale = np.abs(u).max(axis=1, keepdims=True)
    for kind in (0, 1):
        got = run_lagrange(hteno_lib, cuda, kind, u)
        want = oracle.lagrange(kind, u)
        assert np.array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        np.testing.assert_array_equal(got[ok], want[ok])
