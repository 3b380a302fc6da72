"""The allocation-free residual entry point (hteno_residual_noalloc), for callers that cannot
call cudaMalloc: code inside another framework's stream capture or memory pool, or hosts whose
device footprint must stay fixed once running.  It must give the same residual as the
handle-based hteno_residual (which allocates its work buffers) and as the CPU oracle, call after
call, while using its fixed in-library scratch array and allocating nothing.  Collected last so
that a run stopping at the first failure has already run every other test."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the tolerance of the FP64 parity tests

# (seed, (nx, ny), flux, recon, bc): two calls in a row on different grids and states (the
# scratch keeps the previous call's contents), a WENO-JS reconstruction and a periodic grid
CASES = [
    (1, (96, 80), 1, 0, 0),
    (2, (128, 128), 0, 0, 0),
    (3, (72, 40), 1, 3, 0),
    (4, (64, 48), 0, 1, 1),
]


def residual_with_handle(h, cuda, q, cfg):
    with h.Solver(cfg) as s:
        dq = cuda.from_numpy(q).cuda()
        out = cuda.empty_like(dq)
        s.residual(dq, out)
        cuda.cuda.synchronize()
        return out.cpu().numpy()


def noalloc(lib, cuda, cfg, dq, out, stream):
    rc = lib.hteno_residual_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dq.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    return rc


def test_residual_noalloc_matches_handle_residual_and_oracle(hteno_lib, cuda, oracle):
    from hteno import ic

    lib = hteno_lib.lib()
    stream = cuda.cuda.current_stream()
    inputs = []
    for seed, (nx, ny), flux, recon, bc in CASES:
        q = ic.four_quadrant(nx, ny, seed)
        cfg = hteno_lib.config(dims=2, nx=nx, ny=ny, flux=flux, recon=recon, bc=bc)
        want = residual_with_handle(hteno_lib, cuda, q, cfg)
        ref = oracle.fv2d_rhs(q, flux=flux, recon=recon, bc=bc)
        dq = cuda.from_numpy(q).cuda()
        got = cuda.full_like(dq, float("nan"))
        inputs.append((cfg, dq, got, want, ref))
    # the first call on this device sets up the scratch address; every later call must leave
    # the device's free memory unchanged
    cfg, dq, got, _, _ = inputs[0]
    assert noalloc(lib, cuda, cfg, dq, got, stream) == 0
    free0 = cuda.cuda.mem_get_info()[0]
    for cfg, dq, got, want, ref in inputs:
        got.fill_(float("nan"))
        assert noalloc(lib, cuda, cfg, dq, got, stream) == 0
        g = got.cpu().numpy()
        scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
        assert (np.abs(g - ref) / scale).max() <= TOL  # against the CPU oracle
        np.testing.assert_array_equal(g, want)          # the handle path, bit for bit
    assert cuda.cuda.mem_get_info()[0] == free0


def test_residual_noalloc_rejects_oversize_grid(hteno_lib, cuda):
    lib = hteno_lib.lib()
    cfg = hteno_lib.config(dims=2, nx=200, ny=200)  # 40000 cells > HTENO_NOALLOC_MAX_CELLS
    dq = cuda.zeros((4, 200, 200), dtype=cuda.float64, device="cuda")
    rc = lib.hteno_residual_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dq.data_ptr()),
                                    ctypes.c_void_p(dq.data_ptr()), None)
    assert rc == 1  # HTENO_ERR_INVALID_ARG


def test_residual_noalloc_reports_unsupported_boundaries(hteno_lib, cuda):
    lib = hteno_lib.lib()
    dq = cuda.zeros((4, 32, 32), dtype=cuda.float64, device="cuda")
    for bc in (2, 3):  # Taylor, double Mach: their ghost face rows do not fit the fixed array
        cfg = hteno_lib.config(dims=2, nx=32, ny=32, bc=bc)
        rc = lib.hteno_residual_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dq.data_ptr()),
                                        ctypes.c_void_p(dq.data_ptr()), None)
        assert rc == 7  # HTENO_ERR_UNSUPPORTED
