"""The allocation-free residual entry point (hteno_residual_noalloc), for callers that cannot
call cudaMalloc: code inside another framework's stream capture or memory pool, or hosts whose
device footprint must stay fixed once running.  It must give the same residual as the
handle-based hteno_residual (which allocates its work buffers), call after call, while using its
fixed in-library scratch array.  Collected last so that a run stopping at the first failure has
already run every other test."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12  # the tolerance of the FP64 parity tests


def residual_with_handle(h, cuda, q, cfg):
    with h.Solver(cfg) as s:
        dq = cuda.from_numpy(q).cuda()
        out = cuda.empty_like(dq)
        s.residual(dq, out)
        cuda.cuda.synchronize()
        return out.cpu().numpy()


def test_residual_noalloc_matches_handle_residual(hteno_lib, cuda):
    from hteno import ic

    lib = hteno_lib.lib()
    stream = cuda.cuda.current_stream()
    # two calls in a row on different grids and states (the scratch keeps the previous contents)
    for seed, (nx, ny), flux in ((1, (96, 80), 1), (2, (128, 128), 0)):
        q = ic.four_quadrant(nx, ny, seed)
        cfg = hteno_lib.config(dims=2, nx=nx, ny=ny, flux=flux)
        want = residual_with_handle(hteno_lib, cuda, q, cfg)
        dq = cuda.from_numpy(q).cuda()
        got = cuda.full_like(dq, float("nan"))
        rc = lib.hteno_residual_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dq.data_ptr()),
                                        ctypes.c_void_p(got.data_ptr()),
                                        ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        stream.synchronize()
        got = got.cpu().numpy()
        scale = np.abs(want).max(axis=(1, 2), keepdims=True)
        assert (np.abs(got - want) / scale).max() <= TOL
        np.testing.assert_array_equal(got, want)


def test_residual_noalloc_rejects_oversize_grid(hteno_lib, cuda):
    lib = hteno_lib.lib()
    cfg = hteno_lib.config(dims=2, nx=200, ny=200)  # 40000 cells > HTENO_NOALLOC_MAX_CELLS
    dq = cuda.zeros((4, 200, 200), dtype=cuda.float64, device="cuda")
    rc = lib.hteno_residual_noalloc(ctypes.byref(cfg), ctypes.c_void_p(dq.data_ptr()),
                                    ctypes.c_void_p(dq.data_ptr()), None)
    assert rc == 1  # HTENO_ERR_INVALID_ARG
