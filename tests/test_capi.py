"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every symbol that
include/hteno.h declares, and rejects invalid configurations before touching the device."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((REPO / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(hteno_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("hteno_create", "hteno_step", "hteno_set_state", "hteno_get_state",
                 "hteno_lagrange_batch", "hteno_gl3_batch", "hteno_hllc2d_batch"):
        assert must in names


def test_library_exports_every_declared_symbol(hteno_lib):
    lib = hteno_lib.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_invalid_configs_rejected_without_device(hteno_lib):
    h = hteno_lib
    bad = [dict(nx=3), dict(dims=3), dict(cfl=0.0), dict(gamma=1.0), dict(recon=9), dict(xr=-1.0),
           dict(flux=5), dict(bc=4), dict(precision=7), dict(scheme=3)]
    for kw in bad:
        cfg = h.config(**kw)
        handle = ctypes.c_void_p()
        rc = h.lib().hteno_create(ctypes.byref(cfg), ctypes.byref(handle))
        assert rc == 1, (kw, rc)  # HTENO_ERR_INVALID_ARG
        assert not handle.value


def test_boundary_routines_limited_to_fv2d(hteno_lib):
    """TaylorInstBc / doubleMachBc exist for FV::System2D only, and read interior cells 6 away
    from the walls."""
    h = hteno_lib
    for kw, want in ((dict(bc=h.BC_TAYLOR, dims=1), 7), (dict(bc=h.BC_DOUBLE_MACH, scheme=h.SCHEME_HERMITE), 7),
                     (dict(bc=h.BC_DOUBLE_MACH, nx=6), 1), (dict(bc=h.BC_TAYLOR, ny=6), 1)):
        cfg = h.config(**kw)
        handle = ctypes.c_void_p()
        assert h.lib().hteno_create(ctypes.byref(cfg), ctypes.byref(handle)) == want, kw
        assert not handle.value


def test_batch_entry_points_validate_arguments(hteno_lib):
    lib = hteno_lib.lib()
    # negative counts and bad directions are rejected before any launch
    assert lib.hteno_lagrange_batch(0, 0, None, None, -1, None) == 1
    assert lib.hteno_hllc2d_batch(0, 1.4, 3, None, None, None, 10, None) == 1
    assert lib.hteno_ssprk3_batch(None, None, None, 0.1, 4, None, 10, None) == 1
    # n == 0 is a no-op
    assert lib.hteno_gl3_batch(0, None, None, 0, None) == 0


def test_status_strings(hteno_lib):
    lib = hteno_lib.lib()
    assert lib.hteno_status_string(5).decode() == "NaN in state"
    assert "sm_103a" in hteno_lib.version()


def test_initial_data_generators():
    from hteno import ic

    q = ic.four_quadrant(32, 16, 7)
    assert q.shape == (4, 16, 32)
    np.testing.assert_array_equal(q, ic.four_quadrant(32, 16, 7))
    assert not np.array_equal(q, ic.four_quadrant(32, 16, 8))
    rho, p = q[0], 0.4 * (q[3] - 0.5 * (q[1] ** 2 + q[2] ** 2) / q[0])
    assert rho.min() >= 0.1 and rho.max() <= 1.5 and p.min() >= 0.03 - 1e-12
    assert len(np.unique(rho)) == 4  # four constant quadrants
    s = ic.sod(10)
    assert s.shape == (3, 10) and s[0, 0] == 1.0 and s[0, -1] == 0.125
    b = ic.gaussian_blobs_shock(64, 64, 1)
    assert b.shape == (4, 64, 64) and b[0].max() > 2.0


def test_batch_rejects_unsupported_configs(hteno_lib):
    """Batches hold mixed-precision FV 2D grids only; configs are checked before any device work."""
    h = hteno_lib
    with pytest.raises(h.HtenoError):
        h.Batch([h.config(dims=2, nx=32, ny=32, precision=0)])
    with pytest.raises(h.HtenoError):
        h.Batch([h.config(dims=2, nx=4, ny=32, precision=1)])
    with pytest.raises(h.HtenoError):
        h.Batch([h.config(dims=1, nx=32, precision=1)])
