"""ctypes wrapper of the CPU oracle (oracle/build/liboracle.so) -- test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.  The
oracle restates the reference solver (see oracle.hpp); it is never part of the GPU library.
Array layouts match include/hteno.h.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libhteno_ref.so"

_D = ctypes.POINTER(ctypes.c_double)
_lib = None


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE), "oracle"], check=True)
        _lib = ctypes.CDLL(str(LIB))
        d, i, l = ctypes.c_double, ctypes.c_int, ctypes.c_long
        _lib.orc_fv2d_run.restype = i
        _lib.orc_fv1d_run.restype = i
        _lib.orc_hermite2d_run.restype = i
        _lib.orc_hermite1d_run.restype = i
    return _lib


def _c(x):
    return ctypes.c_double(float(x))


def lagrange(kind: int, u: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty((u.shape[0], 2))
    lib().orc_lagrange_recon(kind, _p(u), _p(out), ctypes.c_long(u.shape[0]))
    return out


def gl3(u: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.empty((u.shape[0], 3))
    lib().orc_gl3(_p(u), _p(out), ctypes.c_long(u.shape[0]))
    return out


def hermite(kind: int, dx: float, u: np.ndarray, d: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.empty((u.shape[0], 4))
    lib().orc_hermite_recon(kind, _c(dx), _p(u), _p(d), _p(out), ctypes.c_long(u.shape[0]))
    return out


def hlimiter(dx: float, u: np.ndarray, d: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(u, dtype=np.float64)
    d = np.ascontiguousarray(d, dtype=np.float64)
    out = np.empty(u.shape[0])
    lib().orc_hermite_limiter(_c(dx), _p(u), _p(d), _p(out), ctypes.c_long(u.shape[0]))
    return out


def ssprk3(q0, qn, rhs, dt, stage) -> np.ndarray:
    out = np.empty_like(q0)
    lib().orc_ssprk3(_p(q0), _p(qn), _p(rhs), _c(dt), stage, _p(out), ctypes.c_long(q0.size))
    return out


def hllc2d(gamma, direction, ql, qr) -> np.ndarray:
    out = np.empty_like(ql)
    lib().orc_hllc2d(_c(gamma), direction, _p(ql), _p(qr), _p(out), ctypes.c_long(ql.shape[0]))
    return out


def hllc1d(gamma, ql, qr) -> np.ndarray:
    out = np.empty_like(ql)
    lib().orc_hllc1d(_c(gamma), _p(ql), _p(qr), _p(out), ctypes.c_long(ql.shape[0]))
    return out


def roe2d(gamma, direction, qa, qb):
    n = qa.shape[0]
    R = np.empty((n, 16))
    L = np.empty((n, 16))
    lib().orc_roe2d(_c(gamma), direction, _p(qa), _p(qb), _p(R), _p(L), ctypes.c_long(n))
    return R, L


def rusanov2d(gamma, direction, qa, qb, ql, qr) -> np.ndarray:
    R, L = roe2d(gamma, direction, qa, qb)
    out = np.empty_like(ql)
    lib().orc_rusanov2d(_c(gamma), direction, _p(ql), _p(qr), _p(L), _p(R), _p(out),
                        ctypes.c_long(ql.shape[0]))
    return out


def drusanov2d(gamma, direction, qa, qb, ql, qr, dql, dqr) -> np.ndarray:
    R, L = roe2d(gamma, direction, qa, qb)
    out = np.empty_like(ql)
    lib().orc_drusanov2d(_c(gamma), direction, _p(ql), _p(qr), _p(dql), _p(dqr), _p(L), _p(R),
                         _p(out), ctypes.c_long(ql.shape[0]))
    return out


def fv2d_run(q, nsteps, t_final=1e30, xl=0.0, xr=1.0, yb=0.0, yt=1.0, cfl=0.4, gamma=1.4,
             bc=0, flux=0, recon=0):
    q = np.ascontiguousarray(q, dtype=np.float64)
    ny, nx = q.shape[1], q.shape[2]
    out = np.empty_like(q)
    t = ctypes.c_double()
    n = lib().orc_fv2d_run(nx, ny, _c(xl), _c(xr), _c(yb), _c(yt), _c(cfl), _c(gamma), bc, flux,
                           recon, _c(t_final), int(nsteps), _p(q), _p(out), ctypes.byref(t))
    return out, t.value, n


def fv2d_rhs(q, xl=0.0, xr=1.0, yb=0.0, yt=1.0, gamma=1.4, bc=0, flux=0, recon=0):
    q = np.ascontiguousarray(q, dtype=np.float64)
    ny, nx = q.shape[1], q.shape[2]
    out = np.empty_like(q)
    lib().orc_fv2d_rhs(nx, ny, _c(xl), _c(xr), _c(yb), _c(yt), _c(gamma), bc, flux, recon,
                       _p(q), _p(out))
    return out


def fv1d_run(q, nsteps, t_final=1e30, xl=0.0, xr=1.0, cfl=0.5, gamma=1.4, bc=0, flux=0, recon=1):
    q = np.ascontiguousarray(q, dtype=np.float64)
    nx = q.shape[1]
    out = np.empty_like(q)
    t = ctypes.c_double()
    n = lib().orc_fv1d_run(nx, _c(xl), _c(xr), _c(cfl), _c(gamma), bc, flux, recon, _c(t_final),
                           int(nsteps), _p(q), _p(out), ctypes.byref(t))
    return out, t.value, n


def hermite2d_run(q, v, w, nsteps, t_final=1e30, xl=0.0, xr=1.0, yb=0.0, yt=1.0, cfl=0.4,
                  gamma=1.4, bc=0):
    q, v, w = (np.ascontiguousarray(a, dtype=np.float64) for a in (q, v, w))
    ny, nx = q.shape[1], q.shape[2]
    qo, vo, wo = np.empty_like(q), np.empty_like(q), np.empty_like(q)
    t = ctypes.c_double()
    n = lib().orc_hermite2d_run(nx, ny, _c(xl), _c(xr), _c(yb), _c(yt), _c(cfl), _c(gamma), bc,
                                _c(t_final), int(nsteps), _p(q), _p(v), _p(w), _p(qo), _p(vo),
                                _p(wo), ctypes.byref(t))
    return qo, vo, wo, t.value, n


def hermite1d_run(q, v, nsteps, t_final=1e30, xl=0.0, xr=1.0, cfl=0.4, gamma=1.4):
    q, v = (np.ascontiguousarray(a, dtype=np.float64) for a in (q, v))
    nx = q.shape[1]
    qo, vo = np.empty_like(q), np.empty_like(q)
    t = ctypes.c_double()
    n = lib().orc_hermite1d_run(nx, _c(xl), _c(xr), _c(cfl), _c(gamma), _c(t_final), int(nsteps),
                                _p(q), _p(v), _p(qo), _p(vo), ctypes.byref(t))
    return qo, vo, t.value, n
