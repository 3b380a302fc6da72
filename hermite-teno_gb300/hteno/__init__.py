"""Python binding of libhteno (the GB300 Hermite-TENO hot path) over its C-ABI (include/hteno.h).

This is a thin ctypes layer: every call goes through the same extern "C" entry points a C or
C++ host would bind.  Array arguments are numpy arrays (host) or torch CUDA tensors (device).
The library must be built first (`hteno.build.build_library()`); importing this module never
falls back to anything else.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import ic  # noqa: F401  (initial-data generators)

_PKG = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("HTENO_LIB", _PKG / "lib" / "libhteno.so"))

HOST, DEVICE = 0, 1
SCHEME_FV, SCHEME_HERMITE = 0, 1
RECON_TENO5, RECON_TENO5I, RECON_LINEAR = 0, 1, 2
RECON_WENO5JS, RECON_WENO5Z, RECON_WENO5N, RECON_TENO5N, RECON_TENO5A = 3, 4, 5, 6, 7
FLUX_RUSANOV, FLUX_HLLC = 0, 1
BC_ZEROGRAD, BC_PERIODIC, BC_TAYLOR, BC_DOUBLE_MACH = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1

STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
          4: "non-positive density or pressure", 5: "NaN in state", 6: "device wait timed out",
          7: "unsupported configuration"}


class HtenoError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        self.code = code
        super().__init__(f"hteno status {code} ({STATUS.get(code, '?')}){': ' + msg if msg else ''}")


class Config(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int), ("scheme", ctypes.c_int), ("nx", ctypes.c_int),
                ("ny", ctypes.c_int), ("xl", ctypes.c_double), ("xr", ctypes.c_double),
                ("yb", ctypes.c_double), ("yt", ctypes.c_double), ("cfl", ctypes.c_double),
                ("gamma", ctypes.c_double), ("t_init", ctypes.c_double), ("recon", ctypes.c_int),
                ("flux", ctypes.c_int), ("bc", ctypes.c_int), ("precision", ctypes.c_int),
                ("reserved", ctypes.c_int * 8)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_long), ("ms", ctypes.c_double),
                ("bytes_per_launch", ctypes.c_double), ("flops_per_launch", ctypes.c_double)]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)


def lib() -> ctypes.CDLL:
    """Load libhteno.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} is missing: build it with hteno.build.build_library()")
        L = ctypes.CDLL(str(LIB_PATH))
        vp, i, d, l = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_long
        L.hteno_version.restype = ctypes.c_char_p
        L.hteno_last_error.restype = ctypes.c_char_p
        L.hteno_last_error.argtypes = [vp]
        L.hteno_status_string.restype = ctypes.c_char_p
        L.hteno_config_default.argtypes = [ctypes.POINTER(Config)]
        L.hteno_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.hteno_destroy.argtypes = [vp]
        L.hteno_set_stream.argtypes = [vp, vp]
        L.hteno_set_state.argtypes = [vp, vp, i]
        L.hteno_get_state.argtypes = [vp, vp, i]
        L.hteno_set_moments.argtypes = [vp, vp, vp, i]
        L.hteno_get_moments.argtypes = [vp, vp, vp, i]
        L.hteno_step.argtypes = [vp, i, d]
        L.hteno_step_async.argtypes = [vp, i, d]
        L.hteno_sync.argtypes = [vp]
        L.hteno_get_time.argtypes = [vp, _D, ctypes.POINTER(l), _D]
        L.hteno_launches_per_step.argtypes = [vp, ctypes.POINTER(i)]
        L.hteno_residual.argtypes = [vp, vp, vp]
        L.hteno_lagrange_batch.argtypes = [i, i, vp, vp, l, vp]
        L.hteno_gl3_batch.argtypes = [i, vp, vp, l, vp]
        L.hteno_hermite_batch.argtypes = [i, i, d, vp, vp, vp, l, vp]
        L.hteno_hlimiter_batch.argtypes = [i, d, vp, vp, vp, l, vp]
        L.hteno_hllc2d_batch.argtypes = [i, d, i, vp, vp, vp, l, vp]
        L.hteno_hllc1d_batch.argtypes = [i, d, vp, vp, vp, l, vp]
        L.hteno_rusanov2d_batch.argtypes = [i, d, i, vp, vp, vp, vp, vp, l, vp]
        L.hteno_drusanov2d_batch.argtypes = [i, d, i, vp, vp, vp, vp, vp, vp, vp, l, vp]
        L.hteno_ssprk3_batch.argtypes = [vp, vp, vp, d, i, vp, l, vp]
        L.hteno_enable_kernel_timing.argtypes = [vp, i]
        L.hteno_kernel_timing.argtypes = [vp, ctypes.POINTER(KernelTime), i, ctypes.POINTER(i)]
        L.hteno_measure_fma_peak.argtypes = [i, _D]
        L.hteno_get_status.argtypes = [vp, ctypes.POINTER(i)]
        L.hteno_set_strict.argtypes = [vp, i]
        L.hteno_set_fp64_fused.argtypes = [vp, i]
        L.hteno_get_counters.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.hteno_residual_noalloc.argtypes = [ctypes.POINTER(Config), vp, vp, vp]
        L.hteno_batch_create.argtypes = [ctypes.POINTER(Config), i, ctypes.POINTER(vp)]
        L.hteno_batch_destroy.argtypes = [vp]
        L.hteno_batch_size.argtypes = [vp, ctypes.POINTER(i)]
        L.hteno_batch_set_stream.argtypes = [vp, vp]
        L.hteno_batch_set_state.argtypes = [vp, i, vp, i]
        L.hteno_batch_get_state.argtypes = [vp, i, vp, i]
        L.hteno_batch_step.argtypes = [vp, i, d]
        L.hteno_batch_step_async.argtypes = [vp, i, d]
        L.hteno_batch_sync.argtypes = [vp]
        L.hteno_batch_get_time.argtypes = [vp, i, _D, ctypes.POINTER(l), ctypes.POINTER(i)]
        L.hteno_batch_tile.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i)]
        L.hteno_batch_get_counters.argtypes = [vp, i, ctypes.POINTER(ctypes.c_longlong)]
        L.hteno_batch_last_error.restype = ctypes.c_char_p
        L.hteno_batch_last_error.argtypes = [vp]
        L.hteno_set_router.argtypes = [vp, vp, ctypes.c_float, i]
        L.hteno_router_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.hteno_set_router_schedule.argtypes = [vp, i, i]
        L.hteno_router_audit64.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.hteno_kxrcf.argtypes = [vp, vp]
        L.hteno_harvest.argtypes = [vp, d, ctypes.c_ulonglong, vp, vp, l, ctypes.POINTER(l)]
        L.hteno_mlp_create.argtypes = [ctypes.c_ulonglong, ctypes.POINTER(vp)]
        L.hteno_mlp_destroy.argtypes = [vp]
        L.hteno_mlp_set_params.argtypes = [vp, vp]
        L.hteno_mlp_get_params.argtypes = [vp, vp]
        L.hteno_mlp_grad.argtypes = [vp, vp, vp, l, vp, vp]
        L.hteno_mlp_train.argtypes = [vp, vp, vp, l, i, l, ctypes.c_float, vp]
        L.hteno_mlp_predict.argtypes = [vp, vp, l, vp]
        L.hteno_mlp_pack.argtypes = [vp, vp, vp, l]
        L.hteno_mlp_set_wait_limit.argtypes = [vp, ctypes.c_uint]
        L.hteno_mlp_last_error.restype = ctypes.c_char_p
        L.hteno_mlp_last_error.argtypes = [vp]
        _lib = L
    return _lib


def _ptr(a):
    """Host numpy array -> (pointer, HOST); torch CUDA tensor -> (pointer, DEVICE)."""
    if isinstance(a, np.ndarray):
        assert a.dtype == np.float64 and a.flags.c_contiguous
        return ctypes.c_void_p(a.ctypes.data), HOST
    if hasattr(a, "data_ptr"):
        assert str(a.dtype) == "torch.float64" and a.is_contiguous()
        return ctypes.c_void_p(a.data_ptr()), (DEVICE if a.is_cuda else HOST)
    raise TypeError(type(a))


def _check(rc: int, handle=None) -> None:
    if rc != 0:
        msg = lib().hteno_last_error(handle).decode() if handle else ""
        raise HtenoError(rc, msg)


def config(**kw) -> Config:
    c = Config()
    lib().hteno_config_default(ctypes.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


class Solver:
    """Owner of one hteno_solver handle (mirrors FV::System2D & co.: ctor, IC, timeStepping)."""

    def __init__(self, cfg: Config | None = None, **kw):
        self.cfg = cfg if cfg is not None else config(**kw)
        h = ctypes.c_void_p()
        _check(lib().hteno_create(ctypes.byref(self.cfg), ctypes.byref(h)))
        self.h = h
        self.nvar = 4 if self.cfg.dims == 2 else 3
        self.shape = (self.nvar, self.cfg.ny, self.cfg.nx) if self.cfg.dims == 2 else (self.nvar, self.cfg.nx)

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().hteno_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, q) -> None:
        p, where = _ptr(q)
        _check(lib().hteno_set_state(self.h, p, where), self.h)

    def set_moments(self, v, w=None) -> None:
        pv, where = _ptr(v)
        pw = _ptr(w)[0] if w is not None else ctypes.c_void_p()
        _check(lib().hteno_set_moments(self.h, pv, pw, where), self.h)

    def get_state(self, out=None):
        out = np.empty(self.shape) if out is None else out
        p, where = _ptr(out)
        _check(lib().hteno_get_state(self.h, p, where), self.h)
        return out

    def get_moments(self):
        v = np.empty(self.shape)
        w = np.empty(self.shape) if self.cfg.dims == 2 else None
        _check(lib().hteno_get_moments(self.h, _ptr(v)[0], _ptr(w)[0] if w is not None else None, HOST), self.h)
        return (v, w) if w is not None else v

    def step(self, nsteps: int, t_final: float = float("inf")) -> None:
        _check(lib().hteno_step(self.h, int(nsteps), float(t_final)), self.h)

    def step_async(self, nsteps: int, t_final: float = float("inf")) -> None:
        _check(lib().hteno_step_async(self.h, int(nsteps), float(t_final)), self.h)

    def sync(self) -> None:
        _check(lib().hteno_sync(self.h), self.h)

    def time(self):
        t, n, dt = ctypes.c_double(), ctypes.c_long(), ctypes.c_double()
        _check(lib().hteno_get_time(self.h, ctypes.byref(t), ctypes.byref(n), ctypes.byref(dt)), self.h)
        return t.value, n.value, dt.value

    def status(self) -> int:
        """Sticky health flags: bit 0 NaN seen, bit 1 non-positive density/pressure seen."""
        f = ctypes.c_int()
        _check(lib().hteno_get_status(self.h, ctypes.byref(f)), self.h)
        return f.value

    def counters(self) -> dict:
        """Work counters since set_state (FV 2D): cell-stages whose exactly zero residual was taken
        without computing their faces, and mixed-path tiles staged by a TMA box copy."""
        a = (ctypes.c_longlong * 2)()
        _check(lib().hteno_get_counters(self.h, a), self.h)
        return {"uniform_cells": a[0], "tma_tiles": a[1]}

    def uniform_cells(self) -> int:
        return self.counters()["uniform_cells"]

    def set_strict(self, on: bool = True) -> None:
        _check(lib().hteno_set_strict(self.h, int(bool(on))), self.h)

    def set_fp64_fused(self, on: bool = True) -> None:
        """Plain FP64 FV 2D stepping as one fused launch per stage (the same bits)."""
        _check(lib().hteno_set_fp64_fused(self.h, int(bool(on))), self.h)

    def launches_per_step(self) -> int:
        n = ctypes.c_int()
        _check(lib().hteno_launches_per_step(self.h, ctypes.byref(n)), self.h)
        return n.value

    def set_stream(self, stream_ptr: int) -> None:
        _check(lib().hteno_set_stream(self.h, ctypes.c_void_p(stream_ptr)), self.h)

    def kxrcf(self, flags) -> None:
        """KXRCF troubled-cell flags (FV 1D) into the CUDA uint8 tensor `flags` [nx]."""
        _check(lib().hteno_kxrcf(self.h, flags.data_ptr()), self.h)

    def harvest(self, keep: float, seed: int, x, y) -> int:
        """Training rows of the learned classifier from the current state into the CUDA tensors
        x (int16 [cap, 8], BF16 bits) and y (uint8 [cap]); returns the number offered."""
        n = ctypes.c_long()
        _check(lib().hteno_harvest(self.h, float(keep), int(seed), x.data_ptr(), y.data_ptr(),
                                   x.shape[0], ctypes.byref(n)), self.h)
        return n.value

    def set_router(self, mlp, threshold: float = 0.9, audit_every: int = 0) -> None:
        """Learned routing (mixed FV 2D): stencils the classifier marks confidently smooth take
        the linear weights; `mlp` None switches it off.  Keep `mlp` alive meanwhile."""
        self._router = mlp
        _check(lib().hteno_set_router(self.h, mlp.h if mlp is not None else None, float(threshold),
                                      int(audit_every)), self.h)

    def set_router_schedule(self, classify_every: int = 1, margin: int = 0) -> None:
        """Classify every `classify_every` steps; keep a route bit only where it is set on every
        face within `margin` faces (call after set_router)."""
        _check(lib().hteno_set_router_schedule(self.h, int(classify_every), int(margin)), self.h)

    def router_audit64(self) -> dict:
        """Classify the current state and count the routed stencils whose plain FP64 TENO cut-off
        (on the double state) would drop a candidate."""
        a = (ctypes.c_longlong * 4)()
        _check(lib().hteno_router_audit64(self.h, a), self.h)
        return {"routed": a[0], "misrouted64": a[1], "routed_resolved": a[2], "misrouted64_resolved": a[3]}

    def router_stats(self) -> dict:
        a = (ctypes.c_longlong * 7)()
        _check(lib().hteno_router_stats(self.h, a), self.h)
        return {"seen": a[0], "routed": a[1], "misrouted": a[2], "smooth": a[3], "flat": a[4],
                "audits": a[5], "network_rows": a[6]}

    def residual(self, q_dev, rhs_dev) -> None:
        _check(lib().hteno_residual(self.h, _ptr(q_dev)[0], _ptr(rhs_dev)[0]), self.h)


class Batch:
    """Owner of one hteno_batch handle: independent mixed-precision FV 2D grids stepped together."""

    def __init__(self, cfgs):
        arr = (Config * len(cfgs))(*cfgs)
        h = ctypes.c_void_p()
        rc = lib().hteno_batch_create(arr, len(cfgs), ctypes.byref(h))
        if rc != 0:
            raise HtenoError(rc, "batch create")
        self.h = h
        self.shapes = [(4, c.ny, c.nx) for c in cfgs]

    def _check(self, rc):
        if rc != 0:
            raise HtenoError(rc, lib().hteno_batch_last_error(self.h).decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().hteno_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        return len(self.shapes)

    def set_stream(self, stream_ptr: int) -> None:
        self._check(lib().hteno_batch_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def set_state(self, i: int, q) -> None:
        p, where = _ptr(q)
        self._check(lib().hteno_batch_set_state(self.h, i, p, where))

    def get_state(self, i: int, out=None):
        out = np.empty(self.shapes[i]) if out is None else out
        p, where = _ptr(out)
        self._check(lib().hteno_batch_get_state(self.h, i, p, where))
        return out

    def step(self, nsteps: int, t_final: float = float("inf")) -> None:
        self._check(lib().hteno_batch_step(self.h, int(nsteps), float(t_final)))

    def step_async(self, nsteps: int, t_final: float = float("inf")) -> None:
        self._check(lib().hteno_batch_step_async(self.h, int(nsteps), float(t_final)))

    def sync(self) -> None:
        self._check(lib().hteno_batch_sync(self.h))

    def time(self, i: int):
        t, n, st = ctypes.c_double(), ctypes.c_long(), ctypes.c_int()
        self._check(lib().hteno_batch_get_time(self.h, i, ctypes.byref(t), ctypes.byref(n), ctypes.byref(st)))
        return t.value, n.value, st.value

    def counters(self, i: int) -> dict:
        a = (ctypes.c_longlong * 2)()
        self._check(lib().hteno_batch_get_counters(self.h, i, a))
        return {"uniform_cells": a[0], "tma_tiles": a[1]}

    def tile(self):
        tx, ty, nt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(lib().hteno_batch_tile(self.h, ctypes.byref(tx), ctypes.byref(ty), ctypes.byref(nt)))
        return tx.value, ty.value, nt.value


class Mlp:
    """The learned stencil classifier (6 -> 32 -> 32 -> 3, BF16 on the tensor cores).  Inputs and
    labels are CUDA tensors (torch): x uint16/int16 [n, 8] BF16 bits, y uint8 [n]."""

    def __init__(self, seed: int = 0):
        h = ctypes.c_void_p()
        rc = lib().hteno_mlp_create(seed, ctypes.byref(h))
        if rc != 0:
            raise HtenoError(rc, "mlp create")
        self.h = h
        self.nparams = lib().hteno_mlp_num_params()

    def _check(self, rc):
        if rc != 0:
            raise HtenoError(rc, lib().hteno_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().hteno_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        self._check(lib().hteno_mlp_get_params(self.h, out.ctypes.data))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self._check(lib().hteno_mlp_set_params(self.h, p.ctypes.data))

    def grad(self, x, y):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = ctypes.c_float()
        self._check(lib().hteno_mlp_grad(self.h, x.data_ptr(), y.data_ptr(), x.shape[0], g.ctypes.data,
                                         ctypes.byref(loss)))
        return g, loss.value

    def train(self, x, y, epochs: int, batch: int, lr: float) -> float:
        loss = ctypes.c_float()
        self._check(lib().hteno_mlp_train(self.h, x.data_ptr(), y.data_ptr(), x.shape[0], epochs, batch,
                                          ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value

    def predict(self, x, out):
        self._check(lib().hteno_mlp_predict(self.h, x.data_ptr(), x.shape[0], out.data_ptr()))
        return out

    def set_wait_limit(self, polls: int) -> None:
        """Polls of each tensor-core completion wait before a call reports a timeout (test hook)."""
        self._check(lib().hteno_mlp_set_wait_limit(self.h, int(polls)))

    def pack(self, xf, out):
        self._check(lib().hteno_mlp_pack(self.h, xf.data_ptr(), out.data_ptr(), xf.shape[0]))
        return out


def measure_fma_peak(kind: int) -> float:
    """Measured FMA throughput of the current device in TFLOP/s (kind 0 FP64, 1 FP32)."""
    out = ctypes.c_double()
    _check(lib().hteno_measure_fma_peak(kind, ctypes.byref(out)))
    return out.value


def version() -> str:
    return lib().hteno_version().decode()
