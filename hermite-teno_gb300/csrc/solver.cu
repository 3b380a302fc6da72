// Solver handles and the C-ABI around the scheme back ends (include/hteno.h).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "hteno_internal.h"

namespace hteno {

int set_error(hteno_solver* s, int code, const char* fmt, ...) {
  if (s) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    s->err = buf;
  }
  return code;
}

int cuda_error(hteno_solver* s, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HTENO_OK;
  return set_error(s, e == cudaErrorMemoryAllocation ? HTENO_ERR_OOM : HTENO_ERR_CUDA,
                   "%s: %s", what, cudaGetErrorString(e));
}

int trace_kind(hteno_solver* s, const char* name, double bytes, double flops) {
  for (size_t k = 0; k < s->kinds.size(); ++k)
    if (s->kinds[k].name == name) {
      s->kinds[k].bytes = bytes;
      s->kinds[k].flops = flops;
      return int(k);
    }
  hteno_solver::TraceKind t;
  t.name = name;
  t.bytes = bytes;
  t.flops = flops;
  s->kinds.push_back(t);
  return int(s->kinds.size() - 1);
}

void trace_begin(hteno_solver* s, int kind) {
  if (!s->timing) return;
  if (s->ev_used * 2 + 2 > s->ev.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return;
    s->ev.push_back(a);
    s->ev.push_back(b);
    s->ev_kind.push_back(kind);
  }
  s->ev_kind[s->ev_used] = kind;
  cudaEventRecord(s->ev[2 * s->ev_used], s->stream);
}

void trace_end(hteno_solver* s) {
  if (!s->timing || s->ev_used * 2 + 2 > s->ev.size()) return;
  cudaEventRecord(s->ev[2 * s->ev_used + 1], s->stream);
  ++s->ev_used;
}

namespace {

bool is_hermite(const hteno_solver* s) { return s->cfg.scheme == HTENO_SCHEME_HERMITE; }

int backend_setup(hteno_solver* s) {
  if (s->cfg.dims == 2) return is_hermite(s) ? hermite2d_setup(s) : fv2d_setup(s);
  return is_hermite(s) ? hermite1d_setup(s) : fv1d_setup(s);
}
int backend_prepare(hteno_solver* s) {
  if (s->cfg.dims == 2) return is_hermite(s) ? hermite2d_prepare(s) : fv2d_prepare(s);
  return is_hermite(s) ? hermite1d_prepare(s) : fv1d_prepare(s);
}
int backend_step(hteno_solver* s, int n) {
  if (s->cfg.dims == 2) return is_hermite(s) ? hermite2d_step_async(s, n) : fv2d_step_async(s, n);
  return is_hermite(s) ? hermite1d_step_async(s, n) : fv1d_step_async(s, n);
}

__global__ void k_set_target(StepState* st, double t_final) {
  st->t_final = t_final;
  st->done = 0;
}

int copy_in(hteno_solver* s, double* dst, const double* src, size_t n, int where) {
  if (!src) return set_error(s, HTENO_ERR_INVALID_ARG, "null input pointer");
  cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(double),
                                  where == HTENO_DEVICE ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyHostToDevice,
                                  s->stream);
  return cuda_error(s, e, "state copy in");
}
int copy_out(hteno_solver* s, double* dst, const double* src, size_t n, int where) {
  if (!dst) return set_error(s, HTENO_ERR_INVALID_ARG, "null output pointer");
  cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(double),
                                  where == HTENO_DEVICE ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyDeviceToHost,
                                  s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  return cuda_error(s, e, "state copy out");
}

void release(hteno_solver* s) {
  cudaFree(s->route_x);
  cudaFree(s->route_y);
  cudaFree(s->route_tmp);
  cudaFree(s->audit);
  cudaFree(s->route_rows);
  cudaFree(s->deep);
  cudaFree(s->ghost_faces);
  cudaFree(s->fused64);
  cudaFree(s->q);
  cudaFree(s->q0);
  cudaFree(s->v);
  cudaFree(s->v0);
  cudaFree(s->w);
  cudaFree(s->w0);
  cudaFree(s->work);
  cudaFree(s->dstate);
  if (s->hstate) cudaFreeHost(s->hstate);
  for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
  if (s->fork_ev) cudaEventDestroy(s->fork_ev);
  if (s->join_ev) cudaEventDestroy(s->join_ev);
  if (s->side_stream) cudaStreamDestroy(s->side_stream);
  if (s->step_graph) cudaGraphExecDestroy(s->step_graph);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
}

}  // namespace

int make_side_stream(hteno_solver* s) {
  if (!s->side || s->side_stream) return HTENO_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&s->side_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming);
  return e == cudaSuccess ? HTENO_OK : cuda_error(s, e, "side stream");
}
}  // namespace hteno

using namespace hteno;

extern "C" {

const char* hteno_version(void) { return "hteno-gb300 1.0 (sm_103a)"; }

const char* hteno_status_string(int st) {
  switch (st) {
    case HTENO_OK: return "ok";
    case HTENO_ERR_INVALID_ARG: return "invalid argument";
    case HTENO_ERR_OOM: return "out of device memory";
    case HTENO_ERR_CUDA: return "CUDA error";
    case HTENO_ERR_NONPHYSICAL: return "non-positive density or pressure";
    case HTENO_ERR_NAN: return "NaN in state";
    case HTENO_ERR_TIMEOUT: return "device wait timed out";
    case HTENO_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown status";
  }
}

void hteno_config_default(hteno_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->dims = 2;
  c->scheme = HTENO_SCHEME_FV;
  c->nx = 64;
  c->ny = 64;
  c->xl = 0.0;
  c->xr = 1.0;
  c->yb = 0.0;
  c->yt = 1.0;
  c->cfl = 0.4;
  c->gamma = 1.4;
  c->t_init = 0.0;
  c->recon = HTENO_RECON_TENO5;
  c->flux = HTENO_FLUX_RUSANOV;
  c->bc = HTENO_BC_ZEROGRAD;
  c->precision = HTENO_PREC_FP64;
}

int hteno_create(const hteno_config* cfg, hteno_solver** out) {
  if (!cfg || !out) return HTENO_ERR_INVALID_ARG;
  *out = nullptr;
  const hteno_config& c = *cfg;
  if (c.dims != 1 && c.dims != 2) return HTENO_ERR_INVALID_ARG;
  if (c.scheme != HTENO_SCHEME_FV && c.scheme != HTENO_SCHEME_HERMITE) return HTENO_ERR_INVALID_ARG;
  if (c.nx < 6 || (c.dims == 2 && c.ny < 6)) return HTENO_ERR_INVALID_ARG;
  if (c.nx > (1 << 16) * 16 || (c.dims == 2 && (long long)c.nx * c.ny > (1ll << 31)))
    return HTENO_ERR_INVALID_ARG;
  if (!(c.xr > c.xl) || (c.dims == 2 && !(c.yt > c.yb))) return HTENO_ERR_INVALID_ARG;
  if (!(c.cfl > 0.0) || !(c.gamma > 1.0)) return HTENO_ERR_INVALID_ARG;
  if (c.bc >= HTENO_BC_TAYLOR && c.bc <= HTENO_BC_DOUBLE_MACH &&
      (c.dims != 2 || c.scheme != HTENO_SCHEME_FV))
    return HTENO_ERR_UNSUPPORTED;  // the reference's other solvers have no such routines wired
  if (c.bc >= HTENO_BC_TAYLOR && (c.nx < 7 || c.ny < 7)) return HTENO_ERR_INVALID_ARG;
  if (c.recon < 0 || c.recon > 7 || c.flux < 0 || c.flux > 1 || c.bc < 0 || c.bc > 3 ||
      c.precision < 0 || c.precision > 1)
    return HTENO_ERR_INVALID_ARG;

  hteno_solver* s = new (std::nothrow) hteno_solver();
  if (!s) return HTENO_ERR_OOM;
  s->cfg = c;
  if (c.dims == 1) s->cfg.ny = 1;
  s->nvar = c.dims == 2 ? 4 : 3;
  s->ncell = size_t(s->cfg.nx) * s->cfg.ny;
  s->dx = (c.xr - c.xl) / c.nx;
  s->dy = c.dims == 2 ? (c.yt - c.yb) / c.ny : 1.0;
  cudaGetDevice(&s->device);
  // HTENO_UNIFORM_SKIP=0 computes uniform regions in full (a check that skipping them is exact)
  const char* us = std::getenv("HTENO_UNIFORM_SKIP");
  s->uniform_skip = !(us && us[0] == '0');
  // HTENO_TMA=0 stages every tile of the mixed FV 2D kernel cell by cell (the same bits)
  const char* tma = std::getenv("HTENO_TMA");
  s->tma = !(tma && tma[0] == '0');
  // HTENO_SIDE_STREAM=0 runs the FV 2D / Hermite 2D y-direction kernels after the x ones on one stream
  const char* side = std::getenv("HTENO_SIDE_STREAM");
  s->side = !(side && side[0] == '0');

  auto fail = [&](int code) {
    release(s);
    delete s;
    return code;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(HTENO_ERR_CUDA);
  s->own_stream = true;
  const size_t bytes = s->ncell * s->nvar * sizeof(double);
  if (cudaMalloc(&s->q, bytes) != cudaSuccess || cudaMalloc(&s->q0, bytes) != cudaSuccess)
    return fail(HTENO_ERR_OOM);
  if (c.scheme == HTENO_SCHEME_HERMITE) {
    if (cudaMalloc(&s->v, bytes) != cudaSuccess || cudaMalloc(&s->v0, bytes) != cudaSuccess)
      return fail(HTENO_ERR_OOM);
    if (c.dims == 2 &&
        (cudaMalloc(&s->w, bytes) != cudaSuccess || cudaMalloc(&s->w0, bytes) != cudaSuccess))
      return fail(HTENO_ERR_OOM);
  }
  if (cudaMalloc(&s->dstate, sizeof(StepState)) != cudaSuccess) return fail(HTENO_ERR_OOM);
  if (cudaMallocHost(&s->hstate, sizeof(StepState)) != cudaSuccess) return fail(HTENO_ERR_OOM);
  std::memset(s->hstate, 0, sizeof(StepState));
  s->hstate->t = c.t_init;
  // dt = cfl * pow(min(dx, dy), 3/3) (FV_System2D.cpp:633) or cfl * pow(dx, 5/3) for the
  // Hermite 1D scheme (FVHermite_System1D.cpp:396)
  if (c.dims == 1 && c.scheme == HTENO_SCHEME_HERMITE)
    s->hstate->dt_scale = c.cfl * std::pow(s->dx, 5.0 / 3.0);
  else if (c.dims == 1)
    s->hstate->dt_scale = c.cfl * std::pow(s->dx, 3.0 / 3.0);
  else
    s->hstate->dt_scale = c.cfl * std::pow(std::fmin(s->dx, s->dy), 3.0 / 3.0);
  if (cudaMemcpy(s->dstate, s->hstate, sizeof(StepState), cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(HTENO_ERR_CUDA);
  const int rc = backend_setup(s);
  if (rc != HTENO_OK) return fail(rc);
  *out = s;
  return HTENO_OK;
}

int hteno_destroy(hteno_solver* s) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  if (s->stream) cudaStreamSynchronize(s->stream);
  release(s);
  delete s;
  return HTENO_OK;
}

int hteno_set_stream(hteno_solver* s, void* stream) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  cudaStreamSynchronize(s->stream);
  if (s->side_stream) cudaStreamSynchronize(s->side_stream);
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->stream = static_cast<cudaStream_t>(stream);
  s->own_stream = false;
  return HTENO_OK;
}

int hteno_set_state(hteno_solver* s, const double* q, int where) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  int rc = copy_in(s, s->q, q, s->ncell * s->nvar, where);
  if (rc) return rc;
  s->hstate->t = s->cfg.t_init;
  s->hstate->dt = 0.0;
  s->hstate->t_final = s->cfg.t_init;
  s->hstate->maxbits = 0ull;
  s->hstate->steps = 0;
  s->hstate->done = 0;
  s->hstate->status = 0;
  s->hstate->uniform = 0;
  s->hstate->tma_tiles = 0;
  cudaError_t e = cudaMemcpyAsync(s->dstate, s->hstate, sizeof(StepState), cudaMemcpyHostToDevice,
                                  s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "state reset");
  rc = backend_prepare(s);
  if (rc) return rc;
  return cuda_error(s, cudaStreamSynchronize(s->stream), "set_state");
}

int hteno_get_state(hteno_solver* s, double* q, int where) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  return copy_out(s, q, s->q, s->ncell * s->nvar, where);
}

int hteno_set_moments(hteno_solver* s, const double* v, const double* w, int where) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  if (!is_hermite(s)) return set_error(s, HTENO_ERR_UNSUPPORTED, "moments need a Hermite scheme");
  int rc = copy_in(s, s->v, v, s->ncell * s->nvar, where);
  if (rc) return rc;
  if (s->cfg.dims == 2) {
    rc = copy_in(s, s->w, w, s->ncell * s->nvar, where);
    if (rc) return rc;
  }
  rc = backend_prepare(s);
  if (rc) return rc;
  return cuda_error(s, cudaStreamSynchronize(s->stream), "set_moments");
}

int hteno_get_moments(hteno_solver* s, double* v, double* w, int where) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  if (!is_hermite(s)) return set_error(s, HTENO_ERR_UNSUPPORTED, "moments need a Hermite scheme");
  int rc = copy_out(s, v, s->v, s->ncell * s->nvar, where);
  if (rc || s->cfg.dims == 1) return rc;
  return copy_out(s, w, s->w, s->ncell * s->nvar, where);
}

int hteno_step_async(hteno_solver* s, int nsteps, double t_final) {
  if (!s || nsteps < 0 || std::isnan(t_final)) return HTENO_ERR_INVALID_ARG;
  if (nsteps == 0) return HTENO_OK;
  k_set_target<<<1, 1, 0, s->stream>>>(s->dstate, t_final);
  int rc = cuda_error(s, cudaGetLastError(), "k_set_target");
  if (rc) return rc;
  return backend_step(s, nsteps);
}

int hteno_sync(hteno_solver* s) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(s->hstate, s->dstate, sizeof(StepState), cudaMemcpyDeviceToHost,
                                  s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "sync");
  if (s->hstate->status & 4)
    return set_error(s, HTENO_ERR_TIMEOUT, "a bounded device-side wait gave up (TMA tile copy)");
  if (s->strict && (s->hstate->status & 1))
    return set_error(s, HTENO_ERR_NAN, "NaN in the conserved state");
  if (s->strict && (s->hstate->status & 2))
    return set_error(s, HTENO_ERR_NONPHYSICAL, "non-positive density or pressure in the state");
  return HTENO_OK;
}

// Synchronous stepping issues the steps in growing chunks and stops issuing once the device
// state shows t >= t_final, so a large step budget (advance to tmax) costs no idle launches.
int hteno_step(hteno_solver* s, int nsteps, double t_final) {
  if (!s || nsteps < 0 || std::isnan(t_final)) return HTENO_ERR_INVALID_ARG;
  int chunk = 32;
  for (int left = nsteps; left > 0;) {
    const int n = left < chunk ? left : chunk;
    int rc = hteno_step_async(s, n, t_final);
    if (rc) return rc;
    rc = hteno_sync(s);
    if (rc) return rc;
    left -= n;
    if (s->hstate->done || !(s->hstate->t < t_final)) break;
    chunk = chunk < 1024 ? chunk * 2 : 1024;
  }
  return HTENO_OK;
}

int hteno_get_time(hteno_solver* s, double* t, long* steps, double* last_dt) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(s->hstate, s->dstate, sizeof(StepState), cudaMemcpyDeviceToHost,
                                  s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "get_time");
  if (t) *t = s->hstate->t;
  if (steps) *steps = static_cast<long>(s->hstate->steps);
  if (last_dt) *last_dt = s->hstate->dt;
  return HTENO_OK;
}

int hteno_get_status(hteno_solver* s, int* flags) {
  if (!s || !flags) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(s->hstate, s->dstate, sizeof(StepState), cudaMemcpyDeviceToHost,
                                  s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "get_status");
  *flags = s->hstate->status;
  return HTENO_OK;
}

int hteno_get_counters(hteno_solver* s, long long* counters) {
  if (!s || !counters) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(s->hstate, s->dstate, sizeof(StepState), cudaMemcpyDeviceToHost,
                                  s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "get_counters");
  counters[0] = static_cast<long long>(s->hstate->uniform);
  counters[1] = static_cast<long long>(s->hstate->tma_tiles);
  return HTENO_OK;
}

int hteno_set_strict(hteno_solver* s, int on) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  s->strict = on != 0;
  return HTENO_OK;
}

int hteno_set_fp64_fused(hteno_solver* s, int on) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  const hteno_config& c = s->cfg;
  if (c.dims != 2 || c.scheme != HTENO_SCHEME_FV || c.precision != HTENO_PREC_FP64 ||
      c.bc > HTENO_BC_PERIODIC)
    return set_error(s, HTENO_ERR_UNSUPPORTED,
                     "fused stages: plain FP64 FV 2D with zero-gradient or periodic boundaries");
  return fv2d_fp64_set_fused(s, on);
}

int hteno_launches_per_step(hteno_solver* s, int* launches) {
  if (!s || !launches) return HTENO_ERR_INVALID_ARG;
  *launches = s->launches_per_step;
  return HTENO_OK;
}

int hteno_harvest(hteno_solver* s, double keep, unsigned long long seed, unsigned short* x,
                  unsigned char* y, long capacity, long* count) {
  if (!s || !x || !y || capacity < 0 || !(keep >= 0.0) || keep > 1.0 || !count)
    return HTENO_ERR_INVALID_ARG;
  if (is_hermite(s) || s->cfg.precision != HTENO_PREC_FP64)
    return set_error(s, HTENO_ERR_UNSUPPORTED, "stencils are recorded by the plain FP64 FV solvers");
  unsigned long long* dcount = nullptr;
  cudaError_t e = cudaMallocAsync(&dcount, sizeof(unsigned long long), s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "harvest counter");
  cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s->stream);
  int rc = s->cfg.dims == 2 ? fv2d_harvest_entry(s, keep, seed, x, y, capacity, dcount)
                            : fv1d_harvest(s, keep, seed, x, y, capacity, dcount);
  unsigned long long h = 0;
  if (rc == HTENO_OK) {
    e = cudaMemcpyAsync(&h, dcount, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    rc = cuda_error(s, e, "harvest count");
  }
  cudaFreeAsync(dcount, s->stream);
  cudaStreamSynchronize(s->stream);
  *count = long(h);
  return rc;
}

int hteno_kxrcf(hteno_solver* s, unsigned char* flags) {
  if (!s || !flags) return HTENO_ERR_INVALID_ARG;
  if (s->cfg.dims != 1 || is_hermite(s))
    return set_error(s, HTENO_ERR_UNSUPPORTED, "the KXRCF sensor belongs to the FV 1D scheme");
  return fv1d_kxrcf(s, flags);
}

const char* hteno_last_error(hteno_solver* s) { return s ? s->err.c_str() : "null handle"; }

int hteno_enable_kernel_timing(hteno_solver* s, int on) {
  if (!s) return HTENO_ERR_INVALID_ARG;
  cudaStreamSynchronize(s->stream);
  s->timing = on != 0;
  s->ev_used = 0;
  for (auto& k : s->kinds) {
    k.launches = 0;
    k.ms = 0;
  }
  return HTENO_OK;
}

int hteno_kernel_timing(hteno_solver* s, hteno_kernel_time* out, int max, int* count) {
  if (!s || (max > 0 && !out)) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "kernel timing");
  for (size_t i = 0; i < s->ev_used; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s->ev[2 * i], s->ev[2 * i + 1]) == cudaSuccess) {
      s->kinds[s->ev_kind[i]].ms += ms;
      s->kinds[s->ev_kind[i]].launches += 1;
    }
  }
  s->ev_used = 0;
  if (count) *count = int(s->kinds.size());
  for (int k = 0; k < max && k < int(s->kinds.size()); ++k) {
    std::memset(&out[k], 0, sizeof(out[k]));
    std::snprintf(out[k].name, sizeof(out[k].name), "%s", s->kinds[k].name.c_str());
    out[k].launches = s->kinds[k].launches;
    out[k].ms = s->kinds[k].ms;
    out[k].bytes_per_launch = s->kinds[k].bytes;
    out[k].flops_per_launch = s->kinds[k].flops;
  }
  return HTENO_OK;
}

int hteno_residual(hteno_solver* s, const double* q, double* rhs) {
  if (!s || !q || !rhs) return HTENO_ERR_INVALID_ARG;
  if (s->cfg.dims != 2 || is_hermite(s))
    return set_error(s, HTENO_ERR_UNSUPPORTED, "residual is exposed for the FV 2D scheme");
  int rc = fv2d_residual(s, q, rhs);
  if (rc) return rc;
  return cuda_error(s, cudaStreamSynchronize(s->stream), "residual");
}

}  // extern "C"
