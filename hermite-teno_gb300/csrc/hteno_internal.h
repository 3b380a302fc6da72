// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hteno.h"
#include "device_math.cuh"

namespace hteno {

// Device-resident time-stepping state; the host never reads it inside a step loop.
struct StepState {
  double t;          // simulation time
  double dt;         // dt of the current step
  double t_final;    // stop time of the current hteno_step call
  double dt_scale;   // cfl * min(dx, dy) (or cfl * dx^(5/3) for the Hermite 1D scheme)
  unsigned long long maxbits;  // running max wave speed (bit pattern of a non-negative double)
  long long steps;   // completed steps
  int done;          // 1 once t >= t_final: the remaining launches of the call are no-ops
  int status;        // bit 0: NaN seen; bit 1: non-positive density/pressure seen;
                     // bit 2: a bounded device-side wait gave up (the step's results are void)
  unsigned long long uniform;  // cell-stages given their exactly zero residual (uniform regions)
  unsigned long long tma_tiles;  // mixed FV 2D tiles staged by a TMA box copy
};

// Per-device upload of the constant block of one translation unit.
template <typename Sym>
inline cudaError_t upload_const(const Sym& sym, unsigned long long* mask, std::mutex* mu) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(*mu);
  if (dev < 64 && (*mask & (1ull << dev))) return cudaSuccess;
  DevConst h;
  fill_dev_const(&h);
  e = cudaMemcpyToSymbol(sym, &h, sizeof(DevConst));
  if (e == cudaSuccess && dev < 64) *mask |= (1ull << dev);
  return e;
}

}  // namespace hteno

struct hteno_solver {
  hteno_config cfg;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int nvar = 4;
  size_t ncell = 0;
  double dx = 0, dy = 0;

  // conserved state (double) and the step-start copy
  double* q = nullptr;
  double* q0 = nullptr;
  // Hermite moments and their step-start copies
  double* v = nullptr;
  double* v0 = nullptr;
  double* w = nullptr;
  double* w0 = nullptr;
  // scheme work buffers (layout owned by the scheme's translation unit)
  void* work = nullptr;
  size_t work_bytes = 0;

  hteno::StepState* dstate = nullptr;  // device
  hteno::StepState* hstate = nullptr;  // pinned host mirror

  int launches_per_step = 0;
  int tile_variant = -1;  // mixed FV 2D: tile shape picked by the tuner (-1: not yet)
  // mixed FV 2D: TMA tensor maps (CUtensorMap, 128 bytes each) of the three stage inputs, made
  // for the tile shape tmap_variant; tma false (HTENO_TMA=0) loads every tile cell by cell
  alignas(64) unsigned char tmap[3][128] = {};
  int tmap_variant = -1;
  bool tmap_ok = false;
  bool tma = true;
  uint8_t* deep = nullptr;  // plain FV 2D: cells of uniform 7 x 7 neighbourhoods (per stage)
  bool uniform_skip = true;  // FV 2D: uniform regions take their exactly zero residual directly
  double* ghost_faces = nullptr;  // plain FV 2D with HTENO_BC_TAYLOR / _DOUBLE_MACH: ghost face rows
  double* fused64 = nullptr;  // plain FV 2D in fused stages: q1, q2 and their primitives [4][4][ncell]
  // plain FV 2D and Hermite 2D: the y-direction face and flux kernels run on side_stream beside
  // the x-direction ones (forked before the faces, joined before the update); side = false keeps
  // one stream
  cudaStream_t side_stream = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  bool side = true;
  cudaGraphExec_t step_graph = nullptr;  // 1D schemes: a run of steps replayed as one graph
  // learned routing (mixed FV 2D): classifier, threshold, audit period, masks, audit sums
  hteno_mlp* router = nullptr;
  float router_thr = 0.9f;
  int audit_every = 0;
  int router_every = 1;    // classify every router_every steps; the masks serve the steps between
  int router_margin = 0;   // a route bit is kept only where it is set on every face this near
  uint8_t* route_tmp = nullptr;  // erosion scratch (one mask)
  long router_steps = 0;
  uint8_t* route_x = nullptr;
  uint8_t* route_y = nullptr;
  unsigned long long* audit = nullptr;  // [7]: seen, routed, misrouted, smooth, flat; rows asked; audited steps
  uint4* route_rows = nullptr;          // non-flat stencils handed to the network
  long route_cap = 0;
  bool strict = false;
  std::string err;

  // per-kernel event timing (hteno_enable_kernel_timing)
  struct TraceKind {
    std::string name;
    double bytes = 0, flops = 0;
    long launches = 0;
    double ms = 0;
  };
  bool timing = false;
  std::vector<TraceKind> kinds;
  std::vector<cudaEvent_t> ev;      // pairs: ev[2k] start, ev[2k+1] stop
  std::vector<int> ev_kind;
  size_t ev_used = 0;
};

namespace hteno {

int set_error(hteno_solver* s, int code, const char* fmt, ...);

// Tracing: bracket one launch with events when timing is on.  kind ids are per solver.
int trace_kind(hteno_solver* s, const char* name, double bytes_per_launch, double flops_per_launch);
void trace_begin(hteno_solver* s, int kind);
void trace_end(hteno_solver* s);
int cuda_error(hteno_solver* s, cudaError_t e, const char* what);

// Scheme back ends (one translation unit each).
int fv2d_setup(hteno_solver* s);
int fv2d_prepare(hteno_solver* s);  // after set_state: primitives of the new state
int fv2d_step_async(hteno_solver* s, int nsteps);
int fv2d_residual(hteno_solver* s, const double* q, double* rhs);
int fv2d_fp64_set_fused(hteno_solver* s, int on);  // plain FV 2D: one launch per stage
int make_side_stream(hteno_solver* s);  // side_stream and its fork/join events, unless side is off

int fv1d_setup(hteno_solver* s);
int fv1d_prepare(hteno_solver* s);
int fv1d_step_async(hteno_solver* s, int nsteps);
int fv1d_kxrcf(hteno_solver* s, uint8_t* flags);
int fv1d_harvest(hteno_solver* s, double p, unsigned long long seed, uint16_t* X, uint8_t* Y,
                 long cap, unsigned long long* count);
int fv2d_harvest_entry(hteno_solver* s, double p, unsigned long long seed, uint16_t* X, uint8_t* Y,
                       long cap, unsigned long long* count);

int hermite2d_setup(hteno_solver* s);
int hermite2d_prepare(hteno_solver* s);
int hermite2d_step_async(hteno_solver* s, int nsteps);

int hermite1d_setup(hteno_solver* s);
int hermite1d_prepare(hteno_solver* s);
int hermite1d_step_async(hteno_solver* s, int nsteps);

}  // namespace hteno
