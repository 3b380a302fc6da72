// Mixed-precision FV 2D path: one fused launch per RK stage (fv2d_fused.cuh), with the tile
// shape picked per solver by timing the candidates on the solver's own grid and state.
#include <algorithm>
#include <cstdlib>

#include "fv2d_fused.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

// MINB > 1 asks the compiler to fit MINB blocks per SM in registers (more warps to hide latency,
// at the price of a few spills); the tuner keeps whichever shape and register budget runs
// fastest.  Every variant gives the same bits (tested): this unit is compiled without implicit
// fused multiply-adds, so no instantiation can contract an expression differently.
template <int TX, int TY, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_fused(Geo G, int stage, fused::StageArgs a) {
  if (a.st && a.st->done) return;
  extern __shared__ __align__(16) unsigned char smem[];
  auto& S = *reinterpret_cast<fused::Smem<TX, TY>*>(smem);
  int bad = 0;
  const double ms = fused::tile_stage<TX, TY, NT>(c_dev, G, blockIdx.x * TX, blockIdx.y * TY,
                                                  stage, a, S, bad);
  if (stage == 3) {
    block_max_to(ms, &a.st->maxbits);
    if (bad) atomicOr(&a.st->status, bad);
  }
}

// Max wave speed of a state in double (timeStepping, FV_System2D.cpp:622-633): the first dt.
__global__ void k_max_speed(Geo G, const double* __restrict__ q, StepState* st) {
  const size_t nc = size_t(G.nx) * G.ny;
  double ms = 0.0;
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < nc;
       k += size_t(gridDim.x) * blockDim.x) {
    const double r = q[k], u = q[nc + k] / r, v = q[2 * nc + k] / r;
    const double p = (q[3 * nc + k] - 0.5 * (q[nc + k] * u + q[2 * nc + k] * v)) * G.g1;
    const double c = sqrt(fabs(G.gamma * p / r));
    ms = fmax(ms, fmax(fmax(u - c, fabs(u + c)), fmax(v - c, fabs(v + c))));
  }
  block_max_to(ms, &st->maxbits);
}

struct Variant {
  int tx, ty, nt;
  size_t smem;
  const char* name;
  void (*launch)(cudaStream_t, const Geo&, int, const fused::StageArgs&);
  cudaError_t (*prepare)();
};

template <int TX, int TY, int NT, int MINB>
void launch_v(cudaStream_t cs, const Geo& G, int stage, const fused::StageArgs& a) {
  const dim3 grid(unsigned((G.nx + TX - 1) / TX), unsigned((G.ny + TY - 1) / TY));
  k_fused<TX, TY, NT, MINB><<<grid, NT, fused::smem_bytes<TX, TY>(), cs>>>(G, stage, a);
}

template <int TX, int TY, int NT, int MINB>
cudaError_t prepare_v() {
  return cudaFuncSetAttribute(k_fused<TX, TY, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(fused::smem_bytes<TX, TY>()));
}

#define HTENO_VARIANT(TX, TY, NT, MINB)                                                           \
  { TX, TY, NT, fused::smem_bytes<TX, TY>(), "fused_" #TX "x" #TY "_" #NT "_b" #MINB,               \
    launch_v<TX, TY, NT, MINB>, prepare_v<TX, TY, NT, MINB> }

const Variant kVariants[] = {
    HTENO_VARIANT(32, 16, 256, 1), HTENO_VARIANT(32, 8, 256, 1),  HTENO_VARIANT(16, 16, 256, 1),
    HTENO_VARIANT(64, 8, 256, 1),  HTENO_VARIANT(32, 32, 512, 1), HTENO_VARIANT(16, 8, 128, 1),
    HTENO_VARIANT(32, 16, 256, 3), HTENO_VARIANT(64, 8, 256, 3),
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

// HTENO_FV2D_TILE=<index> forces a tile shape (0-based index into kVariants); the results do
// not depend on it (every face is computed from the same data with the same arithmetic).
int forced_variant() {
  const char* e = std::getenv("HTENO_FV2D_TILE");
  if (!e || !*e) return -1;
  const int v = std::atoi(e);
  return v >= 0 && v < kNumVariants ? v : -1;
}

void launch_stage(hteno_solver* s, const Geo& G, int stage, const fused::StageArgs& a) {
  const Variant& V = kVariants[s->tile_variant < 0 ? 0 : s->tile_variant];
  const double nc = double(G.nx) * G.ny;
  const double nf = double(G.nx + 1) * G.ny + double(G.ny + 1) * G.nx;
  const double fluxf = G.flux == HTENO_FLUX_HLLC ? kFluxFlopsHllc : kFluxFlopsRusanov;
  // compulsory DRAM bytes: stage 1 reads q^n and writes q1 (64 B per cell); stages 2 and 3
  // read q_s and q^n and write q_{s+1} (96 B); the residual reads q and writes rhs
  const double bytes = stage == 2 || stage == 3 ? 96.0 * nc : 64.0 * nc;
  const int kind = trace_kind(s, stage == 2 || stage == 3 ? "fused_s23" : "fused_s1", bytes,
                              (kFacesFlops + fluxf) * nf + kUpdateFlops * nc);
  trace_begin(s, kind);
  V.launch(s->stream, G, stage, a);
  trace_end(s);
}

}  // namespace

size_t fv2d_fused_work_bytes(int nx, int ny) { return 4 * size_t(nx) * ny * sizeof(double) + 256; }

int fv2d_fused_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  for (int v = 0; v < kNumVariants; ++v) {
    const cudaError_t e = kVariants[v].prepare();
    if (e != cudaSuccess) return cuda_error(s, e, "fused kernel attributes");
  }
  s->tile_variant = forced_variant();
  return HTENO_OK;
}

// After a new state: the first dt's wave speed, and (once per solver) the tile shape, timed as
// residual evaluations of this state into the scratch buffer.
int fv2d_fused_prepare(hteno_solver* s, const Geo& G, double* scratch) {
  k_max_speed<<<304, 256, 0, s->stream>>>(G, s->q, s->dstate);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(s, e, "max speed");
  if (s->tile_variant >= 0) return HTENO_OK;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "tuner events");
  fused::StageArgs args{s->q, nullptr, scratch, nullptr};
  args.skip_uniform = false;  // time the full work, not the (mostly uniform) initial state
  int best = 0;
  float best_ms = 3.4e38f;
  for (int v = 0; v < kNumVariants; ++v) {
    kVariants[v].launch(s->stream, G, 0, args);  // warm
    cudaEventRecord(a, s->stream);
    for (int r = 0; r < 3; ++r) kVariants[v].launch(s->stream, G, 0, args);
    cudaEventRecord(b, s->stream);
    e = cudaEventSynchronize(b);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return cuda_error(s, e, "tile tuner");
  s->tile_variant = best;
  return HTENO_OK;
}

// One SSP-RK3 step: q -> q0buf (stage 1), q0buf -> qc (stage 2, base q), qc -> q (stage 3).
// With a router the classifier first writes the route masks from the step-start state; the
// three stages use them, and every `audit_every` steps the stages also evaluate the plain TENO
// cut-off of every stencil and count how the routing compares.
void fv2d_fused_step(hteno_solver* s, const Geo& G, double* qc) {
  fused::StageArgs a1{s->q, nullptr, s->q0, s->dstate}, a2{s->q0, s->q, qc, s->dstate},
      a3{qc, s->q, s->q, s->dstate};
  a1.skip_uniform = a2.skip_uniform = a3.skip_uniform = s->uniform_skip;
  if (s->router) {
    const int kc = trace_kind(s, "classify", 0.0, 0.0);
    trace_begin(s, kc);
    mlp_classify(s->router, G, s->q, s->route_x, s->route_y, s->router_thr, s->route_rows, s->audit + 5,
                 s->route_cap, s->stream);
    trace_end(s);
    const bool aud = s->audit_every > 0 && s->router_steps % s->audit_every == 0;
    for (fused::StageArgs* a : {&a1, &a2, &a3}) {
      a->mx = s->route_x;
      a->my = s->route_y;
      a->audit = aud ? s->audit : nullptr;
    }
    if (aud) ++s->audits;
    ++s->router_steps;
  }
  launch_stage(s, G, 1, a1);
  launch_stage(s, G, 2, a2);
  launch_stage(s, G, 3, a3);
}

void fv2d_fused_residual(hteno_solver* s, const Geo& G, const double* q, double* rhs) {
  fused::StageArgs a{q, nullptr, rhs, nullptr};
  a.skip_uniform = s->uniform_skip;
  launch_stage(s, G, 0, a);
}

const char* fv2d_fused_variant_name(int v) {
  return v >= 0 && v < kNumVariants ? kVariants[v].name : "untuned";
}

}  // namespace hteno

using namespace hteno;

extern "C" {

int hteno_set_router(hteno_solver* s, hteno_mlp* m, float threshold, int audit_every) {
  if (!s || !(threshold > 0.f && threshold < 1.f) || audit_every < 0) return HTENO_ERR_INVALID_ARG;
  if (s->cfg.dims != 2 || s->cfg.scheme != HTENO_SCHEME_FV || s->cfg.precision != HTENO_PREC_MIXED)
    return set_error(s, HTENO_ERR_UNSUPPORTED, "learned routing runs on the mixed FV 2D path");
  if (s->cfg.recon != HTENO_RECON_TENO5 && s->cfg.recon != HTENO_RECON_TENO5I)
    return set_error(s, HTENO_ERR_UNSUPPORTED, "learned routing predicts TENO cut-offs (teno5, teno5i)");
  cudaStreamSynchronize(s->stream);
  if (!m) {
    s->router = nullptr;
    s->launches_per_step = 2 + 3;
    return HTENO_OK;
  }
  const size_t bx = size_t(s->cfg.nx + 1) * s->cfg.ny, by = size_t(s->cfg.ny + 1) * s->cfg.nx;
  if (bx + by >= (size_t(1) << 29))  // a network row carries (face << 3 | bit) in 32 bits
    return set_error(s, HTENO_ERR_UNSUPPORTED, "learned routing takes grids of fewer than 2^29 faces");
  if (!s->route_x) {
    // rows for the network: every stencil of every face, at most 256 M rows (4 GB)
    s->route_cap = long(std::min<size_t>(8 * (bx + by), size_t(256) << 20));
    cudaError_t e = cudaMalloc(&s->route_x, (bx + 3) & ~size_t(3));
    if (e == cudaSuccess) e = cudaMalloc(&s->route_y, (by + 3) & ~size_t(3));
    if (e == cudaSuccess) e = cudaMalloc(&s->audit, 6 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->route_rows, size_t(s->route_cap) * sizeof(uint4));
    if (e != cudaSuccess) return cuda_error(s, e, "route masks");
  }
  cudaMemset(s->audit, 0, 6 * sizeof(unsigned long long));
  s->router = m;
  s->router_thr = threshold;
  s->audit_every = audit_every;
  s->router_steps = 0;
  s->audits = 0;
  s->launches_per_step = 2 + 3 + 2;
  return HTENO_OK;
}

int hteno_router_stats(hteno_solver* s, long long* stats) {
  if (!s || !stats) return HTENO_ERR_INVALID_ARG;
  if (!s->router || !s->audit) return set_error(s, HTENO_ERR_UNSUPPORTED, "no router set");
  unsigned long long h[6] = {0, 0, 0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(h, s->audit, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "router stats");
  for (int k = 0; k < 5; ++k) stats[k] = (long long)h[k];
  stats[5] = s->audits;
  stats[6] = (long long)h[5];
  const int rc = mlp_status(s->router, s->stream);
  return rc == HTENO_OK ? HTENO_OK : set_error(s, rc, "classifier tensor-core wait timed out");
}

}  // extern "C"
