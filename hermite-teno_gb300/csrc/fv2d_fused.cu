// Mixed-precision FV 2D path: one fused launch per RK stage (fv2d_fused.cuh), with the tile
// shape picked per solver by timing the candidates on the solver's own grid and state.
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <algorithm>
#include <cstdlib>
#include <cstring>

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
// tm: tensor map of a.qin for the TMA staging of interior tiles (used when has_tm).
template <int TX, int TY, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_fused(Geo G, int stage, fused::StageArgs a,
                                                    const __grid_constant__ CUtensorMap tm, int has_tm) {
  if (a.st && a.st->done) return;
  extern __shared__ __align__(128) unsigned char smem[];
  auto& S = *reinterpret_cast<fused::Smem<TX, TY>*>(smem);
  a.tmap = has_tm && (tc::smem_u32(&S.c[0][0]) & 127u) == 0 ? &tm : nullptr;
  // an audited step that runs (not past the stop time) counts once
  if (stage == 1 && a.audit && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
    atomicAdd(a.audit + 6, 1ull);
  uint32_t phase = 0;
  if (a.tmap) fused::tma_setup(S);
  int bad = 0;
  const double ms = fused::tile_stage<TX, TY, NT>(c_dev, G, blockIdx.x * TX, blockIdx.y * TY,
                                                  stage, a, S, bad, phase);
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

// Erosion of a route mask [rows][cols] along one axis: a bit stays set only where it is set on
// every face within `d` along that axis; faces past the ends of the array count as unset, so
// bits within d of the grid's edges clear.  Two passes (along and across) make the square
// neighbourhood.
__global__ void k_erode(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, int rows, int cols,
                        int d, int along_rows, const StepState* __restrict__ st) {
  if (st && st->done) return;
  const long k = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (k >= long(rows) * cols) return;
  const int r = int(k / cols), c = int(k - long(r) * cols);
  const int pos = along_rows ? r : c, n = along_rows ? rows : cols;
  unsigned v = in[k];
  if (pos < d || pos + d >= n) {
    v = 0u;
  } else {
    for (int o = -d; o <= d && v; ++o)
      v &= in[along_rows ? k + long(o) * cols : k + o];
  }
  out[k] = uint8_t(v);
}

void erode_mask(hteno_solver* s, uint8_t* mask, int rows, int cols) {
  const long n = long(rows) * cols;
  const unsigned grid = unsigned((n + 255) / 256);
  k_erode<<<grid, 256, 0, s->stream>>>(mask, s->route_tmp, rows, cols, s->router_margin, 0, s->dstate);
  k_erode<<<grid, 256, 0, s->stream>>>(s->route_tmp, mask, rows, cols, s->router_margin, 1, s->dstate);
}

struct Variant {
  int tx, ty, nt;
  size_t smem;
  const char* name;
  void (*launch)(cudaStream_t, const Geo&, int, const fused::StageArgs&, const CUtensorMap*);
  cudaError_t (*prepare)();
};

template <int TX, int TY, int NT, int MINB>
void launch_v(cudaStream_t cs, const Geo& G, int stage, const fused::StageArgs& a, const CUtensorMap* tm) {
  const dim3 grid(unsigned((G.nx + TX - 1) / TX), unsigned((G.ny + TY - 1) / TY));
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  k_fused<TX, TY, NT, MINB><<<grid, NT, fused::smem_bytes<TX, TY>(), cs>>>(G, stage, a, tm ? *tm : none,
                                                                          tm ? 1 : 0);
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

// Tensor maps of the three stage inputs (q, q0, the work state) for the variant in use, made
// once per variant; all null when the grid cannot be staged by TMA.
void ensure_maps(hteno_solver* s, const Geo& G, const Variant& V, const double* qc) {
  const int v = s->tile_variant < 0 ? 0 : s->tile_variant;
  if (s->tmap_variant == v) return;
  s->tmap_variant = v;
  const double* bufs[3] = {s->q, s->q0, qc};
  s->tmap_ok = true;
  for (int k = 0; k < 3; ++k)
    s->tmap_ok = s->tmap_ok && fused::encode_box_map(reinterpret_cast<CUtensorMap*>(s->tmap[k]), bufs[k], G.nx,
                                              G.ny, V.tx + 8, V.ty + 6);
}

void launch_stage(hteno_solver* s, const Geo& G, int stage, const fused::StageArgs& a,
                  int map = -1) {
  const Variant& V = kVariants[s->tile_variant < 0 ? 0 : s->tile_variant];
  const CUtensorMap* tm = map >= 0 && s->tmap_ok && s->tma
                              ? reinterpret_cast<const CUtensorMap*>(s->tmap[map]) : nullptr;
  const double nc = double(G.nx) * G.ny;
  const double nf = double(G.nx + 1) * G.ny + double(G.ny + 1) * G.nx;
  const double fluxf = G.flux == HTENO_FLUX_HLLC ? kFluxFlopsHllc : kFluxFlopsRusanov;
  // compulsory DRAM bytes: stage 1 reads q^n and writes q1 (64 B per cell); stages 2 and 3
  // read q_s and q^n and write q_{s+1} (96 B); the residual reads q and writes rhs
  const double bytes = stage == 2 || stage == 3 ? 96.0 * nc : 64.0 * nc;
  const int kind = trace_kind(s, stage == 2 || stage == 3 ? "fused_s23" : "fused_s1", bytes,
                              (kFacesFlops + fluxf) * nf + kUpdateFlops * nc);
  trace_begin(s, kind);
  V.launch(s->stream, G, stage, a, tm);
  trace_end(s);
}

}  // namespace

// Tensor map of one [4][ny][nx] double state buffer for a box_x x box_y x 4 box; false when the
// grid cannot be staged by TMA (nx odd: the row stride is not a multiple of 16 bytes) or encoding
// fails.
bool fused::encode_box_map(CUtensorMap* m, const double* base, int nx, int ny, int box_x, int box_y) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (!encode || (nx & 1) || (reinterpret_cast<uintptr_t>(base) & 15)) return false;
  const cuuint64_t dims[3] = {cuuint64_t(nx), cuuint64_t(ny), 4};
  const cuuint64_t strides[2] = {cuuint64_t(nx) * sizeof(double), cuuint64_t(nx) * ny * sizeof(double)};
  const cuuint32_t box[3] = {cuuint32_t(box_x), cuuint32_t(box_y), 4};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(base), dims, strides, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

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
  s->router_steps = 0;  // a new state: the next step classifies (route masks are per state)
  if (s->audit) cudaMemsetAsync(s->audit, 0, 7 * sizeof(unsigned long long), s->stream);
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
    kVariants[v].launch(s->stream, G, 0, args, nullptr);  // warm
    cudaEventRecord(a, s->stream);
    for (int r = 0; r < 3; ++r) kVariants[v].launch(s->stream, G, 0, args, nullptr);
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
// With a router the classifier writes the route masks from the step-start state every
// `router_every` steps (eroded by `router_margin` faces, so that a route outlives no
// discontinuity that could reach its stencil before the next classification); the stages use
// them, and every `audit_every` steps the stages also evaluate the plain TENO cut-off of every
// stencil and count how the routing compares.
void fv2d_fused_step(hteno_solver* s, const Geo& G, double* qc) {
  fused::StageArgs a1{s->q, nullptr, s->q0, s->dstate}, a2{s->q0, s->q, qc, s->dstate},
      a3{qc, s->q, s->q, s->dstate};
  a1.skip_uniform = a2.skip_uniform = a3.skip_uniform = s->uniform_skip;
  if (s->router) {
    if (s->router_steps % s->router_every == 0) {
      const int kc = trace_kind(s, "classify", 0.0, 0.0);
      trace_begin(s, kc);
      mlp_classify(s->router, G, s->q, s->route_x, s->route_y, s->router_thr, s->route_rows,
                   s->audit + 5, s->route_cap, s->stream, s->dstate);
      if (s->router_margin > 0) {
        erode_mask(s, s->route_x, G.ny, G.nx + 1);
        erode_mask(s, s->route_y, G.ny + 1, G.nx);
      }
      trace_end(s);
    }
    const bool aud = s->audit_every > 0 && s->router_steps % s->audit_every == 0;
    for (fused::StageArgs* a : {&a1, &a2, &a3}) {
      a->mx = s->route_x;
      a->my = s->route_y;
      a->audit = aud ? s->audit : nullptr;
    }
    ++s->router_steps;
  }
  ensure_maps(s, G, kVariants[s->tile_variant < 0 ? 0 : s->tile_variant], qc);
  launch_stage(s, G, 1, a1, 0);
  launch_stage(s, G, 2, a2, 1);
  launch_stage(s, G, 3, a3, 2);
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
    if (e == cudaSuccess) e = cudaMalloc(&s->audit, 7 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&s->route_rows, size_t(s->route_cap) * sizeof(uint4));
    if (e != cudaSuccess) return cuda_error(s, e, "route masks");
  }
  cudaMemset(s->audit, 0, 7 * sizeof(unsigned long long));
  cudaMemset(s->route_x, 0, bx);
  cudaMemset(s->route_y, 0, by);
  s->router = m;
  s->router_thr = threshold;
  s->audit_every = audit_every;
  s->router_steps = 0;
  s->launches_per_step = 2 + 3 + 2;
  return HTENO_OK;
}

int hteno_set_router_schedule(hteno_solver* s, int classify_every, int margin) {
  if (!s || classify_every < 1 || margin < 0) return HTENO_ERR_INVALID_ARG;
  if (!s->router || !s->route_x) return set_error(s, HTENO_ERR_UNSUPPORTED, "no router set");
  if (margin > 0 && !s->route_tmp) {
    const size_t bx = size_t(s->cfg.nx + 1) * s->cfg.ny, by = size_t(s->cfg.ny + 1) * s->cfg.nx;
    const cudaError_t e = cudaMalloc(&s->route_tmp, std::max(bx, by));
    if (e != cudaSuccess) return cuda_error(s, e, "route erosion buffer");
  }
  cudaStreamSynchronize(s->stream);
  s->router_every = classify_every;
  s->router_margin = margin;
  s->router_steps = 0;  // the next step classifies
  return HTENO_OK;
}

int hteno_router_audit64(hteno_solver* s, long long* counts) {
  if (!s || !counts) return HTENO_ERR_INVALID_ARG;
  if (!s->router || !s->route_x) return set_error(s, HTENO_ERR_UNSUPPORTED, "no router set");
  const Geo G = geo_of(s);
  int rc = mlp_classify(s->router, G, s->q, s->route_x, s->route_y, s->router_thr, s->route_rows,
                        s->audit + 5, s->route_cap, s->stream, nullptr);
  if (rc != HTENO_OK) return set_error(s, rc, "classification");
  if (s->router_margin > 0) {
    erode_mask(s, s->route_x, G.ny, G.nx + 1);
    erode_mask(s, s->route_y, G.ny + 1, G.nx);
  }
  rc = fv2d_audit64(s, G, s->q, s->route_x, s->route_y, counts);
  if (rc != HTENO_OK) return rc;
  rc = mlp_status(s->router, s->stream);
  return rc == HTENO_OK ? HTENO_OK : set_error(s, rc, "classifier tensor-core wait timed out");
}

int hteno_router_stats(hteno_solver* s, long long* stats) {
  if (!s || !stats) return HTENO_ERR_INVALID_ARG;
  if (!s->router || !s->audit) return set_error(s, HTENO_ERR_UNSUPPORTED, "no router set");
  unsigned long long h[7] = {0, 0, 0, 0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(h, s->audit, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "router stats");
  for (int k = 0; k < 5; ++k) stats[k] = (long long)h[k];
  stats[5] = (long long)h[6];
  stats[6] = (long long)h[5];
  const int rc = mlp_status(s->router, s->stream);
  return rc == HTENO_OK ? HTENO_OK : set_error(s, rc, "classifier tensor-core wait timed out");
}

}  // extern "C"
