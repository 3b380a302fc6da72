// Mixed-precision FV 2D path: one fused launch per RK stage (fv2d_fused.cuh), with the tile
// shape picked per solver by timing the candidates on the solver's own grid and state.
#include <cstdlib>

#include "fv2d_fused.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) k_fused(Geo G, int stage, fused::StageArgs a) {
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

template <int TX, int TY, int NT>
void launch_v(cudaStream_t cs, const Geo& G, int stage, const fused::StageArgs& a) {
  const dim3 grid(unsigned((G.nx + TX - 1) / TX), unsigned((G.ny + TY - 1) / TY));
  k_fused<TX, TY, NT><<<grid, NT, fused::smem_bytes<TX, TY>(), cs>>>(G, stage, a);
}

template <int TX, int TY, int NT>
cudaError_t prepare_v() {
  return cudaFuncSetAttribute(k_fused<TX, TY, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(fused::smem_bytes<TX, TY>()));
}

#define HTENO_VARIANT(TX, TY, NT) \
  { TX, TY, NT, fused::smem_bytes<TX, TY>(), "fused_" #TX "x" #TY "_" #NT, launch_v<TX, TY, NT>, prepare_v<TX, TY, NT> }

const Variant kVariants[] = {
    HTENO_VARIANT(32, 16, 256), HTENO_VARIANT(32, 8, 256),  HTENO_VARIANT(16, 16, 256),
    HTENO_VARIANT(64, 8, 256),  HTENO_VARIANT(32, 32, 512), HTENO_VARIANT(16, 8, 128),
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
void fv2d_fused_step(hteno_solver* s, const Geo& G, double* qc) {
  launch_stage(s, G, 1, fused::StageArgs{s->q, nullptr, s->q0, s->dstate});
  launch_stage(s, G, 2, fused::StageArgs{s->q0, s->q, qc, s->dstate});
  launch_stage(s, G, 3, fused::StageArgs{qc, s->q, s->q, s->dstate});
}

void fv2d_fused_residual(hteno_solver* s, const Geo& G, const double* q, double* rhs) {
  launch_stage(s, G, 0, fused::StageArgs{q, nullptr, rhs, nullptr});
}

const char* fv2d_fused_variant_name(int v) {
  return v >= 0 && v < kNumVariants ? kVariants[v].name : "untuned";
}

}  // namespace hteno
