// Many independent FV::System2D instances of uneven grid sizes advanced together (mixed
// precision).  Each instance keeps the reference's semantics (its own timeStepping loop and dt,
// FV_System2D.cpp:614-651); the batch runs one persistent launch per RK stage over the tiles of
// all instances, and a whole step (dt of every instance, 3 stages, time update) is captured once
// in a CUDA graph and replayed.  The tile shape is picked by timing the candidates on the
// batch's own instances.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>

#include "fv2d_fused.cuh"

struct hteno_batch;

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

struct BInst {
  Geo G;
  double* q;   // state
  double* q1;  // stage-1 state
  double* q2;  // stage-2 state (residual scratch while tuning)
  StepState* st;
  int has_tm;  // tm valid: TMA staging of the instance's interior tiles
  alignas(64) CUtensorMap tm[3];  // of q, q1, q2 for the tile shape in use (stages 1, 2, 3 read them)
};

// One launch per stage over every tile of every instance: block b takes jobs b, b + grid, ...
template <int TX, int TY, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_batch_stage(const BInst* __restrict__ inst,
                                                    const int4* __restrict__ jobs, int njobs,
                                                    int stage) {
  extern __shared__ __align__(128) unsigned char smem[];
  auto& S = *reinterpret_cast<fused::Smem<TX, TY>*>(smem);
  // TMA box copies (tensor maps in the instance records, global memory): one mbarrier per block,
  // its phase tracked across the block's tiles
  const bool tma_ok = stage != 0 && (tc::smem_u32(&S.c[0][0]) & 127u) == 0;
  uint32_t phase = 0;
  if (tma_ok) fused::tma_setup(S);
  for (int j = blockIdx.x; j < njobs; j += gridDim.x) {
    const int4 job = jobs[j];
    const BInst& I = inst[job.x];
    if (stage != 0 && I.st->done) continue;  // uniform over the block
    fused::StageArgs a;
    if (stage == 0) a = fused::StageArgs{I.q, nullptr, I.q2, nullptr};
    else if (stage == 1) a = fused::StageArgs{I.q, nullptr, I.q1, I.st};
    else if (stage == 2) a = fused::StageArgs{I.q1, I.q, I.q2, I.st};
    else a = fused::StageArgs{I.q2, I.q, I.q, I.st};
    a.skip_uniform = stage != 0;  // stage 0 only times tile shapes: the full work
    a.tmap = tma_ok && I.has_tm ? &I.tm[stage - 1] : nullptr;
    int bad = 0;
    const double ms = fused::tile_stage<TX, TY, NT>(c_dev, I.G, job.y, job.z, stage, a, S, bad, phase);
    if (bad & 4) break;  // a box copy that did not complete: no further copies into this block
    if (stage == 3) {
      block_max_to(ms, &I.st->maxbits);
      if (bad) atomicOr(&I.st->status, bad);
    }
  }
}

__global__ void k_batch_begin(StepState* st, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  StepState* s = st + i;
  if (s->done) return;
  if (!(s->t < s->t_final)) {
    s->done = 1;
    return;
  }
  const double M = __longlong_as_double(static_cast<long long>(s->maxbits));
  double dt = s->dt_scale / M;
  dt = s->t + dt > s->t_final ? s->t_final - s->t : dt;
  s->dt = dt;
  s->maxbits = 0ull;
}

__global__ void k_batch_end(StepState* st, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || st[i].done) return;
  st[i].t += st[i].dt;
  st[i].steps += 1;
}

__global__ void k_batch_set_target(StepState* st, int n, double t_final) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  st[i].t_final = t_final;
  st[i].done = 0;
}

// Max wave speed of one instance's state (the first dt after set_state), double.
__global__ void k_inst_max_speed(const BInst* __restrict__ inst, int i) {
  const BInst& I = inst[i];
  const size_t nc = size_t(I.G.nx) * I.G.ny;
  const double* q = I.q;
  double ms = 0.0;
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < nc;
       k += size_t(gridDim.x) * blockDim.x) {
    const double r = q[k], u = q[nc + k] / r, v = q[2 * nc + k] / r;
    const double p = (q[3 * nc + k] - 0.5 * (q[nc + k] * u + q[2 * nc + k] * v)) * I.G.g1;
    const double c = sqrt(fabs(I.G.gamma * p / r));
    ms = fmax(ms, fmax(fmax(u - c, fabs(u + c)), fmax(v - c, fabs(v + c))));
  }
  block_max_to(ms, &I.st->maxbits);
}

struct BVariant {
  int tx, ty, nt;
  size_t smem;
  const char* name;
  void (*launch)(cudaStream_t, int grid, const BInst*, const int4*, int, int);
  cudaError_t (*prepare)(int* blocks_per_sm);
};

template <int TX, int TY, int NT, int MINB>
void blaunch(cudaStream_t cs, int grid, const BInst* inst, const int4* jobs, int njobs, int stage) {
  k_batch_stage<TX, TY, NT, MINB><<<grid, NT, fused::smem_bytes<TX, TY>(), cs>>>(inst, jobs, njobs, stage);
}

template <int TX, int TY, int NT, int MINB>
cudaError_t bprepare(int* blocks_per_sm) {
  cudaError_t e = cudaFuncSetAttribute(k_batch_stage<TX, TY, NT, MINB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(fused::smem_bytes<TX, TY>()));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_batch_stage<TX, TY, NT, MINB>,
                                                       NT, fused::smem_bytes<TX, TY>());
}

// MINB > 1: the register budget of MINB blocks per SM (as for the single-grid kernel).  Every
// candidate gives the same bits: this unit is compiled without implicit contraction.
#define HTENO_BVARIANT(TX, TY, NT, MINB)                                                          \
  { TX, TY, NT, fused::smem_bytes<TX, TY>(), "batch_" #TX "x" #TY "_" #NT "_b" #MINB,              \
    blaunch<TX, TY, NT, MINB>, bprepare<TX, TY, NT, MINB> }

const BVariant kBVariants[] = {
    HTENO_BVARIANT(32, 16, 256, 1), HTENO_BVARIANT(32, 8, 256, 1),  HTENO_BVARIANT(16, 16, 256, 1),
    HTENO_BVARIANT(64, 8, 256, 1),  HTENO_BVARIANT(32, 32, 512, 1), HTENO_BVARIANT(16, 8, 128, 1),
    HTENO_BVARIANT(32, 16, 256, 3), HTENO_BVARIANT(64, 8, 256, 3),
};
constexpr int kNumBVariants = sizeof(kBVariants) / sizeof(kBVariants[0]);

}  // namespace
}  // namespace hteno

using namespace hteno;

struct hteno_batch {
  int n = 0;
  std::vector<hteno_config> cfg;
  std::vector<BInst> hinst;
  std::vector<size_t> ncell;
  BInst* dinst = nullptr;
  StepState* dstate = nullptr;
  StepState* hstate = nullptr;  // pinned mirror
  double* pool = nullptr;
  int4* jobs[kNumBVariants] = {nullptr};
  int njobs[kNumBVariants] = {0};
  int grid[kNumBVariants] = {0};
  int variant = -1;
  int forced = -1;
  int maps_variant = -1;  // tile shape the instances' tensor maps were made for
  bool tma = true;        // HTENO_TMA=0: every tile loads cell by cell
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  std::string err;
};

namespace {

int bfail(hteno_batch* b, int code, const char* msg) {
  if (b) b->err = msg;
  return code;
}

void brelease(hteno_batch* b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (int v = 0; v < kNumBVariants; ++v) cudaFree(b->jobs[v]);
  cudaFree(b->pool);
  cudaFree(b->dinst);
  cudaFree(b->dstate);
  if (b->hstate) cudaFreeHost(b->hstate);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
}

int bcuda(hteno_batch* b, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HTENO_OK;
  b->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? HTENO_ERR_OOM : HTENO_ERR_CUDA;
}

// One step of every instance on stream cs: dt, 3 stages, time update.
void launch_step(hteno_batch* b, cudaStream_t cs) {
  const int v = b->variant;
  const unsigned nb = unsigned((b->n + 127) / 128);
  k_batch_begin<<<nb, 128, 0, cs>>>(b->dstate, b->n);
  for (int stage = 1; stage <= 3; ++stage)
    kBVariants[v].launch(cs, b->grid[v], b->dinst, b->jobs[v], b->njobs[v], stage);
  k_batch_end<<<nb, 128, 0, cs>>>(b->dstate, b->n);
}

// Tile-shape tuner: each candidate evaluates the residual of every instance (into the stage-2
// buffers) three times; the fastest is kept.
int tune(hteno_batch* b) {
  if (b->forced >= 0) {
    b->variant = b->forced;
    return HTENO_OK;
  }
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return bfail(b, HTENO_ERR_CUDA, "tuner events");
  int best = 0;
  float best_ms = 3.4e38f;
  cudaError_t e = cudaSuccess;
  for (int v = 0; v < kNumBVariants; ++v) {
    kBVariants[v].launch(b->stream, b->grid[v], b->dinst, b->jobs[v], b->njobs[v], 0);
    cudaEventRecord(e0, b->stream);
    for (int r = 0; r < 3; ++r)
      kBVariants[v].launch(b->stream, b->grid[v], b->dinst, b->jobs[v], b->njobs[v], 0);
    cudaEventRecord(e1, b->stream);
    e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return bcuda(b, e, "tile tuner");
  b->variant = best;
  return HTENO_OK;
}

// Tensor maps of every instance's three state buffers for the tile shape in use (boxes of
// TX + 8 x TY + 6 cells x 4 planes), in the instance records the stage kernel reads.
int ensure_maps(hteno_batch* b) {
  if (b->maps_variant == b->variant) return HTENO_OK;
  const BVariant& V = kBVariants[b->variant];
  for (int i = 0; i < b->n; ++i) {
    BInst& I = b->hinst[i];
    I.has_tm = 0;
    if (b->tma && I.G.bc < HTENO_BC_TAYLOR)
      I.has_tm = fused::encode_box_map(&I.tm[0], I.q, I.G.nx, I.G.ny, V.tx + 8, V.ty + 6) &&
                 fused::encode_box_map(&I.tm[1], I.q1, I.G.nx, I.G.ny, V.tx + 8, V.ty + 6) &&
                 fused::encode_box_map(&I.tm[2], I.q2, I.G.nx, I.G.ny, V.tx + 8, V.ty + 6);
  }
  cudaError_t e = cudaMemcpyAsync(b->dinst, b->hinst.data(), b->n * sizeof(BInst), cudaMemcpyHostToDevice,
                                  b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "instance tensor maps");
  b->maps_variant = b->variant;
  return HTENO_OK;
}

// Capture one step into a graph on the batch's stream (rebuilt when the stream changes).
int ensure_graph(hteno_batch* b) {
  if (b->variant < 0) {
    const int rc = tune(b);
    if (rc) return rc;
  }
  {
    const int rc = ensure_maps(b);
    if (rc) return rc;
  }
  if (b->graph && b->graph_stream == b->stream) return HTENO_OK;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaStream_t cap;
  cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bcuda(b, e, "capture stream");
  cudaGraph_t g = nullptr;
  e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    launch_step(b, cap);
    e = cudaStreamEndCapture(cap, &g);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cap);
  if (e != cudaSuccess) return bcuda(b, e, "step graph");
  b->graph_stream = b->stream;
  return HTENO_OK;
}

}  // namespace

extern "C" {

int hteno_batch_create(const hteno_config* cfgs, int n, hteno_batch** out) {
  if (!cfgs || !out || n <= 0 || n > (1 << 20)) return HTENO_ERR_INVALID_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    const hteno_config& c = cfgs[i];
    if (c.dims != 2 || c.scheme != HTENO_SCHEME_FV || c.precision != HTENO_PREC_MIXED)
      return HTENO_ERR_UNSUPPORTED;
    if (c.nx < 6 || c.ny < 6 || (long long)c.nx * c.ny > (1ll << 30) || !(c.xr > c.xl) ||
        !(c.yt > c.yb) || !(c.cfl > 0.0) || !(c.gamma > 1.0) || c.recon < 0 || c.recon > 7 ||
        c.flux < 0 || c.flux > 1 || c.bc < 0 || c.bc > 3 ||
        (c.bc >= HTENO_BC_TAYLOR && (c.nx < 7 || c.ny < 7)))
      return HTENO_ERR_INVALID_ARG;
  }
  hteno_batch* b = new (std::nothrow) hteno_batch();
  if (!b) return HTENO_ERR_OOM;
  auto fail = [&](int code) {
    brelease(b);
    delete b;
    return code;
  };
  b->n = n;
  b->cfg.assign(cfgs, cfgs + n);
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess) return fail(HTENO_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(HTENO_ERR_CUDA);
  b->own_stream = true;

  // state pool: q, q1, q2 of every instance, 256-byte aligned
  size_t total = 0;
  std::vector<size_t> off(n);
  b->ncell.resize(n);
  for (int i = 0; i < n; ++i) {
    b->ncell[i] = size_t(cfgs[i].nx) * cfgs[i].ny;
    off[i] = total;
    total += 3 * ((4 * b->ncell[i] * sizeof(double) + 255) & ~size_t(255));
  }
  if (cudaMalloc(&b->pool, total) != cudaSuccess) return fail(HTENO_ERR_OOM);
  if (cudaMalloc(&b->dstate, n * sizeof(StepState)) != cudaSuccess) return fail(HTENO_ERR_OOM);
  if (cudaMallocHost(&b->hstate, n * sizeof(StepState)) != cudaSuccess) return fail(HTENO_ERR_OOM);
  if (cudaMalloc(&b->dinst, n * sizeof(BInst)) != cudaSuccess) return fail(HTENO_ERR_OOM);
  b->hinst.resize(n);
  for (int i = 0; i < n; ++i) {
    const hteno_config& c = cfgs[i];
    BInst& I = b->hinst[i];
    I.G.nx = c.nx;
    I.G.ny = c.ny;
    I.G.bc = c.bc;
    I.G.recon = c.recon;
    I.G.flux = c.flux;
    I.G.dx = (c.xr - c.xl) / c.nx;
    I.G.dy = (c.yt - c.yb) / c.ny;
    I.G.area = I.G.dx * I.G.dy;
    I.G.gamma = c.gamma;
    I.G.g1 = c.gamma - 1.0;
    I.G.x0 = c.xl;
    I.G.y0 = c.yb;
    I.G.t0 = c.t_init;
    fill_bc_consts(c.gamma, I.G.bq, &I.G.ctan, &I.G.c16, &I.G.s3);
    const size_t bytes = (4 * b->ncell[i] * sizeof(double) + 255) & ~size_t(255);
    char* base = reinterpret_cast<char*>(b->pool) + off[i];
    I.q = reinterpret_cast<double*>(base);
    I.q1 = reinterpret_cast<double*>(base + bytes);
    I.q2 = reinterpret_cast<double*>(base + 2 * bytes);
    I.st = b->dstate + i;
    StepState& s = b->hstate[i];
    std::memset(&s, 0, sizeof(s));
    s.t = c.t_init;
    s.t_final = c.t_init;
    s.dt_scale = c.cfl * std::pow(std::fmin(I.G.dx, I.G.dy), 3.0 / 3.0);
  }
  if (cudaMemcpy(b->dinst, b->hinst.data(), n * sizeof(BInst), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->dstate, b->hstate, n * sizeof(StepState), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(b->pool, 0, total) != cudaSuccess)
    return fail(HTENO_ERR_CUDA);

  // job lists (instance, i0, j0) per tile shape; persistent grid = resident blocks on all SMs
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int v = 0; v < kNumBVariants; ++v) {
    const BVariant& V = kBVariants[v];
    int per_sm = 0;
    if (V.prepare(&per_sm) != cudaSuccess || per_sm < 1) return fail(HTENO_ERR_CUDA);
    std::vector<int4> jl;
    for (int i = 0; i < n; ++i)
      for (int j0 = 0; j0 < cfgs[i].ny; j0 += V.ty)
        for (int i0 = 0; i0 < cfgs[i].nx; i0 += V.tx) jl.push_back(make_int4(i, i0, j0, 0));
    b->njobs[v] = int(jl.size());
    b->grid[v] = std::max(1, std::min(int(jl.size()), sms * per_sm));
    if (cudaMalloc(&b->jobs[v], jl.size() * sizeof(int4)) != cudaSuccess) return fail(HTENO_ERR_OOM);
    if (cudaMemcpy(b->jobs[v], jl.data(), jl.size() * sizeof(int4), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(HTENO_ERR_CUDA);
  }
  const char* e = std::getenv("HTENO_FV2D_TILE");
  if (e && *e) {
    const int v = std::atoi(e);
    if (v >= 0 && v < kNumBVariants) b->forced = v;
  }
  const char* tma = std::getenv("HTENO_TMA");
  b->tma = !(tma && tma[0] == '0');
  *out = b;
  return HTENO_OK;
}

int hteno_batch_destroy(hteno_batch* b) {
  if (!b) return HTENO_ERR_INVALID_ARG;
  brelease(b);
  delete b;
  return HTENO_OK;
}

int hteno_batch_size(hteno_batch* b, int* n) {
  if (!b || !n) return HTENO_ERR_INVALID_ARG;
  *n = b->n;
  return HTENO_OK;
}

int hteno_batch_set_stream(hteno_batch* b, void* stream) {
  if (!b) return HTENO_ERR_INVALID_ARG;
  cudaStreamSynchronize(b->stream);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->stream = static_cast<cudaStream_t>(stream);
  b->own_stream = false;
  return HTENO_OK;
}

int hteno_batch_set_state(hteno_batch* b, int i, const double* q, int where) {
  if (!b || i < 0 || i >= b->n || !q) return HTENO_ERR_INVALID_ARG;
  const BInst& I = b->hinst[i];
  cudaError_t e = cudaMemcpyAsync(I.q, q, 4 * b->ncell[i] * sizeof(double),
                                  where == HTENO_DEVICE ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyHostToDevice,
                                  b->stream);
  StepState& s = b->hstate[i];
  std::memset(&s, 0, sizeof(s));
  s.t = b->cfg[i].t_init;
  s.t_final = b->cfg[i].t_init;
  s.dt_scale = b->cfg[i].cfl * std::pow(std::fmin(I.G.dx, I.G.dy), 3.0 / 3.0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->dstate + i, &s, sizeof(StepState), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) {
    k_inst_max_speed<<<64, 256, 0, b->stream>>>(b->dinst, i);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return bcuda(b, e, "batch set_state");
}

int hteno_batch_get_state(hteno_batch* b, int i, double* q, int where) {
  if (!b || i < 0 || i >= b->n || !q) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(q, b->hinst[i].q, 4 * b->ncell[i] * sizeof(double),
                                  where == HTENO_DEVICE ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyDeviceToHost,
                                  b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return bcuda(b, e, "batch get_state");
}

int hteno_batch_step_async(hteno_batch* b, int nsteps, double t_final) {
  if (!b || nsteps < 0) return HTENO_ERR_INVALID_ARG;
  int rc = ensure_graph(b);
  if (rc) return rc;
  k_batch_set_target<<<unsigned((b->n + 127) / 128), 128, 0, b->stream>>>(b->dstate, b->n, t_final);
  cudaError_t e = cudaGetLastError();
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) e = cudaGraphLaunch(b->graph, b->stream);
  return bcuda(b, e, "batch step launch");
}

int hteno_batch_sync(hteno_batch* b) {
  if (!b) return HTENO_ERR_INVALID_ARG;
  cudaError_t e = cudaMemcpyAsync(b->hstate, b->dstate, b->n * sizeof(StepState),
                                  cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return bcuda(b, e, "batch sync");
}

// Growing chunks of steps; stops issuing once every instance has reached t_final.
int hteno_batch_step(hteno_batch* b, int nsteps, double t_final) {
  if (!b || nsteps < 0) return HTENO_ERR_INVALID_ARG;
  int chunk = 32;
  for (int left = nsteps; left > 0;) {
    const int n = left < chunk ? left : chunk;
    int rc = hteno_batch_step_async(b, n, t_final);
    if (rc) return rc;
    rc = hteno_batch_sync(b);
    if (rc) return rc;
    left -= n;
    bool all = true;
    for (int i = 0; i < b->n && all; ++i)
      all = b->hstate[i].done || !(b->hstate[i].t < t_final);
    if (all) break;
    chunk = chunk < 1024 ? chunk * 2 : 1024;
  }
  return HTENO_OK;
}

int hteno_batch_get_time(hteno_batch* b, int i, double* t, long* steps, int* status) {
  if (!b || i < 0 || i >= b->n) return HTENO_ERR_INVALID_ARG;
  const StepState& s = b->hstate[i];
  if (t) *t = s.t;
  if (steps) *steps = long(s.steps);
  if (status) *status = s.status;
  return HTENO_OK;
}

int hteno_batch_get_counters(hteno_batch* b, int i, long long* counters) {
  if (!b || i < 0 || i >= b->n || !counters) return HTENO_ERR_INVALID_ARG;
  const StepState& s = b->hstate[i];
  counters[0] = (long long)s.uniform;
  counters[1] = (long long)s.tma_tiles;
  return HTENO_OK;
}

int hteno_batch_tile(hteno_batch* b, int* tx, int* ty, int* threads) {
  if (!b) return HTENO_ERR_INVALID_ARG;
  if (b->variant < 0) {
    const int rc = tune(b);
    if (rc) return rc;
  }
  const BVariant& V = kBVariants[b->variant];
  if (tx) *tx = V.tx;
  if (ty) *ty = V.ty;
  if (threads) *threads = V.nt;
  return HTENO_OK;
}

const char* hteno_batch_last_error(hteno_batch* b) { return b ? b->err.c_str() : "null handle"; }

}  // extern "C"
