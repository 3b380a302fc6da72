// FV::System1D on the GPU (FV_System1D.cpp:158-292): characteristic reconstruction (teno5,
// teno5i as shipped, or linear) from a 6-cell stencil, HLLC or characteristic Rusanov, SSP-RK3.
// One thread per face / per cell; a 1D grid of a few hundred cells is a latency case, so a step
// is 2 + 3 x 2 small launches that the host replays without synchronising (dt on the device).
// In double the bit-reproducible functions (parity_math.cuh) are used; compiled with
// --fmad=false.
#include <type_traits>

#include "hteno_internal.h"
#include "parity_math.cuh"
#include "harvest.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

constexpr int kThreads = 64;

struct Geo1 {
  int nx, bc, recon, flux;
  double dx, area, gamma, g1;
};

__device__ __forceinline__ void cell_prim1(double g1, const double* q, double* w, double& h,
                                           double& sr) {
  w[0] = q[0];
  w[1] = q[1] / q[0];
  w[2] = (q[2] - 0.5 * q[1] * w[1]) * g1;
  h = (q[2] + w[2]) / w[0];  // calcPrimitiveVariable (FV_System1D.cpp:95-119)
  sr = sqrt(fabs(w[0]));
}

__global__ void k1_init(Geo1 G, const double* __restrict__ q, StepState* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ms = 0.0;
  if (i < G.nx) {
    double qq[3] = {q[i], q[G.nx + i], q[2 * G.nx + i]}, w[3], h, sr;
    cell_prim1(G.g1, qq, w, h, sr);
    ms = par::max_speed1(G.gamma, w);
  }
  block_max_to(ms, &st->maxbits);
}

// face f in [0, nx] between cells f-1 and f (FV_System1D.cpp:194-235)
template <typename T>
__global__ void __launch_bounds__(kThreads) k1_flux(Geo1 G, const double* __restrict__ q,
                                                    T* __restrict__ F, const StepState* st) {
  if (st->done) return;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f > G.nx) return;
  const int n = G.nx;
  double qa[3], qb[3], wa[3], wb[3], ha, hb, sa, sb;
  const int ca = bmap(f - 1, n, G.bc), cb = bmap(f, n, G.bc);
  for (int v = 0; v < 3; ++v) {
    qa[v] = q[v * n + ca];
    qb[v] = q[v * n + cb];
  }
  cell_prim1(G.g1, qa, wa, ha, sa);
  cell_prim1(G.g1, qb, wb, hb, sb);
  T Ff[3];
  if constexpr (std::is_same<T, double>::value) {
    double R[9], L[9], ch[3][6];
    par::eig1(G.g1, sa, wa[1], ha, sb, wb[1], hb, R, L);
    for (int m = 0; m < 6; ++m) {
      const int c = bmap(f - 3 + m, n, G.bc);
      const double qq[3] = {q[c], q[n + c], q[2 * n + c]};
      double cc[3];
      par::mv3(L, qq, cc);
      for (int r = 0; r < 3; ++r) ch[r][m] = cc[r];
    }
    double cl[3], cr[3], ql[3], qr[3];
    for (int r = 0; r < 3; ++r) par::lagrange_recon(c_dev, G.recon, ch[r], cl[r], cr[r]);
    par::mv3(R, cl, ql);  // transformToConservative (FV_System1D.h:48-51)
    par::mv3(R, cr, qr);
    if (G.flux == HTENO_FLUX_HLLC) par::hllc1(G.g1, ql, qr, Ff);
    else par::rusanov1(G.gamma, G.g1, L, R, ql, qr, Ff);
  } else {
    const Roe1<T> R = roe1<T>(T(G.g1), T(sa), T(wa[1]), T(ha), T(sb), T(wb[1]), T(hb));
    T ch[3][6];
    for (int m = 0; m < 6; ++m) {
      const int c = bmap(f - 3 + m, n, G.bc);
      T qq[3] = {T(q[c]), T(q[n + c]), T(q[2 * n + c])}, cc[3];
      roe1_left(R, qq, cc);
      for (int r = 0; r < 3; ++r) ch[r][m] = cc[r];
    }
    T cl[3], cr[3], ql[3], qr[3];
    for (int r = 0; r < 3; ++r) lagrange_recon(c_dev, G.recon, ch[r], cl[r], cr[r]);
    roe1_right(R, cl, ql);
    roe1_right(R, cr, qr);
    if (G.flux == HTENO_FLUX_HLLC) hllc1(T(G.g1), ql, qr, Ff);
    else rusanov1(T(G.gamma), T(G.g1), R, ql, qr, Ff);
  }
  for (int v = 0; v < 3; ++v) F[v * (n + 1) + f] = Ff[v];
}

// The FP64 face kernel with the work of a face spread over 8 lanes: lane l = r + 4 s (r < 3 the
// characteristic field, s the side) projects its field's 6-cell stencil and reconstructs one side;
// the group's lane 0 gathers the six values, projects back and computes the flux.  A 1D grid has
// a few hundred faces: spreading each face's FP64 work over more lanes and warps (hence SMs)
// shortens the step; every value is computed with the same operations as in k1_flux.
__global__ void __launch_bounds__(kThreads) k1_flux_lanes(Geo1 G, const double* __restrict__ q,
                                                          double* __restrict__ F,
                                                          const StepState* st) {
  if (st->done) return;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = gid >> 3, l = gid & 7;
  const bool live = f <= G.nx;
  const int fc = live ? f : G.nx;  // lanes past the last face compute that face, store nothing
  const int n = G.nx;
  double qa[3], qb[3], wa[3], wb[3], ha, hb, sa, sb;
  const int ca = bmap(fc - 1, n, G.bc), cb = bmap(fc, n, G.bc);
  for (int v = 0; v < 3; ++v) {
    qa[v] = q[v * n + ca];
    qb[v] = q[v * n + cb];
  }
  cell_prim1(G.g1, qa, wa, ha, sa);
  cell_prim1(G.g1, qb, wb, hb, sb);
  double R[9], L[9];
  par::eig1(G.g1, sa, wa[1], ha, sb, wb[1], hb, R, L);
  const int r = l & 3, side = l >> 2;
  double val = 0.0;
  if (r < 3) {
    double ch[6];
    for (int m = 0; m < 6; ++m) {
      const int c = bmap(fc - 3 + m, n, G.bc);
      double sum = L[3 * r] * q[c];  // row r of par::mv3
      sum = sum + L[3 * r + 1] * q[n + c];
      sum = sum + L[3 * r + 2] * q[2 * n + c];
      ch[m] = sum;
    }
    val = par::lagrange_side(c_dev, G.recon, ch, side);
  }
  const int base = int(threadIdx.x & 31u) & ~7;
  double cl[3], cr[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    cl[k] = __shfl_sync(0xffffffffu, val, base + k);
    cr[k] = __shfl_sync(0xffffffffu, val, base + 4 + k);
  }
  if (l != 0 || !live) return;
  double ql[3], qr[3], Ff[3];
  par::mv3(R, cl, ql);  // transformToConservative (FV_System1D.h:48-51)
  par::mv3(R, cr, qr);
  if (G.flux == HTENO_FLUX_HLLC) par::hllc1(G.g1, ql, qr, Ff);
  else par::rusanov1(G.gamma, G.g1, L, R, ql, qr, Ff);
  for (int v = 0; v < 3; ++v) F[v * (n + 1) + f] = Ff[v];
}

// rhs (FV_System1D.cpp:237-240) + RungeKutta3 (:243-272); max wave speed on the last stage
template <typename T>
__global__ void k1_update(Geo1 G, int stage, const T* __restrict__ F, double* __restrict__ q,
                          double* __restrict__ q0, StepState* st) {
  if (st->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = G.nx;
  double ms = 0.0;
  int bad = 0;
  if (i < n) {
    const double dt = st->dt;
    double qn[3];
    for (int v = 0; v < 3; ++v) {
      const double rhs = (double(F[v * (n + 1) + i]) - double(F[v * (n + 1) + i + 1])) / G.area;
      const double cur = q[v * n + i];
      double base;
      if (stage == 1) {
        q0[v * n + i] = cur;
        base = cur;
      } else {
        base = q0[v * n + i];
      }
      qn[v] = ssprk3(base, cur, rhs, dt, stage);
      q[v * n + i] = qn[v];
    }
    double w[3], h, sr;
    cell_prim1(G.g1, qn, w, h, sr);
    if (stage == 3) ms = par::max_speed1(G.gamma, w);
    bad = (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2])) ? 1 : 0;
    bad |= (qn[0] <= 0.0 || w[2] <= 0.0) ? 2 : 0;
  }
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad) atomicOr(&st->status, bad);
}

// Training stencils of the learned classifier (harvest.cuh): every face, 3 characteristic
// fields, both sides, each kept with probability p.
__global__ void __launch_bounds__(kThreads) k1_harvest(Geo1 G, const double* __restrict__ q, double p,
                                                       unsigned long long seed, uint16_t* X, uint8_t* Y,
                                                       long cap, unsigned long long* count) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f > G.nx) return;
  const int n = G.nx;
  double qa[3], qb[3], wa[3], wb[3], ha, hb, sa, sb;
  const int ca = bmap(f - 1, n, G.bc), cb = bmap(f, n, G.bc);
  for (int v = 0; v < 3; ++v) {
    qa[v] = q[v * n + ca];
    qb[v] = q[v * n + cb];
  }
  cell_prim1(G.g1, qa, wa, ha, sa);
  cell_prim1(G.g1, qb, wb, hb, sb);
  double R[9], L[9], ch[3][6];
  par::eig1(G.g1, sa, wa[1], ha, sb, wb[1], hb, R, L);
  for (int m = 0; m < 6; ++m) {
    const int c = bmap(f - 3 + m, n, G.bc);
    const double qq[3] = {q[c], q[n + c], q[2 * n + c]};
    double cc[3];
    par::mv3(L, qq, cc);
    for (int r = 0; r < 3; ++r) ch[r][m] = cc[r];
  }
  for (int r = 0; r < 3; ++r)
    harvest::emit_both(ch[r], G.recon == HTENO_RECON_TENO5I, seed, (uint64_t(r) << 40) + uint64_t(f),
                       p, X, Y, cap, count);
}

// KXRCF troubled-cell sensor of FV::System1D::rhs (FV_System1D.cpp:166-192): from the density
// averages, the two one-sided face values of the upwind face (chosen by the sign of rho*u),
// flagged when |h1 - h2| / ((dx/2)^1.5 |rho_i|) > 1.  The reference computes the flag for cells
// s+1 .. nxx-s-2 of its ghost-padded array (every interior cell) and reconstructs with teno5i
// either way; here the flags are an output.
__global__ void k1_kxrcf(Geo1 G, const double* __restrict__ q, double crm, uint8_t* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G.nx) return;
  const int n = G.nx;
  auto rho = [&](int k) { return q[bmap(k, n, G.bc)]; };
  double h1, h2;
  if (q[n + i] < 0.0) {
    h1 = (2.0 * rho(i - 1) + 5.0 * rho(i) - rho(i + 1)) / 6.0;
    h2 = (-rho(i - 2) + 5.0 * rho(i - 1) + 2.0 * rho(i)) / 6.0;
  } else {
    h2 = (2.0 * rho(i) + 5.0 * rho(i + 1) - rho(i + 2)) / 6.0;
    h1 = (-rho(i - 1) + 5.0 * rho(i) + 2.0 * rho(i + 1)) / 6.0;
  }
  flag[i] = fabs(h1 - h2) / (crm * fabs(rho(i))) > 1.0 ? 1 : 0;
}

Geo1 geo1_of(const hteno_solver* s) {
  Geo1 G;
  G.nx = s->cfg.nx;
  G.bc = s->cfg.bc;
  G.recon = s->cfg.recon;
  G.flux = s->cfg.flux;
  G.dx = s->dx;
  G.area = s->dx;
  G.gamma = s->cfg.gamma;
  G.g1 = s->cfg.gamma - 1.0;
  return G;
}

template <typename T>
void launch_step(hteno_solver* s, const Geo1& G, cudaStream_t cs) {
  const unsigned gf = unsigned((G.nx + 1 + kThreads - 1) / kThreads);
  const unsigned gc = unsigned((G.nx + kThreads - 1) / kThreads);
  T* F = static_cast<T*>(s->work);
  k_begin_step<<<1, 1, 0, cs>>>(s->dstate);
  const unsigned gl = unsigned((8 * (G.nx + 1) + kThreads - 1) / kThreads);
  for (int stage = 1; stage <= 3; ++stage) {
    if constexpr (std::is_same<T, double>::value)
      k1_flux_lanes<<<gl, kThreads, 0, cs>>>(G, s->q, F, s->dstate);
    else
      k1_flux<T><<<gf, kThreads, 0, cs>>>(G, s->q, F, s->dstate);
    k1_update<T><<<gc, kThreads, 0, cs>>>(G, stage, F, s->q, s->q0, s->dstate);
  }
  k_end_step<<<1, 1, 0, cs>>>(s->dstate);
}

// A 1D step is 8 small launches whose CPU launch cost exceeds their GPU time; runs of
// kGraphSteps steps are captured once into a graph (the solver's buffers are fixed) and replayed.
constexpr int kGraphSteps = 16;

void launch_steps(hteno_solver* s, const Geo1& G, int n, cudaStream_t cs) {
  for (int k = 0; k < n; ++k) {
    if (s->cfg.precision == HTENO_PREC_MIXED) launch_step<float>(s, G, cs);
    else launch_step<double>(s, G, cs);
  }
}

cudaError_t ensure_graph(hteno_solver* s, const Geo1& G) {
  if (s->step_graph) return cudaSuccess;
  cudaStream_t cap;
  cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  cudaGraph_t g = nullptr;
  e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    launch_steps(s, G, kGraphSteps, cap);
    e = cudaStreamEndCapture(cap, &g);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&s->step_graph, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cap);
  return e;
}

}  // namespace

int fv1d_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  s->work_bytes = 3 * size_t(s->cfg.nx + 1) * sizeof(double);
  cudaError_t e = cudaMalloc(&s->work, s->work_bytes);
  if (e != cudaSuccess) return cuda_error(s, e, "work buffer");
  s->launches_per_step = 2 + 3 * 2;
  return HTENO_OK;
}

int fv1d_prepare(hteno_solver* s) {
  const Geo1 G = geo1_of(s);
  k1_init<<<unsigned((G.nx + 127) / 128), 128, 0, s->stream>>>(G, s->q, s->dstate);
  return cuda_error(s, cudaGetLastError(), "k1_init");
}

int fv1d_harvest(hteno_solver* s, double p, unsigned long long seed, uint16_t* X, uint8_t* Y,
                 long cap, unsigned long long* count) {
  const Geo1 G = geo1_of(s);
  k1_harvest<<<unsigned((G.nx + 1 + kThreads - 1) / kThreads), kThreads, 0, s->stream>>>(
      G, s->q, p, seed, X, Y, cap, count);
  return cuda_error(s, cudaGetLastError(), "harvest");
}

int fv1d_kxrcf(hteno_solver* s, uint8_t* flags) {
  const Geo1 G = geo1_of(s);
  const double crm = pow(G.dx / 2.0, 1.5);  // circleRadMod (FV_System1D.cpp:19)
  k1_kxrcf<<<unsigned((G.nx + kThreads - 1) / kThreads), kThreads, 0, s->stream>>>(G, s->q, crm, flags);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  return cuda_error(s, e, "kxrcf");
}

int fv1d_step_async(hteno_solver* s, int nsteps) {
  const Geo1 G = geo1_of(s);
  int left = nsteps;
  if (!s->timing && nsteps >= kGraphSteps) {  // per-kernel timing needs the plain launches
    const cudaError_t e = ensure_graph(s, G);
    if (e != cudaSuccess) return cuda_error(s, e, "fv1d step graph");
    for (; left >= kGraphSteps; left -= kGraphSteps) {
      const cudaError_t el = cudaGraphLaunch(s->step_graph, s->stream);
      if (el != cudaSuccess) return cuda_error(s, el, "fv1d graph launch");
    }
  }
  launch_steps(s, G, left, s->stream);
  return cuda_error(s, cudaGetLastError(), "fv1d step launch");
}

}  // namespace hteno
