// FV::System2D on the GPU (FV_System2D.cpp:363-651): characteristic TENO5 per direction,
// transverse three-point Gauss-Legendre WENO5-JS along each face, HLLC or characteristic
// Rusanov at the Gauss points, SSP-RK3.  This file holds the host dispatch and the mixed path
// (T = float for reconstruction and fluxes; the conserved state, its step-start copy, the
// primitive recovery and the RK update stay double).  The plain FP64 path is the
// bit-reproducible one in fv2d_fp64.cu.
//
// One stage = 5 launches, one step = 3 stages + 2 bookkeeping launches:
//   faces<X>, faces<Y> : Roe average -> L, project the 6-cell stencil, TENO5 both sides for the
//                        4 characteristic fields (stored per face, face basis)
//   flux<X>,  flux<Y>  : GL3 over the 5 faces j-2..j+2 (each in its own basis, as the reference
//                        does), R back-projection, flux at 3 Gauss points, quadrature sum
//   update             : flux difference, SSP-RK3 stage, primitives of the new state and, on the
//                        last stage, the max wave speed that sets the next dt
// The host never synchronises inside hteno_step: dt, t and the stop flag live on the device.
#include <algorithm>

#include "fv2d_common.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

// primitives of one cell: calcPrimitiveVariable (FV_System2D.cpp:226-263)
__device__ __forceinline__ void cell_prim(double g1, const double* q, double& u, double& v,
                                          double& p, double& h, double& sr) {
  u = q[1] / q[0];
  v = q[2] / q[0];
  p = (q[3] - 0.5 * (q[1] * u + q[2] * v)) * g1;
  h = (q[3] + p) / q[0];
  sr = sqrt(fabs(q[0]));
}

// maxSpeed over both directions (Equations_Euler2D.cpp:207-219; timeStepping :625-633)
__device__ __forceinline__ double cell_max_speed(double gamma, double rho, double u, double v,
                                                 double p) {
  const double c = sqrt(fabs(gamma * p / rho));
  return fmax(fmax(u - c, fabs(u + c)), fmax(v - c, fabs(v + c)));
}

__global__ void k_prim(Geo G, const double* __restrict__ q, double* __restrict__ prim,
                       StepState* st, int do_max) {
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  if (k < nc) {
    double qq[4] = {q[k], q[nc + k], q[2 * nc + k], q[3 * nc + k]};
    double u, v, p, h, sr;
    cell_prim(G.g1, qq, u, v, p, h, sr);
    prim[k] = u;
    prim[nc + k] = v;
    prim[2 * nc + k] = h;
    prim[3 * nc + k] = sr;
    ms = cell_max_speed(G.gamma, qq[0], u, v, p);
  }
  if (do_max) block_max_to(ms, &st->maxbits);
}

// ---- face reconstruction -------------------------------------------------------------------
// DIR 1: faces f in [0, nx] between cells (f-1, j) and (f, j); DIR 2: faces g in [0, ny]
// between (i, g-1) and (i, g).  Stencil cells f-3 .. f+2 along the sweep (FV_System2D.cpp:
// 372-400), boundary-mapped.
template <typename T, int DIR>
__global__ void __launch_bounds__(kFaceThreads) k_faces(Geo G, const double* __restrict__ q,
                                                        const double* __restrict__ prim,
                                                        T* __restrict__ fc, T* __restrict__ froe,
                                                        const StepState* st) {
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;  // faces along the sweep
  const int nt = DIR == 1 ? G.ny : G.nx;          // transverse extent
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (idx >= long(nf) * nt) return;
  int f, t;
  if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
  else { t = int(idx % nt); f = int(idx / nt); }
  const size_t nc = size_t(G.nx) * G.ny;
  const int ns = DIR == 1 ? G.nx : G.ny;
  auto cell = [&](int s) -> size_t {
    const int m = bmap(s, ns, G.bc);
    return DIR == 1 ? size_t(t) * G.nx + m : size_t(m) * G.nx + t;
  };
  const size_t ca = cell(f - 1), cb = cell(f);
  const Roe2<T> R = roe2<T>(T(G.g1), T(prim[3 * nc + ca]), T(prim[ca]), T(prim[nc + ca]),
                            T(prim[2 * nc + ca]), T(prim[3 * nc + cb]), T(prim[cb]),
                            T(prim[nc + cb]), T(prim[2 * nc + cb]));
  T ch[4][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const size_t c = cell(f - 3 + m);
    T qq[4] = {T(q[c]), T(q[nc + c]), T(q[2 * nc + c]), T(q[3 * nc + c])};
    T cc[4];
    roe_left(R, DIR, qq, cc);
#pragma unroll
    for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
  }
  const size_t nface = size_t(nf) * nt;
  const size_t o = DIR == 1 ? size_t(t) * nf + f : size_t(f) * nt + t;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    T a, b;
    lagrange_recon(c_dev, G.recon, ch[r], a, b);
    fc[r * nface + o] = a;
    fc[(4 + r) * nface + o] = b;
  }
  froe[0 * nface + o] = R.vxm;
  froe[1 * nface + o] = R.vym;
  froe[2 * nface + o] = R.hm;
  froe[3 * nface + o] = R.qm;
  froe[4 * nface + o] = R.cm;
  froe[5 * nface + o] = R.rcm;
  froe[6 * nface + o] = R.b1;
}

// ---- transverse quadrature + flux ------------------------------------------------------------
template <typename T, int DIR>
__global__ void __launch_bounds__(kFaceThreads) k_flux(Geo G, const T* __restrict__ fc,
                                                       const T* __restrict__ froe,
                                                       T* __restrict__ F, const StepState* st) {
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (idx >= long(nf) * nt) return;
  int f, t;
  if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
  else { t = int(idx % nt); f = int(idx / nt); }
  const size_t nface = size_t(nf) * nt;
  auto fidx = [&](int tt) -> size_t {
    const int m = bmap(tt, nt, G.bc);
    return DIR == 1 ? size_t(m) * nf + f : size_t(f) * nt + m;
  };
  size_t nb[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) nb[m] = fidx(t - 2 + m);
  T g[8][3];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    T u5[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) u5[m] = fc[r * nface + nb[m]];
    gl3(c_dev, u5, g[r][0], g[r][1], g[r][2]);
  }
  const size_t o = nb[2];
  Roe2<T> R;
  R.vxm = froe[o];
  R.vym = froe[nface + o];
  R.hm = froe[2 * nface + o];
  R.qm = froe[3 * nface + o];
  R.cm = froe[4 * nface + o];
  R.rcm = froe[5 * nface + o];
  R.b1 = froe[6 * nface + o];
  T acc[4];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    T cl[4] = {g[0][m], g[1][m], g[2][m], g[3][m]};
    T cr[4] = {g[4][m], g[5][m], g[6][m], g[7][m]};
    T ql[4], qr[4], Fm[4];
    roe_right(R, DIR, cl, ql);
    roe_right(R, DIR, cr, qr);
    if (G.flux == HTENO_FLUX_HLLC) hllc2(T(G.g1), DIR, ql, qr, Fm);
    else rusanov2(T(G.gamma), T(G.g1), DIR, R, ql, qr, Fm);
    const T wm = Cst<T>::gl3w(c_dev, m);
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[v] = m == 0 ? wm * Fm[v] : acc[v] + wm * Fm[v];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) F[v * nface + o] = acc[v];
}

// ---- residual + SSP-RK3 stage ----------------------------------------------------------------
// rhs (FV_System2D.cpp:562-572), RungeKutta3 (:575-612), calcPrimitiveVariable of the result.
// stage 0 writes the residual itself to out (hteno_residual).
template <typename T>
__global__ void k_update(Geo G, int stage, const T* __restrict__ fx, const T* __restrict__ fy,
                         double* __restrict__ q, double* __restrict__ q0,
                         double* __restrict__ prim, double* __restrict__ out, StepState* st) {
  if (st && st->done) return;
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  int bad = 0;
  if (k < nc) {
    const int i = int(k % G.nx), j = int(k / G.nx);
    const size_t nxf = size_t(G.nx + 1) * G.ny, nyf = size_t(G.ny + 1) * G.nx;
    const size_t ox = size_t(j) * (G.nx + 1) + i, oy = size_t(j) * G.nx + i;
    double rhs[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double dfx = double(fx[v * nxf + ox]) - double(fx[v * nxf + ox + 1]);
      const double dfy = double(fy[v * nyf + oy]) - double(fy[v * nyf + oy + G.nx]);
      rhs[v] = (dfx * G.dy + dfy * G.dx) / G.area;
    }
    if (stage == 0) {
#pragma unroll
      for (int v = 0; v < 4; ++v) out[v * nc + k] = rhs[v];
    } else {
      const double dt = st->dt;
      double qn[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double cur = q[v * nc + k];
        double base;
        if (stage == 1) {
          q0[v * nc + k] = cur;
          base = cur;
        } else {
          base = q0[v * nc + k];
        }
        qn[v] = ssprk3(base, cur, rhs[v], dt, stage);
        q[v * nc + k] = qn[v];
      }
      double u, vv, p, h, sr;
      cell_prim(G.g1, qn, u, vv, p, h, sr);
      prim[k] = u;
      prim[nc + k] = vv;
      prim[2 * nc + k] = h;
      prim[3 * nc + k] = sr;
      if (stage == 3) ms = cell_max_speed(G.gamma, qn[0], u, vv, p);
      bad = (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2]) || isnan(qn[3])) ? 1 : 0;
      bad |= (qn[0] <= 0.0 || p <= 0.0) ? 2 : 0;
    }
  }
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad && st) atomicOr(&st->status, bad);
}

template <typename T>
int launch_stage(hteno_solver* s, const Geo& G, const Work<T>& W, int stage, const double* q,
                 double* out) {
  cudaStream_t cs = s->stream;
  const int nx = G.nx, ny = G.ny;
  const long nxf = long(nx + 1) * ny, nyf = long(ny + 1) * nx;
  const double nc_d = double(nx) * ny;
  StepState* st = stage == 0 ? nullptr : s->dstate;
  const double fluxf = G.flux == HTENO_FLUX_HLLC ? kFluxFlopsHllc : kFluxFlopsRusanov;
  // compulsory DRAM bytes: faces read q + primitives once per cell and write 15 values per face;
  // flux reads 15 and writes 4 values per face; update reads fluxes, q, q0 and writes q, prims
  const int kf_x = trace_kind(s, "faces_x", nc_d * 64 + double(nxf) * 15 * sizeof(T), kFacesFlops * nxf);
  const int kf_y = trace_kind(s, "faces_y", nc_d * 64 + double(nyf) * 15 * sizeof(T), kFacesFlops * nyf);
  const int kx = trace_kind(s, "flux_x", double(nxf) * 19 * sizeof(T), fluxf * nxf);
  const int ky = trace_kind(s, "flux_y", double(nyf) * 19 * sizeof(T), fluxf * nyf);
  const int ku = trace_kind(s, "update", nc_d * 128 + double(nxf + nyf) * 4 * sizeof(T),
                            kUpdateFlops * nc_d);
  trace_begin(s, kf_x);
  k_faces<T, 1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, q, W.prim, W.xc, W.xroe, st);
  trace_end(s);
  trace_begin(s, kf_y);
  k_faces<T, 2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, q, W.prim, W.yc, W.yroe, st);
  trace_end(s);
  trace_begin(s, kx);
  k_flux<T, 1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, W.xc, W.xroe, W.fx, st);
  trace_end(s);
  trace_begin(s, ky);
  k_flux<T, 2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, W.yc, W.yroe, W.fy, st);
  trace_end(s);
  const size_t nc = size_t(nx) * ny;
  trace_begin(s, ku);
  k_update<T><<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, stage, W.fx, W.fy, s->q, s->q0,
                                                         W.prim, out, st);
  trace_end(s);
  return HTENO_OK;
}

Geo geo_of(const hteno_solver* s) {
  Geo G;
  G.nx = s->cfg.nx;
  G.ny = s->cfg.ny;
  G.bc = s->cfg.bc;
  G.recon = s->cfg.recon;
  G.flux = s->cfg.flux;
  G.dx = s->dx;
  G.dy = s->dy;
  G.area = s->dx * s->dy;
  G.gamma = s->cfg.gamma;
  G.g1 = s->cfg.gamma - 1.0;
  return G;
}

}  // namespace

int fv2d_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  if (fv2d_fp64_setup(s) != HTENO_OK) return HTENO_ERR_CUDA;
  const int nx = s->cfg.nx, ny = s->cfg.ny;
  s->work_bytes = s->cfg.precision == HTENO_PREC_MIXED ? work_bytes<float>(nx, ny)
                                                       : work_bytes<double>(nx, ny);
  cudaError_t e = cudaMalloc(&s->work, s->work_bytes);
  if (e != cudaSuccess) return cuda_error(s, e, "work buffer");
  s->launches_per_step = 2 + 3 * 5;
  return HTENO_OK;
}

int fv2d_prepare(hteno_solver* s) {
  const Geo G = geo_of(s);
  const size_t nc = size_t(G.nx) * G.ny;
  if (s->cfg.precision == HTENO_PREC_MIXED)
    k_prim<<<unsigned((nc + 255) / 256), 256, 0, s->stream>>>(G, s->q, carve<float>(s->work, G.nx, G.ny).prim,
                                                             s->dstate, 1);
  else
    fv2d_fp64_prim(s, G, carve<double>(s->work, G.nx, G.ny), s->q, s->dstate, 1);
  return cuda_error(s, cudaGetLastError(), "primitives");
}

int fv2d_step_async(hteno_solver* s, int nsteps) {
  const Geo G = geo_of(s);
  for (int n = 0; n < nsteps; ++n) {
    k_begin_step<<<1, 1, 0, s->stream>>>(s->dstate);
    for (int stage = 1; stage <= 3; ++stage) {
      if (s->cfg.precision == HTENO_PREC_MIXED)
        launch_stage(s, G, carve<float>(s->work, G.nx, G.ny), stage, s->q, nullptr);
      else
        fv2d_fp64_stage(s, G, carve<double>(s->work, G.nx, G.ny), stage, s->q, nullptr);
    }
    k_end_step<<<1, 1, 0, s->stream>>>(s->dstate);
  }
  return cuda_error(s, cudaGetLastError(), "fv2d step launch");
}

int fv2d_residual(hteno_solver* s, const double* q, double* rhs) {
  const Geo G = geo_of(s);
  const size_t nc = size_t(G.nx) * G.ny;
  if (s->cfg.precision == HTENO_PREC_MIXED) {
    Work<float> W = carve<float>(s->work, G.nx, G.ny);
    k_prim<<<unsigned((nc + 255) / 256), 256, 0, s->stream>>>(G, q, W.prim, s->dstate, 0);
    launch_stage(s, G, W, 0, q, rhs);
  } else {
    Work<double> W = carve<double>(s->work, G.nx, G.ny);
    fv2d_fp64_prim(s, G, W, q, nullptr, 0);
    fv2d_fp64_stage(s, G, W, 0, q, rhs);
  }
  return cuda_error(s, cudaGetLastError(), "fv2d residual launch");
}

}  // namespace hteno
