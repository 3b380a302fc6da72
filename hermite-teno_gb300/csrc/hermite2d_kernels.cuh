// Kernels of FVHermite::System2D, templated on the compute type.  Included by hermite2d.cu
// (float instantiation, fused multiply-adds allowed) and hermite2d_fp64.cu (double
// instantiation, compiled with --fmad=false and routed through the bit-reproducible
// parity functions).  Each including translation unit owns its constant block.
#pragma once

#include <type_traits>

#include "hermite_math.cuh"
#include "hteno_internal.h"
#include "parity_math.cuh"

namespace hteno {

constexpr int kHFaceThreads = 128;
constexpr int kHFluxThreads = 64;

struct GeoH {
  int nx, ny;
  double dx, dy, area, gamma, g1, g3;  // g3 = gamma - 3 as the reference computes it
};

template <typename T>
struct WorkH {
  double* prim;   // [4][nc] u, v, h, sqrt|rho|
  double* vs;     // [4][nc] unlimited stage moments
  double* ws;
  T* xc;          // [24][ny][nx+1]: kind a (0 u-, 1 u+, 2 vn-, 3 vn+, 4 vt-, 5 vt+) x field r
  T* xroe;        // [7][ny][nx+1]
  T* yc;          // [24][ny+1][nx]
  T* yroe;        // [7][ny+1][nx]
  T* fx;          // [12][ny][nx+1]: kind (0 u, 1 moment along the sweep, 2 cross moment) x field
  T* fy;          // [12][ny+1][nx]
};

template <typename T>
size_t work_bytes_h(int nx, int ny) {
  const size_t nc = size_t(nx) * ny, nxf = size_t(nx + 1) * ny, nyf = size_t(ny + 1) * nx;
  return 12 * nc * sizeof(double) + (24 + 7 + 12) * (nxf + nyf) * sizeof(T) + 256 * 12;
}

template <typename T>
WorkH<T> carve_h(void* base, int nx, int ny) {
  const size_t nc = size_t(nx) * ny, nxf = size_t(nx + 1) * ny, nyf = size_t(ny + 1) * nx;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  WorkH<T> w;
  w.prim = reinterpret_cast<double*>(take(4 * nc * sizeof(double)));
  w.vs = reinterpret_cast<double*>(take(4 * nc * sizeof(double)));
  w.ws = reinterpret_cast<double*>(take(4 * nc * sizeof(double)));
  w.xc = reinterpret_cast<T*>(take(24 * nxf * sizeof(T)));
  w.xroe = reinterpret_cast<T*>(take(7 * nxf * sizeof(T)));
  w.yc = reinterpret_cast<T*>(take(24 * nyf * sizeof(T)));
  w.yroe = reinterpret_cast<T*>(take(7 * nyf * sizeof(T)));
  w.fx = reinterpret_cast<T*>(take(12 * nxf * sizeof(T)));
  w.fy = reinterpret_cast<T*>(take(12 * nyf * sizeof(T)));
  return w;
}

int hermite2d_fp64_setup(hteno_solver* s);
void hermite2d_fp64_step(hteno_solver* s, const GeoH& G);
void hermite2d_fp64_prim(hteno_solver* s, const GeoH& G);

namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

__device__ __forceinline__ void cell_prim(double g1, const double* q, double& u, double& v,
                                          double& p, double& h, double& sr) {
  u = q[1] / q[0];
  v = q[2] / q[0];
  p = (q[3] - 0.5 * (q[1] * u + q[2] * v)) * g1;
  h = (q[3] + p) / q[0];
  sr = sqrt(fabs(q[0]));
}
__device__ __forceinline__ double cell_max_speed(double gamma, double rho, double u, double v,
                                                 double p) {
  const double c = sqrt(fabs(gamma * p / rho));
  return fmax(fmax(u - c, fabs(u + c)), fmax(v - c, fabs(v + c)));
}

__global__ void kh_prim(GeoH G, const double* __restrict__ q, double* __restrict__ prim,
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

// Gauss-Seidel hermiteLimiter sweep.  DIR 1: line = row j, field e, walks i and updates v;
// DIR 2: line = column i, field e, walks j and updates w.  The neighbour beyond the last cell is
// the zero-gradient ghost, which holds the pre-sweep value.
template <typename T, int DIR>
__global__ void kh_limit(GeoH G, HermiteK<T> K, const double* __restrict__ q, double* d,
                         const StepState* st) {
  if (st->done) return;
  const int nl = DIR == 1 ? G.ny : G.nx;  // number of lines
  const int n = DIR == 1 ? G.nx : G.ny;   // length of a line
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 4 * nl) return;
  const int line = idx % nl, e = idx / nl;
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t stride = DIR == 1 ? 1 : size_t(G.nx);
  const size_t base = size_t(e) * nc + (DIR == 1 ? size_t(line) * G.nx : size_t(line));
  T um = T(q[base]), u0 = um, up;
  T dm = T(d[base]);                       // ghost before the first cell: old value of cell 0
  T dcur = dm;
  for (int s = 0; s < n; ++s) {
    const size_t o = base + size_t(s) * stride;
    const size_t on = base + size_t(s + 1 < n ? s + 1 : n - 1) * stride;
    up = T(q[on]);
    const T dn = T(d[on]);                 // not yet updated (or the ghost = old last value)
    T uu[3] = {um, u0, up};
    T dd[3] = {dm, dcur, dn};
    T lim;
    if constexpr (std::is_same<T, double>::value) lim = par::hermite_limiter(K, uu, dd);
    else lim = hermite_limiter(K, uu, dd);
    d[o] = double(lim);
    dm = lim;
    um = u0;
    u0 = up;
    dcur = dn;
  }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(kHFaceThreads) kh_faces(GeoH G, HermiteK<T> K,
                                                         const double* __restrict__ q,
                                                         const double* __restrict__ v,
                                                         const double* __restrict__ w,
                                                         const double* __restrict__ prim,
                                                         T* __restrict__ fc, T* __restrict__ froe,
                                                         const StepState* st) {
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (idx >= long(nf) * nt) return;
  int f, t;
  if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
  else { t = int(idx % nt); f = int(idx / nt); }
  const size_t nc = size_t(G.nx) * G.ny;
  const int ns = DIR == 1 ? G.nx : G.ny;
  auto cell = [&](int s) -> size_t {
    const int m = bmap(s, ns, HTENO_BC_ZEROGRAD);
    return DIR == 1 ? size_t(t) * G.nx + m : size_t(m) * G.nx + t;
  };
  const double* mn = DIR == 1 ? v : w;  // moment along the sweep (HTENO)
  const double* mt = DIR == 1 ? w : v;  // cross moment (TENO5)
  const size_t ca = cell(f - 1), cb = cell(f);
  const size_t nface = size_t(nf) * nt;
  const size_t o = DIR == 1 ? size_t(t) * nf + f : size_t(f) * nt + t;
  if constexpr (std::is_same<T, double>::value) {
    const par::Eig E = par::eig(G.g1, DIR, prim[3 * nc + ca], prim[ca], prim[nc + ca],
                                prim[2 * nc + ca], prim[3 * nc + cb], prim[cb], prim[nc + cb],
                                prim[2 * nc + cb]);
    {
      double A[4][4], B[4][4];
      for (int m = 0; m < 4; ++m) {
        const size_t c = cell(f - 2 + m);
        const double a4[4] = {q[c], q[nc + c], q[2 * nc + c], q[3 * nc + c]};
        const double b4[4] = {mn[c], mn[nc + c], mn[2 * nc + c], mn[3 * nc + c]};
        double ca4[4], cb4[4];
        par::left(E, DIR, a4, ca4);
        par::left(E, DIR, b4, cb4);
        for (int r = 0; r < 4; ++r) {
          A[r][m] = ca4[r];
          B[r][m] = cb4[r];
        }
      }
      for (int r = 0; r < 4; ++r) {
        double h[4];
        par::hermite_recon(c_dev, K, 0, A[r], B[r], h);
        for (int a = 0; a < 4; ++a) fc[(a * 4 + r) * nface + o] = h[a];
      }
    }
    {
      double C[4][6];
      for (int m = 0; m < 6; ++m) {
        const size_t c = cell(f - 3 + m);
        const double c4[4] = {mt[c], mt[nc + c], mt[2 * nc + c], mt[3 * nc + c]};
        double cc[4];
        par::left(E, DIR, c4, cc);
        for (int r = 0; r < 4; ++r) C[r][m] = cc[r];
      }
      for (int r = 0; r < 4; ++r) {
        double a, b;
        par::lagrange_recon(c_dev, HTENO_RECON_TENO5, C[r], a, b);
        fc[(4 * 4 + r) * nface + o] = a;
        fc[(5 * 4 + r) * nface + o] = b;
      }
    }
    froe[0 * nface + o] = E.vxm;
    froe[1 * nface + o] = E.vym;
    froe[2 * nface + o] = E.hm;
    froe[3 * nface + o] = E.qm;
    froe[4 * nface + o] = E.cm;
    froe[5 * nface + o] = E.rcm;
    froe[6 * nface + o] = E.b1;
    return;
  }
  const Roe2<T> R = roe2<T>(T(G.g1), T(prim[3 * nc + ca]), T(prim[ca]), T(prim[nc + ca]),
                            T(prim[2 * nc + ca]), T(prim[3 * nc + cb]), T(prim[cb]),
                            T(prim[nc + cb]), T(prim[2 * nc + cb]));
  {
    T A[4][4], B[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const size_t c = cell(f - 2 + m);
      T a4[4] = {T(q[c]), T(q[nc + c]), T(q[2 * nc + c]), T(q[3 * nc + c])};
      T b4[4] = {T(mn[c]), T(mn[nc + c]), T(mn[2 * nc + c]), T(mn[3 * nc + c])};
      T ca4[4], cb4[4];
      roe_left(R, DIR, a4, ca4);
      roe_left(R, DIR, b4, cb4);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        A[r][m] = ca4[r];
        B[r][m] = cb4[r];
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      T h[4];
      hermite_recon(c_dev, K, 0, A[r], B[r], h);
      fc[(0 * 4 + r) * nface + o] = h[0];
      fc[(1 * 4 + r) * nface + o] = h[1];
      fc[(2 * 4 + r) * nface + o] = h[2];
      fc[(3 * 4 + r) * nface + o] = h[3];
    }
  }
  {
    T C[4][6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const size_t c = cell(f - 3 + m);
      T c4[4] = {T(mt[c]), T(mt[nc + c]), T(mt[2 * nc + c]), T(mt[3 * nc + c])};
      T cc[4];
      roe_left(R, DIR, c4, cc);
#pragma unroll
      for (int r = 0; r < 4; ++r) C[r][m] = cc[r];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      T a, b;
      lagrange_recon(c_dev, HTENO_RECON_TENO5, C[r], a, b);
      fc[(4 * 4 + r) * nface + o] = a;
      fc[(5 * 4 + r) * nface + o] = b;
    }
  }
  froe[0 * nface + o] = R.vxm;
  froe[1 * nface + o] = R.vym;
  froe[2 * nface + o] = R.hm;
  froe[3 * nface + o] = R.qm;
  froe[4 * nface + o] = R.cm;
  froe[5 * nface + o] = R.rcm;
  froe[6 * nface + o] = R.b1;
}

template <typename T, int DIR>
__global__ void __launch_bounds__(kHFluxThreads) kh_flux(GeoH G, const T* __restrict__ fc,
                                                        const T* __restrict__ froe,
                                                        T* __restrict__ F, const StepState* st) {
  // GL3 values of the 24 face arrays at the 3 Gauss points, per thread, in shared memory
  __shared__ T sg[kHFluxThreads][24][3];
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  const bool live = idx < long(nf) * nt;
  int f = 0, t = 0;
  if (live) {
    if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
    else { t = int(idx % nt); f = int(idx / nt); }
  }
  const size_t nface = size_t(nf) * nt;
  auto fidx = [&](int tt) -> size_t {
    const int m = bmap(tt, nt, HTENO_BC_ZEROGRAD);
    return DIR == 1 ? size_t(m) * nf + f : size_t(f) * nt + m;
  };
  if (!live) return;
  size_t nb[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) nb[m] = fidx(t - 2 + m);
  T (*g)[3] = sg[threadIdx.x];
  for (int a = 0; a < 24; ++a) {
    T u5[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) u5[m] = fc[size_t(a) * nface + nb[m]];
    if constexpr (std::is_same<T, double>::value) par::gl3(c_dev, u5, g[a]);
    else gl3(c_dev, u5, g[a][0], g[a][1], g[a][2]);
  }
  const size_t o = nb[2];
  T acc[12];
  if constexpr (std::is_same<T, double>::value) {
    par::Eig E;
    E.vxm = froe[o];
    E.vym = froe[nface + o];
    E.hm = froe[2 * nface + o];
    E.qm = froe[3 * nface + o];
    E.cm = froe[4 * nface + o];
    E.rcm = froe[5 * nface + o];
    E.b1 = froe[6 * nface + o];
    const double vn = DIR == 1 ? E.vxm : E.vym;
    E.t0r = vn * E.cm;
    E.b2 = E.qm * E.b1;
    E.s0 = vn * E.rcm;
    E.s1 = E.b1 * vn;
    E.t2 = 0.5 * E.b1;
    double Fk[3][12];
    for (int m = 0; m < 3; ++m) {
      double X[6][4];
      for (int a = 0; a < 6; ++a) {
        const double c[4] = {g[4 * a + 0][m], g[4 * a + 1][m], g[4 * a + 2][m], g[4 * a + 3][m]};
        par::right(E, DIR, c, X[a]);
      }
      double fu[4], fn[4], ft[4];
      par::rusanov(G.gamma, G.g1, DIR, E, X[0], X[1], fu);
      par::drusanov(G.gamma, G.g1, G.g3, DIR, E, X[0], X[1], X[2], X[3], fn);
      par::drusanov(G.gamma, G.g1, G.g3, DIR, E, X[0], X[1], X[4], X[5], ft);
      const double wm = c_dev.gl3w[m];
      for (int k = 0; k < 4; ++k) {
        Fk[m][k] = wm * fu[k];
        Fk[m][4 + k] = wm * fn[k];
        Fk[m][8 + k] = wm * ft[k];
      }
    }
    for (int k = 0; k < 12; ++k) acc[k] = (Fk[0][k] + Fk[1][k]) + Fk[2][k];
  } else {
    Roe2<T> R;
    R.vxm = froe[o];
    R.vym = froe[nface + o];
    R.hm = froe[2 * nface + o];
    R.qm = froe[3 * nface + o];
    R.cm = froe[4 * nface + o];
    R.rcm = froe[5 * nface + o];
    R.b1 = froe[6 * nface + o];
    const T gm = T(G.gamma), g1 = T(G.g1);
    for (int m = 0; m < 3; ++m) {
      T X[6][4];
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        T c[4] = {g[4 * a + 0][m], g[4 * a + 1][m], g[4 * a + 2][m], g[4 * a + 3][m]};
        roe_right(R, DIR, c, X[a]);
      }
      T fu[4], fn[4], ft[4];
      rusanov2(gm, g1, DIR, R, X[0], X[1], fu);
      drusanov2(gm, g1, DIR, R, X[0], X[1], X[2], X[3], fn);
      drusanov2(gm, g1, DIR, R, X[0], X[1], X[4], X[5], ft);
      const T wm = Cst<T>::gl3w(c_dev, m);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        acc[k] = m == 0 ? wm * fu[k] : acc[k] + wm * fu[k];
        acc[4 + k] = m == 0 ? wm * fn[k] : acc[4 + k] + wm * fn[k];
        acc[8 + k] = m == 0 ? wm * ft[k] : acc[8 + k] + wm * ft[k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) F[size_t(k) * nface + o] = acc[k];
}

// rhs (:710-730) and RungeKutta3 (:733-782) for u, v, w
template <typename T>
__global__ void kh_update(GeoH G, int stage, const T* __restrict__ fx, const T* __restrict__ fy,
                          double* __restrict__ q, double* __restrict__ q0,
                          double* __restrict__ v, double* __restrict__ v0,
                          double* __restrict__ vs, double* __restrict__ w,
                          double* __restrict__ w0, double* __restrict__ ws,
                          double* __restrict__ prim, StepState* st) {
  if (st->done) return;
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  int bad = 0;
  if (k < nc) {
    const int i = int(k % G.nx), j = int(k / G.nx);
    const size_t nxf = size_t(G.nx + 1) * G.ny, nyf = size_t(G.ny + 1) * G.nx;
    const size_t ox = size_t(j) * (G.nx + 1) + i, oy = size_t(j) * G.nx + i;
    const double dt = st->dt;
    double qn[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      // kinds: x-sweep (0 u, 1 v, 2 w), y-sweep (0 u, 1 w, 2 v)
      const double ru = ((double(fx[(0 + e) * nxf + ox]) - double(fx[(0 + e) * nxf + ox + 1])) * G.dy +
                         (double(fy[(0 + e) * nyf + oy]) - double(fy[(0 + e) * nyf + oy + G.nx])) * G.dx) / G.area + 0.0;
      const double rv = ((double(fx[(4 + e) * nxf + ox]) - double(fx[(4 + e) * nxf + ox + 1])) * G.dy +
                         (double(fy[(8 + e) * nyf + oy]) - double(fy[(8 + e) * nyf + oy + G.nx])) * G.dx) / G.area + 0.0;
      const double rw = ((double(fx[(8 + e) * nxf + ox]) - double(fx[(8 + e) * nxf + ox + 1])) * G.dy +
                         (double(fy[(4 + e) * nyf + oy]) - double(fy[(4 + e) * nyf + oy + G.nx])) * G.dx) / G.area + 0.0;
      const size_t c = size_t(e) * nc + k;
      double bq, bv, bw, cq = q[c], cv, cw;
      if (stage == 1) {
        bq = cq; bv = v[c]; bw = w[c];   // save() after the first rhs: limited moments
        q0[c] = bq; v0[c] = bv; w0[c] = bw;
        cv = bv; cw = bw;
      } else {
        bq = q0[c]; bv = v0[c]; bw = w0[c];
        cv = vs[c]; cw = ws[c];          // unlimited stage values (cell.v1 / cell.v2)
      }
      qn[e] = ssprk3(bq, cq, ru, dt, stage);
      const double nv = ssprk3(bv, cv, rv, dt, stage);
      const double nw = ssprk3(bw, cw, rw, dt, stage);
      q[c] = qn[e];
      v[c] = nv;
      vs[c] = nv;
      w[c] = nw;
      ws[c] = nw;
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
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad) atomicOr(&st->status, bad);
}

GeoH geo_of(const hteno_solver* s) {
  GeoH G;
  G.nx = s->cfg.nx;
  G.ny = s->cfg.ny;
  G.dx = s->dx;
  G.dy = s->dy;
  G.area = s->dx * s->dy;
  G.gamma = s->cfg.gamma;
  G.g1 = s->cfg.gamma - 1.0;
  G.g3 = s->cfg.gamma - 3.0;
  return G;
}

template <typename T>
void launch_step(hteno_solver* s, const GeoH& G) {
  cudaStream_t cs = s->stream;
  const WorkH<T> W = carve_h<T>(s->work, G.nx, G.ny);
  const HermiteK<T> K = make_hermite_k<T>(s->dx);  // setGridSize(dx) for both directions
  const int nx = G.nx, ny = G.ny;
  const long nxf = long(nx + 1) * ny, nyf = long(ny + 1) * nx;
  const size_t nc = size_t(nx) * ny;
  const double ncd = double(nc);
  const int k_lx = trace_kind(s, "h_limit_x", ncd * 4 * 8 * 3, 0);
  const int k_ly = trace_kind(s, "h_limit_y", ncd * 4 * 8 * 3, 0);
  const int k_fx = trace_kind(s, "h_faces_x", ncd * 128 + double(nxf) * 31 * sizeof(T), 0);
  const int k_fy = trace_kind(s, "h_faces_y", ncd * 128 + double(nyf) * 31 * sizeof(T), 0);
  const int k_x = trace_kind(s, "h_flux_x", double(nxf) * 43 * sizeof(T), 0);
  const int k_y = trace_kind(s, "h_flux_y", double(nyf) * 43 * sizeof(T), 0);
  const int k_u = trace_kind(s, "h_update", ncd * 8 * 40 + double(nxf + nyf) * 12 * sizeof(T), 0);
  k_begin_step<<<1, 1, 0, cs>>>(s->dstate);
  for (int stage = 1; stage <= 3; ++stage) {
    trace_begin(s, k_lx);
    kh_limit<T, 1><<<unsigned((4 * ny + 63) / 64), 64, 0, cs>>>(G, K, s->q, s->v, s->dstate);
    trace_end(s);
    trace_begin(s, k_ly);
    kh_limit<T, 2><<<unsigned((4 * nx + 63) / 64), 64, 0, cs>>>(G, K, s->q, s->w, s->dstate);
    trace_end(s);
    trace_begin(s, k_fx);
    kh_faces<T, 1><<<unsigned((nxf + kHFaceThreads - 1) / kHFaceThreads), kHFaceThreads, 0, cs>>>(
        G, K, s->q, s->v, s->w, W.prim, W.xc, W.xroe, s->dstate);
    trace_end(s);
    trace_begin(s, k_fy);
    kh_faces<T, 2><<<unsigned((nyf + kHFaceThreads - 1) / kHFaceThreads), kHFaceThreads, 0, cs>>>(
        G, K, s->q, s->v, s->w, W.prim, W.yc, W.yroe, s->dstate);
    trace_end(s);
    trace_begin(s, k_x);
    kh_flux<T, 1><<<unsigned((nxf + kHFluxThreads - 1) / kHFluxThreads), kHFluxThreads, 0, cs>>>(
        G, W.xc, W.xroe, W.fx, s->dstate);
    trace_end(s);
    trace_begin(s, k_y);
    kh_flux<T, 2><<<unsigned((nyf + kHFluxThreads - 1) / kHFluxThreads), kHFluxThreads, 0, cs>>>(
        G, W.yc, W.yroe, W.fy, s->dstate);
    trace_end(s);
    trace_begin(s, k_u);
    kh_update<T><<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, stage, W.fx, W.fy, s->q, s->q0,
                                                            s->v, s->v0, W.vs, s->w, s->w0, W.ws,
                                                            W.prim, s->dstate);
    trace_end(s);
  }
  k_end_step<<<1, 1, 0, cs>>>(s->dstate);
}

}  // namespace
}  // namespace hteno
