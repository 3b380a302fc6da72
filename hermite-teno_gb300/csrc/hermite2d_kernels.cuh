// Kernels of FVHermite::System2D, templated on the compute type.  Included by hermite2d.cu
// (float instantiation, fused multiply-adds allowed) and hermite2d_fp64.cu (double
// instantiation, compiled with --fmad=false and routed through the bit-reproducible
// parity functions).  Each including translation unit owns its constant block.
#pragma once

#include <type_traits>

#include "hermite_math.cuh"
#include "hteno_internal.h"
#include "mixed_conv.cuh"
#include "parity_math.cuh"

namespace hteno {

constexpr int kHFaceThreads = 128;
constexpr int kHFluxThreads = 64;

struct GeoH {
  int nx, ny;
  double dx, dy, area, gamma, g1, g3;  // g3 = gamma - 3 as the reference computes it
  double rdx, rdy;                     // 1/dx, 1/dy
  float rdxf, rdyf;                    // the same in float (mixed-precision update)
};

// Loads of the double state into the compute type and back: for float on the integer pipes
// (mix::d2f / f2d), for double the identity.
template <typename T>
__device__ __forceinline__ T from_d(double x) {
  if constexpr (std::is_same<T, float>::value) return mix::d2f(x);
  else return x;
}
template <typename T>
__device__ __forceinline__ double to_d(T x) {
  if constexpr (std::is_same<T, float>::value) return mix::f2d(x);
  else return x;
}

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
  // the state as the face kernels read it, in the compute type: for double the state arrays
  // themselves (set by the launcher); for float copies written by the kernels that produce the
  // state (update, limiter), so each cell is converted once per stage, not once per stencil use
  T* qt;          // [4][nc]
  T* vt;          // [4][nc] limited moments
  T* wt;
  T* primt;       // [4][nc] u, v, h, sqrt|rho|
};

template <typename T>
size_t work_bytes_h(int nx, int ny) {
  const size_t nc = size_t(nx) * ny, nxf = size_t(nx + 1) * ny, nyf = size_t(ny + 1) * nx;
  const size_t copies = std::is_same<T, float>::value ? 16 * nc * sizeof(float) + 256 * 4 : 0;
  return 12 * nc * sizeof(double) + (24 + 7 + 12) * (nxf + nyf) * sizeof(T) + 256 * 12 + copies;
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
  w.qt = nullptr;
  w.vt = w.wt = w.primt = nullptr;
  if constexpr (std::is_same<T, float>::value) {
    w.qt = reinterpret_cast<T*>(take(4 * nc * sizeof(T)));
    w.vt = reinterpret_cast<T*>(take(4 * nc * sizeof(T)));
    w.wt = reinterpret_cast<T*>(take(4 * nc * sizeof(T)));
    w.primt = reinterpret_cast<T*>(take(4 * nc * sizeof(T)));
  }
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

// Mixed precision, after a new state: the float copies of the state and of its primitives that
// the face kernels read, and the first dt's max wave speed.
__global__ void kh_prim_f(GeoH G, const double* __restrict__ q, float* __restrict__ qt,
                          float* __restrict__ primt, StepState* st) {
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  if (k < nc) {
    double qq[4] = {q[k], q[nc + k], q[2 * nc + k], q[3 * nc + k]};
    double u, v, p, h, sr;
    cell_prim(G.g1, qq, u, v, p, h, sr);
#pragma unroll
    for (int e = 0; e < 4; ++e) qt[e * nc + k] = mix::d2f(qq[e]);
    primt[k] = mix::d2f(u);
    primt[nc + k] = mix::d2f(v);
    primt[2 * nc + k] = mix::d2f(h);
    primt[3 * nc + k] = mix::d2f(sr);
    ms = cell_max_speed(G.gamma, qq[0], u, v, p);
  }
  block_max_to(ms, &st->maxbits);
}

// Gauss-Seidel hermiteLimiter sweeps of both directions in one launch.  Blocks [0, nbx): x lines
// (line = row j of field e, walks i, updates v); blocks [nbx, ...): y lines (column i, walks j,
// updates w).  The two directions touch different arrays, so they run side by side.  The
// neighbour beyond the last cell is the zero-gradient ghost, which holds the pre-sweep value; the
// one before the first cell is the first cell (old value).
//
// Each block takes 32 lines of one field.  The sweep itself is sequential along a line (each cell
// reads its left neighbour's limited value), so one thread walks each line; the block stages the
// lines through shared memory in chunks of kLimChunk cells with coalesced loads and stores (along
// the rows for x lines, across the columns for y lines), keeping the global-memory latency off
// the sweep's dependency chain.
constexpr int kLimLines = 32, kLimChunk = 64, kLimThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kLimThreads) kh_limit(GeoH G, HermiteK<T> K,
                                                        const double* __restrict__ q,
                                                        double* __restrict__ v,
                                                        double* __restrict__ w, int nbx,
                                                        const StepState* st) {
  if (st->done) return;
  constexpr int L = kLimLines, C = kLimChunk;
  __shared__ double sq[C + 1][L + 1];
  __shared__ double sd[C + 1][L + 1];
  const bool xd = int(blockIdx.x) < nbx;
  const int b = xd ? int(blockIdx.x) : int(blockIdx.x) - nbx;
  const int nl = xd ? G.ny : G.nx;  // number of lines
  const int n = xd ? G.nx : G.ny;   // length of a line
  const int nlb = (nl + L - 1) / L;
  const int e = b / nlb, l0 = (b - e * nlb) * L;
  double* __restrict__ d = xd ? v : w;
  const size_t nc = size_t(G.nx) * G.ny;
  auto at = [&](int l, int s) -> size_t {
    return size_t(e) * nc + (xd ? size_t(l) * G.nx + s : size_t(s) * G.nx + l);
  };
  const int tid = threadIdx.x;
  const bool sweeper = tid < L && l0 + tid < nl;
  T um = T(0), u0 = T(0), dm = T(0), dcur = T(0);
  if (sweeper) {
    um = from_d<T>(q[at(l0 + tid, 0)]);
    u0 = um;
    dm = from_d<T>(d[at(l0 + tid, 0)]);
    dcur = dm;
  }
  for (int c0 = 0; c0 < n; c0 += C) {
    const int cnt = min(C, n - c0);
    // cells c0 .. c0 + cnt of each line (the last is the look-ahead, clamped to the line's end);
    // every d value read here is a pre-sweep value: the sweep has written cells < c0 only
    for (int it = tid; it < (cnt + 1) * L; it += kLimThreads) {
      int l, k;
      if (xd) { k = it % (cnt + 1); l = it / (cnt + 1); }
      else { l = it % L; k = it / L; }
      if (l0 + l < nl) {
        const size_t o = at(l0 + l, min(c0 + k, n - 1));
        sq[k][l] = q[o];
        sd[k][l] = d[o];
      }
    }
    __syncthreads();
    if (sweeper) {
      for (int k = 0; k < cnt; ++k) {
        const T up = from_d<T>(sq[k + 1][tid]);
        const T dn = from_d<T>(sd[k + 1][tid]);  // not yet limited (or the ghost = pre-sweep last value)
        T uu[3] = {um, u0, up};
        T dd[3] = {dm, dcur, dn};
        T lim;
        if constexpr (std::is_same<T, double>::value) lim = par::hermite_limiter(K, uu, dd);
        else lim = hermite_limiter(K, uu, dd);
        sd[k][tid] = to_d<T>(lim);
        dm = lim;
        um = u0;
        u0 = up;
        dcur = dn;
      }
    }
    __syncthreads();
    for (int it = tid; it < cnt * L; it += kLimThreads) {
      int l, k;
      if (xd) { k = it % cnt; l = it / cnt; }
      else { l = it % L; k = it / L; }
      if (l0 + l < nl) d[at(l0 + l, c0 + k)] = sd[k][l];
    }
    __syncthreads();
  }
}

// Mixed precision: the same sweeps with the float limiter restated so that the part that waits
// for the left neighbour's limited value d0 is short.  hermiteLimiter's result is
//   lim = [w0 (p0/lw0 - Q) + w1 p1 + w2 p2] / (w0 + w1 + w2),  w_k = lw_k (1 + tau / (s_k + eps))
// where only p0 = P - d0/4 and s0 = |(a ud0 + B) ud0 + C|/6720 (ud0 = d0 dif, the smoothness
// measure fullPointsSI expanded in ud0) depend on d0.  Every other quantity of a cell is computed
// off the sweep's chain, before the sweep reaches the cell: B, C, s1, s2, E = P/lw0 - Q,
// M = lw1 r1 + lw2 r2, L = lw1 p1 + lw2 p2, N = lw1 r1 p1 + lw2 r2 p2 with r_k = 1/(s_k + eps).
// The sweep then evaluates, per cell,
//   tau = (|s0 - s1| + |s0 - s2|)^2 / 4,  w0 = lw0 (1 + tau / (s0 + eps)),
//   lim = (w0 (E - d0 / (4 lw0)) + L + tau N) / (w0 + lw1 + lw2 + tau M).
// The block's four warps work as a pipeline over chunks of kLimChunkF cells: warp 0 sweeps its
// 32 lines through chunk s while warps 1-3 load chunk s + 1, precompute its per-cell quantities
// into the other half of a double buffer, and store the limited values of chunk s - 1; one block
// barrier per chunk hands the buffers over.  The sweep, the only sequential part, so runs back to
// back instead of waiting for each chunk's loads, precompute and stores.
constexpr int kLimChunkF = 16;

__global__ void __launch_bounds__(kLimThreads, 4) kh_limit_f(GeoH G, HermiteK<float> K,
                                                          const double* __restrict__ q,
                                                          double* __restrict__ v,
                                                          double* __restrict__ w,
                                                          float* __restrict__ vt,
                                                          float* __restrict__ wt, int nbx,
                                                          const StepState* st) {
  if (st->done) return;
  constexpr int L = kLimLines, C = kLimChunkF, NP = kLimThreads - 32;  // NP producer threads
  constexpr float lw0 = 1.0f - 2e-5f, lw1 = 1e-5f, lw2 = 1e-5f, eps = float(HTENO_LAG_EPS);
  __shared__ float pre[2][8][C][L + 1];
  __shared__ float su[C + 2][L + 1];  // cells c0 - 1 .. c0 + C of the chunk being prepared (clamped)
  __shared__ float sd[C][L + 1];      // pre-sweep d of cells c0 + 1 .. c0 + C (clamped)
  __shared__ float outf[2][C][L + 1];  // limited values (their double copies are exact)
  const bool xd = int(blockIdx.x) < nbx;
  const int b = xd ? int(blockIdx.x) : int(blockIdx.x) - nbx;
  const int nl = xd ? G.ny : G.nx;
  const int n = xd ? G.nx : G.ny;
  const int nlb = (nl + L - 1) / L;
  const int e = b / nlb, l0 = (b - e * nlb) * L;
  double* __restrict__ d = xd ? v : w;
  float* __restrict__ dt = xd ? vt : wt;
  const size_t nc = size_t(G.nx) * G.ny;
  auto at = [&](int l, int s) -> size_t {
    return size_t(e) * nc + (xd ? size_t(l) * G.nx + s : size_t(s) * G.nx + l);
  };
  const int tid = threadIdx.x;
  const bool sweeper_warp = tid < 32;
  const bool sweeper = sweeper_warp && l0 + tid < nl;
  const int ptid = tid - 32;
  const float dif = K.dif, rdif = K.rdif;
  const int nchunks = (n + C - 1) / C;
  // x lines: consecutive threads take consecutive cells of a row; y lines: consecutive lines
  // (columns) of a cell row; both coalesce
  auto slot = [&](int it, int rows, int& l, int& k) {
    if (xd) { l = it / rows; k = it - l * rows; }
    else { l = it % L; k = it / L; }
  };
  // producers: the raw inputs of a chunk are loaded into registers one step before they are
  // staged (bu: cells c0 - 1 .. c0 + C, bd: pre-sweep d of cells c0 + 1 .. c0 + C, clamped), so the
  // loads are in flight during a whole step
  constexpr int NU = ((C + 2) * L + NP - 1) / NP, ND = (C * L + NP - 1) / NP;
  double bu[NU], bd[ND];
  auto fetch = [&](int c) {
    const int c0 = c * C, cnt = min(C, n - c0);
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      const int it = ptid + NP * j;
      int l, k;
      slot(it, C + 2, l, k);
      bu[j] = (it < (C + 2) * L && l0 + l < nl && k < cnt + 2)
                  ? q[at(l0 + l, min(max(c0 - 1 + k, 0), n - 1))] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const int it = ptid + NP * j;
      int l, k;
      slot(it, C, l, k);
      bd[j] = (it < C * L && l0 + l < nl && k < cnt) ? d[at(l0 + l, min(c0 + 1 + k, n - 1))] : 0.0;
    }
  };
  // producers: stage the fetched chunk c, start fetching chunk c + 1, then compute chunk c's
  // per-cell quantities into pre[buf]
  auto prepare = [&](int c, int buf) {
    const int c0 = c * C, cnt = min(C, n - c0);
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      const int it = ptid + NP * j;
      int l, k;
      slot(it, C + 2, l, k);
      if (it < (C + 2) * L && k < cnt + 2) su[k][l] = mix::d2f(bu[j]);
    }
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const int it = ptid + NP * j;
      int l, k;
      slot(it, C, l, k);
      if (it < C * L && k < cnt) sd[k][l] = mix::d2f(bd[j]);
    }
    if (c + 1 < nchunks) fetch(c + 1);
    asm volatile("bar.sync 1, %0;" ::"n"(NP));
    for (int it = ptid; it < cnt * L; it += NP) {
      const int l = it % L, k = it / L;
      const float u0 = su[k][l], u1 = su[k + 1][l], u2 = su[k + 2][l];
      const float ud2 = sd[k][l] * dif;
      const float p1 = (u1 - u0) * rdif, p2 = (u2 - u1) * rdif;
      const float s1 = (u0 - u1) * (u0 - u1), s2 = (u1 - u2) * (u1 - u2);
      const float r1 = 1.0f / (s1 + eps), r2 = 1.0f / (s2 + eps);
      constexpr float k6720 = 1.0f / 6720.0f;
      const float B = (1029270.0f * u2 - 2129184.0f * u1 + 1099914.0f * u0 - 494958.0f * ud2) * k6720;
      const float Cc = ((-1029270.0f * u0 + 2129184.0f * u1 - 1099914.0f * u2 + 281121.0f * ud2) * ud2 +
                        (1099445.0f * u2 - 4317056.0f * u1 + 2118166.0f * u0) * u2 +
                        4317056.0f * (u1 - u0) * u1 + 1099445.0f * u0 * u0) * k6720;
      const float P = 0.75f * (u2 - u0) * rdif - 0.25f * sd[k][l];
      pre[buf][0][k][l] = B;
      pre[buf][1][k][l] = Cc;
      pre[buf][2][k][l] = s1;
      pre[buf][3][k][l] = s2;
      pre[buf][4][k][l] = P * (1.0f / lw0) - ((lw1 / lw0) * p1 + (lw2 / lw0) * p2);
      pre[buf][5][k][l] = lw1 * r1 + lw2 * r2;
      pre[buf][6][k][l] = lw1 * p1 + lw2 * p2;
      pre[buf][7][k][l] = lw1 * r1 * p1 + lw2 * r2 * p2;
    }
  };
  // producers: the limited values of chunk c (in outf[buf]) to global memory
  auto store = [&](int c, int buf) {
    const int c0 = c * C, cnt = min(C, n - c0);
    for (int it = ptid; it < cnt * L; it += NP) {
      int l, k;
      slot(it, cnt, l, k);
      if (l0 + l < nl) {
        const size_t o = at(l0 + l, c0 + k);
        const float x = outf[buf][k][l];
        d[o] = mix::f2d(x);
        dt[o] = x;
      }
    }
  };
  float d0 = sweeper ? mix::d2f(d[at(l0 + tid, 0)]) : 0.f;  // ghost before the first cell
  if (!sweeper_warp) {
    fetch(0);
    prepare(0, 0);
  }
  __syncthreads();
  for (int s = 0; s <= nchunks; ++s) {
    if (sweeper_warp) {
      if (s < nchunks && sweeper) {
        const int cnt = min(C, n - s * C), buf = s & 1;
        constexpr float a = 281121.0f / 6720.0f, c4 = 0.25f / lw0;
        for (int k = 0; k < cnt; ++k) {
          const float ud0 = d0 * dif;
          const float s0 = fabsf(fmaf(fmaf(a, ud0, pre[buf][0][k][tid]), ud0, pre[buf][1][k][tid]));
          const float t = fabsf(s0 - pre[buf][2][k][tid]) + fabsf(s0 - pre[buf][3][k][tid]);
          const float tau = 0.25f * t * t;
          const float w0 = lw0 * fmaf(tau, __fdividef(1.0f, s0 + eps), 1.0f);
          const float num = fmaf(w0, fmaf(-c4, d0, pre[buf][4][k][tid]),
                                 fmaf(tau, pre[buf][7][k][tid], pre[buf][6][k][tid]));
          const float den = w0 + fmaf(tau, pre[buf][5][k][tid], lw1 + lw2);
          d0 = __fdividef(num, den);
          outf[buf][k][tid] = d0;
        }
      }
    } else {
      if (s + 1 < nchunks) prepare(s + 1, (s + 1) & 1);
      if (s >= 1) store(s - 1, (s - 1) & 1);
    }
    __syncthreads();
  }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(kHFaceThreads) kh_faces(GeoH G, HermiteK<T> K,
                                                         const T* __restrict__ q,
                                                         const T* __restrict__ v,
                                                         const T* __restrict__ w,
                                                         const T* __restrict__ prim,
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
  const T* mn = DIR == 1 ? v : w;  // moment along the sweep (HTENO)
  const T* mt = DIR == 1 ? w : v;  // cross moment (TENO5)
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
  const Roe2<T> R = roe2<T>(T(G.g1), prim[3 * nc + ca], prim[ca], prim[nc + ca], prim[2 * nc + ca],
                            prim[3 * nc + cb], prim[cb], prim[nc + cb], prim[2 * nc + cb]);
  {
    T A[4][4], B[4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const size_t c = cell(f - 2 + m);
      T a4[4] = {q[c], q[nc + c], q[2 * nc + c], q[3 * nc + c]};
      T b4[4] = {mn[c], mn[nc + c], mn[2 * nc + c], mn[3 * nc + c]};
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
      T c4[4] = {mt[c], mt[nc + c], mt[2 * nc + c], mt[3 * nc + c]};
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
  // GL3 values of the 24 face arrays at the 3 Gauss points, per thread, in shared memory: for
  // float [array][point][thread] (a warp's accesses fall in 32 distinct banks); for double
  // [thread][array][point] with a one-value pad per thread (par::gl3 writes 3 contiguous values;
  // the odd stride of 73 values spreads a warp's 8-byte accesses over all banks)
  constexpr int kSgT = std::is_same<T, double>::value ? 73 : 72;
  __shared__ T sg[kHFluxThreads * kSgT];
  auto gat = [&](int a, int m) -> T& {
    if constexpr (std::is_same<T, double>::value) return sg[threadIdx.x * kSgT + a * 3 + m];
    else return sg[(a * 3 + m) * kHFluxThreads + threadIdx.x];
  };
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
  for (int a = 0; a < 24; ++a) {
    T u5[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) u5[m] = fc[size_t(a) * nface + nb[m]];
    if constexpr (std::is_same<T, double>::value) par::gl3(c_dev, u5, &gat(a, 0));
    else gl3(c_dev, u5, gat(a, 0), gat(a, 1), gat(a, 2));
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
        const double c[4] = {gat(4 * a + 0, m), gat(4 * a + 1, m), gat(4 * a + 2, m), gat(4 * a + 3, m)};
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
        T c[4] = {gat(4 * a + 0, m), gat(4 * a + 1, m), gat(4 * a + 2, m), gat(4 * a + 3, m)};
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
__global__ void __launch_bounds__(256, 4) kh_update(GeoH G, int stage, const T* __restrict__ fx, const T* __restrict__ fy,
                          double* __restrict__ q, double* __restrict__ q0,
                          double* __restrict__ v, double* __restrict__ v0,
                          double* __restrict__ vs, double* __restrict__ w,
                          double* __restrict__ w0, double* __restrict__ ws,
                          double* __restrict__ prim, float* __restrict__ qt,
                          float* __restrict__ primt, StepState* st) {
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
    if constexpr (std::is_same<T, float>::value) {
      // mixed precision: the residual from the float fluxes in float (a difference of two
      // nearby fluxes is exact in float; otherwise its rounding is far below the fluxes' own),
      // the RK stage in double with FMAs; the conversions on the integer pipes; primitives with
      // a refined float reciprocal of rho.  The FP64 pipe (1/64 of the float rate) does only
      // the accumulation and the primitives.
      auto rhs = [&](int kx, int ky, int e) {
        const float dfx = fx[(kx + e) * nxf + ox] - fx[(kx + e) * nxf + ox + 1];
        const float dfy = fy[(ky + e) * nyf + oy] - fy[(ky + e) * nyf + oy + G.nx];
        return mix::f2d(fmaf(dfx, G.rdxf, dfy * G.rdyf));
      };
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const double ru = rhs(0, 0, e), rv = rhs(4, 8, e), rw = rhs(8, 4, e);
        const size_t c = size_t(e) * nc + k;
        double bq, bv, bw, cq = q[c], cv, cw;
        if (stage == 1) {
          bq = cq; bv = v[c]; bw = w[c];
          q0[c] = bq; v0[c] = bv; w0[c] = bw;
          cv = bv; cw = bw;
        } else {
          bq = q0[c]; bv = v0[c]; bw = w0[c];
          cv = vs[c]; cw = ws[c];
        }
        qn[e] = mix::rk_stage(bq, cq, ru, dt, stage);
        const double nv = mix::rk_stage(bv, cv, rv, dt, stage);
        const double nw = mix::rk_stage(bw, cw, rw, dt, stage);
        q[c] = qn[e];
        qt[c] = mix::d2f(qn[e]);
        v[c] = nv;
        vs[c] = nv;
        w[c] = nw;
        ws[c] = nw;
      }
      const float fr = mix::d2f(qn[0]);
      double ir = mix::f2d(__frcp_rn(fr));
      ir = fma(ir, fma(-qn[0], ir, 1.0), ir);
      const double u = qn[1] * ir, vv = qn[2] * ir;
      const double p = (qn[3] - 0.5 * (qn[1] * u + qn[2] * vv)) * G.g1;
      primt[k] = mix::d2f(u);
      primt[nc + k] = mix::d2f(vv);
      primt[2 * nc + k] = mix::d2f((qn[3] + p) * ir);
      primt[3 * nc + k] = Cst<float>::sqrt_(fabsf(fr));
      if (stage == 3) {
        const float fu = mix::d2f(u), fv = mix::d2f(vv);
        const float cs = sqrtf(fabsf(float(G.gamma) * mix::d2f(p) / fr));
        ms = mix::f2d(fmaxf(fmaxf(fu - cs, fabsf(fu + cs)), fmaxf(fv - cs, fabsf(fv + cs))));
      }
      bad = (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2]) || isnan(qn[3]) || isnan(p)) ? 1 : 0;
      bad |= (qn[0] <= 0.0 || p <= 0.0) ? 2 : 0;
    } else {
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
  G.rdx = 1.0 / s->dx;
  G.rdy = 1.0 / s->dy;
  G.rdxf = float(G.rdx);
  G.rdyf = float(G.rdy);
  return G;
}

template <typename T>
void launch_step(hteno_solver* s, const GeoH& G) {
  cudaStream_t cs = s->stream;
  WorkH<T> W = carve_h<T>(s->work, G.nx, G.ny);
  if constexpr (std::is_same<T, double>::value) {
    W.qt = s->q;
    W.vt = s->v;
    W.wt = s->w;
    W.primt = W.prim;
  }
  const HermiteK<T> K = make_hermite_k<T>(s->dx);  // setGridSize(dx) for both directions
  const int nx = G.nx, ny = G.ny;
  const long nxf = long(nx + 1) * ny, nyf = long(ny + 1) * nx;
  const size_t nc = size_t(nx) * ny;
  const double ncd = double(nc);
  const int k_l = trace_kind(s, "h_limit", ncd * 4 * 8 * 6, 0);
  const int nbx = 4 * ((ny + kLimLines - 1) / kLimLines), nby = 4 * ((nx + kLimLines - 1) / kLimLines);
  const int k_fx = trace_kind(s, "h_faces_x", ncd * 128 + double(nxf) * 31 * sizeof(T), 0);
  const int k_fy = trace_kind(s, "h_faces_y", ncd * 128 + double(nyf) * 31 * sizeof(T), 0);
  const int k_x = trace_kind(s, "h_flux_x", double(nxf) * 43 * sizeof(T), 0);
  const int k_y = trace_kind(s, "h_flux_y", double(nyf) * 43 * sizeof(T), 0);
  const int k_u = trace_kind(s, "h_update", ncd * 8 * 40 + double(nxf + nyf) * 12 * sizeof(T), 0);
  k_begin_step<<<1, 1, 0, cs>>>(s->dstate);
  for (int stage = 1; stage <= 3; ++stage) {
    trace_begin(s, k_l);
    if constexpr (std::is_same<T, float>::value)
      kh_limit_f<<<unsigned(nbx + nby), kLimThreads, 0, cs>>>(G, K, s->q, s->v, s->w, W.vt, W.wt, nbx,
                                                               s->dstate);
    else
      kh_limit<T><<<unsigned(nbx + nby), kLimThreads, 0, cs>>>(G, K, s->q, s->v, s->w, nbx, s->dstate);
    trace_end(s);
    // the y faces and fluxes beside the x ones on the side stream (one stream while timing)
    // (if the fork cannot be recorded, the y kernels stay on the solver's stream)
    const bool fork = s->side_stream && !s->timing &&
                      cudaEventRecord(s->fork_ev, cs) == cudaSuccess &&
                      cudaStreamWaitEvent(s->side_stream, s->fork_ev, 0) == cudaSuccess;
    cudaStream_t ys = fork ? s->side_stream : cs;
    trace_begin(s, k_fx);
    kh_faces<T, 1><<<unsigned((nxf + kHFaceThreads - 1) / kHFaceThreads), kHFaceThreads, 0, cs>>>(
        G, K, W.qt, W.vt, W.wt, W.primt, W.xc, W.xroe, s->dstate);
    trace_end(s);
    trace_begin(s, k_fy);
    kh_faces<T, 2><<<unsigned((nyf + kHFaceThreads - 1) / kHFaceThreads), kHFaceThreads, 0, ys>>>(
        G, K, W.qt, W.vt, W.wt, W.primt, W.yc, W.yroe, s->dstate);
    trace_end(s);
    trace_begin(s, k_x);
    kh_flux<T, 1><<<unsigned((nxf + kHFluxThreads - 1) / kHFluxThreads), kHFluxThreads, 0, cs>>>(
        G, W.xc, W.xroe, W.fx, s->dstate);
    trace_end(s);
    trace_begin(s, k_y);
    kh_flux<T, 2><<<unsigned((nyf + kHFluxThreads - 1) / kHFluxThreads), kHFluxThreads, 0, ys>>>(
        G, W.yc, W.yroe, W.fy, s->dstate);
    trace_end(s);
    // the join; if it cannot be recorded, wait for the side stream on the host instead
    if (fork && (cudaEventRecord(s->join_ev, ys) != cudaSuccess ||
                 cudaStreamWaitEvent(cs, s->join_ev, 0) != cudaSuccess))
      cudaStreamSynchronize(ys);
    trace_begin(s, k_u);
    float *qtf = nullptr, *primtf = nullptr;
    if constexpr (std::is_same<T, float>::value) {
      qtf = W.qt;
      primtf = W.primt;
    }
    kh_update<T><<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, stage, W.fx, W.fy, s->q, s->q0,
                                                            s->v, s->v0, W.vs, s->w, s->w0, W.ws,
                                                            W.prim, qtf, primtf, s->dstate);
    trace_end(s);
  }
  k_end_step<<<1, 1, 0, cs>>>(s->dstate);
}

}  // namespace
}  // namespace hteno
