// FVHermite::System1D on the GPU (FVHermite_System1D.cpp:183-405): periodic boundaries, LMPE
// troubled-cell detection, conditional derivative limiter, htenoi on troubled cells and linear
// Hermite reconstruction elsewhere, Rusanov + dRusanov, SSP-RK3, dt = cfl dx^(5/3) / max speed.
//
// The LMPE scan (:239-257) is sequential along x (a cell flagged by its left neighbour is
// skipped) and its flags live on the ghost-padded index space [0, nx + 2k) and are never reset;
// the limiter (:259-273) runs once per rhs over the padded range when any flag is set, updating
// the moments in place (a Gauss-Seidel sweep that also limits the left ghost first).  Both are
// one thread per conserved field walking the line; faces and updates are one thread per face /
// cell.  In double the bit-reproducible functions (parity_math.cuh) are used; compiled with
// --fmad=false.
#include <type_traits>

#include "hermite_math.cuh"
#include "hteno_internal.h"
#include "parity_math.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

constexpr int kGhost = 4;  // k of FVHermite::System1D (:24)
constexpr int kS = 1;      // s (:25)

struct GeoH1 {
  int nx, nxx;
  double dx, area, gamma, g1, g3;  // g3 = gamma - 3 as the reference computes it
};

template <typename T>
struct WorkH1 {
  double* vs;            // [3][nx] unlimited stage moments
  double* vpad;          // [3][nxx] padded moments during the limiter sweep
  unsigned char* flags;  // [nxx][3] LMPE flags (persist)
  T* Fu;                 // [3][nx+1]
  T* Fv;                 // [3][nx+1]
};

template <typename T>
size_t work_bytes_h1(int nx) {
  const int nxx = nx + 2 * kGhost;
  return 3 * size_t(nx) * 8 + 3 * size_t(nxx) * 8 + 3 * size_t(nxx) + 2 * 3 * size_t(nx + 1) * sizeof(T) + 256 * 5;
}

template <typename T>
WorkH1<T> carve_h1(void* base, int nx) {
  const int nxx = nx + 2 * kGhost;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  WorkH1<T> w;
  w.vs = reinterpret_cast<double*>(take(3 * size_t(nx) * 8));
  w.vpad = reinterpret_cast<double*>(take(3 * size_t(nxx) * 8));
  w.flags = reinterpret_cast<unsigned char*>(take(3 * size_t(nxx)));
  w.Fu = reinterpret_cast<T*>(take(3 * size_t(nx + 1) * sizeof(T)));
  w.Fv = reinterpret_cast<T*>(take(3 * size_t(nx + 1) * sizeof(T)));
  return w;
}

__device__ __forceinline__ int wrap(int i, int n) {  // padded index -> interior (periodic)
  int m = i - kGhost;
  m %= n;
  return m < 0 ? m + n : m;
}

__device__ __forceinline__ void prim1(double g1, const double* q, double* w, double& h, double& sr) {
  w[0] = q[0];
  w[1] = q[1] / q[0];
  w[2] = (q[2] - 0.5 * q[1] * w[1]) * g1;
  h = (q[2] + w[2]) / w[0];
  sr = sqrt(fabs(w[0]));
}

__global__ void kh1_init(GeoH1 G, const double* __restrict__ q, StepState* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ms = 0.0;
  if (i < G.nx) {
    double qq[3] = {q[i], q[G.nx + i], q[2 * G.nx + i]}, w[3], h, sr;
    prim1(G.g1, qq, w, h, sr);
    ms = par::max_speed1(G.gamma, w);
  }
  block_max_to(ms, &st->maxbits);
}

// LMPE + conditional limiter; one block, thread e < 3 owns field e.
template <typename T>
__global__ void kh1_sensor(GeoH1 G, HermiteK<T> K, const double* __restrict__ q, double* v,
                           WorkH1<T> W, const StepState* st) {
  __shared__ int any;
  if (st->done) return;
  const int e = threadIdx.x;
  const int n = G.nx, nxx = G.nxx;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  if (e < 3) {
    const double* u = q + size_t(e) * n;
    unsigned char* fl = W.flags;
    for (int i = kS + 1; i < nxx - kS - 1; ++i) {
      if (fl[3 * i + e]) continue;
      const double um = u[wrap(i - 1, n)], u0 = u[wrap(i, n)], up = u[wrap(i + 1, n)];
      const double A = fabs(-um + 2.0 * u0 - up) / 2.0;
      if (A > 0.5 * G.dx) {
        const double xc = (-2. * um + 3. * u0 - up) / (-um + 2.0 * u0 - up) * G.dx;
        if (0.0 <= xc && xc <= 3. * G.dx) {
          fl[3 * i + e] = 1;
          fl[3 * (i - 1) + e] = 1;
          fl[3 * (i + 1) + e] = 1;
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0;
    for (int i = kS + 1; i < nxx - kS - 1 && !a; ++i)
      a = W.flags[3 * i] | W.flags[3 * i + 1] | W.flags[3 * i + 2];
    any = a;
  }
  __syncthreads();
  if (!any || e >= 3) return;
  // padded moments with periodic ghosts, then the in-place sweep over [k-1, nxx-k+1)
  double* vp = W.vpad + size_t(e) * nxx;
  for (int i = 0; i < nxx; ++i) vp[i] = v[size_t(e) * n + wrap(i, n)];
  const double* u = q + size_t(e) * n;
  for (int i = kGhost - 1; i < nxx - kGhost + 1; ++i) {
    T uu[3] = {T(u[wrap(i - 1, n)]), T(u[wrap(i, n)]), T(u[wrap(i + 1, n)])};
    T dd[3] = {T(vp[i - 1]), T(vp[i]), T(vp[i + 1])};
    if constexpr (std::is_same<T, double>::value) vp[i] = par::hermite_limiter(K, uu, dd);
    else vp[i] = double(hermite_limiter(K, uu, dd));
  }
  for (int i = 0; i < n; ++i) v[size_t(e) * n + i] = vp[i + kGhost];
}

// face f in [0, nx] between interior cells f-1 and f (padded cell f + k - 1 and its neighbour)
template <typename T>
__global__ void kh1_faces(GeoH1 G, HermiteK<T> K, const double* __restrict__ q,
                          const double* __restrict__ v, WorkH1<T> W, const StepState* st) {
  if (st->done) return;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = G.nx;
  if (f > n) return;
  const int ip = f + kGhost - 1;  // padded index of the left cell
  double qa[3], qb[3], wa[3], wb[3], ha, hb, sa, sb;
  const int ca = wrap(ip, n), cb = wrap(ip + 1, n);
  for (int c = 0; c < 3; ++c) {
    qa[c] = q[c * n + ca];
    qb[c] = q[c * n + cb];
  }
  prim1(G.g1, qa, wa, ha, sa);
  prim1(G.g1, qb, wb, hb, sb);
  T fu[3], fv[3];
  if constexpr (std::is_same<T, double>::value) {
    double R[9], L[9], A[3][4], B[3][4];
    par::eig1(G.g1, sa, wa[1], ha, sb, wb[1], hb, R, L);
    for (int m = 0; m < 4; ++m) {
      const int c = wrap(ip - 1 + m, n);
      const double a3[3] = {q[c], q[n + c], q[2 * n + c]};
      const double b3[3] = {v[c], v[n + c], v[2 * n + c]};
      double ca3[3], cb3[3];
      par::mv3(L, a3, ca3);
      par::mv3(L, b3, cb3);
      for (int r = 0; r < 3; ++r) {
        A[r][m] = ca3[r];
        B[r][m] = cb3[r];
      }
    }
    double cl[4][3];
    for (int r = 0; r < 3; ++r) {
      double o[4];
      par::hermite_recon(c_dev, K, W.flags[3 * ip + r] ? 1 : 2, A[r], B[r], o);
      for (int a = 0; a < 4; ++a) cl[a][r] = o[a];
    }
    double X[4][3];
    for (int a = 0; a < 4; ++a) par::mv3(R, cl[a], X[a]);
    par::rusanov1(G.gamma, G.g1, L, R, X[0], X[1], fu);
    par::drusanov1(G.gamma, G.g1, G.g3, L, R, X[0], X[1], X[2], X[3], fv);
  } else {
    const Roe1<T> R = roe1<T>(T(G.g1), T(sa), T(wa[1]), T(ha), T(sb), T(wb[1]), T(hb));
    T A[3][4], B[3][4];
    for (int m = 0; m < 4; ++m) {
      const int c = wrap(ip - 1 + m, n);
      T a3[3] = {T(q[c]), T(q[n + c]), T(q[2 * n + c])};
      T b3[3] = {T(v[c]), T(v[n + c]), T(v[2 * n + c])};
      T ca3[3], cb3[3];
      roe1_left(R, a3, ca3);
      roe1_left(R, b3, cb3);
      for (int r = 0; r < 3; ++r) {
        A[r][m] = ca3[r];
        B[r][m] = cb3[r];
      }
    }
    T cl[4][3];
    for (int r = 0; r < 3; ++r) {
      T o[4];
      hermite_recon(c_dev, K, W.flags[3 * ip + r] ? 1 : 2, A[r], B[r], o);
      for (int a = 0; a < 4; ++a) cl[a][r] = o[a];
    }
    T X[4][3];
    for (int a = 0; a < 4; ++a) roe1_right(R, cl[a], X[a]);
    rusanov1(T(G.gamma), T(G.g1), R, X[0], X[1], fu);
    drusanov1(T(G.gamma), T(G.g1), R, X[0], X[1], X[2], X[3], fv);
  }
  for (int c = 0; c < 3; ++c) {
    W.Fu[c * (n + 1) + f] = fu[c];
    W.Fv[c * (n + 1) + f] = fv[c];
  }
}

template <typename T>
__global__ void kh1_update(GeoH1 G, int stage, WorkH1<T> W, double* __restrict__ q,
                           double* __restrict__ q0, double* __restrict__ v,
                           double* __restrict__ v0, StepState* st) {
  if (st->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = G.nx;
  double ms = 0.0;
  int bad = 0;
  if (i < n) {
    const double dt = st->dt;
    double qn[3];
    for (int c = 0; c < 3; ++c) {
      const double ru = (double(W.Fu[c * (n + 1) + i]) - double(W.Fu[c * (n + 1) + i + 1])) / G.area;
      const double rv = (double(W.Fv[c * (n + 1) + i]) - double(W.Fv[c * (n + 1) + i + 1])) / G.area;
      const size_t o = size_t(c) * n + i;
      double bq, bv, cq = q[o], cv;
      if (stage == 1) {
        bq = cq; bv = v[o];
        q0[o] = bq; v0[o] = bv;
        cv = bv;
      } else {
        bq = q0[o]; bv = v0[o];
        cv = W.vs[o];
      }
      qn[c] = ssprk3(bq, cq, ru, dt, stage);
      const double nv = ssprk3(bv, cv, rv, dt, stage);
      q[o] = qn[c];
      v[o] = nv;
      W.vs[o] = nv;
    }
    double w[3], h, sr;
    prim1(G.g1, qn, w, h, sr);
    if (stage == 3) ms = par::max_speed1(G.gamma, w);
    bad = (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2])) ? 1 : 0;
    bad |= (qn[0] <= 0.0 || w[2] <= 0.0) ? 2 : 0;
  }
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad) atomicOr(&st->status, bad);
}

GeoH1 geo_of(const hteno_solver* s) {
  GeoH1 G;
  G.nx = s->cfg.nx;
  G.nxx = s->cfg.nx + 2 * kGhost;
  G.dx = s->dx;
  G.area = s->dx;
  G.gamma = s->cfg.gamma;
  G.g1 = s->cfg.gamma - 1.0;
  G.g3 = s->cfg.gamma - 3.0;
  return G;
}

template <typename T>
void launch_step(hteno_solver* s, const GeoH1& G) {
  cudaStream_t cs = s->stream;
  const WorkH1<T> W = carve_h1<T>(s->work, G.nx);
  const HermiteK<T> K = make_hermite_k<T>(s->dx);
  const unsigned gf = unsigned((G.nx + 1 + 63) / 64), gc = unsigned((G.nx + 63) / 64);
  k_begin_step<<<1, 1, 0, cs>>>(s->dstate);
  for (int stage = 1; stage <= 3; ++stage) {
    kh1_sensor<T><<<1, 32, 0, cs>>>(G, K, s->q, s->v, W, s->dstate);
    kh1_faces<T><<<gf, 64, 0, cs>>>(G, K, s->q, s->v, W, s->dstate);
    kh1_update<T><<<gc, 64, 0, cs>>>(G, stage, W, s->q, s->q0, s->v, s->v0, s->dstate);
  }
  k_end_step<<<1, 1, 0, cs>>>(s->dstate);
}

}  // namespace

int hermite1d_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  s->work_bytes = s->cfg.precision == HTENO_PREC_MIXED ? work_bytes_h1<float>(s->cfg.nx)
                                                       : work_bytes_h1<double>(s->cfg.nx);
  cudaError_t e = cudaMalloc(&s->work, s->work_bytes);
  if (e != cudaSuccess) return cuda_error(s, e, "work buffer");
  cudaMemset(s->v, 0, s->ncell * 3 * sizeof(double));
  s->launches_per_step = 2 + 3 * 3;
  return HTENO_OK;
}

int hermite1d_prepare(hteno_solver* s) {
  const GeoH1 G = geo_of(s);
  // a new initial state starts with cleared troubled-cell flags (fresh storage in the reference)
  unsigned char* flags = s->cfg.precision == HTENO_PREC_MIXED ? carve_h1<float>(s->work, G.nx).flags
                                                              : carve_h1<double>(s->work, G.nx).flags;
  cudaMemsetAsync(flags, 0, 3 * size_t(G.nxx), s->stream);
  kh1_init<<<unsigned((G.nx + 127) / 128), 128, 0, s->stream>>>(G, s->q, s->dstate);
  return cuda_error(s, cudaGetLastError(), "kh1_init");
}

int hermite1d_step_async(hteno_solver* s, int nsteps) {
  const GeoH1 G = geo_of(s);
  for (int n = 0; n < nsteps; ++n) {
    if (s->cfg.precision == HTENO_PREC_MIXED) launch_step<float>(s, G);
    else launch_step<double>(s, G);
  }
  return cuda_error(s, cudaGetLastError(), "hermite1d step launch");
}

}  // namespace hteno
