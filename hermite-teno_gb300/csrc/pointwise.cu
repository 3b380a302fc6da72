// Pointwise batch kernels: one reference function per entry point (see include/hteno.h).
// They exist so that each building block of the solver kernels can be checked against the
// oracle in isolation; the solver kernels call the same device functions: the bit-reproducible
// ones (parity_math.cuh) in double, the fast ones (device_math.cuh) in float.  Compiled with
// --fmad=false.
#include <cstdio>

#include <type_traits>

#include "hermite_math.cuh"
#include "hteno_internal.h"
#include "parity_math.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

inline int prep(void* stream, cudaStream_t* st) {
  *st = static_cast<cudaStream_t>(stream);
  return upload_const(c_dev, &g_mask, &g_mu) == cudaSuccess ? HTENO_OK : HTENO_ERR_CUDA;
}
inline int finish() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HTENO_OK : HTENO_ERR_CUDA;
}
inline unsigned grid_for(long n, int bs) { return static_cast<unsigned>((n + bs - 1) / bs); }

template <typename T>
__global__ void k_lagrange(int kind, const double* __restrict__ u, double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T v[6];
  for (int m = 0; m < 6; ++m) v[m] = static_cast<T>(u[6 * k + m]);
  T a, b;
  if constexpr (std::is_same<T, double>::value) par::lagrange_recon(c_dev, kind, v, a, b);
  else lagrange_recon(c_dev, kind, v, a, b);
  out[2 * k] = a;
  out[2 * k + 1] = b;
}

template <typename T>
__global__ void k_gl3(const double* __restrict__ u, double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T v[5];
  for (int m = 0; m < 5; ++m) v[m] = static_cast<T>(u[5 * k + m]);
  T a, b, c;
  if constexpr (std::is_same<T, double>::value) {
    double o[3];
    par::gl3(c_dev, v, o);
    a = o[0]; b = o[1]; c = o[2];
  } else {
    gl3(c_dev, v, a, b, c);
  }
  out[3 * k] = a;
  out[3 * k + 1] = b;
  out[3 * k + 2] = c;
}

template <typename T>
__global__ void k_hermite(int kind, HermiteK<T> K, const double* __restrict__ u,
                          const double* __restrict__ d, double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T uu[4], dd[4], o[4];
  for (int m = 0; m < 4; ++m) {
    uu[m] = static_cast<T>(u[4 * k + m]);
    dd[m] = static_cast<T>(d[4 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) par::hermite_recon(c_dev, K, kind, uu, dd, o);
  else hermite_recon(c_dev, K, kind, uu, dd, o);
  for (int m = 0; m < 4; ++m) out[4 * k + m] = o[m];
}

template <typename T>
__global__ void k_hlimiter(HermiteK<T> K, const double* __restrict__ u, const double* __restrict__ d,
                           double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T uu[3], dd[3];
  for (int m = 0; m < 3; ++m) {
    uu[m] = static_cast<T>(u[3 * k + m]);
    dd[m] = static_cast<T>(d[3 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) out[k] = par::hermite_limiter(K, uu, dd);
  else out[k] = hermite_limiter(K, uu, dd);
}

template <typename T>
__global__ void k_hllc2(T g1, int dir, const double* __restrict__ ql, const double* __restrict__ qr,
                        double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T a[4], b[4], F[4];
  for (int m = 0; m < 4; ++m) {
    a[m] = static_cast<T>(ql[4 * k + m]);
    b[m] = static_cast<T>(qr[4 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) par::hllc(g1, dir, a, b, F);
  else hllc2(g1, dir, a, b, F);
  for (int m = 0; m < 4; ++m) out[4 * k + m] = F[m];
}

template <typename T>
__global__ void k_hllc1(T g1, const double* __restrict__ ql, const double* __restrict__ qr,
                        double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T a[3], b[3], F[3];
  for (int m = 0; m < 3; ++m) {
    a[m] = static_cast<T>(ql[3 * k + m]);
    b[m] = static_cast<T>(qr[3 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) par::hllc1(g1, a, b, F);
  else hllc1(g1, a, b, F);
  for (int m = 0; m < 3; ++m) out[3 * k + m] = F[m];
}

// Roe state of the cell pair (qa, qb) as eigen2DEuler computes it (FV_System2D.cpp:265-361)
template <typename T>
__device__ __forceinline__ Roe2<T> roe_of_pair(T g1, const double* qa, const double* qb) {
  double wa[4], wb[4];
  primitive2(double(g1), qa, wa);
  primitive2(double(g1), qb, wb);
  const double ha = (qa[3] + wa[3]) / wa[0], hb = (qb[3] + wb[3]) / wb[0];
  return roe2<T>(g1, T(sqrt(fabs(wa[0]))), T(wa[1]), T(wa[2]), T(ha), T(sqrt(fabs(wb[0]))),
                 T(wb[1]), T(wb[2]), T(hb));
}

template <typename T>
__global__ void k_rusanov2(T g, T g1, int dir, const double* __restrict__ qa,
                           const double* __restrict__ qb, const double* __restrict__ ql,
                           const double* __restrict__ qr, double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T a[4], b[4], F[4];
  for (int m = 0; m < 4; ++m) {
    a[m] = static_cast<T>(ql[4 * k + m]);
    b[m] = static_cast<T>(qr[4 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) {
    double wa[4], wb[4];
    par::primitive(g1, qa + 4 * k, wa);
    par::primitive(g1, qb + 4 * k, wb);
    const par::Eig E = par::eig(g1, dir, sqrt(fabs(wa[0])), wa[1], wa[2], (qa[4 * k + 3] + wa[3]) / wa[0],
                                sqrt(fabs(wb[0])), wb[1], wb[2], (qb[4 * k + 3] + wb[3]) / wb[0]);
    par::rusanov(g, g1, dir, E, a, b, F);
  } else {
    Roe2<T> s = roe_of_pair(g1, qa + 4 * k, qb + 4 * k);
    rusanov2(g, g1, dir, s, a, b, F);
  }
  for (int m = 0; m < 4; ++m) out[4 * k + m] = F[m];
}

template <typename T>
__global__ void k_drusanov2(T g, T g1, T g3, int dir, const double* __restrict__ qa,
                            const double* __restrict__ qb, const double* __restrict__ ql,
                            const double* __restrict__ qr, const double* __restrict__ dql,
                            const double* __restrict__ dqr, double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  T a[4], b[4], da[4], db[4], F[4];
  for (int m = 0; m < 4; ++m) {
    a[m] = static_cast<T>(ql[4 * k + m]);
    b[m] = static_cast<T>(qr[4 * k + m]);
    da[m] = static_cast<T>(dql[4 * k + m]);
    db[m] = static_cast<T>(dqr[4 * k + m]);
  }
  if constexpr (std::is_same<T, double>::value) {
    double wa[4], wb[4];
    par::primitive(g1, qa + 4 * k, wa);
    par::primitive(g1, qb + 4 * k, wb);
    const par::Eig E = par::eig(g1, dir, sqrt(fabs(wa[0])), wa[1], wa[2], (qa[4 * k + 3] + wa[3]) / wa[0],
                                sqrt(fabs(wb[0])), wb[1], wb[2], (qb[4 * k + 3] + wb[3]) / wb[0]);
    par::drusanov(g, g1, g3, dir, E, a, b, da, db, F);
  } else {
    Roe2<T> s = roe_of_pair(g1, qa + 4 * k, qb + 4 * k);
    drusanov2(g, g1, dir, s, a, b, da, db, F);
  }
  for (int m = 0; m < 4; ++m) out[4 * k + m] = F[m];
}

__global__ void k_ssprk3(const double* __restrict__ q0, const double* __restrict__ qn,
                         const double* __restrict__ rhs, double dt, int stage,
                         double* __restrict__ out, long n) {
  long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[k] = ssprk3(q0[k], qn[k], rhs[k], dt, stage);
}

}  // namespace
}  // namespace hteno

using namespace hteno;

#define HTENO_CHECK_N(n, ...)                                         \
  do {                                                                \
    if ((n) < 0) return HTENO_ERR_INVALID_ARG;                        \
    if ((n) == 0) return HTENO_OK;                                    \
    if (__VA_ARGS__) return HTENO_ERR_INVALID_ARG;                    \
  } while (0)

extern "C" {

int hteno_lagrange_batch(int kind, int precision, const double* u, double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !u || !out || kind < 0 || kind > 7);
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_lagrange<float><<<grid_for(n, 256), 256, 0, st>>>(kind, u, out, n);
  else
    k_lagrange<double><<<grid_for(n, 256), 256, 0, st>>>(kind, u, out, n);
  return finish();
}

int hteno_gl3_batch(int precision, const double* u, double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !u || !out);
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_gl3<float><<<grid_for(n, 256), 256, 0, st>>>(u, out, n);
  else
    k_gl3<double><<<grid_for(n, 256), 256, 0, st>>>(u, out, n);
  return finish();
}

int hteno_hermite_batch(int kind, int precision, double dx, const double* u, const double* d,
                        double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !u || !d || !out || kind < 0 || kind > 2 || !(dx != 0.0));
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_hermite<float><<<grid_for(n, 256), 256, 0, st>>>(kind, make_hermite_k<float>(dx), u, d, out, n);
  else
    k_hermite<double><<<grid_for(n, 256), 256, 0, st>>>(kind, make_hermite_k<double>(dx), u, d, out, n);
  return finish();
}

int hteno_hlimiter_batch(int precision, double dx, const double* u, const double* d, double* out,
                         long n, void* stream) {
  HTENO_CHECK_N(n, !u || !d || !out || !(dx != 0.0));
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_hlimiter<float><<<grid_for(n, 256), 256, 0, st>>>(make_hermite_k<float>(dx), u, d, out, n);
  else
    k_hlimiter<double><<<grid_for(n, 256), 256, 0, st>>>(make_hermite_k<double>(dx), u, d, out, n);
  return finish();
}

int hteno_hllc2d_batch(int precision, double gamma, int dir, const double* ql, const double* qr,
                       double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !ql || !qr || !out || (dir != 1 && dir != 2));
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_hllc2<float><<<grid_for(n, 256), 256, 0, st>>>(float(gamma - 1.0), dir, ql, qr, out, n);
  else
    k_hllc2<double><<<grid_for(n, 256), 256, 0, st>>>(gamma - 1.0, dir, ql, qr, out, n);
  return finish();
}

int hteno_hllc1d_batch(int precision, double gamma, const double* ql, const double* qr,
                       double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !ql || !qr || !out);
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_hllc1<float><<<grid_for(n, 256), 256, 0, st>>>(float(gamma - 1.0), ql, qr, out, n);
  else
    k_hllc1<double><<<grid_for(n, 256), 256, 0, st>>>(gamma - 1.0, ql, qr, out, n);
  return finish();
}

int hteno_rusanov2d_batch(int precision, double gamma, int dir, const double* qa, const double* qb,
                          const double* ql, const double* qr, double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !qa || !qb || !ql || !qr || !out || (dir != 1 && dir != 2));
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_rusanov2<float><<<grid_for(n, 256), 256, 0, st>>>(float(gamma), float(gamma - 1.0), dir, qa,
                                                         qb, ql, qr, out, n);
  else
    k_rusanov2<double><<<grid_for(n, 256), 256, 0, st>>>(gamma, gamma - 1.0, dir, qa, qb, ql, qr,
                                                          out, n);
  return finish();
}

int hteno_drusanov2d_batch(int precision, double gamma, int dir, const double* qa,
                           const double* qb, const double* ql, const double* qr,
                           const double* dql, const double* dqr, double* out, long n,
                           void* stream) {
  HTENO_CHECK_N(n, !qa || !qb || !ql || !qr || !dql || !dqr || !out || (dir != 1 && dir != 2));
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  if (precision == HTENO_PREC_MIXED)
    k_drusanov2<float><<<grid_for(n, 256), 256, 0, st>>>(float(gamma), float(gamma - 1.0),
                                                          float(gamma - 3.0), dir, qa, qb, ql, qr,
                                                          dql, dqr, out, n);
  else
    k_drusanov2<double><<<grid_for(n, 256), 256, 0, st>>>(gamma, gamma - 1.0, gamma - 3.0, dir, qa,
                                                           qb, ql, qr, dql, dqr, out, n);
  return finish();
}

int hteno_ssprk3_batch(const double* q0, const double* qn, const double* rhs, double dt, int stage,
                       double* out, long n, void* stream) {
  HTENO_CHECK_N(n, !q0 || !qn || !rhs || !out || stage < 1 || stage > 3);
  cudaStream_t st;
  if (prep(stream, &st)) return HTENO_ERR_CUDA;
  k_ssprk3<<<grid_for(n, 256), 256, 0, st>>>(q0, qn, rhs, dt, stage, out, n);
  return finish();
}

}  // extern "C"
