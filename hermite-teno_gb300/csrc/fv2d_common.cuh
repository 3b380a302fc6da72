// Layout and launch constants shared by the FV 2D translation units (fv2d.cu: mixed FP32 path
// and host dispatch; fv2d_fp64.cu: bit-reproducible FP64 path).
#pragma once

#include "hteno_internal.h"

namespace hteno {

struct Geo {
  int nx, ny, bc, recon, flux;
  double dx, dy, area, gamma, g1;
};

// Work buffer: primitives (double) and per-face intermediates (compute type T).
template <typename T>
struct Work {
  double* prim;  // [4][ncell]: u, v, h, sqrt|rho|
  T* xc;         // [8][ny][nx+1]  characteristic face values (l0..l3, r0..r3), face basis
  T* xroe;       // [7][ny][nx+1]  vxm, vym, hm, qm, cm, rcm, b1
  T* yc;         // [8][ny+1][nx]
  T* yroe;       // [7][ny+1][nx]
  T* fx;         // [4][ny][nx+1]  face fluxes (Gauss-Legendre quadrature of the face)
  T* fy;         // [4][ny+1][nx]
};

template <typename T>
inline size_t work_bytes(int nx, int ny) {
  const size_t nc = size_t(nx) * ny, nxf = size_t(nx + 1) * ny, nyf = size_t(ny + 1) * nx;
  return 4 * nc * sizeof(double) + (8 + 7 + 4) * (nxf + nyf) * sizeof(T) + 256 * 8;
}

template <typename T>
inline Work<T> carve(void* base, int nx, int ny) {
  const size_t nc = size_t(nx) * ny, nxf = size_t(nx + 1) * ny, nyf = size_t(ny + 1) * nx;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  Work<T> w;
  w.prim = reinterpret_cast<double*>(take(4 * nc * sizeof(double)));
  w.xc = reinterpret_cast<T*>(take(8 * nxf * sizeof(T)));
  w.xroe = reinterpret_cast<T*>(take(7 * nxf * sizeof(T)));
  w.yc = reinterpret_cast<T*>(take(8 * nyf * sizeof(T)));
  w.yroe = reinterpret_cast<T*>(take(7 * nyf * sizeof(T)));
  w.fx = reinterpret_cast<T*>(take(4 * nxf * sizeof(T)));
  w.fy = reinterpret_cast<T*>(take(4 * nyf * sizeof(T)));
  return w;
}

// Algorithmic flops of the reference per face / per cell of one stage, op-counted on the oracle
// build (oracle/opcount.cpp): +, -, *, /, sqrt count one each, pow one per call.
constexpr double kFacesFlops = 1131.0;        // Roe average, 6 projections, TENO5 x 4 fields
constexpr double kFluxFlopsHllc = 1603.07;    // GL3 x 8, 6 back-projections, 3 HLLC, quadrature
constexpr double kFluxFlopsRusanov = 1628.0;  // the same with characteristic Rusanov
constexpr double kUpdateFlops = 52.0;         // primitives, flux difference, RK stage

constexpr int kFaceThreads = 128;

inline Geo geo_of(const hteno_solver* s) {
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

// Mixed path, one fused launch per stage (fv2d_fused.cu).  Work buffer: one extra state.
size_t fv2d_fused_work_bytes(int nx, int ny);
int fv2d_fused_setup(hteno_solver* s);
int fv2d_fused_prepare(hteno_solver* s, const Geo& G, double* scratch);
void fv2d_fused_step(hteno_solver* s, const Geo& G, double* qc);
void fv2d_fused_residual(hteno_solver* s, const Geo& G, const double* q, double* rhs);
const char* fv2d_fused_variant_name(int v);
// Tensor-core classifier (mlp.cu): route masks of a grid from its state; timeout status.
int mlp_classify(hteno_mlp* m, const Geo& G, const double* q, uint8_t* mx, uint8_t* my, float thr,
                 uint4* rows, unsigned long long* info, unsigned long long* nrows, long cap,
                 cudaStream_t st);
int mlp_status(hteno_mlp* m, cudaStream_t st);

// Training stencils of the learned classifier from the current FP64 state (fv2d_fp64.cu).
int fv2d_harvest(hteno_solver* s, const Geo& G, const Work<double>& W, double p,
                 unsigned long long seed, uint16_t* X, uint8_t* Y, long cap,
                 unsigned long long* count);

// Bit-reproducible FP64 path (fv2d_fp64.cu)
int fv2d_fp64_setup(hteno_solver* s);
void fv2d_fp64_prim(hteno_solver* s, const Geo& G, const Work<double>& W, const double* q,
                    StepState* st, int do_max);
void fv2d_fp64_stage(hteno_solver* s, const Geo& G, const Work<double>& W, int stage,
                     const double* q, double* out);

}  // namespace hteno
