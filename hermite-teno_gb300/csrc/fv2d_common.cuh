// Layout and launch constants shared by the FV 2D translation units (fv2d.cu: mixed FP32 path
// and host dispatch; fv2d_fp64.cu: bit-reproducible FP64 path).
#pragma once

#include "hteno_internal.h"

namespace hteno {

struct Geo {
  int nx, ny, bc, recon, flux;
  double dx, dy, area, gamma, g1;
  // boundaries whose ghosts are not copies of interior cells (HTENO_BC_TAYLOR, _DOUBLE_MACH)
  double x0, y0;        // xl, yb: cell centres
  double t0;            // time of a residual evaluation (the stepping kernels read the step state)
  double bq[4][4];      // fixed ghost states (fill_bc_consts)
  double ctan, c16, s3;
};

// State of cell (i, j) with the ghosts FV::System2D fills (6 layers; further cells read as the
// outermost ghost)
// (FV_System2D.cpp:114-224).  Zero-gradient and periodic ghosts copy interior cells.
// TaylorInstBc (:154-182): x ghosts of interior rows mirror the row with the x momentum negated;
// the ghost rows of every column hold the fixed bottom / top states.  doubleMachBc (:184-224):
// below the first row, columns with x <= 1/6 hold conservativeOfDoubleMach2D at the ghost's
// centre, the others mirror the column with the y momentum negated; above the last row, the
// state of interior cell (0, 6) where x < 1/6 + tan(pi/6) (y_top + (1 + m) dy + 20 t), of cell
// (nx - 7, 6) elsewhere (m = j - ny); the x ghosts of every row copy its first / last column.
// Positions are computed with explicitly rounded operations, as the reference's expressions
// round them, in any translation unit.
__device__ __forceinline__ void bc_state(const Geo& G, const double* __restrict__ q, int i, int j,
                                         double t, double* out) {
  const size_t nc = size_t(G.nx) * G.ny;
  auto ld = [&](int ii, int jj) {
    const size_t k = size_t(jj) * G.nx + ii;
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = q[v * nc + k];
  };
  auto cp = [&](const double* s) {
#pragma unroll
    for (int v = 0; v < 4; ++v) out[v] = s[v];
  };
  if (G.bc >= HTENO_BC_TAYLOR) {  // cells past the ghost layers (tiles overhanging the grid)
    i = min(max(i, -6), G.nx + 5);
    j = min(max(j, -6), G.ny + 5);
  }
  if (G.bc == HTENO_BC_TAYLOR) {
    if (j < 0) return cp(G.bq[0]);
    if (j >= G.ny) return cp(G.bq[1]);
    if (i < 0) { ld(-1 - i, j); out[1] = -out[1]; return; }
    if (i >= G.nx) { ld(2 * G.nx - 1 - i, j); out[1] = -out[1]; return; }
    return ld(i, j);
  }
  if (G.bc == HTENO_BC_DOUBLE_MACH) {
    const int ic = min(max(i, 0), G.nx - 1);
    if (j >= 0 && j < G.ny) return ld(ic, j);
    const double x = __dadd_rn(__dmul_rn(__dadd_rn(__dsub_rn(double(ic + 6), 6.0), 0.5), G.dx), G.x0);
    if (j < 0) {
      if (x <= G.c16) {
        const double y = __dadd_rn(__dmul_rn(__dadd_rn(__dsub_rn(double(j + 6), 6.0), 0.5), G.dy), G.y0);
        return cp(x < __dadd_rn(G.c16, __ddiv_rn(y, G.s3)) ? G.bq[2] : G.bq[3]);
      }
      ld(ic, -1 - j);
      out[2] = -out[2];
      return;
    }
    const double ytop = __dadd_rn(__dmul_rn(__dadd_rn(__dsub_rn(double(G.ny + 5), 6.0), 0.5), G.dy), G.y0);
    const double span = __dadd_rn(__dadd_rn(ytop, __dmul_rn(__dadd_rn(1.0, double(j - G.ny)), G.dy)),
                                  __dmul_rn(20.0, t));
    const double hx = __dadd_rn(__dmul_rn(G.ctan, span), G.c16);
    return x < hx ? ld(0, 6) : ld(G.nx - 7, 6);
  }
  int ii = i, jj = j;
  if (G.bc == HTENO_BC_PERIODIC) {
    ii %= G.nx;
    ii = ii < 0 ? ii + G.nx : ii;
    jj %= G.ny;
    jj = jj < 0 ? jj + G.ny : jj;
  } else {
    ii = min(max(ii, 0), G.nx - 1);
    jj = min(max(jj, 0), G.ny - 1);
  }
  ld(ii, jj);
}

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
  G.x0 = s->cfg.xl;
  G.y0 = s->cfg.yb;
  G.t0 = s->hstate ? s->hstate->t : 0.0;
  fill_bc_consts(s->cfg.gamma, G.bq, &G.ctan, &G.c16, &G.s3);
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
                 uint4* rows, unsigned long long* nrows, long cap, cudaStream_t st,
                 const StepState* sst);
int mlp_status(hteno_mlp* m, cudaStream_t st);

// Training stencils of the learned classifier from the current FP64 state (fv2d_fp64.cu).
int fv2d_harvest(hteno_solver* s, const Geo& G, const Work<double>& W, double p,
                 unsigned long long seed, uint16_t* X, uint8_t* Y, long cap,
                 unsigned long long* count);

// FP64 judge of learned routing (fv2d_fp64.cu): counts[0] routed stencils of the masks, counts[1]
// those whose plain FP64 TENO cut-off on the double state drops a candidate; counts[2], [3] the
// same over the stencils whose variation is resolved in float.
int fv2d_audit64(hteno_solver* s, const Geo& G, const double* q, const uint8_t* mx, const uint8_t* my,
                 long long* counts);

// Bit-reproducible FP64 path (fv2d_fp64.cu)
int fv2d_fp64_setup(hteno_solver* s);
void fv2d_fp64_prim(hteno_solver* s, const Geo& G, const Work<double>& W, const double* q,
                    StepState* st, int do_max);
void fv2d_fp64_stage(hteno_solver* s, const Geo& G, const Work<double>& W, int stage,
                     const double* q, double* out);
// One fused launch per stage instead of five (hteno_set_fp64_fused): the same bits.
void fv2d_fp64_fused_step(hteno_solver* s, const Geo& G, const Work<double>& W);

}  // namespace hteno
