// Plain FP64 path of FV::System2D, bit-reproducible against the reference's arithmetic
// (see parity_math.cuh).  This translation unit is compiled with --fmad=false.
//
// Per stage (FV_System2D.cpp:363-573): faces<X>, faces<Y> (Roe average, characteristic
// projection of the 6-cell stencil, TENO5 on the 4 fields), flux<X>, flux<Y> (GL3 along the face
// over the face values of the 5 neighbouring faces, each in its own basis as in the reference;
// back-projection with the face's R; HLLC or Rusanov at the 3 Gauss points; quadrature), update
// (flux difference, SSP-RK3 stage, primitives of the new state, max wave speed on stage 3).
#include "fv2d_common.cuh"
#include "parity_math.cuh"
#include "harvest.cuh"

namespace hteno {
namespace {

__constant__ DevConst c_dev;
unsigned long long g_mask = 0;
std::mutex g_mu;

#include "common_kernels.cuh"

// primitives: calcPrimitiveVariable (FV_System2D.cpp:226-263)
// The three divisions by rho share one correctly rounded reciprocal (par::quot: the same bits as
// the divisions, Markstein).
__device__ __forceinline__ void cell_prim(double g1, const double* q, double* w, double& h,
                                          double& sr) {
  const par::Den d = par::den_of(q[0]);
  w[0] = q[0];
  w[1] = par::quot(q[1], d);
  w[2] = par::quot(q[2], d);
  w[3] = (q[3] - 0.5 * (q[1] * w[1] + q[2] * w[2])) * g1;  // par::primitive's pressure
  sr = sqrt(fabs(w[0]));
  h = par::quot(q[3] + w[3], d);
}

__global__ void kp_prim(Geo G, const double* __restrict__ q, double* __restrict__ prim,
                        StepState* st, int do_max) {
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  if (k < nc) {
    double qq[4] = {q[k], q[nc + k], q[2 * nc + k], q[3 * nc + k]}, w[4], h, sr;
    cell_prim(G.g1, qq, w, h, sr);
    prim[k] = w[1];
    prim[nc + k] = w[2];
    prim[2 * nc + k] = h;
    prim[3 * nc + k] = sr;
    ms = par::max_speed2(G.gamma, w);
  }
  if (do_max) block_max_to(ms, &st->maxbits);
}

// ---- uniform regions ---------------------------------------------------------------------------
// deep[k] = 1 when the 7 x 7 block of cells centred on cell k (boundary-mapped as every stencil
// maps it) holds one state, bit for bit, and that state is tame: density and pressure positive
// and within [2^-64, 2^64], Mach number at most 8.  Every input of the two x fluxes and of the two
// y fluxes of cell k then comes from identical cells, so each pair is computed from identical
// data, and the pair's difference -- the cell's residual -- is exactly +0 as long as the flux is
// finite.  The bounds make it so: reconstructing identical values through the characteristic
// basis (condition ~ Mach^2) returns the state to a relative 2^-40, positive, and no product of
// the face or flux arithmetic leaves the double range.  The stage skips the faces only such cells
// use and gives such cells a zero residual: the results are the same bits as the full stage.
__device__ __forceinline__ int cmap_any(int i, int n, int bc) {  // any offset (tiles past the edge)
  if (bc == HTENO_BC_PERIODIC) {
    i %= n;
    return i < 0 ? i + n : i;
  }
  return min(max(i, 0), n - 1);
}

__global__ void __launch_bounds__(256) kp_deep(Geo G, const double* __restrict__ q,
                                               uint8_t* __restrict__ deep, StepState* st) {
  if (st && st->done) return;
  constexpr int TX = 32, TY = 8, W = TX + 6, H = TY + 6;
  __shared__ unsigned long long key[4][H][W];
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const size_t nc = size_t(G.nx) * G.ny;
  const bool ghosts = G.bc >= HTENO_BC_TAYLOR;  // ghosts that are not copies: compare their states
  const double t = st ? st->t : G.t0;
  for (int it = threadIdx.x; it < W * H; it += blockDim.x) {
    const int y = it / W, x = it - y * W;
    double qq[4];
    if (ghosts) {
      bc_state(G, q, i0 - 3 + x, j0 - 3 + y, t, qq);
    } else {
      const size_t k = size_t(cmap_any(j0 - 3 + y, G.ny, G.bc)) * G.nx + cmap_any(i0 - 3 + x, G.nx, G.bc);
#pragma unroll
      for (int v = 0; v < 4; ++v) qq[v] = q[v * nc + k];
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) key[v][y][x] = static_cast<unsigned long long>(__double_as_longlong(qq[v]));
  }
  __syncthreads();
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int gi = i0 + tx, gj = j0 + ty;
  bool u = false;
  if (gi < G.nx && gj < G.ny) {
    const unsigned long long c0 = key[0][ty + 3][tx + 3], c1 = key[1][ty + 3][tx + 3];
    const unsigned long long c2 = key[2][ty + 3][tx + 3], c3 = key[3][ty + 3][tx + 3];
    const double qc[4] = {__longlong_as_double(static_cast<long long>(c0)),
                          __longlong_as_double(static_cast<long long>(c1)),
                          __longlong_as_double(static_cast<long long>(c2)),
                          __longlong_as_double(static_cast<long long>(c3))};
    double w[4];
    par::primitive(G.g1, qc, w);
    constexpr double lo = 0x1p-64, hi = 0x1p64;
    u = w[0] >= lo && w[0] <= hi && w[3] >= lo && w[3] <= hi &&
        w[1] * w[1] + w[2] * w[2] <= 64.0 * (G.gamma * w[3] / w[0]);
#pragma unroll
    for (int dy = 0; dy < 7; ++dy)
#pragma unroll
      for (int dx = 0; dx < 7; ++dx)
        u &= key[0][ty + dy][tx + dx] == c0 && key[1][ty + dy][tx + dx] == c1 &&
             key[2][ty + dy][tx + dx] == c2 && key[3][ty + dy][tx + dx] == c3;
    deep[size_t(gj) * G.nx + gi] = u ? 1 : 0;
  }
  // cells given their zero residual this stage (every thread reaches the count)
  const int n = __syncthreads_count(u);
  if (threadIdx.x == 0 && n && st) atomicAdd(&st->uniform, (unsigned long long)n);
}

template <int DIR>
__global__ void __launch_bounds__(kFaceThreads) kp_faces(Geo G, const double* __restrict__ q,
                                                         const double* __restrict__ prim,
                                                         double* __restrict__ fc,
                                                         double* __restrict__ froe,
                                                         const StepState* st,
                                                         const uint8_t* __restrict__ deep = nullptr) {
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
    const int m = bmap(s, ns, G.bc);
    return DIR == 1 ? size_t(t) * G.nx + m : size_t(m) * G.nx + t;
  };
  if (deep) {
    // no flux face computed this stage reads this face: those are the faces (f, t + m), |m| <= 2,
    // whose two cells are not both deep
    const int a = bmap(f - 1, ns, G.bc), b = bmap(f, ns, G.bc);
    bool skip = true;
#pragma unroll
    for (int m = -2; m <= 2; ++m) {
      const int tt = bmap(t + m, nt, G.bc);
      const size_t ka = DIR == 1 ? size_t(tt) * G.nx + a : size_t(a) * G.nx + tt;
      const size_t kb = DIR == 1 ? size_t(tt) * G.nx + b : size_t(b) * G.nx + tt;
      skip = skip && deep[ka] && deep[kb];
    }
    if (skip) return;
  }
  const size_t ca = cell(f - 1), cb = cell(f);
  const par::Eig E = par::eig(G.g1, DIR, prim[3 * nc + ca], prim[ca], prim[nc + ca],
                              prim[2 * nc + ca], prim[3 * nc + cb], prim[cb], prim[nc + cb],
                              prim[2 * nc + cb]);
  double ch[4][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const size_t c = cell(f - 3 + m);
    const double qq[4] = {q[c], q[nc + c], q[2 * nc + c], q[3 * nc + c]};
    double cc[4];
    par::left(E, DIR, qq, cc);
#pragma unroll
    for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
  }
  const size_t nface = size_t(nf) * nt;
  const size_t o = DIR == 1 ? size_t(t) * nf + f : size_t(f) * nt + t;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double a, b;
    par::lagrange_recon(c_dev, G.recon, ch[r], a, b);
    fc[r * nface + o] = a;
    fc[(4 + r) * nface + o] = b;
  }
  froe[0 * nface + o] = E.vxm;
  froe[1 * nface + o] = E.vym;
  froe[2 * nface + o] = E.hm;
  froe[3 * nface + o] = E.qm;
  froe[4 * nface + o] = E.cm;
  froe[5 * nface + o] = E.rcm;
  froe[6 * nface + o] = E.b1;
}

// Training stencils of the learned classifier from the current state (see harvest.cuh): every
// face of direction DIR, 4 characteristic fields, both sides, each kept with probability p.
template <int DIR>
__global__ void __launch_bounds__(kFaceThreads) kp_harvest(Geo G, const double* __restrict__ q,
                                                           const double* __restrict__ prim, double p,
                                                           unsigned long long seed, uint16_t* X,
                                                           uint8_t* Y, long cap,
                                                           unsigned long long* count) {
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
    const int m = bmap(s, ns, G.bc);
    return DIR == 1 ? size_t(t) * G.nx + m : size_t(m) * G.nx + t;
  };
  const size_t ca = cell(f - 1), cb = cell(f);
  const par::Eig E = par::eig(G.g1, DIR, prim[3 * nc + ca], prim[ca], prim[nc + ca],
                              prim[2 * nc + ca], prim[3 * nc + cb], prim[cb], prim[nc + cb],
                              prim[2 * nc + cb]);
  double ch[4][6];
  for (int m = 0; m < 6; ++m) {
    const size_t c = cell(f - 3 + m);
    const double qq[4] = {q[c], q[nc + c], q[2 * nc + c], q[3 * nc + c]};
    double cc[4];
    par::left(E, DIR, qq, cc);
    for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
  }
  for (int r = 0; r < 4; ++r) {
    const uint64_t id = ((uint64_t(DIR) * 4 + r) << 40) + uint64_t(idx);
    harvest::emit_both(ch[r], G.recon == HTENO_RECON_TENO5I, seed, id, p, X, Y, cap, count);
  }
}

// FP64 judge of a mixed-precision solver's learned routing: for every face whose route byte
// (layout of the mixed stage kernel's masks: x faces [ny][nx+1], y faces [ny+1][nx]) routes a
// stencil, the face's characteristic stencils in double from the double state (Roe average of
// the two cells, the 6 cells projected) and, per routed (field, side), the TENO cut-off the plain
// FP64 solver decides on that stencil.  out[0] += routed stencils, out[1] += those whose cut-off
// drops a candidate (pattern != 7); out[2], out[3]: the same over the routed stencils whose
// variation is resolved in float (max - min of the 5-value window above 2^-16 of its largest
// magnitude, ~500 float ulps).  Below that the window's shape -- and the cut-off decided on it --
// is set by the rounding noise the float fluxes leave in the state, and linear weights there
// change the solution by no more than that noise.
template <int DIR>
__global__ void __launch_bounds__(kFaceThreads) kp_audit64(Geo G, const double* __restrict__ q,
                                                           const uint8_t* __restrict__ mask,
                                                           unsigned long long* out) {
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  int routed = 0, wrong = 0, routed_r = 0, wrong_r = 0;
  if (idx < long(nf) * nt) {
    int f, t;
    if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
    else { t = int(idx % nt); f = int(idx / nt); }
    const uint8_t route = mask[DIR == 1 ? size_t(t) * nf + f : size_t(f) * nt + t];
    if (route) {
      const size_t nc = size_t(G.nx) * G.ny;
      const int ns = DIR == 1 ? G.nx : G.ny;
      auto cell = [&](int s) -> size_t {
        const int m = bmap(s, ns, G.bc);
        return DIR == 1 ? size_t(t) * G.nx + m : size_t(m) * G.nx + t;
      };
      double qa[4], qb[4], wa[4], wb[4], ha, hb, sra, srb;
      const size_t ca = cell(f - 1), cb = cell(f);
      for (int v = 0; v < 4; ++v) {
        qa[v] = q[v * nc + ca];
        qb[v] = q[v * nc + cb];
      }
      cell_prim(G.g1, qa, wa, ha, sra);
      cell_prim(G.g1, qb, wb, hb, srb);
      const par::Eig E = par::eig(G.g1, DIR, sra, wa[1], wa[2], ha, srb, wb[1], wb[2], hb);
      double ch[4][6];
      for (int m = 0; m < 6; ++m) {
        const size_t c = cell(f - 3 + m);
        const double qq[4] = {q[c], q[nc + c], q[2 * nc + c], q[3 * nc + c]};
        double cc[4];
        par::left(E, DIR, qq, cc);
        for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
      }
      for (int b = 0; b < 8; ++b) {
        if (!((route >> b) & 1)) continue;
        const double* v = ch[b >> 1] + (b & 1);  // side 1 reconstructs from cells 1..5
        double SI[3];
        par::lagrange_si(v, SI);
        const int bad = par::teno_decide(v, SI, G.recon == HTENO_RECON_TENO5I) != 7;
        double lo = v[0], hi = v[0];
        for (int m = 1; m < 5; ++m) {
          lo = fmin(lo, v[m]);
          hi = fmax(hi, v[m]);
        }
        const int res = (hi - lo) > 0x1p-16 * fmax(fabs(lo), fabs(hi));
        routed += 1;
        wrong += bad;
        routed_r += res;
        wrong_r += res & bad;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    routed += __shfl_xor_sync(0xffffffffu, routed, o);
    wrong += __shfl_xor_sync(0xffffffffu, wrong, o);
    routed_r += __shfl_xor_sync(0xffffffffu, routed_r, o);
    wrong_r += __shfl_xor_sync(0xffffffffu, wrong_r, o);
  }
  if ((threadIdx.x & 31) == 0 && routed) {
    atomicAdd(out, (unsigned long long)routed);
    if (wrong) atomicAdd(out + 1, (unsigned long long)wrong);
    if (routed_r) atomicAdd(out + 2, (unsigned long long)routed_r);
    if (wrong_r) atomicAdd(out + 3, (unsigned long long)wrong_r);
  }
}

// kp_faces for boundaries whose ghosts are not copies of interior cells (HTENO_BC_TAYLOR,
// _DOUBLE_MACH): every state comes from bc_state(), the primitives of the two Roe cells are
// computed from their states (calcPrimitiveVariable covers the ghosts, :231-262), and the face
// rows -2, -1, nt, nt + 1 that the transverse GL3 reads are computed too (the reference sweeps
// every row, :373-400), into gfc [4 rows][8][nf].
template <int DIR>
__global__ void __launch_bounds__(kFaceThreads) kp_faces_g(Geo G, const double* __restrict__ q,
                                                           double* __restrict__ fc,
                                                           double* __restrict__ froe,
                                                           double* __restrict__ gfc,
                                                           const StepState* st,
                                                           const uint8_t* __restrict__ deep) {
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (idx >= long(nf) * (nt + 4)) return;
  int f, t;
  if (DIR == 1) { f = int(idx % nf); t = int(idx / nf) - 2; }
  else { t = int(idx % (nt + 4)) - 2; f = int(idx / (nt + 4)); }
  const int ns = DIR == 1 ? G.nx : G.ny;
  if (deep) {
    // the fluxes that read this face value are those of faces (f, t + m), |m| <= 2, of the
    // interior rows; skipped when every one of them is (both of its cells deep)
    const int a = min(max(f - 1, 0), ns - 1), b = min(max(f, 0), ns - 1);
    bool skip = true;
#pragma unroll
    for (int m = -2; m <= 2; ++m) {
      const int tt = t + m;
      if (tt < 0 || tt >= nt) continue;
      const size_t ka = DIR == 1 ? size_t(tt) * G.nx + a : size_t(a) * G.nx + tt;
      const size_t kb = DIR == 1 ? size_t(tt) * G.nx + b : size_t(b) * G.nx + tt;
      skip = skip && deep[ka] && deep[kb];
    }
    if (skip) return;
  }
  const double tm = st ? st->t : G.t0;
  auto state = [&](int s, double* o) {
    if (DIR == 1) bc_state(G, q, s, t, tm, o);
    else bc_state(G, q, t, s, tm, o);
  };
  double qa[4], qb[4], wa[4], wb[4], ha, hb, sra, srb;
  state(f - 1, qa);
  state(f, qb);
  cell_prim(G.g1, qa, wa, ha, sra);
  cell_prim(G.g1, qb, wb, hb, srb);
  const par::Eig E = par::eig(G.g1, DIR, sra, wa[1], wa[2], ha, srb, wb[1], wb[2], hb);
  double ch[4][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    double qq[4], cc[4];
    state(f - 3 + m, qq);
    par::left(E, DIR, qq, cc);
#pragma unroll
    for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
  }
  const bool interior = t >= 0 && t < nt;
  const size_t nface = size_t(nf) * nt;
  const size_t o = DIR == 1 ? size_t(t) * nf + f : size_t(f) * nt + t;
  const size_t go = size_t(t < 0 ? t + 2 : t - nt + 2) * 8 * nf + f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    double va, vb;
    par::lagrange_recon(c_dev, G.recon, ch[r], va, vb);
    if (interior) {
      fc[r * nface + o] = va;
      fc[(4 + r) * nface + o] = vb;
    } else {
      gfc[go + r * nf] = va;
      gfc[go + (4 + r) * nf] = vb;
    }
  }
  if (!interior) return;
  froe[0 * nface + o] = E.vxm;
  froe[1 * nface + o] = E.vym;
  froe[2 * nface + o] = E.hm;
  froe[3 * nface + o] = E.qm;
  froe[4 * nface + o] = E.cm;
  froe[5 * nface + o] = E.rcm;
  froe[6 * nface + o] = E.b1;
}

template <int DIR>
__global__ void __launch_bounds__(kFaceThreads) kp_flux(Geo G, const double* __restrict__ fc,
                                                        const double* __restrict__ froe,
                                                        double* __restrict__ F,
                                                        const StepState* st,
                                                        const uint8_t* __restrict__ deep = nullptr,
                                                        const double* __restrict__ gfc = nullptr) {
  if (st && st->done) return;
  const int nf = DIR == 1 ? G.nx + 1 : G.ny + 1;
  const int nt = DIR == 1 ? G.ny : G.nx;
  const long idx = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (idx >= long(nf) * nt) return;
  int f, t;
  if (DIR == 1) { f = int(idx % nf); t = int(idx / nf); }
  else { t = int(idx % nt); f = int(idx / nt); }
  if (deep) {  // both cells deep: neither reads this flux
    const int ns = DIR == 1 ? G.nx : G.ny;
    const int a = bmap(f - 1, ns, G.bc), b = bmap(f, ns, G.bc);
    const size_t ka = DIR == 1 ? size_t(t) * G.nx + a : size_t(a) * G.nx + t;
    const size_t kb = DIR == 1 ? size_t(t) * G.nx + b : size_t(b) * G.nx + t;
    if (deep[ka] && deep[kb]) return;
  }
  const size_t nface = size_t(nf) * nt;
  size_t nb[5];
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    const int mm = bmap(t - 2 + m, nt, G.bc);
    nb[m] = DIR == 1 ? size_t(mm) * nf + f : size_t(f) * nt + mm;
  }
  double g[8][3];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    double u5[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const int tr = t - 2 + m;
      if (gfc && (tr < 0 || tr >= nt))  // a face row of the ghosts (kp_faces_g)
        u5[m] = gfc[(size_t(tr < 0 ? tr + 2 : tr - nt + 2) * 8 + r) * nf + f];
      else
        u5[m] = fc[r * nface + nb[m]];
    }
    par::gl3(c_dev, u5, g[r]);
  }
  const size_t o = nb[2];
  par::Eig E;
  E.vxm = froe[o];
  E.vym = froe[nface + o];
  E.hm = froe[2 * nface + o];
  E.qm = froe[3 * nface + o];
  E.cm = froe[4 * nface + o];
  E.rcm = froe[5 * nface + o];
  E.b1 = froe[6 * nface + o];
  const double vn = DIR == 1 ? E.vxm : E.vym;  // derived scalars, recomputed bit-identically
  E.t0r = vn * E.cm;
  E.b2 = E.qm * E.b1;
  E.s0 = vn * E.rcm;
  E.s1 = E.b1 * vn;
  E.t2 = 0.5 * E.b1;
  double Fm[3][4];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const double cl[4] = {g[0][m], g[1][m], g[2][m], g[3][m]};
    const double cr[4] = {g[4][m], g[5][m], g[6][m], g[7][m]};
    double ql[4], qr[4], Fl[4];
    par::right(E, DIR, cl, ql);
    par::right(E, DIR, cr, qr);
    if (G.flux == HTENO_FLUX_HLLC) par::hllc(G.g1, DIR, ql, qr, Fl);
    else par::rusanov(G.gamma, G.g1, DIR, E, ql, qr, Fl);
#pragma unroll
    for (int v = 0; v < 4; ++v) Fm[m][v] = c_dev.gl3w[m] * Fl[v];
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) F[v * nface + o] = (Fm[0][v] + Fm[1][v]) + Fm[2][v];
}

// rhs (FV_System2D.cpp:562-572) + RungeKutta3 (:575-612); stage 0 writes the residual
__global__ void kp_update(Geo G, int stage, const double* __restrict__ fx,
                          const double* __restrict__ fy, double* __restrict__ q,
                          double* __restrict__ q0, double* __restrict__ prim,
                          double* __restrict__ out, StepState* st,
                          const uint8_t* __restrict__ deep = nullptr) {
  if (st && st->done) return;
  const size_t nc = size_t(G.nx) * G.ny;
  const size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double ms = 0.0;
  int bad = 0;
  if (k < nc) {
    const int i = int(k % G.nx), j = int(k / G.nx);
    const size_t nxf = size_t(G.nx + 1) * G.ny, nyf = size_t(G.ny + 1) * G.nx;
    const size_t ox = size_t(j) * (G.nx + 1) + i, oy = size_t(j) * G.nx + i;
    double rhs[4] = {0.0, 0.0, 0.0, 0.0};  // a deep cell's flux pairs are equal: residual +0
    if (!(deep && deep[k])) {
      const par::Den da = par::den_of(G.area);  // the four divisions by the cell area
#pragma unroll
      for (int v = 0; v < 4; ++v)
        rhs[v] = par::quot((fx[v * nxf + ox] - fx[v * nxf + ox + 1]) * G.dy +
                               (fy[v * nyf + oy] - fy[v * nyf + oy + G.nx]) * G.dx,
                           da) + 0.0;
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
      double w[4], h, sr;
      cell_prim(G.g1, qn, w, h, sr);
      prim[k] = w[1];
      prim[nc + k] = w[2];
      prim[2 * nc + k] = h;
      prim[3 * nc + k] = sr;
      if (stage == 3) ms = par::max_speed2(G.gamma, w);
      bad = (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2]) || isnan(qn[3])) ? 1 : 0;
      bad |= (qn[0] <= 0.0 || w[3] <= 0.0) ? 2 : 0;
    }
  }
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad && st) atomicOr(&st->status, bad);
}

// ---- one fused launch per stage (hteno_set_fp64_fused) -------------------------------------------
// The five launches of a stage (uniform test, faces x/y, fluxes x/y, update) as one kernel over
// tiles of TX x TY cells, face values and fluxes in shared memory, the same arithmetic in the same
// order as the launches above (the same bits).  Per tile: (A) the state with a 3-cell halo; (B) the
// uniform cells of the tile (kp_deep's test); (C) the x face values of rows -2 .. TY+1 that the x
// fluxes of non-uniform cells read, (D) those x fluxes, (E) their difference times dy per cell;
// (F, G) the same for y; (H) the residual and the SSP-RK3 stage.  The Roe average of a face is
// computed again for its flux rather than kept, and 32 x 16 tiles (104 KB of shared memory) let two
// tiles share an SM, so that one tile's phases fill the other's barrier waits.  Stage buffers: a stage reads its input state and primitives with halos from
// qin / pin, the step-start state pointwise from qbase, and writes qout / pout; stage 3 writes the
// state in place over the step-start copy, which only the owning thread reads.  Zero-gradient and
// periodic boundaries (the halo is mapped as every stencil maps it).
constexpr int kS64X = 32, kS64Y = 16, kS64Threads = 256;  // two tiles per SM

template <int TX, int TY>
struct S64Smem {
  static constexpr int C = (TY + 4) * (TX + 1) > (TY + 1) * (TX + 4) ? (TY + 4) * (TX + 1)
                                                                      : (TY + 1) * (TX + 4);
  static constexpr int F = (TY + 1) * (TX + 1);
  double q[4][TY + 6][TX + 6];
  double c[8][C];   // face values of one direction (x: rows -2 .. TY+1 x TX+1; y: TY+1 x columns -2 .. TX+1)
  double f[4][F];   // fluxes of one direction
  double rx[4][TY][TX];  // (fx_i - fx_i+1) * dy of each cell
  unsigned char deep[TY][TX];
  unsigned char fneed[F];
};

template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, 2) kp_stage64(Geo G, int stage, const double* __restrict__ qin,
                                                  const double* qbase, double* qout,
                                                  const double* __restrict__ pin,
                                                  double* __restrict__ pout, StepState* st,
                                                  int skip_uniform) {
  if (st->done) return;
  extern __shared__ __align__(16) unsigned char s64raw[];
  S64Smem<TX, TY>& S = *reinterpret_cast<S64Smem<TX, TY>*>(s64raw);
  constexpr int XF = TX + 1, YC = TX + 4;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int wx = min(TX, G.nx - i0), wy = min(TY, G.ny - j0);
  const size_t nc = size_t(G.nx) * G.ny;
  const int tid = threadIdx.x;
  auto row = [&](int j) { return cmap_any(j0 + j, G.ny, G.bc); };
  auto col = [&](int i) { return cmap_any(i0 + i, G.nx, G.bc); };
  // A: state tile, halo 3
  for (int it = tid; it < (TY + 6) * (TX + 6); it += NT) {
    const int y = it / (TX + 6), x = it - y * (TX + 6);
    const size_t k = size_t(row(y - 3)) * G.nx + col(x - 3);
#pragma unroll
    for (int v = 0; v < 4; ++v) S.q[v][y][x] = qin[v * nc + k];
  }
  __syncthreads();
  // B: uniform cells (kp_deep)
  int nd = 0;
  for (int it = tid; it < TY * TX; it += NT) {
    const int ty = it / TX, tx = it - ty * TX;
    bool u = false;
    if (skip_uniform && ty < wy && tx < wx) {
      const double qc[4] = {S.q[0][ty + 3][tx + 3], S.q[1][ty + 3][tx + 3], S.q[2][ty + 3][tx + 3],
                            S.q[3][ty + 3][tx + 3]};
      double w[4];
      par::primitive(G.g1, qc, w);
      constexpr double lo = 0x1p-64, hi = 0x1p64;
      u = w[0] >= lo && w[0] <= hi && w[3] >= lo && w[3] <= hi &&
          w[1] * w[1] + w[2] * w[2] <= 64.0 * (G.gamma * w[3] / w[0]);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const long long c = __double_as_longlong(qc[v]);
        for (int dy = 0; dy < 7; ++dy)
#pragma unroll
          for (int dx = 0; dx < 7; ++dx) u &= __double_as_longlong(S.q[v][ty + dy][tx + dx]) == c;
      }
    }
    S.deep[ty][tx] = u ? 1 : 0;
    nd += u ? 1 : 0;
  }
  const int n1 = __syncthreads_count(nd >= 1), n2 = __syncthreads_count(nd >= 2);
  if (tid == 0 && n1 + n2) atomicAdd(&st->uniform, (unsigned long long)(n1 + n2));
  const bool all_uniform = n1 + n2 == wx * wy;
  if (!all_uniform) {
    // ---- x faces: flux (t, f) is needed when a non-uniform cell of the tile reads it
    for (int it = tid; it < TY * XF; it += NT) {
      const int t = it / XF, f = it - t * XF;
      S.fneed[it] = t < wy && f <= wx &&
                    ((f >= 1 && !S.deep[t][f - 1]) || (f < wx && !S.deep[t][f]));
    }
    __syncthreads();
    // C: x face values of rows -2 .. wy + 1 (kp_faces<1>)
    for (int it = tid; it < (TY + 4) * XF; it += NT) {
      const int r = it / XF - 2, f = it - (r + 2) * XF;
      if (r > wy + 1 || f > wx) continue;
      bool need = false;
#pragma unroll
      for (int m = -2; m <= 2; ++m) {
        const int t = r + m;
        need |= t >= 0 && t < wy && S.fneed[t * XF + f];
      }
      if (!need) continue;
      const size_t ca = size_t(row(r)) * G.nx + col(f - 1), cb = size_t(row(r)) * G.nx + col(f);
      const par::Eig E = par::eig(G.g1, 1, pin[3 * nc + ca], pin[ca], pin[nc + ca], pin[2 * nc + ca],
                                  pin[3 * nc + cb], pin[cb], pin[nc + cb], pin[2 * nc + cb]);
      double ch[4][6];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const double qq[4] = {S.q[0][r + 3][f + m], S.q[1][r + 3][f + m], S.q[2][r + 3][f + m],
                              S.q[3][r + 3][f + m]};
        double cc[4];
        par::left(E, 1, qq, cc);
#pragma unroll
        for (int a = 0; a < 4; ++a) ch[a][m] = cc[a];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        double lo, hi;
        par::lagrange_recon(c_dev, G.recon, ch[a], lo, hi);
        S.c[a][it] = lo;
        S.c[4 + a][it] = hi;
      }
    }
    __syncthreads();
    // D: x fluxes (kp_flux<1>)
    for (int it = tid; it < TY * XF; it += NT) {
      if (!S.fneed[it]) continue;
      const int t = it / XF, f = it - t * XF;
      double g[8][3];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        double u5[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) u5[m] = S.c[a][(t + m) * XF + f];
        par::gl3(c_dev, u5, g[a]);
      }
      const size_t ca = size_t(row(t)) * G.nx + col(f - 1), cb = size_t(row(t)) * G.nx + col(f);
      const par::Eig E = par::eig(G.g1, 1, pin[3 * nc + ca], pin[ca], pin[nc + ca], pin[2 * nc + ca],
                                  pin[3 * nc + cb], pin[cb], pin[nc + cb], pin[2 * nc + cb]);
      double Fm[3][4];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const double cl[4] = {g[0][m], g[1][m], g[2][m], g[3][m]};
        const double cr[4] = {g[4][m], g[5][m], g[6][m], g[7][m]};
        double ql[4], qr[4], Fl[4];
        par::right(E, 1, cl, ql);
        par::right(E, 1, cr, qr);
        if (G.flux == HTENO_FLUX_HLLC) par::hllc(G.g1, 1, ql, qr, Fl);
        else par::rusanov(G.gamma, G.g1, 1, E, ql, qr, Fl);
#pragma unroll
        for (int v = 0; v < 4; ++v) Fm[m][v] = c_dev.gl3w[m] * Fl[v];
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) S.f[v][it] = (Fm[0][v] + Fm[1][v]) + Fm[2][v];
    }
    __syncthreads();
    // E: x flux difference times dy of each non-uniform cell (kp_update's first term)
    for (int it = tid; it < TY * TX; it += NT) {
      const int t = it / TX, i = it - t * TX;
      if (t < wy && i < wx && !S.deep[t][i]) {
#pragma unroll
        for (int v = 0; v < 4; ++v) S.rx[v][t][i] = (S.f[v][t * XF + i] - S.f[v][t * XF + i + 1]) * G.dy;
      }
    }
    // ---- y faces: flux (g, t) of face row g (between cell rows g - 1 and g), column t
    for (int it = tid; it < (TY + 1) * TX; it += NT) {
      const int g = it / TX, t = it - g * TX;
      S.fneed[it] = g <= wy && t < wx &&
                    ((g >= 1 && !S.deep[g - 1][t]) || (g < wy && !S.deep[g][t]));
    }
    __syncthreads();
    // F: y face values of columns -2 .. wx + 1 (kp_faces<2>)
    for (int it = tid; it < (TY + 1) * YC; it += NT) {
      const int g = it / YC, cc = it - g * YC - 2;
      if (g > wy || cc > wx + 1) continue;
      bool need = false;
#pragma unroll
      for (int m = -2; m <= 2; ++m) {
        const int t = cc + m;
        need |= t >= 0 && t < wx && S.fneed[g * TX + t];
      }
      if (!need) continue;
      const size_t ca = size_t(row(g - 1)) * G.nx + col(cc), cb = size_t(row(g)) * G.nx + col(cc);
      const par::Eig E = par::eig(G.g1, 2, pin[3 * nc + ca], pin[ca], pin[nc + ca], pin[2 * nc + ca],
                                  pin[3 * nc + cb], pin[cb], pin[nc + cb], pin[2 * nc + cb]);
      double ch[4][6];
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const double qq[4] = {S.q[0][g + m][cc + 3], S.q[1][g + m][cc + 3], S.q[2][g + m][cc + 3],
                              S.q[3][g + m][cc + 3]};
        double c4[4];
        par::left(E, 2, qq, c4);
#pragma unroll
        for (int a = 0; a < 4; ++a) ch[a][m] = c4[a];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        double lo, hi;
        par::lagrange_recon(c_dev, G.recon, ch[a], lo, hi);
        S.c[a][it] = lo;
        S.c[4 + a][it] = hi;
      }
    }
    __syncthreads();
    // G: y fluxes (kp_flux<2>)
    for (int it = tid; it < (TY + 1) * TX; it += NT) {
      if (!S.fneed[it]) continue;
      const int g = it / TX, t = it - g * TX;
      double gg[8][3];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        double u5[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) u5[m] = S.c[a][g * YC + t + m];
        par::gl3(c_dev, u5, gg[a]);
      }
      const size_t ca = size_t(row(g - 1)) * G.nx + col(t), cb = size_t(row(g)) * G.nx + col(t);
      const par::Eig E = par::eig(G.g1, 2, pin[3 * nc + ca], pin[ca], pin[nc + ca], pin[2 * nc + ca],
                                  pin[3 * nc + cb], pin[cb], pin[nc + cb], pin[2 * nc + cb]);
      double Fm[3][4];
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const double cl[4] = {gg[0][m], gg[1][m], gg[2][m], gg[3][m]};
        const double cr[4] = {gg[4][m], gg[5][m], gg[6][m], gg[7][m]};
        double ql[4], qr[4], Fl[4];
        par::right(E, 2, cl, ql);
        par::right(E, 2, cr, qr);
        if (G.flux == HTENO_FLUX_HLLC) par::hllc(G.g1, 2, ql, qr, Fl);
        else par::rusanov(G.gamma, G.g1, 2, E, ql, qr, Fl);
#pragma unroll
        for (int v = 0; v < 4; ++v) Fm[m][v] = c_dev.gl3w[m] * Fl[v];
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) S.f[v][it] = (Fm[0][v] + Fm[1][v]) + Fm[2][v];
    }
    __syncthreads();
  }
  // H: residual and SSP-RK3 stage (kp_update)
  double ms = 0.0;
  int bad = 0;
  const double dt = st->dt;
  for (int it = tid; it < TY * TX; it += NT) {
    const int t = it / TX, i = it - t * TX;
    if (t >= wy || i >= wx) continue;
    const size_t k = size_t(j0 + t) * G.nx + (i0 + i);
    double rhs[4] = {0.0, 0.0, 0.0, 0.0};  // a uniform cell's flux pairs are equal: residual +0
    if (!S.deep[t][i]) {
      const par::Den da = par::den_of(G.area);
#pragma unroll
      for (int v = 0; v < 4; ++v)
        rhs[v] = par::quot(S.rx[v][t][i] + (S.f[v][t * TX + i] - S.f[v][(t + 1) * TX + i]) * G.dx,
                           da) + 0.0;
    }
    double qn[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const double cur = S.q[v][t + 3][i + 3];
      const double base = stage == 1 ? cur : qbase[v * nc + k];
      qn[v] = ssprk3(base, cur, rhs[v], dt, stage);
      qout[v * nc + k] = qn[v];
    }
    double w[4], h, sr;
    cell_prim(G.g1, qn, w, h, sr);
    pout[k] = w[1];
    pout[nc + k] = w[2];
    pout[2 * nc + k] = h;
    pout[3 * nc + k] = sr;
    if (stage == 3) ms = fmax(ms, par::max_speed2(G.gamma, w));
    bad |= (isnan(qn[0]) || isnan(qn[1]) || isnan(qn[2]) || isnan(qn[3])) ? 1 : 0;
    bad |= (qn[0] <= 0.0 || w[3] <= 0.0) ? 2 : 0;
  }
  if (stage == 3) block_max_to(ms, &st->maxbits);
  if (bad) atomicOr(&st->status, bad);
}

}  // namespace

int fv2d_fp64_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  if (s->cfg.precision == HTENO_PREC_FP64 && !s->deep) {
    const cudaError_t e = cudaMalloc(&s->deep, size_t(s->cfg.nx) * s->cfg.ny);
    if (e != cudaSuccess) return cuda_error(s, e, "uniform-region flags");
  }
  if (s->cfg.precision == HTENO_PREC_FP64 && make_side_stream(s) != HTENO_OK) return HTENO_ERR_CUDA;
  if (s->cfg.precision == HTENO_PREC_FP64 && s->cfg.bc >= HTENO_BC_TAYLOR && !s->ghost_faces) {
    const size_t n = size_t(32) * (s->cfg.nx + 1) + size_t(32) * (s->cfg.ny + 1);
    const cudaError_t e = cudaMalloc(&s->ghost_faces, n * sizeof(double));
    if (e != cudaSuccess) return cuda_error(s, e, "ghost face rows");
  }
  return HTENO_OK;
}

int fv2d_fp64_set_fused(hteno_solver* s, int on) {
  if (!on) {
    cudaFree(s->fused64);
    s->fused64 = nullptr;
    s->launches_per_step = 2 + 3 * (5 + (s->uniform_skip ? 1 : 0));
    return HTENO_OK;
  }
  if (!s->fused64) {
    cudaError_t e = cudaFuncSetAttribute(kp_stage64<kS64X, kS64Y, kS64Threads>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(sizeof(S64Smem<kS64X, kS64Y>)));
    if (e != cudaSuccess) return cuda_error(s, e, "fused stage shared memory");
    e = cudaMalloc(&s->fused64, 16 * s->ncell * sizeof(double));
    if (e != cudaSuccess) return cuda_error(s, e, "fused stage buffers");
  }
  s->launches_per_step = 2 + 3;
  return HTENO_OK;
}

void fv2d_fp64_fused_step(hteno_solver* s, const Geo& G, const Work<double>& W) {
  cudaStream_t cs = s->stream;
  const size_t nc = size_t(G.nx) * G.ny;
  const long nxf = long(G.nx + 1) * G.ny, nyf = long(G.ny + 1) * G.nx;
  const double ncd = double(nc);
  const double fluxf = G.flux == HTENO_FLUX_HLLC ? kFluxFlopsHllc : kFluxFlopsRusanov;
  // algorithmic bytes per cell: state with halo (38 x 22 / 32 x 16), step-start state, new state
  // and its primitives written, the Roe cells' primitives with their halo (36 x 20 / 32 x 16)
  const int kind = trace_kind(s, "stage", ncd * 193.0,
                              (kFacesFlops + fluxf) * double(nxf + nyf) + kUpdateFlops * ncd);
  double* q1 = s->fused64;
  double* q2 = q1 + 4 * nc;
  double* p1 = q2 + 4 * nc;
  double* p2 = p1 + 4 * nc;
  const dim3 grid(unsigned((G.nx + kS64X - 1) / kS64X), unsigned((G.ny + kS64Y - 1) / kS64Y));
  const size_t smem = sizeof(S64Smem<kS64X, kS64Y>);
  const int skip = s->uniform_skip ? 1 : 0;
  const double* qin[3] = {s->q, q1, q2};
  double* qout[3] = {q1, q2, s->q};
  const double* pin[3] = {W.prim, p1, p2};
  double* pout[3] = {p1, p2, W.prim};
  for (int stage = 1; stage <= 3; ++stage) {
    trace_begin(s, kind);
    kp_stage64<kS64X, kS64Y, kS64Threads><<<grid, kS64Threads, smem, cs>>>(G, stage, qin[stage - 1], s->q, qout[stage - 1],
                                                pin[stage - 1], pout[stage - 1], s->dstate, skip);
    trace_end(s);
  }
}

void fv2d_fp64_prim(hteno_solver* s, const Geo& G, const Work<double>& W, const double* q,
                    StepState* st, int do_max) {
  const size_t nc = size_t(G.nx) * G.ny;
  kp_prim<<<unsigned((nc + 255) / 256), 256, 0, s->stream>>>(G, q, W.prim, st, do_max);
}

void fv2d_fp64_stage(hteno_solver* s, const Geo& G, const Work<double>& W, int stage,
                     const double* q, double* out) {
  cudaStream_t cs = s->stream;
  const int nx = G.nx, ny = G.ny;
  const long nxf = long(nx + 1) * ny, nyf = long(ny + 1) * nx;
  const double ncd = double(nx) * ny;
  StepState* st = stage == 0 ? nullptr : s->dstate;
  const double fluxf = G.flux == HTENO_FLUX_HLLC ? kFluxFlopsHllc : kFluxFlopsRusanov;
  const int kf_x = trace_kind(s, "faces_x", ncd * 64 + double(nxf) * 15 * 8, kFacesFlops * nxf);
  const int kf_y = trace_kind(s, "faces_y", ncd * 64 + double(nyf) * 15 * 8, kFacesFlops * nyf);
  const int kx = trace_kind(s, "flux_x", double(nxf) * 19 * 8, fluxf * nxf);
  const int ky = trace_kind(s, "flux_y", double(nyf) * 19 * 8, fluxf * nyf);
  const int ku = trace_kind(s, "update", ncd * 128 + double(nxf + nyf) * 4 * 8, kUpdateFlops * ncd);
  // uniform regions (stepping only): the faces only deep cells use are skipped
  const uint8_t* deep = stage > 0 && s->uniform_skip ? s->deep : nullptr;
  if (deep) {
    const int ku0 = trace_kind(s, "uniform", ncd * 32, 0.0);
    trace_begin(s, ku0);
    kp_deep<<<dim3(unsigned((nx + 31) / 32), unsigned((ny + 7) / 8)), 256, 0, cs>>>(G, q, s->deep, st);
    trace_end(s);
  }
  // ghost face rows of the x faces ([4][8][nx + 1]) and of the y faces ([4][8][ny + 1])
  double* gx = s->ghost_faces;
  double* gy = gx ? gx + size_t(32) * (nx + 1) : nullptr;
  // the y-direction kernels touch none of the x-direction kernels' outputs: while stepping they
  // run on the side stream beside them, so that each kernel's last, partly filled wave of
  // blocks overlaps the other direction's work (one stream while kernels are being timed)
  // (if the fork cannot be recorded, the y kernels stay on the solver's stream)
  const bool fork = stage > 0 && s->side_stream && !s->timing &&
                    cudaEventRecord(s->fork_ev, cs) == cudaSuccess &&
                    cudaStreamWaitEvent(s->side_stream, s->fork_ev, 0) == cudaSuccess;
  cudaStream_t ys = fork ? s->side_stream : cs;
  trace_begin(s, kf_x);
  if (gx) {
    const long n = long(nx + 1) * (ny + 4);
    kp_faces_g<1><<<unsigned((n + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
        G, q, W.xc, W.xroe, gx, st, deep);
  } else {
    kp_faces<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
        G, q, W.prim, W.xc, W.xroe, st, deep);
  }
  trace_end(s);
  trace_begin(s, kf_y);
  if (gy) {
    const long n = long(ny + 1) * (nx + 4);
    kp_faces_g<2><<<unsigned((n + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, ys>>>(
        G, q, W.yc, W.yroe, gy, st, deep);
  } else {
    kp_faces<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, ys>>>(
        G, q, W.prim, W.yc, W.yroe, st, deep);
  }
  trace_end(s);
  trace_begin(s, kx);
  kp_flux<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, W.xc, W.xroe, W.fx, st, deep, gx);
  trace_end(s);
  trace_begin(s, ky);
  kp_flux<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, ys>>>(
      G, W.yc, W.yroe, W.fy, st, deep, gy);
  trace_end(s);
  // the join; if it cannot be recorded, wait for the side stream on the host instead
  if (fork && (cudaEventRecord(s->join_ev, ys) != cudaSuccess ||
               cudaStreamWaitEvent(cs, s->join_ev, 0) != cudaSuccess))
    cudaStreamSynchronize(ys);
  const size_t nc = size_t(nx) * ny;
  trace_begin(s, ku);
  kp_update<<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, stage, W.fx, W.fy, s->q, s->q0,
                                                       W.prim, out, st, deep);
  trace_end(s);
}

int fv2d_audit64(hteno_solver* s, const Geo& G, const double* q, const uint8_t* mx, const uint8_t* my,
                 long long* counts) {
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, 4 * sizeof(unsigned long long), s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "audit counters");
  cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), s->stream);
  const long nxf = long(G.nx + 1) * G.ny, nyf = long(G.ny + 1) * G.nx;
  kp_audit64<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, s->stream>>>(G, q, mx, d);
  kp_audit64<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, s->stream>>>(G, q, my, d);
  unsigned long long h[4] = {0, 0, 0, 0};
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(d, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_error(s, e, "FP64 routing audit");
  for (int k = 0; k < 4; ++k) counts[k] = (long long)h[k];
  return HTENO_OK;
}

int fv2d_harvest(hteno_solver* s, const Geo& G, const Work<double>& W, double p,
                 unsigned long long seed, uint16_t* X, uint8_t* Y, long cap,
                 unsigned long long* count) {
  const long nxf = long(G.nx + 1) * G.ny, nyf = long(G.ny + 1) * G.nx;
  kp_harvest<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, s->stream>>>(
      G, s->q, W.prim, p, seed, X, Y, cap, count);
  kp_harvest<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, s->stream>>>(
      G, s->q, W.prim, p, seed, X, Y, cap, count);
  return cuda_error(s, cudaGetLastError(), "harvest");
}

// ---- Residual without any device allocation --------------------------------------------------
// Some callers cannot allocate device memory: code running inside another framework's stream
// capture or memory pool, or a host that must keep its device footprint fixed after start-up.
// hteno_residual_noalloc serves them with the FP64 residual above, its work buffers taken from
// the fixed-size array below instead of cudaMalloc.  The array is part of the loaded module: every
// GPU that loads the library holds it until the process exits.  All calls share it, so two calls
// that overlap on the GPU race; it keeps the last call's contents, and nothing in it has to start
// at zero because each launch writes every element it later reads.
namespace {

constexpr int kNoAllocMaxCells = HTENO_NOALLOC_MAX_CELLS;
constexpr int kNoAllocMaxEdge = HTENO_NOALLOC_MAX_EDGE;  // bound on nx + ny
constexpr size_t kNoAllocBytes =
    4 * size_t(kNoAllocMaxCells) * sizeof(double) +
    19 * (2 * size_t(kNoAllocMaxCells) + size_t(kNoAllocMaxEdge)) * sizeof(double) + 256 * 8;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

void* g_noalloc_ptr[64] = {nullptr};
unsigned long long g_noalloc_const = 0;
std::mutex g_noalloc_mu;

}  // namespace

}  // namespace hteno

using namespace hteno;

extern "C" int hteno_residual_noalloc(const hteno_config* cfg, const double* q, double* rhs,
                                      void* stream) {
  if (!cfg || !q || !rhs) return HTENO_ERR_INVALID_ARG;
  const hteno_config& c = *cfg;
  if (c.dims != 2 || c.scheme != HTENO_SCHEME_FV || c.precision != HTENO_PREC_FP64)
    return HTENO_ERR_UNSUPPORTED;
  if (c.nx < 6 || c.ny < 6 || !(c.xr > c.xl) || !(c.yt > c.yb) || !(c.gamma > 1.0) ||
      c.recon < HTENO_RECON_TENO5 || c.recon > HTENO_RECON_TENO5A || c.flux < 0 || c.flux > 1 ||
      c.bc < HTENO_BC_ZEROGRAD || c.bc > HTENO_BC_DOUBLE_MACH)
    return HTENO_ERR_INVALID_ARG;
  // the Taylor and double-Mach boundaries need ghost face rows beyond the scratch layout
  if (c.bc >= HTENO_BC_TAYLOR) return HTENO_ERR_UNSUPPORTED;
  // size limit of the fixed scratch array
  if ((long long)c.nx * c.ny > kNoAllocMaxCells || c.nx + c.ny > kNoAllocMaxEdge)
    return HTENO_ERR_INVALID_ARG;
  if (work_bytes<double>(c.nx, c.ny) > kNoAllocBytes) return HTENO_ERR_INVALID_ARG;

  // one-time set-up per device, with that device current: the scratch address (a host-side
  // stand-in is not a device address) and this file's constant block
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return HTENO_ERR_CUDA;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return HTENO_ERR_CUDA;
      g_noalloc_ptr[dev] = ptr;
    }
    scratch = g_noalloc_ptr[dev];
  }
  if (upload_const(c_dev, &g_noalloc_const, &g_mu) != cudaSuccess) return HTENO_ERR_CUDA;

  Geo G{};  // every field set, as geo_of() sets them for a solver
  G.nx = c.nx;
  G.ny = c.ny;
  G.bc = c.bc;
  G.recon = c.recon;
  G.flux = c.flux;
  G.dx = (c.xr - c.xl) / c.nx;
  G.dy = (c.yt - c.yb) / c.ny;
  G.area = G.dx * G.dy;
  G.gamma = c.gamma;
  G.g1 = c.gamma - 1.0;
  G.x0 = c.xl;
  G.y0 = c.yb;
  G.t0 = c.t_init;
  fill_bc_consts(c.gamma, G.bq, &G.ctan, &G.c16, &G.s3);
  const Work<double> W = carve<double>(scratch, c.nx, c.ny);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const long nxf = long(c.nx + 1) * c.ny, nyf = long(c.ny + 1) * c.nx;
  const size_t nc = size_t(c.nx) * c.ny;
  kp_prim<<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, q, W.prim, nullptr, 0);
  kp_faces<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, q, W.prim, W.xc, W.xroe, nullptr);
  kp_faces<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, q, W.prim, W.yc, W.yroe, nullptr);
  kp_flux<1><<<unsigned((nxf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, W.xc, W.xroe, W.fx, nullptr);
  kp_flux<2><<<unsigned((nyf + kFaceThreads - 1) / kFaceThreads), kFaceThreads, 0, cs>>>(
      G, W.yc, W.yroe, W.fy, nullptr);
  kp_update<<<unsigned((nc + 255) / 256), 256, 0, cs>>>(G, 0, W.fx, W.fy, nullptr, nullptr,
                                                       W.prim, rhs, nullptr);
  return cudaGetLastError() == cudaSuccess ? HTENO_OK : HTENO_ERR_CUDA;
}
