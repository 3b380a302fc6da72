// Fused mixed-precision stage of FV::System2D (FV_System2D.cpp:363-612) for one tile of cells:
// residual of both directions and the SSP-RK3 stage combination in one pass, so a stage reads
// the conserved state once and writes it once.
//
//   A  load the tile plus a 3-cell halo of q (double) into shared memory as float, with the
//      primitives u, v, H, sqrt|rho| of every loaded cell (calcPrimitiveVariable, :226-263);
//      tiles whose halo lies inside the grid are staged by one TMA box copy of the four planes
//      (a tensor map over this GPU's own state buffer), the others cell by cell with the
//      boundary condition applied
//   B  x faces of rows -2 .. TY+1: Roe average, L projection of the 6-cell stencil, TENO5 (or
//      teno5i / linear) for 4 fields on both sides -> 8 characteristic values per face
//   C  x faces of rows 0 .. TY-1: GL3 across rows r-2 .. r+2 (each face in its own basis, as
//      the reference), R back-projection with the face's Roe state, HLLC or Rusanov at the 3
//      Gauss points, quadrature (:432-497)
//   D, E the same for the y faces
//   F  flux difference in double, SSP-RK3 in double (Schemes_SSPRK.cpp:3-15); on the last
//      stage the pressure (double, refined reciprocal), the health flags and the max wave
//      speed that sets the next dt (timeStepping, :622-633)
//
// Reconstruction, smoothness indicators and fluxes run in float; the state, the RK accumulation
// and the pressure check stay double.  Stage buffers: a stage reads its input state with halos
// from `qin` (never written during the stage), the step-start state pointwise from `qbase`
// and writes `qout`; stage 3 writes in place over the step-start state, which only the owning
// thread reads.  Included by the translation units that launch it (single-grid and batched).
#pragma once

#include <cuda.h>  // CUtensorMap

#include "fv2d_common.cuh"
#include "mixed_conv.cuh"
#include "tc_ptx.cuh"

namespace hteno {
namespace fused {

// Cell index with the boundary condition applied for any offset (tiles may run past the edge
// of small grids): zero-gradient clamps, periodic wraps.
__device__ __forceinline__ int cmap(int i, int n, int bc) {
  if (bc == HTENO_BC_PERIODIC) {
    i %= n;
    return i < 0 ? i + n : i;
  }
  return min(max(i, 0), n - 1);
}

using mix::d2f;
using mix::f2d;
using mix::rk_stage;

template <int TX, int TY>
struct Shape {
  static constexpr int W = TX + 6, H = TY + 6;   // loaded cells, halo 3
  static constexpr int XF = TX + 1, XR = TY + 4;  // x faces: columns 0..TX, rows -2..TY+1
  static constexpr int YF = TY + 1, YC = TX + 4;  // y faces: rows 0..TY, columns -2..TX+1
  static constexpr int XN = XF * XR, YN = YF * YC;
  static constexpr int FN = XN > YN ? XN : YN;
};

template <int TX, int TY>
struct Smem {
  float q[4][TY + 6][TX + 6];
  float p[4][TY + 6][TX + 6];  // u, v, H, sqrt|rho|
  // c, fx, fy are dead during phase A: the TMA box of the double state (stage_box) lands there
  alignas(128) float c[8][Shape<TX, TY>::FN];
  float fx[4][TY][TX + 1];
  float fy[4][TY + 1][TX];
  float wtab[2][8][3];  // TENO weights per cut-off pattern, minus and plus side
  alignas(8) uint64_t bar;  // completion of the TMA box
};

// The TMA box of a tile: columns i0 - 4 .. i0 + TX + 3 (an even start: the box's x offset times
// 8 bytes must be a multiple of 16), rows j0 - 3 .. j0 + TY + 2, the four conserved planes.
template <int TX, int TY>
struct Box {
  static constexpr int X = TX + 8, Y = TY + 6;
  static constexpr unsigned kBytes = unsigned(X) * Y * 4 * sizeof(double);
};
template <int TX, int TY>
__device__ __forceinline__ double (*stage_box(Smem<TX, TY>& S))[Box<TX, TY>::Y][Box<TX, TY>::X] {
  static_assert(Box<TX, TY>::kBytes <= sizeof(S.c) + sizeof(S.fx) + sizeof(S.fy), "TMA box fits");
  return reinterpret_cast<double (*)[Box<TX, TY>::Y][Box<TX, TY>::X]>(&S.c[0][0]);
}
constexpr uint32_t kTmaWaitLimit = 1u << 20;  // polls of the TMA box's mbarrier before giving up

// Tensor map of one [4][ny][nx] double state buffer with a box_x x box_y x 4 box (fv2d_fused.cu);
// false when the grid cannot be staged by TMA (odd nx) or encoding fails.
bool encode_box_map(CUtensorMap* m, const double* base, int nx, int ny, int box_x, int box_y);

template <int TX, int TY>
constexpr size_t smem_bytes() {
  return sizeof(Smem<TX, TY>);
}

// Cut-off pattern of one side of teno5 / teno5i (float).  With all three indicators exactly zero
// (constant data) the three ratios are equal and the pattern is 7 whatever tau is.
__device__ __forceinline__ int teno_pat_s(const float* v, bool improved) {
  float SI0, SI1, SI2;
  lagrange_si(v, SI0, SI1, SI2);
  if (SI0 == 0.f && SI1 == 0.f && SI2 == 0.f) return 7;
  float tau;
  if (!improved) tau = fabsf(lagrange_b35(v) - (SI0 + SI2 + 4.0f * SI1) * (1.0f / 6.0f));
  else tau = fmaxf(fmaxf(SI0, SI1), SI2);
  const float ez = HTENO_F32_EPSZ;
  const float r0 = fmaf(tau, Cst<float>::rcp(SI0 + ez), 1.0f);
  const float r1 = fmaf(tau, Cst<float>::rcp(SI1 + ez), 1.0f);
  const float r2 = fmaf(tau, Cst<float>::rcp(SI2 + ez), 1.0f);
  return teno_pattern(r0, r1, r2, float(HTENO_LAG_CT));
}

// A side's 5-cell window of equal float values, counted by the audit (the classifier hands such
// stencils to nobody).
__device__ __forceinline__ bool flat5(const float* v) {
  return v[1] == v[0] && v[2] == v[0] && v[3] == v[0] && v[4] == v[0];
}

__device__ __forceinline__ float weighted(float p0, float p1, float p2, const float* w) {
  return catchnan(dot3m(p0, w[0], p1, w[1], p2, w[2]));
}

// Audit counters of the learned router: stencils seen, routed to the linear weights, routed
// although the plain TENO cut-off would not have kept all three candidates, all-smooth by TENO,
// flat windows.
struct RouteCount {
  int seen = 0, routed = 0, misrouted = 0, smooth = 0, flat = 0;
};

// One side of teno5 (Schemes_Lagrange.cpp:481-511), teno5i (:1235-1263), linear (:1219-1233) or
// an alternative, u[0..5] -> u^-_{i+1/2} (side 0) or u^+_{i+1/2} (side 1).  With the route bit
// set (learned routing, TENO kinds) the side takes the linear weights without evaluating the
// indicators; when auditing, the plain cut-off is evaluated as well and counted.  The weight
// tables live in shared memory: a per-thread pattern would serialise constant-memory reads.
struct SideOut {
  float v;
  int pat;  // the TENO cut-off pattern evaluated (7 when not evaluated)
};
// Not inlined (8 calls per face in phases B and D); the stencil comes by value so it stays in
// registers.  The caller counts the audit.
static __device__ __noinline__ SideOut side_value(const DevConst& C, int kind,
                                                  const float (*tab)[8][3], float u0, float u1,
                                                  float u2, float u3, float u4, float u5, int side,
                                                  bool routed, bool audit) {
  float p0, p1, p2;
  if (side == 0) {
    p0 = dot3m(C.f_crj[0][1], u2, C.f_crj[1][1], u3, C.f_crj[2][1], u4);
    p1 = dot3m(C.f_crj[0][2], u1, C.f_crj[1][2], u2, C.f_crj[2][2], u3);
    p2 = dot3m(C.f_crj[0][3], u0, C.f_crj[1][3], u1, C.f_crj[2][3], u2);
  } else {
    p0 = dot3m(C.f_crj[0][0], u3, C.f_crj[1][0], u4, C.f_crj[2][0], u5);
    p1 = dot3m(C.f_crj[0][1], u2, C.f_crj[1][1], u3, C.f_crj[2][1], u4);
    p2 = dot3m(C.f_crj[0][2], u1, C.f_crj[1][2], u2, C.f_crj[2][2], u3);
  }
  const float v[5] = {side ? u1 : u0, side ? u2 : u1, side ? u3 : u2, side ? u4 : u3, side ? u5 : u4};
  if (kind == 2) return {dot3m(p0, tab[side][7][0], p1, tab[side][7][1], p2, tab[side][7][2]), 7};
  if (kind >= 3) return {alt_side(kind, p0, p1, p2, v, tab[side], tab[side][7]), 7};
  int pat = 7;
  if (!routed || audit) pat = teno_pat_s(v, kind == 1);
  return {weighted(p0, p1, p2, tab[side][routed ? 7 : pat]), pat};
}

// One side of teno5 / teno5i / linear / an alternative for the stencil u[0..5], with the audit
// of the learned router counted here (TENO kinds).
__device__ __forceinline__ float side_counted(const DevConst& C, int kind, const float (*tab)[8][3],
                                              const float* u, int side, bool routed, bool audit,
                                              RouteCount& rc) {
  const SideOut o = side_value(C, kind, tab, u[0], u[1], u[2], u[3], u[4], u[5], side, routed, audit);
  if (audit && kind <= 1) {
    rc.seen += 1;
    rc.smooth += o.pat == 7;
    rc.flat += flat5(u + side);
    rc.routed += routed;
    rc.misrouted += routed && o.pat != 7;
  }
  return o.v;
}

// GL3 of one face array, not inlined: phases C and E call it 8 times per face each, and inlined
// copies crowd the instruction cache.
struct Gl3f {
  float a, b, c;
};
static __device__ __noinline__ Gl3f gl3_f(const DevConst& C, const float* u) {
  Gl3f g;
  gl3(C, u, g.a, g.b, g.c);
  return g;
}

// The flux at one Gauss point of a face: R back-projection of both sides' characteristic values,
// then HLLC or Rusanov.  Not inlined (3 calls per face in each of phases C and E).
struct F4 {
  float v[4];
};
template <int DIR>
static __device__ __noinline__ F4 gauss_flux(Roe2<float> R, int flux, float g1, float gamma, float l0,
                                             float l1, float l2, float l3, float r0, float r1,
                                             float r2, float r3) {
  const float cl[4] = {l0, l1, l2, l3}, cr[4] = {r0, r1, r2, r3};
  float ql[4], qr[4];
  F4 F;
  roe_right(R, DIR, cl, ql);
  roe_right(R, DIR, cr, qr);
  if (flux == HTENO_FLUX_HLLC) hllc2(g1, DIR, ql, qr, F.v);
  else rusanov2(gamma, g1, DIR, R, ql, qr, F.v);
  return F;
}

// Pointers of one stage of one grid.
struct StageArgs {
  const double* qin;    // input state of the stage (halo reads)
  const double* qbase;  // step-start state (stages 2, 3), read pointwise
  double* qout;         // output state (stages 1-3) or residual (stage 0)
  StepState* st;        // dt, health flags, max wave speed; null for stage 0
  // learned routing (when mx is set): per x face [ny][nx+1] and y face [ny+1][nx] one byte, bit
  // 2r (2r+1) = left (right) side of characteristic field r takes the linear weights
  const uint8_t* mx = nullptr;
  const uint8_t* my = nullptr;
  unsigned long long* audit = nullptr;  // [5] RouteCount sums when auditing this stage
  bool skip_uniform = true;  // tiles of one tame float state get their (exactly zero) residual directly
  // tensor map of qin ([4][ny][nx] doubles, box Box<TX, TY>) for TMA staging of interior tiles;
  // null: every tile loads cell by cell
  const CUtensorMap* tmap = nullptr;
};

// A float state whose fluxes stay finite through the characteristic round trip: density and
// pressure in [2^-16, 2^16], Mach number at most 8 (the round trip's condition is ~ Mach^2, so
// the reconstructed state keeps a relative 2^-12 of float precision and stays positive, and no
// product of the face or flux arithmetic leaves the float range).
__device__ __forceinline__ bool tame_state(float r, float mx, float my, float e, float g1, float gamma) {
  const float ir = __frcp_rn(r);
  const float u = mx * ir, v = my * ir;
  const float p = (e - 0.5f * (mx * u + my * v)) * g1;
  constexpr float lo = 0x1p-16f, hi = 0x1p16f;
  return r >= lo && r <= hi && p >= lo && p <= hi && u * u + v * v <= 64.0f * (gamma * p * ir);
}

// The block's TMA mbarrier (S.bar), initialised once per launch before its first tile when a
// tensor map may be used; tma_phase then tracks the parity of the block's next box copy.
template <int TX, int TY>
__device__ __forceinline__ void tma_setup(Smem<TX, TY>& S) {
  if (threadIdx.x == 0) {
    tc::mbar_init(&S.bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
}

// The tile at (i0, j0) of grid G.  Every thread of the block must call it (barriers inside).
// Returns this thread's max wave speed over the cells it updated (stage 3) and ORs health flags
// into *bad (bit 2: the tile's TMA copy did not complete within the bounded wait; the tile is
// left unwritten and the caller must stop using the block's shared memory for box copies).
// tma_phase: parity of the block's next TMA box copy (tma_setup ran), flipped by each copy.
template <int TX, int TY, int NT>
__device__ __forceinline__ double tile_stage(const DevConst& C, const Geo& G, int i0, int j0,
                                             int stage, const StageArgs& a, Smem<TX, TY>& S,
                                             int& bad, uint32_t& tma_phase) {
  typedef Shape<TX, TY> Sh;
  RouteCount rc;
  // routing is a run-time switch (uniform per launch): the same machine code serves the plain and
  // the routed runs, so a router that routes nothing reproduces the plain run bit for bit
  const bool route_on = a.mx != nullptr;
  const bool audit = route_on && a.audit != nullptr;
  const size_t nc = size_t(G.nx) * G.ny;
  const float g1 = float(G.g1);
  const int tid = threadIdx.x;

  if (tid < 48) {
    const int side = tid / 24, pat = (tid % 24) / 3, k = tid % 3;
    S.wtab[side][pat][k] = side ? C.f_wtab_p[pat][k] : C.f_wtab_m[pat][k];
  }
  // A: state and primitives of the tile and its halo (ghosts as the boundary routine fills them)
  const bool ghosts = G.bc >= HTENO_BC_TAYLOR;
  const double tm = a.st ? a.st->t : G.t0;
  // interior tiles (box inside the grid, no ghost cell in the halo): one TMA copy of the box
  const bool use_tma = a.tmap != nullptr && !ghosts && i0 >= 4 && i0 + TX + 4 <= G.nx && j0 >= 3 &&
                       j0 + TY + 3 <= G.ny;
  if (use_tma) {
    auto box = stage_box(S);
    __syncthreads();  // every thread is done with the box region (a previous tile's fluxes)
    if (tid == 0) {
      tc::fence_proxy_async();  // earlier generic accesses to the box region come first
      tc::mbar_arrive_expect_tx(&S.bar, Box<TX, TY>::kBytes);
      tc::tma_load_3d(&box[0][0][0], a.tmap, i0 - 4, j0 - 3, 0, &S.bar);
    }
    // bounded wait; on giving up (never expected) the block flags the step, waits once more
    // for its copy in flight, and leaves this tile unwritten
    const bool late = __syncthreads_or(!tc::mbar_wait(&S.bar, tma_phase, kTmaWaitLimit));
    if (late) {
      tc::mbar_wait(&S.bar, tma_phase, kTmaWaitLimit);
      if (tid == 0 && a.st) atomicOr(&a.st->status, 4);
      __syncthreads();
      bad |= 4;
      return 0.0;
    }
    tma_phase ^= 1u;
    if (tid == 0 && a.st) atomicAdd(&a.st->tma_tiles, 1ull);
    for (int it = tid; it < Sh::W * Sh::H; it += NT) {
      const int y = it / Sh::W, x = it - y * Sh::W;
      const float r = d2f(box[0][y][x + 1]), mx = d2f(box[1][y][x + 1]);
      const float my = d2f(box[2][y][x + 1]), e = d2f(box[3][y][x + 1]);
      S.q[0][y][x] = r;
      S.q[1][y][x] = mx;
      S.q[2][y][x] = my;
      S.q[3][y][x] = e;
      const float ir = Cst<float>::rcp(r);
      const float u = mx * ir, v = my * ir;
      const float p = (e - 0.5f * fmaf(my, v, mx * u)) * g1;
      S.p[0][y][x] = u;
      S.p[1][y][x] = v;
      S.p[2][y][x] = (e + p) * ir;
      S.p[3][y][x] = Cst<float>::sqrt_(fabsf(r));
    }
  } else {
  for (int it = tid; it < Sh::W * Sh::H; it += NT) {
    const int y = it / Sh::W, x = it - y * Sh::W;
    float r, mx, my, e;
    if (ghosts) {
      double qq[4];
      bc_state(G, a.qin, i0 - 3 + x, j0 - 3 + y, tm, qq);
      r = d2f(qq[0]);
      mx = d2f(qq[1]);
      my = d2f(qq[2]);
      e = d2f(qq[3]);
    } else {
      const int gi = cmap(i0 - 3 + x, G.nx, G.bc), gj = cmap(j0 - 3 + y, G.ny, G.bc);
      const size_t k = size_t(gj) * G.nx + gi;
      r = d2f(__ldg(a.qin + k));
      mx = d2f(__ldg(a.qin + nc + k));
      my = d2f(__ldg(a.qin + 2 * nc + k));
      e = d2f(__ldg(a.qin + 3 * nc + k));
    }
    S.q[0][y][x] = r;
    S.q[1][y][x] = mx;
    S.q[2][y][x] = my;
    S.q[3][y][x] = e;
    const float ir = Cst<float>::rcp(r);
    const float u = mx * ir, v = my * ir;
    const float p = (e - 0.5f * fmaf(my, v, mx * u)) * g1;
    S.p[0][y][x] = u;
    S.p[1][y][x] = v;
    S.p[2][y][x] = (e + p) * ir;
    S.p[3][y][x] = Cst<float>::sqrt_(fabsf(r));
  }
  }
  __syncthreads();

  // Uniform tile: the tile and its 3-cell halo hold one tame float state, bit for bit.  Every flux
  // of every cell of the tile is then computed from identical inputs, each pair's difference is
  // +0, and so is the residual: phases B-E are skipped, the same bits result.  (Not while
  // auditing a router: the audit counts every stencil.)
  bool flat = false;
  if (a.skip_uniform && !audit) {
    const unsigned b0 = __float_as_uint(S.q[0][0][0]), b1 = __float_as_uint(S.q[1][0][0]);
    const unsigned b2 = __float_as_uint(S.q[2][0][0]), b3 = __float_as_uint(S.q[3][0][0]);
    bool same = true;
    for (int it = tid; it < Sh::W * Sh::H; it += NT) {
      const int y = it / Sh::W, x = it - y * Sh::W;
      same = same && __float_as_uint(S.q[0][y][x]) == b0 && __float_as_uint(S.q[1][y][x]) == b1 &&
             __float_as_uint(S.q[2][y][x]) == b2 && __float_as_uint(S.q[3][y][x]) == b3;
    }
    flat = __syncthreads_and(same) &&
           tame_state(S.q[0][0][0], S.q[1][0][0], S.q[2][0][0], S.q[3][0][0], g1, float(G.gamma));
    if (flat && stage > 0 && tid == 0)  // cells of the tile given their zero residual
      atomicAdd(&a.st->uniform, (unsigned long long)(min(TX, G.nx - i0) * min(TY, G.ny - j0)));
  }

  if (!flat) {
  // B: x faces, characteristic reconstruction
  for (int it = tid; it < Sh::XN; it += NT) {
    const int rr = it / Sh::XF, f = it - rr * Sh::XF;
    const int y = rr + 1;
    const int xa = f + 2, xb = f + 3;
    const Roe2<float> R = roe2<float>(g1, S.p[3][y][xa], S.p[0][y][xa], S.p[1][y][xa],
                                      S.p[2][y][xa], S.p[3][y][xb], S.p[0][y][xb],
                                      S.p[1][y][xb], S.p[2][y][xb]);
    float ch[4][6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const float qq[4] = {S.q[0][y][f + m], S.q[1][y][f + m], S.q[2][y][f + m], S.q[3][y][f + m]};
      float cc[4];
      roe_left(R, 1, qq, cc);
#pragma unroll
      for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
    }
    int route = 0;
    bool own = false;
    if (route_on) {
      const int gface = min(i0 + f, G.nx);
      route = a.mx[size_t(cmap(j0 - 2 + rr, G.ny, G.bc)) * (G.nx + 1) + gface];
      own = audit && rr >= 2 && rr < TY + 2 && j0 + rr - 2 < G.ny && i0 + f <= G.nx &&
            (f < TX || i0 + f == G.nx);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      S.c[r][it] = side_counted(C, G.recon, S.wtab, ch[r], 0, (route >> (2 * r)) & 1, own, rc);
      S.c[4 + r][it] = side_counted(C, G.recon, S.wtab, ch[r], 1, (route >> (2 * r + 1)) & 1, own, rc);
    }
  }
  __syncthreads();

  // C: x faces, transverse quadrature and flux
  for (int it = tid; it < Sh::XF * TY; it += NT) {
    const int r = it / Sh::XF, f = it - r * Sh::XF;
    float g[8][3];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float u5[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) u5[m] = S.c[k][(r + m) * Sh::XF + f];
      const Gl3f o = gl3_f(C, u5);
      g[k][0] = o.a;
      g[k][1] = o.b;
      g[k][2] = o.c;
    }
    const int y = r + 3, xa = f + 2, xb = f + 3;
    const Roe2<float> R = roe2<float>(g1, S.p[3][y][xa], S.p[0][y][xa], S.p[1][y][xa],
                                      S.p[2][y][xa], S.p[3][y][xb], S.p[0][y][xb],
                                      S.p[1][y][xb], S.p[2][y][xb]);
    float acc[4];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const F4 Fm = gauss_flux<1>(R, G.flux, g1, float(G.gamma), g[0][m], g[1][m], g[2][m], g[3][m],
                                   g[4][m], g[5][m], g[6][m], g[7][m]);
      const float wm = C.f_gl3w[m];
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[v] = m == 0 ? wm * Fm.v[v] : fmaf(wm, Fm.v[v], acc[v]);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) S.fx[v][r][f] = acc[v];
  }
  __syncthreads();

  // D: y faces, characteristic reconstruction
  for (int it = tid; it < Sh::YN; it += NT) {
    const int gg = it / Sh::YC, cc = it - gg * Sh::YC;
    const int x = cc + 1;
    const int ya = gg + 2, yb = gg + 3;
    const Roe2<float> R = roe2<float>(g1, S.p[3][ya][x], S.p[0][ya][x], S.p[1][ya][x],
                                      S.p[2][ya][x], S.p[3][yb][x], S.p[0][yb][x],
                                      S.p[1][yb][x], S.p[2][yb][x]);
    float ch[4][6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const float qq[4] = {S.q[0][gg + m][x], S.q[1][gg + m][x], S.q[2][gg + m][x],
                           S.q[3][gg + m][x]};
      float cv[4];
      roe_left(R, 2, qq, cv);
#pragma unroll
      for (int r = 0; r < 4; ++r) ch[r][m] = cv[r];
    }
    int route = 0;
    bool own = false;
    if (route_on) {
      const int gface = min(j0 + gg, G.ny);
      route = a.my[size_t(gface) * G.nx + cmap(i0 - 2 + cc, G.nx, G.bc)];
      own = audit && cc >= 2 && cc < TX + 2 && i0 + cc - 2 < G.nx && j0 + gg <= G.ny &&
            (gg < TY || j0 + gg == G.ny);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      S.c[r][it] = side_counted(C, G.recon, S.wtab, ch[r], 0, (route >> (2 * r)) & 1, own, rc);
      S.c[4 + r][it] = side_counted(C, G.recon, S.wtab, ch[r], 1, (route >> (2 * r + 1)) & 1, own, rc);
    }
  }
  __syncthreads();

  // E: y faces, transverse quadrature and flux
  for (int it = tid; it < Sh::YF * TX; it += NT) {
    const int gg = it / TX, col = it - gg * TX;
    float g[8][3];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float u5[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) u5[m] = S.c[k][gg * Sh::YC + col + m];
      const Gl3f o = gl3_f(C, u5);
      g[k][0] = o.a;
      g[k][1] = o.b;
      g[k][2] = o.c;
    }
    const int x = col + 3, ya = gg + 2, yb = gg + 3;
    const Roe2<float> R = roe2<float>(g1, S.p[3][ya][x], S.p[0][ya][x], S.p[1][ya][x],
                                      S.p[2][ya][x], S.p[3][yb][x], S.p[0][yb][x],
                                      S.p[1][yb][x], S.p[2][yb][x]);
    float acc[4];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const F4 Fm = gauss_flux<2>(R, G.flux, g1, float(G.gamma), g[0][m], g[1][m], g[2][m], g[3][m],
                                   g[4][m], g[5][m], g[6][m], g[7][m]);
      const float wm = C.f_gl3w[m];
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[v] = m == 0 ? wm * Fm.v[v] : fmaf(wm, Fm.v[v], acc[v]);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) S.fy[v][gg][col] = acc[v];
  }
  __syncthreads();
  }  // !flat

  // F: residual and SSP-RK3 stage in double
  float msf = 0.f;
  const double dt = stage ? a.st->dt : 0.0;
  const double rdx = 1.0 / G.dx, rdy = 1.0 / G.dy;  // (dfx dy + dfy dx) / (dx dy)
  for (int it = tid; it < TX * TY; it += NT) {
    const int y = it / TX, x = it - y * TX;
    const int gi = i0 + x, gj = j0 + y;
    if (gi >= G.nx || gj >= G.ny) continue;
    const size_t k = size_t(gj) * G.nx + gi;
    double qn[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      // float flux differences are exact in double, so the update stays conservative
      double rhs = 0.0;
      if (!flat) {
        const double dfx = f2d(S.fx[v][y][x]) - f2d(S.fx[v][y][x + 1]);
        const double dfy = f2d(S.fy[v][y][x]) - f2d(S.fy[v][y + 1][x]);
        rhs = fma(dfx, rdx, dfy * rdy);
      }
      if (stage == 0) {
        a.qout[v * nc + k] = rhs;
      } else {
        const double cur = a.qin[v * nc + k];
        const double base = stage == 1 ? cur : a.qbase[v * nc + k];
        qn[v] = rk_stage(base, cur, rhs, dt, stage);
        a.qout[v * nc + k] = qn[v];
      }
    }
    if (stage == 3) {
      // pressure in double with a refined float reciprocal of rho (relative error ~1e-14)
      double ir = f2d(__frcp_rn(d2f(qn[0])));
      ir = fma(ir, fma(-qn[0], ir, 1.0), ir);
      const double p = (qn[3] - 0.5 * (qn[1] * qn[1] + qn[2] * qn[2]) * ir) * G.g1;
      if (isnan(p)) bad |= 1;
      else if (qn[0] <= 0.0 || p <= 0.0) bad |= 2;
      const float fr = d2f(qn[0]), fu = d2f(qn[1] * ir), fv = d2f(qn[2] * ir);
      const float c = Cst<float>::sqrt_(fabsf(float(G.gamma) * d2f(p) * Cst<float>::rcp(fr)));
      const float m = fmaxf(fmaxf(fu - c, fabsf(fu + c)), fmaxf(fv - c, fabsf(fv + c)));
      msf = fmaxf(msf, m);
    }
  }
  if (audit) {
    int v[5] = {rc.seen, rc.routed, rc.misrouted, rc.smooth, rc.flat};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
      if ((threadIdx.x & 31) == 0 && v[k]) atomicAdd(a.audit + k, (unsigned long long)v[k]);
    }
  }
  return f2d(msf);
}

}  // namespace fused
}  // namespace hteno
