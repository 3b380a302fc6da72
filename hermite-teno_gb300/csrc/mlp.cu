// Learned stencil classifier: a 6 -> 32 -> 32 -> 3 MLP (ReLU, sigmoid outputs) that predicts the
// three TENO5 cut-off bits of a normalised 6-cell characteristic stencil (cutOff,
// Schemes_Lagrange.cpp:1141-1149, on the left-biased side; the right side is the mirrored
// stencil).  BF16 operands, FP32 accumulation, on the tcgen05 tensor cores:
//
//   forward   D1 = X W1^T, H1 = relu(D1 + b1); D2 = H1 W2^T, H2 = relu(D2 + b2);
//             D3 = H2 W3^T, p = sigmoid(D3 + b3)
//   backward  dZ3 = (p - y) / n;  dH2 = dZ3 W3;  dZ2 = dH2 * [H2 > 0];  dH1 = dZ2 W2;
//             dZ1 = dH1 * [H1 > 0];  dW3 += dZ3^T H2, dW2 += dZ2^T H1, dW1 += dZ1^T X
//
// One CTA of 128 threads owns a 128-row tile (thread = row = tensor-memory lane); weight
// gradients accumulate in tensor memory across the CTA's tiles and are added to the global
// gradient at the end.  Adam runs on FP32 master weights; the kernels read BF16 images of them.
// No reference counterpart: the reference has no learned component (its precedent is the LMPE
// troubled-cell sensor of FVHermite_System1D.cpp:239-290).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "fv2d_fused.cuh"
#include "hteno_internal.h"
#include "mlp_internal.cuh"

struct hteno_mlp;

namespace hteno {
namespace mlp {
namespace {

constexpr uint32_t kWaitLimit = 1u << 22;  // polls of an mbarrier before giving up

struct Smem {
  alignas(128) unsigned char at[128 * 128 * 2];  // A operand of the weight gradients (rows = outputs)
  alignas(128) unsigned char x[128 * 16 * 2];
  alignas(128) unsigned char xt[16 * 128 * 2];
  alignas(128) unsigned char h1[128 * 32 * 2];
  alignas(128) unsigned char h1t[32 * 128 * 2];
  alignas(128) unsigned char h2[128 * 32 * 2];
  alignas(128) unsigned char h2t[32 * 128 * 2];
  alignas(128) unsigned char dz3[128 * 16 * 2];
  alignas(128) unsigned char dz2[128 * 32 * 2];
  alignas(128) unsigned char w1[32 * 16 * 2];
  alignas(128) unsigned char w2[32 * 32 * 2];
  alignas(128) unsigned char w3[16 * 32 * 2];
  alignas(128) unsigned char w3t[32 * 16 * 2];
  alignas(128) unsigned char w2t[32 * 32 * 2];
  float b1[32], b2[32], b3[16];
  // bias gradients and loss, one slot per warp (summed in warp order at the end: deterministic)
  float gb1[4][32], gb2[4][32], gb3[4][16];
  float loss[4];
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  static constexpr bool kTrain = true;
  static constexpr uint32_t kTmemCols = 256;
};

// Shared memory of the inference kernels (the forward pass only).  A CTA runs kCT tiles of 128
// rows at once, so that each issue-wait-load round trip of a layer serves 512 rows; a tile's X,
// H1 and H2 share one buffer (each is dead once the product that reads it has completed), and its
// three accumulators share 32 tensor-memory columns.  The allocation is padded to 48 KB so that at
// most 4 CTAs share an SM, whose 4 x 128 tensor-memory columns are the SM's 512.
constexpr int kCT = 4;              // tiles per network round
constexpr int kCRound = kCT * 128;  // rows per network round
struct SmemC {
  alignas(128) unsigned char buf[kCT][128 * 32 * 2];
  alignas(128) unsigned char w1[32 * 16 * 2];
  alignas(128) unsigned char w2[32 * 32 * 2];
  alignas(128) unsigned char w3[16 * 32 * 2];
  float b1[32], b2[32], b3[16];
  alignas(8) uint64_t mbar;
  uint32_t tmem;
  static constexpr bool kTrain = false;
  static constexpr uint32_t kTmemCols = 128;
};
constexpr size_t kSmemCBytes = 48 * 1024;
static_assert(sizeof(SmemC) <= kSmemCBytes, "inference shared memory");

// tensor-memory columns
constexpr uint32_t C_D1 = 0, C_D2 = 32, C_D3 = 64, C_DH2 = 80, C_DH1 = 112;
constexpr uint32_t C_GW3 = 144, C_GW2 = 176, C_GW1 = 208;

__device__ __forceinline__ uint64_t desc_k(const unsigned char* base, int K, int kstep) {
  return tc::sdesc(tc::smem_u32(base) + uint32_t(kstep) * 256u, 128u, uint32_t(K / 8) * 128u);
}

// Copies the BF16 weight images into the operand layouts and the FP32 biases.
template <typename SM>
__device__ void load_weights(SM& S, const Weights& W) {
  const __nv_bfloat16* w1 = reinterpret_cast<const __nv_bfloat16*>(W.w1);
  for (int e = threadIdx.x; e < 32 * 16; e += blockDim.x) {
    const int r = e / 16, k = e % 16;
    *reinterpret_cast<__nv_bfloat16*>(S.w1 + tc::kmaj(r, k, 16)) = w1[e];
    if constexpr (SM::kTrain)
      *reinterpret_cast<__nv_bfloat16*>(S.w3t + tc::kmaj(r, k, 16)) =
          reinterpret_cast<const __nv_bfloat16*>(W.w3t)[e];
  }
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int r = e / 32, k = e % 32;
    *reinterpret_cast<__nv_bfloat16*>(S.w2 + tc::kmaj(r, k, 32)) =
        reinterpret_cast<const __nv_bfloat16*>(W.w2)[e];
    if constexpr (SM::kTrain)
      *reinterpret_cast<__nv_bfloat16*>(S.w2t + tc::kmaj(r, k, 32)) =
          reinterpret_cast<const __nv_bfloat16*>(W.w2t)[e];
  }
  for (int e = threadIdx.x; e < 16 * 32; e += blockDim.x) {
    const int r = e / 32, k = e % 32;
    *reinterpret_cast<__nv_bfloat16*>(S.w3 + tc::kmaj(r, k, 32)) =
        reinterpret_cast<const __nv_bfloat16*>(W.w3)[e];
  }
  for (int e = threadIdx.x; e < 32; e += blockDim.x) {
    S.b1[e] = W.b1[e];
    S.b2[e] = W.b2[e];
    if (e < 16) S.b3[e] = W.b3[e];
  }
}

// Issue (thread 0) after a barrier; every thread then waits for completion.  Returns false on
// timeout (uniform over the block).
template <typename SM>
__device__ __forceinline__ bool wait_mma(SM& S, uint32_t& phase, uint32_t limit) {
  const bool ok = !__syncthreads_or(!tc::mbar_wait(&S.mbar, phase, limit));
  if (ok) phase ^= 1u;  // on timeout `phase` stays the pending one
  tc::fence_after();
  return ok;
}

__device__ __forceinline__ void before_issue() {
  tc::fence_proxy_async();
  tc::fence_before();
  __syncthreads();
}

__device__ __forceinline__ float rbf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Forward pass of the tile whose inputs are in S.x / S.xt; leaves z1..z3 per thread.
// keep_t: also store H1^T / H2^T (needed by the weight gradients).
template <typename SM>
__device__ __forceinline__ bool forward(SM& S, uint32_t tbase, uint32_t& phase, float* h1,
                                        float* h2, float* z3, bool keep_t, uint32_t limit) {
  const int row = threadIdx.x;
  const uint32_t lane_addr = tbase + (uint32_t(threadIdx.x & ~31) << 16);
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    tc::mma_bf16(tbase + C_D1, desc_k(S.x, 16, 0), desc_k(S.w1, 16, 0), tc::idesc_bf16(128, 32), 0);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
  tc::tmem_ld16(lane_addr + C_D1, h1);
  tc::tmem_ld16(lane_addr + C_D1 + 16, h1 + 16);
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    h1[c] = fmaxf(h1[c] + S.b1[c], 0.0f);
    tc::st_bf16(S.h1, tc::kmaj(row, c, 32), h1[c]);
    if constexpr (SM::kTrain)
      if (keep_t) tc::st_bf16(S.h1t, tc::kmaj(c, row, 128), h1[c]);
  }
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    for (int s = 0; s < 2; ++s)
      tc::mma_bf16(tbase + C_D2, desc_k(S.h1, 32, s), desc_k(S.w2, 32, s), tc::idesc_bf16(128, 32), s);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
  tc::tmem_ld16(lane_addr + C_D2, h2);
  tc::tmem_ld16(lane_addr + C_D2 + 16, h2 + 16);
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    h2[c] = fmaxf(h2[c] + S.b2[c], 0.0f);
    tc::st_bf16(S.h2, tc::kmaj(row, c, 32), h2[c]);
    if constexpr (SM::kTrain)
      if (keep_t) tc::st_bf16(S.h2t, tc::kmaj(c, row, 128), h2[c]);
  }
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    for (int s = 0; s < 2; ++s)
      tc::mma_bf16(tbase + C_D3, desc_k(S.h2, 32, s), desc_k(S.w3, 32, s), tc::idesc_bf16(128, 16), s);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
  float d3[16];
  tc::tmem_ld16(lane_addr + C_D3, d3);
#pragma unroll
  for (int k = 0; k < 3; ++k) z3[k] = d3[k] + S.b3[k];
  return true;
}

// Two floats -> two BF16 (round to nearest even) with negative results clamped to +0: ReLU then
// rounding, in one instruction.  lo goes to the lower address.
__device__ __forceinline__ uint32_t pack_relu(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

// Bias, ReLU and BF16 rounding of this thread's 32-column accumulator row, stored as its row of
// the next layer's A operand (four 16-byte rows of K-major core matrices).
__device__ __forceinline__ void hidden_row(uint32_t taddr, const float* b, unsigned char* dst, int row) {
  float h[32];
  tc::tmem_ld16(taddr, h);
  tc::tmem_ld16(taddr + 16, h + 16);
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = 8 * g + 2 * j;
      w[j] = pack_relu(h[c] + b[c], h[c + 1] + b[c + 1]);
    }
    *reinterpret_cast<uint4*>(dst + tc::kmaj(row, 8 * g, 32)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Forward pass of up to kCT tiles at once (inference): thread r holds row r of tile t in in[t]
// (6 BF16 features in .x .y .z); n valid rows in all, tiles beyond them are not computed.  Leaves
// the three output logits of each of its rows in z.  Returns false on a timed-out wait (uniform).
__device__ __forceinline__ bool forward_rows(SmemC& S, uint32_t tbase, uint32_t& phase, const uint4* in,
                                             int n, float (*z)[3], uint32_t limit) {
  const int row = threadIdx.x;
  const int ntile = (n + 127) >> 7;
  const uint32_t lane_addr = tbase + (uint32_t(threadIdx.x & ~31) << 16);
#pragma unroll
  for (int t = 0; t < kCT; ++t)
    if (t < ntile) {
      *reinterpret_cast<uint4*>(S.buf[t] + tc::kmaj(row, 0, 16)) = make_uint4(in[t].x, in[t].y, in[t].z, 0u);
      *reinterpret_cast<uint4*>(S.buf[t] + tc::kmaj(row, 8, 16)) = make_uint4(0u, 0u, 0u, 0u);
    }
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    for (int t = 0; t < ntile; ++t)
      tc::mma_bf16(tbase + 32 * t, desc_k(S.buf[t], 16, 0), desc_k(S.w1, 16, 0), tc::idesc_bf16(128, 32), 0);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
#pragma unroll
  for (int t = 0; t < kCT; ++t)
    if (t < ntile) hidden_row(lane_addr + 32 * t, S.b1, S.buf[t], row);
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    for (int t = 0; t < ntile; ++t)
      for (int k = 0; k < 2; ++k)
        tc::mma_bf16(tbase + 32 * t, desc_k(S.buf[t], 32, k), desc_k(S.w2, 32, k), tc::idesc_bf16(128, 32), k);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
#pragma unroll
  for (int t = 0; t < kCT; ++t)
    if (t < ntile) hidden_row(lane_addr + 32 * t, S.b2, S.buf[t], row);
  before_issue();
  if (threadIdx.x == 0) {
    tc::fence_after();
    for (int t = 0; t < ntile; ++t)
      for (int k = 0; k < 2; ++k)
        tc::mma_bf16(tbase + 32 * t, desc_k(S.buf[t], 32, k), desc_k(S.w3, 32, k), tc::idesc_bf16(128, 16), k);
    tc::commit(&S.mbar);
  }
  if (!wait_mma(S, phase, limit)) return false;
#pragma unroll
  for (int t = 0; t < kCT; ++t)
    if (t < ntile) {
      float d3[16];
      tc::tmem_ld16(lane_addr + 32 * t, d3);
#pragma unroll
      for (int k = 0; k < 3; ++k) z[t][k] = d3[k] + S.b3[k];
    }
  return true;
}

// Writes one input row (6 features, bf16 bits) into S.x and S.xt.
template <typename SM>
__device__ __forceinline__ void put_input(SM& S, int row, const uint16_t* f) {
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const uint16_t bits = k < 6 ? f[k] : uint16_t(0);
    *reinterpret_cast<uint16_t*>(S.x + tc::kmaj(row, k, 16)) = bits;
    if constexpr (SM::kTrain) *reinterpret_cast<uint16_t*>(S.xt + tc::kmaj(k, row, 128)) = bits;
  }
}

template <typename SM>
__device__ void setup(SM& S, const Weights& W) {
  if constexpr (SM::kTrain) {
    for (int e = threadIdx.x; e < int(sizeof(S.at) / 16); e += blockDim.x)
      reinterpret_cast<uint4*>(S.at)[e] = make_uint4(0, 0, 0, 0);
  }
  load_weights(S, W);
  if constexpr (SM::kTrain) {
    for (int e = threadIdx.x; e < 4 * 32; e += blockDim.x) {
      S.gb1[e / 32][e % 32] = 0.f;
      S.gb2[e / 32][e % 32] = 0.f;
      if (e % 32 < 16) S.gb3[e / 32][e % 32] = 0.f;
    }
    if (threadIdx.x < 4) S.loss[threadIdx.x] = 0.f;
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&S.mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&S.tmem, SM::kTmemCols);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
}

template <typename SM>
__device__ void teardown(SM& S, uint32_t tbase) {
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (threadIdx.x < 32) tc::tmem_dealloc(tbase, SM::kTmemCols);
}

// Gradient of the mean BCE loss over `n_total` rows: each CTA writes its partial gradient (padded
// layout) to Gp[blockIdx.x] and its partial loss sum to Lp[blockIdx.x]; k_reduce_grad adds the
// partials in CTA order, so the gradient does not depend on the order in which CTAs finish.
// `limit`: polls of each tensor-core completion wait before the kernel gives up.
__global__ void __launch_bounds__(128) k_train(Weights W, const uint16_t* __restrict__ X,
                                               const uint8_t* __restrict__ Y, long n, long n_total,
                                               float* __restrict__ Gp, float* __restrict__ Lp,
                                               int* __restrict__ err, uint32_t limit) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>(smem_raw);
  setup(S, W);
  const uint32_t tbase = S.tmem;
  const uint32_t lane_addr = tbase + (uint32_t(threadIdx.x & ~31) << 16);
  const int row = threadIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float inv_n = 1.0f / float(n_total);
  uint32_t phase = 0;
  bool ok = true;
  int tiles_done = 0;
  const long ntiles = (n + 127) / 128;
  for (long t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++tiles_done) {
    const long r = t * 128 + row;
    const bool valid = r < n;
    uint16_t f[6] = {0, 0, 0, 0, 0, 0};
    uint8_t y = 0;
    if (valid) {
      const uint4 raw = *reinterpret_cast<const uint4*>(X + r * 8);
      const uint16_t* p = reinterpret_cast<const uint16_t*>(&raw);
#pragma unroll
      for (int k = 0; k < 6; ++k) f[k] = p[k];
      y = Y[r];
    }
    put_input(S, row, f);
    float h1[32], h2[32], z3[3];
    ok = forward(S, tbase, phase, h1, h2, z3, true, limit);
    if (!ok) break;
    // loss and dZ3
    float dz3[3], l = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float yk = float((y >> k) & 1);
      const float z = z3[k];
      const float pk = 1.0f / (1.0f + __expf(-z));
      l += fmaxf(z, 0.f) - z * yk + log1pf(__expf(-fabsf(z)));
      dz3[k] = valid ? (pk - yk) * inv_n : 0.f;
    }
    if (!valid) l = 0.f;
    l = warp_sum(l);
    if (lane == 0) S.loss[warp] += l;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float v = k < 3 ? dz3[k] : 0.f;
      tc::st_bf16(S.dz3, tc::kmaj(row, k, 16), v);
      tc::st_bf16(S.at, tc::kmaj(k, row, 128), v);
    }
    // bias gradients sum the same BF16-rounded error terms the matrix products use
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float s = warp_sum(rbf(dz3[k]));
      if (lane == 0) S.gb3[warp][k] += s;
    }
    before_issue();
    if (threadIdx.x == 0) {
      tc::fence_after();
      tc::mma_bf16(tbase + C_DH2, desc_k(S.dz3, 16, 0), desc_k(S.w3t, 16, 0), tc::idesc_bf16(128, 32), 0);
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tbase + C_GW3, desc_k(S.at, 128, s), desc_k(S.h2t, 128, s), tc::idesc_bf16(128, 32),
                     (tiles_done > 0 || s > 0) ? 1 : 0);
      tc::commit(&S.mbar);
    }
    if (!(ok = wait_mma(S, phase, limit))) break;
    // dZ2
    float d[32];
    tc::tmem_ld16(lane_addr + C_DH2, d);
    tc::tmem_ld16(lane_addr + C_DH2 + 16, d + 16);
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      const float v = h2[c] > 0.f ? d[c] : 0.f;
      tc::st_bf16(S.dz2, tc::kmaj(row, c, 32), v);
      tc::st_bf16(S.at, tc::kmaj(c, row, 128), v);
      const float s = warp_sum(rbf(v));
      if (lane == 0) S.gb2[warp][c] += s;
    }
    before_issue();
    if (threadIdx.x == 0) {
      tc::fence_after();
      for (int s = 0; s < 2; ++s)
        tc::mma_bf16(tbase + C_DH1, desc_k(S.dz2, 32, s), desc_k(S.w2t, 32, s), tc::idesc_bf16(128, 32), s);
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tbase + C_GW2, desc_k(S.at, 128, s), desc_k(S.h1t, 128, s), tc::idesc_bf16(128, 32),
                     (tiles_done > 0 || s > 0) ? 1 : 0);
      tc::commit(&S.mbar);
    }
    if (!(ok = wait_mma(S, phase, limit))) break;
    // dZ1
    tc::tmem_ld16(lane_addr + C_DH1, d);
    tc::tmem_ld16(lane_addr + C_DH1 + 16, d + 16);
#pragma unroll
    for (int c = 0; c < 32; ++c) {
      const float v = h1[c] > 0.f ? d[c] : 0.f;
      tc::st_bf16(S.at, tc::kmaj(c, row, 128), v);
      const float s = warp_sum(rbf(v));
      if (lane == 0) S.gb1[warp][c] += s;
    }
    before_issue();
    if (threadIdx.x == 0) {
      tc::fence_after();
      for (int s = 0; s < 8; ++s)
        tc::mma_bf16(tbase + C_GW1, desc_k(S.at, 128, s), desc_k(S.xt, 128, s), tc::idesc_bf16(128, 16),
                     (tiles_done > 0 || s > 0) ? 1 : 0);
      tc::commit(&S.mbar);
    }
    if (!(ok = wait_mma(S, phase, limit))) break;
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    // give in-flight MMAs a bounded chance to finish before the columns are released
    tc::mbar_wait(&S.mbar, phase, kWaitLimit);
  }
  // this CTA's partial gradient, every entry of the padded layout written once: rows of the
  // accumulators live in lanes 0..31 (warp 0).  The padded entries are exact zeros (zero input
  // columns 6..15, zero output rows 3..15); a CTA without a completed tile writes zeros.
  if (threadIdx.x < 32) {
    const bool have = ok && tiles_done > 0;
    float* g = Gp + size_t(blockIdx.x) * kParams;
    float v[16];
    for (int h = 0; h < 2; ++h) {
      if (have) tc::tmem_ld16(lane_addr + C_GW3 + 16 * h, v);
      if (row < 16)
        for (int c = 0; c < 16; ++c) g[kOffW3 + row * 32 + 16 * h + c] = have ? v[c] : 0.f;
      if (have) tc::tmem_ld16(lane_addr + C_GW2 + 16 * h, v);
      for (int c = 0; c < 16; ++c) g[kOffW2 + row * 32 + 16 * h + c] = have ? v[c] : 0.f;
    }
    if (have) tc::tmem_ld16(lane_addr + C_GW1, v);
    for (int c = 0; c < 16; ++c) g[kOffW1 + row * 16 + c] = have ? v[c] : 0.f;
    g[kOffB1 + row] = have ? ((S.gb1[0][row] + S.gb1[1][row]) + S.gb1[2][row]) + S.gb1[3][row] : 0.f;
    g[kOffB2 + row] = have ? ((S.gb2[0][row] + S.gb2[1][row]) + S.gb2[2][row]) + S.gb2[3][row] : 0.f;
    if (row < 16)
      g[kOffB3 + row] = have ? ((S.gb3[0][row] + S.gb3[1][row]) + S.gb3[2][row]) + S.gb3[3][row] : 0.f;
    if (row == 0) Lp[blockIdx.x] = have ? ((S.loss[0] + S.loss[1]) + S.loss[2]) + S.loss[3] : 0.f;
  }
  teardown(S, tbase);
}

// Probabilities of the three cut-off bits for n rows (rounds of kCRound rows per CTA).
__global__ void __launch_bounds__(128, 4) k_predict(Weights W, const uint16_t* __restrict__ X, long n,
                                                    float* __restrict__ P, int* __restrict__ err,
                                                    uint32_t limit) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemC& S = *reinterpret_cast<SmemC*>(smem_raw);
  setup(S, W);
  const uint32_t tbase = S.tmem;
  uint32_t phase = 0;
  bool ok = true;
  const long nround = (n + kCRound - 1) / kCRound;
  for (long rd = blockIdx.x; rd < nround && ok; rd += gridDim.x) {
    const long base = rd * kCRound;
    const int m = int(n - base < kCRound ? n - base : kCRound);
    uint4 in[kCT];
    float z[kCT][3];
#pragma unroll
    for (int t = 0; t < kCT; ++t) {
      const int k = t * 128 + int(threadIdx.x);
      in[t] = k < m ? *reinterpret_cast<const uint4*>(X + (base + k) * 8) : make_uint4(0u, 0u, 0u, 0u);
    }
    ok = forward_rows(S, tbase, phase, in, m, z, limit);
    if (ok)
#pragma unroll
      for (int t = 0; t < kCT; ++t) {
        const int k = t * 128 + int(threadIdx.x);
        if (k < m)
          for (int j = 0; j < 3; ++j) P[(base + k) * 3 + j] = 1.0f / (1.0f + __expf(-z[t][j]));
      }
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    tc::mbar_wait(&S.mbar, phase, kWaitLimit);
  }
  teardown(S, tbase);
}

// The non-flat stencils of one face of a mixed FV 2D grid, as network rows: the 8 stencils the
// fused stage kernel reconstructs (4 characteristic fields x 2 sides, float, from the double
// state as that kernel sees it), each normalised to [-1, 1] in BF16, with (face << 3 | bit) in
// .w (bit = 2 * field + side).  cq: the 6 cells' conserved values; cp: u, v, H and sqrt|rho| of
// the face's two cells.  Stencils whose six float values are equal are flat and left out: the
// stage kernel takes the linear weights for flat windows by itself.  Returns the bit mask of the
// rows written.
__device__ __forceinline__ uint32_t stencil_rows(float g1, int dir, const float (&cq)[6][4],
                                                 const float (&cp)[2][4], uint32_t face, uint4 (&row)[8]) {
  const Roe2<float> R = roe2<float>(g1, cp[0][3], cp[0][0], cp[0][1], cp[0][2], cp[1][3], cp[1][0],
                                    cp[1][1], cp[1][2]);
  float ch[4][6];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    float cc[4];
    roe_left(R, dir, cq[m], cc);
#pragma unroll
    for (int r = 0; r < 4; ++r) ch[r][m] = cc[r];
  }
  uint32_t keep = 0;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const int r = b >> 1, side = b & 1;
    float w[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) w[side ? 5 - m : m] = ch[r][m];
    float mean = 0.f, hi = w[0], lo = w[0];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      mean += w[m];
      hi = fmaxf(hi, w[m]);
      lo = fminf(lo, w[m]);
    }
    row[b] = make_uint4(0u, 0u, 0u, 0u);
    if (hi == lo) continue;
    mean *= (1.0f / 6.0f);
    const float inv = 1.0f / (hi - lo);
    uint32_t f[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const __nv_bfloat16 bv = __float2bfloat16_rn(fminf(1.f, fmaxf(-1.f, (w[m] - mean) * inv)));
      f[m] = *reinterpret_cast<const uint16_t*>(&bv);
    }
    row[b] = make_uint4(f[0] | (f[1] << 16), f[2] | (f[3] << 16), f[4] | (f[5] << 16), face << 3 | uint32_t(b));
    keep |= 1u << b;
  }
  return keep;
}

// Faces per block of the routing pass: A along the sweep direction x B lines across it.
template <int DIR>
struct RouteTile {
  static constexpr int A = DIR == 1 ? 64 : 8, B = DIR == 1 ? 4 : 32;
};

// Learned routing of a mixed FV 2D grid, pass 1 (masks zeroed beforehand), one launch per
// direction: a block stages the float conserved values of its (A + 5) x B cells in shared memory
// (each cell converted once), then one thread per face appends the face's non-flat stencils to
// the row list; appends are aggregated per block, one atomic per block.  A face whose six cells
// are equal has only flat stencils and is skipped before its primitives and eigenvectors.  Rows beyond `cap` are dropped (their stencils keep full TENO).
template <int DIR>
__global__ void __launch_bounds__(256, 6) k_route_prep(Geo G, const double* __restrict__ q, int tiles_a,
                                                    uint4* __restrict__ rows,
                                                    unsigned long long* __restrict__ nrows, long cap,
                                                    const StepState* __restrict__ sst) {
  if (sst && sst->done) return;  // a step after the stop time: no rows (uniform over the block)
  constexpr int A = RouteTile<DIR>::A, B = RouteTile<DIR>::B, L = A + 5, NC = L * B;
  static_assert(A * B == 256, "one face per thread");
  __shared__ float sq[4][NC];  // conserved values, float
  __shared__ int warp_tot[8];
  __shared__ unsigned long long block_base;
  const size_t nc = size_t(G.nx) * G.ny;
  const float g1 = float(G.g1);
  const int n_along = DIR == 1 ? G.nx : G.ny, n_across = DIR == 1 ? G.ny : G.nx;
  const int f0 = int(blockIdx.x % unsigned(tiles_a)) * A, l0 = int(blockIdx.x / unsigned(tiles_a)) * B;
  // staged cell e: along index f0 - 3 + a, line l0 + b; e = b * L + a (x) or a * B + b (y), so
  // that consecutive e are consecutive in memory.  All of a thread's loads are issued before
  // the first conversion.
  constexpr int NS = (NC + 255) / 256;
  double raw[NS][4];
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    const int e = int(threadIdx.x) + 256 * j;
    if (e < NC) {
      const int a = DIR == 1 ? e % L : e / B, b = DIR == 1 ? e / L : e % B;
      const int line = min(l0 + b, n_across - 1);  // lines past the grid: their faces are not listed
      const int ia = fused::cmap(f0 - 3 + a, n_along, G.bc);
      const size_t k = DIR == 1 ? size_t(line) * G.nx + ia : size_t(ia) * G.nx + line;
#pragma unroll
      for (int v = 0; v < 4; ++v) raw[j][v] = __ldg(q + v * nc + k);
    }
  }
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    const int e = int(threadIdx.x) + 256 * j;
    if (e < NC)
#pragma unroll
      for (int v = 0; v < 4; ++v) sq[v][e] = fused::d2f(raw[j][v]);
  }
  __syncthreads();
  const int fa = DIR == 1 ? int(threadIdx.x) % A : int(threadIdx.x) / B;
  const int fb = DIR == 1 ? int(threadIdx.x) / A : int(threadIdx.x) % B;
  const int fi = f0 + fa, line = l0 + fb;
  uint4 row[8];
  uint32_t keep = 0;
  if (fi <= n_along && line < n_across) {
    float cq[6][4];
    bool same = true;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int e = DIR == 1 ? fb * L + fa + m : (fa + m) * B + fb;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        cq[m][v] = sq[v][e];
        same = same && cq[m][v] == cq[0][v];
      }
    }
    if (!same) {
      float cp[2][4];  // primitives of the face's two cells
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float* c = cq[2 + h];
        // the fused stage kernel's phase-A arithmetic (this unit is also compiled without
        // implicit contraction), so the stencils are the bits that kernel reconstructs
        const float ir = Cst<float>::rcp(c[0]);
        const float u = c[1] * ir, v = c[2] * ir;
        const float p = (c[3] - 0.5f * fmaf(c[2], v, c[1] * u)) * g1;
        cp[h][0] = u;
        cp[h][1] = v;
        cp[h][2] = (c[3] + p) * ir;
        cp[h][3] = Cst<float>::sqrt_(fabsf(c[0]));
      }
      const long nxf = long(G.nx + 1) * G.ny;
      const long face = DIR == 1 ? long(line) * (G.nx + 1) + fi : nxf + long(fi) * G.nx + line;
      keep = stencil_rows(g1, DIR, cq, cp, uint32_t(face), row);
    }
  }
  const int nmine = __popc(keep);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = nmine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < 8; ++w) {
      const int t = warp_tot[w];
      warp_tot[w] = tot;
      tot += t;
    }
    block_base = tot ? atomicAdd(nrows, (unsigned long long)tot) : 0ull;
  }
  __syncthreads();
  const unsigned long long base = block_base + warp_tot[wid] + (incl - nmine);
#pragma unroll
  for (int b = 0; b < 8; ++b)
    if (keep >> b & 1u) {
      const unsigned long long slot = base + __popc(keep & ((1u << b) - 1u));
      if (slot < (unsigned long long)cap) rows[slot] = row[b];
    }
}

// Pass 2: the network over the appended rows, in rounds of kCRound rows per CTA; a row whose three
// logits all exceed zthr sets its bit in its face's mask byte.
__global__ void __launch_bounds__(128, 4) k_route_rows(Weights W, const uint4* __restrict__ rows,
                                                       const unsigned long long* __restrict__ nrows,
                                                       long cap, long nxf, uint8_t* __restrict__ mx,
                                                       uint8_t* __restrict__ my, float zthr,
                                                       int* __restrict__ err, uint32_t limit) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemC& S = *reinterpret_cast<SmemC*>(smem_raw);
  const long n = long(min(*nrows, (unsigned long long)cap));
  const long nround = (n + kCRound - 1) / kCRound;
  if (long(blockIdx.x) >= nround) return;  // uniform over the block; no tensor memory taken
  setup(S, W);
  const uint32_t tbase = S.tmem;
  uint32_t phase = 0;
  bool ok = true;
  // this thread's rows of round rd (zero beyond the list)
  auto fetch = [&](long rd, uint4* in) {
    const long base = rd * kCRound;
#pragma unroll
    for (int t = 0; t < kCT; ++t) {
      const long k = base + t * 128 + int(threadIdx.x);
      in[t] = rd < nround && k < n ? rows[k] : make_uint4(0u, 0u, 0u, 0u);
    }
  };
  uint4 in[kCT], next[kCT];
  fetch(blockIdx.x, in);
  for (long rd = blockIdx.x; rd < nround && ok; rd += gridDim.x) {
    const long base = rd * kCRound;
    const int m = int(n - base < kCRound ? n - base : kCRound);
    fetch(rd + gridDim.x, next);  // in flight during this round's products
    float z[kCT][3];
    ok = forward_rows(S, tbase, phase, in, m, z, limit);
    if (ok)
#pragma unroll
      for (int t = 0; t < kCT; ++t) {
        const int k = t * 128 + int(threadIdx.x);
        if (k < m && z[t][0] > zthr && z[t][1] > zthr && z[t][2] > zthr) {
          const long face = long(in[t].w >> 3);
          uint8_t* mk = face < nxf ? mx + face : my + (face - nxf);
          const size_t a = reinterpret_cast<size_t>(mk);
          atomicOr(reinterpret_cast<unsigned int*>(a & ~size_t(3)), (1u << (in[t].w & 7u)) << (8 * (a & 3)));
        }
      }
#pragma unroll
    for (int t = 0; t < kCT; ++t) in[t] = next[t];
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    tc::mbar_wait(&S.mbar, phase, kWaitLimit);
  }
  teardown(S, tbase);
}

// Adam on the FP32 master parameters (padded layout), then the BF16 images.
__global__ void k_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M,
                       float* __restrict__ V, float lr, float b1, float b2, float eps, int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float mh = m / (1.f - powf(b1, float(t))), vh = v / (1.f - powf(b2, float(t)));
  P[i] -= lr * mh / (sqrtf(vh) + eps);
}

// G = the sum of the nblk per-CTA partial gradients, added in CTA order; *loss += the sum of the
// partial losses in CTA order (one thread).  Deterministic for a given grid.
__global__ void k_reduce_grad(const float* __restrict__ Gp, const float* __restrict__ Lp, int nblk,
                              float* __restrict__ G, float* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) {
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += Gp[size_t(b) * kParams + i];
    G[i] = s;
  } else if (i == kParams) {
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += Lp[b];
    *loss += s;
  }
}

__global__ void k_images(const float* __restrict__ P, Weights W) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(W.w1);
  __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(W.w2);
  __nv_bfloat16* w3 = reinterpret_cast<__nv_bfloat16*>(W.w3);
  __nv_bfloat16* w3t = reinterpret_cast<__nv_bfloat16*>(W.w3t);
  __nv_bfloat16* w2t = reinterpret_cast<__nv_bfloat16*>(W.w2t);
  if (e < 32 * 16) {
    const int r = e / 16, k = e % 16;
    w1[e] = __float2bfloat16_rn(k < 6 ? P[kOffW1 + e] : 0.f);
    w3t[e] = __float2bfloat16_rn(k < 3 ? P[kOffW3 + k * 32 + r] : 0.f);  // W3^T[j][k]
  }
  if (e < 32 * 32) {
    const int r = e / 32, k = e % 32;
    w2[e] = __float2bfloat16_rn(P[kOffW2 + e]);
    w2t[e] = __float2bfloat16_rn(P[kOffW2 + k * 32 + r]);  // W2^T[i][j]
  }
  if (e < 16 * 32) {
    const int r = e / 32;
    w3[e] = __float2bfloat16_rn(r < 3 ? P[kOffW3 + e] : 0.f);
  }
  if (e < 32) {
    W.b1[e] = P[kOffB1 + e];
    W.b2[e] = P[kOffB2 + e];
    if (e < 16) W.b3[e] = e < 3 ? P[kOffB3 + e] : 0.f;
  }
}

// Converts float rows [n][6] to the bf16 training layout [n][8].
__global__ void k_pack_inputs(const float* __restrict__ in, uint16_t* __restrict__ out, long n) {
  const long r = blockIdx.x * long(blockDim.x) + threadIdx.x;
  if (r >= n) return;
  for (int k = 0; k < 8; ++k) {
    const __nv_bfloat16 b = __float2bfloat16_rn(k < 6 ? in[r * 6 + k] : 0.f);
    out[r * 8 + k] = *reinterpret_cast<const uint16_t*>(&b);
  }
}

}  // namespace

size_t smem_bytes() { return sizeof(Smem); }

}  // namespace mlp
}  // namespace hteno

using namespace hteno;
using namespace hteno::mlp;

struct hteno_mlp {
  Weights W{};          // device images
  float* P = nullptr;   // FP32 master parameters (padded)
  float* G = nullptr;   // gradient (padded), the ordered sum of the per-CTA partials
  float* Gp = nullptr;  // per-CTA partial gradients [2 * sms][kParams] and partial losses
  float* Lp = nullptr;
  float* M = nullptr;   // Adam moments
  float* V = nullptr;
  float* loss = nullptr;
  int* err = nullptr;
  void* img = nullptr;  // backing store of W
  int t = 0;            // Adam step
  uint32_t wait_limit = kWaitLimit;  // polls of a tensor-core completion wait
  int sms = 148;
  cudaStream_t stream = nullptr;
  std::string msg;
};

namespace {

int merr(hteno_mlp* m, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HTENO_OK;
  m->msg = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? HTENO_ERR_OOM : HTENO_ERR_CUDA;
}

int set_attr() {
  static int done = 0;
  if (done) return HTENO_OK;
  const int sm = int(mlp::smem_bytes());
  const int smc = int(mlp::kSmemCBytes);
  if (cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
      cudaFuncSetAttribute(k_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, smc) != cudaSuccess ||
      cudaFuncSetAttribute(k_route_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, smc) != cudaSuccess)
    return HTENO_ERR_CUDA;
  done = 1;
  return HTENO_OK;
}

int check_err(hteno_mlp* m) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return merr(m, e, "mlp");
  if (h) {
    m->msg = "tensor-core wait timed out";
    cudaMemsetAsync(m->err, 0, sizeof(int), m->stream);
    return HTENO_ERR_TIMEOUT;
  }
  return HTENO_OK;
}

// compact public layout <-> padded internal layout
void to_padded(const float* c, float* p) {
  std::memset(p, 0, kParams * sizeof(float));
  for (int j = 0; j < 32; ++j)
    for (int i = 0; i < 6; ++i) p[kOffW1 + j * 16 + i] = c[j * 6 + i];
  for (int j = 0; j < 32; ++j) p[kOffB1 + j] = c[192 + j];
  for (int e = 0; e < 1024; ++e) p[kOffW2 + e] = c[224 + e];
  for (int j = 0; j < 32; ++j) p[kOffB2 + j] = c[1248 + j];
  for (int e = 0; e < 96; ++e) p[kOffW3 + e] = c[1280 + e];
  for (int k = 0; k < 3; ++k) p[kOffB3 + k] = c[1376 + k];
}
void from_padded(const float* p, float* c) {
  for (int j = 0; j < 32; ++j)
    for (int i = 0; i < 6; ++i) c[j * 6 + i] = p[kOffW1 + j * 16 + i];
  for (int j = 0; j < 32; ++j) c[192 + j] = p[kOffB1 + j];
  for (int e = 0; e < 1024; ++e) c[224 + e] = p[kOffW2 + e];
  for (int j = 0; j < 32; ++j) c[1248 + j] = p[kOffB2 + j];
  for (int e = 0; e < 96; ++e) c[1280 + e] = p[kOffW3 + e];
  for (int k = 0; k < 3; ++k) c[1376 + k] = p[kOffB3 + k];
}

int refresh_images(hteno_mlp* m) {
  k_images<<<4, 256, 0, m->stream>>>(m->P, m->W);
  return merr(m, cudaGetLastError(), "weight images");
}

}  // namespace

namespace hteno {

// Route masks of a mixed FV 2D grid from its current state: the masks are zeroed, k_route_prep
// (x faces, then y faces) lists the non-flat stencils (at most `cap` rows, scratch owned by the caller), k_route_rows runs
// the network on them.  *nrows receives the number of non-flat stencils.
int mlp_classify(hteno_mlp* m, const Geo& G, const double* q, uint8_t* mx, uint8_t* my, float thr,
                 uint4* rows, unsigned long long* nrows, long cap, cudaStream_t st,
                 const StepState* sst) {
  const long nxf = long(G.nx + 1) * G.ny, nyf = long(G.ny + 1) * G.nx;
  cudaMemsetAsync(mx, 0, size_t(nxf), st);
  cudaMemsetAsync(my, 0, size_t(nyf), st);
  cudaMemsetAsync(nrows, 0, sizeof(unsigned long long), st);
  {
    using T1 = RouteTile<1>;
    using T2 = RouteTile<2>;
    const int ta1 = (G.nx + 1 + T1::A - 1) / T1::A, tb1 = (G.ny + T1::B - 1) / T1::B;
    const int ta2 = (G.ny + 1 + T2::A - 1) / T2::A, tb2 = (G.nx + T2::B - 1) / T2::B;
    k_route_prep<1><<<unsigned(ta1) * unsigned(tb1), 256, 0, st>>>(G, q, ta1, rows, nrows, cap, sst);
    k_route_prep<2><<<unsigned(ta2) * unsigned(tb2), 256, 0, st>>>(G, q, ta2, rows, nrows, cap, sst);
  }
  const float zthr = std::log(thr / (1.0f - thr));  // sigmoid(z) > thr  <=>  z > logit(thr)
  k_route_rows<<<4 * m->sms, 128, mlp::kSmemCBytes, st>>>(m->W, rows, nrows, cap, nxf, mx, my, zthr,
                                                          m->err, m->wait_limit);
  return cudaGetLastError() == cudaSuccess ? HTENO_OK : HTENO_ERR_CUDA;
}

int mlp_status(hteno_mlp* m, cudaStream_t st) {
  int h = 0;
  if (cudaMemcpyAsync(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return HTENO_ERR_CUDA;
  return h ? HTENO_ERR_TIMEOUT : HTENO_OK;
}

}  // namespace hteno

extern "C" {

int hteno_mlp_create(unsigned long long seed, hteno_mlp** out) {
  if (!out) return HTENO_ERR_INVALID_ARG;
  *out = nullptr;
  hteno_mlp* m = new (std::nothrow) hteno_mlp();
  if (!m) return HTENO_ERR_OOM;
  auto fail = [&](int code) {
    cudaFree(m->P); cudaFree(m->G); cudaFree(m->M); cudaFree(m->V); cudaFree(m->loss);
    cudaFree(m->err); cudaFree(m->img); cudaFree(m->Gp); cudaFree(m->Lp);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return code;
  };
  if (set_attr() != HTENO_OK) return fail(HTENO_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(HTENO_ERR_CUDA);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t pb = kParams * sizeof(float);
  if (cudaMalloc(&m->P, pb) || cudaMalloc(&m->G, pb) || cudaMalloc(&m->M, pb) || cudaMalloc(&m->V, pb) ||
      cudaMalloc(&m->loss, sizeof(float)) || cudaMalloc(&m->err, sizeof(int)) ||
      cudaMalloc(&m->img, kImageBytes) || cudaMalloc(&m->Gp, 2 * size_t(m->sms) * pb) ||
      cudaMalloc(&m->Lp, 2 * size_t(m->sms) * sizeof(float)))
    return fail(HTENO_ERR_OOM);
  char* b = static_cast<char*>(m->img);
  m->W.w1 = b; m->W.w2 = b + 1024; m->W.w3 = b + 3072; m->W.w3t = b + 4096; m->W.w2t = b + 5120;
  m->W.b1 = reinterpret_cast<float*>(b + 7168);
  m->W.b2 = m->W.b1 + 32;
  m->W.b3 = m->W.b2 + 32;
  // He-uniform initialisation of the weights, zero biases
  std::mt19937_64 rng(seed);
  std::vector<float> c(kPublicParams, 0.f), p(kParams);
  auto uni = [&](float a) { return float((double(rng() >> 11) * 0x1.0p-53 * 2.0 - 1.0) * a); };
  for (int e = 0; e < 192; ++e) c[e] = uni(std::sqrt(6.f / 6.f));
  for (int e = 0; e < 1024; ++e) c[224 + e] = uni(std::sqrt(6.f / 32.f));
  for (int e = 0; e < 96; ++e) c[1280 + e] = uni(std::sqrt(6.f / 32.f));
  to_padded(c.data(), p.data());
  if (cudaMemcpy(m->P, p.data(), pb, cudaMemcpyHostToDevice) || cudaMemset(m->G, 0, pb) ||
      cudaMemset(m->M, 0, pb) || cudaMemset(m->V, 0, pb) || cudaMemset(m->err, 0, sizeof(int)) ||
      cudaMemset(m->img, 0, kImageBytes))
    return fail(HTENO_ERR_CUDA);
  if (refresh_images(m) != HTENO_OK || cudaStreamSynchronize(m->stream) != cudaSuccess)
    return fail(HTENO_ERR_CUDA);
  *out = m;
  return HTENO_OK;
}

int hteno_mlp_destroy(hteno_mlp* m) {
  if (!m) return HTENO_ERR_INVALID_ARG;
  cudaStreamSynchronize(m->stream);
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->M); cudaFree(m->V); cudaFree(m->loss);
  cudaFree(m->err); cudaFree(m->img); cudaFree(m->Gp); cudaFree(m->Lp);
  cudaStreamDestroy(m->stream);
  delete m;
  return HTENO_OK;
}

int hteno_mlp_num_params(void) { return kPublicParams; }

int hteno_mlp_set_params(hteno_mlp* m, const float* params) {
  if (!m || !params) return HTENO_ERR_INVALID_ARG;
  std::vector<float> p(kParams);
  to_padded(params, p.data());
  cudaError_t e = cudaMemcpyAsync(m->P, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return merr(m, e, "set params");
  m->t = 0;
  cudaMemsetAsync(m->M, 0, kParams * sizeof(float), m->stream);
  cudaMemsetAsync(m->V, 0, kParams * sizeof(float), m->stream);
  const int rc = refresh_images(m);
  return rc ? rc : merr(m, cudaStreamSynchronize(m->stream), "set params");
}

int hteno_mlp_get_params(hteno_mlp* m, float* params) {
  if (!m || !params) return HTENO_ERR_INVALID_ARG;
  std::vector<float> p(kParams);
  cudaError_t e = cudaMemcpyAsync(p.data(), m->P, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return merr(m, e, "get params");
  from_padded(p.data(), params);
  return HTENO_OK;
}

// Gradient of the mean BCE loss over n rows (x: device bf16 [n][8], y: device u8 [n]); grads in
// the public layout (host), *loss = mean loss.
int hteno_mlp_grad(hteno_mlp* m, const uint16_t* x, const uint8_t* y, long n, float* grads, float* loss) {
  if (!m || !x || !y || n <= 0 || !grads) return HTENO_ERR_INVALID_ARG;
  cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
  const long tiles = (n + 127) / 128;
  const int grid = int(std::min<long>(tiles, 2L * m->sms));
  k_train<<<grid, 128, mlp::smem_bytes(), m->stream>>>(m->W, x, y, n, n, m->Gp, m->Lp, m->err,
                                                       m->wait_limit);
  k_reduce_grad<<<(kParams + 256) / 256, 256, 0, m->stream>>>(m->Gp, m->Lp, grid, m->G, m->loss);
  int rc = merr(m, cudaGetLastError(), "k_train");
  if (rc) return rc;
  rc = check_err(m);
  if (rc) return rc;
  std::vector<float> g(kParams);
  float l = 0.f;
  cudaError_t e = cudaMemcpyAsync(g.data(), m->G, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return merr(m, e, "grad copy");
  from_padded(g.data(), grads);
  if (loss) *loss = l / float(n);
  return HTENO_OK;
}

// Mini-batch Adam over the n rows for `epochs` passes (batches are contiguous slices; shuffle the
// data beforehand).  *loss receives the mean loss of the last epoch.
int hteno_mlp_train(hteno_mlp* m, const uint16_t* x, const uint8_t* y, long n, int epochs, long batch,
                    float lr, float* loss) {
  if (!m || !x || !y || n <= 0 || epochs < 0 || batch <= 0 || !(lr > 0.f)) return HTENO_ERR_INVALID_ARG;
  float last = 0.f;
  for (int ep = 0; ep < epochs; ++ep) {
    cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
    for (long off = 0; off < n; off += batch) {
      const long nb = std::min(batch, n - off);
      const long tiles = (nb + 127) / 128;
      const int grid = int(std::min<long>(tiles, 2L * m->sms));
      k_train<<<grid, 128, mlp::smem_bytes(), m->stream>>>(m->W, x + off * 8, y + off, nb, nb, m->Gp,
                                                           m->Lp, m->err, m->wait_limit);
      k_reduce_grad<<<(kParams + 256) / 256, 256, 0, m->stream>>>(m->Gp, m->Lp, grid, m->G, m->loss);
      ++m->t;
      k_adam<<<(kParams + 255) / 256, 256, 0, m->stream>>>(m->P, m->G, m->M, m->V, lr, 0.9f, 0.999f,
                                                           1e-8f, m->t);
      k_images<<<4, 256, 0, m->stream>>>(m->P, m->W);
    }
    int rc = merr(m, cudaGetLastError(), "train launch");
    if (rc) return rc;
    rc = check_err(m);
    if (rc) return rc;
    float l = 0.f;
    cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
    last = l / float(n);
  }
  if (loss) *loss = last;
  return HTENO_OK;
}

// Probabilities of the three cut-off bits: x device bf16 [n][8] -> p device float [n][3].
int hteno_mlp_predict(hteno_mlp* m, const uint16_t* x, long n, float* p) {
  if (!m || !x || n <= 0 || !p) return HTENO_ERR_INVALID_ARG;
  const long rounds = (n + mlp::kCRound - 1) / mlp::kCRound;
  const int grid = int(std::min<long>(rounds, 4L * m->sms));
  k_predict<<<grid, 128, mlp::kSmemCBytes, m->stream>>>(m->W, x, n, p, m->err, m->wait_limit);
  const int rc = merr(m, cudaGetLastError(), "k_predict");
  return rc ? rc : check_err(m);
}

// float [n][6] (device) -> bf16 training rows [n][8] (device).
int hteno_mlp_pack(hteno_mlp* m, const float* in, uint16_t* out, long n) {
  if (!m || !in || !out || n <= 0) return HTENO_ERR_INVALID_ARG;
  k_pack_inputs<<<unsigned((n + 255) / 256), 256, 0, m->stream>>>(in, out, n);
  const int rc = merr(m, cudaGetLastError(), "pack");
  return rc ? rc : merr(m, cudaStreamSynchronize(m->stream), "pack");
}

int hteno_mlp_set_wait_limit(hteno_mlp* m, unsigned int polls) {
  if (!m) return HTENO_ERR_INVALID_ARG;
  m->wait_limit = polls;
  return HTENO_OK;
}

const char* hteno_mlp_last_error(hteno_mlp* m) { return m ? m->msg.c_str() : "null handle"; }

}  // extern "C"
