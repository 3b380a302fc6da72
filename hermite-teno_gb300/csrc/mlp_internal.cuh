// Parameter layout of the stencil classifier (6 -> 32 -> 32 -> 3), shared by the training
// kernels (mlp.cu) and the solver's router.
#pragma once

#include <stdint.h>

#include "tc_ptx.cuh"

namespace hteno {
namespace mlp {

// FP32 master parameters, padded so that every operand has a tensor-core friendly shape:
// W1 [32][16] (inputs 6..15 zero), b1 [32], W2 [32][32], b2 [32], W3 [16][32] (rows 3..15 zero),
// b3 [16].  The public layout drops the padding: W1 [32][6], b1, W2, b2, W3 [3][32], b3 [3].
constexpr int kOffW1 = 0, kOffB1 = 512, kOffW2 = 544, kOffB2 = 1568, kOffW3 = 1600, kOffB3 = 2112;
constexpr int kParams = 2128;
constexpr int kPublicParams = 192 + 32 + 1024 + 32 + 96 + 3;
constexpr size_t kImageBytes = 7680;

// Device images read by the kernels: BF16 weights in row-major [rows][K] (w1 [32][16],
// w2 [32][32], w3 [16][32], w3t = W3^T [32][16], w2t = W2^T [32][32]) and FP32 biases.
struct Weights {
  void* w1;
  void* w2;
  void* w3;
  void* w3t;
  void* w2t;
  float* b1;
  float* b2;
  float* b3;
};

size_t smem_bytes();

}  // namespace mlp
}  // namespace hteno
