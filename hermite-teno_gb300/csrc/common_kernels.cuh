// Kernels and device helpers shared by the solver back ends.  Included by each back end's
// translation unit inside its anonymous namespace (each gets a private copy).
#pragma once

// Boundary index map: zero-gradient reads the nearest interior cell (zeroGradBc,
// FV_System2D.cpp:134-152), periodic wraps (periodicBc, :76-99).  |offset| <= n.
__device__ __forceinline__ int bmap(int i, int n, int bc) {
  if (bc == HTENO_BC_PERIODIC) {
    i = i < 0 ? i + n : i;
    return i >= n ? i - n : i;
  }
  return min(max(i, 0), n - 1);
}

// Block-wide max of a non-negative double folded into *bits (NaN is skipped, as fmax skips it
// in the reference's reduction).  Every thread of the block must call it.
__device__ __forceinline__ void block_max_to(double v, unsigned long long* bits) {
  __shared__ double red[32];
  if (isnan(v)) v = 0.0;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0 && v > 0.0)
      atomicMax(bits, static_cast<unsigned long long>(__double_as_longlong(v)));
  }
}

// Start of one step of timeStepping() (FV_System2D.cpp:622-645): stop when t >= t_final,
// otherwise dt = dt_scale / max wave speed, clipped to t_final.
__global__ void k_begin_step(StepState* st) {
  if (st->done) return;
  if (!(st->t < st->t_final)) {
    st->done = 1;
    return;
  }
  const double M = __longlong_as_double(static_cast<long long>(st->maxbits));
  double dt = st->dt_scale / M;
  dt = st->t + dt > st->t_final ? st->t_final - st->t : dt;
  st->dt = dt;
  st->maxbits = 0ull;
}

__global__ void k_end_step(StepState* st) {
  if (st->done) return;
  st->t += st->dt;
  st->steps += 1;
}
