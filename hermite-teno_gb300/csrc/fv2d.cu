// FV::System2D on the GPU (FV_System2D.cpp:363-651): characteristic TENO5 per direction,
// transverse three-point Gauss-Legendre WENO5-JS along each face, HLLC or characteristic
// Rusanov at the Gauss points, SSP-RK3.  Host dispatch of the two precisions:
//
//   plain FP64 (fv2d_fp64.cu): bit-reproducible; 5 launches per stage (faces x/y, flux x/y,
//     update) through per-face work arrays, or one fused launch per stage over 32 x 32 tiles
//     (hteno_set_fp64_fused, the same bits);
//   mixed (fv2d_fused.cu): reconstruction and fluxes in float, state and RK accumulation in
//     double; one fused launch per stage over tiles held in shared memory.
//
// One step = k_begin_step, 3 stages, k_end_step.  The host never synchronises inside
// hteno_step: dt, t and the stop flag live on the device.
#include "fv2d_common.cuh"

namespace hteno {
namespace {

#include "common_kernels.cuh"

}  // namespace

int fv2d_setup(hteno_solver* s) {
  if (fv2d_fp64_setup(s) != HTENO_OK) return HTENO_ERR_CUDA;
  const int nx = s->cfg.nx, ny = s->cfg.ny;
  if (s->cfg.precision == HTENO_PREC_MIXED) {
    const int rc = fv2d_fused_setup(s);
    if (rc != HTENO_OK) return rc;
    s->work_bytes = fv2d_fused_work_bytes(nx, ny);
    s->launches_per_step = 2 + 3;
  } else {
    s->work_bytes = work_bytes<double>(nx, ny);
    s->launches_per_step = 2 + 3 * (5 + (s->uniform_skip ? 1 : 0));  // + the uniform-region test
  }
  cudaError_t e = cudaMalloc(&s->work, s->work_bytes);
  if (e != cudaSuccess) return cuda_error(s, e, "work buffer");
  return HTENO_OK;
}

int fv2d_prepare(hteno_solver* s) {
  const Geo G = geo_of(s);
  if (s->cfg.precision == HTENO_PREC_MIXED)
    return fv2d_fused_prepare(s, G, static_cast<double*>(s->work));
  fv2d_fp64_prim(s, G, carve<double>(s->work, G.nx, G.ny), s->q, s->dstate, 1);
  return cuda_error(s, cudaGetLastError(), "primitives");
}

int fv2d_step_async(hteno_solver* s, int nsteps) {
  const Geo G = geo_of(s);
  for (int n = 0; n < nsteps; ++n) {
    k_begin_step<<<1, 1, 0, s->stream>>>(s->dstate);
    if (s->cfg.precision == HTENO_PREC_MIXED) {
      fv2d_fused_step(s, G, static_cast<double*>(s->work));
    } else {
      const Work<double> W = carve<double>(s->work, G.nx, G.ny);
      if (s->fused64) fv2d_fp64_fused_step(s, G, W);
      else for (int stage = 1; stage <= 3; ++stage) fv2d_fp64_stage(s, G, W, stage, s->q, nullptr);
    }
    k_end_step<<<1, 1, 0, s->stream>>>(s->dstate);
  }
  return cuda_error(s, cudaGetLastError(), "fv2d step launch");
}

int fv2d_residual(hteno_solver* s, const double* q, double* rhs) {
  const Geo G = geo_of(s);
  if (s->cfg.precision == HTENO_PREC_MIXED) {
    fv2d_fused_residual(s, G, q, rhs);
  } else {
    Work<double> W = carve<double>(s->work, G.nx, G.ny);
    fv2d_fp64_prim(s, G, W, q, nullptr, 0);
    fv2d_fp64_stage(s, G, W, 0, q, rhs);
  }
  return cuda_error(s, cudaGetLastError(), "fv2d residual launch");
}

int fv2d_harvest_entry(hteno_solver* s, double p, unsigned long long seed, uint16_t* X, uint8_t* Y,
                       long cap, unsigned long long* count) {
  const Geo G = geo_of(s);
  return fv2d_harvest(s, G, carve<double>(s->work, G.nx, G.ny), p, seed, X, Y, cap, count);
}

}  // namespace hteno
