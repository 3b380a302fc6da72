// FVHermite::System2D on the GPU (FVHermite_System2D.cpp:393-819): cell averages u and first
// moments v = du/dx, w = du/dy.  Per stage:
//   limit             : hermiteLimiter on v along x and on w along y.  The reference updates in
//                       place while sweeping (limitDerivatives, :393-427), i.e. a Gauss-Seidel
//                       sweep: one thread per (row, field) resp. (column, field) walks the line.
//   prim              : primitives of u
//   faces<X>, <Y>     : Roe average; HTENO on (L u, L v_n) over 4 cells, TENO5 on L v_t over 6
//   flux<X>, <Y>      : GL3 along the face for the 24 face arrays, R back-projection, Rusanov for u
//                       and dRusanov for the two moments at 3 Gauss points
//   update            : flux differences and SSP-RK3 for u, v, w.  RungeKutta3 saves v0, w0
//                       after the first rhs (the limited moments) and combines later stages with
//                       the unlimited stage values, so those are kept in vs, ws.
// Boundaries are zero-gradient (the reference's Hermite 2D rhs).  T = double or float.
#include "hermite2d_kernels.cuh"

namespace hteno {

int hermite2d_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess || hermite2d_fp64_setup(s) != HTENO_OK)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  if (s->cfg.bc != HTENO_BC_ZEROGRAD)
    return set_error(s, HTENO_ERR_UNSUPPORTED, "the Hermite 2D scheme uses zero-gradient boundaries");
  if (make_side_stream(s) != HTENO_OK) return HTENO_ERR_CUDA;
  const int nx = s->cfg.nx, ny = s->cfg.ny;
  s->work_bytes = s->cfg.precision == HTENO_PREC_MIXED ? work_bytes_h<float>(nx, ny)
                                                       : work_bytes_h<double>(nx, ny);
  cudaError_t e = cudaMalloc(&s->work, s->work_bytes);
  if (e != cudaSuccess) return cuda_error(s, e, "work buffer");
  e = cudaMemset(s->v, 0, s->ncell * 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(s->w, 0, s->ncell * 4 * sizeof(double));
  if (e != cudaSuccess) return cuda_error(s, e, "moment buffers");
  s->launches_per_step = 2 + 3 * 6;  // limiter, faces x/y, fluxes x/y, update
  return HTENO_OK;
}

int hermite2d_prepare(hteno_solver* s) {
  const GeoH G = geo_of(s);
  const size_t nc = size_t(G.nx) * G.ny;
  if (s->cfg.precision == HTENO_PREC_MIXED) {
    const WorkH<float> W = carve_h<float>(s->work, G.nx, G.ny);
    kh_prim_f<<<unsigned((nc + 255) / 256), 256, 0, s->stream>>>(G, s->q, W.qt, W.primt, s->dstate);
  } else
    hermite2d_fp64_prim(s, G);
  return cuda_error(s, cudaGetLastError(), "kh_prim");
}

int hermite2d_step_async(hteno_solver* s, int nsteps) {
  const GeoH G = geo_of(s);
  for (int n = 0; n < nsteps; ++n) {
    if (s->cfg.precision == HTENO_PREC_MIXED) launch_step<float>(s, G);
    else hermite2d_fp64_step(s, G);
  }
  return cuda_error(s, cudaGetLastError(), "hermite2d step launch");
}

}  // namespace hteno
