// FVHermite::System2D, plain FP64 path: the double instantiation of the Hermite 2D kernels,
// compiled with --fmad=false so that every operation rounds as in the reference (the device
// functions are the bit-reproducible ones of parity_math.cuh).
#include "hermite2d_kernels.cuh"

namespace hteno {

int hermite2d_fp64_setup(hteno_solver* s) {
  if (upload_const(c_dev, &g_mask, &g_mu) != cudaSuccess)
    return set_error(s, HTENO_ERR_CUDA, "constant upload failed");
  return HTENO_OK;
}

void hermite2d_fp64_step(hteno_solver* s, const GeoH& G) { launch_step<double>(s, G); }

void hermite2d_fp64_prim(hteno_solver* s, const GeoH& G) {
  const size_t nc = size_t(G.nx) * G.ny;
  kh_prim<<<unsigned((nc + 255) / 256), 256, 0, s->stream>>>(G, s->q, carve_h<double>(s->work, G.nx, G.ny).prim,
                                                            s->dstate, 1);
}

}  // namespace hteno
