// FVHermite::System1D back end (placeholder until the Hermite kernels land).
#include "hteno_internal.h"
namespace hteno {
int hermite1d_setup(hteno_solver* s) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 1D not built"); }
int hermite1d_prepare(hteno_solver* s) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 1D not built"); }
int hermite1d_step_async(hteno_solver* s, int) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 1D not built"); }
}
