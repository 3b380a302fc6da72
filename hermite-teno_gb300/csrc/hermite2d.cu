// FVHermite::System2D back end (placeholder until the Hermite kernels land).
#include "hteno_internal.h"
namespace hteno {
int hermite2d_setup(hteno_solver* s) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 2D not built"); }
int hermite2d_prepare(hteno_solver* s) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 2D not built"); }
int hermite2d_step_async(hteno_solver* s, int) { return set_error(s, HTENO_ERR_UNSUPPORTED, "Hermite 2D not built"); }
}
