/*
 * hteno.h -- C-ABI of the GB300 (sm_103a) implementation of the Hermite-TENO solver hot path:
 * the semi-discrete residual and the SSP-RK3 stage update of the reference's FV::System2D,
 * FV::System1D, FVHermite::System2D and FVHermite::System1D (indrow/Hermite-TENO).
 *
 * Conventions
 *   - Every entry point returns an hteno_status; nothing here calls exit() or throws.
 *   - Conserved state is SoA: q[var][j][i] (2D, var = rho, rho*u, rho*v, E) or q[var][i]
 *     (1D, var = rho, rho*u, E), interior cells only, row-major in i.  Ghost cells are implicit:
 *     zero-gradient boundaries read the nearest interior cell, periodic ones wrap.
 *   - "Batch" entry points take DEVICE pointers and an optional cudaStream_t (NULL = legacy
 *     default stream) and are asynchronous.  Solver set/get take HOST or DEVICE pointers
 *     (where = HTENO_HOST / HTENO_DEVICE) and synchronise their stream before returning.
 *   - A solver handle owns its device buffers; one handle per host thread.  Handles are
 *     independent and not internally locked.
 */
#ifndef HTENO_H
#define HTENO_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  HTENO_OK = 0,
  HTENO_ERR_INVALID_ARG = 1,
  HTENO_ERR_OOM = 2,
  HTENO_ERR_CUDA = 3,
  HTENO_ERR_NONPHYSICAL = 4, /* density or pressure <= 0 seen in the state */
  HTENO_ERR_NAN = 5,         /* a NaN appeared in the state */
  HTENO_ERR_TIMEOUT = 6,     /* a bounded device-side wait gave up */
  HTENO_ERR_UNSUPPORTED = 7
} hteno_status;

typedef enum { HTENO_HOST = 0, HTENO_DEVICE = 1 } hteno_where;

typedef enum { HTENO_SCHEME_FV = 0, HTENO_SCHEME_HERMITE = 1 } hteno_scheme;

/* Reconstruction.  FV: Schemes::Lagrange::teno5 / teno5i / linear, and the reference's other
 * selectable 5th-order schemes weno5JS, weno5Z, weno5N, teno5N, teno5a
 * (Schemes_Lagrange.cpp:358-594, 1265-1294).  Hermite 2D: hteno (the reference's choice).
 * Hermite 1D: LMPE routing (htenoi on troubled cells, linear elsewhere,
 * FVHermite_System1D.cpp:239-290). */
typedef enum {
  HTENO_RECON_TENO5 = 0,
  HTENO_RECON_TENO5I = 1,
  HTENO_RECON_LINEAR = 2,
  HTENO_RECON_WENO5JS = 3,
  HTENO_RECON_WENO5Z = 4,
  HTENO_RECON_WENO5N = 5,
  HTENO_RECON_TENO5N = 6,
  HTENO_RECON_TENO5A = 7
} hteno_recon;

typedef enum { HTENO_FLUX_RUSANOV = 0, HTENO_FLUX_HLLC = 1 } hteno_flux;
/* Boundaries: zeroGradBc and periodicBc (FV_System2D.cpp:114-152), and for the FV 2D scheme the
 * two routines the reference ships beside them in rhs() (:366-368):
 * HTENO_BC_TAYLOR = TaylorInstBc (:154-182): reflective side walls (x momentum mirrored), fixed
 *   bottom state (rho, u, v, p) = (2, 0, 0, 1) and top state (1, 0, 0, 2.5) -- the Rayleigh-Taylor
 *   setup on [0, 0.25] x [0, 1];
 * HTENO_BC_DOUBLE_MACH = doubleMachBc (:184-224): the double Mach reflection on [0, 4] x [0, 1]
 *   (post-shock inflow below x <= 1/6, reflective wall beyond it, time-dependent top boundary
 *   following the Mach-10 shock, zero-gradient sides).  Needs nx, ny >= 7. */
typedef enum {
  HTENO_BC_ZEROGRAD = 0,
  HTENO_BC_PERIODIC = 1,
  HTENO_BC_TAYLOR = 2,
  HTENO_BC_DOUBLE_MACH = 3
} hteno_bc;

/* HTENO_PREC_FP64: everything in double (the plain method).
 * HTENO_PREC_MIXED: reconstruction, smoothness indicators and fluxes in float; RK stage
 * accumulation of the conserved variables and the primitive (pressure) recovery in double. */
typedef enum { HTENO_PREC_FP64 = 0, HTENO_PREC_MIXED = 1 } hteno_precision;

/* Replaces the reference solver constructors, e.g. FV::System2D(xl, xr, nx, yb, yt, ny,
 * cflnumber, tmax, tInit, specificHeatRatio) (FV_System2D.h:12-15; FV_System1D.h:12-14;
 * FVHermite_System2D.h:16-19; FVHermite_System1D.h:12-14).  The scheme, flux, reconstruction
 * and boundary choices the reference makes by commenting code in or out are fields here. */
typedef struct {
  int dims;      /* 1 or 2 */
  int scheme;    /* hteno_scheme */
  int nx, ny;    /* interior cells (ny ignored for dims == 1) */
  double xl, xr, yb, yt;
  double cfl;
  double gamma;  /* specific heat ratio */
  double t_init; /* tInit */
  int recon;     /* hteno_recon */
  int flux;      /* hteno_flux */
  int bc;        /* hteno_bc */
  int precision; /* hteno_precision */
  int reserved[8];
} hteno_config;

typedef struct hteno_solver hteno_solver;

/* Fills *cfg with the FV::System2D defaults of the reference as shipped:
 * 2D, FV, TENO5, Rusanov, zero-gradient, FP64, gamma 1.4, CFL 0.4, [0,1]^2. */
void hteno_config_default(hteno_config* cfg);

/* Creates a solver (device buffers on the current device, its own stream).  Environment read at
 * creation: HTENO_UNIFORM_SKIP=0 computes uniform regions in full instead of taking their exactly
 * zero residual (the results are the same bits either way); HTENO_FV2D_TILE=<k> fixes the tile
 * candidate of the mixed FV 2D kernel instead of timing them (same bits for every candidate);
 * HTENO_SIDE_STREAM=0 runs the y-direction face and flux kernels of plain FV 2D and Hermite 2D
 * after the x-direction ones on the solver's stream instead of beside them on a second stream of
 * its own (the same bits). */
int hteno_create(const hteno_config* cfg, hteno_solver** out);
int hteno_destroy(hteno_solver* s);

/* Selects the CUDA stream the solver launches on (default: a stream the solver creates). */
int hteno_set_stream(hteno_solver* s, void* cuda_stream);

/* Initial data (replaces the reference's IC methods, e.g. FV_System2D.cpp:101-112).
 * q: conserved state [nvar][ny][nx].  Resets the time to t_init and the step count to 0. */
int hteno_set_state(hteno_solver* s, const double* q, int where);
int hteno_get_state(hteno_solver* s, double* q, int where);
/* Hermite schemes: first moments v (d/dx) and, in 2D, w (d/dy), same layout as q. */
int hteno_set_moments(hteno_solver* s, const double* v, const double* w, int where);
int hteno_get_moments(hteno_solver* s, double* v, double* w, int where);

/* Advances at most nsteps SSP-RK3 steps, stopping when t reaches t_final (the loop of
 * timeStepping(), FV_System2D.cpp:614-651, with dt = cfl*min(dx,dy)/max wave speed and the
 * last step clipped to t_final).  Issues the steps in chunks, checking the device time
 * between chunks, so a large nsteps (advance to t_final) launches no idle steps. */
int hteno_step(hteno_solver* s, int nsteps, double t_final);
/* Issues exactly nsteps steps without synchronising (steps after t_final are no-ops on the
 * device); for timing loops.  Call hteno_sync() before reading results. */
int hteno_step_async(hteno_solver* s, int nsteps, double t_final);
int hteno_sync(hteno_solver* s);
int hteno_get_time(hteno_solver* s, double* t, long* steps, double* last_dt);

/* Number of kernel launches hteno_step_async issues per step for this configuration. */
int hteno_launches_per_step(hteno_solver* s, int* launches);

/* Health flags of the state, sticky since the last hteno_set_state: bit 0 = a NaN appeared,
 * bit 1 = a non-positive density or pressure appeared.  The reference solver keeps stepping in
 * both cases (its positivity checks are commented out, e.g. FV_System2D.cpp:236-250), and so does
 * this library: by default hteno_step/hteno_sync return HTENO_OK and only record the flags.
 * With strict mode on they return HTENO_ERR_NAN / HTENO_ERR_NONPHYSICAL instead. */
int hteno_get_status(hteno_solver* s, int* flags);
int hteno_set_strict(hteno_solver* s, int on);

/* Plain FP64 FV 2D stepping as one fused launch per stage (on = 1) instead of five (uniform-region
 * test, faces x/y, fluxes x/y, update; on = 0, the default): tiles of 32 x 16 cells with their
 * face values and fluxes in shared memory, so a stage reads the state once (with a 3-cell halo)
 * and writes it once.  The same arithmetic in the same order: the same bits as the default path
 * (FV_System2D.cpp:363-612, a stage of timeStepping).  Zero-gradient and periodic boundaries;
 * other configurations return HTENO_ERR_UNSUPPORTED.  Holds 4 more state-sized buffers while on. */
int hteno_set_fp64_fused(hteno_solver* s, int on);

/* Work counters since the last hteno_set_state (FV 2D stepping), a measurement aid with no
 * reference counterpart (the reference computes every face):
 *   counters[0]: cell-stages whose residual was taken as exactly zero without computing their
 *                faces (uniform regions: the plain path's cells whose 7 x 7 neighbourhood holds
 *                one tame state, the mixed path's tiles of one tame float state; the same bits
 *                as computing them);
 *   counters[1]: mixed-path tiles whose state was staged by one TMA box copy (interior tiles of
 *                grids with an even nx; the others load cell by cell). */
int hteno_get_counters(hteno_solver* s, long long* counters);

/* Message of the last failed call on this handle ("" if none). */
const char* hteno_last_error(hteno_solver* s);
const char* hteno_status_string(int status);

/* ---- Pointwise batch kernels (device pointers), one reference function each ------------- */

/* Schemes::Lagrange::teno5 / teno5i / linear (Schemes_Lagrange.cpp:481-511, 1235-1263,
 * 1219-1233) and the alternatives of hteno_recon: u[n][6] -> out[n][2] =
 * (u^-_{i+1/2}, u^+_{i+1/2}).  kind: hteno_recon.
 * precision: HTENO_PREC_FP64 computes in double, HTENO_PREC_MIXED in float. */
int hteno_lagrange_batch(int kind, int precision, const double* u, double* out, long n,
                         void* stream);
/* Schemes::Lagrange::weno5JS3PointsQuadrature (Schemes_Lagrange.cpp:1171-1217):
 * u[n][5] -> out[n][3]. */
int hteno_gl3_batch(int precision, const double* u, double* out, long n, void* stream);
/* Schemes::Hermite::hteno / htenoi / linear (Schemes_Hermite.cpp:295-379, 670-758, 760-812)
 * after setGridSize(dx): u[n][4], d[n][4] -> out[n][4] = (u^-, u^+, d^-, d^+). kind 0/1/2. */
int hteno_hermite_batch(int kind, int precision, double dx, const double* u, const double* d,
                        double* out, long n, void* stream);
/* Schemes::Hermite::hermiteLimiter (Schemes_Hermite.cpp:634-662): u[n][3], d[n][3] -> out[n]. */
int hteno_hlimiter_batch(int precision, double dx, const double* u, const double* d, double* out,
                         long n, void* stream);
/* Equations::Euler2D::HLLC (Equations_Euler2D.cpp:372-428): ql[n][4], qr[n][4] -> out[n][4]. */
int hteno_hllc2d_batch(int precision, double gamma, int dir, const double* ql, const double* qr,
                       double* out, long n, void* stream);
/* Equations::Euler1D::HLLC (Equations_Euler1D.cpp:156-210): [n][3]. */
int hteno_hllc1d_batch(int precision, double gamma, const double* ql, const double* qr,
                       double* out, long n, void* stream);
/* Characteristic Rusanov as called in FV_System2D.cpp:460-464: the face eigenvectors are the
 * Roe average of the cell pair (qa, qb) (eigen2DEuler, FV_System2D.cpp:265-361);
 * Rusanov(ql, qr, ..., L, R, maxLocalWaveSpeed(w(ql), w(qr)), dir).  All [n][4]. */
int hteno_rusanov2d_batch(int precision, double gamma, int dir, const double* qa,
                          const double* qb, const double* ql, const double* qr, double* out,
                          long n, void* stream);
/* Derivative-moment Rusanov (Equations_Euler2D.cpp:352-360) as called in
 * FVHermite_System2D.cpp:553-589, eigenvectors from the cell pair (qa, qb).  All [n][4]. */
int hteno_drusanov2d_batch(int precision, double gamma, int dir, const double* qa,
                           const double* qb, const double* ql, const double* qr,
                           const double* dql, const double* dqr, double* out, long n,
                           void* stream);
/* Schemes::SSPRK::RungeKuttaIII (Schemes_SSPRK.cpp:3-15), elementwise over n doubles. */
int hteno_ssprk3_batch(const double* q0, const double* qn, const double* rhs, double dt,
                       int stage, double* out, long n, void* stream);
/* One residual evaluation of FV::System2D::rhs (FV_System2D.cpp:363-573) at state q[4][ny][nx]
 * (device) into rhs[4][ny][nx] (device), using the solver's configuration and buffers. */
int hteno_residual(hteno_solver* s, const double* q, double* rhs);

/* ---- Batches of independent 2D grids (mixed precision FV) --------------------------------- */

/* n independent FV::System2D instances (FV_System2D.h:12-20), each with its own config (dims 2,
 * scheme FV, precision HTENO_PREC_MIXED; grid sizes may differ and need not be square), advanced
 * together: each instance keeps its own time, dt and stop test exactly as its own
 * timeStepping() loop would (FV_System2D.cpp:614-651).  One persistent launch per RK stage
 * covers the tiles of every instance; a whole step is captured once in a CUDA graph and
 * replayed; the tile shape is picked by timing the candidates on the batch itself (first step,
 * or hteno_batch_tile).  No reference counterpart for the batching itself: the reference runs
 * one grid per process. */
typedef struct hteno_batch hteno_batch;
int hteno_batch_create(const hteno_config* cfgs, int n, hteno_batch** out);
int hteno_batch_destroy(hteno_batch* b);
int hteno_batch_size(hteno_batch* b, int* n);
int hteno_batch_set_stream(hteno_batch* b, void* cuda_stream);
/* State of instance i, SoA [4][ny_i][nx_i]; resets that instance's time to its t_init. */
int hteno_batch_set_state(hteno_batch* b, int i, const double* q, int where);
int hteno_batch_get_state(hteno_batch* b, int i, double* q, int where);
/* Up to nsteps steps of every instance; an instance stops once its time reaches t_final. */
int hteno_batch_step(hteno_batch* b, int nsteps, double t_final);
int hteno_batch_step_async(hteno_batch* b, int nsteps, double t_final);
int hteno_batch_sync(hteno_batch* b);
/* Time, completed steps and health flags of instance i as of the last hteno_batch_sync. */
int hteno_batch_get_time(hteno_batch* b, int i, double* t, long* steps, int* status);
/* Work counters of instance i as of the last hteno_batch_sync, as hteno_get_counters reports
 * them for a solver (uniform cell-stages, tiles staged by TMA), since its last set_state. */
int hteno_batch_get_counters(hteno_batch* b, int i, long long* counters);
/* Tile shape in use (tunes first if needed). */
int hteno_batch_tile(hteno_batch* b, int* tx, int* ty, int* threads);
const char* hteno_batch_last_error(hteno_batch* b);

/* ---- Learned stencil classifier (tensor cores) -------------------------------------------- */

/* A 6 -> 32 -> 32 -> 3 MLP (ReLU hidden layers, sigmoid outputs) predicting the three TENO5
 * cut-off bits (cutOff, Schemes_Lagrange.cpp:1141-1149) of the left-biased side of a normalised
 * 6-cell characteristic stencil (u - mean) / (max - min + 1e-30); the right side is the mirrored
 * stencil.  BF16 weights and activations, FP32 accumulation, tcgen05 tensor cores for inference
 * and training (forward, backward, weight gradients); Adam on FP32 master weights.  No
 * reference counterpart (the reference's precedent for a cell sensor is the LMPE flag of
 * FVHermite_System1D.cpp:239-290).
 * Parameter vector (hteno_mlp_num_params() floats): W1 [32][6], b1 [32], W2 [32][32], b2 [32],
 * W3 [3][32], b3 [3]; W[out][in].  Inputs: device BF16 rows [n][8] (6 features, 2 zeros);
 * labels: device bytes [n], bit k = cut-off bit k. */
typedef struct hteno_mlp hteno_mlp;
int hteno_mlp_create(unsigned long long seed, hteno_mlp** out);
int hteno_mlp_destroy(hteno_mlp* m);
int hteno_mlp_num_params(void);
int hteno_mlp_set_params(hteno_mlp* m, const float* params); /* host */
int hteno_mlp_get_params(hteno_mlp* m, float* params);       /* host */
/* KXRCF troubled-cell flags of an FV 1D solver's current state (FV::System1D::rhs,
 * FV_System1D.cpp:166-192): flags[nx] (device bytes) = 1 where |h1 - h2| / ((dx/2)^1.5 |rho|) > 1,
 * h1, h2 the two one-sided density values at the upwind face.  The reference computes the flag
 * and reconstructs with teno5i either way; here it is an output (the reference's precedent for a
 * troubled-cell sensor, beside LMPE and the learned router). */
int hteno_kxrcf(hteno_solver* s, unsigned char* flags);
/* Records training rows from the current state of a plain FP64 FV solver (2D or 1D): for
 * every face, characteristic field and side (the right side as the mirrored stencil), kept with
 * probability `keep` (deterministic in `seed`), the normalised 6-cell characteristic stencil the
 * reconstruction sees (x, BF16 [capacity][8], device) and the cut-off bits the plain solver
 * decides for it (y [capacity], device).  *count = rows offered (only the first `capacity` are
 * written). */
int hteno_harvest(hteno_solver* s, double keep, unsigned long long seed, unsigned short* x,
                  unsigned char* y, long capacity, long* count);
/* Gradient (host, parameter layout) and mean loss of the mean binary cross-entropy over n rows. */
int hteno_mlp_grad(hteno_mlp* m, const unsigned short* x, const unsigned char* y, long n,
                   float* grads, float* loss);
/* Mini-batch Adam, `epochs` passes over the rows in order; *loss = mean loss of the last pass. */
int hteno_mlp_train(hteno_mlp* m, const unsigned short* x, const unsigned char* y, long n,
                    int epochs, long batch, float lr, float* loss);
/* p [n][3] (device): probabilities of the three cut-off bits. */
int hteno_mlp_predict(hteno_mlp* m, const unsigned short* x, long n, float* p);
/* float rows [n][6] (device) -> BF16 rows [n][8] (device). */
int hteno_mlp_pack(hteno_mlp* m, const float* in, unsigned short* out, long n);
/* Polls of each tensor-core completion wait of the classifier's kernels before the call gives up
 * with HTENO_ERR_TIMEOUT (default 2^22, far beyond any completion).  The kernel that gives up
 * still waits, with the default bound, for its own products in flight and frees its tensor
 * memory, so the handle stays usable.  A test hook for the bounded-wait path; no reference
 * counterpart. */
int hteno_mlp_set_wait_limit(hteno_mlp* m, unsigned int polls);
const char* hteno_mlp_last_error(hteno_mlp* m);

/* Learned routing of a mixed-precision FV 2D solver: before every step the classifier marks,
 * from the step-start state, each (face, field, side) stencil whose three predicted cut-off
 * probabilities all exceed `threshold`; the three stages of that step reconstruct those with the
 * optimal linear weights (Schemes::Lagrange::linear, Schemes_Lagrange.cpp:1219-1233, the TENO5
 * result when all three candidates are kept) and skip the nonlinear weights; every other stencil
 * takes full TENO.  Every `audit_every` steps (0: never) the stages also evaluate the plain TENO
 * cut-off of every stencil and count the routing errors.  m = NULL switches routing off; the
 * classifier must outlive its use by the solver.  HTENO_ERR_UNSUPPORTED unless the solver is
 * mixed-precision FV 2D with teno5 or teno5i and has fewer than 2^29 faces. */
int hteno_set_router(hteno_solver* s, hteno_mlp* m, float threshold, int audit_every);
/* Classification schedule of a router (defaults 1 and 0: every step, masks used as classified).
 * The classifier runs on the step-start state every `classify_every` steps and its masks serve
 * the steps up to the next classification; a stencil's route bit is then kept only where the
 * same bit is set on every face within `margin` faces along and across the face direction
 * (faces within `margin` of the grid's edge keep none).  A discontinuity moves at most
 * cfl * classify_every cells between classifications, so margin >= ceil(cfl * classify_every)
 * keeps every routed stencil clear of any discontinuity the classifier saw.  The next step after
 * this call (or after hteno_set_state) classifies.  HTENO_ERR_UNSUPPORTED without a router.
 * No reference counterpart (the reference has no learned sensor). */
int hteno_set_router_schedule(hteno_solver* s, int classify_every, int margin);
/* stats[7]: audited stencils, routed, misrouted (routed though plain TENO cut a candidate),
 * all-smooth by plain TENO, flat (a window of equal float values: the stage kernel takes the
 * linear weights for it without the network or the indicators -- plain TENO keeps all three
 * candidates there), number of audited steps, and the number of stencils the last
 * classification handed to the network; sums since the last hteno_set_router or hteno_set_state.
 * Also reports a classifier timeout. */
int hteno_router_stats(hteno_solver* s, long long* stats);

/* The FP64 judge of the routing: classifies the solver's current state as a step does (with the
 * schedule's erosion), then, for every stencil the masks route, evaluates in double from the
 * double state (Roe average and projection in double) the TENO cut-off the plain FP64 solver
 * decides (cutOff, Schemes_Lagrange.cpp:1141-1149).  counts[0] = routed stencils, counts[1] =
 * those the FP64 cut-off would not reconstruct with all three candidates; counts[2], counts[3] =
 * the same over the routed stencils whose variation is resolved in float (max - min of the
 * window above 2^-16 of its largest magnitude): on the others the window's shape, and the cut-off
 * decided on it, is the rounding noise of the float fluxes.  Synchronous; the masks it leaves
 * are those of the current state.  No reference counterpart. */
int hteno_router_audit64(hteno_solver* s, long long* counts);

/* ---- Tracing: per-kernel CUDA-event timing of hteno_step ---------------------------------- */

/* When enabled, every kernel launch of hteno_step[_async] is bracketed by CUDA events on the
 * solver's stream; hteno_kernel_timing() then reports, per kernel kind, the launch count, the
 * summed device time and the algorithmic DRAM bytes and flops of one launch.  Enabling resets
 * the counters.  (No reference counterpart: the reference's only timer is a clock() around
 * timeStepping, FVHermite_System1D.cpp:388-404.) */
typedef struct {
  char name[32];
  long launches;
  double ms;             /* summed event time */
  double bytes_per_launch; /* algorithmic DRAM bytes of one launch */
  double flops_per_launch; /* algorithmic floating-point operations of one launch */
} hteno_kernel_time;

int hteno_enable_kernel_timing(hteno_solver* s, int on);
/* Fills up to max entries (one per kernel kind); *count receives the number of kinds. */
int hteno_kernel_timing(hteno_solver* s, hteno_kernel_time* out, int max, int* count);

/* Measured throughput of this device's FMA pipes, for roofline denominators:
 * kind 0 = FP64 FMA, 1 = FP32 FMA; result in TFLOP/s (2 flops per FMA). */
int hteno_measure_fma_peak(int kind, double* tflops);

/* ---- Residual without device allocation -------------------------------------------------- */

/* Same computation as hteno_residual (one evaluation of FV::System2D::rhs in FP64) without a
 * solver handle and without allocating device memory, for callers that cannot call cudaMalloc:
 * code inside another framework's stream capture or memory pool, or hosts whose device footprint
 * must stay fixed after start-up.  No reference counterpart: the reference has no device and no
 * allocation constraints.
 *   cfg: dims 2, scheme FV, precision FP64, any recon (0..7) and flux, bc zero-gradient or
 *   periodic (HTENO_BC_TAYLOR and HTENO_BC_DOUBLE_MACH need ghost face rows that the fixed array
 *   does not hold: HTENO_ERR_UNSUPPORTED); q, rhs: DEVICE pointers [4][ny][nx]; stream may be
 *   NULL.  Asynchronous.
 * Limits: nx * ny <= HTENO_NOALLOC_MAX_CELLS and nx + ny <= HTENO_NOALLOC_MAX_EDGE; larger grids
 * return HTENO_ERR_INVALID_ARG.  Its work buffers live in one fixed array (about 6 MB) inside
 * the library, held by every GPU that loads the library until the process exits.
 * The first call on each device looks up that array's address (cudaGetSymbolAddress) and
 * uploads constants; make that first call before any stream capture.  All calls share the array,
 * so calls that overlap on the GPU race with each other. */
#define HTENO_NOALLOC_MAX_CELLS 16384
#define HTENO_NOALLOC_MAX_EDGE 4096
int hteno_residual_noalloc(const hteno_config* cfg, const double* q, double* rhs, void* stream);

/* Version string of the library build. */
const char* hteno_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HTENO_H */
