/*
 * tlq.h -- C ABI of the GB300 hydrodynamic step (libtlq.so).
 *
 * Drop-in for the hot path of tlaloque, the loop body of
 * source/mainHD.f90:74-99 and the external subroutines it calls.  All entry
 * points are extern "C", take plain pointers and sizes, return an int status
 * (TLQ_OK = 0) and never abort or exit.  Host arrays are borrowed for the
 * duration of one call and use the reference's layout
 *     A(1:5, -1:nx+2, -1:ny+2, -1:nz+2)   (real(8), variable fastest,
 *                                          column-major; nghost = 2)
 * The device state is owned by the context.  A context is not thread-safe;
 * it owns (or borrows) one CUDA stream and every call is ordered on it.
 */
#ifndef TLQ_H
#define TLQ_H

#ifdef __cplusplus
extern "C" {
#endif

#define TLQ_ABI_VERSION 1

/* Status codes.  The reference has no error convention beyond `stop`. */
enum {
  TLQ_OK = 0,
  TLQ_ERR_CUDA = 1,          /* a CUDA runtime/driver call failed (see tlq_last_error) */
  TLQ_ERR_CONFIG = 2,        /* invalid or unsupported configuration */
  TLQ_ERR_NONFINITE_DT = 3,  /* the CFL reduction saw a NaN/Inf signal speed */
  TLQ_ERR_NEG_DENSITY = 4,   /* an interior cell has rho <= 0 after the step */
  TLQ_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
  TLQ_ERR_ARG = 6,           /* NULL or out-of-range argument */
  TLQ_ERR_STATE = 7,         /* call out of order (e.g. tlq_step before tlq_upload) */
  TLQ_ERR_NOMEM = 8          /* device or pinned-host allocation failed */
};

/* Boundary kinds: source/constants.f90:20-23 (same values). */
enum { TLQ_BC_OUTFLOW = 1, TLQ_BC_REFLECTIVE = 2, TLQ_BC_PERIODIC = 3, TLQ_BC_INFLOW = 4 };
/* Slope limiters: source/constants.f90:26-31 (same values). */
enum {
  TLQ_LIMITER_NONE = 1, TLQ_LIMITER_VANLEER = 2, TLQ_LIMITER_MINMOD = 3,
  TLQ_LIMITER_UMIST = 4, TLQ_LIMITER_WOODWARD = 5, TLQ_LIMITER_SUPERBEE = 6
};
/* Riemann solver: source/HLLC.f90 (linked by the reference Makefile) or source/HLL.f90. */
enum { TLQ_SOLVER_HLLC = 0, TLQ_SOLVER_HLL = 1 };
/* Radiative cooling: off; the reference's single exponential step
 * (source/cooling.f90:47-119); its sub-cycled extension (nsub = 1 is the
 * reference formula exactly); the learned surrogate (mixed form only, the
 * exact integrator as its fallback); the exact integrator: the sub-cycled
 * one in the limit of infinitely many sub-steps, in closed form (find_coef's
 * log-linear interpolation makes Lambda(T) a piecewise power law, whose
 * cooling integrates exactly: Townsend 2009), with the reference formula
 * for a cell whose cooling number Lambda n^2 dt / E_th is at most
 * cool_sub_frac. */
enum { TLQ_COOL_NONE = 0, TLQ_COOL_REF = 1, TLQ_COOL_SUBCYCLE = 2, TLQ_COOL_MLP = 3, TLQ_COOL_EXACT = 4 };
/* Arithmetic of the fused step: plain FP64 (matches the reference), or
 * mixed (FP32 reconstruction and Riemann fluxes, FP64 accumulation). */
enum { TLQ_PREC_FP64 = 0, TLQ_PREC_MIXED = 1 };

/* Runtime image of user/parameters.f90 (compile-time parameters there). */
typedef struct tlq_config {
  int nx, ny, nz;                 /* interior cells, parameters.f90:23-25 (each >= 2) */
  double xl, xr, yl, yr, zl, zr;  /* domain, parameters.f90:37-42 */
  double gamma;                   /* parameters.f90:43 */
  double cfl;                     /* parameters.f90:46 */
  double eta;                     /* artificial viscosity, parameters.f90:47 */
  double mu0;                     /* mean particle mass for calcTemp, parameters.f90:44 */
  double cooling_limit;           /* parameters.f90:49 */
  int limiter;                    /* TLQ_LIMITER_*, parameters.f90:18 */
  int solver;                     /* TLQ_SOLVER_* */
  int bc[6];                      /* x-, x+, y-, y+, z-, z+ = LB, RB, DB, TB, FB, BB (parameters.f90:10-15) */
  int cooling;                    /* TLQ_COOL_* (the reference's -DCOOL) */
  int cool_max_sub;               /* TLQ_COOL_SUBCYCLE: max sub-steps per step */
  double cool_sub_frac;           /* TLQ_COOL_SUBCYCLE: max Lambda n^2 h / E_th per sub-step;
                                     TLQ_COOL_EXACT, TLQ_COOL_MLP: the largest cooling number that
                                     takes the reference's single exponential step */
  int precision;                  /* TLQ_PREC_* */
  int device;                     /* CUDA device ordinal */
  double cool_mlp_tol;            /* TLQ_COOL_MLP: residual tolerance |T_pred - T_int|/T of an accepted
                                     cell, in (0, 1e-3] (default 1e-3; smaller trades speed for energy
                                     accuracy: more cells fall back) */
  int self_gravity;               /* the reference's -DGRAV: MultiGrid (sources.f90:99-193) before each
                                     stage, PHIT = PHIP + PHI (HLLC.f90:15-24); needs nx = ny = nz = 2^L,
                                     2 <= nx <= 1024 */
  int grav_bc;                    /* TLQ_GBC_*: the potential's values on the mesh faces */
} tlq_config;

/* Self-gravity boundary values.  ZERO: the reference's serial build, which
 * never imposes any (its neighbour ranks stay 0, so the `left < 0` tests of
 * sources.f90:112-130 fail) -- the face ghosts keep their first value, 0.
 * MULTIPOLE: its MPI build on one rank (no neighbours): the multipole
 * expansion to l = 4 (sources.f90:599-787) every 10 steps; not with
 * periodic boundaries (that build exchanges the potential's ghosts there). */
enum { TLQ_GBC_ZERO = 0, TLQ_GBC_MULTIPOLE = 1 };

/* spherical_wind_type, source/winds.f90:5-16 (same fields, same order). */
typedef struct tlq_wind {
  double xc, yc, zc;  /* source centre [code units of x] */
  double vx, vy, vz;  /* source velocity added to the radial wind */
  double radius;      /* cells with dist < radius are overwritten */
  double mdot;        /* mass-loss rate */
  double vinf;        /* terminal speed */
  double temp;        /* wind temperature [K] */
  double mu;          /* wind mean particle mass [AMU] */
} tlq_wind;

/* plane_wind_type, source/winds.f90:15-28: a uniform stream entering
 * through one face (plane 1..6 = left, right, front, back, bottom, top; the
 * velocity points into the box).  Imposed like the reference's
 * imposePlaneWind (winds.f90:92-147), which writes every i, j and the top
 * three z-planes k = nz..nz+2 whatever the plane. */
typedef struct tlq_plane_wind {
  int plane;
  double rho;   /* density */
  double vel;   /* speed */
  double temp;  /* temperature [K] */
  double mu;    /* mean particle mass [AMU] */
} tlq_plane_wind;

/* Learned cooling surrogate (build-defined; the reference has none).  A
 * 3-64-64-64-1 SiLU network maps (log10 n, log10 T, log10 tau), tau =
 * Lambda(T) n^2 dt / E_th the step's cooling number, to r with
 * ln(T/T_new) = tau (1 + tau r) (exact to first order in tau whatever r is).
 * It is trained on the GPU on pairs from the exact integrator (the sub-cycled
 * integrator's limit of infinitely many sub-steps, in closed form; pairs from
 * the sub-cycled integrator itself, sub-steps of sub_frac and sub_frac/2
 * Richardson-extrapolated, remain available but keep a one-sided error of
 * ~1e-5 T where cooling runs away, which a network trained on them
 * inherits).  In the step a cell whose tau exceeds the context's
 * cool_sub_frac and lies inside the training box takes
 * T_pred = max(T exp(-tau (1 + tau r)), T_0) when the a-posteriori energy
 * residual |T_pred - T_ex|/T <= cool_mlp_tol, T_ex the exact integrator's
 * temperature (TLQ_COOL_EXACT's closed form), and its cooling does not reach
 * the table's first temperature T_0 within the step; every other such cell
 * takes T_ex.  Training ignores the pairs that reach the table's first temperature
 * T_0 within the step and weighs pairs with tau < 1e-5 by (tau/1e-5)^2 (their
 * r is lost to FP64 round-off). */
#define TLQ_MLP_NPARAM 8641
typedef struct tlq_surrogate_opts {
  long long nsamples;      /* training pairs (default 2e7; 1 % held out) */
  int epochs;              /* passes over the pairs (default 30) */
  int batch;               /* minibatch (default 4096) */
  float lr;                /* Adam learning rate, cosine-decayed to lr/20 (default 3e-3) */
  unsigned long long seed;
  double box[6];           /* training box: log10 n, log10 T, log10 tau (lo, hi pairs;
                              default -4 4, 4 8.5, -8 1) */
  double sub_frac;         /* the pairs' integrator: 0 (default) the exact closed form, > 0 the
                              sub-cycled one with sub-steps of at most this tau, extrapolated */
  int max_sub;             /* sub-cycled pairs: max sub-steps (default 20000) */
} tlq_surrogate_opts;

typedef struct tlq_surrogate_report {
  double loss_first, loss_last;  /* minibatch MSE of y at the first and last step */
  double val_rmse_y;             /* RMSE of y = 1 + tau r on the held-out pairs that do not reach T_0
                                    (the other metrics too) */
  double val_max_rel_T;          /* max |T_pred - T_exact| / T on the held-out pairs (T_pred
                                    clamped at the table's first temperature, as in the step) */
  double val_p99_rel_T;          /* 99th percentile of the same */
  double val_accept;             /* fraction of held-out pairs within the step's 1e-3 check */
  double ms_generate, ms_train;  /* wall time of pair generation and training */
  long long steps;               /* optimiser steps */
} tlq_surrogate_report;

typedef struct tlq_stats {
  long long steps;      /* tlq_step/tlq_advance iterations since tlq_upload */
  double t, dt;         /* simulated time and the dt of the last step */
  int status;           /* sticky device status (TLQ_OK or the first error seen) */
  int graph;            /* 1 if steps are replayed from a captured CUDA graph */
  double ms_stage1;     /* average device time of the last timed stage-1 launches */
  double ms_stage2;     /* average device time of the last timed stage-2 launches */
  long long timed;      /* number of timed steps behind the averages */
  double bytes_state;   /* device bytes held for the mesh state */
  long long cool_mlp;      /* TLQ_COOL_MLP: cell-steps cooled by the network (since upload) */
  long long cool_fallback; /* TLQ_COOL_MLP: cell-steps with tau above cool_sub_frac cooled by the exact
                              integrator's closed form instead of the network: outside its box, failing
                              the residual check, or taken to the table's first temperature within the
                              step (stage 2 does those of the table's first segment itself) */
  double ms_cool;          /* TLQ_COOL_MLP: average device time of the timed cooling passes */
  long long cool_single;   /* TLQ_COOL_MLP: cell-steps with tau <= cool_sub_frac, cooled by the exact
                              integrator's single exponential step (the network has nothing to gain;
                              stage 2 does these, so their time is in ms_stage2, not ms_cool) */
  double ms_grav;          /* self-gravity: average device time of the timed steps' two MultiGrid solves
                              (ms_stage1/ms_stage2 then time the stage kernels alone) */
} tlq_stats;

typedef struct tlq_ctx tlq_ctx;

/* Defaults = user/parameters.f90 (50^3 on [-1,1]^3, gamma 5/3, cfl 0.4,
 * eta 0.005, van Leer, reflective, no cooling) with the HLLC solver. */
void tlq_config_default(tlq_config* cfg);

/* Context life cycle: initmain's allocation (source/init.f90:82-88). */
int tlq_create(const tlq_config* cfg, tlq_ctx** out);
int tlq_destroy(tlq_ctx* ctx);
/* Order the context's work on a caller-owned cudaStream_t (NULL: own stream). */
int tlq_set_stream(tlq_ctx* ctx, void* cuda_stream);

/* Cooling table, loaddata (source/cooling.f90:21-45): n rows of (T [K],
 * log10 Lambda), i.e. the file's second column negated.  Copied. */
int tlq_set_cooling_table(tlq_ctx* ctx, const double* T, const double* log10_lambda, int n);
/* Spherical winds applied in borders (user/user.f90:57-70).  Copied. */
int tlq_set_winds(tlq_ctx* ctx, const tlq_wind* winds, int n);
/* Plane winds imposed with the spherical ones in every ghost fill of the
 * step (user_boundaries), at most 6; n = 0 clears them. */
int tlq_set_plane_winds(tlq_ctx* ctx, const tlq_plane_wind* w, int n);
/* Point masses (x, y, z, M per mass) of pgravity (source/pointsource_gravity.f90:12-39);
 * the reference hard-codes M = 8 Msun (:23).  Copied; enables the source term. */
int tlq_set_point_masses(tlq_ctx* ctx, const double* xyzm, int n);

/* State transfer.  tlq_upload takes U after borders(U,1) (mainHD.f90:38) and
 * computes calc_prims + the first CFL dt on the device.  tlq_download writes
 * U and/or UPrim (either may be NULL) for output (HydroCore.f90:253).
 * Download is exact on the interior and the first ghost layer of each face;
 * the second ghost layer and edge/corner ghosts are never read by the step
 * and are returned as stored (unspecified). */
int tlq_upload(tlq_ctx* ctx, const double* U);
int tlq_download(tlq_ctx* ctx, double* U, double* UPrim);
int tlq_set_time(tlq_ctx* ctx, double t, int it);
int tlq_get_time(tlq_ctx* ctx, double* t, int* it, double* dt);

/* One iteration of mainHD.f90:74-99 (time_step, two HLL[C] stages, borders,
 * step, calc_prims, cooling).  Returns t, it and the dt used (any may be
 * NULL); waits for the step to finish.  tlq_advance runs n iterations with no
 * host round trip (replayed from a CUDA graph after the first call).
 * tlq_run_until runs while t < tfin (at most max_steps iterations). */
int tlq_step(tlq_ctx* ctx, double* t, int* it, double* dt);
int tlq_advance(tlq_ctx* ctx, int nsteps);
int tlq_run_until(tlq_ctx* ctx, double tfin, int max_steps, double* t, int* it, double* dt);
/* The end time of the run: steps start only while t < tfin (mainHD.f90:61);
 * +inf by default (tlq_run_until sets it for its call only). */
int tlq_set_tfin(tlq_ctx* ctx, double tfin);
int tlq_synchronize(tlq_ctx* ctx);

/* Diagnostics. */
int tlq_stats_get(tlq_ctx* ctx, tlq_stats* out);
int tlq_enable_timing(tlq_ctx* ctx, int on);
const char* tlq_last_error(tlq_ctx* ctx);
const char* tlq_status_string(int status);
/* Global sums over the interior: mass, x/y/z momentum, total energy. */
int tlq_conserved_sums(tlq_ctx* ctx, double out[5]);

/* Cooling surrogate: train on the GPU with the context's cooling table and
 * physics (stores the network in the context), read or install a network. */
void tlq_surrogate_opts_default(tlq_surrogate_opts* opts);
int tlq_train_cooling_surrogate(tlq_ctx* ctx, const tlq_surrogate_opts* opts, tlq_surrogate_report* report);
int tlq_get_cooling_surrogate(tlq_ctx* ctx, float* params, float* norm6, double* box6);
int tlq_set_cooling_surrogate(tlq_ctx* ctx, const float* params, const float* norm6, const double* box6);
/* Training pairs (context's table and physics) from the exact integrator's
 * closed form (sub_frac 0) or from the sub-cycled integrator (sub-steps of
 * at most sub_frac and sub_frac/2, at most max_sub, extrapolated): X = raw
 * features (3 per pair), Y = targets, raw = (n, T, T_new, dt) per pair (may
 * be NULL).  Host arrays. */
int tlq_cooling_pairs(tlq_ctx* ctx, long long n, unsigned long long seed, const double* box6, double sub_frac,
                      int max_sub, float* X, float* Y, double* raw);
/* Context-free network pieces on host arrays (normalised features): loss
 * sum_i w_i (y_i - t_i)^2 / n (w_i = Wt[i], or 1 when Wt is NULL) and its
 * gradient w.r.t. the 8641 FP32 parameters, and inference.  Training weighs
 * each pair by max(tau exp(-t tau), 1e-2)^2, the sensitivity of T_new/T to y. */
int tlq_mlp_loss_grad(const float* params, const float* X, const float* Y, const float* Wt, int n, float* grad,
                      float* loss);
int tlq_mlp_infer(const float* params, const float* X, int n, float* Y);

/* Output, source/HydroCore.f90:253-395 (`output`): UPrim of the current
 * state (after the steps queued so far) written in the reference's format --
 * BIN (all cells, little-endian, file points<rank>N<nout>.bin), DAT (text,
 * the interior, points<rank>N<nout>.dat; needs |nx - nz| <= 2, the
 * reference's loop bounds) or VTK (big-endian structured points,
 * EPV<rank>N<nout>.vtk) -- under outputpath.  Asynchronous: the snapshot is
 * formed behind the queued steps, copied on a copy stream and written by a
 * host thread while later steps run; one output is in flight at a time
 * (the next call waits for the previous one).  tlq_output_wait waits and
 * returns the write's status. */
enum { TLQ_OUT_DAT = 1, TLQ_OUT_VTK = 2, TLQ_OUT_BIN = 3 }; /* constants.f90:35-37 */
int tlq_output(tlq_ctx* ctx, int format, const char* outputpath, int nout, int rank);
int tlq_output_wait(tlq_ctx* ctx);

/* Stage tiling (no counterpart in the reference): the z-chunk length of the
 * stage grid (>= 8 planes, or nz; default 64 for nz >= 128, 32 for nz >= 32,
 * else nz), and the measuring autotuner that picks it -- from the cache file
 * (JSON keyed by GPU name, mesh size and form; NULL = no cache) or timed now
 * over `steps` steps per candidate (8, 16, 32, 64, 128) from the current
 * state, which is restored afterwards. */
int tlq_set_tiling(tlq_ctx* ctx, int zlen);
int tlq_get_tiling(const tlq_ctx* ctx, int* zlen);
int tlq_autotune(tlq_ctx* ctx, const char* cache_path, int steps, int* chosen);

/* ---- Batched ensemble (no counterpart in the reference, which runs one mesh
 * per process): many independent meshes of uneven sizes, each with its own
 * configuration, tables, winds, point masses, clock and dt, advanced together
 * by one persistent launch per stage over all members' tiles, the step
 * replayed from one CUDA graph.  Members run the mixed-precision step
 * (TLQ_PREC_MIXED; any cooling; a member with the cooling surrogate adds its
 * three cooling passes to the captured step).  Member i is a tlq_ctx
 * (tlq_batch_member) for every set-up and I/O call (tables, winds, masses,
 * upload, download, get_time); it must not be destroyed on its own.  A
 * member's failure (non-finite dt, non-positive density) stops that member
 * only. ------------------------------------------------------------------- */
typedef struct tlq_batch tlq_batch;
typedef struct tlq_batch_stats {
  int members;
  long long cells;            /* interior cells of all members */
  long long steps;            /* batch steps run */
  long long steps_timed;
  double ms_per_step;         /* average device time of the timed batch steps */
  int items;                  /* tiles in the work list */
  int blocks;                 /* persistent blocks per launch */
  int launches_per_step;
  int graph;                  /* 1 once the step is a captured graph */
} tlq_batch_stats;
int tlq_batch_create(const tlq_config* cfgs, int nmembers, tlq_batch** out);
int tlq_batch_destroy(tlq_batch* b);
int tlq_batch_size(const tlq_batch* b);
tlq_ctx* tlq_batch_member(tlq_batch* b, int i);
/* z-chunk length (planes per tile, >= 8) of member i; default by nz. */
int tlq_batch_set_tiling(tlq_batch* b, int i, int zlen);
int tlq_batch_get_tiling(const tlq_batch* b, int i, int* zlen);
/* Autotuner: per distinct mesh size, the z-chunk length from the cache file
 * (JSON, keyed by GPU name and size; NULL = no cache) or measured now over
 * `steps` steps from the members' current state (restored afterwards);
 * chosen[i] (may be NULL) receives member i's length. */
int tlq_batch_autotune(tlq_batch* b, const char* cache_path, int steps, int* chosen);
/* `steps` batch steps (every member whose t < its tfin advances one step). */
int tlq_batch_run(tlq_batch* b, int steps);
int tlq_batch_synchronize(tlq_batch* b);
/* Per-member status (TLQ_OK or the member's sticky error). */
int tlq_batch_status(tlq_batch* b, int* status);
int tlq_batch_enable_timing(tlq_batch* b, int on);
int tlq_batch_stats_get(tlq_batch* b, tlq_batch_stats* s);
const char* tlq_batch_last_error(const tlq_batch* b);

/* ---- Per-routine entry points (unit parity; host arrays in the reference
 * layout; each replaces the external subroutine cited). ------------------- */
/* calc_prims, source/HydroCore.f90:1-33 (all cells incl. ghosts). */
int tlq_calc_prims(tlq_ctx* ctx, double* UPrim, const double* U);
/* time_step, source/HydroCore.f90:113-155. */
int tlq_time_step(tlq_ctx* ctx, const double* UPrim, double* dt);
/* HLLCFluxes / HLLFluxes (choice 1 or 2), source/HLLC.f90:64-496 and
 * source/HLL.f90:71-297: F, G, H on faces i, j, k in 0..n; other entries of
 * F, G, H are left as passed. */
int tlq_fluxes(tlq_ctx* ctx, const double* U, double* F, double* G, double* H,
               const double* UPrim, int choice);
/* Godunov, source/HLLC.f90:1-62; with point masses set and UPrim given, adds
 * dt * S_Solver(UPrim, phi) (source/sources.f90:872-897, HLLC.f90:39-41). */
int tlq_godunov(tlq_ctx* ctx, double* UPPP, const double* UU, const double* F, const double* G,
                const double* H, const double* UPrim, double dt);
/* borders, source/boundaries.f90:1-26 (order 1 or 2; non-MPI branches) with
 * user_boundaries' spherical winds, in place. */
int tlq_borders(tlq_ctx* ctx, double* U, int order);
/* step, source/HydroCore.f90:170-211: U = UP + eta*Lap(U_old) on the
 * interior, ghost layers of U from UP, t += dt, it += 1. */
int tlq_viscous_step(tlq_ctx* ctx, double* U, const double* UP, double* t, int* it, double dt);
/* apply_cooling, source/cooling.f90:47-119 (or the sub-cycled form). */
int tlq_cooling(tlq_ctx* ctx, double* UPrim, double* U, double dt);
/* pointmass_potential, source/pointsource_gravity.f90:12-39:
 * phi(0:nx+1, 0:ny+1, 0:nz+1) -= sum_s G M_s / r. */
int tlq_point_potential(tlq_ctx* ctx, double* phi);
/* S_Solver, source/sources.f90:872-897. */
int tlq_gravity_source(tlq_ctx* ctx, const double* UPrim, const double* phi, double* S);
/* MultiGrid, source/sources.f90:99-193: one call on the density of U
 * (reference layout), the potential phi(0:nx+1, 0:ny+1, 0:nz+1) in and out,
 * it the step counter (multipole faces when it % 10 == 0); *cycles receives
 * the V-cycles run (may be NULL).  Needs self_gravity in the configuration. */
int tlq_multigrid(tlq_ctx* ctx, const double* U, double* phi, int it, int* cycles);

/* ---- Measurement (no counterpart in the reference) ----------------------
 * Throughput of the FP64 pipe of `device`, for the plain FP64 step's
 * roofline: independent dependency chains of FMA, IEEE division and IEEE
 * square root, timed with CUDA events (~10 ms of GPU time).  Writes the
 * operations per second of each. */
int tlq_measure_fp64_rate(int device, double* fma_per_s, double* div_per_s, double* sqrt_per_s);

/* ---- Allocation-free entry point (no counterpart in the reference) ------
 * time_step for callers that cannot allocate device memory: hosts whose GPU
 * memory belongs to an arena or pool allocator (an extra cudaMalloc can fail
 * once the pool has reserved the device, and it fragments the arena), or
 * step loops that cannot take cudaMalloc/cudaFree's implicit device
 * synchronisation.  Takes no context: d_uprim (UPrim in the reference layout
 * above, on the device) and d_dt (one double) are device buffers the caller
 * owns; dt is written to *d_dt asynchronously on cuda_stream (NULL: the
 * legacy default stream).  Calls no cudaMalloc, cudaFree or other allocating
 * routine.  Its reduction scratch is one fixed device variable inside the
 * library (72 bytes, held by every GPU that loads the library until exit),
 * so:
 *   - NULL pointers and sizes < 1 are rejected with TLQ_ERR_ARG;
 *   - every call asks the runtime for the variable's device address in the
 *     current context (cudaGetSymbolAddress, which allocates nothing); the
 *     first call in a context (on a device, or after cudaDeviceReset) loads
 *     the library's module there, so make that first call outside any
 *     stream capture;
 *   - all calls share the variable: calls that overlap on the GPU
 *     (concurrent streams, several host threads) race and must be serialised
 *     by the caller.
 * The return code covers the arguments and the launch only: it is known
 * before the kernel runs.  A state whose signal speeds give no finite,
 * positive dt (a NaN or infinite speed, or all speeds zero) is not reported
 * by the return code, as tlq_time_step reports it with TLQ_ERR_NONFINITE_DT:
 * the dt written to *d_dt is then NaN, infinite or not positive, so check
 * that it is finite and > 0 before using it. */
int tlq_time_step_noalloc(const double* d_uprim, int nx, int ny, int nz, double dx, double dy, double dz,
                          double gamma, double cfl, double* d_dt, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* TLQ_H */
