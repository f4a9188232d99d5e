/*
 * tlq_oracle.h -- CPU restatement of tlaloque's hydrodynamic time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the CUDA path is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it; the product library (libtlq) never links or calls it.
 *
 * Every routine restates one Fortran routine of tlaloque (cited file:line,
 * paths relative to the tlaloque source tree) in plain scalar C, FP64, with
 * the same loop ranges, the same branch order, the same evaluation order of
 * every expression (Fortran left-to-right association) and no FMA
 * contraction (built with -ffp-contract=off).  Loop nests are ordered with x
 * innermost (cache friendly) instead of the reference's k-innermost order;
 * every cell/face is computed independently, so the results are identical.
 *
 * Array layout is the reference's: A(1:5, -1:nx+2, -1:ny+2, -1:nz+2),
 * variable fastest, column-major (nghost = 2, user/parameters.f90:35).
 */
#ifndef TLQ_ORACLE_H
#define TLQ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary kinds, source/constants.f90:20-23. */
enum { TLQO_BC_OUTFLOW = 1, TLQO_BC_REFLECTIVE = 2, TLQO_BC_PERIODIC = 3, TLQO_BC_INFLOW = 4 };
/* Slope limiters, source/constants.f90:26-31. */
enum { TLQO_LIM_NONE = 1, TLQO_LIM_VANLEER = 2, TLQO_LIM_MINMOD = 3, TLQO_LIM_UMIST = 4,
       TLQO_LIM_WOODWARD = 5, TLQO_LIM_SUPERBEE = 6 };
/* Riemann solvers: source/HLLC.f90 (linked by the Makefile) and source/HLL.f90. */
enum { TLQO_SOLVER_HLLC = 0, TLQO_SOLVER_HLL = 1 };
/* Cooling modes: none; the reference's single exponential step
 * (source/cooling.f90:47-119); the sub-cycled integrator built on it. */
/* TLQO_COOL_EXACT: the sub-cycled integrator in the limit of infinitely many
 * sub-steps (closed form), with the reference formula for a cell that needs
 * one sub-step.  Value 4 (3 is the GPU's learned surrogate). */
enum { TLQO_COOL_NONE = 0, TLQO_COOL_REF = 1, TLQO_COOL_SUBCYCLE = 2, TLQO_COOL_EXACT = 4 };

/* Boundary values of the self-gravity potential on the mesh faces: the
 * reference's serial build never imposes any (they stay 0), its MPI build on
 * one rank imposes the multipole expansion (source/sources.f90:683-787)
 * every 10 steps.  The two also fill coarse-level ghosts in different orders. */
enum { TLQO_GBC_ZERO = 0, TLQO_GBC_MULTIPOLE = 1 };

/* spherical_wind_type, source/winds.f90:5-16 (same field order). */
typedef struct tlqo_wind {
  double xc, yc, zc, vx, vy, vz, radius, mdot, vinf, temp, mu;
} tlqo_wind;

/* plane_wind_type, source/winds.f90:15-28 (plane 1..6: left, right, front,
 * back, bottom, top). */
typedef struct tlqo_plane_wind {
  int plane;
  double rho, vel, temp, mu;
} tlqo_plane_wind;

/* Runtime image of user/parameters.f90 plus the per-run tables. */
typedef struct tlqo_params {
  int nx, ny, nz;                       /* nxtot.. (parameters.f90:23-25), no MPI split */
  double xl, xr, yl, yr, zl, zr;        /* parameters.f90:37-42 */
  double gamma, cfl, eta, mu0;          /* parameters.f90:43-47 */
  double cooling_limit;                 /* parameters.f90:49 */
  int limiter;                          /* parameters.f90:18 */
  int solver;                           /* TLQO_SOLVER_* */
  int bc[6];                            /* LB, RB, DB, TB, FB, BB = x-, x+, y-, y+, z-, z+ */
  int cooling;                          /* TLQO_COOL_* */
  int ncool;                            /* nptsT (cooling.f90:32) */
  const double* coolT;                  /* cooltable(1,:) : T [K] */
  const double* coolC;                  /* cooltable(2,:) : log10 Lambda (= -b of the file) */
  int cool_max_sub;                     /* sub-cycled integrator: max sub-steps */
  double cool_sub_frac;                 /* sub-cycled integrator: max ce*h per sub-step */
  int nwinds;
  const tlqo_wind* winds;
  int nmasses;                          /* point masses, source/pointsource_gravity.f90 */
  const double* masses;                 /* 4 per mass: x, y, z, M [g] */
  int nthreads;                         /* OpenMP threads (<=0: runtime default) */
  int nplanes;                          /* plane winds, imposed after the spherical ones */
  const tlqo_plane_wind* planes;
  int self_gravity;                     /* -DGRAV: MultiGrid in every Godunov (HLLC.f90:15-24) */
  int grav_bc;                          /* TLQO_GBC_*; nx = ny = nz = 2^L required */
} tlqo_params;

/* Size in doubles of one conserved/primitive array (5 vars incl. ghosts). */
long tlqo_array_len(const tlqo_params* p);
/* Size in doubles of the potential array phi(0:nx+1, 0:ny+1, 0:nz+1). */
long tlqo_phi_len(const tlqo_params* p);

/* Per-routine restatements (host arrays in the reference layout). */
void tlqo_calc_prims(const tlqo_params* p, double* UPrim, const double* U);
double tlqo_time_step(const tlqo_params* p, const double* UPrim);
void tlqo_fluxes(const tlqo_params* p, const double* U, double* F, double* G, double* H,
                 const double* UPrim, int choice);
void tlqo_godunov(const tlqo_params* p, double* UPPP, const double* UU, const double* F,
                  const double* G, const double* H, double dt, const double* S);
void tlqo_borders(const tlqo_params* p, double* U, int order);
void tlqo_impose_winds(const tlqo_params* p, double* U);
void tlqo_step(const tlqo_params* p, double* U, const double* UP, double* UPP,
               double* t, int* it, double dt);
void tlqo_cooling(const tlqo_params* p, double* UPrim, double* U, double dt);
void tlqo_point_potential(const tlqo_params* p, double* phi);
/* Self-gravity (source/sources.f90:99-485): levels L with nx = 2^L (-1 when
 * the mesh is not such a cube); the work array's length in doubles; one
 * MultiGrid call on the density U(1, 0:nx+1, ...) of the conserved array U,
 * phi (nx+2)^3 in and out, it the step counter.  Returns the V-cycles run. */
int tlqo_mg_levels(const tlqo_params* p);
long tlqo_mg_work_len(const tlqo_params* p);
int tlqo_multigrid(const tlqo_params* p, const double* U, double* phi, int it, double* work);
void tlqo_gravity_source(const tlqo_params* p, const double* UPrim, const double* phi, double* S);
double tlqo_cool_coef(const tlqo_params* p, double temp);
/* The exact integrator's closed form (TLQO_COOL_EXACT): G at the table
 * nodes (ncool values), and the temperature after a step of cooling number
 * tau of a cell at temp >= T_0 whose find_coef value is lam. */
void tlqo_cool_gcum(const tlqo_params* p, double* gcum);
double tlqo_cool_exact_T(const tlqo_params* p, const double* gcum, double temp, double lam, double tau);

/* Whole-run state of the main loop, source/mainHD.f90:22-100. */
typedef struct tlqo_state {
  double *U, *UP, *UPP, *UPrim, *F, *G, *H, *S, *PHI;  /* PHI, S: NULL without gravity */
  double t, dt;
  int it;
  double *PHIG, *PHIT, *MGW;  /* self-gravity potential, PHIP + PHIG, MultiGrid work (else NULL) */
} tlqo_state;

/* mainHD.f90:38-44: borders(U,1), calc_prims(UPrim,U) (+ point potential). */
void tlqo_init(const tlqo_params* p, tlqo_state* s);
/* mainHD.f90:61-100: at most nsteps loop iterations while t < tfin.
 * Returns the number of iterations run. */
int tlqo_run(const tlqo_params* p, tlqo_state* s, int nsteps, double tfin);

#ifdef __cplusplus
}
#endif
#endif
