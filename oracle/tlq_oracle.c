/*
 * tlq_oracle.c -- CPU restatement of tlaloque's hydrodynamic time step.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never shipped or
 * called by the product.  See tlq_oracle.h for the conventions (reference
 * layout, evaluation order, no FMA contraction).  Build with
 *   gcc -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared
 * Citations are file:line in the tlaloque source tree.
 */
#include "tlq_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* source/constants.f90:6-15 (cgs).  PI is the reference's truncated value. */
#define AMU 1.660538782e-24
#define KB 1.380650400e-16
#define GR 6.67430e-8
#define PI_REF 3.14159265358979
/* apply_cooling's temperature floor, source/cooling.f90:56. */
#define T_FLOOR 10.0

#define NTHREADS(p) ((p)->nthreads > 0 ? (p)->nthreads : omp_default_threads())

static int omp_default_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Fortran MIN/MAX of two reals (ties and NaNs never matter for valid states). */
static inline double mn(double a, double b) { return (b < a) ? b : a; }
static inline double mx(double a, double b) { return (b > a) ? b : a; }
/* Fortran SIGN(1.0, a) with gfortran's default -fsign-zero semantics. */
static inline double sgn1(double a) { return copysign(1.0, a); }

/* Offset of U(e, i, j, k), e in 0..4, i in -1..nx+2 (reference layout). */
static inline long IX(const tlqo_params* p, int e, int i, int j, int k) {
  return (long)e + 5L * ((long)(i + 1) + (long)(p->nx + 4) * ((long)(j + 1) + (long)(p->ny + 4) * (long)(k + 1)));
}
/* Offset of phi(i, j, k), i in 0..nx+1 (pointsource_gravity.f90:14). */
static inline long PX(const tlqo_params* p, int i, int j, int k) {
  return (long)i + (long)(p->nx + 2) * ((long)j + (long)(p->ny + 2) * (long)k);
}

long tlqo_array_len(const tlqo_params* p) { return 5L * (p->nx + 4) * (long)(p->ny + 4) * (long)(p->nz + 4); }
long tlqo_phi_len(const tlqo_params* p) { return (long)(p->nx + 2) * (long)(p->ny + 2) * (long)(p->nz + 2); }

static inline double DX(const tlqo_params* p) { return (p->xr - p->xl) / (double)p->nx; }
static inline double DY(const tlqo_params* p) { return (p->yr - p->yl) / (double)p->ny; }
static inline double DZ(const tlqo_params* p) { return (p->zr - p->zl) / (double)p->nz; }

/* xcoord/ycoord/zcoord, source/HydroCore.f90:35-77, one rank (coords = 0). */
static inline double xcoord(const tlqo_params* p, int i) { double dx = DX(p); return (p->xl + dx * (double)i) - dx / 2.0; }
static inline double ycoord(const tlqo_params* p, int j) { double dy = DY(p); return (p->yl + dy * (double)j) - dy / 2.0; }
static inline double zcoord(const tlqo_params* p, int k) { double dz = DZ(p); return (p->zl + dz * (double)k) - dz / 2.0; }

/* ---------------------------------------------------------------------------
 * calc_prims, source/HydroCore.f90:1-33: all cells including ghosts.
 * ------------------------------------------------------------------------- */
void tlqo_calc_prims(const tlqo_params* p, double* W, const double* U) {
  const double g = p->gamma;
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = -1; k <= p->nz + 2; ++k)
    for (int j = -1; j <= p->ny + 2; ++j)
      for (int i = -1; i <= p->nx + 2; ++i) {
        const double* u = U + IX(p, 0, i, j, k);
        double* w = W + IX(p, 0, i, j, k);
        w[0] = u[0];
        w[1] = u[1] / u[0];
        w[2] = u[2] / u[0];
        w[3] = u[3] / u[0];
        w[4] = (g - 1.0) * (u[4] - 0.5 * ((u[1] * u[1] + u[2] * u[2]) + u[3] * u[3]) / u[0]);
        w[4] = mx(w[4], 1e-20);
      }
}

/* csound, source/HydroCore.f90:157-168. */
static inline double csound(double g, double pres, double den) { return sqrt(g * pres / den); }

/* ---------------------------------------------------------------------------
 * time_step, source/HydroCore.f90:113-155 (no MPI: dt = dtp).
 * ------------------------------------------------------------------------- */
double tlqo_time_step(const tlqo_params* p, const double* W) {
  double maxvx = 0.0, maxvy = 0.0, maxvz = 0.0;
  const double g = p->gamma;
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p)) reduction(max : maxvx, maxvy, maxvz)
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i) {
        const double* w = W + IX(p, 0, i, j, k);
        double cs = csound(g, w[4], w[0]);
        maxvx = mx(maxvx, fabs(w[1]) + cs);
        maxvy = mx(maxvy, fabs(w[2]) + cs);
        maxvz = mx(maxvz, fabs(w[3]) + cs);
      }
  double m = mn(mn(DX(p) / maxvx, DY(p) / maxvy), DZ(p) / maxvz);
  return p->cfl * m / sqrt(3.0);
}

/* prim2f, source/HydroCore.f90:213-251.  d = 1, 2, 3. */
static inline void prim2f(double g1, double* ff, const double* w, int d) {
  double e = w[d] * (0.5 * w[0] * ((w[1] * w[1] + w[2] * w[2]) + w[3] * w[3]) + g1 * w[4]);
  if (d == 1) {
    ff[0] = w[0] * w[1];
    ff[1] = w[0] * w[1] * w[1] + w[4];
    ff[2] = w[0] * w[1] * w[2];
    ff[3] = w[0] * w[1] * w[3];
  } else if (d == 2) {
    ff[0] = w[0] * w[2];
    ff[1] = w[0] * w[1] * w[2];
    ff[2] = w[0] * w[2] * w[2] + w[4];
    ff[3] = w[0] * w[2] * w[3];
  } else {
    ff[0] = w[0] * w[3];
    ff[1] = w[0] * w[1] * w[3];
    ff[2] = w[0] * w[2] * w[3];
    ff[3] = w[0] * w[3] * w[3] + w[4];
  }
  ff[4] = e;
}

/* limiter's contained function average, source/HLLC.f90:586-636. */
static inline double average(double a, double b, int opt) {
  double s, c, d, r;
  switch (opt) {
    case TLQO_LIM_NONE:
      return 0.5 * (a + b);
    case TLQO_LIM_VANLEER:
      if (a * b <= 0.0) return 0.0;
      return a * b * (a + b) / (a * a + b * b);
    case TLQO_LIM_MINMOD:
      s = sgn1(a);
      return s * mx(0.0, mn(fabs(a), s * b));
    case TLQO_LIM_UMIST:
      s = sgn1(a);
      c = 0.25 * a + 0.75 * b;
      d = 0.75 * a + 0.25 * b;
      r = mn(mn(mn(2.0 * fabs(a), 2.0 * s * b), s * c), s * d);
      return s * mx(0.0, r);
    case TLQO_LIM_WOODWARD:
      s = sgn1(a);
      c = 0.5 * (a + b);
      r = mn(mn(2.0 * fabs(a), 2.0 * s * b), s * c);
      return s * mx(0.0, r);
    case TLQO_LIM_SUPERBEE:
      s = sgn1(b);
      c = mn(2.0 * fabs(b), s * a);
      d = mn(fabs(b), 2.0 * s * a);
      return s * mx(mx(0.0, c), d);
    default:
      return NAN; /* the reference stops here (HLLC.f90:630-633) */
  }
}

/* limiter, source/HLLC.f90:560-583: reconstructs pl, pr in place. */
static inline void limiter(const double* pll, double* pl, double* pr, const double* prr, int lim) {
  for (int e = 0; e < 5; ++e) {
    double dl = pl[e] - pll[e];
    double dm = pr[e] - pl[e];
    double dr = prr[e] - pr[e];
    double al = average(dl, dm, lim);
    double ar = average(dm, dr, lim);
    pl[e] = pl[e] + 0.5 * al;
    pr[e] = pr[e] - 0.5 * ar;
  }
}

/* One Riemann flux at a face in direction d (1..3).
 * HLLC: HLLCFluxes branches, source/HLLC.f90:99-136 (x; y :139-176; z :179-216),
 *       wavespeed source/HLLC.f90:498-518.
 * HLL:  HLLFluxes branches, source/HLL.f90:106-129, wavespeed source/HLL.f90:299-317.
 * UL, UR are the cell-centred conserved states of the two cells (the star /
 * HLL states use them even when wl, wr are reconstructed). */
static inline void riemann(const tlqo_params* p, double* ff, const double* wl, const double* wr,
                           const double* UL, const double* UR, int d) {
  const double g = p->gamma, g1 = p->gamma / (p->gamma - 1.0);
  double csl = csound(g, wl[4], wl[0]);
  double csr = csound(g, wr[4], wr[0]);
  double sl = mn(wl[d] - csl, wr[d] - csr);
  double sr = mx(wl[d] + csl, wr[d] + csr);
  if (p->solver == TLQO_SOLVER_HLL) {
    if (sl >= 0) {
      prim2f(g1, ff, wl, d);
    } else if (sr <= 0) {
      prim2f(g1, ff, wr, d);
    } else {
      double fl[5], fr[5];
      prim2f(g1, fl, wl, d);
      prim2f(g1, fr, wr, d);
      for (int e = 0; e < 5; ++e) ff[e] = (sr * fl[e] - sl * fr[e] + sl * sr * (UR[e] - UL[e])) / (sr - sl);
    }
    return;
  }
  double sst = (wr[4] - wl[4] + wl[0] * wl[d] * (sl - wl[d]) - wr[0] * wr[d] * (sr - wr[d])) /
               (wl[0] * (sl - wl[d]) - wr[0] * (sr - wr[d]));
  if (sl >= 0) {
    prim2f(g1, ff, wl, d);
  } else if (sr <= 0) {
    prim2f(g1, ff, wr, d);
  } else if (sst >= 0) {
    double fl[5], us[5];
    prim2f(g1, fl, wl, d);
    double rhostr = wl[0] * (sl - wl[d]) / (sl - sst);
    us[0] = rhostr;
    for (int e = 1; e <= 3; ++e) us[e] = (e == d) ? rhostr * sst : rhostr * wl[e];
    us[4] = rhostr * (UL[4] / wl[0] + (sst - wl[d]) * (sst + wl[4] / (wl[0] * (sl - wl[d]))));
    for (int e = 0; e < 5; ++e) ff[e] = fl[e] + sl * (us[e] - UL[e]);
  } else if (sst <= 0) {
    double fr[5], us[5];
    prim2f(g1, fr, wr, d);
    double rhostr = wr[0] * (sr - wr[d]) / (sr - sst);
    us[0] = rhostr;
    for (int e = 1; e <= 3; ++e) us[e] = (e == d) ? rhostr * sst : rhostr * wr[e];
    us[4] = rhostr * (UR[4] / wr[0] + (sst - wr[d]) * (sst + wr[4] / (wr[0] * (sr - wr[d]))));
    for (int e = 0; e < 5; ++e) ff[e] = fr[e] + sr * (us[e] - UR[e]);
  }
  /* NaN sst falls through every branch: the reference then leaves the face
   * flux untouched; here it is left as passed in. */
}

/* ---------------------------------------------------------------------------
 * HLLCFluxes / HLLFluxes, source/HLLC.f90:64-496 and source/HLL.f90:71-297.
 * Faces (i+1/2, j, k), (i, j+1/2, k), (i, j, k+1/2) for i, j, k in 0..n.
 * ------------------------------------------------------------------------- */
void tlqo_fluxes(const tlqo_params* p, const double* U, double* F, double* G, double* H,
                 const double* W, int choice) {
  const int lim = p->limiter;
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 0; k <= p->nz; ++k)
    for (int j = 0; j <= p->ny; ++j)
      for (int i = 0; i <= p->nx; ++i) {
        double a[5], b[5], c[5], d[5];
        /* x direction */
        for (int e = 0; e < 5; ++e) {
          b[e] = W[IX(p, e, i, j, k)];
          c[e] = W[IX(p, e, i + 1, j, k)];
        }
        if (choice == 2) {
          for (int e = 0; e < 5; ++e) {
            a[e] = W[IX(p, e, i - 1, j, k)];
            d[e] = W[IX(p, e, i + 2, j, k)];
          }
          limiter(a, b, c, d, lim);
        }
        riemann(p, F + IX(p, 0, i, j, k), b, c, U + IX(p, 0, i, j, k), U + IX(p, 0, i + 1, j, k), 1);
        /* y direction */
        for (int e = 0; e < 5; ++e) {
          b[e] = W[IX(p, e, i, j, k)];
          c[e] = W[IX(p, e, i, j + 1, k)];
        }
        if (choice == 2) {
          for (int e = 0; e < 5; ++e) {
            a[e] = W[IX(p, e, i, j - 1, k)];
            d[e] = W[IX(p, e, i, j + 2, k)];
          }
          limiter(a, b, c, d, lim);
        }
        riemann(p, G + IX(p, 0, i, j, k), b, c, U + IX(p, 0, i, j, k), U + IX(p, 0, i, j + 1, k), 2);
        /* z direction */
        for (int e = 0; e < 5; ++e) {
          b[e] = W[IX(p, e, i, j, k)];
          c[e] = W[IX(p, e, i, j, k + 1)];
        }
        if (choice == 2) {
          for (int e = 0; e < 5; ++e) {
            a[e] = W[IX(p, e, i, j, k - 1)];
            d[e] = W[IX(p, e, i, j, k + 2)];
          }
          limiter(a, b, c, d, lim);
        }
        riemann(p, H + IX(p, 0, i, j, k), b, c, U + IX(p, 0, i, j, k), U + IX(p, 0, i, j, k + 1), 3);
      }
}

/* ---------------------------------------------------------------------------
 * Godunov, source/HLLC.f90:1-62: interior update, plus dt*S (HLLC.f90:39-41)
 * when a gravity source S is given.
 * ------------------------------------------------------------------------- */
void tlqo_godunov(const tlqo_params* p, double* UPPP, const double* UU, const double* F,
                  const double* G, const double* H, double dt, const double* S) {
  const double dtdx = dt / DX(p), dtdy = dt / DY(p), dtdz = dt / DZ(p);
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i)
        for (int e = 0; e < 5; ++e) {
          long c = IX(p, e, i, j, k);
          double v = UU[c] - dtdx * (F[c] - F[IX(p, e, i - 1, j, k)]) - dtdy * (G[c] - G[IX(p, e, i, j - 1, k)]) -
                     dtdz * (H[c] - H[IX(p, e, i, j, k - 1)]);
          if (S) v = v + dt * S[c];
          UPPP[c] = v;
        }
}

/* Copy or mirror one cell: dst = src with the momentum component `flip`
 * (1..3, 0 = none) negated. */
static inline void bc_cell(double* U, long dst, long src, int flip) {
  for (int e = 0; e < 5; ++e) U[dst + e] = (flip > 0 && e == flip) ? -U[src + e] : U[src + e];
}

/* One boundary face fill.  axis 0/1/2, side 0 = low, 1 = high; `layer` is the
 * ghost layer (1 = adjacent, 2 = outer); `srcidx` the interior index read. */
static void fill_plane(const tlqo_params* p, double* U, int axis, int dstidx, int srcidx, int flip) {
  int n[3] = {p->nx, p->ny, p->nz};
  int ua = (axis == 0) ? 1 : 0, vb = (axis == 2) ? 1 : 2;
  for (int b = -1; b <= n[vb] + 2; ++b)
    for (int a = -1; a <= n[ua] + 2; ++a) {
      int di[3], si[3];
      di[axis] = dstidx; si[axis] = srcidx;
      di[ua] = si[ua] = a;
      di[vb] = si[vb] = b;
      bc_cell(U, IX(p, 0, di[0], di[1], di[2]), IX(p, 0, si[0], si[1], si[2]), flip);
    }
}

/* Periodic two-layer copy with the Fortran array-assignment semantics
 * (right-hand side read before any element is written). */
static void fill_plane_pair(const tlqo_params* p, double* U, int axis, int d0, int s0) {
  int n[3] = {p->nx, p->ny, p->nz};
  int ua = (axis == 0) ? 1 : 0, vb = (axis == 2) ? 1 : 2;
  for (int b = -1; b <= n[vb] + 2; ++b)
    for (int a = -1; a <= n[ua] + 2; ++a) {
      double tmp[10];
      for (int l = 0; l < 2; ++l) {
        int si[3]; si[axis] = s0 + l; si[ua] = a; si[vb] = b;
        for (int e = 0; e < 5; ++e) tmp[5 * l + e] = U[IX(p, e, si[0], si[1], si[2])];
      }
      for (int l = 0; l < 2; ++l) {
        int di[3]; di[axis] = d0 + l; di[ua] = a; di[vb] = b;
        for (int e = 0; e < 5; ++e) U[IX(p, e, di[0], di[1], di[2])] = tmp[5 * l + e];
      }
    }
}

/* boundariesI, non-MPI branch, source/boundaries.f90:179-259.
 * Order: x- (LB), x+ (RB), y+ (TB), y- (DB), z+ (BB), z- (FB). */
static void boundaries1(const tlqo_params* p, double* U) {
  const int n[3] = {p->nx, p->ny, p->nz};
  /* (axis, side) in the reference's order */
  const int order[6][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 0}, {2, 1}, {2, 0}};
  for (int q = 0; q < 6; ++q) {
    int axis = order[q][0], side = order[q][1];
    int bc = p->bc[2 * axis + side];
    int dst = side ? n[axis] + 1 : 0;
    int src_in = side ? n[axis] : 1;
    if (bc == TLQO_BC_OUTFLOW) fill_plane(p, U, axis, dst, src_in, 0);
    else if (bc == TLQO_BC_REFLECTIVE) fill_plane(p, U, axis, dst, src_in, axis + 1);
    else if (bc == TLQO_BC_PERIODIC) fill_plane(p, U, axis, dst, side ? 1 : n[axis], 0);
    /* BC_INFLOW: empty stub in the reference (boundaries.f90:191-192) */
  }
}

/* boundariesII, non-MPI branch, source/boundaries.f90:432-533.
 * Order: x- (LB), x+ (RB), y- (DB), y+ (TB), z- (FB), z+ (BB). */
static void boundaries2(const tlqo_params* p, double* U) {
  const int n[3] = {p->nx, p->ny, p->nz};
  for (int axis = 0; axis < 3; ++axis)
    for (int side = 0; side < 2; ++side) {
      int bc = p->bc[2 * axis + side];
      int N = n[axis];
      if (bc == TLQO_BC_PERIODIC) {
        if (side == 0) fill_plane_pair(p, U, axis, -1, N - 1);  /* U(-1:0) = U(n-1:n) */
        else fill_plane_pair(p, U, axis, N + 1, 1);             /* U(n+1:n+2) = U(1:2) */
      } else if (bc == TLQO_BC_OUTFLOW) {
        if (side == 0) { fill_plane(p, U, axis, 0, 1, 0); fill_plane(p, U, axis, -1, 1, 0); }
        else { fill_plane(p, U, axis, N + 1, N, 0); fill_plane(p, U, axis, N + 2, N, 0); }
      } else if (bc == TLQO_BC_REFLECTIVE) {
        if (side == 0) { fill_plane(p, U, axis, 0, 1, axis + 1); fill_plane(p, U, axis, -1, 2, axis + 1); }
        else { fill_plane(p, U, axis, N + 1, N, axis + 1); fill_plane(p, U, axis, N + 2, N - 1, axis + 1); }
      }
    }
}

/* ---------------------------------------------------------------------------
 * imposeSphericalWind for every wind, user/user.f90:57-70 ->
 * source/winds.f90:32-90: all cells including ghosts.
 * ------------------------------------------------------------------------- */
void tlqo_impose_winds(const tlqo_params* p, double* U) {
  const double g = p->gamma;
  for (int s = 0; s < p->nwinds; ++s) {
    const tlqo_wind* w = &p->winds[s];
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
    for (int k = -1; k <= p->nz + 2; ++k)
      for (int j = -1; j <= p->ny + 2; ++j)
        for (int i = -1; i <= p->nx + 2; ++i) {
          double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
          double dist = sqrt((x - w->xc) * (x - w->xc) + (y - w->yc) * (y - w->yc) + (z - w->zc) * (z - w->zc));
          if (dist < w->radius) {
            double dens = w->mdot / (w->vinf * dist * dist * 4.0 * PI_REF);
            double vx = w->vinf * (x - w->xc) / dist + w->vx;
            double vy = w->vinf * (y - w->yc) / dist + w->vy;
            double vz = w->vinf * (z - w->zc) / dist + w->vz;
            double pres = dens * KB * w->temp / (w->mu * AMU);
            double* u = U + IX(p, 0, i, j, k);
            u[0] = dens;
            u[1] = dens * vx;
            u[2] = dens * vy;
            u[3] = dens * vz;
            u[4] = 0.5 * dens * ((vx * vx + vy * vy) + vz * vz) + pres / (g - 1.0);
          }
        }
  }
  /* imposePlaneWind, source/winds.f90:92-147: i over nxmin..nxmax, j over
   * nymin..nymax, k over nz..nzmax (the top three z-planes, whatever the
   * plane); pres = dens/(mu AMU) KB temp. */
  for (int s = 0; s < p->nplanes; ++s) {
    const tlqo_plane_wind* w = &p->planes[s];
    double vx = 0.0, vy = 0.0, vz = 0.0;
    switch (w->plane) {
      case 1: vx = w->vel; break;
      case 2: vx = -w->vel; break;
      case 3: vy = w->vel; break;
      case 4: vy = -w->vel; break;
      case 5: vz = w->vel; break;
      case 6: vz = -w->vel; break;
      default: break;
    }
    const double pres = w->rho / (w->mu * AMU) * KB * w->temp;
    for (int i = -1; i <= p->nx + 2; ++i)
      for (int j = -1; j <= p->ny + 2; ++j)
        for (int k = p->nz; k <= p->nz + 2; ++k) {
          double* u = U + IX(p, 0, i, j, k);
          u[0] = w->rho;
          u[1] = w->rho * vx;
          u[2] = w->rho * vy;
          u[3] = w->rho * vz;
          u[4] = 0.5 * w->rho * ((vx * vx + vy * vy) + vz * vz) + pres / (g - 1.0);
        }
  }
}

/* borders, source/boundaries.f90:1-26. */
void tlqo_borders(const tlqo_params* p, double* U, int order) {
  if (order == 1) boundaries1(p, U);
  else boundaries2(p, U);
  tlqo_impose_winds(p, U);
}

/* ---------------------------------------------------------------------------
 * step, source/HydroCore.f90:170-211.  UPP is the global scratch the
 * reference overwrites with the old U (UPP = U, :182).
 * ------------------------------------------------------------------------- */
void tlqo_step(const tlqo_params* p, double* U, const double* UP, double* UPP, double* t, int* it, double dt) {
  const long n = tlqo_array_len(p);
  const double eta = p->eta;
  memcpy(UPP, U, (size_t)n * sizeof(double));
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i)
        for (int e = 0; e < 5; ++e) {
          long c = IX(p, e, i, j, k);
          U[c] = UP[c] + eta * (UPP[IX(p, e, i + 1, j, k)] + UPP[IX(p, e, i - 1, j, k)] + UPP[IX(p, e, i, j + 1, k)] +
                                UPP[IX(p, e, i, j - 1, k)] + UPP[IX(p, e, i, j, k + 1)] + UPP[IX(p, e, i, j, k - 1)] -
                                6.0 * UPP[c]);
        }
  /* Ghost planes of U from UP (:195-206): every cell outside the interior. */
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = -1; k <= p->nz + 2; ++k)
    for (int j = -1; j <= p->ny + 2; ++j)
      for (int i = -1; i <= p->nx + 2; ++i) {
        int inside = i >= 1 && i <= p->nx && j >= 1 && j <= p->ny && k >= 1 && k <= p->nz;
        if (!inside)
          for (int e = 0; e < 5; ++e) U[IX(p, e, i, j, k)] = UP[IX(p, e, i, j, k)];
      }
  *t = *t + dt;
  *it = *it + 1;
}

/* ---------------------------------------------------------------------------
 * Cooling, source/cooling.f90:47-159.
 * ------------------------------------------------------------------------- */

/* find_coef, source/cooling.f90:121-144: first table entry with T_i > temp,
 * log-linear interpolation.  Above the last entry the reference leaves coef
 * undefined; this restatement (and the GPU path) hold it at the last entry. */
double tlqo_cool_coef(const tlqo_params* p, double temp) {
  for (int i = 1; i < p->ncool; ++i) {
    if (p->coolT[i] > temp) {
      double T0 = log10(p->coolT[i - 1]);
      double C0 = p->coolC[i - 1];
      double T1 = log10(p->coolT[i]);
      double C1 = p->coolC[i];
      return pow(10.0, (C1 - C0) / (T1 - T0) * (log10(temp) - T0) + C0);
    }
  }
  return pow(10.0, p->coolC[p->ncool - 1]);
}

/* calcTemp, source/cooling.f90:146-159. */
static inline double calc_temp(const tlqo_params* p, const double* w) { return w[4] * p->mu0 * AMU / (w[0] * KB); }

/* The exact integrator (TLQO_COOL_EXACT): the temperature after a step of a
 * cell at temp >= T_0 with cooling number tau = ce*dt (ce = Lambda n^2 / E_th
 * at temp).  At fixed density, d ln T/dt = -ce(T) is the sub-cycled
 * integrator's equation in the limit of infinitely many sub-steps; with
 * E_th proportional to T it is dT/dt = -kappa Lambda(T), and find_coef's
 * interpolation, log-linear between nodes (cooling.f90:133-140), makes
 * Lambda(T) = Lambda_i (T/T_i)^s_i on [T_i, T_{i+1}) a power law, held at
 * the last node's value above the table.  So the step integrates in closed
 * form (exact integration of a piecewise power-law cooling function:
 * Townsend 2009, ApJS 181, 391): with a = 1 - s_i, the cell stays in its
 * segment while tau <= (1 - (T_i/T)^a)/a and then ends at
 * T (1 - a tau)^(1/a); otherwise it crosses T_i with budget
 * B = (tau - tau_i) T/Lambda(T) left of G(T) = int_{T_0}^{T} dT'/Lambda,
 * and ends in the segment j whose nodes bracket G(T_i) - B (G at the nodes
 * is a running sum of the segments' integrals).  Below T_0 nothing cools, so
 * a cell that reaches T_0 within the step ends there. */
static double seg_slope(const tlqo_params* p, int i) {
  if (i >= p->ncool - 1) return 0.0; /* held above the last node */
  return (p->coolC[i + 1] - p->coolC[i]) / (log10(p->coolT[i + 1]) - log10(p->coolT[i]));
}

/* x^(1/a) of the power-law solution, its a -> 0 limit exp(lim_arg). */
static double pow_inv(double base, double a, double lim_arg) {
  return fabs(a) < 1e-9 ? exp(lim_arg) : pow(base, 1.0 / a);
}

/* G at the nodes: gcum[0] = 0, gcum[i+1] = gcum[i] + int_{T_i}^{T_{i+1}} dT/Lambda. */
void tlqo_cool_gcum(const tlqo_params* p, double* gcum) {
  gcum[0] = 0.0;
  for (int i = 0; i + 1 < p->ncool; ++i) {
    const double a = 1.0 - seg_slope(p, i), Li = pow(10.0, p->coolC[i]), r = p->coolT[i + 1] / p->coolT[i];
    const double g = fabs(a) < 1e-9 ? (p->coolT[i] / Li) * log(r) : (p->coolT[i] / Li) * (pow(r, a) - 1.0) / a;
    gcum[i + 1] = gcum[i] + g;
  }
}

double tlqo_cool_exact_T(const tlqo_params* p, const double* gcum, double temp, double lam, double tau) {
  const int n = p->ncool;
  int lo = 1, hi = n; /* first node above temp (n: none), as find_coef */
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (p->coolT[mid] > temp) hi = mid; else lo = mid + 1;
  }
  const int i = lo - 1; /* segment: T_i <= temp < T_{i+1}, n-1 at or above the last node */
  const double a = 1.0 - seg_slope(p, i), xlo = p->coolT[i] / temp;
  const double tau_i = fabs(a) < 1e-9 ? -log(xlo) : (1.0 - pow(xlo, a)) / a;
  if (tau <= tau_i) return temp * pow_inv(1.0 - a * tau, a, -tau);
  const double G = gcum[i] - (tau - tau_i) * temp / lam; /* G(T_new) */
  if (!(G > 0.0)) return p->coolT[0];
  lo = 0;
  hi = i - 1; /* last node j < i with gcum[j] <= G */
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (gcum[mid] <= G) lo = mid; else hi = mid - 1;
  }
  const int j = lo;
  const double aj = 1.0 - seg_slope(p, j), q = (G - gcum[j]) * pow(10.0, p->coolC[j]) / p->coolT[j];
  return p->coolT[j] * pow_inv(1.0 + aj * q, aj, q);
}

/* One cell of apply_cooling (source/cooling.f90:64-117) and, for
 * TLQO_COOL_SUBCYCLE, the sub-cycled integrator built on it: the step is cut
 * into nsub equal sub-steps, nsub = ceil(ce*dt / cool_sub_frac) clamped to
 * [1, cool_max_sub], each applying the reference's exponential factor with
 * its limiter and floor at the current temperature.  nsub = 1 is exactly the
 * reference formula.  TLQO_COOL_EXACT takes the same single step when
 * ce*dt <= cool_sub_frac and the closed form above otherwise. */
static void cool_cell(const tlqo_params* p, const double* gcum, double* w, double* u, double dt) {
  const double g = p->gamma;
  const double Tmin = p->coolT[0];
  double temp = calc_temp(p, w);
  if (!(temp >= Tmin)) return;
  double ETH = w[4] / (g - 1);
  double vel2 = w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
  double EK = 0.5 * w[0] * vel2;
  double aloss = tlqo_cool_coef(p, temp);
  double numdens = w[0] / (p->mu0 * AMU);
  double ce = aloss * (numdens * numdens) / ETH;
  if (p->cooling == TLQO_COOL_EXACT && ce * dt > p->cool_sub_frac) {
    const double Tn = tlqo_cool_exact_T(p, gcum, temp, aloss, ce * dt);
    w[4] = w[4] * (Tn / temp);
    ETH = w[4] / (g - 1);
    u[4] = EK + ETH;
    return;
  }
  int nsub = 1;
  if (p->cooling == TLQO_COOL_SUBCYCLE && ce * dt > p->cool_sub_frac) {
    double q = ceil(ce * dt / p->cool_sub_frac);
    nsub = (q > (double)p->cool_max_sub) ? p->cool_max_sub : (int)q;
    if (nsub < 1) nsub = 1;
  }
  double h = (nsub == 1) ? dt : dt / (double)nsub;
  for (int s = 0; s < nsub; ++s) {
    if (s > 0) {
      temp = calc_temp(p, w);
      if (!(temp >= Tmin)) break;
      ETH = w[4] / (g - 1);
      aloss = tlqo_cool_coef(p, temp);
      ce = aloss * (numdens * numdens) / ETH;
    }
    double cool_factor = exp(-ce * (h));
    if (cool_factor < 1.0 - p->cooling_limit) cool_factor = 1.0 - p->cooling_limit;
    double new_temp = temp * cool_factor;
    int floored = 0;
    if (new_temp < T_FLOOR) {
      cool_factor = T_FLOOR / temp;
      floored = 1;
    }
    w[4] = w[4] * cool_factor;
    if (floored) break;
  }
  ETH = w[4] / (g - 1);
  u[4] = EK + ETH;
}

void tlqo_cooling(const tlqo_params* p, double* W, double* U, double dt) {
  if (p->cooling == TLQO_COOL_NONE || p->ncool < 2) return;
  double* gcum = NULL;
  if (p->cooling == TLQO_COOL_EXACT) {
    gcum = (double*)malloc((size_t)p->ncool * sizeof(double));
    tlqo_cool_gcum(p, gcum);
  }
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i) cool_cell(p, gcum, W + IX(p, 0, i, j, k), U + IX(p, 0, i, j, k), dt);
  free(gcum);
}

/* ---------------------------------------------------------------------------
 * Gravity: pointmass_potential (source/pointsource_gravity.f90:12-39) with the
 * masses given at run time, and S_Solver (source/sources.f90:872-897).
 * ------------------------------------------------------------------------- */
void tlqo_point_potential(const tlqo_params* p, double* phi) {
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 0; k <= p->nz + 1; ++k)
    for (int j = 0; j <= p->ny + 1; ++j)
      for (int i = 0; i <= p->nx + 1; ++i) {
        double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
        double v = phi[PX(p, i, j, k)];
        for (int s = 0; s < p->nmasses; ++s) {
          const double* m = p->masses + 4 * s;
          double r = sqrt((m[0] - x) * (m[0] - x) + (m[1] - y) * (m[1] - y) + (m[2] - z) * (m[2] - z));
          v = v - GR * m[3] / r;
        }
        phi[PX(p, i, j, k)] = v;
      }
}

void tlqo_gravity_source(const tlqo_params* p, const double* W, const double* phi, double* S) {
  const double dx = DX(p), dy = DY(p), dz = DZ(p);
  memset(S, 0, (size_t)tlqo_array_len(p) * sizeof(double));
#pragma omp parallel for collapse(2) num_threads(NTHREADS(p))
  for (int k = 1; k <= p->nz; ++k)
    for (int j = 1; j <= p->ny; ++j)
      for (int i = 1; i <= p->nx; ++i) {
        double fg1 = (phi[PX(p, i + 1, j, k)] - phi[PX(p, i - 1, j, k)]) / (2.0 * dx);
        double fg2 = (phi[PX(p, i, j + 1, k)] - phi[PX(p, i, j - 1, k)]) / (2.0 * dy);
        double fg3 = (phi[PX(p, i, j, k + 1)] - phi[PX(p, i, j, k - 1)]) / (2.0 * dz);
        const double* w = W + IX(p, 0, i, j, k);
        double* s = S + IX(p, 0, i, j, k);
        s[0] = 0.0;
        s[1] = -w[0] * fg1;
        s[2] = -w[0] * fg2;
        s[3] = -w[0] * fg3;
        s[4] = -w[1] * w[0] * fg1 - w[2] * w[0] * fg2 - w[3] * w[0] * fg3;
      }
}

/* ---------------------------------------------------------------------------
 * Self-gravity: MultiGrid (source/sources.f90:99-193) with its restriction,
 * prolongation, residual and smoother (:196-485), and the multipole boundary
 * values (Moments, phi_*boundaries, :599-787).  Meshes are cubes of
 * N = 2^L cells (parameters.f90:22-25, lvlm = size = L), so the coarsest
 * level holds one cell.  Level arrays are (n+2)^3, index (i, j, k) with
 * i in 0..n+1, i fastest -- the layout of the potential phi(0:nx+1, ...).
 *
 * Boundary modes (the reference's two builds, see TLQO_GBC_*): the serial
 * build never sets its neighbour ranks (globals left..back stay 0), so its
 * `left < 0` tests fail and the level-0 ghost values are never imposed; the
 * MPI build on one rank has no neighbours (all < 0) and imposes multipole
 * values every 10 steps, with each moment the single rank's sum (the serial
 * build leaves those sums unassigned, sources.f90:634-641, 667-669).  The
 * two builds also fill the error ghosts of the coarse levels in different
 * statement orders (:262-283 vs :285-290), which the corner values show.
 * ------------------------------------------------------------------------- */
static inline long MG(int n, int i, int j, int k) {
  return (long)i + (long)(n + 2) * ((long)j + (long)(n + 2) * (long)k);
}
static inline long mg_cells(int n) { return (long)(n + 2) * (n + 2) * (long)(n + 2); }

int tlqo_mg_levels(const tlqo_params* p) {
  if (p->nx != p->ny || p->nx != p->nz || p->nx < 1 || (p->nx & (p->nx - 1))) return -1;
  int L = 0;
  while ((1 << L) < p->nx) ++L;
  return L;
}

long tlqo_mg_work_len(const tlqo_params* p) {
  const int L = tlqo_mg_levels(p);
  if (L < 0) return 0;
  long len = 0;
  for (int l = 0; l <= L; ++l) len += 3 * mg_cells(p->nx >> l);
  return len;
}

/* Error, Residue and ret of level l inside the work array. */
static void mg_level(const tlqo_params* p, double* work, int l, double** err, double** res, double** ret) {
  long off = 0;
  for (int q = 0; q < l; ++q) off += 3 * mg_cells(p->nx >> q);
  const long c = mg_cells(p->nx >> l);
  *err = work + off;
  *res = work + off + c;
  *ret = work + off + 2 * c;
}

/* x**n for a run-time integer n as gfortran evaluates it (exponentiation by
 * squaring, the binary method). */
static double powi(double x, int n) {
  unsigned m = n < 0 ? (unsigned)(-n) : (unsigned)n;
  double y = (m % 2) ? x : 1.0;
  while (m >>= 1) {
    x = x * x;
    if (m % 2) y = y * x;
  }
  return n < 0 ? 1.0 / y : y;
}

/* Legendre and aLegendre, sources.f90:9-96 (x**2 as x*x, x**3 as x*x*x,
 * x**4 as (x*x)*(x*x); real exponents through pow). */
static double legendre(double x, int l) {
  const double x2 = x * x;
  switch (l) {
    case 0: return 1.0;
    case 1: return x;
    case 2: return 0.5 * (3.0 * x2 - 1.0);
    case 3: return 0.5 * (5.0 * (x2 * x) - 3.0 * x);
    default: return (1.0 / 8.0) * ((35.0 * (x2 * x2) - 30.0 * x2) + 3.0);
  }
}

static double alegendre(double x, int l, int m) {
  const double x2 = x * x, s = 1.0 - x2;
  switch (l) {
    case 0: return 1.0;
    case 1: return m == 0 ? x : -pow(s, 1.0 / 2.0);
    case 2:
      if (m == 0) return 0.50 * (3.0 * x2 - 1.0);
      if (m == 1) return -(3.0 * x * pow(s, 1.0 / 2.0));
      return 3.0 * s;
    case 3:
      if (m == 0) return 0.50 * (5.0 * (x2 * x) - 3.0 * x);
      if (m == 1) return (3.0 / 2.0) * (1.0 - 5.0 * x2) * pow(s, 1.0 / 2.0);
      if (m == 2) return 15.0 * x * s;
      return -(15.0 * pow(s, 3.0 / 2.0));
    default:
      if (m == 0) return (1.0 / 8.0) * ((35.0 * (x2 * x2) - 30.0 * x2) + 3.0);
      if (m == 1) return -((5.0 / 2.0) * (7.0 * (x2 * x) - 3.0 * x) * pow(s, 1.0 / 2.0));
      if (m == 2) return (15.0 / 2.0) * (7.0 * x2 - 1.0) * s;
      if (m == 3) return -(105.0 * x * pow(s, 3.0 / 2.0));
      return 105.0 * (s * s);
  }
}

/* pangle, aangle, distance (sources.f90:558-596) of a cell centre. */
static void sph_coords(const tlqo_params* p, int i, int j, int k, double* coth, double* fi, double* r) {
  const double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
  const double thet = acos(z / sqrt((x * x + y * y) + z * z));
  double f = atan2(y, x);
  if (f < 0) f = f + 2. * PI_REF;
  *r = sqrt((x * x + y * y) + z * z);
  *coth = cos(thet);
  *fi = f;
}

/* Moments, sources.f90:599-681 (one rank: each moment the rank's sum). */
static void mg_moments(const tlqo_params* p, const double* U, double c0[5], double cm[5][5], double sm[5][5]) {
  const int n = p->nx;
  const double ddx = DX(p), ddy = DY(p), ddz = DZ(p);
  for (int l = 0; l <= 4; ++l) {
    c0[l] = 0.0;
    for (int m = 0; m <= 4; ++m) cm[l][m] = sm[l][m] = 0.0;
  }
  for (int l = 1; l <= 4; ++l) {
    double c0mp = 0.0;
    for (int m = 1; m <= l; ++m) {
      double cmp = 0.0, smp = 0.0;
      c0mp = 0.0;
      const double c = 2.0 * tgamma((double)(l - m) + 1.0) / tgamma((double)(l + m) + 1.0);
      for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j)
          for (int k = 1; k <= n; ++k) {
            double coth, fi, r;
            sph_coords(p, i, j, k, &coth, &fi, &r);
            const double rho = U[IX(p, 0, i, j, k)];
            const double rl = powi(r, l);
            c0mp = c0mp + legendre(coth, l) * rl * rho * ddx * ddy * ddz;
            cmp = cmp + alegendre(coth, l, m) * cos((double)m * fi) * rl * rho * ddx * ddy * ddz;
            smp = smp + alegendre(coth, l, m) * sin((double)m * fi) * rl * rho * ddx * ddy * ddz;
          }
      cm[l][m] = c * cmp;
      sm[l][m] = c * smp;
    }
    c0[l] = c0mp;
  }
  double c0mp = 0.0;
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n; ++j)
      for (int k = 1; k <= n; ++k) {
        double coth, fi, r;
        sph_coords(p, i, j, k, &coth, &fi, &r);
        const double rho = U[IX(p, 0, i, j, k)];
        c0mp = c0mp + legendre(coth, 0) * powi(r, 0) * rho * ddx * ddy * ddz;
      }
  c0[0] = c0mp;
}

/* phi_x/y/zboundaries, sources.f90:683-787: the multipole expansion at the
 * centre of one ghost cell. */
static double multipole_phi(const tlqo_params* p, int i, int j, int k, const double c0[5], double cm[5][5],
                            double sm[5][5]) {
  double coth, fi, rb;
  sph_coords(p, i, j, k, &coth, &fi, &rb);
  double phi = 0.0;
  phi = phi - c0[0] / rb;
  for (int l = 1; l <= 4; ++l) {
    phi = phi - c0[l] * legendre(coth, l) / powi(rb, l + 1);
    for (int m = 1; m <= l; ++m)
      phi = phi - 2.0 * (cm[l][m] * cos((double)m * fi) + sm[l][m] * sin((double)m * fi)) * alegendre(coth, l, m) /
                      powi(rb, l + 1);
  }
  return GR * phi;
}

static void mg_boundaries(const tlqo_params* p, const double* U, double* phi) {
  const int n = p->nx;
  double c0[5], cm[5][5], sm[5][5];
  mg_moments(p, U, c0, cm, sm);
  const int b[2] = {0, n + 1};
  for (int f = 0; f < 2; ++f) /* x faces: j, k */
    for (int j = 1; j <= n; ++j)
      for (int k = 1; k <= n; ++k) phi[MG(n, b[f], j, k)] = multipole_phi(p, b[f], j, k, c0, cm, sm);
  for (int f = 0; f < 2; ++f) /* y faces: i, k */
    for (int i = 1; i <= n; ++i)
      for (int k = 1; k <= n; ++k) phi[MG(n, i, b[f], k)] = multipole_phi(p, i, b[f], k, c0, cm, sm);
  for (int f = 0; f < 2; ++f) /* z faces: i, j */
    for (int i = 1; i <= n; ++i)
      for (int j = 1; j <= n; ++j) phi[MG(n, i, j, b[f])] = multipole_phi(p, i, j, b[f], c0, cm, sm);
}

/* The error's ghost values on a coarse level: var = -(first interior layer)
 * per face, in each build's statement order (sources.f90:262-290). */
static void mg_ghosts(int n, double* v, int bc) {
#define FACE_X(I, SRC) for (int k = 0; k <= n + 1; ++k) for (int j = 0; j <= n + 1; ++j) v[MG(n, I, j, k)] = -v[MG(n, SRC, j, k)]
#define FACE_Y(J, SRC) for (int k = 0; k <= n + 1; ++k) for (int i = 0; i <= n + 1; ++i) v[MG(n, i, J, k)] = -v[MG(n, i, SRC, k)]
#define FACE_Z(K, SRC) for (int j = 0; j <= n + 1; ++j) for (int i = 0; i <= n + 1; ++i) v[MG(n, i, j, K)] = -v[MG(n, i, j, SRC)]
  if (bc == TLQO_GBC_MULTIPOLE) { /* MPI build: x-, x+, y-, y+, z-, z+ */
    FACE_X(0, 1); FACE_X(n + 1, n); FACE_Y(0, 1); FACE_Y(n + 1, n); FACE_Z(0, 1); FACE_Z(n + 1, n);
  } else { /* serial build: x-, y-, z-, x+, y+, z+ */
    FACE_X(0, 1); FACE_Y(0, 1); FACE_Z(0, 1); FACE_X(n + 1, n); FACE_Y(n + 1, n); FACE_Z(n + 1, n);
  }
#undef FACE_X
#undef FACE_Y
#undef FACE_Z
}

/* One smoother update (sources.f90:447-449 and :378-379, w = 1). */
static inline double mg_update(int n, const double* v, const double* src, int i, int j, int k, double dxl) {
  const double w = 1.0;
  double a = v[MG(n, i + 1, j, k)] + v[MG(n, i - 1, j, k)];
  a = a + v[MG(n, i, j + 1, k)];
  a = a + v[MG(n, i, j - 1, k)];
  a = a + v[MG(n, i, j, k + 1)];
  a = a + v[MG(n, i, j, k - 1)];
  a = a - src[MG(n, i, j, k)] * (dxl * dxl);
  return ((1.0 / 6.0) * a) * w + (1.0 - w) * v[MG(n, i, j, k)];
}

/* poisson_solver, sources.f90:218-485 (Solve: Gauss-Seidel in i, j, k order
 * until the summed change is <= 0.001; Relax: it-1 = 5 passes of the two
 * half-sweeps).  Returns Dif. */
static double mg_poisson(const tlqo_params* p, const double* src, double* v, int n, int solve, int level) {
  const double dxl = (p->xr - p->xl) / (double)n;
  double Dif = 0.0;
  if (level > 0) mg_ghosts(n, v, p->grav_bc);
  if (solve) {
    Dif = 1000.0;
    while (Dif > 0.001) {
      double difp = 0.0;
      for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j)
          for (int k = 1; k <= n; ++k) {
            const double d1 = v[MG(n, i, j, k)];
            v[MG(n, i, j, k)] = mg_update(n, v, src, i, j, k, dxl);
            difp = difp + fabs(v[MG(n, i, j, k)] - d1);
          }
      Dif = difp;
    }
    return Dif;
  }
  for (int iter = 1; iter <= 5; ++iter) {
    double difp = 0.0;
    for (int half = 0; half < 2; ++half)
      for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j) {
          /* the reference's test repeats one condition: i even and j odd */
          const int s = (i % 2 == 0) && (j % 2 == 1);
          int start = s ? 1 : 2;
          if (half) start = s ? 2 : 1;
          for (int k = start; k <= n; k += 2) {
            const double d1 = v[MG(n, i, j, k)];
            v[MG(n, i, j, k)] = mg_update(n, v, src, i, j, k, dxl);
            difp = difp + fabs(v[MG(n, i, j, k)] - d1);
          }
        }
    Dif = difp;
  }
  return Dif;
}

/* resid, sources.f90:196-216 (fine level of n cells). */
static void mg_resid(int n, double dxl, const double* v, const double* src, double* res) {
  for (long q = 0; q < mg_cells(n); ++q) res[q] = src[q] - 0.0;
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        double g = v[MG(n, i - 1, j, k)] + v[MG(n, i + 1, j, k)];
        g = g + v[MG(n, i, j - 1, k)];
        g = g + v[MG(n, i, j + 1, k)];
        g = g + v[MG(n, i, j, k - 1)];
        g = g + v[MG(n, i, j, k + 1)];
        g = (g - 6.0 * v[MG(n, i, j, k)]) / (dxl * dxl);
        res[MG(n, i, j, k)] = src[MG(n, i, j, k)] - g;
      }
}

/* restriction, sources.f90:118-137: coarse (nc cells) from fine (2 nc). */
static void mg_restrict(int nc, const double* f, double* c) {
  const int nf = 2 * nc;
  for (int k = 1; k <= nc; ++k)
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        const int i1 = 2 * i - 1, j1 = 2 * j - 1, k1 = 2 * k - 1;
        double a = f[MG(nf, i1, j1, k1)] + f[MG(nf, i1 + 1, j1, k1)];
        a = a + f[MG(nf, i1, j1 + 1, k1)];
        a = a + f[MG(nf, i1, j1, k1 + 1)];
        a = a + f[MG(nf, i1 + 1, j1 + 1, k1)];
        a = a + f[MG(nf, i1 + 1, j1, k1 + 1)];
        a = a + f[MG(nf, i1, j1 + 1, k1 + 1)];
        a = a + f[MG(nf, i1 + 1, j1 + 1, k1 + 1)];
        c[MG(nc, i, j, k)] = (1.0 / 8.0) * a;
      }
}

/* One child of prolongation (sources.f90:139-194): the coarse cell (i,j,k)
 * and its neighbours toward the child, di/dj/dk = -1 or +1. */
static inline double mg_child(int nc, const double* c, int i, int j, int k, int di, int dj, int dk) {
  double a = 27.0 * c[MG(nc, i, j, k)] + 9.0 * c[MG(nc, i + di, j, k)];
  a = a + 9.0 * c[MG(nc, i, j + dj, k)];
  a = a + 9.0 * c[MG(nc, i, j, k + dk)];
  a = a + 3.0 * c[MG(nc, i + di, j + dj, k)];
  a = a + 3.0 * c[MG(nc, i + di, j, k + dk)];
  a = a + 3.0 * c[MG(nc, i, j + dj, k + dk)];
  a = a + c[MG(nc, i + di, j + dj, k + dk)];
  return (1.0 / 64.0) * a;
}

static void mg_prolong(int nc, const double* c, double* f) {
  const int nf = 2 * nc;
  for (long q = 0; q < mg_cells(nf); ++q) f[q] = 0.0;
  for (int k = 1; k <= nc; ++k)
    for (int j = 1; j <= nc; ++j)
      for (int i = 1; i <= nc; ++i) {
        const int i1 = 2 * i - 1, j1 = 2 * j - 1, k1 = 2 * k - 1;
        for (int dk = 0; dk < 2; ++dk)
          for (int dj = 0; dj < 2; ++dj)
            for (int di = 0; di < 2; ++di)
              f[MG(nf, i1 + di, j1 + dj, k1 + dk)] = mg_child(nc, c, i, j, k, di ? 1 : -1, dj ? 1 : -1, dk ? 1 : -1);
      }
}

int tlqo_multigrid(const tlqo_params* p, const double* U, double* phi, int it, double* work) {
  const int L = tlqo_mg_levels(p);
  if (L < 0) return -1;
  const int n = p->nx;
  if (it % 10 == 0 && p->grav_bc == TLQO_GBC_MULTIPOLE) mg_boundaries(p, U, phi);
  double *E0, *R0, *T0;
  mg_level(p, work, 0, &E0, &R0, &T0);
  for (int k = 0; k <= n + 1; ++k)
    for (int j = 0; j <= n + 1; ++j)
      for (int i = 0; i <= n + 1; ++i) R0[MG(n, i, j, k)] = 4.0 * PI_REF * GR * U[IX(p, 0, i, j, k)];
  memcpy(E0, phi, (size_t)mg_cells(n) * sizeof(double));
  double Dif = 1.e28;
  int iter = 0;
  while (Dif > 10.0 && iter < 31) {
    iter = iter + 1;
    for (int lv = 1; lv <= L; ++lv) {
      double *E, *R, *T;
      mg_level(p, work, lv, &E, &R, &T);
      memset(E, 0, (size_t)mg_cells(n >> lv) * sizeof(double));
    }
    Dif = mg_poisson(p, R0, E0, n, 0, 0);
    for (int level = 1; level <= L; ++level) {
      const int nl = n >> level;
      double *Ef, *Rf, *Tf, *E, *R, *T;
      mg_level(p, work, level - 1, &Ef, &Rf, &Tf);
      mg_level(p, work, level, &E, &R, &T);
      mg_resid(2 * nl, (p->xr - p->xl) / (double)(2 * nl), Ef, Rf, Tf);
      mg_restrict(nl, Tf, R);
      Dif = mg_poisson(p, R, E, nl, level == L, level);
    }
    for (int level = L - 1; level >= 0; --level) {
      const int nl = n >> level;
      double *E, *R, *T, *Ec, *Rc, *Tc;
      mg_level(p, work, level, &E, &R, &T);
      mg_level(p, work, level + 1, &Ec, &Rc, &Tc);
      mg_prolong(nl / 2, Ec, T);
      for (long q = 0; q < mg_cells(nl); ++q) E[q] = E[q] + T[q];
      Dif = mg_poisson(p, R, E, nl, 0, level);
    }
  }
  memcpy(phi, E0, (size_t)mg_cells(n) * sizeof(double));
  return iter;
}

/* PHIT = PHIP + PHI (HLLC.f90:22), over the whole (n+2)^3 array. */
static void mg_total(const tlqo_params* p, const tlqo_state* s) {
  const long c = tlqo_phi_len(p);
  for (long q = 0; q < c; ++q) s->PHIT[q] = (s->PHI ? s->PHI[q] : 0.0) + s->PHIG[q];
}

/* ---------------------------------------------------------------------------
 * Main loop, source/mainHD.f90:38-44 and :61-100.
 * ------------------------------------------------------------------------- */
void tlqo_init(const tlqo_params* p, tlqo_state* s) {
  tlqo_borders(p, s->U, 1);
  tlqo_calc_prims(p, s->UPrim, s->U);
  if (p->nmasses > 0 && s->PHI) {
    memset(s->PHI, 0, (size_t)tlqo_phi_len(p) * sizeof(double));
    tlqo_point_potential(p, s->PHI);
  }
  if (p->self_gravity && s->PHIG && s->MGW) { /* mainHD.f90:50-52, it = 0, PHI starting at 0 */
    memset(s->PHIG, 0, (size_t)tlqo_phi_len(p) * sizeof(double));
    tlqo_multigrid(p, s->U, s->PHIG, s->it, s->MGW);
  }
}

/* Godunov's gravity (HLLC.f90:15-24): with self-gravity MultiGrid on the
 * density of U (both stages pass U as UU), PHIT = PHIP + PHI, S from PHIT;
 * with point masses alone S from their potential. */
static void gravity(const tlqo_params* p, tlqo_state* s) {
  if (p->self_gravity) {
    tlqo_multigrid(p, s->U, s->PHIG, s->it, s->MGW);
    mg_total(p, s);
    tlqo_gravity_source(p, s->UPrim, s->PHIT, s->S);
  } else {
    tlqo_gravity_source(p, s->UPrim, s->PHI, s->S);
  }
}

int tlqo_run(const tlqo_params* p, tlqo_state* s, int nsteps, double tfin) {
  const int grav = ((p->nmasses > 0 && s->PHI) || (p->self_gravity && s->PHIG && s->PHIT && s->MGW)) && s->S;
  int n = 0;
  while (n < nsteps && s->t < tfin) {
    s->dt = tlqo_time_step(p, s->UPrim);
    tlqo_fluxes(p, s->U, s->F, s->G, s->H, s->UPrim, 1);
    double dth = s->dt / 2.0;
    if (grav) gravity(p, s);
    tlqo_godunov(p, s->UPP, s->U, s->F, s->G, s->H, dth, grav ? s->S : NULL);
    tlqo_borders(p, s->UPP, 2);
    tlqo_calc_prims(p, s->UPrim, s->UPP);
    tlqo_fluxes(p, s->UPP, s->F, s->G, s->H, s->UPrim, 2);
    if (grav) gravity(p, s);
    tlqo_godunov(p, s->UP, s->U, s->F, s->G, s->H, s->dt, grav ? s->S : NULL);
    tlqo_borders(p, s->UP, 1);
    tlqo_step(p, s->U, s->UP, s->UPP, &s->t, &s->it, s->dt);
    tlqo_calc_prims(p, s->UPrim, s->U);
    if (p->cooling != TLQO_COOL_NONE) tlqo_cooling(p, s->UPrim, s->U, s->dt);
    ++n;
  }
  return n;
}
