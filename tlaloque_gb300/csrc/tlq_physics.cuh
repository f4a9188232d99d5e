// tlq_physics.cuh -- per-cell and per-face arithmetic of tlaloque's step.
//
// Shared by the per-routine kernels (reference layout) and the fused stage
// kernels.  Every expression keeps the reference's evaluation order
// (Fortran left-to-right association); the FP64 translation units are built
// with -fmad=false so that no a*b+c is contracted, which makes the plain FP64
// path bit-identical to the reference arithmetic (IEEE division and square
// root are correctly rounded on the GPU).  Citations: file:line in the
// tlaloque source tree.
#pragma once

#include <cstdint>

namespace tlq {

// source/constants.f90:6-15 (cgs).  PI is the reference's truncated value.
constexpr double AMU = 1.660538782e-24;
constexpr double KB = 1.380650400e-16;
constexpr double GR = 6.67430e-8;
constexpr double PI_REF = 3.14159265358979;
constexpr double T_FLOOR = 10.0;  // source/cooling.f90:56

constexpr int BC_OUTFLOW = 1, BC_REFLECTIVE = 2, BC_PERIODIC = 3, BC_INFLOW = 4;
constexpr int LIM_NONE = 1, LIM_VANLEER = 2, LIM_MINMOD = 3, LIM_UMIST = 4, LIM_WOODWARD = 5,
              LIM_SUPERBEE = 6;
constexpr int SOLVER_HLLC = 0, SOLVER_HLL = 1;
constexpr int COOL_NONE = 0, COOL_REF = 1, COOL_SUBCYCLE = 2, COOL_MLP = 3, COOL_EXACT = 4;

// Fortran MIN/MAX of two reals (no NaN or signed-zero tie matters for valid
// states); SIGN(1.0, a) with gfortran's default signed-zero semantics.
template <class R> __host__ __device__ __forceinline__ R mn(R a, R b) { return (b < a) ? b : a; }
template <class R> __host__ __device__ __forceinline__ R mx(R a, R b) { return (b > a) ? b : a; }
__device__ __forceinline__ double sgn1(double a) { return copysign(1.0, a); }
__device__ __forceinline__ float sgn1(float a) { return copysignf(1.0f, a); }

// One spherical wind (source/winds.f90:5-16) plus the index box of the cells
// it can touch, so that cells far from the source skip the exact test.
struct Wind {
  double xc, yc, zc, vx, vy, vz, radius, mdot, vinf, temp, mu;
  int ilo, ihi, jlo, jhi, klo, khi;
};

// plane_wind_type, source/winds.f90:15-28.
constexpr int MAX_PLANE_WINDS = 6;
struct PlaneWind {
  int plane;  // PLANE_LEFT .. PLANE_TOP = 1..6 (winds.f90:15-20)
  double rho, vel, temp, mu;
};

// Cooling table on the device: T (ascending), log10 T, log10 Lambda, and
// FP32 copies of the three columns for the mixed-precision step.
struct CoolTable {
  const double* T;
  const double* logT;
  const double* C;
  int n;
  const float* Tf;
  const float* logTf;
  const float* Cf;
  // the exact integrator's closed form (COOL_EXACT): per segment the power
  // law's slope (0 above the last node) and at each node G(T_i), the
  // integral of 1/Lambda from the first node; FP64 and FP32 images
  const double* slope;
  const double* gcum;
  const float* slopef;
  const float* gcumf;
  // a table whose nodes are uniform in log10 T (within a third of a step):
  // log10 T_0 and 1/step, from which the FP32 searches guess a cell's
  // segment; dl_inv = 0 for any other table
  float lt0, dl_inv;
};

// Static description of the mesh and the physics switches, passed by value.
struct Params {
  int nx, ny, nz;
  double xl, yl, zl, dx, dy, dz;
  double gamma, g1;  // g1 = gamma/(gamma-1), folded like the reference's constant
  double cfl, eta, mu0, cooling_limit, cool_sub_frac;
  int limiter, solver, cooling, cool_max_sub;
  int bc[6];
  int nwinds;
  const Wind* winds;
  int nplanes;
  PlaneWind planes[MAX_PLANE_WINDS];
  CoolTable cool;
  int gravity;        // point-mass source term on
  // FP32 images of per-run constants for the mixed-precision kernels, formed
  // on the host once (an FP64 division or double->float conversion costs
  // ~64 FP32 slots on GB300, and every thread of every tile would repeat it)
  float f_gamma, f_g1, f_eta;
  float f_inv_dx, f_inv_dy, f_inv_dz;  // 1/dx ...
  float f_hdx, f_hdy, f_hdz;           // 0.5/dx ... (gravity's central differences)
  float f_cT;                          // mu0 AMU / KB: T = (p/rho) f_cT
  float f_inv_muamu;                   // 1/(mu0 AMU): n = rho f_inv_muamu
  float f_cool_sub_frac, f_cooling_limit;
  float f_mlp_tol;  // the surrogate's residual tolerance
  // the cooling switch near the table's first temperature T_0, decided in
  // FP64 without divisions: (gamma-1) mu0 AMU and T_0 KB (tlq_stage_mixed.cuh)
  double c_edge_p, c_edge_rho;
};

// ---------------------------------------------------------------------------
// Coordinates, source/HydroCore.f90:35-77 (one rank: coords = 0).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double xcoord(const Params& p, int i) { return (p.xl + p.dx * (double)i) - p.dx / 2.0; }
__device__ __forceinline__ double ycoord(const Params& p, int j) { return (p.yl + p.dy * (double)j) - p.dy / 2.0; }
__device__ __forceinline__ double zcoord(const Params& p, int k) { return (p.zl + p.dz * (double)k) - p.dz / 2.0; }

// ---------------------------------------------------------------------------
// calc_prims for one cell, source/HydroCore.f90:14-21.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void cons2prim(R g, const R* u, R* w) {
  w[0] = u[0];
  w[1] = u[1] / u[0];
  w[2] = u[2] / u[0];
  w[3] = u[3] / u[0];
  w[4] = (g - R(1.0)) * (u[4] - R(0.5) * ((u[1] * u[1] + u[2] * u[2]) + u[3] * u[3]) / u[0]);
  w[4] = mx(w[4], R(1e-20));
}

// csound, source/HydroCore.f90:157-168.
template <class R> __device__ __forceinline__ R csound(R g, R pres, R den) { return sqrt(g * pres / den); }

// ---------------------------------------------------------------------------
// limiter / average, source/HLLC.f90:560-638 (HLL.f90:319-397 is identical).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R average(R a, R b, int opt) {
  R s, c, d, r;
  switch (opt) {
    case LIM_NONE:
      return R(0.5) * (a + b);
    case LIM_VANLEER:
      if constexpr (sizeof(R) == 4) {
        // FP32 (mixed form): products of two differences underflow FP32
        // for cgs-scale densities (|drho| ~ 1e-25 g/cm^3 squared is below
        // FLT_MIN), so a and b are first scaled by the power of two 2^-E
        // that brings the larger magnitude to [1, 2) (E from its exponent
        // bits; both scalings exact).  The limiter is homogeneous of degree
        // 1: the scaled result times 2^E.  The scaled denominator lies in
        // [1, 8], within the fast division's range.
        const unsigned eb = __float_as_uint(fmaxf(fabsf(a), fabsf(b))) & 0x7f800000u;
        const float s = __uint_as_float(0x7f000000u - eb);
        const float x = a * s, y = b * s, xy = x * y;
        if (!(xy > 0.0f)) return R(0.0);
        return __fdividef(xy * (x + y), fmaf(x, x, y * y)) * __uint_as_float(eb);
      } else {
        if (a * b <= R(0.0)) return R(0.0);
        return a * b * (a + b) / (a * a + b * b);
      }
    case LIM_MINMOD:
      s = sgn1(a);
      return s * mx(R(0.0), mn(fabs(a), s * b));
    case LIM_UMIST:
      s = sgn1(a);
      c = R(0.25) * a + R(0.75) * b;
      d = R(0.75) * a + R(0.25) * b;
      r = mn(mn(mn(R(2.0) * fabs(a), R(2.0) * s * b), s * c), s * d);
      return s * mx(R(0.0), r);
    case LIM_WOODWARD:
      s = sgn1(a);
      c = R(0.5) * (a + b);
      r = mn(mn(R(2.0) * fabs(a), R(2.0) * s * b), s * c);
      return s * mx(R(0.0), r);
    default:  // LIM_SUPERBEE (the configuration is validated on the host)
      s = sgn1(b);
      c = mn(R(2.0) * fabs(b), s * a);
      d = mn(fabs(b), R(2.0) * s * a);
      return s * mx(mx(R(0.0), c), d);
  }
}

// Reconstruct the left/right states of one face in place (HLLC.f90:574-583).
template <class R>
__device__ __forceinline__ void limiter(const R* pll, R* pl, R* pr, const R* prr, int lim) {
#pragma unroll
  for (int e = 0; e < 5; ++e) {
    R dl = pl[e] - pll[e];
    R dm = pr[e] - pl[e];
    R dr = prr[e] - pr[e];
    R al = average(dl, dm, lim);
    R ar = average(dm, dr, lim);
    pl[e] = pl[e] + R(0.5) * al;
    pr[e] = pr[e] - R(0.5) * ar;
  }
}

// Select component d (1..3) of a primitive vector without local memory.
template <class R> __device__ __forceinline__ R comp(const R* w, int d) { return d == 1 ? w[1] : (d == 2 ? w[2] : w[3]); }

// prim2f, source/HydroCore.f90:213-251, for a runtime direction d.  The
// tangential momentum fluxes are (rho*u_lo)*u_hi with lo < hi the two
// component indices, exactly as the reference writes each case.
template <class R>
__device__ __forceinline__ void prim2f(R g1, R* ff, const R* w, int d) {
  const R un = comp(w, d);
  const R mn_ = w[0] * un;
  ff[0] = mn_;
#pragma unroll
  for (int e = 1; e <= 3; ++e) {
    const R lo = (e < d) ? w[e] : un;
    const R hi = (e < d) ? un : w[e];
    const R t = w[0] * lo * hi;
    ff[e] = (e == d) ? t + w[4] : t;
  }
  ff[4] = un * (R(0.5) * w[0] * ((w[1] * w[1] + w[2] * w[2]) + w[3] * w[3]) + g1 * w[4]);
}

// ---------------------------------------------------------------------------
// Riemann flux at one face in direction d (1..3).
//   HLLC: HLLCFluxes branches (source/HLLC.f90:99-136, :139-176, :179-216)
//         with wavespeed (:498-518).
//   HLL:  HLLFluxes branches (source/HLL.f90:106-129) with wavespeed (:299-317).
// UL, UR are the cell-centred conserved states of the two cells; the HLLC
// star state and the HLL average use them even when wl, wr are
// reconstructed (the reference's choice).  Returns false when the wave
// speeds are NaN (no branch taken; the reference then leaves the flux as it
// was, here the caller keeps its previous value).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ bool riemann(int solver, R g, R g1, R* ff, const R* wl, const R* wr, const R* UL,
                                        const R* UR, int d) {
  const R ul = comp(wl, d), ur = comp(wr, d);
  const R csl = csound(g, wl[4], wl[0]);
  const R csr = csound(g, wr[4], wr[0]);
  const R sl = mn(ul - csl, ur - csr);
  const R sr = mx(ul + csl, ur + csr);
  if (solver == SOLVER_HLL) {
    if (sl >= R(0)) {
      prim2f(g1, ff, wl, d);
    } else if (sr <= R(0)) {
      prim2f(g1, ff, wr, d);
    } else {
      R fl[5], fr[5];
      prim2f(g1, fl, wl, d);
      prim2f(g1, fr, wr, d);
#pragma unroll
      for (int e = 0; e < 5; ++e) ff[e] = (sr * fl[e] - sl * fr[e] + sl * sr * (UR[e] - UL[e])) / (sr - sl);
    }
    return true;  // NaN speeds take the HLL average branch, as in the reference
  }
  const R sst = (wr[4] - wl[4] + wl[0] * ul * (sl - ul) - wr[0] * ur * (sr - ur)) /
                (wl[0] * (sl - ul) - wr[0] * (sr - ur));
  // Branch order of the reference: sl>=0, sr<=0, sst>=0, sst<=0.  The two
  // star branches share one code path on the selected side.
  bool star, left;
  if (sl >= R(0)) { star = false; left = true; }
  else if (sr <= R(0)) { star = false; left = false; }
  else if (sst >= R(0)) { star = true; left = true; }
  else if (sst <= R(0)) { star = true; left = false; }
  else return false;
  // element-wise selects (a pointer to one of two register arrays would
  // force both into local memory)
  R w[5], uc[5];
#pragma unroll
  for (int e = 0; e < 5; ++e) {
    w[e] = left ? wl[e] : wr[e];
    uc[e] = left ? UL[e] : UR[e];
  }
  prim2f(g1, ff, w, d);
  if (star) {
    const R s = left ? sl : sr;
    const R un = left ? ul : ur;
    const R a = w[0] * (s - un);
    const R rhostr = a / (s - sst);
    R us[5];
    us[0] = rhostr;
#pragma unroll
    for (int e = 1; e <= 3; ++e) us[e] = (e == d) ? rhostr * sst : rhostr * w[e];
    us[4] = rhostr * (uc[4] / w[0] + (sst - un) * (sst + w[4] / a));
#pragma unroll
    for (int e = 0; e < 5; ++e) ff[e] = ff[e] + s * (us[e] - uc[e]);
  }
  return true;
}

// ---------------------------------------------------------------------------
// imposeSphericalWind for one cell, source/winds.f90:55-87.  Returns true and
// writes the conserved wind state when the cell centre lies inside.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool wind_cell(const Params& p, const Wind& w, int i, int j, int k, double* u) {
  if (i < w.ilo || i > w.ihi || j < w.jlo || j > w.jhi || k < w.klo || k > w.khi) return false;
  const double x = xcoord(p, i), y = ycoord(p, j), z = zcoord(p, k);
  const double dist = sqrt((x - w.xc) * (x - w.xc) + (y - w.yc) * (y - w.yc) + (z - w.zc) * (z - w.zc));
  if (!(dist < w.radius)) return false;
  const double dens = w.mdot / (w.vinf * dist * dist * 4.0 * PI_REF);
  const double vx = w.vinf * (x - w.xc) / dist + w.vx;
  const double vy = w.vinf * (y - w.yc) / dist + w.vy;
  const double vz = w.vinf * (z - w.zc) / dist + w.vz;
  const double pres = dens * KB * w.temp / (w.mu * AMU);
  u[0] = dens;
  u[1] = dens * vx;
  u[2] = dens * vy;
  u[3] = dens * vz;
  u[4] = 0.5 * dens * ((vx * vx + vy * vy) + vz * vz) + pres / (p.gamma - 1.0);
  return true;
}

// All winds in order (user/user.f90:64-68): later winds override earlier ones.
// imposePlaneWind, source/winds.f90:92-147: every i, j and k = nz..nz+2
// (the reference's loop writes the top three z-planes whatever the plane),
// the velocity along the plane's normal.
__device__ __forceinline__ void plane_wind_cell(const Params& p, const PlaneWind& w, int k, double* u) {
  if (k < p.nz) return;
  double vx = 0.0, vy = 0.0, vz = 0.0;
  switch (w.plane) {
    case 1: vx = w.vel; break;
    case 2: vx = -w.vel; break;
    case 3: vy = w.vel; break;
    case 4: vy = -w.vel; break;
    case 5: vz = w.vel; break;
    case 6: vz = -w.vel; break;
    default: break;
  }
  const double pres = w.rho / (w.mu * AMU) * KB * w.temp;
  u[0] = w.rho;
  u[1] = w.rho * vx;
  u[2] = w.rho * vy;
  u[3] = w.rho * vz;
  u[4] = 0.5 * w.rho * ((vx * vx + vy * vy) + vz * vz) + pres / (p.gamma - 1.0);
}

// Whether a cell may write ghost images (within two cells of a face) or lie
// in a spherical wind's index box or a plane wind's planes.
__device__ __forceinline__ bool near_boundary_or_wind(const Params& p, int i, int j, int k) {
  if (i <= 2 || j <= 2 || k <= 2 || i >= p.nx - 1 || j >= p.ny - 1 || k >= p.nz - 1) return true;
  if (p.nplanes > 0 && k >= p.nz) return true;
  for (int s = 0; s < p.nwinds; ++s) {
    const Wind& w = p.winds[s];
    if (i >= w.ilo && i <= w.ihi && j >= w.jlo && j <= w.jhi && k >= w.klo && k <= w.khi) return true;
  }
  return false;
}

// near_boundary_or_wind ruled out for whole planes of a tile (columns
// i0..i1 x j0..j1): `ij` when some column lies within two cells of an x or y
// face, and the z range [klo, khi] of the spherical winds whose index boxes
// meet the tile's columns.  Formed once per tile (the winds' boxes are read
// from memory there, not per cell); plane k of the tile may hold a cell for
// which near_boundary_or_wind is true only if may_be_special(k).
struct TileSpecial {
  bool ij;
  int klo, khi;
  __device__ __forceinline__ bool may_be_special(const Params& p, int k) const {
    return ij || k <= 2 || k >= p.nz - 1 || (p.nplanes > 0 && k >= p.nz) || (k >= klo && k <= khi);
  }
};
__device__ __forceinline__ TileSpecial tile_special(const Params& p, int i0, int i1, int j0, int j1) {
  TileSpecial t;
  t.ij = i0 <= 2 || j0 <= 2 || i1 >= p.nx - 1 || j1 >= p.ny - 1;
  t.klo = 1 << 30;
  t.khi = -(1 << 30);
  for (int s = 0; s < p.nwinds; ++s) {
    const Wind& w = p.winds[s];
    if (i1 >= w.ilo && i0 <= w.ihi && j1 >= w.jlo && j0 <= w.jhi) {
      t.klo = min(t.klo, w.klo);
      t.khi = max(t.khi, w.khi);
    }
  }
  return t;
}

// user_boundaries: the spherical winds, then the plane winds.
__device__ __forceinline__ void winds_cell(const Params& p, int i, int j, int k, double* u) {
  for (int s = 0; s < p.nwinds; ++s) wind_cell(p, p.winds[s], i, j, k, u);
  for (int s = 0; s < p.nplanes; ++s) plane_wind_cell(p, p.planes[s], k, u);
}

// ---------------------------------------------------------------------------
// Cooling, source/cooling.f90:64-159.
// ---------------------------------------------------------------------------
// find_coef (:121-144): first entry with T_i > temp (a lower-bound search
// returns the same index as the reference's linear scan on an ascending
// table); held at the last entry above the table (undefined there in the
// reference).
__device__ __forceinline__ double cool_coef(const CoolTable& t, double temp) {
  int lo = 1, hi = t.n;  // search i in [1, n-1] (0-based) with T[i] > temp
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (t.T[mid] > temp) hi = mid; else lo = mid + 1;
  }
  if (lo >= t.n) return pow(10.0, t.C[t.n - 1]);
  const double T0 = t.logT[lo - 1], C0 = t.C[lo - 1];
  const double T1 = t.logT[lo], C1 = t.C[lo];
  return pow(10.0, (C1 - C0) / (T1 - T0) * (log10(temp) - T0) + C0);
}

// The exact integrator (COOL_EXACT): the temperature after a step of
// cooling number tau (= ce dt, ce = Lambda n^2 / E_th at temp) of a cell at
// temp >= T_0 whose find_coef value is lam.  At fixed density the
// sub-cycled integrator's equation, d ln T/dt = -ce(T), becomes
// dT/dt = -kappa Lambda(T) in its limit of infinitely many sub-steps, and
// find_coef's log-linear interpolation makes Lambda a power law on each
// table segment (held constant above the table), so the step integrates in
// closed form (exact integration of a piecewise power-law cooling function,
// Townsend 2009, ApJS 181, 391).  With a = 1 - slope of temp's segment i,
// the cell stays in it while tau <= (1 - (T_i/temp)^a)/a and ends at
// temp (1 - a tau)^(1/a); otherwise it reaches T_i with a budget
// B = (tau - tau_i) temp/lam of G left, G(T_new) = G(T_i) - B, found in the
// segment j whose nodes bracket it.  Nothing cools below T_0: a cell that
// reaches it ends there.
__device__ __forceinline__ double cool_exact_T(const CoolTable& t, double temp, double lam, double tau) {
  int lo = 1, hi = t.n;  // first node above temp (n: none), as find_coef
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t.T[mid] > temp) hi = mid; else lo = mid + 1;
  }
  const int i = lo - 1;
  const double a = 1.0 - t.slope[i], xlo = t.T[i] / temp;
  const double tau_i = fabs(a) < 1e-9 ? -log(xlo) : (1.0 - pow(xlo, a)) / a;
  if (tau <= tau_i) return temp * (fabs(a) < 1e-9 ? exp(-tau) : pow(1.0 - a * tau, 1.0 / a));
  const double G = t.gcum[i] - (tau - tau_i) * temp / lam;
  if (!(G > 0.0)) return t.T[0];
  lo = 0;
  hi = i - 1;  // last node j < i with G(T_j) <= G
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.gcum[mid] <= G) lo = mid; else hi = mid - 1;
  }
  const double aj = 1.0 - t.slope[lo], q = (G - t.gcum[lo]) * pow(10.0, t.C[lo]) / t.T[lo];
  return t.T[lo] * (fabs(aj) < 1e-9 ? exp(q) : pow(1.0 + aj * q, 1.0 / aj));
}

// apply_cooling for one interior cell (:68-112), and the sub-cycled
// integrator built on it (nsub equal sub-steps; nsub = 1 is the reference
// formula); COOL_EXACT takes the same single step when ce dt <= cool_sub_frac
// and the closed form above otherwise.  w is the primitive state (w[4]
// updated), u4 the total energy.
__device__ __forceinline__ void cool_cell(const Params& p, double* w, double& u4, double dt) {
  const double g = p.gamma;
  const double Tmin = p.cool.T[0];
  double temp = w[4] * p.mu0 * AMU / (w[0] * KB);
  if (!(temp >= Tmin)) return;
  double ETH = w[4] / (g - 1.0);
  const double vel2 = w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
  const double EK = 0.5 * w[0] * vel2;
  double aloss = cool_coef(p.cool, temp);
  const double numdens = w[0] / (p.mu0 * AMU);
  double ce = aloss * (numdens * numdens) / ETH;
  if (p.cooling == COOL_EXACT && ce * dt > p.cool_sub_frac) {
    const double Tn = cool_exact_T(p.cool, temp, aloss, ce * dt);
    w[4] = w[4] * (Tn / temp);
    ETH = w[4] / (g - 1.0);
    u4 = EK + ETH;
    return;
  }
  int nsub = 1;
  if (p.cooling == COOL_SUBCYCLE && ce * dt > p.cool_sub_frac) {
    const double q = ceil(ce * dt / p.cool_sub_frac);
    nsub = (q > (double)p.cool_max_sub) ? p.cool_max_sub : (int)q;
    if (nsub < 1) nsub = 1;
  }
  const double h = (nsub == 1) ? dt : dt / (double)nsub;
  for (int s = 0; s < nsub; ++s) {
    if (s > 0) {
      temp = w[4] * p.mu0 * AMU / (w[0] * KB);
      if (!(temp >= Tmin)) break;
      ETH = w[4] / (g - 1.0);
      aloss = cool_coef(p.cool, temp);
      ce = aloss * (numdens * numdens) / ETH;
    }
    double cool_factor = exp(-ce * (h));
    if (cool_factor < 1.0 - p.cooling_limit) cool_factor = 1.0 - p.cooling_limit;
    const double new_temp = temp * cool_factor;
    bool floored = false;
    if (new_temp < T_FLOOR) {
      cool_factor = T_FLOOR / temp;
      floored = true;
    }
    w[4] = w[4] * cool_factor;
    if (floored) break;
  }
  ETH = w[4] / (g - 1.0);
  u4 = EK + ETH;
}

// S_Solver for one interior cell, source/sources.f90:885-893.  f1..f3 are the
// centred potential differences phi(+1) - phi(-1) per axis.
__device__ __forceinline__ void gravity_cell(const Params& p, const double* w, double dpx, double dpy, double dpz,
                                             double* s) {
  const double fg1 = dpx / (2.0 * p.dx);
  const double fg2 = dpy / (2.0 * p.dy);
  const double fg3 = dpz / (2.0 * p.dz);
  s[0] = 0.0;
  s[1] = -w[0] * fg1;
  s[2] = -w[0] * fg2;
  s[3] = -w[0] * fg3;
  s[4] = -w[1] * w[0] * fg1 - w[2] * w[0] * fg2 - w[3] * w[0] * fg3;
}

// Per-cell CFL signal speeds of time_step (source/HydroCore.f90:138-143).
__device__ __forceinline__ void signal_speeds(double g, const double* w, double* v3) {
  const double cs = csound(g, w[4], w[0]);
  v3[0] = fabs(w[1]) + cs;
  v3[1] = fabs(w[2]) + cs;
  v3[2] = fabs(w[3]) + cs;
}

// NaN-propagating maximum for the CFL reduction (a NaN speed must surface as
// a non-finite dt instead of being dropped).
__device__ __forceinline__ double max_nan(double a, double b) { return (a != a || a > b) ? a : b; }

// dt from the three maxima, source/HydroCore.f90:144.
__host__ __device__ __forceinline__ double cfl_dt(double cfl, double dx, double dy, double dz, double mvx, double mvy,
                                                  double mvz) {
  const double m = mn(mn(dx / mvx, dy / mvy), dz / mvz);
  return cfl * m / sqrt(3.0);
}

}  // namespace tlq
