// tlq_stage_mixed.cuh -- the mixed-precision form of the two stage kernels.
//
// Same step and same fusion as tlq_stage.cuh, with a different split of the
// arithmetic, chosen for GB300 (FP64 at 1/64 of the FP32 rate):
//   FP32  primitives, limiter reconstruction, HLL/HLLC fluxes, flux
//         divergence, gravity source, viscosity Laplacian, cooling, signal
//         speeds;
//   FP64  the state in HBM, the conserved-variable accumulation
//         U + dU, the pressure of cells with kinetic/total energy > 0.99,
//         winds and ghost images, the CFL reduction across blocks and dt.
// Conversions between the two go through the integer pipe (tlq_convert.cuh).
// The state stays FP64 in HBM (same layout, same tensor maps), so the two
// forms share every other kernel and the host code.
#pragma once

#include "tlq_convert.cuh"
#include "tlq_stage.cuh"

namespace tlq {

// Geometry of the planes a stage stages in shared memory (x fastest, tile
// cell (tx, ty) at (OY + ty, 2 + tx)).  Stage 1 (first-order fluxes of U and
// the viscosity Laplacian of U) needs a 1-cell halo; its box is 2 cells wide
// in x all the same (a TMA box of FP64 values starts on a 16-byte boundary,
// an even cell index) and 1 cell high in y.  Stage 2 (second-order fluxes of
// UPP) needs 2 cells on each side.
template <int S>
struct MGeo {
  static constexpr int OY = (S == 1) ? 1 : 2;
  static constexpr int PX = MTX + 4, PY = MTY + 2 * OY, PB = PX * PY;
};

// One plane of FP32 values (5 variables), 128-byte aligned: the TMA writes
// stage 2's planes straight into these.
template <int S>
struct alignas(128) PlaneF {
  float v[5][MGeo<S>::PY][MGeo<S>::PX];
};

// Blocks per SM each stage is built for (registers per thread <= 65536 /
// (blocks x MNT)); the shared memory of both fits 5 blocks of 128 threads.
#ifndef TLQ_MB1
#define TLQ_MB1 5
#endif
#ifndef TLQ_MB2
#define TLQ_MB2 5
#endif
template <int S>
struct MixedBlocks {
  static constexpr int value = (S == 1) ? TLQ_MB1 : TLQ_MB2;
};

// Stage 1: U arrives in FP64 (one TMA landing slot; the next plane is
// requested as soon as this one is converted, a whole plane's work ahead of
// its use), converted per plane to FP32 conserved values (4-plane ring: the
// Laplacian of plane k reads k-1..k+1, and plane k+2's conversion may run
// beside it) and primitives (2-plane ring: the faces of plane k read k and
// k+1).
struct MixedSmem1 {
  double raw[5 * MGeo<1>::PB];
  PlaneF<1> cu[4];
  PlaneF<1> prm[2];
  float fx[5][MTY][MTX + 1];
  float fy[5][MTY + 1][MTX];
  float fz[2][5][MTY][MTX];
  uint64_t bar[1];
  double red[96];
  int flag;
  int abort;
};
// Stage 2: UPP's FP32 primitives land by TMA in a 4-plane ring (the faces of
// plane k read k-1..k+2; plane k+3 is requested into k-1's slot once those
// faces are done).  Each thread's cell operands of the plane (the old U, the
// viscosity term, the potential's six neighbours) are copied from HBM into
// its own slots before the face phase and read after it.
struct MixedSmem2 {
  PlaneF<2> prm[4];
  double uop[5][MNT];
  float lvp[5][MNT];
  float php[6][MNT];
  float fx[5][MTY][MTX + 1];
  float fy[5][MTY + 1][MTX];
  float fz[2][5][MTY][MTX];
  uint64_t bar[4];
  double red[96];
  TileSpecial tspec;  // the tile's boundary/wind pre-test (block-uniform)
  int flag;
  int abort;
};
template <int S>
struct MixedSmemSel;
template <>
struct MixedSmemSel<1> {
  using type = MixedSmem1;
  static constexpr int nbar = 1;
};
template <>
struct MixedSmemSel<2> {
  using type = MixedSmem2;
  static constexpr int nbar = 4;
};
template <int S>
using MixedSmem = typename MixedSmemSel<S>::type;


// One cell: FP64 conserved (stride vs) -> FP32 conserved and primitives.
// The pressure of a cell whose kinetic energy exceeds 0.99 of its total
// energy is recovered in FP64 (FP32 would lose it to cancellation).  The
// sums are written with explicit-rounding intrinsics, so the compiler cannot
// contract them differently in the kernels that inline this (the stages,
// the surrogate's passes): every kernel gets the same bits for a cell.
__device__ __forceinline__ void mixed_cell(float gm1, const double* u, long long vs, float* cf, float* w) {
#pragma unroll
  for (int e = 0; e < 5; ++e) cf[e] = d2f(u[e * vs]);
  const float inv = 1.0f / cf[0];
  w[0] = cf[0];
  w[1] = cf[1] * inv;
  w[2] = cf[2] * inv;
  w[3] = cf[3] * inv;
  const float ek =
      __fmul_rn(0.5f, __fmaf_rn(cf[3], w[3], __fmaf_rn(cf[2], w[2], __fmul_rn(cf[1], w[1]))));
  const bool kin = ek > __fmul_rn(0.99f, cf[4]);
  float p = __fmul_rn(gm1, __fsub_rn(cf[4], ek));
  // a branch the whole warp skips unless one of its cells needs FP64 (the
  // FP64 division would otherwise be evaluated for every cell)
  if (__any_sync(__activemask(), kin)) {
    if (kin) {
      const double r = u[0], m1 = u[vs], m2 = u[2 * vs], m3 = u[3 * vs], E = u[4 * vs];
      const double k2 = __fma_rn(m3, m3, __fma_rn(m2, m2, __dmul_rn(m1, m1)));
      p = d2f(__dmul_rn((double)gm1, __dsub_rn(E, __ddiv_rn(__dmul_rn(0.5, k2), r))));
    }
  }
  w[4] = fmaxf(p, 1e-20f);
}

// Cooling in FP32 (the mixed form's cooling source; same algorithm as
// cool_cell: the reference's exponential factor, its limiter and floor,
// sub-cycled when asked).  The total energy changes by the thermal energy
// removed, accumulated in FP64.
// lo: the table entry the search returns (the first with T > temp, n above
// the table), kept from the previous call as the first guess: a sub-cycled
// cell's temperature moves little between sub-steps, and when the guess is
// still the first entry above temp (the entry below it is not) the search is
// skipped and the result is the same.
// The first table node above temp (1..n-1; n above the table), as find_coef
// picks it: on a table uniform in log10 T (t.dl_inv > 0) from a guess at the
// segment from lt = log10 T, moved to the node that satisfies the search's
// condition (the guess decides only how many loads that takes: one or two
// instead of a binary search's chain of eight dependent ones); otherwise a
// binary search.
__device__ __forceinline__ int first_above_f(const CoolTable& t, float temp, float lt) {
  int lo;
  if (t.dl_inv > 0.0f) {
    const float x = fminf(fmaxf(__fmul_rn(__fsub_rn(lt, t.lt0), t.dl_inv), 0.0f), (float)(t.n - 1));
    lo = 1 + (int)x;
    while (lo > 1 && t.Tf[lo - 1] > temp) --lo;
    while (lo < t.n && !(t.Tf[lo] > temp)) ++lo;
  } else {
    lo = 1;
    int hi = t.n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t.Tf[mid] > temp) hi = mid; else lo = mid + 1;
    }
  }
  return lo;
}

__device__ __forceinline__ float cool_coef_seg(const CoolTable& t, float temp, int& lo) {
  const float lt = log10f(temp);
  const bool same = lo >= 1 && lo <= t.n && !(t.Tf[lo - 1] > temp) && (lo == t.n || t.Tf[lo] > temp);
  if (!same) lo = first_above_f(t, temp, lt);
  if (lo >= t.n) return exp10f(t.Cf[t.n - 1]);
  const float T0 = t.logTf[lo - 1], C0 = t.Cf[lo - 1];
  const float T1 = t.logTf[lo], C1 = t.Cf[lo];
  return exp10f(__fmaf_rn((C1 - C0) / (T1 - T0), __fsub_rn(lt, T0), C0));
}

__device__ __forceinline__ float cool_coef_f(const CoolTable& t, float temp) {
  int lo = 0;
  return cool_coef_seg(t, temp, lo);
}

// Whether cooling applies (temp >= the table's first temperature T_0,
// cooling.f90:71).  The switch is a jump in the source term; a cell whose
// FP32 temperature falls within 1e-6 of the edge (e.g. a medium initialised
// at the table's lower edge) decides it from the FP64 state, to FP64
// accuracy, so both forms agree: with temp = p mu0 AMU / (rho KB) and
// p = (gamma-1) (E - k2/(2 rho)), temp >= T_0 is
// (gamma-1) mu0 AMU (E rho - k2/2) >= T_0 KB rho^2 for rho > 0 -- no FP64
// division (each costs ~8 FMA slots of GB300's FP64 pipe), and the warp
// takes the branch only when one of its cells is that close to the edge.
__device__ __forceinline__ bool cools_at(const Params& p, float temp, const double* u) {
  const float Tmin = p.cool.Tf[0];
  const bool near = !(fabsf(__fsub_rn(temp, Tmin)) > 1e-6f * Tmin);
  bool yes = temp >= Tmin;
  if (__any_sync(__activemask(), near)) {
    if (near) {
      const double r = u[0];
      const double k2 = __fma_rn(u[3], u[3], __fma_rn(u[2], u[2], __dmul_rn(u[1], u[1])));
      const double lhs = __dmul_rn(p.c_edge_p, __fma_rn(u[4], r, __dmul_rn(-0.5, k2)));
      yes = lhs >= __dmul_rn(p.c_edge_rho, __dmul_rn(r, r));
    }
  }
  return yes;
}

// The exact integrator (COOL_EXACT) in FP32: the same closed form as
// cool_exact_T (tlq_physics.cuh), returning the fractional temperature
// change T_new/temp - 1 (in [T_0/temp - 1, 0]).  The change is formed with
// log1pf/expm1f, which keep their full accuracy under --use_fast_math: with
// tau just above the single-step limit the change is ~1e-3 of T, and a
// power or exponential rounded near 1 would carry ~1e-4 of it.  Sums that
// meet products use explicit-rounding intrinsics (one contraction choice in
// every kernel that inlines this).
__device__ __forceinline__ float cool_exact_dropf(const CoolTable& t, float temp, float lam, float tau) {
  int lo = first_above_f(t, temp, log10f(temp));  // first node above temp (n: none), as find_coef
  int hi;
  const int i = lo - 1;
  const float a = __fsub_rn(1.0f, t.slopef[i]);
  const float lxlo = logf(t.Tf[i] / temp);  // <= 0
  const bool flat = fabsf(a) < 1e-6f;
  const float tau_i = flat ? -lxlo : -expm1f(__fmul_rn(a, lxlo)) / a;
  if (tau <= tau_i) return flat ? expm1f(-tau) : expm1f(log1pf(-__fmul_rn(a, tau)) / a);
  const float G = __fsub_rn(t.gcumf[i], __fmul_rn(__fsub_rn(tau, tau_i), temp) / lam);
  if (!(G > 0.0f)) return __fsub_rn(t.Tf[0] / temp, 1.0f);
  lo = 0;
  hi = i - 1;  // last node j < i with G(T_j) <= G
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.gcumf[mid] <= G) lo = mid; else hi = mid - 1;
  }
  const float aj = __fsub_rn(1.0f, t.slopef[lo]);
  const float q = __fmul_rn(__fsub_rn(G, t.gcumf[lo]), exp10f(t.Cf[lo])) / t.Tf[lo];
  const float lj = logf(t.Tf[lo] / temp);
  const float r = fabsf(aj) < 1e-6f ? q : log1pf(__fmul_rn(aj, q)) / aj;  // ln(T_new/T_j)
  return fmaxf(expm1f(__fadd_rn(lj, r)), __fsub_rn(t.Tf[0] / temp, 1.0f));
}

// Whether cool_exact_dropf takes a cell of the table's first segment
// (the search's first node above temp is node 1) to the table's first
// temperature: tau beyond the segment's own cooling time, with nothing of
// the table below it (G(T_0) = 0).  The same FP32 operations as that
// function's test, so a cell this accepts gets the bits it would give.
__device__ __forceinline__ bool cool_floors_first(const CoolTable& t, float temp, float lam, float tau) {
  const float a = __fsub_rn(1.0f, t.slopef[0]);
  const float lxlo = logf(t.Tf[0] / temp);
  const bool flat = fabsf(a) < 1e-6f;
  const float tau_i = flat ? -lxlo : -expm1f(__fmul_rn(a, lxlo)) / a;
  if (tau <= tau_i) return false;
  const float G = __fsub_rn(t.gcumf[0], __fmul_rn(__fsub_rn(tau, tau_i), temp) / lam);
  return !(G > 0.0f);
}

// exp(x) - 1 of a cooling factor's exponent (x <= 0): the Taylor series to
// x^5 for |x| < 1/64 (truncation below x^6/720, under 2e-12 of the result),
// expm1f beyond.  Horner steps as explicit FMAs (no contraction choice).
__device__ __forceinline__ float expm1_cool(float x) {
  if (!(fabsf(x) < 0.015625f)) return expm1f(x);
  float r = __fmaf_rn(x, 1.0f / 120.0f, 1.0f / 24.0f);
  r = __fmaf_rn(x, r, 1.0f / 6.0f);
  r = __fmaf_rn(x, r, 0.5f);
  r = __fmaf_rn(x, r, 1.0f);
  return __fmul_rn(x, r);
}

// The cooling of a cell that cools (cools_at), at temperature temp with
// table coefficient aloss (found at table entry seg): w[4] and u4 updated.
__device__ __forceinline__ void cool_cell_known(const Params& p, float cT, float inv_muamu, float gm1, float* w,
                                                double& u4, float dt, float temp, float aloss, int seg) {
  const CoolTable& t = p.cool;
  const float p0 = w[4];
  float ETH = w[4] / gm1;
  const float n = w[0] * inv_muamu;
  float ce = (aloss * n) * (n / ETH);
  int nsub = 1;
  const float frac = p.f_cool_sub_frac;
  if (p.cooling == COOL_EXACT && ce * dt > frac) {
    const float dp = __fmul_rn(w[4], cool_exact_dropf(t, temp, aloss, ce * dt));
    w[4] = __fadd_rn(w[4], dp);
    u4 = u4 + f2d(dp / gm1);
    return;
  }
  if (p.cooling == COOL_SUBCYCLE && ce * dt > frac) {
    const float q = ceilf(ce * dt / frac);
    nsub = (q > (float)p.cool_max_sub) ? p.cool_max_sub : (int)q;
    if (nsub < 1) nsub = 1;
  }
  // Each sub-step's factor f = exp(-ce h) is carried as f - 1 (expm1_cool),
  // and the pressure's relative change over the sub-steps as q = p/p0 - 1:
  // with ce h ~ 1e-3, f itself keeps only the top few digits of f - 1 in
  // FP32 (and p - p0 those of the change), which biased the energy removed
  // by ~1e-3 of itself.
  const float h = dt / (float)nsub;
  float q = 0.0f;
  for (int s = 0; s < nsub; ++s) {
    if (s > 0) {
      temp = (w[4] / w[0]) * cT;
      if (!(temp >= t.Tf[0])) break;  // (after a sub-step the state is no longer the stored one)
      ETH = w[4] / gm1;
      aloss = cool_coef_seg(t, temp, seg);
      ce = (aloss * n) * (n / ETH);
    }
    float fq = expm1_cool(-ce * h);
    if (fq < -p.f_cooling_limit) fq = -p.f_cooling_limit;  // f < 1 - cooling_limit
    bool floored = false;
    if (__fmaf_rn(temp, fq, temp) < (float)T_FLOOR) {
      fq = __fsub_rn((float)T_FLOOR / temp, 1.0f);
      floored = true;
    }
    q = __fadd_rn(q, __fmaf_rn(q, fq, fq));  // (1 + q)(1 + fq) - 1
    w[4] = __fmaf_rn(p0, q, p0);
    if (floored) break;
  }
  u4 = u4 + f2d(__fmul_rn(p0, q) / gm1);
}

__device__ __forceinline__ void cool_cell_f(const Params& p, float cT, float inv_muamu, float gm1, float* w,
                                            double& u4, float dt, const double* u) {
  const float temp = (w[4] / w[0]) * cT;
  if (!cools_at(p, temp, u)) return;
  int seg = 0;  // the table entry of the coefficient
  const float aloss = cool_coef_seg(p.cool, temp, seg);
  cool_cell_known(p, cT, inv_muamu, gm1, w, u4, dt, temp, aloss, seg);
}

// The face-ghost images of a stage-1 cell (borders(UPP, 2), boundaries.f90
// non-MPI branches) as FP32 primitives of UPP: the FP64 image of v (normal
// momentum negated at a reflective face) with the winds applied at the ghost
// cell, through mixed_cell -- what stage 2 forms from UPP.
__device__ __forceinline__ void write_ghost_prims(const Params& p, const Layout& L, float* out, float gm1, int i,
                                                  int j, int k, const double* v) {
  const int c3[3] = {i, j, k};
  const int n3[3] = {p.nx, p.ny, p.nz};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    int tgt[4], flp[4];
    const int m = ghost_targets(2, p.bc[2 * ax], p.bc[2 * ax + 1], c3[ax], n3[ax], tgt, flp);
    for (int q = 0; q < m; ++q) {
      int g3[3] = {i, j, k};
      g3[ax] = tgt[q];
      double g[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) g[e] = (flp[q] && e == ax + 1) ? -v[e] : v[e];
      winds_cell(p, g3[0], g3[1], g3[2], g);
      float cf[5], w[5];
      mixed_cell(gm1, g, 1, cf, w);
      const long long o = L.at(g3[0], g3[1], g3[2]);
#pragma unroll
      for (int e = 0; e < 5; ++e) out[e * L.plane + o] = w[e];
    }
  }
}

// The conserved values of a cell from its FP32 primitives: what HLLC takes
// at the cell centres beside a stage-2 face (UPP is stored as primitives).
__device__ __forceinline__ void prim_cons(const float* w, float igm1, float* u) {
  const float k2 = __fmaf_rn(w[3], w[3], __fmaf_rn(w[2], w[2], __fmul_rn(w[1], w[1])));
  u[0] = w[0];
  u[1] = __fmul_rn(w[0], w[1]);
  u[2] = __fmul_rn(w[0], w[2]);
  u[3] = __fmul_rn(w[0], w[3]);
  u[4] = __fmaf_rn(w[4], igm1, __fmul_rn(__fmul_rn(0.5f, w[0]), k2));
}

// One first-order face flux of stage 1, direction d (1 x, 2 y, 3 z; a
// compile-time constant at every call), from the primitives of the two cells
// beside the face (wl, wr) and their conserved values (uL, uR: the FP32
// image of U), each `VS` floats between variables.
template <int LIM, int SOLV, int VS>
__device__ __forceinline__ void face_flux1(const Params& p, float gf, float g1f, int d, const float* w1,
                                           const float* w2, const float* uL, const float* uR, float* ff) {
  float wl[5], wr[5], UL[5], UR[5];
#pragma unroll
  for (int e = 0; e < 5; ++e) {
    wl[e] = w1[e * VS];
    wr[e] = w2[e * VS];
    UL[e] = uL[e * VS];
    UR[e] = uR[e * VS];
  }
  if (!riemann(SOLV >= 0 ? SOLV : p.solver, gf, g1f, ff, wl, wr, UL, UR, d)) {
#pragma unroll
    for (int e = 0; e < 5; ++e) ff[e] = NAN;
  }
}

// A stage-2 face in its own frame: the velocity components of the four
// cells are loaded normal first, then the two tangential ones in the
// reference's order (on, o1, o2: their offsets from a cell's density, VS
// floats per variable), so that the limiter and the Riemann solver run with
// the face's direction fixed at x -- no selects on a runtime direction --
// and ff comes back in the same frame (ff[1] the normal momentum flux).  The
// tangential momentum fluxes are (rho u_n) u_t here, where the reference
// forms (rho u_lo) u_hi by component index: the same value to FP32
// rounding.
template <int LIM, int SOLV, int VS>
__device__ __forceinline__ void face_flux_frame(const Params& p, float gf, float g1f, float igm1, int on, int o1,
                                                int o2, const float* w0, const float* w1, const float* w2,
                                                const float* w3, float* ff) {
  float wll[5], wl[5], wr[5], wrr[5], UL[5], UR[5];
  auto load = [&](const float* w, float* v) {
    v[0] = w[0];
    v[1] = w[on];
    v[2] = w[o1];
    v[3] = w[o2];
    v[4] = w[4 * VS];
  };
  load(w1, wl);
  load(w2, wr);
  prim_cons(wl, igm1, UL);
  prim_cons(wr, igm1, UR);
  load(w0, wll);
  load(w3, wrr);
  limiter(wll, wl, wr, wrr, LIM >= 0 ? LIM : p.limiter);
  if (!riemann(SOLV >= 0 ? SOLV : p.solver, gf, g1f, ff, wl, wr, UL, UR, 1)) {
#pragma unroll
    for (int e = 0; e < 5; ++e) ff[e] = NAN;
  }
}

// All x, y and z faces of plane k of a tile (x faces (MTX+1) x MTY, y faces
// MTX x (MTY+1), z faces MTX x MTY: no face twice); xy false: only the z
// faces (the plane below a z-chunk).  prm(q) / cu(q): the planes of
// primitives / conserved values of plane q (stage 1; stage 2 forms the
// conserved values from the primitives).
//   Stage 1 (first-order faces, little code per face) evaluates them in
// three rounds of one direction each, the direction known at compile time:
// each thread the left x face, the lower y face and the upper z face of one
// cell, and the tile's right x edge (warp 0) and upper y edge (warp 1) as
// second faces of their rounds.  Stage 2's faces (limiter and HLLC) are one
// flat task list through one copy of the code, each face in its own frame
// (face_flux_frame; the rounds' three copies measured slower there).
template <int STAGE, int LIM, int SOLV, class Smem, class PrmOf, class CuOf>
__device__ __forceinline__ void mixed_faces(const Params& p, Smem& s, int i0, int j0, int k, bool xy, float gf,
                                            float g1f, float igm1, PrmOf prm, CuOf cu) {
  using G = MGeo<STAGE>;
  constexpr int OY = G::OY, PX = G::PX, VS = G::PB;
  constexpr int NXF = (MTX + 1) * MTY, NYF = MTX * (MTY + 1), NZF = MTX * MTY;
  const float* pk = prm(k);
  const float* ck = (STAGE == 1) ? cu(k) : nullptr;
  if constexpr (STAGE == 1) {
    constexpr int NC = MTX * MTY;
    const int tid = threadIdx.x;
    if (xy) {
      for (int t = tid; t < NXF; t += MNT) {  // t >= NC: the right edge, x = MTX
        const int fxl = (t < NC) ? t % MTX : MTX, fyl = (t < NC) ? t / MTX : t - NC;
        const int o = (fyl + OY) * PX + fxl + 1;  // cell i0 - 1 + fxl
        if ((i0 - 1 + fxl <= p.nx) && (j0 + fyl <= p.ny)) {
          float ff[5];
          face_flux1<LIM, SOLV, VS>(p, gf, g1f, 1, pk + o, pk + o + 1, ck + o, ck + o + 1, ff);
#pragma unroll
          for (int e = 0; e < 5; ++e) s.fx[e][fyl][fxl] = ff[e];
        }
      }
      for (int t = (tid + MNT - 32) % MNT; t < NYF; t += MNT) {  // t >= NC: the upper edge, y = MTY
        const int fxl = (t < NC) ? t % MTX : t - NC, fyl = (t < NC) ? t / MTX : MTY;
        const int o = (fyl - 1 + OY) * PX + fxl + 2;  // cell j0 - 1 + fyl
        if ((i0 + fxl <= p.nx) && (j0 - 1 + fyl <= p.ny)) {
          float ff[5];
          face_flux1<LIM, SOLV, VS>(p, gf, g1f, 2, pk + o, pk + o + PX, ck + o, ck + o + PX, ff);
#pragma unroll
          for (int e = 0; e < 5; ++e) s.fy[e][fyl][fxl] = ff[e];
        }
      }
    }
    {
      const int fxl = tid % MTX, fyl = tid / MTX;
      const int o = (fyl + OY) * PX + fxl + 2;
      if (tid < NZF && (i0 + fxl <= p.nx) && (j0 + fyl <= p.ny)) {
        float ff[5];
        face_flux1<LIM, SOLV, VS>(p, gf, g1f, 3, pk + o, prm(k + 1) + o, ck + o, cu(k + 1) + o, ff);
#pragma unroll
        for (int e = 0; e < 5; ++e) s.fz[(k + 1) & 1][e][fyl][fxl] = ff[e];
      }
    }
    return;
  }
  const int tbeg = xy ? 0 : NXF + NYF;
  for (int t = tbeg + (int)threadIdx.x; t < NXF + NYF + NZF; t += MNT) {
    int d, fxl, fyl;
    const float *w0, *w1, *w2, *w3;
    bool valid;
    if (t < NXF) {
      d = 1;
      fxl = t % (MTX + 1);
      fyl = t / (MTX + 1);
      w1 = pk + (fyl + OY) * PX + fxl + 1;  // cell i0 - 1 + fxl
      w0 = w1 - 1;
      w2 = w1 + 1;
      w3 = w1 + 2;
      valid = (i0 - 1 + fxl <= p.nx) && (j0 + fyl <= p.ny);
    } else if (t < NXF + NYF) {
      d = 2;
      const int u = t - NXF;
      fxl = u % MTX;
      fyl = u / MTX;
      w1 = pk + (fyl - 1 + OY) * PX + fxl + 2;  // cell j0 - 1 + fyl
      w0 = w1 - PX;
      w2 = w1 + PX;
      w3 = w1 + 2 * PX;
      valid = (i0 + fxl <= p.nx) && (j0 - 1 + fyl <= p.ny);
    } else {
      d = 3;
      const int u = t - NXF - NYF;
      fxl = u % MTX;
      fyl = u / MTX;
      const int o = (fyl + OY) * PX + fxl + 2;
      w0 = prm(k - 1) + o;
      w1 = pk + o;
      w2 = prm(k + 1) + o;
      w3 = prm(k + 2) + o;
      valid = (i0 + fxl <= p.nx) && (j0 + fyl <= p.ny);
    }
    if (!valid) continue;
    // the face's frame: normal component d, then the other two in order
    const int on = d * VS, o1 = (d == 1 ? 2 : 1) * VS, o2 = (d == 3 ? 2 : 3) * VS;
    float ff[5];
    face_flux_frame<LIM, SOLV, VS>(p, gf, g1f, igm1, on, o1, o2, w0, w1, w2, w3, ff);
    if (d == 1) {
#pragma unroll
      for (int e = 0; e < 5; ++e) s.fx[e][fyl][fxl] = ff[e];
    } else if (d == 2) {  // frame (y, x, z)
      s.fy[0][fyl][fxl] = ff[0];
      s.fy[1][fyl][fxl] = ff[2];
      s.fy[2][fyl][fxl] = ff[1];
      s.fy[3][fyl][fxl] = ff[3];
      s.fy[4][fyl][fxl] = ff[4];
    } else {  // frame (z, x, y)
      float* fz = &s.fz[(k + 1) & 1][0][fyl][fxl];
      constexpr int ZS = MTY * MTX;
      fz[0] = ff[0];
      fz[ZS] = ff[2];
      fz[2 * ZS] = ff[3];
      fz[3 * ZS] = ff[1];
      fz[4 * ZS] = ff[4];
    }
  }
}

// The flux divergence of tile cell (tx, ty) of plane k (minus the gravity
// source, -dt S, when gravity is on): dU of Godunov (HLLC.f90:37-40).
template <int STAGE, class Smem>
__device__ __forceinline__ void flux_divergence(const Params& p, const Smem& s, int k, int tx, int ty, float dtf,
                                                float dtdx, float dtdy, float dtdz, const float* wc, const float* ph,
                                                float* dU) {
  const int cur = (k + 1) & 1, prv = k & 1;
#pragma unroll
  for (int e = 0; e < 5; ++e)
    dU[e] = dtdx * (s.fx[e][ty][tx + 1] - s.fx[e][ty][tx]) + dtdy * (s.fy[e][ty + 1][tx] - s.fy[e][ty][tx]) +
            dtdz * (s.fz[cur][e][ty][tx] - s.fz[prv][e][ty][tx]);
  if (p.gravity) {
    // S_Solver (sources.f90:885-893) from the cell's primitives wc
    const float fg1 = (ph[0] - ph[1]) * p.f_hdx;
    const float fg2 = (ph[2] - ph[3]) * p.f_hdy;
    const float fg3 = (ph[4] - ph[5]) * p.f_hdz;
    float sv[5];
    sv[0] = 0.0f;
    sv[1] = -wc[0] * fg1;
    sv[2] = -wc[0] * fg2;
    sv[3] = -wc[0] * fg3;
    sv[4] = -wc[0] * (wc[1] * fg1 + wc[2] * fg2 + wc[3] * fg3);
#pragma unroll
    for (int e = 0; e < 5; ++e) dU[e] -= dtf * sv[e];
  }
}

// Bounded TMA/mbarrier bookkeeping of one tile: every thread waits for every
// plane in order and tracks the slots' phases; a wait that runs out sets the
// block's abort flag.
struct PlaneWaits {
  uint32_t phase = 0;
  int waited;
  bool failed = false;
  __device__ __forceinline__ void wait(uint64_t* bars, int nslot, int q, int* abort) {
    if (failed) return;
    const int slot = q & (nslot - 1);
    if (!mbar_wait_bounded(&bars[slot], (phase >> slot) & 1u, WAIT_LIMIT)) {
      failed = true;
      *abort = 1;
      return;
    }
    phase ^= 1u << slot;
    waited = q;
  }
  // after an abort, thread 0 lets the copies it issued land (bounded)
  __device__ __forceinline__ void drain(uint64_t* bars, int nslot, int issued) {
    for (int q = waited + 1; q <= issued; ++q) {
      const int slot = q & (nslot - 1);
      mbar_wait_bounded(&bars[slot], (phase >> slot) & 1u, WAIT_LIMIT);
      phase ^= 1u << slot;
    }
  }
};

// One tile (MTX x MTY columns, z-chunk bz of zlen planes) of stage 1: the
// body of the single-mesh kernel and of each work item of the batched
// persistent kernel.  Streams U (FP64) with a 1-cell halo; writes UPP as
// FP32 primitives (and its face-ghost images), and eta * Laplacian(U) in
// FP32 for stage 2.  Leaves every TMA copy it issued completed.
template <int LIM, int SOLV>
__device__ __forceinline__ void mixed_tile1(const CUtensorMap* tm, const StageArgs& a, MixedSmem1& s, int bx, int by,
                                            int bz) {
  using G = MGeo<1>;
  const Params& p = a.p;
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const int i0 = 1 + bx * MTX, j0 = 1 + by * MTY;
  const int k0 = 1 + bz * a.zlen;
  const int k1 = min(p.nz, k0 + a.zlen - 1);
  const Clock* clk = a.clk;
  if (!(clk->t < clk->tfin)) return;  // the loop condition of mainHD.f90:61 (uniform)
  const float dtf = 0.5f * d2f(clk->dt);  // dth = dt/2 (mainHD.f90:78)
  const float gf = p.f_gamma, gm1 = gf - 1.0f, g1f = p.f_g1;
  const float dtdx = dtf * p.f_inv_dx, dtdy = dtf * p.f_inv_dy, dtdz = dtf * p.f_inv_dz;
  const int last = k1 + 1;
  const long long pxy = (long long)L.px * L.nyg;

  if (tid == 0) {
    mbar_init(&s.bar[0], 1);
    s.abort = 0;
    fence_mbar_init();
  }
  __syncthreads();
  int issued = k0 - 2;
  auto issue = [&](int q) {  // thread 0
    fence_proxy_async();
    mbar_arrive_expect_tx(&s.bar[0], 5u * G::PB * 8u);
    tma_load_4d(s.raw, tm, &s.bar[0], bx * MTX, by * MTY + 1, q + 1, 0);
    issued = q;
  };
  PlaneWaits pw;
  pw.waited = k0 - 2;
  // U of plane q (landed) -> FP32 conserved and primitives on the cells its
  // faces and Laplacian read
  auto convert = [&](int q) {
    float* C = &s.cu[q & 3].v[0][0][0];
    float* W = &s.prm[q & 1].v[0][0][0];
    constexpr int NROW = (MTX + 2) * MTY, NCOL = 2 * MTX;
    for (int t = tid; t < NROW + NCOL; t += MNT) {
      int lx, ly;
      if (t < NROW) {
        lx = 1 + t % (MTX + 2);
        ly = 1 + t / (MTX + 2);
      } else {
        const int u = t - NROW;
        lx = 2 + u % MTX;
        ly = (u < MTX) ? 0 : MTY + 1;
      }
      const int o = ly * G::PX + lx;
      float cf[5], w[5];
      mixed_cell(gm1, s.raw + o, G::PB, cf, w);
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        C[e * G::PB + o] = cf[e];
        W[e * G::PB + o] = w[e];
      }
    }
  };
  auto prm = [&](int q) { return &s.prm[q & 1].v[0][0][0]; };
  auto cu = [&](int q) { return &s.cu[q & 3].v[0][0][0]; };

  // prologue: planes k0-1 and k0
  bool aborted = false;
  for (int q = k0 - 1; q <= k0; ++q) {
    if (tid == 0) issue(q);
    pw.wait(s.bar, 1, q, &s.abort);
    convert(q);
    __syncthreads();
    if (s.abort) { aborted = true; break; }
  }
  if (!aborted && tid == 0 && k0 + 1 <= last) issue(k0 + 1);

  const int tx = tid % MTX, ty = tid / MTX;
  const int i = i0 + tx, j = j0 + ty;
  const bool cell_ok = (ty < MTY) && (i <= p.nx) && (j <= p.ny);
  const float etaf = p.f_eta;
  const TileSpecial ts = tile_special(p, i0, min(i0 + MTX - 1, p.nx), j0, min(j0 + MTY - 1, p.ny));
  // k = k0 - 1 computes only the z face below the chunk, through the same
  // (single) copy of the face code as every other plane, so that a cell's
  // arithmetic does not depend on where the z-chunks begin
  for (int k = k0 - 1; k <= k1 && !aborted; ++k) {
    const bool first = k < k0;
    const long long c = L.at(i, j, k);
    float ph[6];
    if (cell_ok && !first) {
      if (p.gravity) {
        ph[0] = a.phif[c + 1]; ph[1] = a.phif[c - 1];
        ph[2] = a.phif[c + L.px]; ph[3] = a.phif[c - L.px];
        ph[4] = a.phif[c + pxy]; ph[5] = a.phif[c - pxy];
      }
    }
    if (!first) {
      // no barrier before the conversion: the previous plane's cell phase,
      // which other warps may still be running, reads the conserved slots
      // of planes k-2..k and no primitive slot
      pw.wait(s.bar, 1, k + 1, &s.abort);
      convert(k + 1);
      __syncthreads();
      if (s.abort) { aborted = true; break; }
      if (tid == 0 && k + 2 <= last) issue(k + 2);
    }
    mixed_faces<1, LIM, SOLV>(p, s, i0, j0, k, !first, gf, g1f, 0.0f, prm, cu);
    __syncthreads();
    if (first || !cell_ok) continue;

    const int lx = tx + 2, ly = ty + 1;
    float wc[5];  // the cell's velocity and density for the gravity source, as mixed_cell forms them
    if (p.gravity) {
      const float* A1 = cu(k);
      const int o = ly * G::PX + lx;
      wc[0] = A1[o];
      const float inv = 1.0f / wc[0];
      wc[1] = A1[G::PB + o] * inv;
      wc[2] = A1[2 * G::PB + o] * inv;
      wc[3] = A1[3 * G::PB + o] * inv;
      wc[4] = 0.0f;
    }
    float dU[5];
    flux_divergence<1>(p, s, k, tx, ty, dtf, dtdx, dtdy, dtdz, wc, ph, dU);
    // step's viscosity, eta * (sum of the 6 neighbours - 6 U), of the U this
    // stage streams (= the old U of stage 2), in FP32 from the ring
    {
      const float* A0 = cu(k - 1);
      const float* A1 = cu(k);
      const float* A2 = cu(k + 1);
      const int o = ly * G::PX + lx;
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        const int oe = e * G::PB + o;
        const float lap = ((A1[oe + 1] + A1[oe - 1]) + (A1[oe + G::PX] + A1[oe - G::PX])) +
                          ((A2[oe] + A0[oe]) - 6.0f * A1[oe]);
        a.lapf[e * L.plane + c] = etaf * lap;
      }
    }
    // UPP = U - dU (Godunov's centre value is U).  UPP is kept in FP32, so
    // it is formed in FP32 from the FP32 state of the ring, and its
    // primitives as mixed_cell forms them, except where FP64 is needed: the
    // pressure of a cell whose kinetic energy exceeds 0.99 of its total
    // energy (FP32 would lose it to cancellation), and the cells whose UPP
    // the boundaries or the winds also need (ghost images, wind overwrite),
    // which take UPP = U - dU in FP64 from the state in HBM.
    float w[5];
    const bool nb = ts.may_be_special(p, k) && near_boundary_or_wind(p, i, j, k);
    bool fp64 = nb;
    if (!fp64) {
      const float* A1 = cu(k);
      const int o = ly * G::PX + lx;
      float uf[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) uf[e] = __fsub_rn(A1[e * G::PB + o], dU[e]);
      const float inv = 1.0f / uf[0];
      w[0] = uf[0];
      w[1] = uf[1] * inv;
      w[2] = uf[2] * inv;
      w[3] = uf[3] * inv;
      const float ek = __fmul_rn(0.5f, __fmaf_rn(uf[3], w[3], __fmaf_rn(uf[2], w[2], __fmul_rn(uf[1], w[1]))));
      fp64 = ek > __fmul_rn(0.99f, uf[4]);
      w[4] = fmaxf(__fmul_rn(gm1, __fsub_rn(uf[4], ek)), 1e-20f);
    }
    if (__any_sync(__activemask(), fp64) && fp64) {
      double up[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) up[e] = a.uold[e * L.plane + c] - f2d(dU[e]);
      if (nb) {
        write_ghost_prims(p, L, a.uppf, gm1, i, j, k, up);  // borders(UPP, 2)
        winds_cell(p, i, j, k, up);
      }
      float cf[5];
      mixed_cell(gm1, up, 1, cf, w);
    }
#pragma unroll
    for (int e = 0; e < 5; ++e) a.uppf[e * L.plane + c] = w[e];
  }
  if (aborted && tid == 0) {
    atomicOr(&const_cast<Clock*>(clk)->status, ST_TIMEOUT);
    pw.drain(s.bar, 1, issued);
  }
}

// One tile of stage 2: streams UPP's FP32 primitives with a 2-cell halo;
// writes U of the next step (FP64) and its face-ghost images, cools, and
// reduces the signal speeds for the next dt.  nblk / bid: the mesh's tiles
// and this one's index, for the dt reduction.  Leaves every TMA copy it
// issued completed.
template <int LIM, int SOLV>
__device__ __forceinline__ void mixed_tile2(const CUtensorMap* tm, const StageArgs& a, MixedSmem2& s, int bx, int by,
                                            int bz, unsigned nblk, unsigned bid) {
  using G = MGeo<2>;
  const Params& p = a.p;
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const int i0 = 1 + bx * MTX, j0 = 1 + by * MTY;
  const int k0 = 1 + bz * a.zlen;
  const int k1 = min(p.nz, k0 + a.zlen - 1);
  Clock* clk = a.clk;
  if (!(clk->t < clk->tfin)) return;  // the loop condition of mainHD.f90:61 (uniform)
  const float dtf = d2f(clk->dt);
  const float gf = p.f_gamma, gm1 = gf - 1.0f, g1f = p.f_g1;
  const float igm1 = __frcp_rn(gm1);
  const float dtdx = dtf * p.f_inv_dx, dtdy = dtf * p.f_inv_dy, dtdz = dtf * p.f_inv_dz;
  const int last = k1 + 2;
  const long long pxy = (long long)L.px * L.nyg;

  if (tid == 0) {
    for (int q = 0; q < 4; ++q) mbar_init(&s.bar[q], 1);
    s.abort = 0;
    s.tspec = tile_special(p, i0, min(i0 + MTX - 1, p.nx), j0, min(j0 + MTY - 1, p.ny));
    fence_mbar_init();
  }
  __syncthreads();
  int issued = k0 - 3;
  auto issue = [&](int q) {  // thread 0: plane q into slot q & 3
    const int slot = q & 3;
    fence_proxy_async();
    mbar_arrive_expect_tx(&s.bar[slot], 5u * G::PB * 4u);
    tma_load_4d(&s.prm[slot], tm, &s.bar[slot], bx * MTX, by * MTY, q + 1, 0);
    issued = q;
  };
  PlaneWaits pw;
  pw.waited = k0 - 3;
  auto prm = [&](int q) { return &s.prm[q & 3].v[0][0][0]; };
  auto nocu = [](int) -> const float* { return nullptr; };

  // prologue: planes k0-2 .. k0+1 (the first z face, k0 - 1/2, reads them)
  if (tid == 0)
    for (int q = k0 - 2; q <= k0 + 1; ++q) issue(q);
  for (int q = k0 - 2; q <= k0 + 1; ++q) pw.wait(s.bar, 4, q, &s.abort);

  const int tx = tid % MTX, ty = tid / MTX;
  const int i = i0 + tx, j = j0 + ty;
  const bool cell_ok = (ty < MTY) && (i <= p.nx) && (j <= p.ny);
  float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
  unsigned nsingle = 0;  // with the surrogate: cells cooled in a single step
  unsigned nfloor = 0;   // ... and first-segment cells taken to the floor
  const float cT = p.f_cT;
  const float inv_muamu = p.f_inv_muamu;
  bool aborted = false;
  for (int k = k0 - 1; k <= k1; ++k) {
    const bool first = k < k0;
    const long long c = L.at(i, j, k);
    double uc[5];
    float lv[5];
    float ph[6];
    bool queued = false;  // with the surrogate: handed to the cooling passes
    if (!first && cell_ok) {
      // the cell's operands in HBM, landing while the faces are evaluated
#pragma unroll
      for (int e = 0; e < 5; ++e) cp_async8(&s.uop[e][tid], &a.uold[e * L.plane + c]);
#pragma unroll
      for (int e = 0; e < 5; ++e) cp_async4(&s.lvp[e][tid], &a.lapf[e * L.plane + c]);
      if (p.gravity) {
        cp_async4(&s.php[0][tid], &a.phif[c + 1]);
        cp_async4(&s.php[1][tid], &a.phif[c - 1]);
        cp_async4(&s.php[2][tid], &a.phif[c + L.px]);
        cp_async4(&s.php[3][tid], &a.phif[c - L.px]);
        cp_async4(&s.php[4][tid], &a.phif[c + pxy]);
        cp_async4(&s.php[5][tid], &a.phif[c - pxy]);
      }
      cp_async_commit();
    }
    if (!first) pw.wait(s.bar, 4, k + 2, &s.abort);
    __syncthreads();
    if (s.abort) { aborted = true; break; }
    mixed_faces<2, LIM, SOLV>(p, s, i0, j0, k, !first, gf, g1f, igm1, prm, nocu);
    __syncthreads();
    if (tid == 0 && k + 3 <= last) issue(k + 3);  // into plane k-1's slot: its faces are done
    if (first) continue;

    if (cell_ok) {
      cp_async_wait_all();  // this thread's own copies: no barrier
#pragma unroll
      for (int e = 0; e < 5; ++e) uc[e] = s.uop[e][tid];
#pragma unroll
      for (int e = 0; e < 5; ++e) lv[e] = s.lvp[e][tid];
      if (p.gravity) {
#pragma unroll
        for (int q = 0; q < 6; ++q) ph[q] = s.php[q][tid];
      }
      float wc[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) wc[e] = s.prm[k & 3].v[e][ty + 2][tx + 2];
      float dU[5];
      flux_divergence<2>(p, s, k, tx, ty, dtf, dtdx, dtdy, dtdz, wc, ph, dU);
      // FP64 accumulation: UP = U - dU (Godunov's centre value is the old U).
      // Away from the boundaries and the winds (which read or overwrite UP):
      // U = U_old - dU + eta Lap in one FP64 addition of the FP32 increment
      // (an FP64 addition costs ~64 FP32 slots on GB300; the gate also keeps
      // the winds' FP64 distance and density off the FP64 pipe)
      const bool special = s.tspec.may_be_special(p, k) && near_boundary_or_wind(p, i, j, k);
      double un[5];
      if (!special) {
#pragma unroll
        for (int e = 0; e < 5; ++e) un[e] = uc[e] + f2d(lv[e] - dU[e]);
      } else {
        double up[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) up[e] = uc[e] - f2d(dU[e]);
        write_ghosts(p, L, a.out, 1, i, j, k, up);  // borders(UP, 1) with the winds
        winds_cell(p, i, j, k, up);
        // step: U = UP + eta * (Laplacian of the old U), from stage 1
#pragma unroll
        for (int e = 0; e < 5; ++e) un[e] = up[e] + f2d(lv[e]);
      }
      float cf[5], w[5];
      mixed_cell(gm1, un, 1, cf, w);  // calc_prims(UPrim, U)
      if (p.cooling == COOL_MLP) {
        // A cell whose tau (Lambda n^2 dt / E_th, formed as the cooling
        // passes form it) is at most the single-step limit takes the exact
        // integrator's single exponential step here (the passes would do the
        // same); so does a cell of the table's first segment that the exact
        // integrator takes to the table's first temperature within the step
        // (a medium sitting at that floor): the network is not asked for
        // those (the passes would hand them to the exact integrator, with
        // these bits).  The passes cool the others and take their signal
        // speeds.
        const float T = (w[4] / w[0]) * cT;
        if (cools_at(p, T, un)) {
          const float nd = w[0] * inv_muamu;
          const float eth = w[4] / gm1;
          int seg = 0;
          const float lam = cool_coef_seg(p.cool, T, seg);
          const float tau = (lam * nd) * (nd / eth) * dtf;
          if (tau > p.f_cool_sub_frac) {
            if (seg == 1 && cool_floors_first(p.cool, T, lam, tau)) {
              // cool_cell_known's exact branch with cool_exact_dropf's floor
              const float dp = __fmul_rn(w[4], __fsub_rn(p.cool.Tf[0] / T, 1.0f));
              w[4] = __fadd_rn(w[4], dp);
              un[4] = un[4] + f2d(dp / gm1);
              ++nfloor;
            } else {
              queued = true;
            }
          } else {
            cool_cell_known(p, cT, inv_muamu, gm1, w, un[4], dtf, T, lam, seg);
            ++nsingle;
          }
        }
      } else if (p.cooling != COOL_NONE) {
        cool_cell_f(p, cT, inv_muamu, gm1, w, un[4], dtf, un);
      }
      {
        // !(rho > 0) on the bits (no FP64 compare): sign set, zero or
        // below the normal range, or not finite
        const int hi = __double2hiint(un[0]);
        if (hi < 0x00100000 || (hi & 0x7ff00000) == 0x7ff00000) atomicOr(&clk->status, ST_NEG_DENSITY);
      }
#pragma unroll
      for (int e = 0; e < 5; ++e) a.out[e * L.plane + c] = un[e];
      if (!queued) {
        const float cs = sqrtf(gf * w[4] / w[0]);
        const float v0 = fabsf(w[1]) + cs, v1 = fabsf(w[2]) + cs, v2 = fabsf(w[3]) + cs;
        m0 = (v0 != v0 || v0 > m0) ? v0 : m0;
        m1 = (v1 != v1 || v1 > m1) ? v1 : m1;
        m2 = (v2 != v2 || v2 > m2) ? v2 : m2;
      }
    }
    if (p.cooling == COOL_MLP) {
      // warp-aggregated append to the cooling queue (interior cell index)
      const unsigned qm = __ballot_sync(0xffffffffu, queued);
      if (qm) {
        const int lane = tid & 31;
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(a.cqcount, (unsigned)__popc(qm));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (queued)
          a.cqueue[base + __popc(qm & ((1u << lane) - 1u))] =
              (unsigned)((i - 1) + p.nx * ((long long)(j - 1) + (long long)p.ny * (k - 1)));
      }
    }
  }

  cp_async_wait_all();  // (a tile that gave up leaves no copy of its own in flight)
  double d0 = f2d(m0), d1 = f2d(m1), d2 = f2d(m2);
  if (aborted) {
    if (tid == 0) {
      atomicOr(&clk->status, ST_TIMEOUT);
      pw.drain(s.bar, 4, issued);
    }
    d0 = d1 = d2 = NAN;
  }
  if (p.cooling == COOL_MLP && a.cool_counts) {
    unsigned v = nsingle, f = nfloor;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      v += __shfl_xor_sync(0xffffffffu, v, off);
      f += __shfl_xor_sync(0xffffffffu, f, off);
    }
    if ((tid & 31) == 0 && v) atomicAdd(&a.cool_counts[2], (unsigned long long)v);
    if ((tid & 31) == 0 && f) atomicAdd(&a.cool_counts[1], (unsigned long long)f);  // the exact integrator's
  }
  if (p.cooling != COOL_MLP) {
    cfl_reduce_finalize_n<MNT>(d0, d1, d2, clk, p, true, s.red, &s.flag, nblk);
  } else {
    // with the surrogate the cooling passes finish the reduction over
    // these block maxima and their own
    cfl_contribute<MNT>(d0, d1, d2, clk, s.red);
  }
}

template <int STAGE, int LIM = -1, int SOLV = -1>
__device__ __forceinline__ void mixed_tile(const CUtensorMap* tm, const StageArgs& a, MixedSmem<STAGE>& s, int bx,
                                           int by, int bz, unsigned nblk, unsigned bid) {
  if constexpr (STAGE == 1)
    mixed_tile1<LIM, SOLV>(tm, a, s, bx, by, bz);
  else
    mixed_tile2<LIM, SOLV>(tm, a, s, bx, by, bz, nblk, bid);
}

template <int STAGE, int LIM = -1, int SOLV = -1>
__global__ void __launch_bounds__(MNT, MixedBlocks<STAGE>::value)
    stage_kernel_mixed(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ StageArgs a) {
  extern __shared__ __align__(128) unsigned char smem_bytes[];
  MixedSmem<STAGE>& s = *reinterpret_cast<MixedSmem<STAGE>*>(smem_bytes);
  mixed_tile<STAGE, LIM, SOLV>(&tm_in, a, s, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z,
                               blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

}  // namespace tlq
