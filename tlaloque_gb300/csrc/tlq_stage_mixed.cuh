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


// Shared memory per block is kept under 57 KB so that 4 blocks fit an SM:
constexpr int MRAW = 1;  // TMA landing slot (raw FP64 plane); the next plane is requested as soon as the
                         // previous one is converted, a whole plane's work (~10 us) ahead of its use
constexpr int MCU = 3;   // FP32 conserved-state ring (faces: planes k, k+1; stage-1 Laplacian: k-1..k+1)
constexpr int MIXED_BLOCKS_PER_SM = 4;

// Ring slots of plane q.  Planes start at k0 - 2 >= -1, so q can be
// negative; C++ '%' keeps the sign of q, hence the offset.
__device__ __forceinline__ int raw_slot(int q) { return (q + 4 * MRAW) % MRAW; }


__device__ __forceinline__ int cu_slot(int q) { return (q + 4 * MCU) % MCU; }

struct MixedSmem {
  double raw[MRAW][5 * MPLANE_BOX];  // TMA landing zone
  float cu[MCU][5][MHY][MHX];         // conserved state of the ring planes (FP32)
  float prm[NRING][5][MHY][MHX];      // primitives of the ring planes (FP32)
  float fx[5][MTY][MTX + 1];
  float fy[5][MTY + 1][MTX];
  float fz[2][5][MTY][MTX];
  uint64_t bar[MRAW];
  double red[96];
  int flag;
  int abort;
};

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
  float p;
  if (ek > __fmul_rn(0.99f, cf[4])) {
    const double r = u[0], m1 = u[vs], m2 = u[2 * vs], m3 = u[3 * vs], E = u[4 * vs];
    const double k2 = __fma_rn(m3, m3, __fma_rn(m2, m2, __dmul_rn(m1, m1)));
    p = d2f(__dmul_rn((double)gm1, __dsub_rn(E, __ddiv_rn(__dmul_rn(0.5, k2), r))));
  } else {
    p = __fmul_rn(gm1, __fsub_rn(cf[4], ek));
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
__device__ __forceinline__ float cool_coef_seg(const CoolTable& t, float temp, int& lo) {
  const bool same = lo >= 1 && lo <= t.n && !(t.Tf[lo - 1] > temp) && (lo == t.n || t.Tf[lo] > temp);
  if (!same) {
    lo = 1;
    int hi = t.n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t.Tf[mid] > temp) hi = mid; else lo = mid + 1;
    }
  }
  if (lo >= t.n) return exp10f(t.Cf[t.n - 1]);
  const float T0 = t.logTf[lo - 1], C0 = t.Cf[lo - 1];
  const float T1 = t.logTf[lo], C1 = t.Cf[lo];
  return exp10f(__fmaf_rn((C1 - C0) / (T1 - T0), __fsub_rn(log10f(temp), T0), C0));
}

__device__ __forceinline__ float cool_coef_f(const CoolTable& t, float temp) {
  int lo = 0;
  return cool_coef_seg(t, temp, lo);
}

// Whether cooling applies (temp >= the table's first temperature,
// cooling.f90:71).  The switch is a jump in the source term; a cell whose
// FP32 temperature falls within 1e-6 of the edge (e.g. a medium initialised
// at exactly the table's lower edge) decides it from the FP64 state with the
// plain step's arithmetic (uncontracted intrinsics), so both forms agree.
__device__ __forceinline__ bool cools_at(const Params& p, float temp, const double* u) {
  const float Tmin = p.cool.Tf[0];
  if (fabsf(__fsub_rn(temp, Tmin)) > 1e-6f * Tmin) return temp >= Tmin;
  const double r = u[0];
  const double k2 = __dadd_rn(__dadd_rn(__dmul_rn(u[1], u[1]), __dmul_rn(u[2], u[2])), __dmul_rn(u[3], u[3]));
  double pr = __dmul_rn(__dsub_rn(p.gamma, 1.0), __dsub_rn(u[4], __ddiv_rn(__dmul_rn(0.5, k2), r)));
  pr = pr > 1e-20 ? pr : 1e-20;
  const double T = __ddiv_rn(__dmul_rn(__dmul_rn(pr, p.mu0), AMU), __dmul_rn(r, KB));
  return T >= p.cool.T[0];
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
  int lo = 1, hi = t.n;  // first node above temp (n: none), as find_coef
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t.Tf[mid] > temp) hi = mid; else lo = mid + 1;
  }
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

__device__ __forceinline__ void cool_cell_f(const Params& p, float cT, float inv_muamu, float gm1, float* w,
                                            double& u4, float dt, const double* u) {
  const CoolTable& t = p.cool;
  float temp = (w[4] / w[0]) * cT;
  if (!cools_at(p, temp, u)) return;
  const float p0 = w[4];
  float ETH = w[4] / gm1;
  int seg = 0;  // the table entry of the last coefficient
  float aloss = cool_coef_seg(t, temp, seg);
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
  const float h = dt / (float)nsub;
  const float fmin = 1.0f - p.f_cooling_limit;
  for (int s = 0; s < nsub; ++s) {
    if (s > 0) {
      temp = (w[4] / w[0]) * cT;
      if (!(temp >= t.Tf[0])) break;  // (after a sub-step the state is no longer the stored one)
      ETH = w[4] / gm1;
      aloss = cool_coef_seg(t, temp, seg);
      ce = (aloss * n) * (n / ETH);
    }
    float f = __expf(-ce * h);
    if (f < fmin) f = fmin;
    bool floored = false;
    if (temp * f < (float)T_FLOOR) {
      f = (float)T_FLOOR / temp;
      floored = true;
    }
    w[4] = w[4] * f;
    if (floored) break;
  }
  u4 = u4 + f2d(__fsub_rn(w[4], p0) / gm1);
}

// One tile (MTX x MTY columns, z-chunk bz of zlen planes) of a stage: the
// body of the single-mesh kernel and of each work item of the batched
// persistent kernel.  LIM / SOLV >= 0 fix the limiter and the Riemann solver
// at compile time (their switches fold away and the face code becomes one
// straight block the compiler can schedule); -1 reads them from the params.  nblk / bid: the mesh's tiles and this one's index, for
// the dt reduction.  Leaves every TMA copy it issued completed.
template <int STAGE, int LIM = -1, int SOLV = -1>
__device__ __forceinline__ void mixed_tile(const CUtensorMap* tm, const StageArgs& a, MixedSmem& s, int bx, int by,
                                           int bz, unsigned nblk, unsigned bid) {
  constexpr int H = STAGE;
  const Params& p = a.p;
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const int i0 = 1 + bx * MTX, j0 = 1 + by * MTY;
  const int k0 = 1 + bz * a.zlen;
  const int k1 = min(p.nz, k0 + a.zlen - 1);
  Clock* clk = a.clk;

  if (!(clk->t < clk->tfin)) return;  // the loop condition of mainHD.f90:61 (uniform)
  const double dtstep = clk->dt;
  const float dtstep_f = d2f(dtstep);
  const float dtf = (STAGE == 1) ? 0.5f * dtstep_f : dtstep_f;
  const float gf = p.f_gamma, gm1 = gf - 1.0f, g1f = p.f_g1;
  const float dtdx = dtf * p.f_inv_dx, dtdy = dtf * p.f_inv_dy, dtdz = dtf * p.f_inv_dz;
  const int last_plane = k1 + H;
  const long long pxy = (long long)L.px * L.nyg;

  if (tid == 0) {
    for (int q = 0; q < MRAW; ++q) mbar_init(&s.bar[q], 1);
    s.abort = 0;
    fence_mbar_init();
  }
  __syncthreads();

  int issued = k0 - H - 1;
  auto issue = [&](int q) {
    const int slot = raw_slot(q);
    fence_proxy_async();
    mbar_arrive_expect_tx(&s.bar[slot], 5u * MPLANE_BOX * 8u);
    tma_load_4d(s.raw[slot], tm, &s.bar[slot], bx * MTX, by * MTY, q + 1, 0);
    issued = q;
  };
  uint32_t phase = 0;
  int waited = k0 - H - 1;
  bool failed = false;
  auto wait_plane = [&](int q) {
    if (failed) return;
    const int slot = raw_slot(q);
    if (!mbar_wait_bounded(&s.bar[slot], (phase >> slot) & 1u, WAIT_LIMIT)) {
      failed = true;
      s.abort = 1;
      return;
    }
    phase ^= 1u << slot;
    waited = q;
  };

  auto convert = [&](int q) {
    const double* r0 = s.raw[raw_slot(q)];
    const int sl = q & 3, sc = cu_slot(q);
    constexpr int RW = MTX + 2 * H;
    constexpr int NROW = RW * MTY, NCOL = MTX * 2 * H;
    for (int t = tid; t < NROW + NCOL; t += MNT) {
      int lx, ly;
      if (t < NROW) {
        lx = 2 - H + t % RW;
        ly = 2 + t / RW;
      } else {
        const int u = t - NROW, r2 = u / MTX;
        lx = 2 + u % MTX;
        ly = (r2 < H) ? (2 - H + r2) : (MTY + 2 + r2 - H);
      }
      float cf[5], w[5];
      mixed_cell(gm1, r0 + ly * MHX + lx, MPLANE_BOX, cf, w);
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        s.cu[sc][e][ly][lx] = cf[e];
        s.prm[sl][e][ly][lx] = w[e];
      }
    }
  };

  auto faces = [&](int k, bool xy) {
    constexpr int NXF = (MTX + 1) * MTY, NYF = MTX * (MTY + 1), NZF = MTX * MTY;
    const int tbeg = xy ? 0 : NXF + NYF;
    const int sk = k & 3;
    constexpr int VS = MPLANE_BOX;
    for (int t = tbeg + tid; t < NXF + NYF + NZF; t += MNT) {
      int d, fxl, fyl;
      const float *w0, *w1, *w2, *w3, *uL, *uR;
      bool valid;
      if (t < NXF) {
        d = 1;
        fxl = t % (MTX + 1);
        fyl = t / (MTX + 1);
        const int ly = fyl + 2;
        w0 = &s.prm[sk][0][ly][fxl];
        w1 = w0 + 1; w2 = w0 + 2; w3 = w0 + 3;
        uL = &s.cu[cu_slot(k)][0][ly][fxl + 1];
        uR = uL + 1;
        valid = (i0 - 1 + fxl <= p.nx) && (j0 + fyl <= p.ny);
      } else if (t < NXF + NYF) {
        d = 2;
        const int u = t - NXF;
        fxl = u % MTX;
        fyl = u / MTX;
        const int lx = fxl + 2;
        w0 = &s.prm[sk][0][fyl][lx];
        w1 = w0 + MHX; w2 = w0 + 2 * MHX; w3 = w0 + 3 * MHX;
        uL = &s.cu[cu_slot(k)][0][fyl + 1][lx];
        uR = uL + MHX;
        valid = (i0 + fxl <= p.nx) && (j0 - 1 + fyl <= p.ny);
      } else {
        d = 3;
        const int u = t - NXF - NYF;
        fxl = u % MTX;
        fyl = u / MTX;
        const int lx = fxl + 2, ly = fyl + 2;
        w0 = &s.prm[(k - 1) & 3][0][ly][lx];
        w1 = &s.prm[k & 3][0][ly][lx];
        w2 = &s.prm[(k + 1) & 3][0][ly][lx];
        w3 = &s.prm[(k + 2) & 3][0][ly][lx];
        uL = &s.cu[cu_slot(k)][0][ly][lx];
        uR = &s.cu[cu_slot(k + 1)][0][ly][lx];
        valid = (i0 + fxl <= p.nx) && (j0 + fyl <= p.ny);
      }
      if (!valid) continue;
      float wll[5], wl[5], wr[5], wrr[5], UL[5], UR[5], ff[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        wl[e] = w1[e * VS];
        wr[e] = w2[e * VS];
        UL[e] = uL[e * VS];
        UR[e] = uR[e * VS];
      }
      if (STAGE == 2) {
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          wll[e] = w0[e * VS];
          wrr[e] = w3[e * VS];
        }
        limiter(wll, wl, wr, wrr, LIM >= 0 ? LIM : p.limiter);
      }
      if (!riemann(SOLV >= 0 ? SOLV : p.solver, gf, g1f, ff, wl, wr, UL, UR, d)) {
#pragma unroll
        for (int e = 0; e < 5; ++e) ff[e] = NAN;
      }
      if (d == 1) {
#pragma unroll
        for (int e = 0; e < 5; ++e) s.fx[e][fyl][fxl] = ff[e];
      } else if (d == 2) {
#pragma unroll
        for (int e = 0; e < 5; ++e) s.fy[e][fyl][fxl] = ff[e];
      } else {
#pragma unroll
        for (int e = 0; e < 5; ++e) s.fz[(k + 1) & 1][e][fyl][fxl] = ff[e];
      }
    }
  };

  // ---- prologue: planes k0-H .. k0+H-1 ---------------------------------------
  if (tid == 0)
    for (int q = k0 - H; q <= min(k0 - H + MRAW - 1, last_plane); ++q) issue(q);
  bool aborted = false;
  for (int q = k0 - H; q <= k0 + H - 1; ++q) {
    wait_plane(q);
    convert(q);
    __syncthreads();
    if (s.abort) { aborted = true; break; }
    if (tid == 0 && q + MRAW <= last_plane && q + MRAW > issued) issue(q + MRAW);
  }

  const int tx = tid % MTX, ty = tid / MTX;
  const int i = i0 + tx, j = j0 + ty;
  const bool cell_ok = (ty < MTY) && (i <= p.nx) && (j <= p.ny);
  float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
  unsigned nsingle = 0;  // stage 2 with the surrogate: cells cooled in a single step
  const float cT = p.f_cT;
  const float inv_muamu = p.f_inv_muamu;
  const float etaf = p.f_eta;
  const float hdx = p.f_hdx, hdy = p.f_hdy, hdz = p.f_hdz;

  // k = k0 - 1 computes only the z face below the chunk, through the same
  // (single) copy of the face code as every other plane, so that a cell's
  // arithmetic does not depend on where the z-chunks begin
  for (int k = k0 - 1; k <= k1 && !aborted; ++k) {
    const bool first = k < k0;
    // Global operands of this cell's update, requested now so that their
    // latency hides behind the conversion and face phases.
    const long long c = L.at(i, j, k);
    double uc[5];
    float lv[5];
    double ph[6];
    bool queued = false;  // stage 2 with the surrogate: handed to the cooling passes
    if (cell_ok && !first) {
#pragma unroll
      for (int e = 0; e < 5; ++e) uc[e] = a.uold[e * L.plane + c];
      if (STAGE == 2) {
#pragma unroll
        for (int e = 0; e < 5; ++e) lv[e] = a.lapf[e * L.plane + c];
      }
      if (p.gravity) {
        ph[0] = a.phi[c + 1]; ph[1] = a.phi[c - 1];
        ph[2] = a.phi[c + L.px]; ph[3] = a.phi[c - L.px];
        ph[4] = a.phi[c + pxy]; ph[5] = a.phi[c - pxy];
      }
    }
    if (!first) {
      wait_plane(k + H);
      // stage 1: the previous plane's Laplacian read the ring slot this
      // conversion overwrites (a 3-plane ring)
      if (STAGE == 1) __syncthreads();
      convert(k + H);
      __syncthreads();  // S1
      if (s.abort) { aborted = true; break; }
      if (tid == 0 && k + H + MRAW <= last_plane && k + H + MRAW > issued) issue(k + H + MRAW);
    }
    faces(k, !first);
    __syncthreads();  // S2
    if (first) continue;

    if (cell_ok) {
      const int cur = (k + 1) & 1, prv = k & 1;
      float dU[5];
#pragma unroll
      for (int e = 0; e < 5; ++e)
        dU[e] = dtdx * (s.fx[e][ty][tx + 1] - s.fx[e][ty][tx]) + dtdy * (s.fy[e][ty + 1][tx] - s.fy[e][ty][tx]) +
                dtdz * (s.fz[cur][e][ty][tx] - s.fz[prv][e][ty][tx]);
      if (p.gravity) {
        float w[5], sv[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) w[e] = s.prm[k & 3][e][ty + 2][tx + 2];
        const float fg1 = (d2f(ph[0]) - d2f(ph[1])) * hdx;
        const float fg2 = (d2f(ph[2]) - d2f(ph[3])) * hdy;
        const float fg3 = (d2f(ph[4]) - d2f(ph[5])) * hdz;
        sv[0] = 0.0f;
        sv[1] = -w[0] * fg1;
        sv[2] = -w[0] * fg2;
        sv[3] = -w[0] * fg3;
        sv[4] = -w[0] * (w[1] * fg1 + w[2] * fg2 + w[3] * fg3);
#pragma unroll
        for (int e = 0; e < 5; ++e) dU[e] -= dtf * sv[e];
      }
      // FP64 accumulation: U' = U - dU (Godunov's centre value is U in both
      // stages; `uold` is the stage-1 input and the stage-2 old state)
      // Stage 2 away from the boundaries and the winds (which read or
      // overwrite UP): U = U_old - dU + eta Lap in one FP64 addition of the
      // FP32 increment (an FP64 addition costs ~64 FP32 slots on GB300).
      // (the gate also keeps the winds' FP64 distance and density, which the
      // compiler would otherwise evaluate for every cell, off the FP64 pipe)
      const bool special = near_boundary_or_wind(p, i, j, k);
      const bool plain2 = STAGE == 2 && !special;
      double up[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) up[e] = plain2 ? uc[e] : uc[e] - f2d(dU[e]);
      if (STAGE == 1) {
        // step's viscosity, eta * (sum of the 6 neighbours - 6 U), of the U
        // this stage streams (= the old U of stage 2), in FP32 from the ring
        const int a0 = cu_slot(k - 1), a1 = cu_slot(k), a2 = cu_slot(k + 1);
        const int lx = tx + 2, ly = ty + 2;
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          const float lap = ((s.cu[a1][e][ly][lx + 1] + s.cu[a1][e][ly][lx - 1]) +
                             (s.cu[a1][e][ly + 1][lx] + s.cu[a1][e][ly - 1][lx])) +
                            ((s.cu[a2][e][ly][lx] + s.cu[a0][e][ly][lx]) - 6.0f * s.cu[a1][e][ly][lx]);
          a.lapf[e * L.plane + c] = etaf * lap;
        }
      }
      if (special) {
        write_ghosts(p, L, a.out, STAGE == 1 ? 2 : 1, i, j, k, up);
        winds_cell(p, i, j, k, up);
      }
      if (STAGE == 1) {
#pragma unroll
        for (int e = 0; e < 5; ++e) a.out[e * L.plane + c] = up[e];
      } else {
        // step: U = UP + eta * (Laplacian of the old U), from stage 1
        double un[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) un[e] = plain2 ? up[e] + f2d(lv[e] - dU[e]) : up[e] + f2d(lv[e]);
        float cf[5], w[5];
        mixed_cell(gm1, un, 1, cf, w);  // calc_prims(UPrim, U)
        if (p.cooling == COOL_MLP) {
          // A cell whose tau (Lambda n^2 dt / E_th, formed as the cooling
          // passes form it) is at most the integrator's sub-step takes the
          // exact integrator's single exponential step here (the passes would
          // do the same); the passes cool the others and take their signal
          // speeds.
          const float T = (w[4] / w[0]) * cT;
          if (cools_at(p, T, un)) {
            const float nd = w[0] * inv_muamu;
            const float eth = w[4] / gm1;
            const float lam = cool_coef_f(p.cool, T);
            const float tau = (lam * nd) * (nd / eth) * dtstep_f;
            if (tau > p.f_cool_sub_frac) {
              queued = true;
            } else {
              cool_cell_f(p, cT, inv_muamu, gm1, w, un[4], dtstep_f, un);
              ++nsingle;
            }
          }
        } else if (p.cooling != COOL_NONE) {
          cool_cell_f(p, cT, inv_muamu, gm1, w, un[4], dtstep_f, un);
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
    }
    if (STAGE == 2 && p.cooling == COOL_MLP) {
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

  double d0 = f2d(m0), d1 = f2d(m1), d2 = f2d(m2);
  if (aborted) {
    if (tid == 0) {
      atomicOr(&clk->status, ST_TIMEOUT);
      for (int q = waited + 1; q <= issued; ++q) {
        const int slot = raw_slot(q);
        mbar_wait_bounded(&s.bar[slot], (phase >> slot) & 1u, WAIT_LIMIT);
        phase ^= 1u << slot;
      }
    }
    d0 = d1 = d2 = NAN;
  }
  if (STAGE == 2 && p.cooling == COOL_MLP && a.cool_counts) {
    unsigned v = nsingle;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((tid & 31) == 0 && v) atomicAdd(&a.cool_counts[2], (unsigned long long)v);
  }
  if (STAGE == 2) {
    if (p.cooling != COOL_MLP) {
      cfl_reduce_finalize_n<MNT>(d0, d1, d2, clk, p, true, s.red, &s.flag, nblk);
    } else {
      // with the surrogate the cooling passes finish the reduction over
      // these block maxima and their own
      cfl_contribute<MNT>(d0, d1, d2, clk, s.red);
    }
  }
}

template <int STAGE, int LIM = -1, int SOLV = -1>
__global__ void __launch_bounds__(MNT, MIXED_BLOCKS_PER_SM)
    stage_kernel_mixed(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ StageArgs a) {
  extern __shared__ __align__(128) unsigned char smem_bytes[];
  MixedSmem& s = *reinterpret_cast<MixedSmem*>(smem_bytes);
  mixed_tile<STAGE, LIM, SOLV>(&tm_in, a, s, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x * gridDim.y * gridDim.z,
                    blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z));
}

}  // namespace tlq
