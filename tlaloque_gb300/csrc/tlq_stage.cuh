// tlq_stage.cuh -- the two fused stage kernels of one hydrodynamic step.
//
// STAGE 1 = HLL[C]Fluxes(U, ..., 1) + Godunov(UPP, U, ..., dt/2) + borders(UPP, 2)
//           (source/mainHD.f90:76-82)
// STAGE 2 = calc_prims(UPP) + HLL[C]Fluxes(UPP, ..., 2) + Godunov(UP, U, ..., dt)
//           + borders(UP, 1) + step + calc_prims(U) + cooling + time_step
//           (source/mainHD.f90:84-97 and the next iteration's :74)
//
// A block owns a TX x TY column tile of interior cells and marches along z
// through a chunk of planes.  One elected thread streams planes of the input
// state (all 5 conserved variables, tile + 2-cell halo) into a 4-slot shared
// ring with 4-D TMA tensor loads completing on mbarriers; the block converts
// each plane to primitives once, computes every x/y/z face flux of the plane
// once (one flat, direction-generic task list), and applies the conservative
// update, sources, ghost fill, viscosity and cooling per cell.
#pragma once

#include "tlq_device.cuh"

namespace tlq {

constexpr int TX = 16, TY = 8, NT = TX * TY;
constexpr int HX = TX + 4, HY = TY + 4;  // halo-2 box
constexpr int PLANE_BOX = HY * HX;

// Tile of the mixed-form kernels (its own constants, so that it can be tuned
// apart from the plain form's): MTX x MTY columns on MNT threads, a multiple
// of 16 columns wide (the FP32 box of a tile starts on a 64-byte boundary).
#ifndef TLQ_MTX
#define TLQ_MTX 16
#endif
#ifndef TLQ_MTY
#define TLQ_MTY 8
#endif
#ifndef TLQ_MNT
#define TLQ_MNT 128
#endif
constexpr int MTX = TLQ_MTX, MTY = TLQ_MTY, MNT = TLQ_MNT;
constexpr int MHX = MTX + 4, MHY = MTY + 4;  // halo-2 box
static_assert(MTX * MTY <= MNT, "one cell per thread");
static_assert(MTX % 16 == 0 && MNT % 32 == 0, "tile shape");
constexpr int NRING = 4;
constexpr long long WAIT_LIMIT = 1LL << 24;  // mbarrier polls before giving up

struct StageArgs {
  Params p;
  Layout L;
  const double* uold;  // STAGE 2: U at the start of the step (Godunov centre, viscosity)
  double* out;         // STAGE 1: UPP; STAGE 2: U of the next step
  double* pout;        // STAGE 2 with cooling: carried (cooled) interior pressure
  const double* phi;   // point-mass potential plane (null without gravity)
  const float* phif;   // mixed form: the same potential rounded to FP32 (what its kernels read)
  Clock* clk;          // time, and the CFL reduction's ticket and maxima
  int zlen;            // planes per block
  int use_p;           // STAGE 1 with cooling: interior pressure from the P plane
  float* lapf;         // mixed form: eta * Laplacian of U (FP32, written by stage 1, read by stage 2)
  float* uppf;         // mixed form, STAGE 1: UPP as FP32 primitives (rho, u, v, w, p), read by stage 2
  unsigned* cqueue;    // mixed form with the cooling surrogate: stage 2 queues the cells that cool
  unsigned* cqcount;   // (beyond a single step of the exact integrator, which it takes itself)
  unsigned long long* cool_counts;  // [2]: the cells stage 2 cooled in a single step
};

template <class R>
struct StageSmem {
  double raw[NRING][5 * PLANE_BOX];  // TMA landing zone (conserved, FP64)
  double praw[NRING][PLANE_BOX];     // TMA landing zone (carried pressure)
  R prm[NRING][5][HY][HX];           // primitives of the ring planes
  R fx[5][TY][TX + 1];               // x-face fluxes of the current plane
  R fy[5][TY + 1][TX];               // y-face fluxes of the current plane
  R fz[2][5][TY][TX];                // z-face fluxes k-1/2, k+1/2
  uint64_t bar[NRING];
  double red[96];
  int flag;
  int abort;
};

// Ghost targets of one interior cell along one axis (boundaries.f90 non-MPI
// branches).  layers = 1: boundariesI (:183-257); layers = 2: boundariesII
// (:433-531).  Returns the number of (target index, flip) pairs.
__device__ __forceinline__ int ghost_targets(int layers, int bclo, int bchi, int c, int n, int* tgt, int* flip) {
  int m = 0;
  if (bclo == BC_OUTFLOW) {
    if (c == 1) { tgt[m] = 0; flip[m++] = 0; if (layers == 2) { tgt[m] = -1; flip[m++] = 0; } }
  } else if (bclo == BC_REFLECTIVE) {
    if (c == 1) { tgt[m] = 0; flip[m++] = 1; }
    if (layers == 2 && c == 2) { tgt[m] = -1; flip[m++] = 1; }
  } else if (bclo == BC_PERIODIC) {
    if (c == n) { tgt[m] = 0; flip[m++] = 0; }
    if (layers == 2 && c == n - 1) { tgt[m] = -1; flip[m++] = 0; }
  }
  if (bchi == BC_OUTFLOW) {
    if (c == n) { tgt[m] = n + 1; flip[m++] = 0; if (layers == 2) { tgt[m] = n + 2; flip[m++] = 0; } }
  } else if (bchi == BC_REFLECTIVE) {
    if (c == n) { tgt[m] = n + 1; flip[m++] = 1; }
    if (layers == 2 && c == n - 1) { tgt[m] = n + 2; flip[m++] = 1; }
  } else if (bchi == BC_PERIODIC) {
    if (c == 1) { tgt[m] = n + 1; flip[m++] = 0; }
    if (layers == 2 && c == 2) { tgt[m] = n + 2; flip[m++] = 0; }
  }
  return m;
}

// Write the face-ghost images of cell (i, j, k), whose value (before the
// wind overwrite) is v, into `out`, then apply the winds at each ghost cell
// (borders applies user_boundaries after the face fill).
__device__ __forceinline__ void write_ghosts(const Params& p, const Layout& L, double* out, int layers, int i, int j,
                                             int k, const double* v) {
  const int c3[3] = {i, j, k};
  const int n3[3] = {p.nx, p.ny, p.nz};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    int tgt[4], flp[4];
    const int m = ghost_targets(layers, p.bc[2 * ax], p.bc[2 * ax + 1], c3[ax], n3[ax], tgt, flp);
    for (int q = 0; q < m; ++q) {
      int g3[3] = {i, j, k};
      g3[ax] = tgt[q];
      double g[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) g[e] = (flp[q] && e == ax + 1) ? -v[e] : v[e];
      winds_cell(p, g3[0], g3[1], g3[2], g);
      const long long o = L.at(g3[0], g3[1], g3[2]);
#pragma unroll
      for (int e = 0; e < 5; ++e) out[e * L.plane + o] = g[e];
    }
  }
}

template <int STAGE, class R>
__global__ void __launch_bounds__(NT, 2)
    stage_kernel(const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_p, StageArgs a) {
  constexpr int H = STAGE;  // reconstruction halo: 1st order needs 1 cell, 2nd order 2
  extern __shared__ __align__(128) unsigned char smem_bytes[];
  StageSmem<R>& s = *reinterpret_cast<StageSmem<R>*>(smem_bytes);
  const Params& p = a.p;
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const int bx = blockIdx.x, by = blockIdx.y;
  const int i0 = 1 + bx * TX, j0 = 1 + by * TY;
  const int k0 = 1 + (int)blockIdx.z * a.zlen;
  const int k1 = min(p.nz, k0 + a.zlen - 1);
  Clock* clk = a.clk;

  if (!(clk->t < clk->tfin)) return;  // the loop condition of mainHD.f90:61 (uniform)
  const double dtstep = clk->dt;
  const double dt = (STAGE == 1) ? dtstep / 2.0 : dtstep;  // dth = dt/2.0 (mainHD.f90:78)
  const double dtdx = dt / p.dx, dtdy = dt / p.dy, dtdz = dt / p.dz;
  const uint32_t box_bytes = 5u * PLANE_BOX * 8u + (a.use_p ? PLANE_BOX * 8u : 0u);
  const int last_plane = k1 + H;

  if (tid == 0) {
    for (int q = 0; q < NRING; ++q) mbar_init(&s.bar[q], 1);
    s.abort = 0;
    fence_mbar_init();
  }
  __syncthreads();

  int issued = k0 - H - 1;  // last plane issued (meaningful in thread 0)
  auto issue = [&](int q) {  // thread 0: plane q of the input into slot q & 3
    const int slot = q & 3;
    fence_proxy_async();
    mbar_arrive_expect_tx(&s.bar[slot], box_bytes);
    tma_load_4d(s.raw[slot], &tm_in, &s.bar[slot], bx * TX, by * TY, q + 1, 0);
    if (a.use_p) tma_load_4d(s.praw[slot], &tm_p, &s.bar[slot], bx * TX, by * TY, q + 1, 0);
    issued = q;
  };
  // Every thread waits for every plane in order and tracks the slot phases.
  uint32_t phase = 0;
  int waited = k0 - H - 1;  // last plane this thread saw land
  bool failed = false;
  auto wait_plane = [&](int q) {
    if (failed) return;
    const int slot = q & 3;
    if (!mbar_wait_bounded(&s.bar[slot], (phase >> slot) & 1u, WAIT_LIMIT)) {
      failed = true;
      s.abort = 1;
      return;
    }
    phase ^= 1u << slot;
    waited = q;
  };

  // Primitives of plane q on the cross-shaped region the faces read.
  auto convert = [&](int q) {
    const int slot = q & 3;
    constexpr int RW = TX + 2 * H;
    constexpr int NROW = RW * TY, NCOL = TX * 2 * H;
    for (int t = tid; t < NROW + NCOL; t += NT) {
      int lx, ly;
      if (t < NROW) {
        lx = 2 - H + t % RW;
        ly = 2 + t / RW;
      } else {
        const int u = t - NROW, r2 = u / TX;
        lx = 2 + u % TX;
        ly = (r2 < H) ? (2 - H + r2) : (TY + 2 + r2 - H);
      }
      const double* r = &s.raw[slot][ly * HX + lx];
      R u[5], w[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) u[e] = (R)r[e * PLANE_BOX];
      cons2prim(R(p.gamma), u, w);
      if (a.use_p) {
        const int i = i0 - 2 + lx, j = j0 - 2 + ly;
        if (i >= 1 && i <= p.nx && j >= 1 && j <= p.ny && q >= 1 && q <= p.nz) w[4] = (R)s.praw[slot][ly * HX + lx];
      }
#pragma unroll
      for (int e = 0; e < 5; ++e) s.prm[slot][e][ly][lx] = w[e];
    }
  };

  // Face fluxes: x and y faces of plane k (when xy) and the z face k+1/2.
  auto faces = [&](int k, bool xy) {
    constexpr int NXF = (TX + 1) * TY, NYF = TX * (TY + 1), NZF = TX * TY;
    const int tbeg = xy ? 0 : NXF + NYF;
    const int sk = k & 3;
    constexpr int VS = PLANE_BOX;  // variable stride in prm and raw
    for (int t = tbeg + tid; t < NXF + NYF + NZF; t += NT) {
      int d, fxl, fyl;
      const R *w0, *w1, *w2, *w3;
      const double *uL, *uR;
      bool valid;
      if (t < NXF) {
        d = 1;
        fxl = t % (TX + 1);
        fyl = t / (TX + 1);
        const int ly = fyl + 2;
        w0 = &s.prm[sk][0][ly][fxl];
        w1 = w0 + 1; w2 = w0 + 2; w3 = w0 + 3;
        uL = &s.raw[sk][ly * HX + fxl + 1];
        uR = uL + 1;
        valid = (i0 - 1 + fxl <= p.nx) && (j0 + fyl <= p.ny);
      } else if (t < NXF + NYF) {
        d = 2;
        const int u = t - NXF;
        fxl = u % TX;
        fyl = u / TX;
        const int lx = fxl + 2;
        w0 = &s.prm[sk][0][fyl][lx];
        w1 = w0 + HX; w2 = w0 + 2 * HX; w3 = w0 + 3 * HX;
        uL = &s.raw[sk][(fyl + 1) * HX + lx];
        uR = uL + HX;
        valid = (i0 + fxl <= p.nx) && (j0 - 1 + fyl <= p.ny);
      } else {
        d = 3;
        const int u = t - NXF - NYF;
        fxl = u % TX;
        fyl = u / TX;
        const int lx = fxl + 2, ly = fyl + 2;
        w0 = &s.prm[(k - 1) & 3][0][ly][lx];
        w1 = &s.prm[k & 3][0][ly][lx];
        w2 = &s.prm[(k + 1) & 3][0][ly][lx];
        w3 = &s.prm[(k + 2) & 3][0][ly][lx];
        uL = &s.raw[k & 3][ly * HX + lx];
        uR = &s.raw[(k + 1) & 3][ly * HX + lx];
        valid = (i0 + fxl <= p.nx) && (j0 + fyl <= p.ny);
      }
      if (!valid) continue;
      R wll[5], wl[5], wr[5], wrr[5], UL[5], UR[5], ff[5];
#pragma unroll
      for (int e = 0; e < 5; ++e) {
        wl[e] = w1[e * VS];
        wr[e] = w2[e * VS];
        UL[e] = (R)uL[e * VS];
        UR[e] = (R)uR[e * VS];
      }
      if (STAGE == 2) {
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          wll[e] = w0[e * VS];
          wrr[e] = w3[e * VS];
        }
        limiter(wll, wl, wr, wrr, p.limiter);
      }
      if (!riemann(p.solver, R(p.gamma), R(p.g1), ff, wl, wr, UL, UR, d)) {
#pragma unroll
        for (int e = 0; e < 5; ++e) ff[e] = R(NAN);
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

  // ---- prologue: planes k0-H .. k0+H-1 and the z face k0-1/2 ---------------
  if (tid == 0)
    for (int q = k0 - H; q <= min(k0 - H + 3, last_plane); ++q) issue(q);
  for (int q = k0 - H; q <= k0 + H - 1; ++q) wait_plane(q);
  __syncthreads();
  const bool aborted0 = s.abort != 0;
  if (!aborted0)
    for (int q = k0 - H; q <= k0 + H - 1; ++q) convert(q);
  __syncthreads();
  if (!aborted0) faces(k0 - 1, false);
  __syncthreads();
  if (STAGE == 2 && tid == 0 && !aborted0 && k0 + 2 <= last_plane) issue(k0 + 2);

  const int tx = tid % TX, ty = tid / TX;
  const int i = i0 + tx, j = j0 + ty;
  const bool cell_ok = (i <= p.nx) && (j <= p.ny);
  double m0 = 0.0, m1 = 0.0, m2 = 0.0;  // CFL maxima (STAGE 2)

  bool aborted = aborted0;
  for (int k = k0; k <= k1 && !aborted; ++k) {
    wait_plane(k + H);
    convert(k + H);   // reads garbage only if the wait gave up; discarded below
    __syncthreads();  // S1
    if (s.abort) { aborted = true; break; }
    if (tid == 0 && k + 3 <= last_plane && k + 3 > issued) issue(k + 3);
    faces(k, true);
    __syncthreads();  // S2

    if (cell_ok) {
      const int cur = (k + 1) & 1, prv = k & 1;
      const long long c = L.at(i, j, k);
      double uc[5], up[5];
      if (STAGE == 1) {
#pragma unroll
        for (int e = 0; e < 5; ++e) uc[e] = s.raw[k & 3][e * PLANE_BOX + (ty + 2) * HX + tx + 2];
      } else {
#pragma unroll
        for (int e = 0; e < 5; ++e) uc[e] = a.uold[e * L.plane + c];
      }
#pragma unroll
      for (int e = 0; e < 5; ++e)
        up[e] = uc[e] - dtdx * ((double)s.fx[e][ty][tx + 1] - (double)s.fx[e][ty][tx]) -
                dtdy * ((double)s.fy[e][ty + 1][tx] - (double)s.fy[e][ty][tx]) -
                dtdz * ((double)s.fz[cur][e][ty][tx] - (double)s.fz[prv][e][ty][tx]);
      if (p.gravity) {  // Godunov's + dt*S (source/HLLC.f90:39-41)
        const double* ph = a.phi;
        const long long pxy = (long long)L.px * L.nyg;
        double w[5], sv[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) w[e] = (double)s.prm[k & 3][e][ty + 2][tx + 2];
        gravity_cell(p, w, ph[c + 1] - ph[c - 1], ph[c + L.px] - ph[c - L.px], ph[c + pxy] - ph[c - pxy], sv);
#pragma unroll
        for (int e = 0; e < 5; ++e) up[e] = up[e] + dt * sv[e];
      }
      // borders: face ghosts from the pre-wind value, then the winds (only
      // cells near a face or in a wind's box can be concerned; the gate also
      // keeps the winds' distance arithmetic from being evaluated everywhere)
      if (near_boundary_or_wind(p, i, j, k)) {
        write_ghosts(p, L, a.out, STAGE == 1 ? 2 : 1, i, j, k, up);
        winds_cell(p, i, j, k, up);
      }
      if (STAGE == 1) {
#pragma unroll
        for (int e = 0; e < 5; ++e) a.out[e * L.plane + c] = up[e];
      } else {
        // step: U = UP + eta*(sum of the 6 neighbours of the old U - 6 U_old)
        const long long pxy = (long long)L.px * L.nyg;
        double un[5], w[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) {
          const double* uo = a.uold + e * L.plane + c;
          un[e] = up[e] + p.eta * (uo[1] + uo[-1] + uo[L.px] + uo[-L.px] + uo[pxy] + uo[-pxy] - 6.0 * uc[e]);
        }
        cons2prim(p.gamma, un, w);  // calc_prims(UPrim, U)
        if (p.cooling != COOL_NONE) {
          cool_cell(p, w, un[4], dtstep);
          a.pout[c] = w[4];
        }
        if (!(un[0] > 0.0)) atomicOr(&clk->status, ST_NEG_DENSITY);
#pragma unroll
        for (int e = 0; e < 5; ++e) a.out[e * L.plane + c] = un[e];
        double v3[3];
        signal_speeds(p.gamma, w, v3);
        m0 = max_nan(m0, v3[0]);
        m1 = max_nan(m1, v3[1]);
        m2 = max_nan(m2, v3[2]);
      }
    }
  }

  if (aborted) {
    // Let the copies still in flight land (bounded) before the block exits,
    // and poison this block's CFL maxima so that the step reports it.
    if (tid == 0) {
      atomicOr(&clk->status, ST_TIMEOUT);
      for (int q = waited + 1; q <= issued; ++q) {
        const int slot = q & 3;
        mbar_wait_bounded(&s.bar[slot], (phase >> slot) & 1u, WAIT_LIMIT);
        phase ^= 1u << slot;
      }
    }
    m0 = m1 = m2 = NAN;
  }
  if (STAGE == 2) cfl_reduce_finalize<NT>(m0, m1, m2, clk, p, true, s.red, &s.flag);
}

}  // namespace tlq
