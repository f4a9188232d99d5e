// tlq_gravity.cu -- self-gravity: the reference's MultiGrid
// (source/sources.f90:99-485) and its multipole boundary values (:531-787)
// on the GPU, run before each stage like Godunov's (HLLC.f90:15-24):
// MultiGrid on the density of the step's U, PHIT = PHIP + PHI, and the
// stage's source term from PHIT.
//
// The mesh is a cube of N = 2^L cells (the reference's lvlm = size); level l
// holds n = N/2^l cells and three arrays (the error E, the residue R and the
// scratch T of the reference's Error/Residue/ret), each (n+2)^3 doubles with
// one ghost layer, index i + (n+2) (j + (n+2) k), i in 0..n+1 -- the layout
// of the reference's level arrays and of phi(0:nx+1, ...).
//
// The smoother is the reference's, in its order.  Its two half-sweeps split
// the cells by k parity and s(i, j) = [i even and j odd] (the reference's
// parity test states that one condition twice), so within a half-sweep a
// cell with s = 0 reads the new value of its x neighbour in rows of even j
// and of its y neighbour in columns of odd i: a Gauss-Seidel order along i
// and j.  A block walks a plane's anti-diagonals i + j = d in order, and
// every other neighbour (east, north, the k planes, the source) still holds
// its value from before the half-sweep.  A relax's ten half-sweeps run in one
// cooperative launch, skewed by a few diagonals per half-sweep, each plane's
// block checking its neighbour planes' progress (k_mg_relax_plane with the
// plane in shared memory up to 128 cells, k_mg_relax_pipe from the level
// arrays above; k_mg_half, one launch per half-sweep, where the planes cannot
// all be resident).  With the order kept and FP64 without contraction, every
// level is bit-identical to a sequential restatement; only the stopping
// test's sum |dphi| is summed in another order (it decides only whether the
// next V-cycle runs).
//
// The reference's loop test (Dif > 10 and fewer than 31 cycles) runs on the
// device, so the solve needs no host round trip: in a CUDA graph the
// V-cycles are the body of a while node whose condition that test sets; run
// directly, a fixed sequence of 31 cycle slots whose launches return once
// the test failed.  Levels of at most 4 cells run inside one block (one
// launch per cycle).
//
// Built with -fmad=false (FP64 as the restatement evaluates it).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>

#include "tlq_convert.cuh"
#include "tlq_ctx.h"

namespace tlq {
namespace {

constexpr int MG_MAXL = 11;         // levels 0..10: meshes up to 1024^3
constexpr int MG_COARSE_N = 4;      // levels of at most this many cells run in the one-block kernel
constexpr int MG_CYCLES = 31;       // the reference's V-cycle cap (sources.f90:140)
constexpr int MG_PF = 4;            // diagonal steps the smoother's loads run ahead
constexpr int MG_MOM_THREADS = 256;
constexpr int MG_MOM_BLOCKS = 152 * 2;
constexpr int MG_SOLVE_LIMIT = 100000;  // coarsest-level Gauss-Seidel passes before giving up
// Polls of a neighbour's progress before a pipelined relax gives up (~1 s);
// TLQ_MG_WAIT_LIMIT in the environment of tlq_create overrides it (a short
// limit lets a test make the wait run out and check the error status).
constexpr long long MG_WAIT_LIMIT = 1LL << 24;

struct MgLevel {
  int n;
  double* E;
  double* R;
  double* T;   // source(i,j,k)*dxl**2 of the smoother, formed once with R
  double dxl;  // (xr - xl) / n (sources.f90:232; x extent for every axis, as there)
};

struct MgCtl {
  int run;     // this MultiGrid call runs (the step runs: t < tfin)
  int active;  // the current V-cycle runs
  int iter;    // V-cycles started
  int status;  // MG_ST_* bits
  double dif;  // the last smoother pass's summed |change| (the reference's Dif)
  double c0[5], cm[5][5], sm[5][5];  // multipole moments (sources.f90:599-681)
  double part[2 * 1024];             // per-plane partial sums of the last pass's |change|
  int abort;                         // a pipelined relax gave up waiting (sticky for the call)
  int prog[1026];                    // pipelined relax: plane k's last finished diagonal, hs*(2n+2) + d
  long long wait_limit;              // polls of a neighbour's progress before giving up (set at allocation)
};

__host__ __device__ __forceinline__ long long mgi(int n, int i, int j, int k) {
  return (long long)i + (long long)(n + 2) * ((long long)j + (long long)(n + 2) * (long long)k);
}

// Where the density of the step's state is read (U(1, 0:nx+1, ...)).
struct DensSoA {
  const double* U;
  Layout L;
  __device__ double operator()(int i, int j, int k) const { return U[L.at(i, j, k)]; }
};
struct DensAoS {
  const double* U;
  Aos A;
  __device__ double operator()(int i, int j, int k) const { return U[A.at(i, j, k)]; }
};

// ---------------------------------------------------------------------------
// Multipole boundary values (sources.f90:9-96, 558-787)
// ---------------------------------------------------------------------------
__device__ double powi(double x, int n) {  // x**n, run-time n: the binary method, as gfortran
  unsigned m = n < 0 ? (unsigned)(-n) : (unsigned)n;
  double y = (m % 2) ? x : 1.0;
  while (m >>= 1) {
    x = x * x;
    if (m % 2) y = y * x;
  }
  return n < 0 ? 1.0 / y : y;
}

__device__ double legendre(double x, int l) {
  const double x2 = x * x;
  switch (l) {
    case 0: return 1.0;
    case 1: return x;
    case 2: return 0.5 * (3.0 * x2 - 1.0);
    case 3: return 0.5 * (5.0 * (x2 * x) - 3.0 * x);
    default: return (1.0 / 8.0) * ((35.0 * (x2 * x2) - 30.0 * x2) + 3.0);
  }
}

// aLegendre with its (1 - x^2)^(1/2) and ^(3/2) as square roots (the
// reference raises to the real powers 1/2 and 3/2; equal up to rounding).
// |x| <= 1 here (x = z/r with r >= |z| in rounded arithmetic), so 1 - x^2 >= 0.
__device__ double alegendre(double x, int l, int m) {
  const double x2 = x * x, s = 1.0 - x2, q = sqrt(s);
  switch (l) {
    case 0: return 1.0;
    case 1: return m == 0 ? x : -q;
    case 2:
      if (m == 0) return 0.50 * (3.0 * x2 - 1.0);
      if (m == 1) return -(3.0 * x * q);
      return 3.0 * s;
    case 3:
      if (m == 0) return 0.50 * (5.0 * (x2 * x) - 3.0 * x);
      if (m == 1) return 1.5 * (1.0 - 5.0 * x2) * q;
      if (m == 2) return 15.0 * x * s;
      return -(15.0 * (s * q));
    default:
      if (m == 0) return (1.0 / 8.0) * ((35.0 * (x2 * x2) - 30.0 * x2) + 3.0);
      if (m == 1) return -(2.5 * (7.0 * (x2 * x) - 3.0 * x) * q);
      if (m == 2) return 7.5 * (7.0 * x2 - 1.0) * s;
      if (m == 3) return -(105.0 * x * (s * q));
      return 105.0 * (s * s);
  }
}

// The spherical quantities of the multipole terms at the centre of cell
// (i, j, k) (pangle, aangle, distance; one rank), by algebra instead of the
// reference's transcendental round trips: cos(theta) = z/r (it forms
// cos(acos(z/r))), and cos(m phi), sin(m phi) from cos phi = x/rho, sin phi
// = y/rho, rho = |(x, y)|, by the Chebyshev recurrence (it takes cos and sin
// of m atan2(y, x)).  Equal up to rounding; on the FP64 pipe these are a few
// operations instead of eleven transcendental functions per cell.
struct Sph {
  double coth, r, c[5], s[5];
};
__device__ Sph sph_terms(const Params& p, int i, int j, int k) {
  const double x = (p.xl + p.dx * (double)i) - p.dx / 2.0;
  const double y = (p.yl + p.dy * (double)j) - p.dy / 2.0;
  const double z = (p.zl + p.dz * (double)k) - p.dz / 2.0;
  Sph o;
  const double rho2 = x * x + y * y;
  o.r = sqrt(rho2 + z * z);
  o.coth = z / o.r;
  const double rho = sqrt(rho2);
  const double c1 = rho > 0.0 ? x / rho : 1.0, s1 = rho > 0.0 ? y / rho : 0.0;
  o.c[0] = 1.0;
  o.s[0] = 0.0;
  o.c[1] = c1;
  o.s[1] = s1;
#pragma unroll
  for (int m = 2; m <= 4; ++m) {
    o.c[m] = 2.0 * c1 * o.c[m - 1] - o.c[m - 2];
    o.s[m] = 2.0 * c1 * o.s[m - 1] - o.s[m - 2];
  }
  return o;
}

// 25 sums per block: c0 l = 0..4, then cm and sm for l = 1..4, m = 1..l.
template <class Dens>
__global__ void __launch_bounds__(MG_MOM_THREADS) k_mg_moments(const MgCtl* c, const Clock* clk, Params p, Dens rho,
                                                             double* part) {
  __shared__ double red[MG_MOM_THREADS / 32][25];
  if (!c->run || clk->it % 10 != 0) return;
  const int n = p.nx;
  const double vol = p.dx, vy = p.dy, vz = p.dz;
  double acc[25];
#pragma unroll
  for (int q = 0; q < 25; ++q) acc[q] = 0.0;
  const long long cells = (long long)n * n * n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < cells;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(q % n), j = 1 + (int)((q / n) % n), k = 1 + (int)(q / ((long long)n * n));
    const Sph sp = sph_terms(p, i, j, k);
    const double coth = sp.coth, r = sp.r;
    // the cell's mass once (the reference multiplies rho dx dy dz into every
    // term; the order of the products only changes the rounding)
    const double dm = rho(i, j, k) * vol * vy * vz;
    acc[0] += dm;  // Legendre(.,0) r**0 = 1
    int slot = 5;
    double rl = 1.0;
#pragma unroll
    for (int l = 1; l <= 4; ++l) {
      rl = rl * r;
      const double w = rl * dm;
      acc[l] += legendre(coth, l) * w;
#pragma unroll
      for (int m = 1; m <= l; ++m, ++slot) {
        const double t = alegendre(coth, l, m) * w;
        acc[slot] += t * sp.c[m];
        acc[slot + 10] += t * sp.s[m];
      }
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 25; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 25) {
    double v = 0.0;
    for (int q = 0; q < MG_MOM_THREADS / 32; ++q) v += red[q][threadIdx.x];
    part[blockIdx.x * 25 + threadIdx.x] = v;
  }
}

__global__ void k_mg_moments_final(MgCtl* c, const Clock* clk, const double* part, int nblocks) {
  // slots 5..14 (cm) and 15..24 (sm): (l, m) = (1,1) (2,1) (2,2) (3,1) .. (4,4)
  constexpr int LS[10] = {1, 2, 2, 3, 3, 3, 4, 4, 4, 4}, MS[10] = {1, 1, 2, 1, 2, 3, 1, 2, 3, 4};
  if (!c->run || clk->it % 10 != 0) return;
  const int q = threadIdx.x;
  if (q >= 25) return;
  double v = 0.0;
  for (int b = 0; b < nblocks; ++b) v += part[b * 25 + q];
  if (q < 5) {
    c->c0[q] = v;
    return;
  }
  const int r = q < 15 ? q - 5 : q - 15, l = LS[r], m = MS[r];
  const double cf = 2.0 * tgamma((double)(l - m) + 1.0) / tgamma((double)(l + m) + 1.0);
  if (q < 15)
    c->cm[l][m] = cf * v;
  else
    c->sm[l][m] = cf * v;
}

// phi_x/y/zboundaries: the six faces' ghost cells (edges untouched).
__global__ void k_mg_faces(const MgCtl* c, const Clock* clk, Params p, double* phi) {
  if (!c->run || clk->it % 10 != 0) return;
  const int n = p.nx;
  const long long per = (long long)n * n;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 6 * per;
       q += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(q / per);
    const int a = 1 + (int)((q % per) / n), b = 1 + (int)(q % n);
    const int bnd = (f & 1) ? n + 1 : 0;
    int i, j, k;
    if (f < 2) { i = bnd; j = a; k = b; }
    else if (f < 4) { i = a; j = bnd; k = b; }
    else { i = a; j = b; k = bnd; }
    const Sph sp = sph_terms(p, i, j, k);
    const double coth = sp.coth, rb = sp.r;
    double v = 0.0;
    v = v - c->c0[0] / rb;
    for (int l = 1; l <= 4; ++l) {
      v = v - c->c0[l] * legendre(coth, l) / powi(rb, l + 1);
      for (int m = 1; m <= l; ++m)
        v = v - 2.0 * (c->cm[l][m] * sp.c[m] + c->sm[l][m] * sp.s[m]) * alegendre(coth, l, m) / powi(rb, l + 1);
    }
    phi[mgi(n, i, j, k)] = 6.67430e-8 * v;
  }
}

// ---------------------------------------------------------------------------
// Cycle control
// ---------------------------------------------------------------------------
__global__ void k_mg_begin(MgCtl* c, const Clock* clk) {
  c->run = clk->t < clk->tfin;  // the loop test of mainHD.f90:61 (the step's)
  c->active = 0;
  c->iter = 0;
  c->dif = 1.e28;
  c->abort = 0;
}

// Residue(0) = 4 pi G dens, Error(0) = phi (sources.f90:136-137).
template <class Dens>
__global__ void k_mg_init(const MgCtl* c, Dens rho, int n, const double* phi, double* E0, double* R0, double* T0,
                          double dxl) {
  if (!c->run) return;
  const long long cells = (long long)(n + 2) * (n + 2) * (n + 2);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < cells;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % (n + 2)), j = (int)((q / (n + 2)) % (n + 2)), k = (int)(q / ((long long)(n + 2) * (n + 2)));
    const double r = 4.0 * 3.14159265358979 * 6.67430e-8 * rho(i, j, k);
    R0[q] = r;
    T0[q] = r * (dxl * dxl);
    E0[q] = phi[q];
  }
}

// The loop test of the V-cycles (sources.f90:140): another cycle while
// Dif > 10 and fewer than 31 ran; the error of every coarse level restarts
// at 0 (:146-148).
// (Every block decides from the same inputs; k_mg_cycle_flag updates them
// after this launch.)
__global__ void k_mg_cycle_begin(const MgCtl* c, double* Ecoarse, long long ncoarse) {
  __shared__ int go;
  if (threadIdx.x == 0) go = c->run && c->dif > 10.0 && c->iter < MG_CYCLES;
  __syncthreads();
  if (!go) return;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ncoarse;
       q += (long long)gridDim.x * blockDim.x)
    Ecoarse[q] = 0.0;
}

// The flag and the count, after every block of k_mg_cycle_begin has read
// the previous values.
__global__ void k_mg_cycle_flag(MgCtl* c) {
  const int go = c->run && c->dif > 10.0 && c->iter < MG_CYCLES;
  c->active = go;
  if (go) c->iter = c->iter + 1;
}

// The same loop test as the condition of a graph's loop node: the step's
// graph runs the V-cycles as the body of a while node, so that cycles after
// convergence are not launched at all.
__global__ void k_mg_loop_test(const MgCtl* c, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, (c->run && c->dif > 10.0 && c->iter < MG_CYCLES) ? 1u : 0u);
}

__global__ void k_mg_cycle_end(MgCtl* c, int nparts) {
  if (!c->active) return;
  double v = 0.0;
  for (int q = 0; q < nparts; ++q) v += c->part[q];
  c->dif = v;
}

// phi = Error(0) (sources.f90:189); PHIT = PHIP + PHI into the stage's
// potential plane (HLLC.f90:22).
// A solve that gave up (a bounded wait or the coarsest solve) marks the
// step's status as timed out.
__global__ void k_mg_end(const MgCtl* c, Clock* clk, int n, const double* E0, double* phig, const double* phip,
                         double* phit, float* phitf, Layout L) {
  if (!c->run) return;
  if (blockIdx.x == 0 && threadIdx.x == 0 && c->status) atomicOr(&clk->status, ST_TIMEOUT);
  const long long cells = (long long)(n + 2) * (n + 2) * (n + 2);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < cells;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % (n + 2)), j = (int)((q / (n + 2)) % (n + 2)), k = (int)(q / ((long long)(n + 2) * (n + 2)));
    const double v = E0[q];
    phig[q] = v;
    if (phit) {
      const long long o = L.at(i, j, k);
      const double pt = phip[o] + v;
      phit[o] = pt;
      if (phitf) phitf[o] = d2f(pt);  // the mixed form's stages read it in FP32
    }
  }
}

// ---------------------------------------------------------------------------
// Level operators
// ---------------------------------------------------------------------------
// One smoother update (sources.f90:378-379, 447-449), sdx = source*dxl**2.
// The reference's tail ((1/6) a) w + (1-w) old with w = 1 equals (1/6) a
// bit for bit unless that is a signed zero or old is not finite (then the
// 0*old term can change the sign or give a NaN): those take the literal
// expression, every other update saves its three FP64 operations (the FP64
// pipe bounds the smoother).
__device__ __forceinline__ double mg_new(double east, double west, double north, double south, double up, double down,
                                         double sdx, double old) {
  double a = east + west;
  a = a + north;
  a = a + south;
  a = a + up;
  a = a + down;
  a = a - sdx;
  double v = (1.0 / 6.0) * a;
  const long long vb = __double_as_longlong(v), ob = __double_as_longlong(old);
  if ((vb & 0x7fffffffffffffffLL) == 0 || ((ob >> 52) & 0x7ff) == 0x7ff) {
    const double w = 1.0;
    v = v * w + (1.0 - w) * old;
  }
  return v;
}

// Cells (i even, j odd) of plane k: none of them shares a face with another,
// so they update in any order (threads t of nt share them).
template <bool TRACK>
__device__ double mg_parallel_plane(const MgLevel& lv, int k, int t, int nt) {
  const int n = lv.n, h = n / 2;
  double acc = 0.0;
  for (int q = t; q < h * h; q += nt) {
    const int i = 2 * (q % h + 1), j = 2 * (q / h) + 1;
    const long long o = mgi(n, i, j, k), s1 = n + 2, s2 = (long long)(n + 2) * (n + 2);
    const double old = lv.E[o];
    const double v = mg_new(lv.E[o + 1], lv.E[o - 1], lv.E[o + s1], lv.E[o - s1], lv.E[o + s2], lv.E[o - s2], lv.T[o],
                            old);
    lv.E[o] = v;
    if (TRACK) acc += fabs(v - old);
  }
  return acc;
}

// The other cells of plane k (s = 0) in the reference's order: anti-diagonal
// d = i + j after anti-diagonal, thread i of the plane's group.  West (i-1,
// j) and south (i, j-1) lie on diagonal d-1: south is this thread's own last
// value, west its neighbour's (pub, double-buffered by diagonal parity).
// The loads of the other neighbours run MG_PF diagonals ahead.  Every thread
// of the block calls this with the same n (uniform barriers); i > n idles.
template <bool TRACK>
__device__ double mg_wave_plane(const MgLevel& lv, int k, int i, double* pub) {
  const int n = lv.n;
  const long long s1 = n + 2, s2 = (long long)(n + 2) * (n + 2);
  double* __restrict__ E = lv.E;
  const double* __restrict__ R = lv.T;
  double rc[MG_PF], re[MG_PF], rn[MG_PF], ru[MG_PF], rd[MG_PF], rs[MG_PF];
  const bool col = i >= 1 && i <= n;
#pragma unroll
  for (int q = 0; q < MG_PF; ++q) {
    const int j = 2 + q - i;
    if (col && j >= 1 && j <= n) {
      const long long o = mgi(n, i, j, k);
      rc[q] = E[o]; re[q] = E[o + 1]; rn[q] = E[o + s1]; ru[q] = E[o + s2]; rd[q] = E[o - s2]; rs[q] = R[o];
    }
  }
  double prev = 0.0, acc = 0.0;
  for (int d0 = 2; d0 <= 2 * n; d0 += MG_PF) {
#pragma unroll
    for (int q = 0; q < MG_PF; ++q) {
      const int d = d0 + q;
      if (d <= 2 * n) {
        const int j = d - i;
        if (col && j >= 1 && j <= n) {
          const long long o = mgi(n, i, j, k);
          const double west = i == 1 ? E[o - 1] : pub[((d - 1) & 1) * (n + 1) + i - 1];
          const double south = j == 1 ? E[o - s1] : prev;
          const double old = rc[q];
          double cur = old;
          if ((i & 1) || !(j & 1)) {  // s = 0: this half-sweep's cell
            cur = mg_new(re[q], west, rn[q], south, ru[q], rd[q], rs[q], old);
            E[o] = cur;
            if (TRACK) acc += fabs(cur - old);
          }
          pub[(d & 1) * (n + 1) + i] = cur;
          prev = cur;
        }
        const int jn = d + MG_PF - i;  // this slot's next diagonal
        if (col && jn >= 1 && jn <= n) {
          const long long o = mgi(n, i, jn, k);
          rc[q] = E[o]; re[q] = E[o + 1]; rn[q] = E[o + s1]; ru[q] = E[o + s2]; rd[q] = E[o - s2]; rs[q] = R[o];
        }
        __syncthreads();
      }
    }
  }
  return acc;
}

// Sum over the block (blockDim.x a multiple of 32), in a fixed order; the
// result in thread 0.
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
  return s;
}

// One half-sweep of a level above MG_COARSE_N cells: block b = plane k = b+1
// (n threads).  half 0: cells with k parity = s; half 1: the others
// (sources.f90:438-452 and :456-468).  part: where the plane's summed
// |change| goes (null: not needed).
template <int NT, bool TRACK>
__global__ void __launch_bounds__(NT) k_mg_half(const MgCtl* c, MgLevel lv, int half, double* part) {
  __shared__ double pub[2 * 1025];
  __shared__ double red[32];
  if (!c->active) return;
  const int k = blockIdx.x + 1;
  const int sk = (k & 1) ^ half;  // the s of this half-sweep's cells in plane k
  double acc;
  if (sk)
    acc = mg_parallel_plane<TRACK>(lv, k, threadIdx.x, blockDim.x);
  else
    acc = mg_wave_plane<TRACK>(lv, k, threadIdx.x + 1, pub);
  if (TRACK) {
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// ---------------------------------------------------------------------------
// A whole relax (5 passes of 2 half-sweeps) in one cooperative launch: block
// b owns plane k = b+1 through all ten half-sweeps, so the half-sweeps of
// neighbouring planes overlap instead of running one after another.  Plane
// k may start diagonals d0..d1 of half-sweep hs once planes k-1 and k+1 have
// finished diagonal d1+1 of half-sweep hs-1: every value it reads from them
// (the cells (i, j, k+-1), i + j <= d1) then holds its hs-1 value, and every
// cell of theirs that reads one of plane k's cells it is about to change
// (the same (i, j)) has read it.  The waits are bounded; a block that gives
// up sets the status and the abort flag and every block leaves.  Values of
// other planes are loaded around L1 (ld.global.cg: L1 is not coherent
// between the SMs of one launch).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }

// Thread 0 waits until planes k-1, k+1 (those in 1..n) reach `need`; false
// when it gave up (the block then leaves the relax).
__device__ bool mg_wait(MgCtl* c, int k, int n, int need, int* s_ok) {
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile int* prog = c->prog;
    volatile int* abort = &c->abort;
    for (int nb = k - 1; nb <= k + 1 && ok; nb += 2) {
      if (nb < 1 || nb > n) continue;
      long long tries = 0;
      while (prog[nb] < need) {
        if (*abort || ++tries > c->wait_limit) {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    if (!ok) {
      atomicOr(&c->status, MG_ST_TIMEOUT);
      atomicExch(&c->abort, 1);
    }
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

__device__ __forceinline__ void mg_publish(MgCtl* c, int k, int value) {
  __syncthreads();  // every thread's stores of the chunk are issued
  if (threadIdx.x == 0) {
    __threadfence();
    atomicExch(&c->prog[k], value);
  }
}

// Time step t of a block processes diagonal d = t - SKEW hs of every
// half-sweep hs at once: a cell of half-sweep hs reads its own plane's
// cells of half-sweep hs-1 on diagonals d-1..d+1 (processed SKEW-1 steps or
// more earlier) and its neighbour planes' cells of hs-1 on diagonal d
// (their step t + 1 - SKEW), so the ten half-sweeps of a relax take
// 2n + 9 SKEW steps instead of 20n.  A plane checks its neighbours once per
// CH steps, which SKEW = CH + 1 allows.

size_t pipe_smem(int n) { return (size_t)10 * 2 * (n + 1) * sizeof(double); }

// NT threads at most, MINB blocks per SM at least, neighbour checks every
// CH steps; the block is n x HG threads: thread t works on one column for the
// K = 10/HG half-sweeps g K .. g K + K-1 of group g = t / n (more warps per
// plane to hide the FP64 latency), loading G of them at a time.  Columns by
// parity: the first n/2 threads of a group take the odd columns, the others
// the even ones.  A step's cells that do not change (the other colour's, or
// on an odd diagonal the wave cells of even columns) then fill whole warps
// (n >= 64), which skip the update: the FP64 pipe charges a warp instruction
// the same with 16 active lanes as with 32 (measured on GB300), so this
// saves a third of the smoother's FP64 issue.  The diagonal's values in
// shared memory are laid out by thread, odd columns first (pslot).
template <int NT, int MINB, int HG, int G, int CH, bool TRACK>
__global__ void __launch_bounds__(NT, MINB) k_mg_relax_pipe(MgCtl* c, MgLevel lv, double* part) {
  constexpr int K = 10 / HG;
  constexpr int SKEW = CH + 1;  // steps between consecutive half-sweeps: a neighbour check per CH steps
  static_assert(K * HG == 10, "HG divides the ten half-sweeps");
  extern __shared__ double pub[];  // per half-sweep, per diagonal parity: the diagonal's values by pslot
  __shared__ double red[32];
  __shared__ int s_ok;
  if (!c->active) return;
  const int n = lv.n, k = blockIdx.x + 1;
  // threads past n x HG (whole warps) only take part in the barriers
  const bool live = (int)threadIdx.x < n * HG;
  const int col = (int)(threadIdx.x % n), hn = n >> 1;
  const int i = col < hn ? 2 * col + 1 : 2 * (col - hn) + 2;
  const int h0 = live ? (int)(threadIdx.x / n) * K : 0;
  // slot of column ii in a diagonal's shared-memory values
  auto pslot = [hn](int ii) { return (ii & 1) ? (ii >> 1) : hn + (ii >> 1) - 1; };
  const long long s1 = n + 2, s2 = (long long)(n + 2) * (n + 2);
  double* __restrict__ E = lv.E;
  const double* __restrict__ Sd = lv.T;
  const int tmax = 2 * n + 9 * SKEW;
  double prev[K];
#pragma unroll
  for (int q = 0; q < K; ++q) prev[q] = 0.0;
  double acc8 = 0.0, acc9 = 0.0;
  for (int t0 = 2; t0 <= tmax; t0 += CH) {
    const int t1 = min(t0 + CH - 1, tmax);
    const int need = t1 + 1 - SKEW;  // the neighbours' last step this chunk reads
    if (need >= 2 && !mg_wait(c, k, n, need, &s_ok)) return;
    for (int t = t0; t <= t1; ++t) {
      // The loads of G half-sweeps before their stores: the cells a step
      // reads and the cells it writes lie SKEW diagonals or more apart,
      // so these loads need not wait behind those stores.
#pragma unroll
      for (int g = 0; g < K; g += G) {
      double rc[K], re[K], rn[K], ru[K], rd[K], rs[K], rw[K], rv[K];
#pragma unroll
      for (int q = g; q < (g + G < K ? g + G : K); ++q) {
        const int hs = h0 + q;
        const int d = t - SKEW * hs, j = d - i;
        if (live && d >= 2 && d <= 2 * n && j >= 1 && j <= n) {
          const long long o = mgi(n, i, j, k);
          const bool par = ((k & 1) ^ (hs & 1)) != 0;
          // whether the cell changes in this half-sweep (the wave cells that
          // do not still pass their value on through shared memory)
          const bool upd = par ? (!(i & 1) && (j & 1)) : ((i & 1) || !(j & 1));
          if (upd || !par) rc[q] = E[o];
          if (upd) {
            re[q] = E[o + 1]; rn[q] = E[o + s1];
            ru[q] = ldcg(E + o + s2); rd[q] = ldcg(E + o - s2); rs[q] = Sd[o];
            // west and south from memory: the parallel cells' (other colour,
            // this plane, hs-1) and the ghosts; the wave cells' others come
            // from this half-sweep's previous diagonal
            rw[q] = (par || i == 1) ? E[o - 1] : 0.0;
            rv[q] = (par || j == 1) ? E[o - s1] : 0.0;
          }
        }
      }
#pragma unroll
      for (int q = g; q < (g + G < K ? g + G : K); ++q) {
        const int hs = h0 + q;
        const int d = t - SKEW * hs;
        if (!live || d < 2 || d > 2 * n) continue;  // (uniform within the group)
        const int j = d - i;
        if (j < 1 || j > n) continue;
        const long long o = mgi(n, i, j, k);
        const bool par = ((k & 1) ^ (hs & 1)) != 0;  // cells (i even, j odd) of this plane
        const double old = rc[q];
        if (par) {
          if (!(i & 1) && (j & 1)) {
            const double v = mg_new(re[q], rw[q], rn[q], rv[q], ru[q], rd[q], rs[q], old);
            E[o] = v;
            if (TRACK && hs == 8) acc8 += fabs(v - old);
            if (TRACK && hs == 9) acc9 += fabs(v - old);
          }
        } else {
          double* pb = pub + hs * 2 * (n + 1);
          const double west = i == 1 ? rw[q] : pb[((d - 1) & 1) * (n + 1) + pslot(i - 1)];
          const double south = j == 1 ? rv[q] : prev[q];
          double cur = old;
          if ((i & 1) || !(j & 1)) {
            cur = mg_new(re[q], west, rn[q], south, ru[q], rd[q], rs[q], old);
            E[o] = cur;
            if (TRACK && hs == 8) acc8 += fabs(cur - old);
            if (TRACK && hs == 9) acc9 += fabs(cur - old);
          }
          pb[(d & 1) * (n + 1) + pslot(i)] = cur;
          prev[q] = cur;
        }
      }
      }
      __syncthreads();
    }
    mg_publish(c, k, t1);
  }
  if (TRACK) {
    const double a = block_sum(acc8, red);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
    const double b = block_sum(acc9, red);
    if (threadIdx.x == 0) part[n + blockIdx.x] = b;
  }
}

// ---------------------------------------------------------------------------
// The same skewed relax with the block's plane held in shared memory (levels
// up to 128 cells: (n+2)^2 doubles, 135 KB at 128).  Only plane k's block
// writes plane k during a relax, so its copy in shared memory is the current
// one: an update reads its old value and its four in-plane neighbours there
// (no L2 round trip per step and no diagonal buffers; the values are the
// same ones the reference's order gives, by the argument above), and
// writes the new value there and to the level array, where the neighbour
// planes read it.  The ghost rows and columns (i or j = 0, n+1) do not
// change during a relax.  Layout: column parity, row, column / 2, so that a
// warp's cells of one diagonal (consecutive columns of one parity) fall on
// distinct banks.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int plane_slot(int n, int i, int j) {
  return ((i & 1) * (n + 2) + j) * ((n >> 1) + 1) + (i >> 1);
}
size_t plane_smem(int n) { return (size_t)(n + 2) * (n + 2) * sizeof(double); }

template <int NT, int HG, int CH, bool TRACK>
__global__ void __launch_bounds__(NT, 1) k_mg_relax_plane(MgCtl* c, MgLevel lv, double* part) {
  constexpr int K = 10 / HG;
  constexpr int SKEW = CH + 1;
  static_assert(K * HG == 10, "HG divides the ten half-sweeps");
  extern __shared__ double P[];
  __shared__ double red[32];
  __shared__ int s_ok;
  if (!c->active) return;
  const int n = lv.n, k = blockIdx.x + 1;
  const long long s2 = (long long)(n + 2) * (n + 2), base = s2 * k;
  double* __restrict__ E = lv.E;
  const double* __restrict__ Sd = lv.T;
  for (int q = threadIdx.x; q < (n + 2) * (n + 2); q += blockDim.x)
    P[plane_slot(n, q % (n + 2), q / (n + 2))] = E[base + q];
  __syncthreads();
  const bool live = (int)threadIdx.x < n * HG;
  const int col = (int)(threadIdx.x % n), hn = n >> 1;
  const int i = col < hn ? 2 * col + 1 : 2 * (col - hn) + 2;  // odd columns first (whole idle warps)
  const int h0 = live ? (int)(threadIdx.x / n) * K : 0;
  const int R = hn + 1, PS = (n + 2) * R;  // row stride and size of one parity's array
  const int de = (i & 1) ? 1 - PS : PS, dw = (i & 1) ? -PS : PS - 1;  // east, west: the other parity
  const int tmax = 2 * n + 9 * SKEW;
  // one half-sweep's cell of a step: whether it changes, where it lies, and
  // its values from the level arrays (the planes above and below, the source)
  struct Fetch {
    double ru, rd, rs;
    long long og;
    int os;
    bool up;
  };
  auto fetch = [&](int t, Fetch* f) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const int hs = h0 + q, d = t - SKEW * hs, j = d - i;
      const bool par = ((k & 1) ^ (hs & 1)) != 0;  // cells (i even, j odd) of this plane
      f[q].up = live && d >= 2 && d <= 2 * n && j >= 1 && j <= n &&
                (par ? (!(i & 1) && (j & 1)) : ((i & 1) || !(j & 1)));
      if (f[q].up) {
        f[q].og = base + i + (long long)(n + 2) * j;
        f[q].os = plane_slot(n, i, j);
        f[q].ru = ldcg(E + f[q].og + s2);
        f[q].rd = ldcg(E + f[q].og - s2);
        f[q].rs = Sd[f[q].og];
      }
    }
  };
  double acc8 = 0.0, acc9 = 0.0;
  for (int t0 = 2; t0 <= tmax; t0 += CH) {
    const int t1 = min(t0 + CH - 1, tmax);
    const int need = t1 + 1 - SKEW;  // the neighbours' last step this chunk reads
    if (need >= 2 && !mg_wait(c, k, n, need, &s_ok)) return;
    // The other planes' values and the source of step t + 1 load while step
    // t computes: the chunk's wait covers every step of the chunk, and a
    // neighbour cannot get SKEW steps ahead of this plane's published
    // progress, so none of them changes before its use.
    Fetch cur[K], nxt[K];
    fetch(t0, cur);
    for (int t = t0; t <= t1; ++t) {
      if (t < t1) fetch(t + 1, nxt);
#pragma unroll
      for (int q = 0; q < K; ++q) {
        if (!cur[q].up) continue;
        const int hs = h0 + q, o = cur[q].os;
        const double old = P[o];
        const double v = mg_new(P[o + de], P[o + dw], P[o + R], P[o - R], cur[q].ru, cur[q].rd, cur[q].rs, old);
        P[o] = v;
        E[cur[q].og] = v;
        if (TRACK && hs == 8) acc8 += fabs(v - old);
        if (TRACK && hs == 9) acc9 += fabs(v - old);
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < K; ++q) cur[q] = nxt[q];
    }
    mg_publish(c, k, t1);
  }
  if (TRACK) {
    const double a = block_sum(acc8, red);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
    const double b = block_sum(acc9, red);
    if (threadIdx.x == 0) part[n + blockIdx.x] = b;
  }
}

// Progress of every plane (and its two ghost planes) to "nothing done".
__global__ void k_mg_prog_reset(MgCtl* c, int n) {
  if (!c->active) return;
  for (int q = threadIdx.x; q <= n + 1; q += blockDim.x) c->prog[q] = -1;
}

// The error's ghosts on a coarse level: -(first interior layer) per face in
// each build's statement order (sources.f90:262-283, 285-290); one block.
__device__ void mg_ghosts(const MgLevel& lv, int bc_multipole) {
  const int n = lv.n, m = n + 2;
  double* E = lv.E;
  const int order_mpi[6] = {0, 1, 2, 3, 4, 5};  // x-, x+, y-, y+, z-, z+
  const int order_ser[6] = {0, 2, 4, 1, 3, 5};  // x-, y-, z-, x+, y+, z+
  for (int s = 0; s < 6; ++s) {
    const int f = bc_multipole ? order_mpi[s] : order_ser[s];
    const int axis = f >> 1, hi = f & 1;
    const int g = hi ? n + 1 : 0, src = hi ? n : 1;
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
      const int a = q % m, b = q / m;
      long long to, from;
      if (axis == 0) { to = mgi(n, g, a, b); from = mgi(n, src, a, b); }
      else if (axis == 1) { to = mgi(n, a, g, b); from = mgi(n, a, src, b); }
      else { to = mgi(n, a, b, g); from = mgi(n, a, b, src); }
      E[to] = -E[from];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(1024) k_mg_ghosts(const MgCtl* c, MgLevel lv, int bc_multipole) {
  if (!c->active) return;
  mg_ghosts(lv, bc_multipole);
}

// resid on the fine level (sources.f90:196-216) and restriction onto the
// coarse one (:118-137), fused: each coarse cell forms its 8 children's
// residuals.  (The reference's ret array of the fine level is not kept: it
// is overwritten before anything reads it.)
__device__ __forceinline__ double mg_resid_cell(const MgLevel& f, int i, int j, int k) {
  const int n = f.n;
  const long long o = mgi(n, i, j, k), s1 = n + 2, s2 = (long long)(n + 2) * (n + 2);
  const double* E = f.E;
  double g = E[o - 1] + E[o + 1];
  g = g + E[o - s1];
  g = g + E[o + s1];
  g = g + E[o - s2];
  g = g + E[o + s2];
  g = (g - 6.0 * E[o]) / (f.dxl * f.dxl);
  return f.R[o] - g;
}

__device__ void mg_resid_restrict(const MgLevel& f, const MgLevel& c, long long t, long long nt) {
  const int nc = c.n;
  for (long long q = t; q < (long long)nc * nc * nc; q += nt) {
    const int i = 1 + (int)(q % nc), j = 1 + (int)((q / nc) % nc), k = 1 + (int)(q / ((long long)nc * nc));
    const int i1 = 2 * i - 1, j1 = 2 * j - 1, k1 = 2 * k - 1;
    double a = mg_resid_cell(f, i1, j1, k1) + mg_resid_cell(f, i1 + 1, j1, k1);
    a = a + mg_resid_cell(f, i1, j1 + 1, k1);
    a = a + mg_resid_cell(f, i1, j1, k1 + 1);
    a = a + mg_resid_cell(f, i1 + 1, j1 + 1, k1);
    a = a + mg_resid_cell(f, i1 + 1, j1, k1 + 1);
    a = a + mg_resid_cell(f, i1, j1 + 1, k1 + 1);
    a = a + mg_resid_cell(f, i1 + 1, j1 + 1, k1 + 1);
    const double r = (1.0 / 8.0) * a;
    c.R[mgi(nc, i, j, k)] = r;
    c.T[mgi(nc, i, j, k)] = r * (c.dxl * c.dxl);
  }
}

__global__ void k_mg_resid_restrict(const MgCtl* c, MgLevel f, MgLevel co) {
  if (!c->active) return;
  mg_resid_restrict(f, co, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// prolongation (sources.f90:139-194) onto a zeroed ret, then
// Error = Error + ret over the whole array (:181): interior cells add their
// trilinear child value, ghosts add 0.
__device__ void mg_prolong_add(const MgLevel& c, const MgLevel& f, long long t, long long nt) {
  const int nf = f.n, nc = c.n, m = nf + 2;
  const long long s1 = nc + 2, s2 = (long long)(nc + 2) * (nc + 2);
  for (long long q = t; q < (long long)m * m * m; q += nt) {
    const int fi = (int)(q % m), fj = (int)((q / m) % m), fk = (int)(q / ((long long)m * m));
    double r = 0.0;
    if (fi >= 1 && fi <= nf && fj >= 1 && fj <= nf && fk >= 1 && fk <= nf) {
      const int i = (fi + 1) >> 1, j = (fj + 1) >> 1, k = (fk + 1) >> 1;
      const long long di = (fi & 1) ? -1 : 1, dj = (fj & 1) ? -s1 : s1, dk = (fk & 1) ? -s2 : s2;
      const long long o = mgi(nc, i, j, k);
      const double* V = c.E;
      double a = 27.0 * V[o] + 9.0 * V[o + di];
      a = a + 9.0 * V[o + dj];
      a = a + 9.0 * V[o + dk];
      a = a + 3.0 * V[o + di + dj];
      a = a + 3.0 * V[o + di + dk];
      a = a + 3.0 * V[o + dj + dk];
      a = a + V[o + di + dj + dk];
      r = (1.0 / 64.0) * a;
    }
    f.E[q] = f.E[q] + r;
  }
}

__global__ void k_mg_prolong_add(const MgCtl* c, MgLevel co, MgLevel f) {
  if (!c->active) return;
  mg_prolong_add(co, f, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// ---------------------------------------------------------------------------
// Levels lc..L (n <= MG_COARSE_N) of one V-cycle in one block
// ---------------------------------------------------------------------------
constexpr int MG_CT = 128;  // threads: (n/2 planes) x n <= 4 x 8, and the level-wide loops

// Relax (5 passes of 2 half-sweeps) on a level of at most 32 cells; the
// wave planes of a half-sweep advance together, thread t <-> (plane slot
// t / n, i = t % n + 1), the parallel planes' cells first (no plane of one
// kind reads a cell of the other kind that the half-sweep writes).
__device__ double mg_relax_block(const MgLevel& lv, double* pub, double* red, bool track) {
  const int n = lv.n;
  double last = 0.0;
  for (int pass = 0; pass < 5; ++pass) {
    double acc = 0.0;
    for (int half = 0; half < 2; ++half) {
      // parallel planes: (k & 1) != half
      for (int k = 1; k <= n; ++k)
        if (((k & 1) ^ half) == 1 && n >= 2) acc += mg_parallel_plane<true>(lv, k, threadIdx.x, blockDim.x);
      const int ps = threadIdx.x / n, i = threadIdx.x % n + 1;
      const int k = 2 * ps + (half ? 1 : 2);  // (k & 1) == half
      const bool mine = ps < n / 2 && k <= n;
      // every thread runs the diagonal loop (uniform barriers); others idle
      const double a = mg_wave_plane<true>(lv, mine ? k : 1, mine ? i : n + 1, pub + (mine ? ps : 0) * 2 * (n + 1));
      acc += mine ? a : 0.0;
      __syncthreads();
    }
    if (track && pass == 4) last = block_sum(acc, red);
  }
  return last;  // (thread 0)
}

// Gauss-Seidel in i, j, k order until the summed change is <= 0.001
// (sources.f90:337-396); one thread, the coarsest level is tiny.
__device__ void mg_solve_block(const MgLevel& lv, MgCtl* c) {
  if (threadIdx.x == 0) {
    const int n = lv.n;
    const long long s1 = n + 2, s2 = (long long)(n + 2) * (n + 2);
    const double dxl2 = lv.dxl * lv.dxl;
    double Dif = 1000.0;
    int passes = 0;
    while (Dif > 0.001) {
      if (++passes > MG_SOLVE_LIMIT) {
        atomicOr(&c->status, MG_ST_SOLVE);
        break;
      }
      double difp = 0.0;
      for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j)
          for (int k = 1; k <= n; ++k) {
            const long long o = mgi(n, i, j, k);
            const double old = lv.E[o];
            const double v = mg_new(lv.E[o + 1], lv.E[o - 1], lv.E[o + s1], lv.E[o - s1], lv.E[o + s2], lv.E[o - s2],
                                    lv.R[o] * dxl2, old);
            lv.E[o] = v;
            difp = difp + fabs(v - old);
          }
      Dif = difp;
    }
  }
  __syncthreads();
}

struct MgLevels {
  MgLevel lv[MG_MAXL];
};

// The part of one V-cycle on levels lc..L: down (relax lc; then per level
// residual + restriction, ghosts, relax or, on L, solve) and up (per level
// prolongation + add, ghosts, relax).  With lc = 0 it is the whole cycle
// and also forms Dif.
__global__ void __launch_bounds__(MG_CT) k_mg_coarse(MgCtl* c, MgLevels levels, int lc, int L, int bc_multipole) {
  __shared__ double pub[16 * 2 * 33];
  __shared__ double red[32];
  if (!c->active) return;
  const long long t = threadIdx.x, nt = blockDim.x;
  // down
  if (lc > 0) mg_ghosts(levels.lv[lc], bc_multipole);
  if (lc == L)
    mg_solve_block(levels.lv[L], c);
  else
    mg_relax_block(levels.lv[lc], pub, red, false);
  for (int l = lc + 1; l <= L; ++l) {
    mg_resid_restrict(levels.lv[l - 1], levels.lv[l], t, nt);
    __syncthreads();
    mg_ghosts(levels.lv[l], bc_multipole);
    if (l == L)
      mg_solve_block(levels.lv[l], c);
    else
      mg_relax_block(levels.lv[l], pub, red, false);
  }
  // up
  for (int l = L - 1; l >= lc; --l) {
    mg_prolong_add(levels.lv[l + 1], levels.lv[l], t, nt);
    __syncthreads();
    if (l > 0) mg_ghosts(levels.lv[l], bc_multipole);
    const double d = mg_relax_block(levels.lv[l], pub, red, l == 0);
    if (l == 0 && threadIdx.x == 0) c->part[0] = d;
  }
}

// One half-sweep launch: a block per plane, a thread per i (n of them).
void launch_half(const MgCtl* c, const MgLevel& lv, int half, double* part, cudaStream_t s) {
  const int nt = lv.n < 32 ? 32 : lv.n;  // whole warps (threads past n idle)
  if (lv.n <= 256) {
    if (part)
      k_mg_half<256, true><<<lv.n, nt, 0, s>>>(c, lv, half, part);
    else
      k_mg_half<256, false><<<lv.n, nt, 0, s>>>(c, lv, half, part);
  } else {
    if (part)
      k_mg_half<1024, true><<<lv.n, nt, 0, s>>>(c, lv, half, part);
    else
      k_mg_half<1024, false><<<lv.n, nt, 0, s>>>(c, lv, half, part);
  }
}

// Whether a level's relax runs as one cooperative launch: every plane's
// block resident at once (checked with the occupancy calculator, once per
// level size; levels of at most 256 cells), unless TLQ_MG_PIPELINE=0 asks
// for the per-half-sweep kernels.
template <int NT, int MINB, int HG, int G, int CH, bool TRACK>
bool pipe_fits(int n, int nt) {
  static int cached[2048] = {0};  // 0 unknown, 1 fits, 2 does not
  if (n >= 2048) return false;
  if (!cached[n]) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mg_relax_pipe<NT, MINB, HG, G, CH, TRACK>, nt, pipe_smem(n));
    cached[n] = (long long)per * sms >= n ? 1 : 2;
  }
  return cached[n] == 1;
}

template <int NT, int MINB, int HG, int G, int CH, bool TRACK>
bool launch_pipe(MgCtl* c, const MgLevel& lv, double* part, cudaStream_t s) {
  const int nt = (lv.n * HG + 31) / 32 * 32;
  if (!pipe_fits<NT, MINB, HG, G, CH, TRACK>(lv.n, nt)) return false;
  k_mg_prog_reset<<<1, 256, 0, s>>>(c, lv.n);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(lv.n);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = pipe_smem(lv.n);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_mg_relax_pipe<NT, MINB, HG, G, CH, TRACK>, c, lv, part) == cudaSuccess;
}

// The shared-memory-plane relax: one block of NT threads per plane, all
// resident at once (with the plane's dynamic shared memory).
template <int NT, int HG, int CH, bool TRACK>
bool launch_plane(MgCtl* c, const MgLevel& lv, double* part, cudaStream_t s) {
  const int n = lv.n;
  const int nt = (n * HG + 31) / 32 * 32;
  static int state = 0;  // 0 unknown, 1 fits, 2 does not (one level size per instantiation)
  if (!state) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    bool ok = cudaFuncSetAttribute(k_mg_relax_plane<NT, HG, CH, TRACK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)plane_smem(n)) == cudaSuccess;
    ok = ok && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mg_relax_plane<NT, HG, CH, TRACK>, nt,
                                                             plane_smem(n)) == cudaSuccess;
    if (!ok) cudaGetLastError();
    state = (ok && (long long)per * sms >= n) ? 1 : 2;
  }
  if (state != 1) return false;
  k_mg_prog_reset<<<1, 256, 0, s>>>(c, n);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = plane_smem(n);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_mg_relax_plane<NT, HG, CH, TRACK>, c, lv, part) == cudaSuccess;
}

template <bool TRACK>
bool launch_plane_any(MgCtl* c, const MgLevel& lv, double* part, cudaStream_t s) {
  switch (lv.n) {
    case 8: return launch_plane<96, 10, 2, TRACK>(c, lv, part, s);
    case 16: return launch_plane<160, 10, 2, TRACK>(c, lv, part, s);
    case 32: return launch_plane<320, 10, 4, TRACK>(c, lv, part, s);
    case 64: return launch_plane<640, 10, 8, TRACK>(c, lv, part, s);
    case 128: return launch_plane<640, 5, 8, TRACK>(c, lv, part, s);
    default: return false;
  }
}

// One relax of a level above MG_COARSE_N cells (sources.f90:398-471); part:
// where the last pass's per-plane |change| sums go (null: not needed).
// Levels up to 128 cells hold their planes in shared memory
// (k_mg_relax_plane) unless TLQ_MG_PLANE=0; the others, and those, then use
// k_mg_relax_pipe.  Its threads per plane (measured on the gravitating
// cloud): 128-cell levels
// 5 x 128 (two half-sweeps each), 64 down to 8: 10 x n; neighbour checks
// every 8 steps on 128 and 64 cells, 4 on 32, 2 below (a relax takes
// 2n + 9 (CH + 1) steps); 256-cell levels need two blocks per SM: 2 x 256,
// checks every 4 steps.
template <bool TRACK>
bool launch_pipe_any(MgCtl* c, const MgLevel& lv, double* part, cudaStream_t s) {
  const char* env = std::getenv("TLQ_MG_PLANE");
  const bool plane = !(env && env[0] == '0');
  if (plane && launch_plane_any<TRACK>(c, lv, part, s)) return true;
  switch (lv.n) {
    case 8: return launch_pipe<96, 1, 10, 1, 2, TRACK>(c, lv, part, s);
    case 16: return launch_pipe<160, 1, 10, 1, 2, TRACK>(c, lv, part, s);
    case 32: return launch_pipe<320, 1, 10, 1, 4, TRACK>(c, lv, part, s);
    case 64: return launch_pipe<640, 1, 10, 1, 8, TRACK>(c, lv, part, s);
    case 128: return launch_pipe<640, 1, 5, 1, 8, TRACK>(c, lv, part, s);
    case 256: return launch_pipe<512, 2, 2, 1, 4, TRACK>(c, lv, part, s);
    default: return false;
  }
}

void launch_relax(MgCtl* c, const MgLevel& lv, double* part, cudaStream_t s) {
  const char* env = std::getenv("TLQ_MG_PIPELINE");
  const bool pipe = !(env && env[0] == '0');
  if (pipe && (part ? launch_pipe_any<true>(c, lv, part, s) : launch_pipe_any<false>(c, lv, part, s))) return;
  for (int h = 0; h < 10; ++h) launch_half(c, lv, h & 1, (part && h >= 8) ? part + (h - 8) * lv.n : nullptr, s);
}

int grid_for(long long work, int threads) {
  return (int)std::max<long long>(1, std::min<long long>((work + threads - 1) / threads, 152LL * 8));
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// The solver's buffers: E of every level (contiguous, so that the coarse
// ones zero in one pass), then R, then T; the control block; the moments'
// block partials.
int mg_levels_of(const tlq_config& c) {
  if (c.nx != c.ny || c.nx != c.nz || c.nx < 2 || (c.nx & (c.nx - 1))) return -1;
  int L = 0;
  while ((1 << L) < c.nx) ++L;
  return L;
}

cudaError_t mg_alloc(tlq_ctx* ctx) {
  const int L = mg_levels_of(ctx->cfg);
  long long cells = 0;
  for (int l = 0; l <= L; ++l) {
    const long long m = (ctx->cfg.nx >> l) + 2;
    cells += m * m * m;
  }
  cudaError_t e = cudaMalloc(&ctx->mg_work, (size_t)cells * 3 * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&ctx->mg_ctl, sizeof(MgCtl));
  if (e != cudaSuccess) return e;
  e = cudaMemset(ctx->mg_ctl, 0, sizeof(MgCtl));
  if (e != cudaSuccess) return e;
  long long limit = MG_WAIT_LIMIT;
  if (const char* env = std::getenv("TLQ_MG_WAIT_LIMIT")) {
    char* end = nullptr;
    const long long v = std::strtoll(env, &end, 10);
    if (end != env && *end == '\0' && v >= 0) limit = v;
  }
  e = cudaMemcpy(reinterpret_cast<char*>(ctx->mg_ctl) + offsetof(MgCtl, wait_limit), &limit, sizeof limit,
                 cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&ctx->mg_mom, (size_t)MG_MOM_BLOCKS * 25 * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaStreamCreateWithFlags(&ctx->mg_body, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  const long long m0 = ctx->cfg.nx + 2;
  e = cudaMalloc(&ctx->phig, (size_t)(m0 * m0 * m0) * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaMemset(ctx->phig, 0, (size_t)(m0 * m0 * m0) * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&ctx->phit, (size_t)ctx->L.plane * sizeof(double));
  if (e != cudaSuccess) return e;
  e = cudaMemset(ctx->phit, 0, (size_t)ctx->L.plane * sizeof(double));
  if (e != cudaSuccess) return e;
  return cudaMemset(ctx->mg_work, 0, (size_t)cells * 3 * sizeof(double));
}

void mg_free(tlq_ctx* ctx) {
  cudaFree(ctx->mg_work); cudaFree(ctx->mg_ctl); cudaFree(ctx->mg_mom); cudaFree(ctx->phig); cudaFree(ctx->phit);
  if (ctx->mg_body) cudaStreamDestroy(ctx->mg_body);
  ctx->mg_work = nullptr; ctx->mg_ctl = nullptr; ctx->mg_mom = nullptr; ctx->phig = nullptr; ctx->phit = nullptr;
  ctx->mg_body = nullptr;
}

namespace {

MgLevels mg_plan(const tlq_ctx* ctx, int L) {
  MgLevels v{};
  long long total = 0;
  for (int l = 0; l <= L; ++l) {
    const long long m = (ctx->cfg.nx >> l) + 2;
    total += m * m * m;
  }
  double* base = static_cast<double*>(ctx->mg_work);
  long long off = 0;
  for (int l = 0; l <= L; ++l) {
    const int n = ctx->cfg.nx >> l;
    const long long m = n + 2;
    v.lv[l].n = n;
    v.lv[l].E = base + off;
    v.lv[l].R = base + total + off;
    v.lv[l].T = base + 2 * total + off;
    v.lv[l].dxl = (ctx->cfg.xr - ctx->cfg.xl) / (double)n;
    off += m * m * m;
  }
  return v;
}

template <class Dens>
cudaError_t enqueue_mg(tlq_ctx* ctx, Dens rho, const Clock* clk, double* phit, cudaStream_t s) {
  const int L = mg_levels_of(ctx->cfg);
  const MgLevels v = mg_plan(ctx, L);
  MgCtl* c = static_cast<MgCtl*>(ctx->mg_ctl);
  const int n = ctx->cfg.nx;
  const bool multipole = ctx->cfg.grav_bc == TLQ_GBC_MULTIPOLE;
  int lc = 0;
  while (lc < L && v.lv[lc].n > MG_COARSE_N) ++lc;
  long long ncoarse = 0;  // E of levels 1..L, contiguous after E of level 0
  for (int l = 1; l <= L; ++l) {
    const long long m = v.lv[l].n + 2;
    ncoarse += m * m * m;
  }
  const long long m0 = n + 2;
  k_mg_begin<<<1, 1, 0, s>>>(c, clk);
  if (multipole) {
    k_mg_moments<<<MG_MOM_BLOCKS, MG_MOM_THREADS, 0, s>>>(c, clk, ctx->P, rho, static_cast<double*>(ctx->mg_mom));
    k_mg_moments_final<<<1, 32, 0, s>>>(c, clk, static_cast<const double*>(ctx->mg_mom), MG_MOM_BLOCKS);
    k_mg_faces<<<grid_for(6LL * n * n, 256), 256, 0, s>>>(c, clk, ctx->P, ctx->phig);
  }
  k_mg_init<<<grid_for(m0 * m0 * m0, 256), 256, 0, s>>>(c, rho, n, ctx->phig, v.lv[0].E, v.lv[0].R, v.lv[0].T,
                                                        v.lv[0].dxl);
  double* part = reinterpret_cast<double*>(reinterpret_cast<char*>(c) + offsetof(MgCtl, part));
  // One V-cycle slot (sources.f90:140-187): its first kernels evaluate the
  // loop test, and every later kernel of a slot that does not run returns.
  auto cycle = [&](cudaStream_t st) {
    k_mg_cycle_begin<<<grid_for(ncoarse, 256), 256, 0, st>>>(c, v.lv[0].E + m0 * m0 * m0, ncoarse);
    k_mg_cycle_flag<<<1, 1, 0, st>>>(c);
    if (lc == 0) {
      k_mg_coarse<<<1, MG_CT, 0, st>>>(c, v, 0, L, multipole ? 1 : 0);
      k_mg_cycle_end<<<1, 1, 0, st>>>(c, 1);
      return;
    }
    // down: level 0 .. lc-1 on the large kernels
    for (int l = 0; l < lc; ++l) {
      if (l > 0) k_mg_ghosts<<<1, 1024, 0, st>>>(c, v.lv[l], multipole ? 1 : 0);
      launch_relax(c, v.lv[l], nullptr, st);
      k_mg_resid_restrict<<<grid_for((long long)v.lv[l + 1].n * v.lv[l + 1].n * v.lv[l + 1].n, 256), 256, 0, st>>>(
          c, v.lv[l], v.lv[l + 1]);
    }
    k_mg_coarse<<<1, MG_CT, 0, st>>>(c, v, lc, L, multipole ? 1 : 0);
    // up: level lc-1 .. 0
    for (int l = lc - 1; l >= 0; --l) {
      const long long mf = v.lv[l].n + 2;
      k_mg_prolong_add<<<grid_for(mf * mf * mf, 256), 256, 0, st>>>(c, v.lv[l + 1], v.lv[l]);
      if (l > 0) k_mg_ghosts<<<1, 1024, 0, st>>>(c, v.lv[l], multipole ? 1 : 0);
      // the last pass of the level-0 relax forms Dif (sources.f90:465-471)
      launch_relax(c, v.lv[l], l == 0 ? part : nullptr, st);
    }
    k_mg_cycle_end<<<1, 1, 0, st>>>(c, 2 * n);
  };
  // Captured into a graph: the cycles are the body of a while node whose
  // condition the loop test sets on the device (before the node and at the
  // end of each cycle), captured on the context's second stream.  Run
  // directly (or with TLQ_MG_GRAPH_LOOP=0): the fixed sequence of 31 slots.
  cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  cudaError_t e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cg, &deps, nullptr, &nd);
  if (e != cudaSuccess) return e;
  const char* env = std::getenv("TLQ_MG_GRAPH_LOOP");
  if (cst == cudaStreamCaptureStatusActive && ctx->mg_body && !(env && env[0] == '0')) {
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, cg, 0, 0);
    if (e != cudaSuccess) return e;
    k_mg_loop_test<<<1, 1, 0, s>>>(c, h);
    e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &cg, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(ctx->mg_body, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cycle(ctx->mg_body);
    k_mg_loop_test<<<1, 1, 0, ctx->mg_body>>>(c, h);
    cudaGraph_t body = nullptr;
    e = cudaStreamEndCapture(ctx->mg_body, &body);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
  } else {
    for (int cyc = 0; cyc < MG_CYCLES; ++cyc) cycle(s);
  }
  k_mg_end<<<grid_for(m0 * m0 * m0, 256), 256, 0, s>>>(c, const_cast<Clock*>(clk), n, v.lv[0].E, ctx->phig, ctx->phi,
                                                       phit, phit ? ctx->phif : nullptr, ctx->L);
  return cudaGetLastError();
}

}  // namespace

cudaError_t enqueue_multigrid_soa(tlq_ctx* ctx, const double* U, cudaStream_t s) {
  return enqueue_mg(ctx, DensSoA{U, ctx->L}, ctx->clk, ctx->phit, s);
}

cudaError_t enqueue_multigrid_aos(tlq_ctx* ctx, const double* U, const Clock* clk, cudaStream_t s) {
  return enqueue_mg(ctx, DensAoS{U, ctx->A}, clk, nullptr, s);
}

int mg_cycles_and_status(tlq_ctx* ctx, int* cycles, int* status) {
  MgCtl h;
  if (cudaMemcpy(&h, ctx->mg_ctl, sizeof(MgCtl), cudaMemcpyDeviceToHost) != cudaSuccess) return TLQ_ERR_CUDA;
  if (cycles) *cycles = h.iter;
  if (status) *status = h.status;
  return TLQ_OK;
}

}  // namespace tlq
