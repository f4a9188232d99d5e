// tlq_api.cu -- host side of libtlq: the C ABI declared in include/tlq.h.
//
// The context owns the whole mesh in HBM (structure-of-arrays, two copies of
// U for ping-pong, UPP, the carried pressure and the potential), the device
// clock, the tensor maps the stage kernels stream through, and one CUDA
// graph per buffer parity so that a step is one graph launch.
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/tlq.h"
#include "tlq_ctx.h"

using namespace tlq;



namespace {

int fail(tlq_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(tlq_ctx* c, cudaError_t e, const char* where) {
  if (c) c->err = std::string(where) + ": " + cudaGetErrorString(e);
  return TLQ_ERR_CUDA;
}

#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);            \
  } while (0)

size_t array_bytes(const tlq_config& c) { return (size_t)5 * (c.nx + 4) * (size_t)(c.ny + 4) * (size_t)(c.nz + 4) * 8; }
size_t phi_bytes(const tlq_config& c) { return (size_t)(c.nx + 2) * (size_t)(c.ny + 2) * (size_t)(c.nz + 2) * 8; }

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 4-D map {x, y, z, var} over a SoA array with `nvar` planes of elements of
// `esize` bytes (8: FP64, 4: FP32); box = the tile plus the halo its kernel
// reads: the plain form's halo-2 box; in the mixed form stage 1's box of U
// (2 cells in x, 1 in y: halo1 = true) and stage 2's halo-2 box of UPP's
// FP32 primitives.
int make_map(tlq_ctx* ctx, CUtensorMap* m, void* base, int nvar, int esize = 8, bool halo1 = false) {
  auto fn = encode_fn();
  if (!fn) return fail(ctx, TLQ_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const Layout& L = ctx->L;
  cuuint64_t dims[4] = {(cuuint64_t)(ctx->cfg.nx + 4), (cuuint64_t)(ctx->cfg.ny + 4), (cuuint64_t)(ctx->cfg.nz + 4),
                        (cuuint64_t)nvar};
  const cuuint64_t es = (cuuint64_t)esize;
  cuuint64_t strides[3] = {(cuuint64_t)L.px * es, (cuuint64_t)L.px * L.nyg * es, (cuuint64_t)L.plane * es};
  const bool mixed = ctx->cfg.precision == TLQ_PREC_MIXED;
  const cuuint32_t bx = (cuuint32_t)(mixed ? MHX : HX);
  const cuuint32_t by = (cuuint32_t)(mixed ? (halo1 ? MTY + 2 : MHY) : HY);
  cuuint32_t box[4] = {bx, by, 1, (cuuint32_t)nvar};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(m, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ctx, TLQ_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return TLQ_OK;
}

int validate(const tlq_config* c, std::string& why) {
  if (c->nx < 2 || c->ny < 2 || c->nz < 2) { why = "nx, ny, nz must be >= 2"; return TLQ_ERR_CONFIG; }
  if (!(c->xr > c->xl) || !(c->yr > c->yl) || !(c->zr > c->zl)) { why = "empty domain"; return TLQ_ERR_CONFIG; }
  if (!(c->gamma > 1.0)) { why = "gamma must be > 1"; return TLQ_ERR_CONFIG; }
  if (c->limiter < TLQ_LIMITER_NONE || c->limiter > TLQ_LIMITER_SUPERBEE) { why = "unknown limiter"; return TLQ_ERR_CONFIG; }
  if (c->solver != TLQ_SOLVER_HLLC && c->solver != TLQ_SOLVER_HLL) { why = "unknown solver"; return TLQ_ERR_CONFIG; }
  for (int q = 0; q < 6; ++q)
    if (c->bc[q] < TLQ_BC_OUTFLOW || c->bc[q] > TLQ_BC_INFLOW) { why = "unknown boundary kind"; return TLQ_ERR_CONFIG; }
  if (c->cooling < TLQ_COOL_NONE || c->cooling > TLQ_COOL_EXACT) { why = "unknown cooling mode"; return TLQ_ERR_CONFIG; }
  if (c->cooling == TLQ_COOL_SUBCYCLE && (c->cool_max_sub < 1 || !(c->cool_sub_frac > 0.0))) {
    why = "sub-cycled cooling needs cool_max_sub >= 1 and cool_sub_frac > 0";
    return TLQ_ERR_CONFIG;
  }
  if ((c->cooling == TLQ_COOL_EXACT || c->cooling == TLQ_COOL_MLP) && !(c->cool_sub_frac > 0.0)) {
    why = "the exact integrator (and the surrogate) needs cool_sub_frac > 0 (its single-step limit)";
    return TLQ_ERR_CONFIG;
  }
  if (c->precision != TLQ_PREC_FP64 && c->precision != TLQ_PREC_MIXED) { why = "unknown precision"; return TLQ_ERR_CONFIG; }
  if (c->cooling == TLQ_COOL_MLP && !(c->cool_mlp_tol > 0.0 && c->cool_mlp_tol <= 1e-3)) {
    why = "the surrogate's residual tolerance must lie in (0, 1e-3]";
    return TLQ_ERR_CONFIG;
  }
  if (c->cooling == TLQ_COOL_MLP && c->precision != TLQ_PREC_MIXED) {
    why = "the cooling surrogate runs in the mixed-precision step";
    return TLQ_ERR_CONFIG;
  }
  for (int q = 0; q < 6; ++q)
    if (c->bc[q] == TLQ_BC_INFLOW) { why = "inflow boundaries are an empty stub in the reference"; return TLQ_ERR_CONFIG; }
  if (c->self_gravity) {
    if (mg_levels_of(*c) < 0 || c->nx > 1024) {
      why = "self-gravity needs nx = ny = nz = 2^L, 2 <= nx <= 1024 (parameters.f90:22-25)";
      return TLQ_ERR_CONFIG;
    }
    if (c->grav_bc != TLQ_GBC_ZERO && c->grav_bc != TLQ_GBC_MULTIPOLE) { why = "unknown grav_bc"; return TLQ_ERR_CONFIG; }
    if (c->grav_bc == TLQ_GBC_MULTIPOLE)
      for (int q = 0; q < 6; ++q)
        if (c->bc[q] == TLQ_BC_PERIODIC) {
          why = "multipole self-gravity boundaries with periodic hydro boundaries (the reference exchanges the "
                "potential's ghosts there instead)";
          return TLQ_ERR_CONFIG;
        }
  }
  return TLQ_OK;
}

void fill_params(tlq_ctx* c) {
  const tlq_config& g = c->cfg;
  Params& p = c->P;
  p.nx = g.nx; p.ny = g.ny; p.nz = g.nz;
  p.xl = g.xl; p.yl = g.yl; p.zl = g.zl;
  p.dx = (g.xr - g.xl) / (double)g.nx;  // parameters.f90:89-91
  p.dy = (g.yr - g.yl) / (double)g.ny;
  p.dz = (g.zr - g.zl) / (double)g.nz;
  p.gamma = g.gamma;
  p.g1 = g.gamma / (g.gamma - 1.0);
  p.cfl = g.cfl; p.eta = g.eta; p.mu0 = g.mu0; p.cooling_limit = g.cooling_limit;
  p.cool_sub_frac = g.cool_sub_frac;
  p.limiter = g.limiter; p.solver = g.solver; p.cooling = g.cooling; p.cool_max_sub = g.cool_max_sub;
  for (int q = 0; q < 6; ++q) p.bc[q] = g.bc[q];
  p.f_gamma = (float)p.gamma; p.f_g1 = (float)p.g1; p.f_eta = (float)p.eta;
  p.f_inv_dx = (float)(1.0 / p.dx); p.f_inv_dy = (float)(1.0 / p.dy); p.f_inv_dz = (float)(1.0 / p.dz);
  p.f_hdx = (float)(0.5 / p.dx); p.f_hdy = (float)(0.5 / p.dy); p.f_hdz = (float)(0.5 / p.dz);
  p.f_cT = (float)(p.mu0 * AMU / KB);
  p.f_inv_muamu = (float)(1.0 / (p.mu0 * AMU));
  p.f_cool_sub_frac = (float)p.cool_sub_frac;
  p.f_mlp_tol = (float)g.cool_mlp_tol;
  p.f_cooling_limit = (float)p.cooling_limit;
  p.c_edge_p = (p.gamma - 1.0) * p.mu0 * AMU;  // c_edge_rho = T_0 KB: set with the cooling table
}

}  // namespace

void invalidate_graphs(tlq_ctx* c) {
  c->gen += 1;
  for (int q = 0; q < 2; ++q) {
    if (c->graph[q]) { cudaGraphExecDestroy(c->graph[q]); c->graph[q] = nullptr; }
    if (c->tgraph[q]) { cudaGraphExecDestroy(c->tgraph[q]); c->tgraph[q] = nullptr; }
  }
}

namespace {

int ensure_routine_scratch(tlq_ctx* ctx) {
  if (ctx->rb[0]) return TLQ_OK;
  const size_t b = array_bytes(ctx->cfg);
  for (int q = 0; q < 6; ++q) {
    cudaError_t e = cudaMalloc(&ctx->rb[q], b);
    if (e != cudaSuccess) return fail(ctx, TLQ_ERR_NOMEM, "per-routine scratch: " + std::string(cudaGetErrorString(e)));
  }
  CK(cudaMalloc(&ctx->rphi, phi_bytes(ctx->cfg)));
  CK(cudaMalloc(&ctx->rclk, sizeof(Clock)));
  return TLQ_OK;
}

// The plain FP64 form carries apply_cooling's UPrim(5) exactly (a plane of
// interior pressures); the mixed form recomputes the pressure from U.
bool carries_pressure(const tlq_ctx* c) {
  return c->cfg.cooling != TLQ_COOL_NONE && c->cfg.precision == TLQ_PREC_FP64;
}

// The device-visible address of a page-locked host array (cudaHostAlloc'd or
// registered), or null for pageable memory.  Layout conversions then read or
// write the host array directly over the host link (no staging copy).
const void* mapped_host(const void* p) {
  static const bool off = [] {
    const char* e = std::getenv("TLQ_HOST_DIRECT");
    return e && e[0] == '0';
  }();
  if (off) return nullptr;  // TLQ_HOST_DIRECT=0: always through the staging buffer
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (at.type == cudaMemoryTypeHost) ? at.devicePointer : nullptr;
}

int status_from_bits(int bits) {
  if (bits & ST_TIMEOUT) return TLQ_ERR_TIMEOUT;
  if (bits & ST_NONFINITE_DT) return TLQ_ERR_NONFINITE_DT;
  if (bits & ST_NEG_DENSITY) return TLQ_ERR_NEG_DENSITY;
  return TLQ_OK;
}

// Enqueue one step (stage 1 + stage 2) on buffer parity `par`; timed: with
// the timing events, recorded as event nodes when the stream is captured.
int enqueue_step(tlq_ctx* ctx, int par, bool timed) {
  StageArgs a{};
  a.p = ctx->P;
  a.L = ctx->L;
  a.clk = ctx->clk;
  a.zlen = ctx->zlen;
  a.phi = ctx->cfg.self_gravity ? ctx->phit : ctx->phi;
  a.phif = ctx->phif;
  a.lapf = ctx->lapf;
  // the mixed form keeps UPP as FP32 primitives in the same allocation
  a.uppf = reinterpret_cast<float*>(ctx->UPP);
  // stage 1: U[par] -> UPP
  a.uold = ctx->U[par];
  a.out = ctx->UPP;
  a.pout = nullptr;
  const bool mixed = ctx->cfg.precision == TLQ_PREC_MIXED;
  a.use_p = (!mixed && ctx->cfg.cooling != TLQ_COOL_NONE) ? 1 : 0;
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[0], ctx->stream, cudaEventRecordExternal));
  // self-gravity: MultiGrid on U's density before each Godunov (both take U
  // as UU, HLLC.f90:15-24 with mainHD.f90:79,87)
  if (ctx->cfg.self_gravity) CK(enqueue_multigrid_soa(ctx, ctx->U[par], ctx->stream));
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[4], ctx->stream, cudaEventRecordExternal));
  if (mixed)
    CK(launch_stage_mixed(1, ctx->tm_U[par], a, ctx->grid, ctx->stream));
  else
    CK(launch_stage(1, ctx->cfg.precision, ctx->tm_U[par], ctx->tm_P, a, ctx->grid, ctx->stream));
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[1], ctx->stream, cudaEventRecordExternal));
  // stage 2: UPP (+ U[par]) -> U[par^1]
  if (ctx->cfg.self_gravity) CK(enqueue_multigrid_soa(ctx, ctx->U[par], ctx->stream));
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[5], ctx->stream, cudaEventRecordExternal));
  a.out = ctx->U[par ^ 1];
  a.pout = ctx->Pc;
  a.use_p = 0;
  a.cqueue = ctx->mlp_cqueue;
  a.cqcount = ctx->mlp_qcount ? ctx->mlp_qcount + 1 : nullptr;
  a.cool_counts = ctx->cool_counts;
  if (mixed)
    CK(launch_stage_mixed(2, ctx->tm_UPP, a, ctx->grid, ctx->stream));
  else
    CK(launch_stage(2, ctx->cfg.precision, ctx->tm_UPP, ctx->tm_P, a, ctx->grid, ctx->stream));
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[2], ctx->stream, cudaEventRecordExternal));
  // surrogate cooling + the dt reduction (stage 2 leaves both to it)
  if (ctx->cfg.cooling == TLQ_COOL_MLP)
    CK(launch_cool_mlp_dt(ctx->P, ctx->L, ctx->U[0], ctx->U[1], ctx->it_base, ctx->clk, ctx->mlp_image,
                          ctx->mlp_norm, ctx->mlp_box, ctx->cool_counts, ctx->mlp_cqueue, ctx->mlp_qcount + 1,
                          ctx->mlp_nqueue, ctx->mlp_qcount + 2, ctx->stream));
  if (timed) CK(cudaEventRecordWithFlags(ctx->ev[3], ctx->stream, cudaEventRecordExternal));
  return TLQ_OK;
}

// The step on parity par as a graph (timed: with the timing events).
int build_graph(tlq_ctx* ctx, int par, bool timed = false) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(ctx, par, timed);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc != TLQ_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(timed ? &ctx->tgraph[par] : &ctx->graph[par], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  return TLQ_OK;
}

int run_steps(tlq_ctx* ctx, int n) {
  if (ctx->cfg.cooling == TLQ_COOL_MLP && !ctx->mlp_ready)
    return fail(ctx, TLQ_ERR_STATE, "surrogate cooling on but no network (train or set one first)");
  for (int q = 0; q < n; ++q) {
    const int par = ctx->cur;
    if (ctx->timing) {  // the same step graph with its events recorded
      if (!ctx->tgraph[par]) {
        int rc = build_graph(ctx, par, true);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(ctx->tgraph[par], ctx->stream));
      CK(cudaEventSynchronize(ctx->ev[3]));
      float a = 0.f, b = 0.f, c = 0.f, g1 = 0.f, g2 = 0.f;
      cudaEventElapsedTime(&a, ctx->ev[4], ctx->ev[1]);
      cudaEventElapsedTime(&b, ctx->ev[5], ctx->ev[2]);
      cudaEventElapsedTime(&c, ctx->ev[2], ctx->ev[3]);
      cudaEventElapsedTime(&g1, ctx->ev[0], ctx->ev[4]);
      cudaEventElapsedTime(&g2, ctx->ev[1], ctx->ev[5]);
      ctx->ms1_acc += a;
      ctx->ms2_acc += b;
      ctx->mscool_acc += c;
      ctx->msgrav_acc += (double)g1 + (double)g2;
      ctx->ntimed += 1;
    } else {
      if (!ctx->graph[par]) {
        int rc = build_graph(ctx, par);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(ctx->graph[par], ctx->stream));
    }
    ctx->cur ^= 1;
    ctx->steps += 1;
  }
  return TLQ_OK;
}

int set_tfin(tlq_ctx* ctx, double tfin) {
  CK(cudaMemcpyAsync(&ctx->clk->tfin, &tfin, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  return TLQ_OK;
}

int read_clock(tlq_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->clk_host, ctx->clk, sizeof(Clock), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // The current buffer follows the number of steps the device really ran.
  ctx->cur = (int)((ctx->clk_host->it - ctx->it_base) & 1LL);
  return TLQ_OK;
}

}  // namespace

int ctx_set_zlen(tlq_ctx* ctx, int zlen) {
  const int nz = ctx->cfg.nz;
  zlen = std::min(zlen, nz);
  if (zlen < 8 && zlen != nz) return fail(ctx, TLQ_ERR_ARG, "z-chunk length must be >= 8 planes (or nz)");
  ctx->zlen = zlen;
  ctx->grid.z = (unsigned)((nz + zlen - 1) / zlen);
  invalidate_graphs(ctx);
  return TLQ_OK;
}

extern "C" {

int tlq_set_tiling(tlq_ctx* ctx, int zlen) {
  if (!ctx) return TLQ_ERR_ARG;
  return ctx_set_zlen(ctx, zlen);
}

int tlq_get_tiling(const tlq_ctx* ctx, int* zlen) {
  if (!ctx || !zlen) return TLQ_ERR_ARG;
  *zlen = ctx->zlen;
  return TLQ_OK;
}

void tlq_config_default(tlq_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->nx = c->ny = c->nz = 50;
  c->xl = c->yl = c->zl = -1.0;
  c->xr = c->yr = c->zr = 1.0;
  c->gamma = 5.0 / 3.0;
  c->cfl = 0.4;
  c->eta = 0.5e-2;
  c->mu0 = 1.0;
  c->cooling_limit = 0.5;
  c->limiter = TLQ_LIMITER_VANLEER;
  c->solver = TLQ_SOLVER_HLLC;
  for (int q = 0; q < 6; ++q) c->bc[q] = TLQ_BC_REFLECTIVE;
  c->cool_mlp_tol = 1e-3;
  c->cooling = TLQ_COOL_NONE;
  c->cool_max_sub = 1;
  c->cool_sub_frac = 0.1;
  c->precision = TLQ_PREC_FP64;
  c->device = 0;
}

const char* tlq_status_string(int s) {
  switch (s) {
    case TLQ_OK: return "ok";
    case TLQ_ERR_CUDA: return "CUDA error";
    case TLQ_ERR_CONFIG: return "invalid configuration";
    case TLQ_ERR_NONFINITE_DT: return "non-finite CFL time step";
    case TLQ_ERR_NEG_DENSITY: return "non-positive density";
    case TLQ_ERR_TIMEOUT: return "device wait timed out";
    case TLQ_ERR_ARG: return "invalid argument";
    case TLQ_ERR_STATE: return "call out of order";
    case TLQ_ERR_NOMEM: return "out of memory";
    default: return "unknown status";
  }
}

const char* tlq_last_error(tlq_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int tlq_create(const tlq_config* cfg, tlq_ctx** out) {
  if (!cfg || !out) return TLQ_ERR_ARG;
  *out = nullptr;
  std::string why;
  int rc = validate(cfg, why);
  if (rc) return rc;
  tlq_ctx* ctx = new tlq_ctx();
  ctx->cfg = *cfg;
  auto bail = [&](int code) { tlq_destroy(ctx); return code; };
  cudaError_t e = cudaSetDevice(cfg->device);
  if (e != cudaSuccess) { tlq_destroy(ctx); return TLQ_ERR_CUDA; }
  fill_params(ctx);
  ctx->A = Aos{cfg->nx, cfg->ny, cfg->nz};
  Layout& L = ctx->L;
  L.px = ((cfg->nx + 4) + 7) / 8 * 8;
  L.nyg = cfg->ny + 4;
  L.nzg = cfg->nz + 4;
  L.plane = (long long)L.px * L.nyg * L.nzg;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(TLQ_ERR_CUDA);
  ctx->own_stream = true;
  const size_t soa = (size_t)L.plane * 5 * sizeof(double);
  if (cudaMalloc(&ctx->U[0], soa) || cudaMalloc(&ctx->U[1], soa) || cudaMalloc(&ctx->UPP, soa) ||
      cudaMalloc(&ctx->Pc, (size_t)L.plane * 8) || cudaMalloc(&ctx->phi, (size_t)L.plane * 8) ||
      cudaMalloc(&ctx->staging, array_bytes(*cfg)))
    return bail(TLQ_ERR_NOMEM);
  cudaMemset(ctx->U[0], 0, soa);
  cudaMemset(ctx->U[1], 0, soa);
  cudaMemset(ctx->UPP, 0, soa);
  cudaMemset(ctx->Pc, 0, (size_t)L.plane * 8);
  cudaMemset(ctx->phi, 0, (size_t)L.plane * 8);
  if (cfg->self_gravity) {
    if (mg_alloc(ctx) != cudaSuccess) return bail(TLQ_ERR_NOMEM);
    ctx->P.gravity = 1;
  }
  if (cfg->precision == TLQ_PREC_MIXED) {
    if (cudaMalloc(&ctx->lapf, (size_t)L.plane * 5 * sizeof(float)) ||
        cudaMalloc(&ctx->phif, (size_t)L.plane * sizeof(float)))
      return bail(TLQ_ERR_NOMEM);
    cudaMemset(ctx->lapf, 0, (size_t)L.plane * 5 * sizeof(float));
    cudaMemset(ctx->phif, 0, (size_t)L.plane * sizeof(float));
  }
  if (cfg->cooling == TLQ_COOL_MLP) {
    const size_t ncell = (size_t)cfg->nx * cfg->ny * cfg->nz;
    if (cudaMalloc(&ctx->mlp_cqueue, ncell * sizeof(unsigned)) ||
        cudaMalloc(&ctx->mlp_nqueue, ncell * sizeof(unsigned)) || cudaMalloc(&ctx->mlp_qcount, 3 * sizeof(unsigned)))
      return bail(TLQ_ERR_NOMEM);
    cudaMemset(ctx->mlp_qcount, 0, 3 * sizeof(unsigned));
  }
  if (cudaMalloc(&ctx->clk, sizeof(Clock)) || cudaMallocHost(&ctx->clk_host, sizeof(Clock))) return bail(TLQ_ERR_NOMEM);
  std::memset(ctx->clk_host, 0, sizeof(Clock));
  ctx->clk_host->tfin = std::numeric_limits<double>::infinity();
  cudaMemcpy(ctx->clk, ctx->clk_host, sizeof(Clock), cudaMemcpyHostToDevice);
  // stage grid: column tiles (TX x TY plain, MTX x MTY mixed), z split into
  // chunks of zlen planes
  const int tx_ = cfg->precision == TLQ_PREC_MIXED ? MTX : TX, ty_ = cfg->precision == TLQ_PREC_MIXED ? MTY : TY;
  const int gx = (cfg->nx + tx_ - 1) / tx_, gy = (cfg->ny + ty_ - 1) / ty_;
  ctx->zlen = cfg->nz >= 128 ? 64 : (cfg->nz >= 32 ? 32 : cfg->nz);
  const int gz = (cfg->nz + ctx->zlen - 1) / ctx->zlen;
  ctx->grid = dim3(gx, gy, gz);
  const int nb = init_blocks(ctx->P);
  if (cudaMalloc(&ctx->sums_partials, sizeof(double) * 5 * (size_t)nb) || cudaMalloc(&ctx->sums_out, sizeof(double) * 5))
    return bail(TLQ_ERR_NOMEM);
  if (prepare_stage_kernels() != cudaSuccess) return bail(TLQ_ERR_CUDA);
  if (cfg->precision == TLQ_PREC_MIXED && prepare_mixed_kernels() != cudaSuccess) return bail(TLQ_ERR_CUDA);
  const bool mixed = cfg->precision == TLQ_PREC_MIXED;
  int r = make_map(ctx, &ctx->tm_U[0], ctx->U[0], 5, 8, mixed);
  if (!r) r = make_map(ctx, &ctx->tm_U[1], ctx->U[1], 5, 8, mixed);
  if (!r) r = make_map(ctx, &ctx->tm_UPP, ctx->UPP, 5, mixed ? 4 : 8);
  if (!r) r = make_map(ctx, &ctx->tm_P, ctx->Pc, 1);
  if (r) return bail(r);
  for (int q = 0; q < 6; ++q) cudaEventCreate(&ctx->ev[q]);
  if (cudaDeviceSynchronize() != cudaSuccess) return bail(TLQ_ERR_CUDA);
  *out = ctx;
  return TLQ_OK;
}

int tlq_destroy(tlq_ctx* ctx) {
  if (!ctx) return TLQ_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  output_free(ctx);
  invalidate_graphs(ctx);
  for (int q = 0; q < 6; ++q)
    if (ctx->ev[q]) cudaEventDestroy(ctx->ev[q]);
  cudaFree(ctx->U[0]); cudaFree(ctx->U[1]); cudaFree(ctx->UPP); cudaFree(ctx->Pc); cudaFree(ctx->phi);
  cudaFree(ctx->lapf);
  cudaFree(ctx->phif);
  mg_free(ctx);
  cudaFree(ctx->mlp_params); cudaFree(ctx->mlp_image); cudaFree(ctx->cool_counts);
  cudaFree(ctx->mlp_cqueue); cudaFree(ctx->mlp_nqueue); cudaFree(ctx->mlp_qcount);
  cudaFree(ctx->clk); cudaFree(ctx->sums_partials); cudaFree(ctx->sums_out);
  cudaFree(ctx->staging);
  cudaFree(ctx->dT); cudaFree(ctx->dlogT); cudaFree(ctx->dC); cudaFree(ctx->dwinds); cudaFree(ctx->dmasses);
  cudaFree(ctx->dTf); cudaFree(ctx->dlogTf); cudaFree(ctx->dCf);
  cudaFree(ctx->dslope); cudaFree(ctx->dgcum); cudaFree(ctx->dslopef); cudaFree(ctx->dgcumf);
  for (int q = 0; q < 6; ++q) cudaFree(ctx->rb[q]);
  cudaFree(ctx->rphi); cudaFree(ctx->rclk);
  if (ctx->clk_host) cudaFreeHost(ctx->clk_host);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return TLQ_OK;
}

int tlq_set_stream(tlq_ctx* ctx, void* s) {
  if (!ctx) return TLQ_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  if (s) {
    ctx->stream = (cudaStream_t)s;
    ctx->own_stream = false;
  } else {
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->own_stream = true;
  }
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_set_cooling_table(tlq_ctx* ctx, const double* T, const double* logL, int n) {
  if (!ctx || !T || !logL || n < 2) return TLQ_ERR_ARG;
  for (int q = 1; q < n; ++q)
    if (!(T[q] >= T[q - 1])) return fail(ctx, TLQ_ERR_ARG, "cooling table temperatures must be ascending");
  std::vector<double> lt(n);
  for (int q = 0; q < n; ++q) lt[q] = std::log10(T[q]);
  cudaFree(ctx->dT); cudaFree(ctx->dlogT); cudaFree(ctx->dC);
  ctx->dT = ctx->dlogT = ctx->dC = nullptr;
  CK(cudaMalloc(&ctx->dT, n * sizeof(double)));
  CK(cudaMalloc(&ctx->dlogT, n * sizeof(double)));
  CK(cudaMalloc(&ctx->dC, n * sizeof(double)));
  CK(cudaMemcpy(ctx->dT, T, n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dC, logL, n * sizeof(double), cudaMemcpyHostToDevice));
  // log10 of the table temperatures is evaluated on the device, like the
  // reference does at each lookup (cooling.f90:135,137).
  CK(cudaMemcpy(ctx->dlogT, T, n * sizeof(double), cudaMemcpyHostToDevice));
  CK(launch_log10_inplace(ctx->dlogT, n, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  // FP32 copies for the mixed-precision step
  std::vector<double> hlt(n);
  CK(cudaMemcpy(hlt.data(), ctx->dlogT, n * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<float> fT(n), flt(n), fC(n);
  for (int q = 0; q < n; ++q) { fT[q] = (float)T[q]; flt[q] = (float)hlt[q]; fC[q] = (float)logL[q]; }
  cudaFree(ctx->dTf); cudaFree(ctx->dlogTf); cudaFree(ctx->dCf);
  ctx->dTf = ctx->dlogTf = ctx->dCf = nullptr;
  CK(cudaMalloc(&ctx->dTf, n * sizeof(float)));
  CK(cudaMalloc(&ctx->dlogTf, n * sizeof(float)));
  CK(cudaMalloc(&ctx->dCf, n * sizeof(float)));
  CK(cudaMemcpy(ctx->dTf, fT.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dlogTf, flt.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dCf, fC.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  // The exact integrator's closed form (COOL_EXACT, and the surrogate's
  // fallback and check): per segment the power law's slope, in find_coef's
  // form (cooling.f90:137-140), 0 above the last node; at each node G(T_i),
  // the running sum of the segments' integrals of 1/Lambda.  FP64 on the
  // host, in the oracle's order of operations.
  std::vector<double> sl(n), gc(n);
  gc[0] = 0.0;
  for (int i = 0; i < n; ++i) {
    sl[i] = (i + 1 < n) ? (logL[i + 1] - logL[i]) / (std::log10(T[i + 1]) - std::log10(T[i])) : 0.0;
    if (i + 1 < n) {
      const double a = 1.0 - sl[i], Li = std::pow(10.0, logL[i]), r = T[i + 1] / T[i];
      const double g = std::fabs(a) < 1e-9 ? (T[i] / Li) * std::log(r) : (T[i] / Li) * (std::pow(r, a) - 1.0) / a;
      gc[i + 1] = gc[i] + g;
    }
  }
  std::vector<float> slf(n), gcf(n);
  for (int q = 0; q < n; ++q) { slf[q] = (float)sl[q]; gcf[q] = (float)gc[q]; }
  cudaFree(ctx->dslope); cudaFree(ctx->dgcum); cudaFree(ctx->dslopef); cudaFree(ctx->dgcumf);
  ctx->dslope = ctx->dgcum = nullptr;
  ctx->dslopef = ctx->dgcumf = nullptr;
  CK(cudaMalloc(&ctx->dslope, n * sizeof(double)));
  CK(cudaMalloc(&ctx->dgcum, n * sizeof(double)));
  CK(cudaMalloc(&ctx->dslopef, n * sizeof(float)));
  CK(cudaMalloc(&ctx->dgcumf, n * sizeof(float)));
  CK(cudaMemcpy(ctx->dslope, sl.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dgcum, gc.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dslopef, slf.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->dgcumf, gcf.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  // nodes uniform in log10 T (each within a third of a step of the line
  // through the first and last): the FP32 searches guess the segment
  float lt0 = 0.0f, dl_inv = 0.0f;
  if (n >= 3) {
    const double l0 = std::log10((double)fT[0]), dl = (std::log10((double)fT[n - 1]) - l0) / (double)(n - 1);
    bool uniform = dl > 0.0;
    for (int q = 0; q < n && uniform; ++q) uniform = std::fabs(std::log10((double)fT[q]) - (l0 + dl * q)) <= dl / 3.0;
    if (uniform) {
      lt0 = (float)l0;
      dl_inv = (float)(1.0 / dl);
    }
  }
  ctx->P.cool = CoolTable{ctx->dT,     ctx->dlogT, ctx->dC,      n,          ctx->dTf, ctx->dlogTf,
                          ctx->dCf,    ctx->dslope, ctx->dgcum, ctx->dslopef, ctx->dgcumf, lt0, dl_inv};
  ctx->cool_tmin = T[0];
  ctx->P.c_edge_rho = T[0] * KB;
  if (!ctx->cool_counts) {
    CK(cudaMalloc(&ctx->cool_counts, 3 * sizeof(unsigned long long)));
    CK(cudaMemset(ctx->cool_counts, 0, 3 * sizeof(unsigned long long)));
  }
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_set_plane_winds(tlq_ctx* ctx, const tlq_plane_wind* w, int n) {
  if (!ctx || n < 0 || n > tlq::MAX_PLANE_WINDS || (n > 0 && !w)) return TLQ_ERR_ARG;
  for (int q = 0; q < n; ++q)
    if (w[q].plane < 1 || w[q].plane > 6) return fail(ctx, TLQ_ERR_ARG, "plane wind: plane must be 1..6");
  ctx->P.nplanes = n;
  for (int q = 0; q < n; ++q) ctx->P.planes[q] = tlq::PlaneWind{w[q].plane, w[q].rho, w[q].vel, w[q].temp, w[q].mu};
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_set_winds(tlq_ctx* ctx, const tlq_wind* w, int n) {
  if (!ctx || n < 0 || (n > 0 && !w)) return TLQ_ERR_ARG;
  cudaFree(ctx->dwinds);
  ctx->dwinds = nullptr;
  ctx->P.nwinds = 0;
  ctx->P.winds = nullptr;
  if (n > 0) {
    std::vector<Wind> hw(n);
    const Params& p = ctx->P;
    for (int q = 0; q < n; ++q) {
      Wind& d = hw[q];
      d.xc = w[q].xc; d.yc = w[q].yc; d.zc = w[q].zc;
      d.vx = w[q].vx; d.vy = w[q].vy; d.vz = w[q].vz;
      d.radius = w[q].radius; d.mdot = w[q].mdot; d.vinf = w[q].vinf; d.temp = w[q].temp; d.mu = w[q].mu;
      // Index box of the cells whose centre can lie within radius (one cell
      // of margin on each side; the exact test runs inside the box).
      auto lo = [](double c, double r, double l, double h) { return (int)std::floor((c - r - l) / h + 0.5) - 1; };
      auto hi = [](double c, double r, double l, double h) { return (int)std::ceil((c + r - l) / h + 0.5) + 1; };
      d.ilo = std::max(-1, lo(d.xc, d.radius, p.xl, p.dx)); d.ihi = std::min(p.nx + 2, hi(d.xc, d.radius, p.xl, p.dx));
      d.jlo = std::max(-1, lo(d.yc, d.radius, p.yl, p.dy)); d.jhi = std::min(p.ny + 2, hi(d.yc, d.radius, p.yl, p.dy));
      d.klo = std::max(-1, lo(d.zc, d.radius, p.zl, p.dz)); d.khi = std::min(p.nz + 2, hi(d.zc, d.radius, p.zl, p.dz));
    }
    CK(cudaMalloc(&ctx->dwinds, n * sizeof(Wind)));
    CK(cudaMemcpy(ctx->dwinds, hw.data(), n * sizeof(Wind), cudaMemcpyHostToDevice));
    ctx->P.nwinds = n;
    ctx->P.winds = ctx->dwinds;
  }
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_set_point_masses(tlq_ctx* ctx, const double* xyzm, int n) {
  if (!ctx || n < 0 || (n > 0 && !xyzm)) return TLQ_ERR_ARG;
  cudaFree(ctx->dmasses);
  ctx->dmasses = nullptr;
  ctx->nmasses = 0;
  ctx->P.gravity = ctx->cfg.self_gravity ? 1 : 0;
  CK(cudaMemsetAsync(ctx->phi, 0, (size_t)ctx->L.plane * 8, ctx->stream));
  if (n > 0) {
    CK(cudaMalloc(&ctx->dmasses, 4 * n * sizeof(double)));
    CK(cudaMemcpy(ctx->dmasses, xyzm, 4 * n * sizeof(double), cudaMemcpyHostToDevice));
    ctx->nmasses = n;
    ctx->P.gravity = 1;
    CK(launch_point_potential_soa(ctx->P, ctx->L, ctx->dmasses, n, ctx->phi, ctx->stream));
  }
  // the mixed stages read the potential in FP32 (self-gravity rewrites it
  // with each solve)
  if (ctx->phif) CK(launch_to_f32(ctx->phi, ctx->phif, ctx->L.plane, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  invalidate_graphs(ctx);
  return TLQ_OK;
}

int tlq_set_time(tlq_ctx* ctx, double t, int it) {
  if (!ctx) return TLQ_ERR_ARG;
  ctx->t0 = t;
  ctx->it0 = it;
  if (ctx->uploaded) {
    CK(cudaMemcpyAsync(&ctx->clk->t, &ctx->t0, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    long long itl = it;
    CK(cudaMemcpyAsync(&ctx->clk->it, &itl, sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const long long base = it - (long long)ctx->cur;
    if (base != ctx->it_base) invalidate_graphs(ctx);  // captured launches read it_base
    ctx->it_base = base;
  }
  return TLQ_OK;
}

int tlq_upload(tlq_ctx* ctx, const double* U) {
  if (!ctx || !U) return TLQ_ERR_ARG;
  if (ctx->cfg.cooling != TLQ_COOL_NONE && !ctx->dT) return fail(ctx, TLQ_ERR_STATE, "cooling on but no cooling table");
  if (ctx->cool_counts) CK(cudaMemsetAsync(ctx->cool_counts, 0, 3 * sizeof(unsigned long long), ctx->stream));
  if (const double* hU = static_cast<const double*>(mapped_host(U))) {
    CK(launch_aos_to_soa(ctx->A, ctx->L, hU, ctx->U[0], ctx->stream));
  } else {
    CK(cudaMemcpyAsync(ctx->staging, U, array_bytes(ctx->cfg), cudaMemcpyHostToDevice, ctx->stream));
    CK(launch_aos_to_soa(ctx->A, ctx->L, ctx->staging, ctx->U[0], ctx->stream));
  }
  Clock c{};
  c.t = ctx->t0;
  c.it = ctx->it0;
  c.tfin = std::numeric_limits<double>::infinity();
  *ctx->clk_host = c;
  CK(cudaMemcpyAsync(ctx->clk, ctx->clk_host, sizeof(Clock), cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->cfg.precision == TLQ_PREC_MIXED)
    CK(launch_init_dt_mixed(ctx->P, ctx->L, ctx->U[0], ctx->clk, init_blocks(ctx->P), ctx->stream));
  else
    CK(launch_init_prims_dt(ctx->P, ctx->L, ctx->U[0], carries_pressure(ctx) ? ctx->Pc : nullptr, ctx->clk,
                            init_blocks(ctx->P), ctx->stream));
  if (ctx->cfg.self_gravity) {  // mainHD.f90:50-52: the first MultiGrid, PHI starting at 0
    const long long m = ctx->cfg.nx + 2;
    CK(cudaMemsetAsync(ctx->phig, 0, (size_t)(m * m * m) * sizeof(double), ctx->stream));
    CK(enqueue_multigrid_soa(ctx, ctx->U[0], ctx->stream));
  }
  ctx->cur = 0;
  if (ctx->it_base != ctx->it0) invalidate_graphs(ctx);  // captured launches read it_base
  ctx->it_base = ctx->it0;
  ctx->steps = 0;
  ctx->uploaded = true;
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_download(tlq_ctx* ctx, double* U, double* W) {
  if (!ctx) return TLQ_ERR_ARG;
  if (!ctx->uploaded) return fail(ctx, TLQ_ERR_STATE, "tlq_download before tlq_upload");
  int rc = read_clock(ctx);
  if (rc) return rc;
  if (U) {
    if (double* hU = static_cast<double*>(const_cast<void*>(mapped_host(U)))) {
      CK(launch_soa_to_aos(ctx->A, ctx->L, ctx->U[ctx->cur], hU, ctx->stream));
    } else {
      CK(launch_soa_to_aos(ctx->A, ctx->L, ctx->U[ctx->cur], ctx->staging, ctx->stream));
      CK(cudaMemcpyAsync(U, ctx->staging, array_bytes(ctx->cfg), cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  if (W) {
    const double* Pc = carries_pressure(ctx) ? ctx->Pc : nullptr;
    if (double* hW = static_cast<double*>(const_cast<void*>(mapped_host(W)))) {
      CK(launch_prims_soa_to_aos(ctx->P, ctx->A, ctx->L, ctx->U[ctx->cur], Pc, hW, ctx->stream));
    } else {
      CK(launch_prims_soa_to_aos(ctx->P, ctx->A, ctx->L, ctx->U[ctx->cur], Pc, ctx->staging, ctx->stream));
      CK(cudaMemcpyAsync(W, ctx->staging, array_bytes(ctx->cfg), cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_get_time(tlq_ctx* ctx, double* t, int* it, double* dt) {
  if (!ctx) return TLQ_ERR_ARG;
  int rc = read_clock(ctx);
  if (rc) return rc;
  if (t) *t = ctx->clk_host->t;
  if (it) *it = (int)ctx->clk_host->it;
  if (dt) *dt = ctx->clk_host->dt_used;
  return status_from_bits(ctx->clk_host->status);
}

int tlq_step(tlq_ctx* ctx, double* t, int* it, double* dt) {
  if (!ctx) return TLQ_ERR_ARG;
  if (!ctx->uploaded) return fail(ctx, TLQ_ERR_STATE, "tlq_step before tlq_upload");
  int rc = run_steps(ctx, 1);
  if (rc) return rc;
  return tlq_get_time(ctx, t, it, dt);
}

int tlq_advance(tlq_ctx* ctx, int n) {
  if (!ctx || n < 0) return TLQ_ERR_ARG;
  if (!ctx->uploaded) return fail(ctx, TLQ_ERR_STATE, "tlq_advance before tlq_upload");
  return run_steps(ctx, n);
}

int tlq_run_until(tlq_ctx* ctx, double tfin, int max_steps, double* t, int* it, double* dt) {
  if (!ctx || max_steps < 0) return TLQ_ERR_ARG;
  if (!ctx->uploaded) return fail(ctx, TLQ_ERR_STATE, "tlq_run_until before tlq_upload");
  int rc = set_tfin(ctx, tfin);
  if (rc) return rc;
  int left = max_steps;
  while (left > 0) {
    // Steps whose start finds t >= tfin do nothing on the device; the host
    // re-reads the clock after each batch and stops once t >= tfin.
    const int batch = std::min(left, 64);
    rc = run_steps(ctx, batch);
    if (rc) break;
    left -= batch;
    rc = read_clock(ctx);
    if (rc) break;
    if (!(ctx->clk_host->t < tfin) || ctx->clk_host->status) break;
  }
  const double inf = std::numeric_limits<double>::infinity();
  int rc2 = set_tfin(ctx, inf);
  if (rc) return rc;
  if (rc2) return rc2;
  return tlq_get_time(ctx, t, it, dt);
}

int tlq_set_tfin(tlq_ctx* ctx, double tfin) {
  if (!ctx || tfin != tfin) return TLQ_ERR_ARG;
  return set_tfin(ctx, tfin);
}

int tlq_synchronize(tlq_ctx* ctx) {
  if (!ctx) return TLQ_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_enable_timing(tlq_ctx* ctx, int on) {
  if (!ctx) return TLQ_ERR_ARG;
  ctx->timing = on != 0;
  ctx->ms1_acc = ctx->ms2_acc = ctx->mscool_acc = ctx->msgrav_acc = 0.0;
  ctx->ntimed = 0;
  return TLQ_OK;
}

int tlq_stats_get(tlq_ctx* ctx, tlq_stats* s) {
  if (!ctx || !s) return TLQ_ERR_ARG;
  std::memset(s, 0, sizeof(*s));
  if (ctx->uploaded) {
    int rc = read_clock(ctx);
    if (rc) return rc;
    s->t = ctx->clk_host->t;
    s->dt = ctx->clk_host->dt_used;
    s->status = status_from_bits(ctx->clk_host->status);
  }
  s->steps = ctx->steps;
  s->graph = (ctx->graph[0] || ctx->graph[1]) ? 1 : 0;
  s->timed = ctx->ntimed;
  s->ms_stage1 = ctx->ntimed ? ctx->ms1_acc / ctx->ntimed : 0.0;
  s->ms_stage2 = ctx->ntimed ? ctx->ms2_acc / ctx->ntimed : 0.0;
  s->ms_cool = ctx->ntimed ? ctx->mscool_acc / ctx->ntimed : 0.0;
  s->ms_grav = ctx->ntimed ? ctx->msgrav_acc / ctx->ntimed : 0.0;
  s->bytes_state = (double)ctx->L.plane * 8.0 * 17.0;
  if (ctx->cool_counts) {
    unsigned long long cc[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(cc, ctx->cool_counts, sizeof(cc), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    s->cool_mlp = (long long)cc[0];
    s->cool_fallback = (long long)cc[1];
    s->cool_single = (long long)cc[2];
  }
  return TLQ_OK;
}

int tlq_conserved_sums(tlq_ctx* ctx, double out[5]) {
  if (!ctx || !out) return TLQ_ERR_ARG;
  if (!ctx->uploaded) return fail(ctx, TLQ_ERR_STATE, "tlq_conserved_sums before tlq_upload");
  int rc = read_clock(ctx);
  if (rc) return rc;
  const int nb = init_blocks(ctx->P);
  CK(launch_conserved_sums(ctx->P, ctx->L, ctx->U[ctx->cur], ctx->sums_partials, nb, ctx->sums_out, ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->sums_out, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

// ---- per-routine entry points ---------------------------------------------
#define NEED(p) \
  if (!(p)) return fail(ctx, TLQ_ERR_ARG, "null array argument")

int tlq_calc_prims(tlq_ctx* ctx, double* W, const double* U) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(W); NEED(U);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], U, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_calc_prims_aos(ctx->P, ctx->A, ctx->rb[1], ctx->rb[0], ctx->stream));
  CK(cudaMemcpyAsync(W, ctx->rb[1], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_time_step(tlq_ctx* ctx, const double* W, double* dt) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(W); NEED(dt);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->rb[0], W, array_bytes(ctx->cfg), cudaMemcpyHostToDevice, ctx->stream));
  Clock c{};
  CK(cudaMemcpyAsync(ctx->rclk, &c, sizeof(Clock), cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_time_step_aos(ctx->P, ctx->A, ctx->rb[0], ctx->rclk, init_blocks(ctx->P), ctx->stream));
  CK(cudaMemcpyAsync(&c, ctx->rclk, sizeof(Clock), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *dt = c.dt;
  return status_from_bits(c.status);
}

int tlq_fluxes(tlq_ctx* ctx, const double* U, double* F, double* G, double* H, const double* W, int choice) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(U); NEED(F); NEED(G); NEED(H); NEED(W);
  if (choice != 1 && choice != 2) return fail(ctx, TLQ_ERR_ARG, "choice must be 1 or 2");
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], U, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[1], W, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[2], F, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[3], G, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[4], H, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_fluxes_aos(ctx->P, ctx->A, ctx->rb[0], ctx->rb[1], ctx->rb[2], ctx->rb[3], ctx->rb[4], choice, ctx->stream));
  CK(cudaMemcpyAsync(F, ctx->rb[2], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(G, ctx->rb[3], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(H, ctx->rb[4], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_godunov(tlq_ctx* ctx, double* UPPP, const double* UU, const double* F, const double* G, const double* H,
                const double* W, double dt) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(UPPP); NEED(UU); NEED(F); NEED(G); NEED(H);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], UU, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[1], F, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[2], G, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[3], H, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[4], UPPP, b, cudaMemcpyHostToDevice, ctx->stream));
  const bool grav = ctx->nmasses > 0 && W;
  if (grav) {
    CK(cudaMemcpyAsync(ctx->rb[5], W, b, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->rphi, 0, phi_bytes(ctx->cfg), ctx->stream));
    CK(launch_point_potential_ref(ctx->P, ctx->dmasses, ctx->nmasses, ctx->rphi, ctx->stream));
  }
  CK(launch_godunov_aos(ctx->P, ctx->A, ctx->rb[4], ctx->rb[0], ctx->rb[1], ctx->rb[2], ctx->rb[3],
                        grav ? ctx->rb[5] : nullptr, grav ? ctx->rphi : nullptr, dt, ctx->stream));
  CK(cudaMemcpyAsync(UPPP, ctx->rb[4], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_borders(tlq_ctx* ctx, double* U, int order) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(U);
  if (order != 1 && order != 2) return fail(ctx, TLQ_ERR_ARG, "order must be 1 or 2");
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], U, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_borders_aos(ctx->P, ctx->A, ctx->rb[0], order, ctx->stream));
  CK(cudaMemcpyAsync(U, ctx->rb[0], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_viscous_step(tlq_ctx* ctx, double* U, const double* UP, double* t, int* it, double dt) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(U); NEED(UP);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[2], U, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[1], UP, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_viscous_step_aos(ctx->P, ctx->A, ctx->rb[0], ctx->rb[1], ctx->rb[2], ctx->stream));
  CK(cudaMemcpyAsync(U, ctx->rb[0], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (t) *t = *t + dt;
  if (it) *it = *it + 1;
  return TLQ_OK;
}

int tlq_cooling(tlq_ctx* ctx, double* W, double* U, double dt) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(W); NEED(U);
  if (ctx->cfg.cooling == TLQ_COOL_NONE) return TLQ_OK;
  if (!ctx->dT) return fail(ctx, TLQ_ERR_STATE, "cooling table not set");
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], W, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rb[1], U, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_cooling_aos(ctx->P, ctx->A, ctx->rb[0], ctx->rb[1], dt, ctx->stream));
  CK(cudaMemcpyAsync(W, ctx->rb[0], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(U, ctx->rb[1], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_multigrid(tlq_ctx* ctx, const double* U, double* phi, int it, int* cycles) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(U); NEED(phi);
  if (!ctx->cfg.self_gravity) return fail(ctx, TLQ_ERR_STATE, "tlq_multigrid needs self_gravity in the configuration");
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const long long m = ctx->cfg.nx + 2;
  const size_t pb = (size_t)(m * m * m) * sizeof(double);
  CK(cudaMemcpyAsync(ctx->rb[0], U, array_bytes(ctx->cfg), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->phig, phi, pb, cudaMemcpyHostToDevice, ctx->stream));
  Clock c{};
  c.it = it;
  c.tfin = std::numeric_limits<double>::infinity();
  CK(cudaMemcpyAsync(ctx->rclk, &c, sizeof(Clock), cudaMemcpyHostToDevice, ctx->stream));
  CK(enqueue_multigrid_aos(ctx, ctx->rb[0], ctx->rclk, ctx->stream));
  CK(cudaMemcpyAsync(phi, ctx->phig, pb, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int st = 0;
  rc = mg_cycles_and_status(ctx, cycles, &st);
  if (rc) return rc;
  if (st & MG_ST_TIMEOUT) return fail(ctx, TLQ_ERR_TIMEOUT, "a pipelined relax gave up waiting for a neighbouring plane");
  if (st) return fail(ctx, TLQ_ERR_TIMEOUT, "coarsest-level solve did not converge");
  return TLQ_OK;
}

int tlq_point_potential(tlq_ctx* ctx, double* phi) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(phi);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = phi_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rphi, phi, b, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->nmasses > 0) CK(launch_point_potential_ref(ctx->P, ctx->dmasses, ctx->nmasses, ctx->rphi, ctx->stream));
  CK(cudaMemcpyAsync(phi, ctx->rphi, b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

int tlq_gravity_source(tlq_ctx* ctx, const double* W, const double* phi, double* S) {
  if (!ctx) return TLQ_ERR_ARG;
  NEED(W); NEED(phi); NEED(S);
  int rc = ensure_routine_scratch(ctx);
  if (rc) return rc;
  const size_t b = array_bytes(ctx->cfg);
  CK(cudaMemcpyAsync(ctx->rb[0], W, b, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->rphi, phi, phi_bytes(ctx->cfg), cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_gravity_source_aos(ctx->P, ctx->A, ctx->rb[0], ctx->rphi, ctx->rb[1], ctx->stream));
  CK(cudaMemcpyAsync(S, ctx->rb[1], b, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TLQ_OK;
}

}  // extern "C"
