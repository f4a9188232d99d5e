// tlq_ctx.h -- the context behind tlq_ctx* (private to libtlq's host code).
#pragma once

#include <string>
#include <thread>
#include <vector>

#include "../../include/tlq.h"
#include "tlq_internal.h"

using namespace tlq;

struct tlq_ctx {
  tlq_config cfg{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Params P{};
  Layout L{};
  Aos A{};
  // device state
  double* U[2] = {nullptr, nullptr};
  double* UPP = nullptr;
  double* Pc = nullptr;   // carried pressure plane (cooling)
  double* phi = nullptr;  // point-mass potential plane
  float* phif = nullptr;  // mixed form: the stages' potential (point masses + self-gravity) in FP32
  // self-gravity (tlq_gravity.cu): multigrid levels, control block, moment
  // partials, the self-gravity potential ((nx+2)^3) and the stages' total
  // potential plane PHIP + PHI (SoA plane layout, like phi)
  void* mg_work = nullptr;
  void* mg_ctl = nullptr;
  void* mg_mom = nullptr;
  cudaStream_t mg_body = nullptr;  // captures a V-cycle into a graph's loop body
  double* phig = nullptr;
  double* phit = nullptr;
  float* lapf = nullptr;  // mixed form: eta * Laplacian of U between the stages
  Clock* clk = nullptr;
  Clock* clk_host = nullptr;  // pinned mirror
  double* sums_partials = nullptr;
  double* sums_out = nullptr;
  double* staging = nullptr;  // one reference-layout array
  // tables
  double *dT = nullptr, *dlogT = nullptr, *dC = nullptr;
  float *dTf = nullptr, *dlogTf = nullptr, *dCf = nullptr;
  double *dslope = nullptr, *dgcum = nullptr;  // the exact integrator's closed form (CoolTable)
  float *dslopef = nullptr, *dgcumf = nullptr;
  Wind* dwinds = nullptr;
  double* dmasses = nullptr;
  int nmasses = 0;
  std::vector<double> masses_host;
  // per-routine scratch (reference layout), allocated on first use
  double* rb[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double* rphi = nullptr;
  Clock* rclk = nullptr;
  // stage launch geometry and tensor maps
  dim3 grid{};
  int zlen = 0;
  CUtensorMap tm_U[2]{}, tm_UPP{}, tm_P{};
  // run state
  int cur = 0;  // U[cur] holds the current state
  long long it_base = 0;
  bool uploaded = false;
  double t0 = 0.0;
  int it0 = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t tgraph[2] = {nullptr, nullptr};  // the same steps with the timing events recorded
  unsigned gen = 0;  // bumped whenever set-up changes what a captured step does
  bool timing = false;
  // timing events: stage-1 start, stage-2 start, stage-2 end, cooling end,
  // and the ends of the two self-gravity solves
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double ms1_acc = 0.0, ms2_acc = 0.0, mscool_acc = 0.0, msgrav_acc = 0.0;
  long long ntimed = 0;
  long long steps = 0;
  // learned cooling surrogate (TLQ_COOL_MLP)
  float* mlp_params = nullptr;             // FP32 master parameters (device)
  void* mlp_image = nullptr;               // the step's image of the network (launch_pack_weights)
  float mlp_norm[6] = {0, 1, 0, 1, 0, 1};  // feature centres and half-widths
  double mlp_box[6] = {0, 0, 0, 0, 0, 0};  // training box of the features (the hull)
  bool mlp_ready = false;
  unsigned long long* cool_counts = nullptr;  // device: cells cooled by the network / the exact integrator /
                                              // a single step
  double cool_tmin = 0.0;                  // the table's first temperature
  unsigned* mlp_cqueue = nullptr;          // cells that cool, queued by stage 2 (capacity nx ny nz)
  unsigned* mlp_nqueue = nullptr;          // cells for the network (capacity nx ny nz)
  unsigned* mlp_qcount = nullptr;          // [1]: cooling queue length, [2]: network queue length (zero
                                           // between steps; [0] unused)
  // output path (tlq_output.cu): device snapshot, page-locked copy, writer thread
  double* out_dev = nullptr;
  double* out_host = nullptr;
  cudaStream_t out_stream = nullptr;
  cudaEvent_t out_ev[2] = {nullptr, nullptr};
  std::thread out_thread;
  int out_rc = 0;
  std::string err;
};

void output_free(tlq_ctx* ctx);  // waits for a pending output, frees its buffers

// Drops the captured step graphs and bumps the set-up generation (tlq_api.cu).
void invalidate_graphs(tlq_ctx* c);

// Z-chunk length of the stage grid (>= 8 planes, or nz): regrids and drops
// the captured graphs (tlq_api.cu).
int ctx_set_zlen(tlq_ctx* ctx, int zlen);

// Self-gravity (tlq_gravity.cu).  mg_levels_of: L with nx = ny = nz = 2^L,
// else -1.  enqueue_multigrid_soa: one MultiGrid call on the density of the
// state U (SoA planes) with the context's clock, then the stages' potential
// plane phit = phi + phig.  enqueue_multigrid_aos: the same on a reference-
// layout array and the given clock, leaving phig only.
namespace tlq {
int mg_levels_of(const tlq_config& c);
cudaError_t mg_alloc(tlq_ctx* ctx);
void mg_free(tlq_ctx* ctx);
cudaError_t enqueue_multigrid_soa(tlq_ctx* ctx, const double* U, cudaStream_t s);
cudaError_t enqueue_multigrid_aos(tlq_ctx* ctx, const double* U, const Clock* clk, cudaStream_t s);
// status bits: the coarsest-level solve did not converge; a pipelined relax
// gave up waiting for a neighbouring plane (its bounded wait ran out)
constexpr int MG_ST_SOLVE = 1;
constexpr int MG_ST_TIMEOUT = 2;
int mg_cycles_and_status(tlq_ctx* ctx, int* cycles, int* status);
}  // namespace tlq
