// tlq_batch.cu -- the batched persistent ensemble: many independent meshes
// (uneven sizes, each with its own physics, clock and dt) advanced together,
// one persistent launch per stage over a work list of all members' tiles,
// the step captured in one CUDA graph, and the z-chunk length of each mesh
// size chosen by a measuring autotuner with a JSON cache.
//
// No counterpart in the reference (one run per process there,
// source/mainHD.f90:61-100); every member is the same step as a single
// context (its tlq_ctx owns the state and is reachable for set-up, upload,
// download and clocks).  Built with --use_fast_math (the mixed form).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "tlq_ctx.h"
#include "tlq_stage_mixed.cuh"

namespace tlq {
namespace {

// One member as the persistent kernels see it (device array).  The tensor
// maps live in global memory (aligned as CUtensorMap requires), written once
// per run call before the launches that read them.
struct MemberDesc {
  CUtensorMap tm_U[2];
  CUtensorMap tm_UPP;
  StageArgs args[2][2];  // [stage - 1][buffer parity]
  long long it_base;     // it at upload: parity = (it - it_base) & 1
  int gx, gy, gz;        // tiles of this mesh
  int pad_;
};

struct Item {  // one tile of one member
  int member, bx, by, bz;
};

// The shared memory of a persistent block: the stage's smem plus the
// current member's arguments (read by every cell of the tile).
template <int STAGE>
struct BatchSmem {
  MixedSmem<STAGE> s;
  alignas(16) StageArgs a;
};

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <int STAGE, int LIM = -1, int SOLV = -1>
__global__ void __launch_bounds__(MNT, MixedBlocks<STAGE>::value)
    stage_kernel_mixed_batch(const MemberDesc* __restrict__ mem, const Item* __restrict__ items, int nitems) {
  extern __shared__ __align__(128) unsigned char smem_bytes[];
  BatchSmem<STAGE>& bs = *reinterpret_cast<BatchSmem<STAGE>*>(smem_bytes);
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const Item it = items[w];
    const MemberDesc& m = mem[it.member];
    // every tile of a member reads its clock before the member's last
    // stage-2 tile advances it (that tile takes the last ticket)
    const Clock* clk = m.args[0][0].clk;
    // a member past its tfin does not step (mainHD.f90:61); checked here so
    // that every tile handed to mixed_tile initialises (and we retire) its
    // barriers
    if (!(clk->t < clk->tfin)) continue;
    const int par = (int)((*(volatile const long long*)&clk->it - m.it_base) & 1LL);
    {
      const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&m.args[STAGE - 1][par]);
      unsigned long long* dst = reinterpret_cast<unsigned long long*>(&bs.a);
      for (int q = threadIdx.x; q < (int)(sizeof(StageArgs) / 8); q += MNT) dst[q] = src[q];
    }
    __syncthreads();
    const CUtensorMap* tm = (STAGE == 1) ? &m.tm_U[par] : &m.tm_UPP;
    const unsigned nblk = (unsigned)(m.gx * m.gy * m.gz);
    const unsigned bid = (unsigned)(it.bx + m.gx * (it.by + m.gy * it.bz));
    mixed_tile<STAGE, LIM, SOLV>(tm, bs.a, bs.s, it.bx, it.by, it.bz, nblk, bid);
    __syncthreads();
    // a tile that gave up on a copy (its member's status says so) may have
    // left it in flight: this block takes no further tile
    if (bs.s.abort) break;
    // the tile's copies have all completed: retire the barriers before the
    // next tile initialises them again
    if (threadIdx.x == 0)
      for (int q = 0; q < MixedSmemSel<STAGE>::nbar; ++q) mbar_inval(&bs.s.bar[q]);
    __syncthreads();
  }
}

static_assert(sizeof(StageArgs) % 8 == 0 && alignof(StageArgs) >= 8, "StageArgs copied as 8-byte words");
static_assert(alignof(MemberDesc) >= 64, "tensor maps 64-byte aligned");

}  // namespace

constexpr int SPEC_LIM = LIM_VANLEER, SPEC_SOLV = SOLVER_HLLC;  // as the single-mesh kernels

cudaError_t prepare_batch_kernels() {
  const void* ks[4] = {(const void*)stage_kernel_mixed_batch<1>, (const void*)stage_kernel_mixed_batch<2>,
                       (const void*)stage_kernel_mixed_batch<1, SPEC_LIM, SPEC_SOLV>,
                       (const void*)stage_kernel_mixed_batch<2, SPEC_LIM, SPEC_SOLV>};
  for (int q = 0; q < 4; ++q) {
    const int smem = (int)(q % 2 == 0 ? sizeof(BatchSmem<1>) : sizeof(BatchSmem<2>));
    const cudaError_t e = cudaFuncSetAttribute(ks[q], cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace tlq

// ===========================================================================
// Host side
// ===========================================================================
using tlq::Item;
using tlq::MemberDesc;

struct tlq_batch {
  std::vector<tlq_ctx*> m;
  std::vector<int> zlen;            // z-chunk length per member
  std::vector<unsigned> gen_seen;   // member set-up generation the graph was built for
  cudaStream_t stream = nullptr;
  std::vector<MemberDesc> h_desc;
  MemberDesc* d_desc = nullptr;
  Item* d_items = nullptr;
  int nitems = 0, cap_items = 0;
  std::vector<unsigned char> h_cool;  // cooling-pass arguments of the surrogate members, in member order
  void* d_cool = nullptr;
  int ncool = 0, cool_blocks = 0;
  int blocks = 0;
  cudaGraphExec_t graph = nullptr;
  bool timing = false;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double ms_acc = 0.0;
  long long steps_timed = 0, steps = 0;
  std::string err;
};

namespace {

int bfail(tlq_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}

#define BCK(call)                                                                                        \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) return bfail(b, TLQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int tiles_z(const tlq_ctx* c, int zlen) { return (c->cfg.nz + zlen - 1) / zlen; }

void fill_desc(tlq_batch* b, int i) {
  tlq_ctx* c = b->m[i];
  MemberDesc& d = b->h_desc[i];
  std::memset(&d, 0, sizeof(d));
  d.tm_U[0] = c->tm_U[0];
  d.tm_U[1] = c->tm_U[1];
  d.tm_UPP = c->tm_UPP;
  for (int st = 1; st <= 2; ++st)
    for (int par = 0; par < 2; ++par) {
      tlq::StageArgs& a = d.args[st - 1][par];
      a.p = c->P;
      a.L = c->L;
      a.clk = c->clk;
      a.zlen = b->zlen[i];
      a.phi = c->phi;
      a.phif = c->phif;
      a.lapf = c->lapf;
      a.uold = c->U[par];
      a.out = (st == 1) ? c->UPP : c->U[par ^ 1];
      a.uppf = reinterpret_cast<float*>(c->UPP);  // stage 1 writes UPP as FP32 primitives
      a.pout = (st == 1) ? nullptr : c->Pc;
      a.use_p = 0;
      a.cqueue = (st == 2) ? c->mlp_cqueue : nullptr;
      a.cqcount = (st == 2 && c->mlp_qcount) ? c->mlp_qcount + 1 : nullptr;
      a.cool_counts = (st == 2) ? c->cool_counts : nullptr;
    }
  d.it_base = c->it_base;
  d.gx = (c->cfg.nx + tlq::MTX - 1) / tlq::MTX;
  d.gy = (c->cfg.ny + tlq::MTY - 1) / tlq::MTY;
  d.gz = tiles_z(c, b->zlen[i]);
}

// Work list of the members in `which` (all when empty), most planes per tile
// first so that the persistent blocks' static stride mixes long and short
// tiles evenly.
std::vector<Item> make_items(const tlq_batch* b, const std::vector<int>& which) {
  std::vector<Item> v;
  std::vector<int> ms = which;
  if (ms.empty())
    for (int i = 0; i < (int)b->m.size(); ++i) ms.push_back(i);
  std::stable_sort(ms.begin(), ms.end(), [&](int x, int y) { return b->zlen[x] > b->zlen[y]; });
  for (int i : ms) {
    const tlq_ctx* c = b->m[i];
    const int gx = (c->cfg.nx + tlq::MTX - 1) / tlq::MTX, gy = (c->cfg.ny + tlq::MTY - 1) / tlq::MTY;
    const int gz = tiles_z(c, b->zlen[i]);
    for (int bz = 0; bz < gz; ++bz)
      for (int by = 0; by < gy; ++by)
        for (int bx = 0; bx < gx; ++bx) v.push_back(Item{i, bx, by, bz});
  }
  return v;
}

int upload_items(tlq_batch* b, const std::vector<Item>& v) {
  if ((int)v.size() > b->cap_items) {
    cudaFree(b->d_items);
    b->d_items = nullptr;
    BCK(cudaMalloc(&b->d_items, v.size() * sizeof(Item)));
    b->cap_items = (int)v.size();
  }
  BCK(cudaMemcpyAsync(b->d_items, v.data(), v.size() * sizeof(Item), cudaMemcpyHostToDevice, b->stream));
  b->nitems = (int)v.size();
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // one persistent grid serves both stages: the smaller residency of the two
  int per_sm = 0, per_sm1 = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tlq::stage_kernel_mixed_batch<2>, tlq::MNT,
                                                sizeof(tlq::BatchSmem<2>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, tlq::stage_kernel_mixed_batch<1>, tlq::MNT,
                                                sizeof(tlq::BatchSmem<1>));
  per_sm = std::min(per_sm, per_sm1);
  b->blocks = std::max(1, std::min(b->nitems, nsm * std::max(per_sm, 1)));
  return TLQ_OK;
}

// Descriptors of all members, and the cooling-pass arguments of the
// surrogate members in `which` (all when empty).
int refresh_desc(tlq_batch* b, const std::vector<int>& which = {}) {
  for (int i = 0; i < (int)b->m.size(); ++i) fill_desc(b, i);
  BCK(cudaMemcpyAsync(b->d_desc, b->h_desc.data(), b->h_desc.size() * sizeof(MemberDesc), cudaMemcpyHostToDevice,
                      b->stream));
  // each surrogate member gets its own blocks of the three cooling passes: one
  // resident wave of the network pass (152 SMs x 3 blocks) shared in
  // proportion to the cells
  const size_t jb = tlq::cool_job_bytes();
  std::vector<int> cool;
  long long cells = 0;
  for (int i = 0; i < (int)b->m.size(); ++i) {
    tlq_ctx* c = b->m[i];
    if (c->cfg.cooling != TLQ_COOL_MLP) continue;
    if (!which.empty() && std::find(which.begin(), which.end(), i) == which.end()) continue;
    cool.push_back(i);
    cells += (long long)c->cfg.nx * c->cfg.ny * c->cfg.nz;
  }
  constexpr long long WAVE = 152 * 3;
  b->ncool = 0;
  b->cool_blocks = 0;
  for (int i : cool) {
    tlq_ctx* c = b->m[i];
    const long long ci = (long long)c->cfg.nx * c->cfg.ny * c->cfg.nz;
    const int nblk = (int)std::max(1LL, std::min((long long)tlq::cool_pass_blocks(c->P), WAVE * ci / cells));
    const MemberDesc& d = b->h_desc[i];
    tlq::fill_cool_job(b->h_cool.data() + b->ncool * jb, c->P, c->L, c->U[0], c->U[1], c->it_base, c->clk,
                       c->mlp_image, c->mlp_norm, c->mlp_box, c->cool_counts, c->mlp_cqueue, c->mlp_qcount + 1,
                       c->mlp_nqueue, c->mlp_qcount + 2, b->cool_blocks, nblk);
    b->cool_blocks += nblk;
    ++b->ncool;
  }
  if (b->ncool) BCK(cudaMemcpyAsync(b->d_cool, b->h_cool.data(), b->ncool * jb, cudaMemcpyHostToDevice, b->stream));
  return TLQ_OK;
}

// One batched step of the members the item list holds: the two persistent
// stage launches, then the surrogate's three cooling passes over the members
// that use it (their stage 2 queued the cooling cells and left the dt
// reduction to them; refresh_desc wrote their arguments).
int enqueue_batch_step(tlq_batch* b) {
  const size_t smem1 = sizeof(tlq::BatchSmem<1>), smem2 = sizeof(tlq::BatchSmem<2>);
  // the specialised kernels when every member uses their limiter and solver
  bool spec = true;
  for (tlq_ctx* c : b->m) spec = spec && c->P.limiter == tlq::SPEC_LIM && c->P.solver == tlq::SPEC_SOLV;
  if (spec) {
    tlq::stage_kernel_mixed_batch<1, tlq::SPEC_LIM, tlq::SPEC_SOLV>
        <<<b->blocks, tlq::MNT, smem1, b->stream>>>(b->d_desc, b->d_items, b->nitems);
    BCK(cudaGetLastError());
    tlq::stage_kernel_mixed_batch<2, tlq::SPEC_LIM, tlq::SPEC_SOLV>
        <<<b->blocks, tlq::MNT, smem2, b->stream>>>(b->d_desc, b->d_items, b->nitems);
  } else {
    tlq::stage_kernel_mixed_batch<1><<<b->blocks, tlq::MNT, smem1, b->stream>>>(b->d_desc, b->d_items, b->nitems);
    BCK(cudaGetLastError());
    tlq::stage_kernel_mixed_batch<2><<<b->blocks, tlq::MNT, smem2, b->stream>>>(b->d_desc, b->d_items, b->nitems);
  }
  BCK(cudaGetLastError());
  if (b->ncool) BCK(tlq::launch_cool_mlp_dt_batch(b->d_cool, b->ncool, b->cool_blocks, b->stream));
  return TLQ_OK;
}

bool graph_stale(const tlq_batch* b) {
  if (!b->graph) return true;
  for (size_t i = 0; i < b->m.size(); ++i)
    if (b->m[i]->gen != b->gen_seen[i]) return true;
  return false;
}

int build_batch_graph(tlq_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  int rc = upload_items(b, make_items(b, {}));
  if (rc) return rc;
  cudaGraph_t g = nullptr;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  rc = enqueue_batch_step(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  BCK(e);
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  BCK(e);
  for (size_t i = 0; i < b->m.size(); ++i) b->gen_seen[i] = b->m[i]->gen;
  return TLQ_OK;
}

// ---- autotuner cache: one JSON object, one entry per line ----------------
std::string device_name() {
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp pr{};
  cudaGetDeviceProperties(&pr, dev);
  return pr.name;
}

std::map<std::string, std::pair<int, double>> read_cache(const char* path, const std::string& gpu) {
  std::map<std::string, std::pair<int, double>> m;
  if (!path || !*path) return m;
  FILE* f = std::fopen(path, "r");
  if (!f) return m;
  char line[512];
  bool same_gpu = false;
  while (std::fgets(line, sizeof line, f)) {
    char name[256];
    if (std::sscanf(line, " \"gpu\": \"%255[^\"]\"", name) == 1) same_gpu = (gpu == name);
    int nx, ny, nz, z;
    double ms;
    char form[16];
    if (std::sscanf(line, " \"%dx%dx%d/%15[a-z0-9_]\": {\"zlen\": %d, \"ms_per_step\": %lf", &nx, &ny, &nz, form, &z,
                    &ms) == 6)
      m[std::to_string(nx) + "x" + std::to_string(ny) + "x" + std::to_string(nz) + "/" + form] = {z, ms};
  }
  std::fclose(f);
  if (!same_gpu) m.clear();
  return m;
}

int write_cache(const char* path, const std::string& gpu, const std::map<std::string, std::pair<int, double>>& m) {
  if (!path || !*path) return TLQ_OK;
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return TLQ_ERR_ARG;
  std::fprintf(f, "{\n  \"gpu\": \"%s\",\n  \"tuned\": {\n", gpu.c_str());
  size_t q = 0;
  for (const auto& kv : m)
    std::fprintf(f, "    \"%s\": {\"zlen\": %d, \"ms_per_step\": %.6f}%s\n", kv.first.c_str(), kv.second.first,
                 kv.second.second, ++q < m.size() ? "," : "");
  std::fprintf(f, "  }\n}\n");
  std::fclose(f);
  return std::rename(tmp.c_str(), path) == 0 ? TLQ_OK : TLQ_ERR_ARG;
}

}  // namespace

extern "C" {

int tlq_batch_create(const tlq_config* cfgs, int n, tlq_batch** out) {
  if (!cfgs || n < 1 || !out) return TLQ_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (cfgs[i].precision != TLQ_PREC_MIXED || cfgs[i].self_gravity) return TLQ_ERR_CONFIG;
  tlq_batch* b = new tlq_batch();
  auto bail = [&](int code) {
    tlq_batch_destroy(b);
    return code;
  };
  for (int i = 0; i < n; ++i) {
    tlq_ctx* c = nullptr;
    const int rc = tlq_create(&cfgs[i], &c);
    if (rc != TLQ_OK) return bail(rc);
    b->m.push_back(c);
    b->zlen.push_back(c->zlen);
    b->gen_seen.push_back(~0u);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(TLQ_ERR_CUDA);
  for (tlq_ctx* c : b->m)
    if (tlq_set_stream(c, b->stream) != TLQ_OK) return bail(TLQ_ERR_CUDA);
  b->h_desc.resize(n);
  if (cudaMalloc(&b->d_desc, n * sizeof(MemberDesc)) != cudaSuccess) return bail(TLQ_ERR_NOMEM);
  b->h_cool.resize((size_t)n * tlq::cool_job_bytes());
  if (cudaMalloc(&b->d_cool, b->h_cool.size()) != cudaSuccess) return bail(TLQ_ERR_NOMEM);
  if (tlq::prepare_batch_kernels() != cudaSuccess) return bail(TLQ_ERR_CUDA);
  for (int q = 0; q < 2; ++q) cudaEventCreate(&b->ev[q]);
  *out = b;
  return TLQ_OK;
}

int tlq_batch_destroy(tlq_batch* b) {
  if (!b) return TLQ_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (tlq_ctx* c : b->m) tlq_destroy(c);  // the batch's stream is borrowed, not destroyed there
  cudaFree(b->d_desc);
  cudaFree(b->d_items);
  cudaFree(b->d_cool);
  for (int q = 0; q < 2; ++q)
    if (b->ev[q]) cudaEventDestroy(b->ev[q]);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return TLQ_OK;
}

int tlq_batch_size(const tlq_batch* b) { return b ? (int)b->m.size() : 0; }

tlq_ctx* tlq_batch_member(tlq_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->m.size()) return nullptr;
  return b->m[i];
}

const char* tlq_batch_last_error(const tlq_batch* b) { return b ? b->err.c_str() : "null batch"; }

int tlq_batch_set_tiling(tlq_batch* b, int i, int zlen) {
  if (!b || i < 0 || i >= (int)b->m.size() || zlen < 8) return TLQ_ERR_ARG;
  b->zlen[i] = std::min(zlen, b->m[i]->cfg.nz);
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return TLQ_OK;
}

int tlq_batch_get_tiling(const tlq_batch* b, int i, int* zlen) {
  if (!b || i < 0 || i >= (int)b->m.size() || !zlen) return TLQ_ERR_ARG;
  *zlen = b->zlen[i];
  return TLQ_OK;
}

int tlq_batch_run(tlq_batch* b, int steps) {
  if (!b || steps < 0) return TLQ_ERR_ARG;
  for (size_t i = 0; i < b->m.size(); ++i) {
    if (!b->m[i]->uploaded) return bfail(b, TLQ_ERR_STATE, "member " + std::to_string(i) + " has no state (tlq_upload)");
    if (b->m[i]->cfg.cooling == TLQ_COOL_MLP && !b->m[i]->mlp_ready)
      return bfail(b, TLQ_ERR_STATE, "member " + std::to_string(i) + " uses the cooling surrogate but has no network");
  }
  int rc = refresh_desc(b);
  if (rc) return rc;
  if (graph_stale(b)) {
    rc = build_batch_graph(b);
    if (rc) return rc;
  }
  if (b->timing) BCK(cudaEventRecord(b->ev[0], b->stream));
  for (int q = 0; q < steps; ++q) BCK(cudaGraphLaunch(b->graph, b->stream));
  if (b->timing) {
    BCK(cudaEventRecord(b->ev[1], b->stream));
    BCK(cudaEventSynchronize(b->ev[1]));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
    b->ms_acc += ms;
    b->steps_timed += steps;
  }
  b->steps += steps;
  return TLQ_OK;
}

int tlq_batch_synchronize(tlq_batch* b) {
  if (!b) return TLQ_ERR_ARG;
  BCK(cudaStreamSynchronize(b->stream));
  return TLQ_OK;
}

int tlq_batch_status(tlq_batch* b, int* status) {
  if (!b || !status) return TLQ_ERR_ARG;
  BCK(cudaStreamSynchronize(b->stream));
  int worst = TLQ_OK;
  for (size_t i = 0; i < b->m.size(); ++i) {
    double t = 0.0, dt = 0.0;
    int it = 0;
    const int rc = tlq_get_time(b->m[i], &t, &it, &dt);
    status[i] = rc;
    if (rc != TLQ_OK && worst == TLQ_OK) worst = rc;
  }
  return worst == TLQ_ERR_CUDA ? TLQ_ERR_CUDA : TLQ_OK;
}

int tlq_batch_enable_timing(tlq_batch* b, int on) {
  if (!b) return TLQ_ERR_ARG;
  b->timing = on != 0;
  b->ms_acc = 0.0;
  b->steps_timed = 0;
  return TLQ_OK;
}

int tlq_batch_stats_get(tlq_batch* b, tlq_batch_stats* s) {
  if (!b || !s) return TLQ_ERR_ARG;
  std::memset(s, 0, sizeof(*s));
  s->members = (int)b->m.size();
  s->steps = b->steps;
  s->steps_timed = b->steps_timed;
  s->ms_per_step = b->steps_timed ? b->ms_acc / (double)b->steps_timed : 0.0;
  s->items = b->nitems;
  s->blocks = b->blocks;
  s->launches_per_step = 2;  // the two stages, and the three cooling passes when a member uses the surrogate
  for (tlq_ctx* c : b->m)
    if (c->cfg.cooling == TLQ_COOL_MLP) {
      s->launches_per_step = 5;
      break;
    }
  long long cells = 0;
  for (tlq_ctx* c : b->m) cells += (long long)c->cfg.nx * c->cfg.ny * c->cfg.nz;
  s->cells = cells;
  s->graph = b->graph ? 1 : 0;
  return TLQ_OK;
}

// For each distinct mesh size: the cached z-chunk length, or one measured
// now.  Every candidate (8, 16, 32, 64, 128 planes, at most nz) is timed over
// `steps` steps (after one warm-up step) of the batch restricted to the
// members of that size, starting each time from the members' current state,
// which is restored afterwards (state, clock).  The winner is written to
// the cache (one JSON object per file, keyed by the GPU's name).
int tlq_batch_autotune(tlq_batch* b, const char* cache_path, int steps, int* chosen) {
  if (!b || steps < 1) return TLQ_ERR_ARG;
  for (size_t i = 0; i < b->m.size(); ++i)
    if (!b->m[i]->uploaded) return bfail(b, TLQ_ERR_STATE, "autotune needs every member's state (tlq_upload)");
  for (size_t i = 0; i < b->m.size(); ++i)
    if (b->m[i]->cfg.cooling == TLQ_COOL_MLP && !b->m[i]->mlp_ready)
      return bfail(b, TLQ_ERR_STATE, "member " + std::to_string(i) + " uses the cooling surrogate but has no network");
  const std::string gpu = device_name();
  auto cache = read_cache(cache_path, gpu);
  std::map<std::string, std::vector<int>> classes;
  for (size_t i = 0; i < b->m.size(); ++i) {
    const tlq_config& c = b->m[i]->cfg;
    classes[std::to_string(c.nx) + "x" + std::to_string(c.ny) + "x" + std::to_string(c.nz) + "/batch_mixed"].push_back(
        (int)i);
  }
  bool wrote = false;
  for (auto& kv : classes) {
    const std::vector<int>& mem = kv.second;
    auto hit = cache.find(kv.first);
    if (hit != cache.end()) {
      for (int i : mem) b->zlen[i] = std::min(hit->second.first, b->m[i]->cfg.nz);
      continue;
    }
    // snapshot the members' current state and clocks
    std::vector<double*> snap(mem.size(), nullptr);
    std::vector<tlq::Clock> clk(mem.size());
    std::vector<int> cur(mem.size());
    for (size_t q = 0; q < mem.size(); ++q) {
      tlq_ctx* c = b->m[mem[q]];
      double t, dt;
      int it;
      tlq_get_time(c, &t, &it, &dt);  // settles c->cur
      cur[q] = c->cur;
      BCK(cudaMalloc(&snap[q], (size_t)c->L.plane * 5 * sizeof(double)));
      BCK(cudaMemcpyAsync(snap[q], c->U[cur[q]], (size_t)c->L.plane * 5 * sizeof(double), cudaMemcpyDeviceToDevice,
                          b->stream));
      BCK(cudaMemcpyAsync(&clk[q], c->clk, sizeof(tlq::Clock), cudaMemcpyDeviceToHost, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
    const int nz = b->m[mem[0]]->cfg.nz;
    int best = b->zlen[mem[0]];
    double best_ms = 1e300;
    for (int z : {8, 16, 32, 64, 128}) {
      if (z > nz && z != 8) continue;
      for (int i : mem) b->zlen[i] = std::min(z, b->m[i]->cfg.nz);
      int rc = refresh_desc(b, mem);
      if (!rc) rc = upload_items(b, make_items(b, mem));
      if (rc) return rc;
      for (int w = 0; w < steps + 1; ++w) {
        if (w == 1) BCK(cudaEventRecord(b->ev[0], b->stream));
        rc = enqueue_batch_step(b);
        if (rc) return rc;
      }
      BCK(cudaEventRecord(b->ev[1], b->stream));
      BCK(cudaEventSynchronize(b->ev[1]));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
      const double per = ms / steps;
      if (per < best_ms) {
        best_ms = per;
        best = z;
      }
      // back to the snapshot
      for (size_t q = 0; q < mem.size(); ++q) {
        tlq_ctx* c = b->m[mem[q]];
        BCK(cudaMemcpyAsync(c->U[cur[q]], snap[q], (size_t)c->L.plane * 5 * sizeof(double),
                            cudaMemcpyDeviceToDevice, b->stream));
        BCK(cudaMemcpyAsync(c->clk, &clk[q], sizeof(tlq::Clock), cudaMemcpyHostToDevice, b->stream));
      }
      BCK(cudaStreamSynchronize(b->stream));
    }
    for (size_t q = 0; q < mem.size(); ++q) {
      cudaFree(snap[q]);
      tlq_ctx* c = b->m[mem[q]];
      if (c->cool_counts) cudaMemsetAsync(c->cool_counts, 0, 3 * sizeof(unsigned long long), b->stream);
    }
    for (int i : mem) b->zlen[i] = std::min(best, b->m[i]->cfg.nz);
    cache[kv.first] = {best, best_ms};
    wrote = true;
  }
  if (wrote && write_cache(cache_path, gpu, cache) != TLQ_OK)
    return bfail(b, TLQ_ERR_ARG, std::string("cannot write the tuning cache ") + (cache_path ? cache_path : ""));
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  if (chosen)
    for (size_t i = 0; i < b->m.size(); ++i) chosen[i] = b->zlen[i];
  return TLQ_OK;
}

// The same tuner for one context: the z-chunk length of its stage grid,
// from the cache or measured over `steps` steps from the current state
// (restored afterwards), keyed by mesh size and form (mixed / fp64).
int tlq_autotune(tlq_ctx* ctx, const char* cache_path, int steps, int* chosen) {
  if (!ctx || steps < 1) return TLQ_ERR_ARG;
  if (!ctx->uploaded) {
    ctx->err = "autotune needs the state (tlq_upload)";
    return TLQ_ERR_STATE;
  }
  const std::string gpu = device_name();
  auto cache = read_cache(cache_path, gpu);
  const tlq_config& c = ctx->cfg;
  const std::string key = std::to_string(c.nx) + "x" + std::to_string(c.ny) + "x" + std::to_string(c.nz) +
                          (c.precision == TLQ_PREC_MIXED ? "/mixed" : "/fp64") +
                          (c.cooling == TLQ_COOL_MLP ? "_mlp" : "");
  auto hit = cache.find(key);
  int best = ctx->zlen;
  if (hit != cache.end()) {
    best = hit->second.first;
  } else {
    double t, dt;
    int it;
    int rc = tlq_get_time(ctx, &t, &it, &dt);
    if (rc != TLQ_OK) return rc;
    const int cur = ctx->cur;
    // the state: U, and the carried cooled pressure of the plain form
    const bool carried = c.cooling != TLQ_COOL_NONE && c.precision == TLQ_PREC_FP64;
    const size_t bytes = (size_t)ctx->L.plane * 5 * sizeof(double);
    const size_t pbytes = carried ? (size_t)ctx->L.plane * sizeof(double) : 0;
    // and the self-gravity potential (each solve starts from the last one)
    const long long mg = c.self_gravity ? (long long)(c.nx + 2) * (c.nx + 2) * (c.nx + 2) : 0;
    const size_t gbytes = (size_t)mg * sizeof(double);
    double* snap = nullptr;
    tlq::Clock clk{};
    if (cudaMalloc(&snap, bytes + pbytes + gbytes) != cudaSuccess) return TLQ_ERR_NOMEM;
    double* gsnap = snap + (bytes + pbytes) / sizeof(double);
    cudaMemcpyAsync(snap, ctx->U[cur], bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (carried) cudaMemcpyAsync(snap + ctx->L.plane * 5, ctx->Pc, pbytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (mg) cudaMemcpyAsync(gsnap, ctx->phig, gbytes, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(&clk, ctx->clk, sizeof(clk), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    const long long steps0 = ctx->steps;
    double best_ms = 1e300;
    for (int z : {8, 16, 32, 64, 128}) {
      if (z > c.nz && z != 8) continue;
      rc = ctx_set_zlen(ctx, std::min(z, c.nz));
      if (rc == TLQ_OK) rc = tlq_advance(ctx, 1);  // warm-up
      if (rc == TLQ_OK) rc = tlq_enable_timing(ctx, 1);
      if (rc == TLQ_OK) rc = tlq_advance(ctx, steps);
      tlq_stats s{};
      if (rc == TLQ_OK) rc = tlq_stats_get(ctx, &s);
      tlq_enable_timing(ctx, 0);
      if (rc != TLQ_OK) {
        cudaFree(snap);
        return rc;
      }
      const double ms = s.ms_stage1 + s.ms_stage2 + s.ms_cool + s.ms_grav;
      if (ms < best_ms) {
        best_ms = ms;
        best = std::min(z, c.nz);
      }
      // back to the snapshot
      cudaMemcpyAsync(ctx->U[cur], snap, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
      if (carried) cudaMemcpyAsync(ctx->Pc, snap + ctx->L.plane * 5, pbytes, cudaMemcpyDeviceToDevice, ctx->stream);
      if (mg) cudaMemcpyAsync(ctx->phig, gsnap, gbytes, cudaMemcpyDeviceToDevice, ctx->stream);
      cudaMemcpyAsync(ctx->clk, &clk, sizeof(clk), cudaMemcpyHostToDevice, ctx->stream);
      if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaFree(snap);
        return TLQ_ERR_CUDA;
      }
      ctx->cur = cur;
    }
    cudaFree(snap);
    ctx->steps = steps0;
    if (ctx->cool_counts) cudaMemsetAsync(ctx->cool_counts, 0, 3 * sizeof(unsigned long long), ctx->stream);
    cache[key] = {best, best_ms};
    if (write_cache(cache_path, gpu, cache) != TLQ_OK) {
      ctx->err = std::string("cannot write the tuning cache ") + (cache_path ? cache_path : "");
      return TLQ_ERR_ARG;
    }
  }
  const int rc = ctx_set_zlen(ctx, best);
  if (rc != TLQ_OK) return rc;
  if (chosen) *chosen = ctx->zlen;
  return TLQ_OK;
}

}  // extern "C"
