// tlq_internal.h -- launchers shared between the kernel translation units and
// the host API (tlq_api.cu).  Not part of the public ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "tlq_stage.cuh"

namespace tlq {

// Reference layout A(5, -1:nx+2, -1:ny+2, -1:nz+2), variable fastest.
struct Aos {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return 5LL * ((long long)(i + 1) + (long long)(nx + 4) * ((long long)(j + 1) + (long long)(ny + 4) * (long long)(k + 1)));
  }
  __host__ __device__ __forceinline__ long long cells() const {
    return (long long)(nx + 4) * (long long)(ny + 4) * (long long)(nz + 4);
  }
};

// Potential phi(0:nx+1, 0:ny+1, 0:nz+1) of the reference (pointsource_gravity.f90:14).
struct PhiLayout {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)i + (long long)(nx + 2) * ((long long)j + (long long)(ny + 2) * (long long)k);
  }
};

constexpr int RED_THREADS = 256;  // block size of the reduction kernels

// Fused step (FP64 instantiations in tlq_kernels.cu).
cudaError_t prepare_stage_kernels();
size_t stage_smem_bytes(int precision);
cudaError_t launch_stage(int stage, int precision, const CUtensorMap& tm_in, const CUtensorMap& tm_p,
                         const StageArgs& a, dim3 grid, cudaStream_t s);

// Mixed-precision stage kernels (tlq_mixed.cu).
cudaError_t prepare_mixed_kernels();
cudaError_t prepare_batch_kernels();  // tlq_batch.cu
size_t mixed_smem_bytes(int stage);
cudaError_t launch_stage_mixed(int stage, const CUtensorMap& tm_in, const StageArgs& a, dim3 grid, cudaStream_t s);
// The first dt of the mixed form (its FP32 signal speeds; tlq_mixed.cu).
cudaError_t launch_init_dt_mixed(const Params& p, const Layout& L, const double* U, Clock* clk, int nblocks,
                                 cudaStream_t s);

// Layout conversions and per-step helpers (SoA device state).
cudaError_t launch_aos_to_soa(const Aos& A, const Layout& L, const double* src, double* dst, cudaStream_t s);
cudaError_t launch_soa_to_aos(const Aos& A, const Layout& L, const double* src, double* dst, cudaStream_t s);
cudaError_t launch_prims_soa_to_aos_clocked(const Params& p, const Aos& A, const Layout& L, const double* U0,
                                            const double* U1, const Clock* clk, long long it_base, const double* P,
                                            double* W, cudaStream_t s);
cudaError_t launch_prims_soa_to_aos(const Params& p, const Aos& A, const Layout& L, const double* U,
                                    const double* P, double* W, cudaStream_t s);
// calc_prims + time_step on the uploaded state; writes P (interior pressure)
// when P is non-null; clk->dt receives the first dt.
cudaError_t launch_init_prims_dt(const Params& p, const Layout& L, const double* U, double* P, Clock* clk,
                                 int nblocks, cudaStream_t s);
int init_blocks(const Params& p);
// dst[q] = FP32 of src[q] (the mixed kernels' rounding), q < n.
cudaError_t launch_to_f32(const double* src, float* dst, long long n, cudaStream_t s);
cudaError_t launch_point_potential_soa(const Params& p, const Layout& L, const double* xyzm, int n, double* phi,
                                       cudaStream_t s);
cudaError_t launch_conserved_sums(const Params& p, const Layout& L, const double* U, double* partials, int nblocks,
                                  double* out5, cudaStream_t s);

// Cooling surrogate (tlq_mlp.cu).
size_t mlp_train_smem();
cudaError_t launch_mlp_grad(const float* P, const float* X, const float* Y, const float* Wt, int nb, float* grad,
                            float* loss, int nblocks, cudaStream_t s);
cudaError_t launch_adam(float* P, float* m, float* v, const float* grad, int n, float lr, float b1, float b2,
                        float eps, int t, cudaStream_t s);
cudaError_t launch_mlp_infer(const float* P, const float* X, int n, float* Y, cudaStream_t s);
// The step's image of a network (its shared-memory layout, mlp_image_bytes()
// of device memory), formed from the FP32 parameters P.
size_t mlp_image_bytes();
cudaError_t launch_pack_weights(const float* P, void* img, cudaStream_t s);
cudaError_t launch_cool_pairs(const Params& p, long long N, unsigned long long seed, const double box[6], float* X,
                              float* Y, float* Wt, double* raw, cudaStream_t s);
cudaError_t launch_gather_pairs(const float* X, const float* Y, const float* Wt, const long long* perm, long long N,
                                float* X2, float* Y2, float* Wt2, cudaStream_t s);
cudaError_t launch_normalise(float* X, long long N, const float norm[6], cudaStream_t s);
// Surrogate cooling + dt reduction of the mixed step (tlq_surrogate.cu).
// Stage 2 cools the cells the exact integrator takes in one step, queues
// the other cells that cool (cqueue) and folds its block maxima into the
// clock's; the sort pass queues those in the training box for the network
// (nqueue) and cools the others with the exact integrator; the network pass
// cools its cells (its prediction, or the exact integrator's where the
// residual check fails); the dt pass finishes the dt reduction.  Queues:
// capacity nx ny nz; counts zero between steps.
cudaError_t launch_cool_mlp_dt(const Params& p, const Layout& L, double* U0, double* U1, long long it_base,
                               Clock* clk, const void* img, const float norm[6], const double box[6],
                               unsigned long long* counts, const unsigned* cqueue, unsigned* cqcount,
                               unsigned* nqueue, unsigned* nqcount, cudaStream_t s);
// The same three passes for several meshes in three launches: fill_cool_job
// writes one mesh's arguments (cool_job_bytes() of them) into a host array
// that is copied to the device; mesh m runs on blocks [blk0, blk0 + nblk) of
// each pass (ranges ascending and back to back from 0, nblk between 1 and
// cool_pass_blocks, nblocks their total).
size_t cool_job_bytes();
int cool_pass_blocks(const Params& p);
void fill_cool_job(void* dst, const Params& p, const Layout& L, double* U0, double* U1, long long it_base, Clock* clk,
                   const void* img, const float norm[6], const double box[6], unsigned long long* counts,
                   const unsigned* cqueue, unsigned* cqcount, unsigned* nqueue, unsigned* nqcount, int blk0,
                   int nblk);
cudaError_t launch_cool_mlp_dt_batch(const void* jobs, int njobs, int nblocks, cudaStream_t s);

// log10 of a small device array in place (cooling-table temperatures).
cudaError_t launch_log10_inplace(double* v, int n, cudaStream_t s);

// Per-routine kernels on the reference layout.
cudaError_t launch_calc_prims_aos(const Params& p, const Aos& A, double* W, const double* U, cudaStream_t s);
cudaError_t launch_time_step_aos(const Params& p, const Aos& A, const double* W, Clock* clk, int nblocks,
                                 cudaStream_t s);
cudaError_t launch_fluxes_aos(const Params& p, const Aos& A, const double* U, const double* W, double* F, double* G,
                              double* H, int choice, cudaStream_t s);
cudaError_t launch_godunov_aos(const Params& p, const Aos& A, double* out, const double* UU, const double* F,
                               const double* G, const double* H, const double* W, const double* phi, double dt,
                               cudaStream_t s);
cudaError_t launch_borders_aos(const Params& p, const Aos& A, double* U, int order, cudaStream_t s);
cudaError_t launch_winds_aos(const Params& p, const Aos& A, double* U, cudaStream_t s);
cudaError_t launch_viscous_step_aos(const Params& p, const Aos& A, double* U, const double* UP, const double* Uold,
                                    cudaStream_t s);
cudaError_t launch_cooling_aos(const Params& p, const Aos& A, double* W, double* U, double dt, cudaStream_t s);
cudaError_t launch_point_potential_ref(const Params& p, const double* xyzm, int n, double* phi, cudaStream_t s);
cudaError_t launch_gravity_source_aos(const Params& p, const Aos& A, const double* W, const double* phi, double* S,
                                      cudaStream_t s);

}  // namespace tlq
