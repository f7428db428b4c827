// nufi_kernels.cuh — launch interface between the host side (nufi_api.cu)
// and the kernels (trace_fp64.cu, trace_split.cu, field_solve.cu).
#pragma once

#include "nufi_common.cuh"

namespace nufi_gb300 {

// Tiling of the trace: a block is 32 spatial nodes (lanes) x `warps`
// warps; each thread owns `ppt` consecutive velocity nodes; `vblocks`
// blocks cover the velocity range (gridDim.y).
struct LaunchShape {
    int warps = 4;
    int ppt = 1;
    int vblocks = 1;
};

// Per-velocity-node constants of the split form.  Axis a, node j is entry
// a * kMaxVelocityTable + j ... stored compactly: offsets vel_off[a].
struct SplitNode {
    double u0;      // grid velocity
    double g;       // FP64 factor of the equilibrium at u0 (see trace_split.cu)
    float u0f;
    float sig_hi, sig_lo;
    float ga, gb;   // FP32 equilibrium factors (meaning depends on f0)
    int S0;         // integer free-streaming shift, reduced mod N
};

// Fixed-order block reduction of one FP64 value per thread into
// partial[blockIdx.y * Ns + s]: lane = spatial node, warps summed in order.
__device__ __forceinline__ void block_reduce_partial(double acc, long long s, long long Ns,
                                                     double *__restrict__ partial)
{
    __shared__ double red[8][32];
    red[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && s < Ns) {
        double t = red[0][threadIdx.x];
        for (int w = 1; w < int(blockDim.y); ++w) t += red[w][threadIdx.x];
        partial[(long long)blockIdx.y * Ns + s] = t;
    }
}

cudaError_t launch_trace_fp64(const Problem &p, const LaunchShape &ls, const double *hist, int n, long long qb,
                              long long qe, int mode, double *partial, unsigned *err, cudaStream_t st);
bool fp64_order_supported(int dim, int order);

cudaError_t launch_trace_split(const Problem &p, const LaunchShape &ls, const float *tables, const SplitNode *nodes,
                               const float2 *phase, int n, long long qb, long long qe, double *partial,
                               unsigned *err, cudaStream_t st);
bool split_supported(int dim, int order, int f0_kind);

// rho[s] = -wv * sum_b partial[b][s], fixed order (drop-in compute_rho).
cudaError_t launch_finalize_rho(const Problem &p, int nvb, const double *partial, double *rho, cudaStream_t st);

// Field-solve resources (twiddles and inverse symbols per axis).
struct SolvePlan {
    double2 *tw[3] = {nullptr, nullptr, nullptr};      // exp(-2 pi i j / N), j < N/2
    double2 *isym[3] = {nullptr, nullptr, nullptr};    // 1 / lambda_a(k)
    double *ksq[3] = {nullptr, nullptr, nullptr};      // (2 pi kfold / L)^2
    int log2n[3] = {0, 0, 0};
    size_t smem = 0;
};

// One block: rho from partials (or from rho_in), FFT, Poisson + spline
// diagonal, inverse FFT, padded slab n (FP64) + FP32 table n, energy n.
cudaError_t launch_field_solve(const Problem &p, const SolvePlan &plan, int nvb, const double *partial,
                               const double *rho_in, double *rho_out, double *hist_slab, float *table_slab,
                               double *energy_out, unsigned *err, cudaStream_t st);
// FP32 table of one FP64 slab (after upload_phi).
cudaError_t field_solve_set_smem(size_t smem);
cudaError_t launch_derive_table(const Problem &p, const double *hist_slab, float *table_slab, cudaStream_t st);

}  // namespace nufi_gb300
