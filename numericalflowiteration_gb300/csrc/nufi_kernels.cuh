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

// Scratch of the trace kernels: per-block partial sums and one arrival
// counter per 32-node spatial tile (zero between launches: the block that
// completes a tile resets its counter).
struct RhoScratch {
    double *partial;     // [vblocks][Ns]
    unsigned *counter;   // [ceil(Ns / 32)]
};

__device__ __forceinline__ void neumaier_add(double &sum, double &comp, double x)
{
    const double t = sum + x;
    comp += (fabs(sum) >= fabs(x)) ? (sum - t) + x : (x - t) + sum;
    sum = t;
}

// rho[s] = -wv * sum over the velocity nodes of one value per thread.
// 1. per block, fixed order: lane = spatial node, warps summed in order,
//    into partial[blockIdx.y][s];
// 2. the last block to arrive for spatial tile blockIdx.x (ticket counter
//    after a fence) sums that tile's gridDim.y partials in fixed order,
//    compensated, and writes rho; so the result does not depend on which
//    block arrives last, and no atomics touch rho.
__device__ __forceinline__ void finish_rho(double acc, long long s, long long Ns, double wv, RhoScratch scr,
                                           double *__restrict__ rho)
{
    __shared__ double red[8][32];
    __shared__ double red_c[8][32];
    __shared__ bool last;
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    red[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && s < Ns) {
        double t = red[0][lane];
        for (int w = 1; w < W; ++w) t += red[w][lane];
        scr.partial[(long long)blockIdx.y * Ns + s] = t;
    }
    __threadfence();
    __syncthreads();
    if (lane == 0 && warp == 0) {
        const unsigned prev = atomicAdd(scr.counter + blockIdx.x, 1u);
        last = (prev == gridDim.y - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int nb = int(gridDim.y);
    const int chunk = (nb + W - 1) / W;
    const int b0 = warp * chunk, b1 = min(nb, b0 + chunk);
    double sum = 0, comp = 0;
    if (s < Ns)
        for (int b = b0; b < b1; ++b) neumaier_add(sum, comp, __ldcg(scr.partial + (long long)b * Ns + s));
    red[warp][lane] = sum;
    red_c[warp][lane] = comp;
    __syncthreads();
    if (warp == 0) {
        if (s < Ns) {
            double t = 0, c = 0;
            for (int w = 0; w < W; ++w) {
                neumaier_add(t, c, red[w][lane]);
                c += red_c[w][lane];
            }
            rho[s] = -wv * (t + c);
        }
        if (lane == 0) scr.counter[blockIdx.x] = 0u;
    }
}

cudaError_t launch_trace_fp64(const Problem &p, const LaunchShape &ls, const double *hist, int n, long long qb,
                              long long qe, int mode, RhoScratch scr, double *rho, unsigned *err, cudaStream_t st);
bool fp64_order_supported(int dim, int order);

cudaError_t launch_trace_split(const Problem &p, const LaunchShape &ls, const float *tables, const SplitNode *nodes,
                               const float2 *phase, int n, long long qb, long long qe, RhoScratch scr, double *rho,
                               unsigned *err, cudaStream_t st);
bool split_supported(int dim, int order, int f0_kind);


// Field-solve resources (twiddles and inverse symbols per axis).
struct SolvePlan {
    double2 *tw[3] = {nullptr, nullptr, nullptr};      // exp(-2 pi i j / N), j < N/2
    double2 *isym[3] = {nullptr, nullptr, nullptr};    // 1 / lambda_a(k)
    double *ksq[3] = {nullptr, nullptr, nullptr};      // (2 pi kfold / L)^2
    int log2n[3] = {0, 0, 0};
    size_t smem = 0;
};

// One block: FFT of rho, Poisson + spline diagonal, inverse FFT, padded
// slab n (FP64) + FP32 table n (when table_slab != null), energy n.
cudaError_t launch_field_solve(const Problem &p, const SolvePlan &plan, const double *rho, double *hist_slab,
                               float *table_slab, double *energy_out, unsigned *err, cudaStream_t st);
// FP32 table of one FP64 slab (after upload_phi).
cudaError_t field_solve_set_smem(size_t smem);
cudaError_t launch_derive_table(const Problem &p, const double *hist_slab, float *table_slab, cudaStream_t st);

}  // namespace nufi_gb300
