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
// The FP64 traces put min(vblocks, 65535) blocks on the grid's y axis and
// stride over the velocity blocks; one partial-sum row per y block.
constexpr int kMaxGridY = 65535;
inline int fp64_rows(const LaunchShape &ls) { return ls.vblocks < kMaxGridY ? ls.vblocks : kMaxGridY; }

// Per-velocity-node constants of the split form.  Axis a, node j is entry
// a * kMaxVelocityTable + j ... stored compactly: offsets vel_off[a].
struct SplitNode {
    double u0;      // grid velocity
    double g;       // FP64 factor of the equilibrium at u0 (see trace_split.cu)
    float u0f;
    float sig_hi, sig_lo;
    float ga, gb;   // FP32 equilibrium factors (meaning depends on f0)
    int S0;         // integer free-streaming shift, reduced mod N
    int S0u;        // the same shift unreduced, floor(u0 dt/dx) (unwrapped positions)
};

__device__ __forceinline__ void neumaier_add(double &sum, double &comp, double x)
{
    const double t = sum + x;
    comp += (fabs(sum) >= fabs(x)) ? (sum - t) + x : (x - t) + sum;
    sum = t;
}

// Trace blocks of (32 lanes = spatial nodes) x W warps: the warps' values
// are summed in fixed order into partial[blockIdx.y][s]; reduce_rho then
// sums the rows.  No atomics touch rho, so runs are bitwise reproducible
// (the reference uses one atomicAdd per point, nufi/cuda_kernel.cu:50).
__device__ __forceinline__ void write_partial_tiled(double acc, long long s, long long Ns,
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

// 1D split kick table of one slab: for cell i the derivative of the cubic
// spline sum on [i, i+1) as a quadratic in xi, times K = -dt^2/dx^2:
// K B, K C as a float2 at [2i, 2i+1] and K A at [2N + i] (3N floats, padded
// to a multiple of 4).  Two loads per lookup, 12 bytes: three shared-memory
// wavefronts per warp instead of four for a float4 with a dead lane; the
// adjoint's reverse sweep, which needs only the derivative K B + 2 K C xi,
// reads the one float2.
__device__ __forceinline__ void store_kick_entry(float *slab, int N, int i, float A, float B, float C)
{
    reinterpret_cast<float2 *>(slab)[i] = make_float2(B, C);
    slab[2 * N + i] = A;
}
// K (A, B, C) of cell i from c[i..i+3]: the derivative of the cubic
// B-spline sum on [i, i+1) as a quadratic in xi, times K = -dt^2/dx^2 (the
// derive_table kernel, and the staged trace when it derives the newest
// table itself).
__device__ __forceinline__ void cubic_kick_poly(double c0, double c1, double c2, double c3, double K, float *slab,
                                                int N, int i)
{
    const double A = (c2 - c0) * 0.5;
    const double B = (c0 - 2.0 * c1) + c2;
    const double C = ((3.0 * (c1 - c2) - c0) + c3) * 0.5;
    store_kick_entry(slab, N, i, float(K * A), float(K * B), float(K * C));
}
__device__ __forceinline__ float kick_lookup(const float *slab, int N, int i, float xi)
{
    const float2 bc = reinterpret_cast<const float2 *>(slab)[i];
    return fmaf(xi, fmaf(xi, bc.y, bc.x), slab[2 * N + i]);
}
__device__ __forceinline__ float kick_lookup_ldg(const float *slab, int N, int i, float xi)
{
    const float2 bc = __ldg(reinterpret_cast<const float2 *>(slab) + i);
    return fmaf(xi, fmaf(xi, bc.y, bc.x), __ldg(slab + 2 * N + i));
}

// Block sums of the four metrics into partial[k * blocks + block] (fixed
// xor-shuffle tree per warp, warps summed in order: deterministic).
__device__ __forceinline__ void write_metrics_block(const double (&m4)[4], double *__restrict__ partial)
{
    __shared__ double red[4][8];
    const int lane = threadIdx.x, warp = threadIdx.y;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        double v = m4[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (warp == 0 && lane < 4) {
        double t = red[lane][0];
        for (int w = 1; w < int(blockDim.y); ++w) t += red[lane][w];
        const long long blocks = (long long)gridDim.x * gridDim.y;
        partial[lane * blocks + (long long)blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
}

// The trace kernels write per-block partial sums of f~ ([rows][Ns]); the
// launchers return the row count through *rows.  mode 0: f~ (eval_ftilda);
// mode 2: the four metrics of f (eval_f) into [4][blocks] block sums.
// grid: the points' grid (metrics on conf_metrics); nullptr: p's own
cudaError_t launch_trace_fp64(const Problem &p, const LaunchShape &ls, const double *hist, int n, long long qb,
                              long long qe, int mode, double *partial, int *rows, unsigned *err, cudaStream_t st,
                              const PointGrid *grid = nullptr);
bool fp64_order_supported(int dim, int order);
// FP64 order-4 trace in cell units (trace_fp64_table.cu): 1D and 2D over
// per-slab FP64 derivative tables of fp64_table_stride doubles per slab
// (written by launch_derive_table64 from each FP64 slab), 3D over each
// slab's double-float (hi, lo) pairs (one float2 per coefficient, the
// slab's own stride).
bool fp64_table_supported(const Problem &p, long long Nt);
long long fp64_table_stride(const Problem &p);
// the FP64 derivative table of one slab (1D, 2D) or its double-float pairs
// (3D); with hist_out (1D), the slab is also copied there
cudaError_t launch_derive_table64(const Problem &p, const double *hist_slab, double *table_slab, cudaStream_t st,
                                  double *hist_out = nullptr);
cudaError_t launch_trace_fp64_table(const Problem &p, const LaunchShape &ls, const double *tables,
                                    const double *hist, int n, long long qb, long long qe, double *partial,
                                    int *rows, unsigned *err, cudaStream_t st);
// eval_ftilda / eval_f / 1D eval_phase_flow at arbitrary points (FP64).
cudaError_t launch_eval_points(const Problem &p, const double *hist, int n, int mode, long long npts,
                               const double *pts, double *f_out, double *feet, unsigned *err, cudaStream_t st);

cudaError_t launch_trace_split(const Problem &p, const LaunchShape &ls, const float *tables, const SplitNode *nodes,
                               const float2 *phase, int n, long long qb, long long qe, double *partial, int *rows,
                               unsigned *err, cudaStream_t st);
bool split_supported(int dim, int order, int f0_kind);

// Staged FP32-split 1D trace (trace_split_staged.cu): persistent grid of
// `ctas` blocks of `threads` (one spatial node each) with `ppt` velocity
// chains per thread; tables streamed through shared memory in chunks of
// `slabs_per_chunk` slabs.
constexpr int kStagedMaxPPT = 8;
struct StagedShape {
    bool ok = false;
    int ctas = 0, threads = 0, ppt = 0, slabs_per_chunk = 0;
    int tpn = 1;  // threads per spatial node (chain groups)
    int ring = 3;  // shared-memory ring slots (0: 2D/3D tables read from global memory)
    size_t smem = 0;
};
StagedShape staged_shape_1d(const Problem &p, int sms, int ctas_per_sm = 1, int threads_per_node = 1);
// FP32-split 2D/3D trace (trace_split_nd.cu).
StagedShape staged_shape_nd(const Problem &p, int sms);
cudaError_t launch_trace_split_nd(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                                  const float2 *phase, int n, long long qb, long long qe, double *partial, int *rows,
                                  unsigned *err, cudaStream_t st);
// rho of the 1D split traces as 64-bit fixed-point sums (scale 2^F): the
// parts of every CTA are added into sum[N] (zero between launches), the
// last CTA (ticket) writes rho (and pub, *err_pub when given) and clears
// the sums.  sum == nullptr: partial rows for reduce_rho instead.
struct RhoFix {
    unsigned long long *sum = nullptr;
    unsigned *ticket = nullptr;
    double scale = 0, limit = 0;
    double *rho = nullptr, *pub = nullptr;
    unsigned *err_pub = nullptr;
    unsigned *seq_pub = nullptr;  // when given: seq written there after rho and the error word
    unsigned seq = 0;
};
// 2^F and the bound on one CTA's scaled part for `ctas` CTAs each adding,
// per node, the f~ of `chains` chains: no node's sum leaves int64.  False
// when F would be below 24 (then the partial rows).
bool rho_fixed_point(const Problem &p, int ctas, int chains, double &scale, double &limit);
// The newest slab of a staged 1D trace given as FP64 coefficients in mapped
// host memory (an upload not yet derived): every CTA derives its kick table
// into its own ring, and CTA 0 also writes the slab and the table into the
// history.  k = the slab (n - 1 of the trace), -1: none.
struct PendingSlab {
    const double *stage = nullptr;
    long long k = -1;
    double *hist_out = nullptr;
    float *table_out = nullptr;
};
cudaError_t launch_trace_split_staged(const Problem &p, const StagedShape &sh, const float *tables,
                                      const SplitNode *nodes, const float2 *phase, int n, long long qb, long long qe,
                                      double *partial, int *rows, unsigned *err, cudaStream_t st,
                                      const RhoFix &fx = RhoFix(), const PendingSlab &pend = PendingSlab());

// Whole FP32-split 1D simulation in one cooperative launch
// (run_split_1d.cu): staged trace, rho, circulant solve and W_n per step,
// separated by bounded grid barriers.  sync = {barrier count, abort flag}.
constexpr int kMaxCtasPerSm = 2;  // whole-run kernel CTAs per SM (energy parts sized for it)
struct PersistentRun {
    bool ok = false;
    int ctas = 0, threads = 0, ppt = 0, slabs_per_chunk = 0, tpn = 1;
    size_t smem = 0;
    unsigned *sync = nullptr;
    double *epart = nullptr;                // [(Nt+1)][N] rho_i phi_i per step and node
    unsigned long long *rho_fix = nullptr;  // [2][N] rho's fixed-point sums, steps n % 2
    double fix_scale = 0, fix_limit = 0;    // 2^F, and the bound on one CTA's scaled part
};

// rho[s] = -wv * sum over the rows of partial[row][s]: one warp per node,
// lanes take rows in a fixed stride with Neumaier compensation, then a
// fixed xor-shuffle tree; deterministic.
// rho[s] = -wv * (sum over the rows of partial); also into pub (and *err
// into *err_pub) when given
cudaError_t launch_reduce_rho(const Problem &p, int rows, const double *partial, double *rho, cudaStream_t st,
                              double *pub = nullptr, const unsigned *err = nullptr, unsigned *err_pub = nullptr);
// dst[0..n) = src[0..n) by a kernel (either side may be mapped pinned host
// memory); *err_dst = *err_src too when err_src is given
cudaError_t launch_copy_words(const double *src, double *dst, long long n, const unsigned *err_src, unsigned *err_dst,
                              cudaStream_t st);
// metrics[k] = sum over the blocks of partial[k][block] (one warp per
// metric, Neumaier lanes and a fixed shuffle tree).
cudaError_t launch_reduce_metrics(long long blocks, const double *partial, double *metrics, cudaStream_t st);


// Field solve as circulant products (field_solve.cu).  green holds
// nconv kernels of Ns values each: [0] spline coefficients c, [1] Poisson
// potential phi at the nodes, and for the 1D split table [2..4] the
// coefficients K A, K B, K C of the per-cell quadratic.
struct SolvePlan {
    double *green = nullptr;
    int nconv = 0;
    int blocks = 0;              // grid of the solve kernel
    int nodes_per_block = 8;     // 1, 2, 4 or 8: warps per block, one node each
    size_t smem = 0;             // rho' (+ green when staged) in shared memory
    bool green_in_smem = false;
    double *energy_partial = nullptr;  // [max(blocks, SMs)]
    unsigned *energy_counter = nullptr;
    // Grids above kCirculantMaxNodes: the same diagonals applied between
    // per-axis DFTs (spectral_*), O(Ns sum_a N_a) instead of O(Ns^2).
    bool spectral = false;
    double2 *diag = nullptr;     // [2][Ns] D_c, D_phi (complex)
    double2 *work = nullptr;     // [3][Ns] rho^, c^, phi^
    double2 *twiddle = nullptr;  // e^{+2 pi i k / N_a}, axes one after another
    double *mean = nullptr;      // [1]
};
constexpr long long kCirculantMaxNodes = 16384;
constexpr int kSpectralMaxAxis = 4096;  // a line (complex FP64) in shared memory

// Poisson + collocation solve of one step: padded slab n (FP64), the FP32
// table n (when table_slab != null) and the electric energy W_n.  With
// err_pub (circulant form only), *err as the solve leaves it is written
// there too, so that a caller reading slab, W and the word from mapped host
// memory needs no further launch; with seq_pub, the blocks' writes are
// fenced at system scope and seq is written there last (the caller may
// wait for it instead of for the stream).
cudaError_t launch_field_solve(const Problem &p, const SolvePlan &plan, const double *rho, double *hist_slab,
                               float *table_slab, double *energy_out, cudaStream_t st, unsigned *err = nullptr,
                               unsigned *err_pub = nullptr, unsigned *seq_pub = nullptr, unsigned seq = 0);
cudaError_t field_solve_prepare(const SolvePlan &plan);

PersistentRun persistent_shape_1d(const Problem &p, const StagedShape &sh, const SolvePlan &plan, int sms);
cudaError_t launch_run_split_1d(const Problem &p, const PersistentRun &pr, const SolvePlan &plan, float *tables,
                                double *hist, const SplitNode *nodes, const float2 *phase, double *rho, double *energy, int n0, int n1, unsigned *err, cudaStream_t st);
// Reverse-mode gradient of J = 2 dt sum_n W_n with respect to f0's
// (alpha, k, u_b, sigma_b), 1D, FP64 (adjoint_1d.cu).  mu: (Nt+1) x P
// slab adjoints (zeroed by the caller), theta_acc: [4][grid_x*grid_y]
// (zeroed by the caller).
constexpr int kAdjointPPT = 4;
struct AdjointPlan {
    bool ok = false;
    int threads = 0, grid_x = 0, grid_y = 0, chunk = 1;
};
AdjointPlan adjoint_plan_1d(const Problem &p);
cudaError_t launch_adjoint_1d(const Problem &p, const AdjointPlan &ap, const double *hist, const double *gc,
                              double *mu, double *lambda, double *theta_acc, int n1, unsigned *err, cudaStream_t st);

// Batched 1D instances (batch_1d.cu).  One descriptor per instance; the
// unit, node and solve-block maps give each CTA its instance.
constexpr int kBatchMaxN = 256;  // spatial nodes per instance (256 % N == 0)
constexpr int kRingSlots = 3;    // shared-memory ring slots of the split traces
struct BatchInst {
    Problem p;
    double *hist;
    float *tables;
    const SplitNode *nodes;
    const float2 *phase;
    const double *green;
    double *partial;  // [units][N]
    double *rho;      // [N]
    double *energy;   // [Nt+1]
    double *epart;    // [solve_blocks]
    unsigned *ecount; // [1], zero between launches
    double *mu;       // [(Nt+1)][P] slab adjoints
    double *muT;      // [(Nt+1)][N][3] kick-table adjoints (A, B, C of each cell; FP32-split adjoint)
    float *muS;       // [(Nt+1)][N][3] one step's kick-table adjoints, folded into muT after the step
    double *lambda;   // [N]
    int Nt, tpn;
    int unit_begin, units;
    int adj_unit_begin, adj_units;
    int solve_begin, solve_blocks;
    long long node_begin;
};
struct BatchLaunch {
    const BatchInst *inst = nullptr;
    const int *unit_inst = nullptr, *node_inst = nullptr, *solve_inst = nullptr, *adj_unit_inst = nullptr;
    int count = 0, precision = 0, ppt = 4, slabs_per_chunk = 8;
    bool pow2 = true;
    size_t smem = 0;
    int units = 0, solve_blocks = 0;
    long long total_nodes = 0;
    int adj_ppt = 2, adj_chunk = 8, adj_units = 0, max_P = 0;
    int ts_max = 0, max_N = 0;  // largest table stride (floats) and N of the batch
    int adj_grid = 0, max_chunks = 0;  // FP32-split adjoint: persistent CTAs, chunks per step
    float *ckpt = nullptr;             // its checkpoints: adj_grid x max_chunks x 4 x kAdjThreads x adj_ppt floats
    double *theta_acc = nullptr;
    unsigned *err = nullptr;
};
cudaError_t launch_batch_trace(const BatchLaunch &L, int n, cudaStream_t st);
cudaError_t launch_batch_step(const BatchLaunch &L, int n, cudaStream_t st);
// The whole FP32-split batched forward, steps n0..n1, as one cooperative
// launch of `ctas` CTAs (batch_run_split_kernel); sync = {barrier count,
// abort flag}.  batch_run_ctas: the co-resident CTAs for L's shape (0: the
// kernel cannot run, use the per-step launches).
int batch_run_ctas(const BatchLaunch &L, int sms);
cudaError_t launch_batch_run(const BatchLaunch &L, int ctas, int n0, int n1, unsigned *sync, cudaStream_t st);
cudaError_t launch_batch_adjoint_step(const BatchLaunch &L, int m, cudaStream_t st);
cudaError_t launch_batch_theta_reduce(const BatchLaunch &L, double *grad, cudaStream_t st);
constexpr int kAdjChunk = 8;  // slabs per checkpointed chunk of the FP32-split adjoint
constexpr int kAdjRing = 2;   // its staged chunks
constexpr int kAdjThreads = 256;  // threads of its CTAs (two per SM)
size_t adjoint_split_smem(const BatchLaunch &L);
int adjoint_split_ctas_per_sm(const BatchLaunch &L, int ppt);

// FP32 table of one FP64 slab (after upload_phi).
// the split kick table of one slab; with hist_out, the slab is also
// copied there (an upload from the mapped pinned block in one launch)
cudaError_t launch_derive_table(const Problem &p, const double *hist_slab, float *table_slab, cudaStream_t st,
                                double *hist_out = nullptr);

}  // namespace nufi_gb300
