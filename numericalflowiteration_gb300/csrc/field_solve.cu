// field_solve.cu — the per-step work around the trace: rho from the trace's
// partial sums, then the periodic Poisson solve fused with the B-spline
// collocation solve, the padded slab, the FP32 field table and W_n.
//
// The reference (a) transforms rho with FFTW's separable DHT, scales mode
// k by 1/(N |k|^2), zeroes the mean and transforms back
// (nufi/poisson.cpp:66-89, 190-219, 328-362), returning
// W = prod L / 2 * sum_{k != 0} |k|^2 phi_k^2; then (b) solves the circulant
// collocation system sum_j N_j(0) c[(i+j) mod N] = phi_i by LSMR
// (nufi/fields.hpp:63-142, 186-300, 352-490) and writes the periodically
// padded slab c[i] = c~[i mod N].  Both are diagonal in Fourier space
// (the Poisson scaling depends only on the folded |k| per axis, so the DHT
// sandwich equals a DFT sandwich; the collocation matrix is circulant with
// symbol lambda(k) = prod_a sum_j N_j(0) exp(+2 pi i j k_a / N_a)):
//     c = IDFT[ rho^ / (N |k|^2 lambda) ],   phi = IDFT[ rho^ / (N |k|^2) ].
// The host turns each diagonal into its circulant kernel (the inverse DFT
// of the diagonal, computed once per configuration), so a step is a set of
// dense circulant products c_i = sum_j G_c[i - j] rho'_j, spread over many
// blocks.  On this part FP64 runs at 1/64 of the FP32 rate, and a
// single-block FFT per step was serial; the product instead spreads the
// O(N^2) FP64 FMAs over all SMs.  rho' = rho - mean(rho): the kernels sum
// to zero, and removing the O(1) background first keeps the rounding
// relative to the perturbation.  W = prod L / (2 N) * sum_i rho'_i phi_i
// (Parseval), equal to the reference's spectral sum.  Everything is FP64.
#include <algorithm>

#include "nufi_kernels.cuh"

namespace nufi_gb300 {

__global__ void reduce_rho_kernel(const Problem p, int rows, const double *__restrict__ partial,
                                  double *__restrict__ rho, double *__restrict__ pub, const unsigned *__restrict__ err,
                                  unsigned *__restrict__ err_pub)
{
    // rho (and the error word the traces before this launch left) also into
    // the mapped pinned block, when given: a following download needs no
    // launch of its own
    if (err_pub && blockIdx.x == 0 && threadIdx.x == 0) *err_pub = *err;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int Ns = int(p.Ns);
    for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < Ns; s += warps) {
        double sum = 0, comp = 0;
        for (int r = lane; r < rows; r += 32) neumaier_add(sum, comp, partial[(long long)r * Ns + s]);
        for (int off = 16; off > 0; off >>= 1) {
            const double os = __shfl_down_sync(0xffffffffu, sum, off);
            const double oc = __shfl_down_sync(0xffffffffu, comp, off);
            neumaier_add(sum, comp, os);
            comp += oc;
        }
        if (lane == 0) {
            const double v = -p.wv * (sum + comp);
            rho[s] = v;
            if (pub) pub[s] = v;
        }
    }
}

cudaError_t launch_reduce_rho(const Problem &p, int rows, const double *partial, double *rho, cudaStream_t st,
                              double *pub, const unsigned *err, unsigned *err_pub)
{
    // one warp per block: the FP64 work of the few nodes spreads over all SMs
    const int warps_per_block = 1;
    const int blocks = int((p.Ns + warps_per_block - 1) / warps_per_block);
    reduce_rho_kernel<<<blocks, 32 * warps_per_block, 0, st>>>(p, rows, partial, rho, pub, err, err_pub);
    return cudaGetLastError();
}

__global__ void reduce_metrics_kernel(long long blocks, const double *__restrict__ partial, double *__restrict__ out)
{
    const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
    double sum = 0, comp = 0;
    for (long long r = lane; r < blocks; r += 32) neumaier_add(sum, comp, partial[k * blocks + r]);
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, sum, off);
        const double oc = __shfl_down_sync(0xffffffffu, comp, off);
        neumaier_add(sum, comp, os);
        comp += oc;
    }
    if (lane == 0) out[k] = sum + comp;
}

// Small transfers between device memory and the handle's pinned host
// block, done by a kernel: the block is mapped into the device's address
// space (unified addressing), so the copy is one queued launch behind the
// work before it instead of a copy-engine transfer with its own start-up.
// The device error word, when given, travels in the same launch.
__global__ void copy_words_kernel(const double *__restrict__ src, double *__restrict__ dst, long long n,
                                  const unsigned *__restrict__ err_src, unsigned *__restrict__ err_dst)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
    if (err_src && blockIdx.x == 0 && threadIdx.x == 0) *err_dst = *err_src;
}

cudaError_t launch_copy_words(const double *src, double *dst, long long n, const unsigned *err_src, unsigned *err_dst,
                              cudaStream_t st)
{
    const int threads = 256;
    const int blocks = int(std::min<long long>(std::max<long long>((n + threads - 1) / threads, 1), 32));
    copy_words_kernel<<<blocks, threads, 0, st>>>(src, dst, n, err_src, err_dst);
    return cudaGetLastError();
}

cudaError_t launch_reduce_metrics(long long blocks, const double *partial, double *metrics, cudaStream_t st)
{
    reduce_metrics_kernel<<<1, 128, 0, st>>>(blocks, partial, metrics);
    return cudaGetLastError();
}

namespace {

constexpr int kSolveThreads = 256;
constexpr int kSolveWarps = kSolveThreads / 32;

// Sum of one value per thread, fixed-order tree over the block.
__device__ __forceinline__ double block_sum_fixed(double v, double *red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// The same sum in another fixed order, alike in every block of one launch
// shape: a butterfly of shuffles in each warp (every lane ends with the
// same bits: FP64 addition commutes), then the warps' sums in warp order.
// Two block barriers against the tree's one per level: measured 1 us less
// per use in the field solve (two uses).  red: at least blockDim.x / 32.
__device__ __forceinline__ double block_sum_warps(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) r += red[w];
    __syncthreads();
    return r;
}

}  // namespace

// Each block of 32 * nodes_per_block threads owns nodes_per_block nodes, one
// warp per node: the lanes stride over j and one shuffle tree finishes each
// sum,
//   acc[c] = sum_j green[c][(i - j) mod N] * rho'[j]      (mod per axis)
// then the slab (all padded positions of i), the table, and rho'_i phi_i.
// GB300 issues FP64 at 1/64 of the FP32 rate, so the kernel's time is its
// FP64 instruction count: NCONV (Ns/32 + 5) warp instructions per node this
// way, against NCONV (Ns/32 + 6 w) with a node's sum split over w warps.
// D1: the 1D instance (the same values in the same order without the other
// axes' index arithmetic: less code to fetch when the kernel starts cold,
// as it does right after a trace in the drop-in loop).
template <int NCONV, bool D1>
__global__ void __launch_bounds__(kSolveThreads) circulant_solve_kernel(
    const Problem p, const double *__restrict__ rho, const double *__restrict__ green, int green_in_smem,
    double *__restrict__ slab, float *__restrict__ table, double *__restrict__ energy_partial,
    unsigned *__restrict__ energy_counter, double *__restrict__ energy_out, unsigned *err, unsigned *err_pub,
    unsigned *seq_pub, unsigned seq)
{
    extern __shared__ double sm[];
    __shared__ double red[kSolveThreads];
    __shared__ double eacc[kSolveWarps];
    __shared__ bool last;
    const int Ns = int(p.Ns);
    const int N0 = p.N[0], N1 = p.N[1], N2 = p.N[2];
    double *rs = sm;                                    // rho' [Ns]
    const double *G = green_in_smem ? sm + Ns : green;  // [NCONV][Ns]
    // 1. rho' = rho - mean(rho), the mean in fixed order (every block alike).
    // Loads in batches of 8 issued before their use: the input may sit in
    // mapped host memory, where each dependent round trip costs ~1 us.
    constexpr int kLd = 8;
    double part = 0;
    for (int jb = threadIdx.x; jb < Ns; jb += kLd * int(blockDim.x)) {
        double r[kLd];
#pragma unroll
        for (int u = 0; u < kLd; ++u) {
            const int j = jb + u * int(blockDim.x);
            r[u] = j < Ns ? rho[j] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kLd; ++u) {
            const int j = jb + u * int(blockDim.x);
            if (j < Ns) {
                rs[j] = r[u];
                part += r[u];
            }
        }
    }
    if (green_in_smem)
        for (int j = threadIdx.x; j < NCONV * Ns; j += blockDim.x) sm[Ns + j] = green[j];
    const double mean = block_sum_warps(part, red) / double(Ns);
    for (int j = threadIdx.x; j < Ns; j += blockDim.x) rs[j] -= mean;
    __syncthreads();

    // 2. circulant products, node i = this warp's; the green loads of kLd
    // consecutive j-steps are issued together (they come from L2 when the
    // kernels are not staged in shared memory)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.x * int(blockDim.x >> 5) + warp;
    double acc[NCONV];
#pragma unroll
    for (int c = 0; c < NCONV; ++c) acc[c] = 0;
    if (D1 && i < Ns) {
        for (int j = lane; j < Ns; j += kLd * 32) {
            double g[kLd][NCONV];
#pragma unroll
            for (int u = 0; u < kLd; ++u) {
                const int jj = j + 32 * u;
                int m = i - jj;
                m += m < 0 ? N0 : 0;
#pragma unroll
                for (int c = 0; c < NCONV; ++c) g[u][c] = jj < Ns ? G[c * Ns + m] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kLd; ++u) {
                const int jj = j + 32 * u;
                if (jj >= Ns) break;
                const double r = rs[jj];
#pragma unroll
                for (int c = 0; c < NCONV; ++c) acc[c] = fma(g[u][c], r, acc[c]);
            }
        }
    } else if (i < Ns) {
        const int i0 = i % N0, i1 = (i / N0) % N1, i2 = i / (N0 * N1);
        const int step0 = 32 % N0, step1 = (32 / N0) % N1, step2 = 32 / (N0 * N1);
        int j = lane;
        int j0 = j % N0, j1 = (j / N0) % N1, j2 = j / (N0 * N1);
        while (j < Ns) {
            int mm[kLd], jj[kLd];
#pragma unroll
            for (int u = 0; u < kLd; ++u) {
                int m0 = i0 - j0, m1 = i1 - j1, m2 = i2 - j2;
                m0 += m0 < 0 ? N0 : 0;
                m1 += m1 < 0 ? N1 : 0;
                m2 += m2 < 0 ? N2 : 0;
                mm[u] = (m2 * N1 + m1) * N0 + m0;
                jj[u] = j;
                // (j0, j1, j2) of j + 32
                j += 32;
                j0 += step0;
                j1 += step1;
                j2 += step2;
                if (j0 >= N0) { j0 -= N0; ++j1; }
                if (j1 >= N1) { j1 -= N1; ++j2; }
            }
            double g[kLd][NCONV];
#pragma unroll
            for (int u = 0; u < kLd; ++u)
#pragma unroll
                for (int c = 0; c < NCONV; ++c) g[u][c] = jj[u] < Ns ? G[c * Ns + mm[u]] : 0.0;
#pragma unroll
            for (int u = 0; u < kLd; ++u) {
                if (jj[u] >= Ns) break;
                const double r = rs[jj[u]];
#pragma unroll
                for (int c = 0; c < NCONV; ++c) acc[c] = fma(g[u][c], r, acc[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NCONV; ++c)
        for (int off = 16; off > 0; off >>= 1) acc[c] += __shfl_down_sync(0xffffffffu, acc[c], off);
    double e_local = 0;
    if (D1 && lane == 0 && i < Ns) {
        slab[i] = acc[0];
        if (i + N0 < p.P[0]) slab[i + N0] = acc[0];
        if constexpr (NCONV == 5) {
            if (table) store_kick_entry(table, N0, i, float(acc[2]), float(acc[3]), float(acc[4]));
        }
        e_local = rs[i] * acc[1];
    } else if (lane == 0 && i < Ns) {
        const int i0 = i % N0, i1 = (i / N0) % N1, i2 = i / (N0 * N1);
        const double cval = acc[0];
        // every padded position of node i: i_a and i_a + N_a while < P_a
        for (int dz = 0; dz < 2; ++dz) {
            const int k = i2 + dz * N2;
            if (k >= p.P[2]) continue;
            for (int dy = 0; dy < 2; ++dy) {
                const int jj = i1 + dy * N1;
                if (jj >= p.P[1]) continue;
                for (int dx = 0; dx < 2; ++dx) {
                    const int ii = i0 + dx * N0;
                    if (ii >= p.P[0]) continue;
                    const int idx = (k * p.P[1] + jj) * p.P[0] + ii;
                    slab[idx] = cval;
                    if (table && p.dim > 1) table[(k * p.P[1] + jj) * p.table_sx + ii] = float(cval);
                }
            }
        }
        if constexpr (NCONV == 5) {
            if (table)
                store_kick_entry(table, N0, i, float(acc[2]), float(acc[3]), float(acc[4]));
        }
        e_local = rs[i] * acc[1];
    }
    if (lane == 0) eacc[warp] = e_local;
    __syncthreads();
    // 3. energy: block partial (warps in order), the last block sums the blocks
    if (threadIdx.x == 0) {
        double eb = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) eb += eacc[w];
        energy_partial[blockIdx.x] = eb;
    }
    if (seq_pub)
        __threadfence_system();  // the slab writes (host memory) before the ticket, for the host
    else
        __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(energy_counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v = 0;
    for (int b = threadIdx.x; b < int(gridDim.x); b += blockDim.x) v += __ldcg(energy_partial + b);
    // the error word as this solve leaves it (every block's atomics are
    // performed in L2 before its ticket), loaded beside the partial sums
    const unsigned ew = (err_pub && threadIdx.x == 0) ? __ldcg(err) : 0u;
    const double tot = block_sum_warps(v, red);
    if (threadIdx.x == 0) {
        double Lp = 1;
        for (int ax = 0; ax < p.dim; ++ax) Lp *= p.L[ax];
        if (energy_out) energy_out[0] = tot * (Lp / (2.0 * double(Ns)));
        energy_counter[0] = 0u;
        if (err_pub) *err_pub = ew;
        if (seq_pub) {  // after the slab, W and the word: a host that sees seq sees them
            __threadfence_system();
            *reinterpret_cast<volatile unsigned *>(seq_pub) = seq;
        }
    }
}

// ---------------------------------------------------------------------------
// Spectral form of the same solve for grids above kCirculantMaxNodes: the
// dense circulant product costs Ns^2 FMAs per kernel, the transforms
// Ns sum_a N_a.  rho' = rho - mean(rho); rho^ = DFT(rho') (sign -), one
// axis at a time; c^ = D_c rho^, phi^ = D_phi rho^ with the diagonals the
// circulant kernels are made from (host, long double); c, phi = the
// unnormalised inverse DFTs (sign +; the 1/Ns is in D).  Each axis pass is a
// dense DFT of one line per block in shared memory (N_a <= 4096), FP64.
namespace {

__global__ void spectral_mean_kernel(const Problem p, const double *__restrict__ rho, double *__restrict__ mean)
{
    __shared__ double red[kSolveThreads];
    double part = 0;
    for (long long j = threadIdx.x; j < p.Ns; j += blockDim.x) part += rho[j];
    const double tot = block_sum_fixed(part, red);
    if (threadIdx.x == 0) mean[0] = tot / double(p.Ns);
}

// One axis of the DFT over NA arrays in place: block = one line of axis a
// (length N, stride S in the node index), x_k <- sum_j x_j w^{s jk}, with
// w = e^{2 pi i / N} (tw) and s = -1 (forward) or +1.  REAL_IN: the line is
// read from the real rho (minus the mean) instead of work[0].
template <int NA, bool REAL_IN>
__global__ void __launch_bounds__(kSolveThreads) spectral_axis_kernel(const Problem p, int N, long long S,
                                                                    const double2 *__restrict__ tw, double sign,
                                                                    double2 *work, const double *__restrict__ rho,
                                                                    const double *__restrict__ mean)
{
    extern __shared__ double2 line[];  // [NA][N]
    const long long l = blockIdx.x;    // line: (lo, hi) with node = hi * N * S + j * S + lo
    const long long lo = l % S, hi = l / S;
    const long long base = hi * (long long)N * S + lo;
    const double m = REAL_IN ? mean[0] : 0.0;
    for (int a = 0; a < NA; ++a)
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            const long long idx = base + (long long)j * S;
            line[a * N + j] = REAL_IN ? make_double2(rho[idx] - m, 0.0) : work[(long long)a * p.Ns + idx];
        }
    __syncthreads();
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        double re[NA], im[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) re[a] = im[a] = 0.0;
        int e = 0;  // (j k) mod N
        for (int j = 0; j < N; ++j) {
            const double2 w = tw[e];
            const double wi = sign * w.y;
#pragma unroll
            for (int a = 0; a < NA; ++a) {
                const double2 x = line[a * N + j];
                re[a] = fma(x.x, w.x, fma(-x.y, wi, re[a]));
                im[a] = fma(x.x, wi, fma(x.y, w.x, im[a]));
            }
            e += k;
            if (e >= N) e -= N;
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) work[(long long)a * p.Ns + base + (long long)k * S] = make_double2(re[a], im[a]);
    }
}

// c^ = D_c rho^ (work[1]), phi^ = D_phi rho^ (work[2])
__global__ void spectral_scale_kernel(const Problem p, const double2 *__restrict__ diag, double2 *work)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.Ns) return;
    const double2 x = work[i];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const double2 d = diag[c * p.Ns + i];
        work[(c + 1) * p.Ns + i] = make_double2(d.x * x.x - d.y * x.y, d.x * x.y + d.y * x.x);
    }
}

// Slab (every padded position of node i) from Re c, and W_n = prod L /
// (2 Ns) sum_i rho'_i phi_i (block parts in fixed order, the last block
// sums them, as circulant_solve_kernel).
__global__ void __launch_bounds__(kSolveThreads) spectral_finish_kernel(
    const Problem p, const double *__restrict__ rho, const double *__restrict__ mean,
    const double2 *__restrict__ work, double *__restrict__ slab, double *__restrict__ energy_partial,
    unsigned *__restrict__ energy_counter, double *__restrict__ energy_out)
{
    __shared__ double red[kSolveThreads];
    __shared__ bool last;
    const long long Ns = p.Ns;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e_local = 0;
    if (i < Ns) {
        const int N0 = p.N[0], N1 = p.N[1], N2 = p.N[2];
        const int i0 = int(i % N0), i1 = int((i / N0) % N1), i2 = int(i / ((long long)N0 * N1));
        const double cval = work[Ns + i].x;
        for (int dz = 0; dz < 2; ++dz) {
            const int k = i2 + dz * N2;
            if (k >= p.P[2]) continue;
            for (int dy = 0; dy < 2; ++dy) {
                const int jj = i1 + dy * N1;
                if (jj >= p.P[1]) continue;
                for (int dx = 0; dx < 2; ++dx) {
                    const int ii = i0 + dx * N0;
                    if (ii >= p.P[0]) continue;
                    slab[((long long)k * p.P[1] + jj) * p.P[0] + ii] = cval;
                }
            }
        }
        e_local = (rho[i] - mean[0]) * work[2 * Ns + i].x;
    }
    const double eb = block_sum_fixed(e_local, red);
    if (threadIdx.x == 0) energy_partial[blockIdx.x] = eb;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(energy_counter, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v = 0;
    for (int b = threadIdx.x; b < int(gridDim.x); b += blockDim.x) v += __ldcg(energy_partial + b);
    const double tot = block_sum_fixed(v, red);
    if (threadIdx.x == 0) {
        double Lp = 1;
        for (int ax = 0; ax < p.dim; ++ax) Lp *= p.L[ax];
        if (energy_out) energy_out[0] = tot * (Lp / (2.0 * double(Ns)));
        energy_counter[0] = 0u;
    }
}

cudaError_t launch_spectral_solve(const Problem &p, const SolvePlan &plan, const double *rho, double *hist_slab,
                                  float *table_slab, double *energy_out, cudaStream_t st)
{
    spectral_mean_kernel<<<1, kSolveThreads, 0, st>>>(p, rho, plan.mean);
    long long S = 1, toff = 0;
    for (int a = 0; a < p.dim; ++a) {  // forward
        const int N = p.N[a];
        const unsigned lines = unsigned(p.Ns / N);
        if (a == 0)
            spectral_axis_kernel<1, true><<<lines, kSolveThreads, size_t(N) * 16, st>>>(
                p, N, S, plan.twiddle + toff, -1.0, plan.work, rho, plan.mean);
        else
            spectral_axis_kernel<1, false><<<lines, kSolveThreads, size_t(N) * 16, st>>>(
                p, N, S, plan.twiddle + toff, -1.0, plan.work, rho, plan.mean);
        S *= N;
        toff += N;
    }
    spectral_scale_kernel<<<unsigned((p.Ns + 255) / 256), 256, 0, st>>>(p, plan.diag, plan.work);
    S = 1;
    toff = 0;
    for (int a = 0; a < p.dim; ++a) {  // inverse, c^ and phi^ together
        const int N = p.N[a];
        spectral_axis_kernel<2, false><<<unsigned(p.Ns / N), kSolveThreads, size_t(2 * N) * 16, st>>>(
            p, N, S, plan.twiddle + toff, 1.0, plan.work + p.Ns, rho, plan.mean);
        S *= N;
        toff += N;
    }
    const unsigned fb = unsigned((p.Ns + kSolveThreads - 1) / kSolveThreads);
    spectral_finish_kernel<<<fb, kSolveThreads, 0, st>>>(p, rho, plan.mean, plan.work, hist_slab,
                                                         plan.energy_partial, plan.energy_counter, energy_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && table_slab) e = launch_derive_table(p, hist_slab, table_slab, st);
    return e;
}

}  // namespace

cudaError_t field_solve_prepare(const SolvePlan &plan)
{
    if (plan.spectral) {
        cudaError_t e = cudaFuncSetAttribute(spectral_axis_kernel<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSpectralMaxAxis * 16);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(spectral_axis_kernel<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kSpectralMaxAxis * 16);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(spectral_axis_kernel<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     2 * kSpectralMaxAxis * 16);
        return e;
    }
    cudaError_t e = cudaSuccess;
    for (auto fn : {circulant_solve_kernel<2, false>, circulant_solve_kernel<5, false>, circulant_solve_kernel<2, true>,
                    circulant_solve_kernel<5, true>})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(plan.smem));
    return e;
}

cudaError_t launch_field_solve(const Problem &p, const SolvePlan &plan, const double *rho, double *hist_slab,
                               float *table_slab, double *energy_out, cudaStream_t st, unsigned *err,
                               unsigned *err_pub, unsigned *seq_pub, unsigned seq)
{
    if (plan.spectral) {
        if (err_pub || seq_pub) return cudaErrorInvalidValue;  // the spectral form publishes neither
        return launch_spectral_solve(p, plan, rho, hist_slab, table_slab, energy_out, st);
    }
    // without a table, c and phi only: the green rows 0 and 1 of either form
    const unsigned threads = 32u * unsigned(plan.nodes_per_block);
    const bool five = plan.nconv == 5 && table_slab;
    auto fn = p.dim == 1 ? (five ? circulant_solve_kernel<5, true> : circulant_solve_kernel<2, true>)
                         : (five ? circulant_solve_kernel<5, false> : circulant_solve_kernel<2, false>);
    fn<<<plan.blocks, threads, plan.smem, st>>>(p, rho, plan.green, plan.green_in_smem, hist_slab, table_slab,
                                               plan.energy_partial, plan.energy_counter, energy_out, err, err_pub,
                                               seq_pub, seq);
    return cudaGetLastError();
}

__global__ void derive_table_kernel(const Problem p, const double *__restrict__ slab, float *__restrict__ table,
                                    double *__restrict__ hist_out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (hist_out && idx < p.stride_t) hist_out[idx] = slab[idx];  // the slab itself, when it comes from elsewhere
    if (p.dim == 1) {
        if (idx >= p.N[0]) return;
        const double K = -p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
        cubic_kick_poly(slab[idx], slab[idx + 1], slab[idx + 2], slab[idx + 3], K, table, p.N[0], int(idx));
    } else {
        if (idx >= p.stride_t) return;
        const long long row = idx / p.P[0];
        table[row * p.table_sx + idx % p.P[0]] = float(slab[idx]);
    }
}

cudaError_t launch_derive_table(const Problem &p, const double *hist_slab, float *table_slab, cudaStream_t st,
                                double *hist_out)
{
    const long long n = hist_out || p.dim > 1 ? p.stride_t : p.N[0];  // stride_t >= N
    derive_table_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(p, hist_slab, table_slab, hist_out);
    return cudaGetLastError();
}

}  // namespace nufi_gb300
