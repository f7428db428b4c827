// batch_1d.cu — many 1D1V instances of uneven grid sizes advanced together.
//
// Every instance keeps its own history, tables, Green's kernels and split
// constants (one nufi handle each); the batch adds the work decomposition.
// A work unit is one CTA of 256 threads over one instance: its N spatial
// nodes x tpn = 256/N thread groups x PPT velocity chains per thread, i.e.
// 256*PPT points whatever the instance, so units of small and large
// instances cost the same per substep and the hardware block scheduler
// balances them.  Per time step n (all instances in lockstep; an instance
// whose Nt < n sits out):
//   trace   one launch over the units of all instances (FP32-split with
//           the tables streamed through a shared-memory ring as in
//           trace_split_staged.cu, or FP64 as trace_fp64.cu); each unit
//           writes its partial row of f~ sums
//   reduce  one warp per (instance, node): rho from the instance's rows
//   solve   blocks of 8 nodes of one instance: the circulant products of
//           field_solve.cu, slab n, table n, W_n (last-block ticket per
//           instance)
// The adjoint (adjoint_1d.cu's mathematics) runs per step m = max Nt .. 0
// as lambda (one block per instance) + the adjoint trace over units.
// The host captures the step loops into CUDA graphs.
#include <algorithm>

#include "adjoint_device.cuh"
#include "split_device.cuh"

namespace nufi_gb300 {

using namespace split;

// Thread -> (spatial node, chain group) of a unit.
struct UnitMap {
    int s, grp, N, tpn;
    long long m0;  // first velocity node of this thread's chains
};

__device__ __forceinline__ UnitMap unit_map(const BatchInst &I, int unit, int ppt)
{
    UnitMap u;
    u.N = I.p.N[0];
    u.tpn = I.tpn;
    u.s = threadIdx.x % u.N;
    u.grp = threadIdx.x / u.N;
    u.m0 = ((long long)unit * u.tpn + u.grp) * ppt;
    return u;
}

// Sum of the tpn groups' values of a node in group order; group 0 holds it.
__device__ __forceinline__ double combine_groups(double acc, const UnitMap &u, double *comb)
{
    if (u.tpn > 1) {
        comb[threadIdx.x] = acc;
        __syncthreads();
        if (u.grp == 0)
            for (int g = 1; g < u.tpn; ++g) acc += comb[g * u.N + u.s];
    }
    return acc;
}

template <int PPT, bool POW2>
__global__ void __launch_bounds__(256, 1) batch_trace_split_kernel(const BatchInst *__restrict__ bi,
                                                                const int *__restrict__ unit_inst, int n, int S,
                                                                unsigned *err)
{
    extern __shared__ __align__(128) float ring[];
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    __shared__ double comb[256];
    const BatchInst &I = bi[unit_inst[blockIdx.x]];
    if (n > I.Nt) return;
    const Problem &p = I.p;
    const UnitMap um = unit_map(I, blockIdx.x - I.unit_begin, PPT);
    const int N = um.N;
    const long long Nm = p.Nm;

    int Ic[PPT], S0m[PPT];
    float xi[PPT], dwT[PPT], dwTc[PPT], shi[PPT], slo[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = um.m0 + q;
        live[q] = m < Nm;
        const SplitNode nd = I.nodes[live[q] ? m : 0];
        S0m[q] = nd.S0 + kMagicBits;
        shi[q] = nd.sig_hi;
        slo[q] = nd.sig_lo;
        Ic[q] = um.s;
        xi[q] = 0.0f;
        dwT[q] = slo[q];
        dwTc[q] = 0.0f;
    }
    if (n > 0) {
        const int TS = int(p.table_stride);
        const int nchunks = (n + S - 1) / S;
        const unsigned slab_bytes = unsigned(TS) * 4u;
        if (threadIdx.x == 0) {
            for (int r = 0; r < kRing; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
            mbar_fence_init();
        }
        __syncthreads();
        auto issue = [&](int j) {
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            const unsigned bytes = unsigned(k_hi - k_lo + 1) * slab_bytes;
            const unsigned bar = smem_addr(&full_bar[j % kRing]);
            mbar_expect_tx(bar, bytes);
            bulk_g2s(smem_addr(ring + (j % kRing) * S * TS), I.tables + (long long)k_lo * TS, bytes, bar);
        };
        if (threadIdx.x == 0)
            for (int j = 0; j < kRing && j < nchunks; ++j) issue(j);
        bool ok = true;
        for (int j = 0; j < nchunks; ++j) {
            const int slot = j % kRing;
            ok &= mbar_wait(smem_addr(&full_bar[slot]), unsigned((j / kRing) & 1));
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            trace_chunk<PPT, POW2>(ring + slot * S * TS, TS, k_hi, k_lo, N, Ic, xi, dwT, dwTc, shi, S0m, err);
            __syncthreads();  // everyone is done with this slot
            if (threadIdx.x == 0 && j + kRing < nchunks) issue(j + kRing);
        }
        if (!ok) atomicOr(err, kErrStageTimeout);
    }
    const F0 f = make_f0(p);
    double acc = 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        const SplitNode nd = I.nodes[um.m0 + q];
        acc += double(delta_f0(f, nd, __ldg(I.phase + Ic[q]), xi[q], (dwT[q] - dwTc[q]) - slo[q])) + nd.g;
    }
    acc = combine_groups(acc, um, comb);
    if (um.grp == 0) I.partial[(long long)(blockIdx.x - I.unit_begin) * N + um.s] = acc;
}

template <int PPT>
__global__ void __launch_bounds__(256, 1) batch_trace_fp64_kernel(const BatchInst *__restrict__ bi,
                                                               const int *__restrict__ unit_inst, int n,
                                                               unsigned *err)
{
    __shared__ double comb[256];
    const BatchInst &I = bi[unit_inst[blockIdx.x]];
    if (n > I.Nt) return;
    const Problem &p = I.p;
    const UnitMap um = unit_map(I, blockIdx.x - I.unit_begin, PPT);
    const double dt = p.dt;
    double x[PPT], u[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = um.m0 + q;
        live[q] = m < p.Nm;
        x[q] = p.xmin[0] + um.s * p.dx[0];
        u[q] = p.vmin[0] + (live[q] ? m : 0) * p.dv[0] + p.dv[0] / 2;
    }
    // eval_ftilda (nufi/rho.hpp:31-61) with the arithmetic of trace_fp64.cu
    for (int k = n - 1; k >= 1; --k) {
        const double *c = I.hist + k * p.hist_stride;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            if (!live[q]) continue;
            x[q] = x[q] - dt * u[q];
            u[q] = u[q] + dt * adj::efield_primal<4>(p, c, x[q], err);
        }
    }
    if (n > 0) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            if (!live[q]) continue;
            x[q] -= dt * u[q];
            u[q] += 0.5 * dt * adj::efield_primal<4>(p, I.hist, x[q], err);
        }
    }
    double acc = 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q)
        if (live[q]) acc += f0_1d(p, x[q], u[q]);
    acc = combine_groups(acc, um, comb);
    if (um.grp == 0) I.partial[(long long)(blockIdx.x - I.unit_begin) * um.N + um.s] = acc;
}

// rho of every instance: one warp per (instance, node), lanes over the
// instance's unit rows in fixed stride with Neumaier compensation.
__global__ void batch_reduce_kernel(const BatchInst *__restrict__ bi, const int *__restrict__ node_inst,
                                    long long total_nodes, int n)
{
    const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (g >= total_nodes) return;
    const BatchInst &I = bi[node_inst[g]];
    if (n > I.Nt) return;
    const int N = I.p.N[0];
    const int s = int(g - I.node_begin);
    double sum = 0, comp = 0;
    for (int r = lane; r < I.units; r += 32) neumaier_add(sum, comp, I.partial[(long long)r * N + s]);
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, sum, off);
        const double oc = __shfl_down_sync(0xffffffffu, comp, off);
        neumaier_add(sum, comp, os);
        comp += oc;
    }
    if (lane == 0) I.rho[s] = -I.p.wv * (sum + comp);
}

// Fixed-order block sum (any multiple of 32 threads).
__device__ __forceinline__ double bsum(double v, double *red)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) t += red[w];
    return t;
}

// Field solve of every instance: block = 8 nodes of one instance, one warp
// per node (circulant products of field_solve.cu; green from global).
template <int NCONV>
__global__ void __launch_bounds__(256, 1) batch_solve_kernel(const BatchInst *__restrict__ bi,
                                                          const int *__restrict__ solve_inst, int n)
{
    __shared__ double rs[kBatchMaxN];
    __shared__ double red[8];
    __shared__ double ered[8];
    __shared__ bool last;
    const BatchInst &I = bi[solve_inst[blockIdx.x]];
    if (n > I.Nt) return;
    const Problem &p = I.p;
    const int N = p.N[0];
    const int lb = blockIdx.x - I.solve_begin;
    double part = 0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double r = __ldcg(I.rho + j);
        rs[j] = r;
        part += r;
    }
    const double mean = bsum(part, red) / double(N);
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) rs[j] -= mean;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = lb * 8 + warp;
    double e_local = 0;
    if (i < N) {
        double a[NCONV];
#pragma unroll
        for (int c = 0; c < NCONV; ++c) a[c] = 0;
        for (int j = lane; j < N; j += 32) {
            int m = i - j;
            m += m < 0 ? N : 0;
            const double r = rs[j];
#pragma unroll
            for (int c = 0; c < NCONV; ++c) a[c] = fma(I.green[c * N + m], r, a[c]);
        }
#pragma unroll
        for (int c = 0; c < NCONV; ++c)
            for (int off = 16; off > 0; off >>= 1) a[c] += __shfl_down_sync(0xffffffffu, a[c], off);
        if (lane == 0) {
            double *slab = I.hist + (long long)n * p.hist_stride;
            slab[i] = a[0];
            for (int q = i + N; q < p.P[0]; q += N) slab[q] = a[0];
            if constexpr (NCONV == 5)
                store_kick_entry(I.tables + (long long)n * p.table_stride, N, i, float(a[2]), float(a[3]),
                                 float(a[4]));
            e_local = rs[i] * a[1];
        }
    }
    if (lane == 0) ered[warp] = e_local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double eb = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) eb += ered[w];
        I.epart[lb] = eb;
        __threadfence();
        last = atomicAdd(I.ecount, 1u) == unsigned(I.solve_blocks - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double tot = 0;
    for (int b = 0; b < I.solve_blocks; ++b) tot += __ldcg(I.epart + b);
    I.energy[n] = tot * (p.L[0] / (2.0 * double(N)));
    *I.ecount = 0u;
}

// lambda_m of every instance (adjoint_1d.cu): one block per instance.
__global__ void batch_adjoint_lambda_kernel(const BatchInst *__restrict__ bi, int m)
{
    __shared__ double mt[kBatchMaxN];
    const BatchInst &I = bi[blockIdx.x];
    if (m > I.Nt) return;
    const Problem &p = I.p;
    const int N = p.N[0], P = p.P[0];
    const double *mu_m = I.mu + (long long)m * P;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double v = mu_m[i];
        for (int q = i + N; q < P; q += N) v += mu_m[q];
        mt[i] = v;
    }
    __syncthreads();
    double b[4];
    bspline_basis<double, 4, 0>(0.0, b);
    const double scale = 2.0 * p.dt * p.L[0] / N;
    const double *slab = I.hist + (long long)m * p.hist_stride;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double phi = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) phi += b[j] * slab[i + j];
        double t = 0;
        for (int j = 0; j < N; ++j) {
            int d = j - i;
            d += d < 0 ? N : 0;
            t = fma(I.green[d], mt[j], t);
        }
        I.lambda[i] = scale * phi + t;
    }
}

template <int PPT>
__global__ void __launch_bounds__(256, 1) batch_adjoint_trace_kernel(const BatchInst *__restrict__ bi,
                                                                  const int *__restrict__ unit_inst, int m,
                                                                  int chunk, double *__restrict__ theta_acc,
                                                                  long long slots, unsigned *err)
{
    extern __shared__ double mu_s[];
    const BatchInst &I = bi[unit_inst[blockIdx.x]];
    if (m > I.Nt) return;
    const Problem &p = I.p;
    const UnitMap um = unit_map(I, blockIdx.x - I.adj_unit_begin, PPT);
    double x[PPT], u[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long mm = um.m0 + q;
        live[q] = mm < p.Nm;
        x[q] = p.xmin[0] + um.s * p.dx[0];
        u[q] = p.vmin[0] + (live[q] ? mm : 0) * p.dv[0] + p.dv[0] / 2;
    }
    const double a = -p.wv * I.lambda[um.s];
    double th[4] = {0, 0, 0, 0};
    adj::adjoint_chains<4, PPT>(p, I.hist, m, chunk, a, x, u, live, mu_s, I.mu, th, err);
    adj::block_theta_add(th, theta_acc, slots, blockIdx.x);
}

// grad[b*4 + i] = sum over instance b's adjoint units of theta_acc[i][unit]
// (one warp per (instance, parameter), fixed order).
__global__ void batch_theta_reduce_kernel(const BatchInst *__restrict__ bi, int count, const double *theta_acc,
                                          long long slots, double *grad)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= 4 * count) return;
    const int b = w / 4, i = w % 4;
    const BatchInst &I = bi[b];
    double sum = 0, comp = 0;
    for (int r = lane; r < I.adj_units; r += 32) neumaier_add(sum, comp, theta_acc[i * slots + I.adj_unit_begin + r]);
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, sum, off);
        const double oc = __shfl_down_sync(0xffffffffu, comp, off);
        neumaier_add(sum, comp, os);
        comp += oc;
    }
    if (lane == 0) grad[w] = sum + comp;
}


// ---------------------------------------------------------------------------
// FP32-split adjoint (1D, N a power of two), with the characteristics
// recomputed in the split arithmetic itself and checkpointed:
//   pass 1  the trace to the foot (slabs m-1..0), in chunks of kAdjChunk
//           slabs aligned at slab 0 (chunk c = slabs [8c, 8c+7]); the chain
//           state entering each chunk (unwrapped cell U, fraction xi, kick
//           sums dwT, dwTc) goes to a checkpoint area of this CTA
//   seed    at the foot: Xbar = a dx df0/dx, Vbar = a (dx/dt) df0/du,
//           thetabar += a df0/dtheta, a = -w lambda_m(s) (x unwrapped)
//   pass 2  chunks c = 0, 1, ...: reload the checkpoint, recompute the
//           chunk's substeps (same operations, so the same bits) keeping
//           each substep's cell and fraction in registers, then run the
//           adjoint of those substeps in ascending k:
//             Xbar <- Xbar + Vbar h g'(xi);  Vbar <- Vbar - Xbar (compensated)
//             kick-table adjoints of slab k: (Abar, Bbar, Cbar) += Vbar h (1, xi, xi^2)
//           (cells and cells per substep; g' = d/dxi of the kick quadratic),
//           summed in shared memory by red.shared.add.f32 and flushed into
//           the instance's FP64 table adjoints after each chunk.
// About three forward passes of work; the adjoint's own recurrences are
// short.  A persistent grid: CTA b handles units b, b + G, ...; its
// checkpoints live in ckpt + b * (chunks * 4 * 256 * PPT) floats.
// ---------------------------------------------------------------------------

// f0 partial derivatives in FP32 at x (unwrapped), u: as adj::f0_grad_1d.
struct F0GradF {
    float fx, fu, dth[4];
};
__device__ __forceinline__ F0GradF f0_grad_1d_f(const Problem &p, float x, float u)
{
    const float alpha = float(p.f0p[0]), k = float(p.f0p[1]);
    const float c0 = 0.398942280401432678f;
    float sk, ck;
    sincosf(k * x, &sk, &ck);
    const float sp = 1.f + alpha * ck;
    float g, gu, gub = 0.f, gsb = 0.f;
    if (p.f0_kind == NUFI_F0_LANDAU) {
        g = c0 * expf(-0.5f * u * u);
        gu = -u * g;
    } else if (p.f0_kind == NUFI_F0_TWO_STREAM) {
        const float e = c0 * expf(-0.5f * u * u);
        g = e * u * u;
        gu = e * u * (2.f - u * u);
    } else {
        const float ubv = float(p.f0p[2]), sb = float(p.f0p[3]);
        const float z = (u - ubv) / sb;
        const float e1 = c0 * expf(-0.5f * u * u), e2 = c0 / sb * expf(-0.5f * z * z);
        g = 0.9f * e1 + 0.1f * e2;
        gu = -0.9f * u * e1 - 0.1f * z / sb * e2;
        gub = 0.1f * z / sb * e2;
        gsb = 0.1f * (z * z - 1.f) / sb * e2;
    }
    F0GradF r;
    r.fx = -alpha * k * sk * g;
    r.fu = sp * gu;
    r.dth[0] = ck * g;
    r.dth[1] = -alpha * x * sk * g;
    r.dth[2] = sp * gub;
    r.dth[3] = sp * gsb;
    return r;
}

// float -> double by bit manipulation (exact for normal numbers; zero and
// subnormals give 0), keeping the conversion off the FP64 pipe.
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0) return 0.0;
    const unsigned long long bits = ((unsigned long long)(b >> 31) << 63) |
                                    ((unsigned long long)(e + (1023u - 127u)) << 52) |
                                    ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

// Shared-memory add without a returned value.
__device__ __forceinline__ void red_shared_add(float *p, float v)
{
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(smem_addr(p)), "f"(v) : "memory");
}

// One split substep with an unwrapped cell count U (J = U & mask): the
// drift of trace_chunk (split_device.cuh) and the kick lookup.
__device__ __forceinline__ float split_substep(int &U, float &xi, float dwT, float dwC, float shi, int S0um, int mask,
                                               const float *tk, int N, int &J)
{
    const float t = ((xi - shi) - dwT) - dwC;
    const float mg = __fadd_rd(t, kMagic);
    U = U - S0um + __float_as_int(mg);
    J = U & mask;
    xi = t - (mg - kMagic);
    return kick_lookup(tk, N, J, xi);
}

template <int PPT>
__global__ void __launch_bounds__(256, 1) batch_adjoint_split_kernel(const BatchInst *__restrict__ bi,
                                                                     const int *__restrict__ unit_inst, int units,
                                                                     int m, int ts_max, int max_chunks,
                                                                     float *__restrict__ ckpt,
                                                                     double *__restrict__ theta_acc, long long slots,
                                                                     unsigned *err)
{
    constexpr int SC = kAdjChunk;
    extern __shared__ __align__(128) float ring[];  // [kRing][SC][ts_max], then [SC][3 max_N]
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    float *accT = ring + size_t(kRing) * SC * ts_max;
    if (threadIdx.x == 0) {
        for (int r = 0; r < kRing; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int t = threadIdx.x;
    float *ck = ckpt + (size_t)blockIdx.x * max_chunks * 4 * 256 * PPT;
    unsigned g = 0;  // chunks consumed by this CTA: slot g % kRing, parity (g / kRing) & 1
    bool ok = true;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const BatchInst &I = bi[unit_inst[unit]];
        if (m > I.Nt) continue;
        const Problem &p = I.p;
        const UnitMap um = unit_map(I, unit - I.adj_unit_begin, PPT);
        const int N = um.N, mask = N - 1, TS = int(p.table_stride);
        const unsigned slab_bytes = unsigned(TS) * 4u;
        const int C = (m + SC - 1) / SC;  // chunks of this step
        auto issue = [&](int c, unsigned gg) {
            const int k_lo = c * SC, k_hi = min(m - 1, k_lo + SC - 1);
            const unsigned bytes = unsigned(k_hi - k_lo + 1) * slab_bytes;
            const unsigned bar = smem_addr(&full_bar[gg % kRing]);
            mbar_expect_tx(bar, bytes);
            bulk_g2s(smem_addr(ring + (gg % kRing) * SC * ts_max), I.tables + (long long)k_lo * TS, bytes, bar);
        };
        int U[PPT], S0um[PPT];
        float xi[PPT], dwT[PPT], dwTc[PPT], shi[PPT], slo[PPT];
        bool live[PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const long long mm = um.m0 + q;
            live[q] = mm < p.Nm;
            const SplitNode nd = I.nodes[live[q] ? mm : 0];
            S0um[q] = nd.S0u + kMagicBits;
            shi[q] = nd.sig_hi;
            slo[q] = nd.sig_lo;
            U[q] = um.s;
            xi[q] = 0.f;
            dwT[q] = slo[q];
            dwTc[q] = 0.f;
        }
        // ---- pass 1: chunks C-1 .. 0 (descending k), checkpoint each entry state
        if (threadIdx.x == 0)
            for (int j = 0; j < kRing && j < C; ++j) issue(C - 1 - j, g + j);
        for (int j = 0; j < C; ++j, ++g) {
            const int c = C - 1 - j;
            float *cp = ck + (size_t)c * 4 * 256 * PPT;
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                cp[(0 * PPT + q) * 256 + t] = __int_as_float(U[q]);
                cp[(1 * PPT + q) * 256 + t] = xi[q];
                cp[(2 * PPT + q) * 256 + t] = dwT[q];
                cp[(3 * PPT + q) * 256 + t] = dwTc[q];
            }
            ok &= mbar_wait(smem_addr(&full_bar[g % kRing]), (g / kRing) & 1u);
            const float *chunk = ring + (g % kRing) * SC * ts_max;
            const int k_lo = c * SC, k_hi = min(m - 1, k_lo + SC - 1);
            float dwC[PPT];
#pragma unroll
            for (int q = 0; q < PPT; ++q) dwC[q] = 0.f;
            for (int k = k_hi; k >= k_lo; --k) {
                const float *tk = chunk + (k - k_lo) * TS;
                const float h = k == 0 ? 0.5f : 1.0f;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    int J;
                    const float kq = split_substep(U[q], xi[q], dwT[q], dwC[q], shi[q], S0um[q], mask, tk, N, J);
                    dwC[q] = fmaf(h, kq, dwC[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < PPT; ++q) kick(dwT[q], dwTc[q], dwC[q]);
            __syncthreads();
            if (threadIdx.x == 0 && j + kRing < C) issue(C - 1 - (j + kRing), g + kRing);
        }
        // ---- seed at the foot
        const float a = float(-p.wv * I.lambda[um.s]);
        const float dx = float(p.dx[0]), dxdt = float(p.dx[0] / p.dt);
        float xb[PPT], vb[PPT], vbc[PPT];
        double th[4] = {0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            xb[q] = vb[q] = vbc[q] = 0.f;
            if (!live[q]) continue;
            const float x = float(p.xmin[0]) + (float(U[q]) + xi[q]) * dx;
            const float u = I.nodes[um.m0 + q].u0f + ((dwT[q] - dwTc[q]) - slo[q]) * dxdt;
            const F0GradF gr = f0_grad_1d_f(p, x, u);
            xb[q] = a * dx * gr.fx;
            vb[q] = a * dxdt * gr.fu;
#pragma unroll
            for (int i = 0; i < 4; ++i) th[i] += double(a) * double(gr.dth[i]);
        }
        // ---- pass 2: chunks 0 .. C-1 (ascending k)
        for (int i = threadIdx.x; i < SC * 3 * N; i += blockDim.x) accT[i] = 0.f;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int j = 0; j < kRing && j < C; ++j) issue(j, g + j);
        for (int c = 0; c < C; ++c, ++g) {
            const float *cp = ck + (size_t)c * 4 * 256 * PPT;
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                U[q] = __float_as_int(cp[(0 * PPT + q) * 256 + t]);
                xi[q] = cp[(1 * PPT + q) * 256 + t];
                dwT[q] = cp[(2 * PPT + q) * 256 + t];
                dwTc[q] = cp[(3 * PPT + q) * 256 + t];
            }
            ok &= mbar_wait(smem_addr(&full_bar[g % kRing]), (g / kRing) & 1u);
            const float *chunk = ring + (g % kRing) * SC * ts_max;
            const int k_lo = c * SC, k_hi = min(m - 1, k_lo + SC - 1);
            // recompute: substep k = k_lo + i keeps its cell and fraction
            int Js[SC][PPT];
            float xs[SC][PPT];
            float dwC[PPT];
#pragma unroll
            for (int q = 0; q < PPT; ++q) dwC[q] = 0.f;
#pragma unroll
            for (int i = SC - 1; i >= 0; --i) {
                const int k = k_lo + i;
                if (k > k_hi) continue;
                const float *tk = chunk + i * TS;
                const float h = k == 0 ? 0.5f : 1.0f;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    int J;
                    const float kq = split_substep(U[q], xi[q], dwT[q], dwC[q], shi[q], S0um[q], mask, tk, N, J);
                    dwC[q] = fmaf(h, kq, dwC[q]);
                    Js[i][q] = J;
                    xs[i][q] = xi[q];
                }
            }
            // adjoint of the chunk's substeps, k ascending
#pragma unroll
            for (int i = 0; i < SC; ++i) {
                const int k = k_lo + i;
                if (k > k_hi) continue;
                const float *tk = chunk + i * TS;
                float *ak = accT + i * 3 * N;
                const float h = k == 0 ? 0.5f : 1.0f;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    const int J = Js[i][q];
                    const float x = xs[i][q];
                    const float b = reinterpret_cast<const float2 *>(tk)[J].y;
                    const float cc = tk[2 * N + J];
                    const float gp = fmaf(2.f * x, cc, b);
                    const float vh = vb[q] * h;
                    if (live[q]) {
                        red_shared_add(ak + J, vh);
                        red_shared_add(ak + N + J, vh * x);
                        red_shared_add(ak + 2 * N + J, vh * x * x);
                    }
                    xb[q] = fmaf(vh, gp, xb[q]);
                    const float y = -xb[q] - vbc[q];
                    const float tt = vb[q] + y;
                    vbc[q] = (tt - vb[q]) - y;
                    vb[q] = tt;
                }
            }
            __syncthreads();
            if (threadIdx.x == 0 && c + kRing < C) issue(c + kRing, g + kRing);
            for (int i = threadIdx.x; i < (k_hi - k_lo + 1) * 3 * N; i += blockDim.x) {
                const float v = accT[i];
                if (v != 0.f) {
                    atomicAdd(I.muT + (long long)k_lo * 3 * N + i, f2d_bits(v));
                    accT[i] = 0.f;
                }
            }
            __syncthreads();
        }
        adj::block_theta_add(th, theta_acc, slots, unit);
    }
    if (!ok) atomicOr(err, kErrStageTimeout);
}

// lambda_m of every instance from the kick-table adjoints of slab m: the
// coefficient adjoint of each cell's quadratic (K A = K (c2 - c0)/2,
// K B = K (c0 - 2 c1 + c2), K C = K (3 (c1 - c2) - c0 + c3)/2), folded
// onto the N nodes, through G_c^T, plus 2 dt L/N phi_m.
__global__ void batch_adjoint_lambda_split_kernel(const BatchInst *__restrict__ bi, int m)
{
    __shared__ double cb[kBatchMaxN + 8];
    __shared__ double mt[kBatchMaxN];
    const BatchInst &I = bi[blockIdx.x];
    if (m > I.Nt) return;
    const Problem &p = I.p;
    const int N = p.N[0], P = p.P[0];
    const double K = -p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
    const double *t = I.muT + (long long)m * 3 * N;
    // padded coefficient adjoint: cell i feeds c[i..i+3]
    for (int q = threadIdx.x; q < P; q += blockDim.x) {
        double v = 0;
        for (int j = 0; j < 4; ++j) {
            const int i = q - j;
            if (i < 0 || i >= N) continue;
            const double A = t[i], B = t[N + i], C = t[2 * N + i];
            const double w = j == 0 ? (-0.5 * A + B - 0.5 * C)
                           : j == 1 ? (-2.0 * B + 1.5 * C)
                           : j == 2 ? (0.5 * A + B - 1.5 * C)
                                    : 0.5 * C;
            v += K * w;
        }
        cb[q] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double v = cb[i];
        for (int q = i + N; q < P; q += N) v += cb[q];
        mt[i] = v;
    }
    __syncthreads();
    double b[4];
    bspline_basis<double, 4, 0>(0.0, b);
    const double scale = 2.0 * p.dt * p.L[0] / N;
    const double *slab = I.hist + (long long)m * p.hist_stride;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double phi = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) phi += b[j] * slab[i + j];
        double s = 0;
        for (int j = 0; j < N; ++j) {
            int d = j - i;
            d += d < 0 ? N : 0;
            s = fma(I.green[d], mt[j], s);
        }
        I.lambda[i] = scale * phi + s;
    }
}

// ---------------------------------------------------------------------------

cudaError_t launch_batch_trace(const BatchLaunch &L, int n, cudaStream_t st)
{
    if (L.precision == NUFI_PREC_FP32_SPLIT) {
        void (*fn)(const BatchInst *, const int *, int, int, unsigned *) = nullptr;
#define NUFI_CASE(K)                                                                                   \
    case K: fn = L.pow2 ? batch_trace_split_kernel<K, true> : batch_trace_split_kernel<K, false>; break;
        switch (L.ppt) {
            NUFI_CASE(1) NUFI_CASE(2) NUFI_CASE(4) NUFI_CASE(8)
        default: return cudaErrorInvalidValue;
        }
#undef NUFI_CASE
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.smem));
        if (e != cudaSuccess) return e;
        fn<<<L.units, 256, L.smem, st>>>(L.inst, L.unit_inst, n, L.slabs_per_chunk, L.err);
    } else {
        switch (L.ppt) {
        case 1: batch_trace_fp64_kernel<1><<<L.units, 256, 0, st>>>(L.inst, L.unit_inst, n, L.err); break;
        case 2: batch_trace_fp64_kernel<2><<<L.units, 256, 0, st>>>(L.inst, L.unit_inst, n, L.err); break;
        case 4: batch_trace_fp64_kernel<4><<<L.units, 256, 0, st>>>(L.inst, L.unit_inst, n, L.err); break;
        default: return cudaErrorInvalidValue;
        }
    }
    return cudaGetLastError();
}

size_t adjoint_split_smem(const BatchLaunch &L)
{
    return (size_t(kRingSlots) * kAdjChunk * L.ts_max + size_t(kAdjChunk) * 3 * L.max_N) * sizeof(float);
}

int adjoint_split_ctas_per_sm(const BatchLaunch &L, int ppt)
{
    int nb = 0;
    void (*fs)(const BatchInst *, const int *, int, int, int, int, float *, double *, long long, unsigned *) =
        ppt == 1 ? batch_adjoint_split_kernel<1> : batch_adjoint_split_kernel<2>;
    const size_t smem = adjoint_split_smem(L);
    if (cudaFuncSetAttribute(fs, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fs, 256, smem) != cudaSuccess) return 0;
    return nb;
}

cudaError_t launch_batch_step(const BatchLaunch &L, int n, cudaStream_t st)
{
    cudaError_t e = launch_batch_trace(L, n, st);
    if (e != cudaSuccess) return e;
    batch_reduce_kernel<<<unsigned((L.total_nodes * 32 + 255) / 256), 256, 0, st>>>(L.inst, L.node_inst,
                                                                                   L.total_nodes, n);
    if (L.precision == NUFI_PREC_FP32_SPLIT)
        batch_solve_kernel<5><<<L.solve_blocks, 256, 0, st>>>(L.inst, L.solve_inst, n);
    else
        batch_solve_kernel<2><<<L.solve_blocks, 256, 0, st>>>(L.inst, L.solve_inst, n);
    return cudaGetLastError();
}

cudaError_t launch_batch_adjoint_step(const BatchLaunch &L, int m, cudaStream_t st)
{
    if (L.precision == NUFI_PREC_FP32_SPLIT) {
        batch_adjoint_lambda_split_kernel<<<L.count, 256, 0, st>>>(L.inst, m);
        void (*fs)(const BatchInst *, const int *, int, int, int, int, float *, double *, long long,
                   unsigned *) = nullptr;
        switch (L.adj_ppt) {
        case 1: fs = batch_adjoint_split_kernel<1>; break;
        case 2: fs = batch_adjoint_split_kernel<2>; break;
        default: return cudaErrorInvalidValue;
        }
        const size_t smem = adjoint_split_smem(L);
        cudaError_t e = cudaFuncSetAttribute(fs, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        fs<<<L.adj_grid, 256, smem, st>>>(L.inst, L.adj_unit_inst, L.adj_units, m, L.ts_max, L.max_chunks, L.ckpt,
                                         L.theta_acc, L.adj_units, L.err);
        return cudaGetLastError();
    }
    batch_adjoint_lambda_kernel<<<L.count, 256, 0, st>>>(L.inst, m);
    const size_t smem = size_t(L.adj_chunk) * L.max_P * sizeof(double);
    void (*fn)(const BatchInst *, const int *, int, int, double *, long long, unsigned *) = nullptr;
    switch (L.adj_ppt) {
    case 1: fn = batch_adjoint_trace_kernel<1>; break;
    case 2: fn = batch_adjoint_trace_kernel<2>; break;
    case 4: fn = batch_adjoint_trace_kernel<4>; break;
    default: return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    fn<<<L.adj_units, 256, smem, st>>>(L.inst, L.adj_unit_inst, m, L.adj_chunk, L.theta_acc, L.adj_units, L.err);
    return cudaGetLastError();
}

cudaError_t launch_batch_theta_reduce(const BatchLaunch &L, double *grad, cudaStream_t st)
{
    batch_theta_reduce_kernel<<<unsigned((4 * L.count * 32 + 255) / 256), 256, 0, st>>>(L.inst, L.count, L.theta_acc,
                                                                                      L.adj_units, grad);
    return cudaGetLastError();
}

}  // namespace nufi_gb300
