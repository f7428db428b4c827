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
            trace_chunk<PPT, POW2, false, 2>(ring + slot * S * TS, TS, k_hi, k_lo, N, Ic, xi, dwT, dwTc, shi, S0m, err);
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
__device__ __forceinline__ void batch_reduce_node(const BatchInst *__restrict__ bi, const int *__restrict__ node_inst,
                                                  long long g, int lane, int n)
{
    const BatchInst &I = bi[node_inst[g]];
    if (n > I.Nt) return;
    const int N = I.p.N[0];
    const int s = int(g - I.node_begin);
    double sum = 0, comp = 0;
    // __ldcg: in the whole-forward kernel the rows were written by other
    // SMs during this launch (L1 is not coherent across SMs)
    for (int r = lane; r < I.units; r += 32) neumaier_add(sum, comp, __ldcg(I.partial + (long long)r * N + s));
    for (int off = 16; off > 0; off >>= 1) {
        const double os = __shfl_down_sync(0xffffffffu, sum, off);
        const double oc = __shfl_down_sync(0xffffffffu, comp, off);
        neumaier_add(sum, comp, os);
        comp += oc;
    }
    if (lane == 0) I.rho[s] = -I.p.wv * (sum + comp);
}

__global__ void batch_reduce_kernel(const BatchInst *__restrict__ bi, const int *__restrict__ node_inst,
                                    long long total_nodes, int n)
{
    const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g >= total_nodes) return;
    batch_reduce_node(bi, node_inst, g, threadIdx.x & 31, n);
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
// per node (circulant products of field_solve.cu; green from global).  The
// body, for solve block b of the batch, called by all 256 threads of a
// block (rs, red, ered, last in shared memory).
template <int NCONV>
__device__ __forceinline__ void batch_solve_block(const BatchInst &I, int b, int n, double *rs, double *red,
                                                  double *ered, bool *last_flag)
{
    bool &last = *last_flag;
    const Problem &p = I.p;
    const int N = p.N[0];
    const int lb = b - I.solve_begin;
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
    if (last && threadIdx.x == 0) {
        __threadfence();
        double tot = 0;
        for (int q = 0; q < I.solve_blocks; ++q) tot += __ldcg(I.epart + q);
        I.energy[n] = tot * (p.L[0] / (2.0 * double(N)));
        *I.ecount = 0u;
    }
}

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
    batch_solve_block<NCONV>(I, blockIdx.x, n, rs, red, ered, &last);
}

// The whole batched FP32-split forward (steps n0..n1 of every instance) in
// one cooperative launch, the treatment run_split_1d.cu gives one 1D run:
// the grid stays resident (co-resident CTAs of 256 threads) and the phases
// of each step are separated by the bounded grid barrier of
// split_device.cuh:
//   trace   units u = blockIdx.x, blockIdx.x + G, ...: the unit's chains
//           through slabs n-1..0 of its instance's tables, streamed through
//           this CTA's shared-memory ring (the chunk counter g runs on over
//           the units, so every slot's phase stays consistent); its
//           partial row, as batch_trace_split_kernel
//   barrier
//   reduce  warps over the (instance, node) pairs: rho (batch_reduce_node)
//   barrier
//   solve   solve blocks b = blockIdx.x, blockIdx.x + G, ...: 8 nodes of one
//           instance each, slab n, table n and W_n (batch_solve_block)
//   barrier
// The next step's bulk copies read the tables the solve wrote (generic
// stores made visible by the barrier); fence.proxy.async.global orders
// them.  An instance whose Nt is below n sits the step out.  Same
// arithmetic as the graph of per-step launches, and so the same results.
template <int PPT, bool POW2>
__global__ void __launch_bounds__(256, 1) batch_run_split_kernel(const BatchInst *__restrict__ bi,
                                                              const int *__restrict__ unit_inst, int units,
                                                              const int *__restrict__ node_inst,
                                                              long long total_nodes,
                                                              const int *__restrict__ solve_inst, int solve_blocks,
                                                              int n0, int n1, int S, int ts_max, unsigned *sync,
                                                              unsigned *err)
{
    extern __shared__ __align__(128) float ring[];  // [kRing][S][ts_max]
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    __shared__ double comb[256];
    __shared__ double rs[kBatchMaxN];
    __shared__ double red[8];
    __shared__ double ered[8];
    __shared__ bool last;
    unsigned *count = sync, *abort = sync + 1;
    unsigned target = 0;
    if (threadIdx.x == 0) {
        for (int r = 0; r < kRing; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
        mbar_fence_init();
    }
    __syncthreads();
    unsigned g = 0;  // chunks this CTA has consumed: slot g % kRing, parity (g / kRing) & 1
    bool ok = true;
    const int warps = int(blockDim.x >> 5), lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int n = n0; n <= n1; ++n) {
        // ---------------- trace of step n over this CTA's units ----------------
        // Slots have a fixed stride (S slabs of the batch's widest table), so
        // thread 0 can fill a slot the current unit has released with the
        // next unit's first chunks (prefetch; never past the step: the next
        // step's newest tables come from this step's solve).
        if (threadIdx.x == 0) fence_proxy_async_global();
        const int SW = S * ts_max;  // floats per slot
        auto live_from = [&](int u) {  // the first unit from u on that takes part in step n
            for (; u < units; u += gridDim.x)
                if (n <= bi[unit_inst[u]].Nt) return u;
            return units;
        };
        const int nchunks = n > 0 ? (n + S - 1) / S : 0;  // the same for every unit of the step
        // chunk j of unit u into slot (gbase + j) % kRing
        auto issue = [&](int u, int j, unsigned gbase) {
            const BatchInst &J = bi[unit_inst[u]];
            const int TS = int(J.p.table_stride);
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            const unsigned bytes = unsigned(k_hi - k_lo + 1) * unsigned(TS) * 4u;
            const unsigned slot = (gbase + unsigned(j)) % kRing;
            const unsigned bar = smem_addr(&full_bar[slot]);
            fence_proxy_async_shared();  // the slot's earlier reads (generic) before the copy
            mbar_expect_tx(bar, bytes);
            bulk_g2s(smem_addr(ring + slot * SW), J.tables + (long long)k_lo * TS, bytes, bar);
        };
        int pre = 0;  // chunks of the current unit already issued by the previous one
        for (int unit = live_from(blockIdx.x); unit < units;) {
            const int nxt = live_from(unit + gridDim.x);
            const BatchInst &I = bi[unit_inst[unit]];
            const Problem &p = I.p;
            const UnitMap um = unit_map(I, unit - I.unit_begin, PPT);
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
            if (nchunks > 0) {
                const int TS = int(p.table_stride);
                if (threadIdx.x == 0) {
                    for (int j = pre; j < kRing && j < nchunks; ++j) issue(unit, j, g);
                    // slots this unit leaves unused take the next unit's first chunks
                    if (nxt < units)
                        for (int jn = 0; jn < kRing - nchunks && jn < nchunks; ++jn) issue(nxt, jn, g + nchunks);
                }
                for (int j = 0; j < nchunks; ++j) {
                    const unsigned gj = g + unsigned(j), slot = gj % kRing;
                    ok &= mbar_wait(smem_addr(&full_bar[slot]), (gj / kRing) & 1u);
                    const int k_hi = n - 1 - j * S;
                    const int k_lo = max(0, k_hi - S + 1);
                    trace_chunk<PPT, POW2, false, 2>(ring + slot * SW, TS, k_hi, k_lo, N, Ic, xi, dwT, dwTc, shi, S0m, err);
                    __syncthreads();  // everyone is done with this slot
                    if (threadIdx.x == 0) {
                        const int jj = j + kRing;
                        if (jj < nchunks)
                            issue(unit, jj, g);
                        else if (nxt < units && jj - nchunks < nchunks)
                            issue(nxt, jj - nchunks, g + nchunks);
                    }
                }
                g += unsigned(nchunks);
                pre = nxt < units ? (nchunks < kRing ? nchunks : kRing) : 0;
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
            if (um.grp == 0) I.partial[(long long)(unit - I.unit_begin) * N + um.s] = acc;
            __syncthreads();  // comb is reused by the next unit
            unit = nxt;
        }
        if (!grid_barrier(count, target, abort, err)) break;
        // ---------------- rho of every instance ----------------
        for (long long gw = (long long)blockIdx.x * warps + warp; gw < total_nodes; gw += (long long)gridDim.x * warps)
            batch_reduce_node(bi, node_inst, gw, lane, n);
        if (!grid_barrier(count, target, abort, err)) break;
        // ---------------- field solve of every instance ----------------
        for (int b = blockIdx.x; b < solve_blocks; b += gridDim.x) {
            const BatchInst &I = bi[solve_inst[b]];
            if (n > I.Nt) continue;
            batch_solve_block<5>(I, b, n, rs, red, ered, &last);
            __syncthreads();  // rs / red / ered / last are reused by the next block
        }
        if (!grid_barrier(count, target, abort, err)) break;
    }
    if (!ok) atomicOr(err, kErrStageTimeout);
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
//           summed in shared memory as scaled integers (native integer
//           reductions; the FP32 shared-memory add is a compare-and-swap
//           loop) and flushed after each chunk into the instance's FP32
//           table adjoints of this step, which a small kernel folds into
//           the FP64 sums after the step.
// Chains go in packed pairs (f32x2).  About three forward passes of work;
// the adjoint's own recurrences are short.  A persistent grid of kAdjThreads-
// thread CTAs: CTA b handles units b, b + G, ...; its checkpoints live in
// ckpt + b * (chunks * 4 * kAdjThreads * PPT) floats.
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
    // high word: sign, exponent + (1023 - 127), top 20 mantissa bits; low word: the last 3
    const unsigned hi = (b & 0x80000000u) | (((b >> 3) & 0x0fffffffu) + ((1023u - 127u) << 20));
    return (b & 0x7f800000u) ? __hiloint2double(int(hi), int(b << 29)) : 0.0;
}

// Shared-memory integer add without a returned value, at a shared-window
// address (a native shared-memory reduction, unlike the FP32 form).
__device__ __forceinline__ void red_shared_add(unsigned addr, int v)
{
    asm volatile("red.shared.add.s32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// 2^k as a float, k in [-126, 127].
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// Fixed-point table adjoints.  In each chunk the adjoint state (Xbar, Vbar,
// and Vbar's compensation) carries a power-of-two scale 2^F, the same for
// the whole CTA, and each term vh (1, xi, xi^2) is added as the integer
// nearest to it.  Integer sums are exact and independent of order.  The
// scale comes from L = sum over the CTA's chains of |Vbar| + 8 |Xbar| at the
// chunk's start: every term of the chunk is at most |Vbar| at its substep,
// and |Vbar| moves by at most |Xbar| per substep (Xbar itself changes by
// vh g', a few per cent of vh at most), so no cell's sum exceeds L.  The
// scale puts 2 L below 2^30.  One term's rounding is 2^-F <= 2^-28 L.
// This adds a thread's share of L to *slot (a warp sum, one shared add per warp).
template <int NP>
__device__ __forceinline__ void adj_bound_add(const unsigned long long (&XB)[NP], const unsigned long long (&VB)[NP],
                                              float *slot)
{
    using namespace split;
    float l = 0.f;
#pragma unroll
    for (int pp = 0; pp < NP; ++pp) {
        float x0, x1, v0, v1;
        f2_unpack(XB[pp], x0, x1);
        f2_unpack(VB[pp], v0, v1);
        l += (fabsf(v0) + fabsf(v1)) + 8.f * (fabsf(x0) + fabsf(x1));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(slot, l);
}

// The change k of the scale exponent F that puts 2 L 2^k in [2^29, 2^30)
// (0 for L = 0 or not finite), keeping F + k in [-120, 120].
__device__ __forceinline__ int adj_rescale(float L, int F)
{
    const unsigned b = __float_as_uint(L);
    const int e = int((b >> 23) & 0xffu);
    if (e == 0 || e == 0xff || (b >> 31)) return 0;
    return max(-120 - F, min(120 - F, 28 - (e - 127)));
}

// Scales the adjoint state by 2^k.
template <int NP>
__device__ __forceinline__ void adj_scale_state(int k, unsigned long long (&XB)[NP], unsigned long long (&VB)[NP],
                                                unsigned long long (&VBC)[NP])
{
    using namespace split;
    if (k == 0) return;
    const float s = pow2f(k);
    const unsigned long long S2 = f2_pack(s, s);
#pragma unroll
    for (int pp = 0; pp < NP; ++pp) {
        XB[pp] = f2_mul(XB[pp], S2);
        VB[pp] = f2_mul(VB[pp], S2);
        VBC[pp] = f2_mul(VBC[pp], S2);
    }
}

// Substeps i = cnt-1 .. 0 of a chunk (slab k_lo + i at chunk + i TS) for PPT
// chains in packed pairs: the drift and kick of trace_chunk (split_device.cuh)
// with an unwrapped cell count U (cell J = U & mask), the chunk's kick sum in
// DC (the slab-0 kick scaled by H0 = 1/2 when the chunk starts at slab 0).
// With SAVE, substep i keeps each pair's cells (J0 | J1 << 16; N <= 256)
// and fractions for the reverse sweep.  FULL: cnt == kAdjChunk.
template <int PPT, bool FULL, bool SAVE>
__device__ __forceinline__ void adj_chunk_primal(const float *__restrict__ chunk, int TS, int N, int mask, int cnt,
                                                 unsigned long long H0, int (&U)[PPT], const int (&S0um)[PPT],
                                                 unsigned long long (&X)[PPT / 2],
                                                 const unsigned long long (&SH)[PPT / 2],
                                                 const unsigned long long (&DT)[PPT / 2],
                                                 unsigned long long (&DC)[PPT / 2], unsigned (&Jp)[kAdjChunk][PPT / 2],
                                                 unsigned long long (&Xs)[kAdjChunk][PPT / 2])
{
    using namespace split;
    constexpr int NP = PPT / 2;
    const unsigned long long MAG2 = f2_pack(kMagic, kMagic);
#pragma unroll
    for (int i = kAdjChunk - 1; i >= 0; --i) {
        if (!FULL && i >= cnt) continue;
        const float *tk = chunk + i * TS;
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
            const unsigned long long t = f2_sub(f2_sub(f2_sub(X[pp], SH[pp]), DT[pp]), DC[pp]);
            const unsigned long long mg = f2_add_rm(t, MAG2);
            float mg0, mg1;
            f2_unpack(mg, mg0, mg1);
            U[2 * pp] = U[2 * pp] - S0um[2 * pp] + __float_as_int(mg0);
            U[2 * pp + 1] = U[2 * pp + 1] - S0um[2 * pp + 1] + __float_as_int(mg1);
            const int J0 = U[2 * pp] & mask, J1 = U[2 * pp + 1] & mask;
            X[pp] = f2_sub(t, f2_sub(mg, MAG2));
            const float2 bc0 = reinterpret_cast<const float2 *>(tk)[J0];
            const float2 bc1 = reinterpret_cast<const float2 *>(tk)[J1];
            // the quadratic per chain in scalar FMAs (the packed form's
            // roundings; its operands arrive in different register pairs)
            float x0, x1;
            f2_unpack(X[pp], x0, x1);
            const unsigned long long kq = f2_pack(fmaf(x0, fmaf(x0, bc0.y, bc0.x), tk[2 * N + J0]),
                                                  fmaf(x1, fmaf(x1, bc1.y, bc1.x), tk[2 * N + J1]));
            DC[pp] = i == 0 ? f2_fma(H0, kq, DC[pp]) : f2_add(DC[pp], kq);
            if constexpr (SAVE) {
                Jp[i][pp] = unsigned(J0) | (unsigned(J1) << 16);
                Xs[i][pp] = X[pp];
            }
        }
    }
}

// The adjoint of a chunk's substeps in ascending k from the kept cells and
// fractions (slab k_lo + i still staged at chunk + i TS): per chain
//   g' = K B + 2 K C xi;  vh = Vbar h;
//   (Abar, Bbar, Cbar)[J] += rint(vh (1, xi, xi^2))  (state scaled by 2^F;
//   shared memory, cell-interleaved: 3 integers per cell from accb, one
//   slab every 3N)
//   Xbar += vh g';  Vbar -= Xbar  (compensated: VBC holds the lost low part)
template <int PPT, bool FULL>
__device__ __forceinline__ void adj_chunk_reverse(const float *__restrict__ chunk, int TS, int N, unsigned accb,
                                                  int cnt, unsigned long long H0,
                                                  const unsigned (&Jp)[kAdjChunk][PPT / 2],
                                                  const unsigned long long (&Xs)[kAdjChunk][PPT / 2],
                                                  unsigned long long (&XB)[PPT / 2], unsigned long long (&VB)[PPT / 2],
                                                  unsigned long long (&VBC)[PPT / 2])
{
    using namespace split;
    constexpr int NP = PPT / 2;
    const int T3 = 3 * N;
#pragma unroll
    for (int i = 0; i < kAdjChunk; ++i) {
        if (!FULL && i >= cnt) continue;
        const float *tk = chunk + i * TS;
        const unsigned base = accb + unsigned(i * T3) * 4u;
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
            const int J0 = int(Jp[i][pp] & 0xffffu), J1 = int(Jp[i][pp] >> 16);
            const unsigned long long x = Xs[i][pp];
            // g' = K B + 2 K C xi from one float2 per chain
            const float2 bc0 = reinterpret_cast<const float2 *>(tk)[J0];
            const float2 bc1 = reinterpret_cast<const float2 *>(tk)[J1];
            float xa, xb;
            f2_unpack(x, xa, xb);
            const unsigned long long gp = f2_pack(fmaf(xa + xa, bc0.y, bc0.x), fmaf(xb + xb, bc1.y, bc1.x));
            const unsigned long long vh = i == 0 ? f2_mul(VB[pp], H0) : VB[pp];
            const unsigned long long vx = f2_mul(vh, x);
            const unsigned long long vxx = f2_mul(vx, x);
            float h0, h1, x0, x1, xx0, xx1;
            f2_unpack(vh, h0, h1);
            f2_unpack(vx, x0, x1);
            f2_unpack(vxx, xx0, xx1);
            const unsigned a0 = base + unsigned(J0) * 12u, a1 = base + unsigned(J1) * 12u;
            red_shared_add(a0, __float2int_rn(h0));
            red_shared_add(a0 + 4u, __float2int_rn(x0));
            red_shared_add(a0 + 8u, __float2int_rn(xx0));
            red_shared_add(a1, __float2int_rn(h1));
            red_shared_add(a1 + 4u, __float2int_rn(x1));
            red_shared_add(a1 + 8u, __float2int_rn(xx1));
            XB[pp] = f2_fma(vh, gp, XB[pp]);
            const unsigned long long z = f2_add(XB[pp], VBC[pp]);
            const unsigned long long tt = f2_sub(VB[pp], z);
            VBC[pp] = f2_add(f2_sub(tt, VB[pp]), z);
            VB[pp] = tt;
        }
    }
}

// Adds a chunk's fixed-point table adjoints (n integers in shared memory,
// units of 2^-F) into the instance's FP32 staging buffer of this step (four
// at a time) and zeroes them; groups of four still zero are skipped.  A sum
// at or beyond 2^30 in magnitude raises kErrAdjointRange.
__device__ __forceinline__ bool adj_flush(int *__restrict__ a, float *__restrict__ dst, int n, int F)
{
    const float u = pow2f(-F);
    auto in_range = [](int v) { return unsigned(v + (1 << 30)) < (1u << 31); };
    bool ok = true;
    const int n4 = n & ~3;
    for (int e = 4 * int(threadIdx.x); e < n4; e += 4 * int(blockDim.x)) {
        const int4 v = *reinterpret_cast<const int4 *>(a + e);
        if ((v.x | v.y | v.z | v.w) != 0) {
            ok &= in_range(v.x) & in_range(v.y) & in_range(v.z) & in_range(v.w);
            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + e), "f"(float(v.x) * u),
                         "f"(float(v.y) * u), "f"(float(v.z) * u), "f"(float(v.w) * u)
                         : "memory");
            *reinterpret_cast<int4 *>(a + e) = make_int4(0, 0, 0, 0);
        }
    }
    for (int e = n4 + int(threadIdx.x); e < n; e += int(blockDim.x)) {
        const int v = a[e];
        if (v != 0) {
            ok &= in_range(v);
            atomicAdd(dst + e, float(v) * u);
            a[e] = 0;
        }
    }
    return ok;
}

// muT[k] += muS[k], muS[k] = 0 for the slabs k < m of every instance (one
// step's table adjoints into the FP64 sums): block (x, instance).
__global__ void batch_adjoint_fold_kernel(const BatchInst *__restrict__ bi, int m)
{
    const BatchInst &I = bi[blockIdx.y];
    if (m > I.Nt) return;
    const long long n = (long long)m * 3 * I.p.N[0];  // a multiple of 4 when N is
    float4 *s4 = reinterpret_cast<float4 *>(I.muS);
    const long long n4 = n >> 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n4; e += (long long)gridDim.x * blockDim.x) {
        const float4 v = s4[e];
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
            double *d = I.muT + 4 * e;
            d[0] += double(v.x);
            d[1] += double(v.y);
            d[2] += double(v.z);
            d[3] += double(v.w);
            s4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    for (long long e = 4 * n4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const float v = I.muS[e];
        if (v != 0.f) {
            I.muT[e] += double(v);
            I.muS[e] = 0.f;
        }
    }
}

template <int PPT>
__global__ void __launch_bounds__(kAdjThreads, 2) batch_adjoint_split_kernel(const BatchInst *__restrict__ bi,
                                                                     const int *__restrict__ unit_inst, int units,
                                                                     int m, int ts_max, int max_chunks,
                                                                     float *__restrict__ ckpt,
                                                                     double *__restrict__ theta_acc, long long slots,
                                                                     unsigned *err)
{
    using namespace split;
    static_assert(PPT % 2 == 0, "chains go in packed pairs");
    constexpr int SC = kAdjChunk, NP = PPT / 2, R = kAdjRing;
    // [R][SC][ts_max] table slabs, then two [SC][N][3] fixed-point table-
    // adjoint buffers (2 SC ts_max integers; 3N <= ts_max), zero between flushes
    extern __shared__ __align__(128) float ring[];
    __shared__ __align__(8) unsigned long long full_bar[R];
    __shared__ float lsum[3];  // scale bounds of chunks c, c + 1, c + 2 (slot c % 3)
    int *acc0 = reinterpret_cast<int *>(ring + size_t(R) * SC * ts_max);
    for (int e = threadIdx.x; e < 2 * SC * ts_max; e += blockDim.x) acc0[e] = 0;
    if (threadIdx.x < 3) lsum[threadIdx.x] = 0.f;
    if (threadIdx.x == 0) {
        for (int r = 0; r < R; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int t = threadIdx.x;
    // checkpoint area of this CTA: [chunk][field][pair][kAdjThreads] packed pairs,
    // written and read once per step with the streaming (evict-first) cache
    // policy so that they pass through L2 without displacing the tables
    unsigned long long *ck =
        reinterpret_cast<unsigned long long *>(ckpt) + (size_t)blockIdx.x * max_chunks * 2 * kAdjThreads * PPT;
    unsigned g = 0;  // chunks consumed by this CTA: slot g % R, parity (g / R) & 1
    bool ok = true, in_range = true;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const BatchInst &I = bi[unit_inst[unit]];
        if (m > I.Nt) continue;
        const Problem &p = I.p;
        // thread t: node s = t % N, velocity chains (unit tpn' + t / N) PPT + q, tpn' = kAdjThreads / N
        UnitMap um;
        um.N = p.N[0];
        um.s = t % um.N;
        um.m0 = ((long long)(unit - I.adj_unit_begin) * (kAdjThreads / um.N) + t / um.N) * PPT;
        const int N = um.N, mask = N - 1, TS = int(p.table_stride), T3 = 3 * N;
        const unsigned slab_bytes = unsigned(TS) * 4u;
        const int C = (m + SC - 1) / SC;  // chunks of this step; chunk c = slabs [c SC, min(m, c SC + SC) - 1]
        auto issue = [&](int c, unsigned gg) {
            const int k_lo = c * SC, k_hi = min(m - 1, k_lo + SC - 1);
            const unsigned bytes = unsigned(k_hi - k_lo + 1) * slab_bytes;
            const unsigned bar = smem_addr(&full_bar[gg % R]);
            mbar_expect_tx(bar, bytes);
            bulk_g2s(smem_addr(ring + (gg % R) * SC * ts_max), I.tables + (long long)k_lo * TS, bytes, bar);
        };
        auto ckp = [&](int c, int field, int pp) -> unsigned long long * {
            return ck + ((size_t(c) * 4 + field) * NP + pp) * kAdjThreads + t;
        };
        // chains past the last velocity node trace node Nm-1 with a zero seed
        int U[PPT], S0um[PPT];
        float dwTc[PPT];
        bool live[PPT];
        unsigned long long X[NP], SH[NP], DT[NP];
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
            float sh[2], sl[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = 2 * pp + h;
                const long long mm = um.m0 + q;
                live[q] = mm < p.Nm;
                const SplitNode nd = I.nodes[live[q] ? mm : p.Nm - 1];
                S0um[q] = nd.S0u + kMagicBits;
                U[q] = um.s;
                dwTc[q] = 0.f;
                sh[h] = nd.sig_hi;
                sl[h] = nd.sig_lo;
            }
            X[pp] = 0ull;
            SH[pp] = f2_pack(sh[0], sh[1]);
            DT[pp] = f2_pack(sl[0], sl[1]);
        }
        unsigned Jp[SC][NP];
        unsigned long long Xs[SC][NP], DC[NP];
        const unsigned long long ONE2 = f2_pack(1.0f, 1.0f), HALF2 = f2_pack(0.5f, 0.5f);
        auto fold = [&]() {
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) {
                float d0, d1, c0, c1;
                f2_unpack(DT[pp], d0, d1);
                f2_unpack(DC[pp], c0, c1);
                kick(d0, dwTc[2 * pp], c0);
                kick(d1, dwTc[2 * pp + 1], c1);
                DT[pp] = f2_pack(d0, d1);
            }
        };
        // ---- pass 1: chunks C-1 .. 0 (descending k), checkpoint each entry state
        if (threadIdx.x == 0)
            for (int j = 0; j < R && j < C; ++j) issue(C - 1 - j, g + j);
        for (int j = 0; j < C; ++j, ++g) {
            const int c = C - 1 - j;
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) {
                __stcs(ckp(c, 0, pp), f2_pack(__int_as_float(U[2 * pp]), __int_as_float(U[2 * pp + 1])));
                __stcs(ckp(c, 1, pp), X[pp]);
                __stcs(ckp(c, 2, pp), DT[pp]);
                __stcs(ckp(c, 3, pp), f2_pack(dwTc[2 * pp], dwTc[2 * pp + 1]));
            }
            ok &= mbar_wait(smem_addr(&full_bar[g % R]), (g / R) & 1u);
            const float *chunk = ring + (g % R) * SC * ts_max;
            const int cnt = min(SC, m - c * SC);
            const unsigned long long H0 = c == 0 ? HALF2 : ONE2;
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) DC[pp] = 0ull;
            if (cnt == SC)
                adj_chunk_primal<PPT, true, false>(chunk, TS, N, mask, cnt, H0, U, S0um, X, SH, DT, DC, Jp, Xs);
            else
                adj_chunk_primal<PPT, false, false>(chunk, TS, N, mask, cnt, H0, U, S0um, X, SH, DT, DC, Jp, Xs);
            fold();
            __syncthreads();
            if (threadIdx.x == 0 && j + R < C) issue(C - 1 - (j + R), g + R);
        }
        // ---- seed at the foot
        const float dx = float(p.dx[0]), dxdt = float(p.dx[0] / p.dt);
        const float a = float(-p.wv * I.lambda[um.s]);
        unsigned long long XB[NP], VB[NP], VBC[NP];
        double th[4] = {0, 0, 0, 0};
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
            float xi2[2], dw2[2], xb2[2], vb2[2];
            f2_unpack(X[pp], xi2[0], xi2[1]);
            f2_unpack(DT[pp], dw2[0], dw2[1]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int q = 2 * pp + h;
                const long long mm = live[q] ? um.m0 + q : p.Nm - 1;
                const SplitNode &nd = I.nodes[mm];
                const float aq = live[q] ? a : 0.f;
                const float x = float(p.xmin[0]) + (float(U[q]) + xi2[h]) * dx;
                const float u = nd.u0f + ((dw2[h] - dwTc[q]) - nd.sig_lo) * dxdt;
                const F0GradF gr = f0_grad_1d_f(p, x, u);
                xb2[h] = aq * dx * gr.fx;
                vb2[h] = aq * dxdt * gr.fu;
#pragma unroll
                for (int i = 0; i < 4; ++i) th[i] += double(aq) * double(gr.dth[i]);
            }
            XB[pp] = f2_pack(xb2[0], xb2[1]);
            VB[pp] = f2_pack(vb2[0], vb2[1]);
            VBC[pp] = 0ull;
        }
        // ---- pass 2: chunks 0 .. C-1 (ascending k); table adjoints of chunk c
        // in buffer c & 1, flushed while the next chunk runs
        if (threadIdx.x == 0)
            for (int j = 0; j < R && j < C; ++j) issue(j, g + j);
        int F = 0;  // the adjoint state's scale exponent in the current chunk
        if (C > 0) {
            adj_bound_add(XB, VB, &lsum[0]);
            __syncthreads();
            F = adj_rescale(lsum[0], 0);
            adj_scale_state(F, XB, VB, VBC);
        }
        auto load_ckpt = [&](int c) {
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) {
                float u0, u1, c0, c1;
                f2_unpack(__ldcs(ckp(c, 0, pp)), u0, u1);
                U[2 * pp] = __float_as_int(u0);
                U[2 * pp + 1] = __float_as_int(u1);
                X[pp] = __ldcs(ckp(c, 1, pp));
                DT[pp] = __ldcs(ckp(c, 2, pp));
                f2_unpack(__ldcs(ckp(c, 3, pp)), c0, c1);
                dwTc[2 * pp] = c0;
                dwTc[2 * pp + 1] = c1;
            }
        };
        if (C > 0) load_ckpt(0);
        for (int c = 0; c < C; ++c, ++g) {
            ok &= mbar_wait(smem_addr(&full_bar[g % R]), (g / R) & 1u);
            const float *chunk = ring + (g % R) * SC * ts_max;
            const int cnt = min(SC, m - c * SC);
            const unsigned long long H0 = c == 0 ? HALF2 : ONE2;
            int *acc = acc0 + (c & 1) * SC * T3;
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) DC[pp] = 0ull;
            if (cnt == SC) {
                adj_chunk_primal<PPT, true, true>(chunk, TS, N, mask, cnt, H0, U, S0um, X, SH, DT, DC, Jp, Xs);
                if (c + 1 < C) load_ckpt(c + 1);
                adj_chunk_reverse<PPT, true>(chunk, TS, N, smem_addr(acc), cnt, H0, Jp, Xs, XB, VB, VBC);
            } else {
                adj_chunk_primal<PPT, false, true>(chunk, TS, N, mask, cnt, H0, U, S0um, X, SH, DT, DC, Jp, Xs);
                if (c + 1 < C) load_ckpt(c + 1);
                adj_chunk_reverse<PPT, false>(chunk, TS, N, smem_addr(acc), cnt, H0, Jp, Xs, XB, VB, VBC);
            }
            if (c + 1 < C) adj_bound_add(XB, VB, &lsum[(c + 1) % 3]);
            __syncthreads();
            if (threadIdx.x == 0) {
                if (c + R < C) issue(c + R, g + R);
                lsum[c % 3] = 0.f;
            }
            in_range &= adj_flush(acc, I.muS + (long long)c * SC * T3, cnt * T3, F);
            if (c + 1 < C) {
                const int k = adj_rescale(lsum[(c + 1) % 3], F);
                adj_scale_state(k, XB, VB, VBC);
                F += k;
            }
        }
        adj::block_theta_add(th, theta_acc, slots, unit);
        __syncthreads();
    }
    if (!ok) atomicOr(err, kErrStageTimeout);
    if (!in_range) atomicOr(err, kErrAdjointRange);
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
            const double A = t[3 * i], B = t[3 * i + 1], C = t[3 * i + 2];
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
    return size_t(kAdjRing + 2) * kAdjChunk * L.ts_max * sizeof(float);
}

int adjoint_split_ctas_per_sm(const BatchLaunch &L, int ppt)
{
    int nb = 0;
    void (*fs)(const BatchInst *, const int *, int, int, int, int, float *, double *, long long, unsigned *) =
        ppt == 2 ? batch_adjoint_split_kernel<2> : batch_adjoint_split_kernel<4>;
    const size_t smem = adjoint_split_smem(L);
    if (cudaFuncSetAttribute(fs, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fs, kAdjThreads, smem) != cudaSuccess) return 0;
    return nb;
}

namespace {

using BatchRunFn = void (*)(const BatchInst *, const int *, int, const int *, long long, const int *, int, int, int,
                            int, int, unsigned *, unsigned *);

template <int PPT>
BatchRunFn batch_run_fn(bool pow2)
{
    return pow2 ? batch_run_split_kernel<PPT, true> : batch_run_split_kernel<PPT, false>;
}

BatchRunFn batch_run_pick(const BatchLaunch &L)
{
    switch (L.ppt) {
    case 1: return batch_run_fn<1>(L.pow2);
    case 2: return batch_run_fn<2>(L.pow2);
    case 4: return batch_run_fn<4>(L.pow2);
    case 8: return batch_run_fn<8>(L.pow2);
    default: return nullptr;
    }
}

}  // namespace

// Co-resident CTAs of the whole-forward kernel for L's shape on a device
// with `sms` multiprocessors (0 if it cannot run).
int batch_run_ctas(const BatchLaunch &L, int sms)
{
    const BatchRunFn fn = batch_run_pick(L);
    if (!fn || L.precision != NUFI_PREC_FP32_SPLIT) return 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.smem)) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 256, L.smem) != cudaSuccess) return 0;
    return std::min(L.units, nb * sms);
}

cudaError_t launch_batch_run(const BatchLaunch &L, int ctas, int n0, int n1, unsigned *sync, cudaStream_t st)
{
    const BatchRunFn fn = batch_run_pick(L);
    if (!fn || ctas < 1) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.smem));
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(sync, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(ctas));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fn, L.inst, L.unit_inst, L.units, L.node_inst, L.total_nodes, L.solve_inst,
                              L.solve_blocks, n0, n1, L.slabs_per_chunk, L.ts_max, sync, L.err);
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
        case 2: fs = batch_adjoint_split_kernel<2>; break;
        case 4: fs = batch_adjoint_split_kernel<4>; break;
        default: return cudaErrorInvalidValue;
        }
        const size_t smem = adjoint_split_smem(L);
        cudaError_t e = cudaFuncSetAttribute(fs, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        fs<<<L.adj_grid, kAdjThreads, smem, st>>>(L.inst, L.adj_unit_inst, L.adj_units, m, L.ts_max, L.max_chunks,
                                                 L.ckpt, L.theta_acc, L.adj_units, L.err);
        if (m > 0) batch_adjoint_fold_kernel<<<dim3(unsigned(std::max(1, L.max_chunks * kAdjChunk * 3 * L.max_N / 4096)),
                                                    unsigned(L.count)),
                                               256, 0, st>>>(L.inst, m);
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
