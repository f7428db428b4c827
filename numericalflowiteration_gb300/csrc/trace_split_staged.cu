// trace_split_staged.cu — FP32-split 1D trace with the field tables staged
// into shared memory by TMA bulk copies.
//
// Why: every SM needs every slab of the history (each point visits all n
// slabs), so with plain global loads nearly every warp's table load of a
// substep pays an L2 round trip (compulsory L1 misses, the long-scoreboard
// stall of the first form).  Here each CTA streams the history through a
// ring of R shared-memory slots, S slabs per slot: one elected thread
// issues cp.async.bulk (global -> shared, completion counted on an
// mbarrier) R chunks ahead, so the loads on the critical path of a substep
// are 16-byte shared-memory reads of a table already on chip.
//
// Geometry: a persistent grid of about one CTA per SM.  Each thread owns
// one spatial node (x-lanes, so the 32 lanes of a warp read neighbouring
// cells: few bank conflicts) and PPT velocity nodes, i.e. PPT
// independent dependency chains.  CTA c owns the velocity nodes c, c + G,
// c + 2G, ... (interleaved, so that each CTA holds a spread of velocities).
// rho: per thread over its chains (FP64), then either into partial[c][s]
// (reduce_rho sums the G rows) or, with a RhoFix, added as a 64-bit
// fixed-point integer (scale 2^F) into fx.sum[s]; the last CTA to finish
// (a ticket) turns the sums into rho and clears them.  The integer sums are
// exact and order-free, so rho is deterministic, and bit for bit that of
// the whole-run kernel (run_split_1d.cu), which sums the same parts alike.
//
// The per-point arithmetic is that of trace_split.cu (same substep order as
// the reference's eval_ftilda, nufi/rho.hpp:31-61).
//
// Every wait on an mbarrier is bounded (kWaitLimit polls); on timeout the
// kernel raises kErrStageTimeout and carries on (no trap, no hang).
#include <algorithm>
#include <cstdlib>

#include "split_device.cuh"

namespace nufi_gb300 {

using namespace split;

template <int PPT, bool POW2, bool UNWRAP>
__global__ void __launch_bounds__(512, 1) trace_split_1d_staged_kernel(const Problem p, const float *__restrict__ tables,
                                                                     const SplitNode *__restrict__ nodes,
                                                                     const float2 *__restrict__ phase, int n,
                                                                     long long q_begin, long long q_end, int S,
                                                                     int Nr, double *__restrict__ partial,
                                                                     const RhoFix fx, const PendingSlab pend,
                                                                     unsigned *err)
{
    extern __shared__ __align__(128) float ring[];
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    __shared__ double combine[256];
    __shared__ bool last;

    const int N = p.N[0];
    const int s = threadIdx.x % Nr;    // spatial node
    const int grp = threadIdx.x / Nr;  // chain group (threads per node > 1)
    const int G = gridDim.x;
    // velocity nodes interleaved over the CTAs: chain j of CTA c is c + j G
    long long mv[PPT];
    int I[PPT], S0m[PPT], Wr[PPT];
    float xi[PPT], dwT[PPT], dwTc[PPT], shi[PPT], slo[PPT];
    bool live[PPT];
    const int log2n = __ffs(N) - 1;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        Wr[q] = 0;
        const long long m = blockIdx.x + (long long)(grp * PPT + q) * G;
        const long long qq = (long long)s * p.Nm + m;
        live[q] = (s < N) && (m < p.Nm) && (qq >= q_begin) && (qq < q_end);
        mv[q] = m < p.Nm ? m : blockIdx.x;
        const SplitNode nd = nodes[mv[q]];
        S0m[q] = nd.S0 + kMagicBits;
        shi[q] = nd.sig_hi;
        slo[q] = nd.sig_lo;
        I[q] = s < N ? s : 0;
        xi[q] = 0.0f;
        dwT[q] = slo[q];
        dwTc[q] = 0.0f;
    }

    if (n > 0) {
        const int TS = int(p.table_stride);       // floats per slab
        const int nchunks = (n + S - 1) / S;
        const unsigned slab_bytes = unsigned(p.table_stride) * 4u;
        if (threadIdx.x == 0) {
            for (int r = 0; r < kRing; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
            mbar_fence_init();
        }
        __syncthreads();
        // chunk j holds slabs k in [k_lo, k_hi], k_hi = n-1-j*S; with a
        // pending newest slab (n - 1), chunk 0 copies only [k_lo, n-2] and
        // the CTA derives slab n - 1's table in place
        const bool fuse = pend.k >= 0 && pend.k == n - 1;
        auto issue = [&](int j) {
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            const int k_top = (fuse && j == 0) ? k_hi - 1 : k_hi;
            const unsigned bytes = unsigned(k_top - k_lo + 1) * slab_bytes;
            const unsigned bar = smem_addr(&full_bar[j % kRing]);
            mbar_expect_tx(bar, bytes);  // 0 bytes: the arrival alone completes the phase
            if (bytes > 0)
                bulk_g2s(smem_addr(ring + (j % kRing) * S * TS), tables + (long long)k_lo * p.table_stride, bytes,
                         bar);
        };
        if (threadIdx.x == 0)
            for (int j = 0; j < kRing && j < nchunks; ++j) issue(j);
        if (fuse) {
            // the table of slab n - 1 from its FP64 coefficients (mapped host
            // memory), as derive_table_kernel computes it
            float *newest = ring + (n - 1 - max(0, n - S)) * TS;  // chunk 0, slot 0
            const double K = -p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                const double c0 = pend.stage[i], c1 = pend.stage[i + 1], c2 = pend.stage[i + 2],
                             c3 = pend.stage[i + 3];
                cubic_kick_poly(c0, c1, c2, c3, K, newest, N, i);
                if (blockIdx.x == 0) cubic_kick_poly(c0, c1, c2, c3, K, pend.table_out, N, i);
            }
            if (blockIdx.x == 0)
                for (long long i = threadIdx.x; i < p.stride_t; i += blockDim.x) pend.hist_out[i] = pend.stage[i];
            __syncthreads();
        }
        bool ok = true;
        for (int j = 0; j < nchunks; ++j) {
            const int slot = j % kRing;
            ok &= mbar_wait(smem_addr(&full_bar[slot]), unsigned((j / kRing) & 1));
            const float *__restrict__ chunk = ring + slot * S * TS;
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            trace_chunk<PPT, POW2, UNWRAP>(chunk, TS, k_hi, k_lo, N, I, xi, dwT, dwTc, shi, S0m, err, &Wr, log2n);
            // everyone is done with this slot.  A CTA barrier here, not the
            // whole-run kernel's per-slot release counts: one launch per step
            // (the drop-in loop) measured 2.5 ms faster over the two-stream run
            // this way, and one substep per loop trip faster than two
            __syncthreads();
            if (threadIdx.x == 0 && j + kRing < nchunks) {
                if (fuse && j == 0) fence_proxy_async_shared();  // the derived table's stores before the copy's
                issue(j + kRing);
            }
        }
        if (!ok) atomicOr(err, kErrStageTimeout);
    }

    const F0 f = make_f0(p);
    // f~ summed as the whole-run kernel sums it (two_sum_acc): the same bits
    double gsum = 0;
    float ds = 0.f, dc = 0.f;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        const SplitNode nd = nodes[mv[q]];
        gsum += nd.g;
        float2 cs = __ldg(phase + I[q]);
        if constexpr (UNWRAP) cs = phase_unwrapped(cs, Wr[q] - n * ((nd.S0u - nd.S0) / N), p.phase_wrap[0]);
        two_sum_acc(ds, dc, delta_f0(f, nd, cs, xi[q], (dwT[q] - dwTc[q]) - slo[q]));
    }
    double acc = gsum + (double(ds) + double(dc));
    // groups of the same node combined in group order
    if (blockDim.x > unsigned(Nr)) {
        if (grp == 1) combine[s] = acc;
        __syncthreads();
        if (grp == 0) acc += combine[s];
    }
    if (!fx.sum) {
        if (grp == 0 && s < N) partial[(long long)blockIdx.x * N + s] = acc;
        return;
    }
    if (grp == 0 && s < N) {
        const double v = acc * fx.scale;
        if (!(fabs(v) < fx.limit)) atomicOr(err, kErrRhoRange);  // outside the host's bound: not expected
        red_global_add_u64(fx.sum + s, (unsigned long long)__double2ll_rn(fmin(fmax(v, -fx.limit), fx.limit)));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(fx.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the error word as the trace leaves it (every CTA's atomics are
    // performed in L2 before its ticket), loaded beside the sums
    const unsigned ew = (fx.err_pub && threadIdx.x == 0) ? __ldcg(err) : 0u;
    const double to_rho = -p.wv / fx.scale;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double r = double((long long)__ldcg(fx.sum + j)) * to_rho;
        fx.rho[j] = r;
        if (fx.pub) fx.pub[j] = r;
        fx.sum[j] = 0ull;
    }
    if (threadIdx.x == 0) {
        *fx.ticket = 0u;
        if (fx.err_pub) *fx.err_pub = ew;
    }
    if (fx.seq_pub) {  // every thread's rho and the word, a system fence each, then seq
        __threadfence_system();
        __syncthreads();
        if (threadIdx.x == 0) *reinterpret_cast<volatile unsigned *>(fx.seq_pub) = fx.seq;
    }
}

namespace {

template <int PPT, bool POW2, bool UNWRAP>
cudaError_t launch_staged_form(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                               const float2 *phase, int n, long long qb, long long qe, double *partial,
                               const RhoFix &fx, const PendingSlab &pend, unsigned *err, cudaStream_t st)
{
    static const cudaError_t attr = cudaFuncSetAttribute(trace_split_1d_staged_kernel<PPT, POW2, UNWRAP>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (attr != cudaSuccess) return attr;
    trace_split_1d_staged_kernel<PPT, POW2, UNWRAP><<<dim3(sh.ctas), dim3(sh.threads), sh.smem, st>>>(
        p, tables, nodes, phase, n, qb, qe, sh.slabs_per_chunk, sh.threads / sh.tpn, partial, fx, pend, err);
    return cudaGetLastError();
}

template <int PPT>
cudaError_t launch_staged_ppt(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                              const float2 *phase, int n, long long qb, long long qe, double *partial,
                              const RhoFix &fx, const PendingSlab &pend, unsigned *err, cudaStream_t st)
{
    const bool pow2 = (p.N[0] & (p.N[0] - 1)) == 0;
    if (phase_wraps(p)) {  // f0's phase at the unwrapped foot (admitted for N a power of two only)
        if (!pow2) return cudaErrorInvalidValue;
        return launch_staged_form<PPT, true, true>(p, sh, tables, nodes, phase, n, qb, qe, partial, fx, pend, err,
                                                   st);
    }
    if (pow2)
        return launch_staged_form<PPT, true, false>(p, sh, tables, nodes, phase, n, qb, qe, partial, fx, pend, err,
                                                    st);
    return launch_staged_form<PPT, false, false>(p, sh, tables, nodes, phase, n, qb, qe, partial, fx, pend, err, st);
}

}  // namespace

StagedShape staged_shape_1d(const Problem &p, int sms, int cps, int tpn_opt)
{
    StagedShape sh;
    if (p.dim != 1 || p.N[0] > 256) return sh;  // not applicable (one thread per spatial node)
    const long long Nm = p.Nm;
    // CTAs per SM (cps): 1 by default; 2 runs two smaller CTAs per SM (more
    // warps, fewer chains each)
    cps = cps == 2 ? 2 : 1;
    int G = int(std::min<long long>(Nm, (long long)sms * cps));
    int ppt = int((Nm + G - 1) / G);
    if (ppt > kStagedMaxPPT) {
        G = int((Nm + kStagedMaxPPT - 1) / kStagedMaxPPT);
        ppt = int((Nm + G - 1) / G);
    }
    // One CTA per SM: the persistent grid must not double up on an SM (an
    // SM holding two CTAs takes twice as long and sets the kernel's time),
    // so each CTA asks for more than half of an SM's shared memory and uses
    // it for a deeper ring.
    const size_t slab_bytes = size_t(p.table_stride) * 4;
    const size_t kOneCtaPerSm = cps == 2 ? 72 * 1024 : 120 * 1024;
    int S = int(std::max<size_t>(1, std::min<size_t>(32, kOneCtaPerSm / (size_t(kRing) * slab_bytes))));
    if (size_t(kRing) * S * slab_bytes > 200 * 1024) return sh;
    // Threads per spatial node: 1 by default (measured faster on the
    // two-stream workload: the loop is bound by shared-memory bandwidth,
    // which more warps do not add); tpn_opt = 2 splits the chains over two
    // threads per node.
    const int Nr = (p.N[0] + 31) / 32 * 32;
    const int tpn = (tpn_opt == 2 && ppt >= 2 && 2 * Nr <= 512) ? 2 : 1;
    sh.ctas = G;
    sh.tpn = tpn;
    sh.ppt = (ppt + tpn - 1) / tpn;
    sh.threads = tpn * Nr;
    sh.slabs_per_chunk = S;
    sh.smem = cps == 2 ? size_t(kRing) * S * slab_bytes : std::max(size_t(kRing) * S * slab_bytes, kOneCtaPerSm);
    sh.ok = true;
    return sh;
}

cudaError_t launch_trace_split_staged(const Problem &p, const StagedShape &sh, const float *tables,
                                      const SplitNode *nodes, const float2 *phase, int n, long long qb, long long qe,
                                      double *partial, int *rows, unsigned *err, cudaStream_t st, const RhoFix &fx,
                                      const PendingSlab &pend)
{
    *rows = fx.sum ? 0 : sh.ctas;  // no rows to reduce: the kernel writes rho itself
    if (pend.k >= 0 && (pend.k != n - 1 || size_t(p.table_stride) * 4 * size_t(sh.slabs_per_chunk) == 0))
        return cudaErrorInvalidValue;  // a pending slab is only the trace's newest
    switch (sh.ppt) {
#define NUFI_CASE(K) \
    case K: return launch_staged_ppt<K>(p, sh, tables, nodes, phase, n, qb, qe, partial, fx, pend, err, st);
        NUFI_CASE(1) NUFI_CASE(2) NUFI_CASE(3) NUFI_CASE(4) NUFI_CASE(5) NUFI_CASE(6) NUFI_CASE(7) NUFI_CASE(8)
#undef NUFI_CASE
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace nufi_gb300
