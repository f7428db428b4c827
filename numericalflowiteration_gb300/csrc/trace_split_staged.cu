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
// cells: conflict-free float4 reads) and PPT velocity nodes, i.e. PPT
// independent dependency chains.  CTA c owns velocity nodes
// [c*Nm/G, (c+1)*Nm/G).  rho: per thread over its chains (FP64) into
// partial[c][s]; reduce_rho sums the G rows.
//
// The per-point arithmetic is that of trace_split.cu (same substep order as
// the reference's eval_ftilda, nufi/rho.hpp:31-61).
//
// Every wait on an mbarrier is bounded (kWaitLimit polls); on timeout the
// kernel raises kErrStageTimeout and carries on (no trap, no hang).
#include <algorithm>

#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr int kRing = 3;
constexpr unsigned kWaitLimit = 1u << 22;

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    for (unsigned it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

template <bool POW2>
__device__ __forceinline__ void drift_split(int &I, float &xi, float dw, float dwc, float shi, float slo, int S0,
                                            int N, unsigned *err)
{
    const float t = (xi - shi) - ((slo - dwc) + dw);
    const float mg = __fadd_rd(t, kMagic);
    const int fi = __float_as_int(mg) - kMagicBits;
    xi = t - (mg - kMagic);
    int J = I - S0 + fi;
    if constexpr (POW2) {
        J &= N - 1;
    } else {
        J += (J < 0) ? N : 0;
        J -= (J >= N) ? N : 0;
        if ((unsigned)J >= (unsigned)N) {
            atomicOr(err, kErrKickRange);
            J = ((J % N) + N) % N;
        }
    }
    I = J;
}

__device__ __forceinline__ void kick_comp(float &dw, float &dwc, float k)
{
    const float y = k - dwc;
    const float t = dw + y;
    dwc = (t - dw) - y;
    dw = t;
}

__device__ __forceinline__ float delta_f0(int kind, float alpha, float kdx, float dx_dt, float ub, float inv_s2,
                                          const SplitNode &nd, float2 cs, float xi, float dw)
{
    float sp, cp;
    sincosf(kdx * xi, &sp, &cp);
    const float c = cs.x * cp - cs.y * sp;
    const float du = dw * dx_dt;
    if (kind == NUFI_F0_LANDAU) {
        const float em = expm1f(-(du * (nd.u0f + 0.5f * du)));
        return nd.ga * (em + alpha * c * (1.0f + em));
    }
    if (kind == NUFI_F0_TWO_STREAM) {
        const float u = nd.u0f + du;
        const float em = expm1f(-(du * (nd.u0f + 0.5f * du)));
        const float diff = nd.ga * (u * u * em + du * (2.0f * nd.u0f + du));
        return diff + alpha * c * (nd.ga * u * u * (1.0f + em));
    }
    const float em1 = expm1f(-(du * (nd.u0f + 0.5f * du)));
    const float em2 = expm1f(-(du * ((nd.u0f - ub) + 0.5f * du)) * inv_s2);
    return nd.ga * em1 + nd.gb * em2 + alpha * c * (nd.ga * (1.0f + em1) + nd.gb * (1.0f + em2));
}

}  // namespace

template <int PPT, bool POW2>
__global__ void __launch_bounds__(256, 1) trace_split_1d_staged_kernel(const Problem p, const float *__restrict__ tables,
                                                                     const SplitNode *__restrict__ nodes,
                                                                     const float2 *__restrict__ phase, int n,
                                                                     long long q_begin, long long q_end, int S,
                                                                     double *__restrict__ partial, unsigned *err)
{
    extern __shared__ __align__(128) float4 ring[];
    __shared__ __align__(8) unsigned long long full_bar[kRing];

    const int N = p.N[0];
    const int s = threadIdx.x;  // spatial node
    const int G = gridDim.x;
    const long long m0 = (long long)blockIdx.x * p.Nm / G;
    const long long m1 = (long long)(blockIdx.x + 1) * p.Nm / G;

    int I[PPT], S0[PPT];
    float xi[PPT], dw[PPT], dwc[PPT], shi[PPT], slo[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = m0 + q;
        const long long qq = (long long)s * p.Nm + m;
        live[q] = (s < N) && (m < m1) && (qq >= q_begin) && (qq < q_end);
        const SplitNode nd = nodes[m < m1 ? m : m0];
        S0[q] = nd.S0;
        shi[q] = nd.sig_hi;
        slo[q] = nd.sig_lo;
        I[q] = s < N ? s : 0;
        xi[q] = 0.0f;
        dw[q] = 0.0f;
        dwc[q] = 0.0f;
    }

    if (n > 0) {
        const int slab_f4 = N;                    // float4 per slab
        const int nchunks = (n + S - 1) / S;
        const unsigned slab_bytes = unsigned(p.table_stride) * 4u;
        if (threadIdx.x == 0) {
            for (int r = 0; r < kRing; ++r) mbar_init(smem_addr(&full_bar[r]), 1);
            mbar_fence_init();
        }
        __syncthreads();
        // chunk j holds slabs k in [k_lo, k_hi], k_hi = n-1-j*S
        auto issue = [&](int j) {
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            const unsigned bytes = unsigned(k_hi - k_lo + 1) * slab_bytes;
            const unsigned bar = smem_addr(&full_bar[j % kRing]);
            mbar_expect_tx(bar, bytes);
            bulk_g2s(smem_addr(ring + (j % kRing) * S * slab_f4), tables + (long long)k_lo * p.table_stride, bytes,
                     bar);
        };
        if (threadIdx.x == 0)
            for (int j = 0; j < kRing && j < nchunks; ++j) issue(j);
        bool ok = true;
        for (int j = 0; j < nchunks; ++j) {
            const int slot = j % kRing;
            ok &= mbar_wait(smem_addr(&full_bar[slot]), unsigned((j / kRing) & 1));
            const float4 *__restrict__ chunk = ring + slot * S * slab_f4;
            const int k_hi = n - 1 - j * S;
            const int k_lo = max(0, k_hi - S + 1);
            for (int k = k_hi; k >= k_lo; --k) {
                const float4 *__restrict__ tk = chunk + (k - k_lo) * slab_f4;
                const float h = (k == 0) ? 0.5f : 1.0f;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    drift_split<POW2>(I[q], xi[q], dw[q], dwc[q], shi[q], slo[q], S0[q], N, err);
                    const float4 T = tk[I[q]];
                    kick_comp(dw[q], dwc[q], h * fmaf(xi[q], fmaf(xi[q], T.z, T.y), T.x));
                }
            }
            __syncthreads();  // everyone is done with this slot
            if (threadIdx.x == 0 && j + kRing < nchunks) issue(j + kRing);
        }
        if (!ok) atomicOr(err, kErrStageTimeout);
    }

    const int kind = p.f0_kind;
    const float alpha = float(p.f0p[0]), kdx = float(p.f0p[1] * p.dx[0]), dx_dt = float(p.dx[0] / p.dt);
    const float ub = float(p.f0p[2]);
    const float inv_s2 = kind == NUFI_F0_BUMP_ON_TAIL ? float(1.0 / (p.f0p[3] * p.f0p[3])) : 0.0f;
    double acc = 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        const SplitNode nd = nodes[m0 + q];
        acc += double(delta_f0(kind, alpha, kdx, dx_dt, ub, inv_s2, nd, __ldg(phase + I[q]), xi[q], dw[q] - dwc[q])) +
               nd.g;
    }
    if (s < N) partial[(long long)blockIdx.x * N + s] = acc;
}

namespace {

template <int PPT>
cudaError_t launch_staged_ppt(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                              const float2 *phase, int n, long long qb, long long qe, double *partial,
                              unsigned *err, cudaStream_t st)
{
    const bool pow2 = (p.N[0] & (p.N[0] - 1)) == 0;
    const dim3 grid(sh.ctas), block(sh.threads);
    if (pow2) {
        static const cudaError_t attr = cudaFuncSetAttribute(trace_split_1d_staged_kernel<PPT, true>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (attr != cudaSuccess) return attr;
        trace_split_1d_staged_kernel<PPT, true><<<grid, block, sh.smem, st>>>(p, tables, nodes, phase, n, qb, qe,
                                                                              sh.slabs_per_chunk, partial, err);
    } else {
        static const cudaError_t attr = cudaFuncSetAttribute(trace_split_1d_staged_kernel<PPT, false>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (attr != cudaSuccess) return attr;
        trace_split_1d_staged_kernel<PPT, false><<<grid, block, sh.smem, st>>>(p, tables, nodes, phase, n, qb, qe,
                                                                               sh.slabs_per_chunk, partial, err);
    }
    return cudaGetLastError();
}

}  // namespace

StagedShape staged_shape_1d(const Problem &p, int sms)
{
    StagedShape sh;
    if (p.dim != 1 || p.N[0] > 256) return sh;  // not applicable (one thread per spatial node)
    const long long Nm = p.Nm;
    int G = int(std::min<long long>(Nm, sms));
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
    const size_t kOneCtaPerSm = 120 * 1024;
    int S = int(std::max<size_t>(1, std::min<size_t>(32, kOneCtaPerSm / (size_t(kRing) * slab_bytes))));
    if (size_t(kRing) * S * slab_bytes > 200 * 1024) return sh;
    sh.ctas = G;
    sh.ppt = ppt;
    sh.threads = (p.N[0] + 31) / 32 * 32;
    sh.slabs_per_chunk = S;
    sh.smem = std::max(size_t(kRing) * S * slab_bytes, kOneCtaPerSm);
    sh.ok = true;
    return sh;
}

cudaError_t launch_trace_split_staged(const Problem &p, const StagedShape &sh, const float *tables,
                                      const SplitNode *nodes, const float2 *phase, int n, long long qb, long long qe,
                                      double *partial, int *rows, unsigned *err, cudaStream_t st)
{
    *rows = sh.ctas;
    switch (sh.ppt) {
#define NUFI_CASE(K) \
    case K: return launch_staged_ppt<K>(p, sh, tables, nodes, phase, n, qb, qe, partial, err, st);
        NUFI_CASE(1) NUFI_CASE(2) NUFI_CASE(3) NUFI_CASE(4) NUFI_CASE(5) NUFI_CASE(6) NUFI_CASE(7) NUFI_CASE(8)
#undef NUFI_CASE
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace nufi_gb300
