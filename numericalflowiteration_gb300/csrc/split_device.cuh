// split_device.cuh — device pieces shared by the FP32-split kernels:
// shared-memory staging (mbarrier + cp.async.bulk), a bounded grid
// barrier for the persistent kernel, and the split-form drift / kick / f0.
#pragma once

#include "nufi_kernels.cuh"

namespace nufi_gb300 {
namespace split {

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr int kRing = kRingSlots;
constexpr unsigned kWaitLimit = 1u << 22;      // polls of an mbarrier
constexpr unsigned kBarrierLimit = 1u << 26;   // polls of the grid barrier

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

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
// from global memory into this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Orders this thread's earlier (generic-proxy) view of global memory before
// its later bulk copies (async proxy) read it.
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Orders this thread's (and, after a __syncwarp, its warp's) earlier
// generic-proxy accesses to shared memory before its later bulk copies.
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory atomic add with acquire-release semantics at CTA scope;
// returns the old value.
__device__ __forceinline__ unsigned atom_add_acq_rel_cta(unsigned *p, unsigned v)
{
    unsigned old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
                 : "=r"(old)
                 : "r"(smem_addr(p)), "r"(v)
                 : "memory");
    return old;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of a cooperative launch: every block adds 1 to *count
// (monotonic over the launch), then waits until it reaches `target`
// (incremented by gridDim.x per barrier).  The wait is bounded; on timeout
// or when another block has already given up (*abort != 0) it raises
// kErrBarrierTimeout, sets *abort and returns false, and the caller leaves
// the kernel (no hang).
// 64-bit integer add into global memory, no value returned
__device__ __forceinline__ void red_global_add_u64(unsigned long long *addr, unsigned long long v)
{
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(addr), "l"(v) : "memory");
}

__device__ __forceinline__ bool grid_barrier(unsigned *count, unsigned &target, unsigned *abort, unsigned *err)
{
    __shared__ int ok;
    __syncthreads();
    target += gridDim.x;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(count, 1u);
        int good = 1;
        for (unsigned it = 0; ld_acquire_gpu(count) < target; ++it) {
            if (it > kBarrierLimit || ld_acquire_gpu(abort) != 0u) {
                good = 0;
                break;
            }
        }
        if (!good) {
            atomicOr(err, kErrBarrierTimeout);
            atomicExch(abort, 1u);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

template <bool POW2>
__device__ __forceinline__ void drift(int &I, float &xi, float dw, float dwc, float shi, float slo, int S0, int N,
                                      unsigned *err)
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

// dw += k with Kahan compensation (dwc = -(low bits lost so far)).
__device__ __forceinline__ void kick(float &dw, float &dwc, float k)
{
    const float y = k - dwc;
    const float t = dw + y;
    dwc = (t - dw) - y;
    dw = t;
}

struct F0 {
    int kind;
    float alpha, kdx, dx_dt, ub, inv_s2;
    bool small;  // |k dx| <= 1/4: sin / cos of k dx xi by their Taylor polynomials
};

__device__ __forceinline__ F0 make_f0(const Problem &p)
{
    F0 f;
    f.kind = p.f0_kind;
    f.alpha = float(p.f0p[0]);
    f.kdx = float(p.f0p[1] * p.dx[0]);
    f.dx_dt = float(p.dx[0] / p.dt);
    f.ub = float(p.f0p[2]);
    f.inv_s2 = p.f0_kind == NUFI_F0_BUMP_ON_TAIL ? float(1.0 / (p.f0p[3] * p.f0p[3])) : 0.0f;
    f.small = fabs(p.f0p[1] * p.dx[0]) <= 0.25;
    return f;
}

// sin a and cos a for |a| <= 1/4 by their Taylor polynomials to a^9 / a^8
// (truncation below 1e-11, far under FP32 rounding).
__device__ __forceinline__ void sincos_small(float a, float &s, float &c)
{
    const float a2 = a * a;
    s = a * fmaf(a2, fmaf(a2, fmaf(a2, fmaf(a2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
    c = fmaf(a2, fmaf(a2, fmaf(a2, fmaf(a2, 1.0f / 40320.0f, -1.0f / 720.0f), 1.0f / 24.0f), -0.5f), 1.0f);
}

// f0(foot) - G(u0) in FP32: f0 = (1 + alpha cos kx) G(u), expm1 form so
// the rounding is relative to the perturbation (see trace_split.cu).
// A thread's f~ sum over its chains as the FP64 part sum_q g_q (constant
// over the run) plus the FP32 deviations summed by Knuth's two-sum: the
// running sum s and the sum c of its exact rounding errors, s + c within
// about 2^-47 of the terms' magnitudes of the exact sum.  The _rn
// intrinsics keep every rounding as written (no FMA contraction).
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x)
{
    const float t = __fadd_rn(s, x);
    const float bb = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(x, bb)));
    s = t;
}

__device__ __forceinline__ float delta_f0(const F0 &f, const SplitNode &nd, float2 cs, float xi, float dw)
{
    float sp, cp;
    if (f.small)
        sincos_small(f.kdx * xi, sp, cp);
    else
        sincosf(f.kdx * xi, &sp, &cp);
    const float c = cs.x * cp - cs.y * sp;  // cos(k x_foot)
    const float du = dw * f.dx_dt;
    if (f.kind == NUFI_F0_LANDAU) {
        const float em = expm1f(-(du * (nd.u0f + 0.5f * du)));
        return nd.ga * (em + f.alpha * c * (1.0f + em));
    }
    if (f.kind == NUFI_F0_TWO_STREAM) {
        const float u = nd.u0f + du;
        const float em = expm1f(-(du * (nd.u0f + 0.5f * du)));
        const float diff = nd.ga * (u * u * em + du * (2.0f * nd.u0f + du));
        return diff + f.alpha * c * (nd.ga * u * u * (1.0f + em));
    }
    const float em1 = expm1f(-(du * (nd.u0f + 0.5f * du)));
    const float em2 = expm1f(-(du * ((nd.u0f - f.ub) + 0.5f * du)) * f.inv_s2);
    return nd.ga * em1 + nd.gb * em2 + f.alpha * c * (nd.ga * (1.0f + em1) + nd.gb * (1.0f + em2));
}

}  // namespace split
}  // namespace nufi_gb300

namespace nufi_gb300 {
namespace split {

// Packed FP32 pairs (two chains per instruction: add / sub / fma .f32x2,
// sm_100 family).  Each op is the IEEE operation of the scalar code on
// both lanes, so the pairs give the same bits as one chain at a time.
__device__ __forceinline__ unsigned long long f2_pack(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_add_rm(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Shared-memory loads at a 32-bit shared-window address.  The paired
// kick-table lookups of the staged traces go through these, so their
// addresses stay 32-bit integer arithmetic (0.9 % off the whole 1D run,
// same bits).  volatile keeps them after the mbarrier wait that makes the
// slab visible.
__device__ __forceinline__ float2 lds_f32x2(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
__device__ __forceinline__ float lds_f32(unsigned addr)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

// (cos, sin) of k x at a foot that wrapped the domain w times (unwrapped
// cell I + N w): the wrapped cell's phase turned by w k L (phase_wrap = k L
// mod 2 pi; the product reduced in FP64 before the FP32 sincos)
__device__ __forceinline__ float2 phase_unwrapped(float2 cs, int w, double phase_wrap)
{
    if (w == 0) return cs;
    const double a = fmod(double(w) * phase_wrap, 6.283185307179586476925286766559);
    float sr, cr;
    sincosf(float(a), &sr, &cr);
    return make_float2(cs.x * cr - cs.y * sr, cs.y * cr + cs.x * sr);
}

template <bool POW2>
__device__ __forceinline__ int wrap_cell(int J, int N, unsigned *err)
{
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
    return J;
}

// Substeps k_hi..k_lo (descending) of PPT chains over a chunk of tables in
// shared memory (slab k at chunk + (k - k_lo) * TS floats, kick_lookup layout).
// State per chain: cell I, fraction xi, and the kick sum in two levels:
// dwT (+ Kahan term dwTc) holds the sum up to the previous chunk and
// starts at sig_lo, the low part of the free-streaming fraction; dwC sums
// this chunk's kicks in plain FP32 and is folded into dwT at the end.
//   drift:  t = ((xi - sig_hi) - dwT) - dwC
//           floor(t) by a round-down add of 1.5*2^23, whose bit pattern
//           minus S0m = S0 + bits(1.5*2^23) moves the cell
//   kick:   dwC += K (A + B xi + C xi^2) of the cell (halved for k = 0)
// With UNWRAP (N a power of two), Wr counts each chain's wraps of the
// domain: the new cell before the mask, divided by N (arithmetic shift by
// log2n), adds to Wr, so the unwrapped cell is I + N Wr - n (S0u - S0).
// Chains go two at a time through the packed FP32 instructions (the FP32
// part of a substep, 9 operations, in 9 instructions for two chains); the
// integer cell update and the two shared loads stay per chain.
template <int PPT, bool POW2, bool UNWRAP = false, int UNROLL = 1>
__device__ __forceinline__ void trace_chunk(const float *__restrict__ chunk, int TS, int k_hi, int k_lo, int N,
                                            int (&I)[PPT], float (&xi)[PPT], float (&dwT)[PPT], float (&dwTc)[PPT],
                                            const float (&shi)[PPT], const int (&S0m)[PPT], unsigned *err,
                                            int (*Wr)[PPT] = nullptr, int log2n = 0)
{
    static_assert(POW2 || !UNWRAP, "wrap counts need N a power of two");
    constexpr int NP = PPT / 2;  // packed pairs; chain PPT-1 alone when PPT is odd
    const unsigned long long MAG2 = f2_pack(kMagic, kMagic);
    unsigned long long X[NP > 0 ? NP : 1], SH[NP > 0 ? NP : 1], DT[NP > 0 ? NP : 1], DC[NP > 0 ? NP : 1];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        X[p] = f2_pack(xi[2 * p], xi[2 * p + 1]);
        SH[p] = f2_pack(shi[2 * p], shi[2 * p + 1]);
        DT[p] = f2_pack(dwT[2 * p], dwT[2 * p + 1]);
        DC[p] = 0ull;
    }
    float dwC_last = 0.0f;
    auto substep = [&](const float *__restrict__ tk, float h) {
        const unsigned long long H2 = f2_pack(h, h);
        // table of this slab in the shared window: (K B, K C) at tb + 8 J, K A at tc + 4 J
        const unsigned tb = smem_addr(tk), tc = tb + unsigned(N) * 8u;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const unsigned long long t = f2_sub(f2_sub(f2_sub(X[p], SH[p]), DT[p]), DC[p]);
            const unsigned long long mg = f2_add_rm(t, MAG2);
            float mg0, mg1;
            f2_unpack(mg, mg0, mg1);
            const int r0 = I[2 * p] - S0m[2 * p] + __float_as_int(mg0);
            const int r1 = I[2 * p + 1] - S0m[2 * p + 1] + __float_as_int(mg1);
            const int J0 = wrap_cell<POW2>(r0, N, err);
            const int J1 = wrap_cell<POW2>(r1, N, err);
            if constexpr (UNWRAP) {
                (*Wr)[2 * p] += r0 >> log2n;
                (*Wr)[2 * p + 1] += r1 >> log2n;
            }
            I[2 * p] = J0;
            I[2 * p + 1] = J1;
            X[p] = f2_sub(t, f2_sub(mg, MAG2));
            const float2 bc0 = lds_f32x2(tb + unsigned(J0) * 8u);
            const float2 bc1 = lds_f32x2(tb + unsigned(J1) * 8u);
            const float a0 = lds_f32(tc + unsigned(J0) * 4u);
            const float a1 = lds_f32(tc + unsigned(J1) * 4u);
            // the quadratic per chain in scalar FMAs (the roundings of the
            // packed form): its operands arrive in different register pairs,
            // which the packed form would first have to move together
            // (62.9 -> 62.5 ms on the whole two-stream run)
            float x0, x1;
            f2_unpack(X[p], x0, x1);
            const float k0 = fmaf(x0, fmaf(x0, bc0.y, bc0.x), a0);
            const float k1 = fmaf(x1, fmaf(x1, bc1.y, bc1.x), a1);
            const unsigned long long kq = f2_pack(k0, k1);
            DC[p] = (h == 1.0f) ? f2_add(DC[p], kq) : f2_fma(H2, kq, DC[p]);
        }
        if constexpr (PPT % 2 == 1) {
            constexpr int q = PPT - 1;
            const float t = ((xi[q] - shi[q]) - dwT[q]) - dwC_last;
            const float mg = __fadd_rd(t, kMagic);
            const int r = I[q] - S0m[q] + __float_as_int(mg);
            const int J = wrap_cell<POW2>(r, N, err);
            if constexpr (UNWRAP) (*Wr)[q] += r >> log2n;
            I[q] = J;
            xi[q] = t - (mg - kMagic);
            // the odd chain keeps the plain loads: with the ordering of
            // volatile loads here the whole run measured 1 % slower
            const float kq = kick_lookup(tk, N, J, xi[q]);
            dwC_last = (h == 1.0f) ? dwC_last + kq : fmaf(h, kq, dwC_last);
        }
    };
    const int k_stop = max(k_lo, 1);
    // UNROLL substeps per loop trip: the whole-run and batch traces take 2
    // (the loop's own work is shared and the second substep's address
    // arithmetic overlaps the first: 62.9 -> 60.7 ms on the whole two-stream
    // run); the per-step staged trace measured faster with 1
#pragma unroll UNROLL
    for (int k = k_hi; k >= k_stop; --k) substep(chunk + (k - k_lo) * TS, 1.0f);
    if (k_lo == 0) substep(chunk, 0.5f);
    // fold this chunk's kicks into the compensated totals
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        f2_unpack(X[p], xi[2 * p], xi[2 * p + 1]);
        float c0, c1;
        f2_unpack(DC[p], c0, c1);
        kick(dwT[2 * p], dwTc[2 * p], c0);
        kick(dwT[2 * p + 1], dwTc[2 * p + 1], c1);
    }
    if constexpr (PPT % 2 == 1) kick(dwT[PPT - 1], dwTc[PPT - 1], dwC_last);
}

}  // namespace split
}  // namespace nufi_gb300
