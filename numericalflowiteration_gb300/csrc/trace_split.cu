// trace_split.cu — FP32-split form of the backward characteristic trace.
//
// State per point (1D): cell index I (int, kept in [0, N)), fraction
// xi in [0, 1) (FP32) and dw, the accumulated kick in cells per substep
// (FP32).  The free-streaming shift of the point's grid velocity,
// w0 = u0 dt / dx, is split once in FP64 into an integer S0 (mod N) and a
// fraction sig = sig_hi + sig_lo; a drift is then
//     t  = (xi - sig_hi) - (sig_lo + dw)
//     I += floor(t) - S0 (mod N),  xi = t - floor(t)  (exact)
// so positions carry ~2^-24 cells of absolute error instead of the
// 2^-24 |x| of a plain FP32 trace, and the large constant part of the
// velocity never meets FP32 rounding.  floor(t) comes from one
// round-down add of 1.5 * 2^23 (valid for |t| < 2^22).
// The kick sum dw is compensated (Kahan: dwc carries the rounding lost by
// each add and is fed back into the next drift), because an uncompensated
// FP32 velocity sum puts O(n^1.5 eps |dw|) into the positions.
//
// The field of slab k is held as, per cell i, the quadratic
// K (A + B xi + C xi^2) = K dS/dxi of the cubic spline on that cell with
// K = -dt^2 / dx^2 (the kick in cells per substep); one 16-byte load and
// two FMAs per substep.  The table is written by the field-solve kernel.
//
// f0 at the foot is evaluated as the difference from its value at the
// grid velocity, f0(x, u) - G(u0) with f0 = (1 + alpha cos kx) G(u), using
// expm1 so that FP32 rounding is relative to the perturbation, not to the
// equilibrium; G(u0) is added back in FP64.  The rho accumulator is FP64.
//
// Same substep order as the reference's eval_ftilda (nufi/rho.hpp:31-61):
// n-1 full drift/kick substeps over slabs n-1..1, then a drift and a half
// kick with slab 0; point convention of nufi/cuda_kernel.cu:37-47.
#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

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

struct F0Split {
    float alpha, kdx, dx_dt, ub, inv_s2;
    int kind;
};

// f0(foot) - G(u0) in FP32 (see file comment).
__device__ __forceinline__ float delta_f0_1d(const F0Split &f, const SplitNode &nd, const float2 cs, float xi, float dw)
{
    float sp, cp;
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
    // bump-on-tail: ga = 0.9 N(u0; 0, 1), gb = 0.1 N(u0; ub, sb)
    const float em1 = expm1f(-(du * (nd.u0f + 0.5f * du)));
    const float em2 = expm1f(-(du * ((nd.u0f - f.ub) + 0.5f * du)) * f.inv_s2);
    return nd.ga * em1 + nd.gb * em2 + f.alpha * c * (nd.ga * (1.0f + em1) + nd.gb * (1.0f + em2));
}

}  // namespace

// dw += k with Kahan compensation (dwc = -(low bits lost so far)).
template <bool COMP>
__device__ __forceinline__ void kick_split(float &dw, float &dwc, float k)
{
    if constexpr (COMP) {
        const float y = k - dwc;
        const float t = dw + y;
        dwc = (t - dw) - y;
        dw = t;
    } else {
        dw += k;
    }
}

template <int PPT, bool POW2, bool COMP>
__global__ void __launch_bounds__(256) trace_split_1d_kernel(const Problem p, const float *__restrict__ tables,
                                                             const SplitNode *__restrict__ nodes,
                                                             const float2 *__restrict__ phase, int n,
                                                             long long q_begin, long long q_end,
                                                             double *__restrict__ partial, unsigned *err)
{
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    const long long s = (long long)blockIdx.x * 32 + lane;
    const long long mb = ((long long)blockIdx.y * W + warp) * PPT;
    const int N = p.N[0];

    int I[PPT], S0[PPT];
    float xi[PPT], dw[PPT], dwc[PPT], shi[PPT], slo[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = mb + q;
        const long long qq = s * p.Nm + m;
        live[q] = (s < p.Ns) && (m < p.Nm) && (qq >= q_begin) && (qq < q_end);
        const SplitNode nd = nodes[m < p.Nm ? m : 0];
        S0[q] = nd.S0;
        shi[q] = nd.sig_hi;
        slo[q] = nd.sig_lo;
        I[q] = int(s < p.Ns ? s : 0);
        xi[q] = 0.0f;
        dw[q] = 0.0f;
        dwc[q] = 0.0f;
    }

    if (n > 0) {
        for (int k = n - 1; k >= 1; --k) {
            const float *__restrict__ tk = tables + (long long)k * p.table_stride;
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                drift_split<POW2>(I[q], xi[q], dw[q], dwc[q], shi[q], slo[q], S0[q], N, err);
                kick_split<COMP>(dw[q], dwc[q], kick_lookup_ldg(tk, N, I[q], xi[q]));
            }
        }
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            drift_split<POW2>(I[q], xi[q], dw[q], dwc[q], shi[q], slo[q], S0[q], N, err);
            kick_split<COMP>(dw[q], dwc[q], 0.5f * kick_lookup_ldg(tables, N, I[q], xi[q]));
        }
    }

    F0Split f;
    f.kind = p.f0_kind;
    f.alpha = float(p.f0p[0]);
    f.kdx = float(p.f0p[1] * p.dx[0]);
    f.dx_dt = float(p.dx[0] / p.dt);
    f.ub = float(p.f0p[2]);
    f.inv_s2 = p.f0_kind == NUFI_F0_BUMP_ON_TAIL ? float(1.0 / (p.f0p[3] * p.f0p[3])) : 0.0f;
    double acc = 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        const SplitNode nd = nodes[mb + q];
        const float df = delta_f0_1d(f, nd, __ldg(phase + I[q]), xi[q], dw[q] - dwc[q]);
        acc += double(df) + nd.g;
    }
    write_partial_tiled(acc, s, p.Ns, partial);
}

bool split_supported(int dim, int order, int f0_kind)
{
    if (order != 4) return false;
    if (dim == 1) return f0_kind == NUFI_F0_LANDAU || f0_kind == NUFI_F0_TWO_STREAM || f0_kind == NUFI_F0_BUMP_ON_TAIL;
    return (dim == 2 || dim == 3) && f0_kind == NUFI_F0_LANDAU;
}

cudaError_t launch_trace_split(const Problem &p, const LaunchShape &ls, const float *tables, const SplitNode *nodes,
                               const float2 *phase, int n, long long qb, long long qe, double *partial, int *rows,
                               unsigned *err, cudaStream_t st)
{
    *rows = ls.vblocks;
    if (p.dim != 1) return cudaErrorNotSupported;
    const dim3 block(32, ls.warps);
    const dim3 grid(unsigned((p.Ns + 31) / 32), unsigned(ls.vblocks));
    const bool pow2 = (p.N[0] & (p.N[0] - 1)) == 0;
#define NUFI_LAUNCH3(PPT, P2, C) \
    trace_split_1d_kernel<PPT, P2, C><<<grid, block, 0, st>>>(p, tables, nodes, phase, n, qb, qe, partial, err);
#define NUFI_LAUNCH(PPT)                                                  \
    if (p.split_plain_kick) {                                             \
        if (pow2) NUFI_LAUNCH3(PPT, true, false) else NUFI_LAUNCH3(PPT, false, false) \
    } else {                                                              \
        if (pow2) NUFI_LAUNCH3(PPT, true, true) else NUFI_LAUNCH3(PPT, false, true) \
    }
    switch (ls.ppt) {
    case 1: NUFI_LAUNCH(1) break;
    case 2: NUFI_LAUNCH(2) break;
    case 4: NUFI_LAUNCH(4) break;
    default: return cudaErrorInvalidValue;
    }
#undef NUFI_LAUNCH
#undef NUFI_LAUNCH3
    return cudaGetLastError();
}

}  // namespace nufi_gb300
