// trace_split_nd.cu — FP32-split trace in 2D2V and 3D3V.
//
// Per axis a the state is the 1D split form (split_device.cuh): integer
// cell I_a, FP32 fraction xi_a in [0, 1), and the kick sum in cells per
// substep in two levels (plain FP32 within a chunk of slabs, Kahan-
// compensated across chunks; the sum starts at the low part of the free-
// streaming fraction).  The field of slab k is its FP32 padded copy written
// by the field solve: the reference layout (x fastest, periodic padding to
// N + 3 per axis) with x rows widened to table_sx floats so that the rows
// one warp spans use disjoint shared-memory banks.  All components
// of E come from one gather of the 4^D window, contracted with the cubic
// B-spline value and derivative bases per axis (the arithmetic of
// splines2d / splines3d::eval and of the reference's separate eval<1,0> /
// eval<0,1> calls, nufi/splines.hpp:117-172, nufi/rho.hpp:213-214, 343-345,
// in FP32):  kick_a = -(dt / dx_a)^2 * dS/dxi_a  (cells per substep).
// f0 is the Landau form (1 + alpha sum_a cos(k x_a)) prod_a g(u_a)
// (nufi/config.hpp:148-149, 233-234), evaluated as f0(foot) - G(u0) with
// expm1; G(u0) is added back in FP64.
//
// Geometry: about one CTA per SM; CTA c owns the velocity nodes c, c + G,
// c + 2G, ... (interleaved: a spread of velocities per CTA) for every
// spatial node.  Thread t owns the spatial
// nodes s = node(t + T j) and visits its items in (j, m) order, PPT at a
// time (one full trace per batch), so the 32 lanes of a warp hold 32
// spatial nodes at one velocity: x fastest, and when N[0] < 32 the
// 32 / N[0] x rows of a warp row_step rows apart (node(v) = v when
// row_step = 0), on disjoint shared-memory banks (see table_sx): neighbouring
// cells, conflict-free gathers.  Each thread is the only one in the CTA to
// touch its nodes, and its items of one node are consecutive, so rho is a
// register sum flushed to partial[c][s] when j changes (FP64, fixed order:
// deterministic).
//
// Tables: with ring > 0 the history is streamed through `ring` shared-
// memory slots of S slabs (cp.async.bulk completing on an mbarrier), one
// chunk stream over all batches so the copies run ahead across batch
// boundaries; the last warp to finish a slot refills it (per-slot count
// in shared memory, acquire-release), so warps wait only for their data;
// with ring == 0 (slabs too large for shared memory) the
// gathers read the tables in global memory.  Every mbarrier wait is
// bounded; a timeout raises kErrStageTimeout (no trap, no hang).
#include <algorithm>

#include "split_device.cuh"

namespace nufi_gb300 {

using namespace split;

namespace {

// Cubic B-spline basis values N[i] and derivatives D[i] on [0, 1)
// (splines1d::N<real,4,0> and <real,4,1>, nufi/splines.hpp:39-79).
__device__ __forceinline__ void cubic_basis(float x, float (&Nv)[4], float (&Dv)[4])
{
    const float x2 = x * x, x3 = x2 * x, u = 1.0f - x;
    constexpr float s6 = 1.0f / 6.0f;
    Nv[0] = u * u * u * s6;
    Nv[1] = fmaf(x2, fmaf(3.0f, x, -6.0f), 4.0f) * s6;
    Nv[3] = x3 * s6;
    Nv[2] = 1.0f - (Nv[0] + Nv[1] + Nv[3]);
    Dv[0] = -0.5f * u * u;
    Dv[1] = x * fmaf(1.5f, x, -2.0f);
    Dv[3] = 0.5f * x2;
    Dv[2] = -(Dv[0] + Dv[1] + Dv[3]);
}

template <int D>
struct Chain {
    int I[D], S0m[D], Wr[D];  // Wr: wraps of the domain per axis (UNWRAP)
    float xi[D], dwT[D], dwTc[D], dwC[D], shi[D];
};

// Drift of one axis: as the 1D chunk loop (split_device.cuh); with UNWRAP
// (N a power of two) the wraps of the domain add to Wr.
template <bool POW2, bool UNWRAP>
__device__ __forceinline__ void drift_axis(int &I, float &xi, float dwT, float dwC, float shi, int S0m, int N,
                                           unsigned *err, int &Wr, int log2n)
{
    static_assert(POW2 || !UNWRAP, "wrap counts need N a power of two");
    const float t = ((xi - shi) - dwT) - dwC;
    const float mg = __fadd_rd(t, kMagic);
    int J = I - S0m + __float_as_int(mg);
    if constexpr (UNWRAP) Wr += J >> log2n;
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
    xi = t - (mg - kMagic);
}

// dS/dxi_a of the FP32 slab window at the chain's cells and fractions.
// Rows j and j+1 of the window go through the packed FP32 instructions
// together (f32x2: the same IEEE operation on both lanes): their x sums
// with the value and derivative bases, then their shares of the y (and z)
// sums, whose two halves are added at the end.
template <int D>
__device__ __forceinline__ void field_grad(const float *__restrict__ slab, int sy, int sz, const Chain<D> &c,
                                           float (&g)[D])
{
    float Nx[4], Dx[4], Ny[4], Dy[4];
    cubic_basis(c.xi[0], Nx, Dx);
    cubic_basis(c.xi[1], Ny, Dy);
    unsigned long long NXX[4], DXX[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        NXX[i] = f2_pack(Nx[i], Nx[i]);
        DXX[i] = f2_pack(Dx[i], Dx[i]);
    }
    const unsigned long long NY01 = f2_pack(Ny[0], Ny[1]), NY23 = f2_pack(Ny[2], Ny[3]);
    const unsigned long long DY01 = f2_pack(Dy[0], Dy[1]), DY23 = f2_pack(Dy[2], Dy[3]);
    // x sums of rows (j, j+1) at plane w: R0 = sum_i v N_i, R1 = sum_i v D_i
    auto rows = [&](const float *w, int j, unsigned long long &R0, unsigned long long &R1) {
        R0 = 0ull;
        R1 = 0ull;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const unsigned long long V = f2_pack(w[j * sy + i], w[(j + 1) * sy + i]);
            R0 = f2_fma(V, NXX[i], R0);
            R1 = f2_fma(V, DXX[i], R1);
        }
    };
    if constexpr (D == 2) {
        const float *w = slab + c.I[1] * sy + c.I[0];
        unsigned long long GX = 0ull, GY = 0ull, R0, R1;
        rows(w, 0, R0, R1);
        GX = f2_fma(R1, NY01, GX);
        GY = f2_fma(R0, DY01, GY);
        rows(w, 2, R0, R1);
        GX = f2_fma(R1, NY23, GX);
        GY = f2_fma(R0, DY23, GY);
        float a, b;
        f2_unpack(GX, a, b);
        g[0] = a + b;
        f2_unpack(GY, a, b);
        g[1] = a + b;
    } else {
        float Nz[4], Dz[4];
        cubic_basis(c.xi[2], Nz, Dz);
        const float *w = slab + c.I[2] * sz + c.I[1] * sy + c.I[0];
        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float *wk = w + k * sz;
            unsigned long long AX = 0ull, AY = 0ull, AZ = 0ull, R0, R1;
            rows(wk, 0, R0, R1);
            AX = f2_fma(R1, NY01, AX);
            AY = f2_fma(R0, DY01, AY);
            AZ = f2_fma(R0, NY01, AZ);
            rows(wk, 2, R0, R1);
            AX = f2_fma(R1, NY23, AX);
            AY = f2_fma(R0, DY23, AY);
            AZ = f2_fma(R0, NY23, AZ);
            float a, b;
            f2_unpack(AX, a, b);
            gx = fmaf(a + b, Nz[k], gx);
            f2_unpack(AY, a, b);
            gy = fmaf(a + b, Nz[k], gy);
            f2_unpack(AZ, a, b);
            gz = fmaf(a + b, Dz[k], gz);
        }
        g[0] = gx;
        g[1] = gy;
        g[2] = gz;
    }
}

}  // namespace

template <int D, int PPT, bool POW2, bool STAGED, bool UNWRAP>
__global__ void __launch_bounds__(512, 1) trace_split_nd_kernel(const Problem p, const float *__restrict__ tables,
                                                                const SplitNode *__restrict__ nodes,
                                                                const float2 *__restrict__ phase, int n,
                                                                long long q_begin, long long q_end, int S, int R,
                                                                double *__restrict__ partial, unsigned *err)
{
    extern __shared__ __align__(128) float ring[];
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    __shared__ unsigned released[kRing];  // warps done with the slot's chunk

    const int T = blockDim.x;
    const int t = threadIdx.x;
    const int G = gridDim.x;
    const int W = T >> 5;
    const long long Ns = p.Ns;
    // velocity nodes interleaved over the CTAs: CTA c owns c, c + G, ...
    const long long Mc = (p.Nm - blockIdx.x + G - 1) / G;
    const long long nj = t < Ns ? (Ns - t + T - 1) / T : 0;  // spatial nodes of this thread
    const long long nj0 = (Ns + T - 1) / T;                  // ... of thread 0 (the most)
    const long long batches = (nj0 * Mc + PPT - 1) / PPT;
    const int sy = p.table_sx, sz = p.table_sx * p.P[1];
    // spatial node of virtual index v (< Ns, so in int range): lane l of
    // warp w takes x = l mod N0 of row y0 + (l / N0) row_step, y0 = w mod
    // row_step, in plane w / row_step (once per batch)
    auto node_of = [&](long long v) -> long long {
        if (p.row_step == 0) return v;
        const int vi = int(v), N0 = p.N[0], w = vi >> 5;
        const int x = vi % N0, r = (vi & 31) / N0;
        return x + (long long)N0 * ((w % p.row_step + r * p.row_step) + (long long)p.N[1] * (w / p.row_step));
    };
    float K[D];
#pragma unroll
    for (int a = 0; a < D; ++a) K[a] = float(-p.dt * p.dt * p.dxinv[a] * p.dxinv[a]);
    const long long slab_f = p.table_stride;

    // chunk stream: chunk g is chunk j = g mod nchunks of batch g / nchunks
    // and covers slabs [k_lo, k_hi]; it lands in ring slot g mod R.  The
    // loops below carry j, the slot and the mbarrier phase along instead of
    // dividing the 64-bit g (a software division, once per slab in 3D,
    // where a chunk is one slab).
    const int nchunks = n > 0 ? (n + S - 1) / S : 0;
    const long long total_chunks = batches * nchunks;
    auto chunk_range = [&](int j, int &k_hi, int &k_lo) {
        k_hi = n - 1 - j * S;
        k_lo = max(0, k_hi - S + 1);
    };
    auto issue = [&](int j, int slot) {
        int k_hi, k_lo;
        chunk_range(j, k_hi, k_lo);
        const unsigned bar = smem_addr(&full_bar[slot]);
        const unsigned bytes = unsigned(k_hi - k_lo + 1) * unsigned(slab_f) * 4u;
        mbar_expect_tx(bar, bytes);
        bulk_g2s(smem_addr(ring + (long long)slot * S * slab_f), tables + (long long)k_lo * slab_f, bytes, bar);
    };
    if constexpr (STAGED) {
        if (t == 0) {
            for (int r = 0; r < R; ++r) {
                mbar_init(smem_addr(&full_bar[r]), 1);
                released[r] = 0;
            }
            mbar_fence_init();
        }
        __syncthreads();
        if (t == 0)
            for (int g0 = 0; g0 < R && g0 < total_chunks; ++g0) issue(g0 % nchunks, g0);
    }
    bool ok = true;
    long long g = 0;     // next chunk of the stream
    int slot = 0;        // its ring slot, g mod R
    unsigned parity = 0;  // its mbarrier phase parity, (g / R) & 1

    long long cur_j = 0;
    double acc = 0;
    for (long long b = 0; b < batches; ++b) {
        Chain<D> ch[PPT];
        bool live[PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const long long k = b * PPT + q;
            const long long j = k / Mc;
            const long long m = blockIdx.x + (k % Mc) * G;
            const long long s = node_of(t + j * T);
            const bool inside = j < nj;
            const long long qq = s * p.Nm + m;
            live[q] = inside && qq >= q_begin && qq < q_end;
            long long rs = inside ? s : 0, rm = m;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                const SplitNode nd = nodes[(a > 0 ? p.M[0] : 0) + (a > 1 ? p.M[1] : 0) + int(rm % p.M[a])];
                ch[q].I[a] = int(rs % p.N[a]);
                ch[q].Wr[a] = 0;
                rs /= p.N[a];
                rm /= p.M[a];
                ch[q].S0m[a] = nd.S0 + kMagicBits;
                ch[q].shi[a] = nd.sig_hi;
                ch[q].xi[a] = 0.0f;
                ch[q].dwT[a] = nd.sig_lo;
                ch[q].dwTc[a] = 0.0f;
                ch[q].dwC[a] = 0.0f;
            }
        }
        auto substep = [&](const float *__restrict__ sl, float h) {
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
#pragma unroll
                for (int a = 0; a < D; ++a)
                    drift_axis<POW2, UNWRAP>(ch[q].I[a], ch[q].xi[a], ch[q].dwT[a], ch[q].dwC[a], ch[q].shi[a],
                                             ch[q].S0m[a], p.N[a], err, ch[q].Wr[a], __ffs(p.N[a]) - 1);
                float gr[D];
                field_grad<D>(sl, sy, sz, ch[q], gr);
#pragma unroll
                for (int a = 0; a < D; ++a) ch[q].dwC[a] = fmaf(h * K[a], gr[a], ch[q].dwC[a]);
            }
        };
        for (int j = 0; j < nchunks; ++j, ++g) {
            int k_hi, k_lo;
            chunk_range(j, k_hi, k_lo);
            const float *__restrict__ base;
            if constexpr (STAGED) {
                ok &= mbar_wait(smem_addr(&full_bar[slot]), parity);
                base = ring + (long long)slot * S * slab_f;
            } else {
                base = tables + (long long)k_lo * slab_f;
            }
            const int k_stop = max(k_lo, 1);
            for (int k = k_hi; k >= k_stop; --k) substep(base + (k - k_lo) * slab_f, 1.0f);
            if (k_lo == 0) substep(base, 0.5f);
#pragma unroll
            for (int q = 0; q < PPT; ++q)
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    kick(ch[q].dwT[a], ch[q].dwTc[a], ch[q].dwC[a]);
                    ch[q].dwC[a] = 0.0f;
                }
            if constexpr (STAGED) {
                // the last warp to finish the slot refills it; no warp
                // waits for another, only for its data
                __syncwarp();
                if ((t & 31) == 0 && atom_add_acq_rel_cta(&released[slot], 1u) == unsigned(W - 1)) {
                    released[slot] = 0;
                    fence_proxy_async_shared();
                    if (g + R < total_chunks) {
                        int jr = j + R;  // chunk g + R is chunk jr mod nchunks of its batch
                        while (jr >= nchunks) jr -= nchunks;
                        issue(jr, slot);
                    }
                }
                if (++slot == R) {
                    slot = 0;
                    parity ^= 1u;
                }
            }
        }
        // f0(foot) - G(u0) in FP32, the FP64 background G(u0) added back
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            const long long k = b * PPT + q;
            const long long j = k / Mc;
            if (j != cur_j) {
                if (cur_j < nj) partial[(long long)blockIdx.x * Ns + node_of(t + cur_j * T)] = acc;
                acc = 0;
                cur_j = j;
            }
            if (!live[q]) continue;
            long long rm = blockIdx.x + (k % Mc) * G;
            float delta = 0.0f, csum = 0.0f, Gf = 1.0f;
            double Gd = 1.0;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                const SplitNode nd = nodes[(a > 0 ? p.M[0] : 0) + (a > 1 ? p.M[1] : 0) + int(rm % p.M[a])];
                rm /= p.M[a];
                const float du = ((ch[q].dwT[a] - ch[q].dwTc[a]) - nd.sig_lo) * float(p.dx[a] / p.dt);
                delta = fmaf(du, nd.u0f + 0.5f * du, delta);
                float2 cs = __ldg(phase + (a > 0 ? p.N[0] : 0) + (a > 1 ? p.N[1] : 0) + ch[q].I[a]);
                if constexpr (UNWRAP)
                    cs = phase_unwrapped(cs, ch[q].Wr[a] - n * ((nd.S0u - nd.S0) / p.N[a]), p.phase_wrap[a]);
                float sp, cp;
                sincosf(float(p.f0p[1] * p.dx[a]) * ch[q].xi[a], &sp, &cp);
                csum += cs.x * cp - cs.y * sp;
                Gf *= nd.ga;
                Gd *= nd.g;
            }
            const float em = expm1f(-delta);
            const float df = Gf * (em + float(p.f0p[0]) * csum * (1.0f + em));
            acc += double(df) + Gd;
        }
    }
    if (cur_j < nj) partial[(long long)blockIdx.x * Ns + node_of(t + cur_j * T)] = acc;
    if (!ok) atomicOr(err, kErrStageTimeout);
}

namespace {

template <int D, int PPT, bool STAGED>
cudaError_t launch_nd(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                      const float2 *phase, int n, long long qb, long long qe, double *partial, unsigned *err,
                      cudaStream_t st)
{
    bool pow2 = true;
    for (int a = 0; a < D; ++a) pow2 = pow2 && ((p.N[a] & (p.N[a] - 1)) == 0);
    void (*fn)(const Problem, const float *, const SplitNode *, const float2 *, int, long long, long long, int, int,
               double *, unsigned *) = pow2 ? trace_split_nd_kernel<D, PPT, true, STAGED, false>
                                            : trace_split_nd_kernel<D, PPT, false, STAGED, false>;
    if (phase_wraps(p)) {  // f0's phase at the unwrapped foot (admitted for every N a power of two)
        if (!pow2) return cudaErrorInvalidValue;
        fn = trace_split_nd_kernel<D, PPT, true, STAGED, true>;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sh.smem));
    if (e != cudaSuccess) return e;
    fn<<<sh.ctas, sh.threads, sh.smem, st>>>(p, tables, nodes, phase, n, qb, qe, sh.slabs_per_chunk,
                                             STAGED ? sh.ring : 1, partial, err);
    return cudaGetLastError();
}

template <int D, int PPT>
cudaError_t launch_nd_mode(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                           const float2 *phase, int n, long long qb, long long qe, double *partial, unsigned *err,
                           cudaStream_t st)
{
    if (sh.ring > 0) return launch_nd<D, PPT, true>(p, sh, tables, nodes, phase, n, qb, qe, partial, err, st);
    return launch_nd<D, PPT, false>(p, sh, tables, nodes, phase, n, qb, qe, partial, err, st);
}

}  // namespace

// One CTA per SM (at most Nm), T = min(512, Ns rounded up to a warp)
// threads; S slabs per ring slot from a 120 KB budget (more than half of
// an SM's shared memory, so no SM holds two CTAs), 3 slots, or 2 when 3 do
// not fit in 220 KB, else the tables stay in global memory.
StagedShape staged_shape_nd(const Problem &p, int sms)
{
    StagedShape sh;
    if (p.dim < 2 || p.order != 4) return sh;
    const size_t slab_bytes = size_t(p.table_stride) * 4;
    const size_t kOneCtaPerSm = 120 * 1024, kMaxSmem = 220 * 1024;
    sh.ctas = int(std::min<long long>(p.Nm, sms));
    sh.threads = int(std::min<long long>(512, (p.Ns + 31) / 32 * 32));
    sh.ppt = p.dim == 2 ? 2 : 1;
    sh.tpn = 1;
    if (size_t(kRing) * slab_bytes <= kMaxSmem) {
        sh.ring = kRing;
        sh.slabs_per_chunk =
            int(std::max<size_t>(1, std::min<size_t>(16, kMaxSmem / (size_t(kRing) * slab_bytes))));
    } else if (2 * slab_bytes <= kMaxSmem) {
        sh.ring = 2;
        sh.slabs_per_chunk = 1;
    } else {
        sh.ring = 0;
        sh.slabs_per_chunk = 16;
    }
    sh.smem = sh.ring > 0 ? std::max(size_t(sh.ring) * sh.slabs_per_chunk * slab_bytes, kOneCtaPerSm) : 0;
    sh.ok = true;
    return sh;
}

cudaError_t launch_trace_split_nd(const Problem &p, const StagedShape &sh, const float *tables, const SplitNode *nodes,
                                  const float2 *phase, int n, long long qb, long long qe, double *partial, int *rows,
                                  unsigned *err, cudaStream_t st)
{
    *rows = sh.ctas;
    if (p.dim == 2) return launch_nd_mode<2, 2>(p, sh, tables, nodes, phase, n, qb, qe, partial, err, st);
    if (p.dim == 3) return launch_nd_mode<3, 1>(p, sh, tables, nodes, phase, n, qb, qe, partial, err, st);
    return cudaErrorNotSupported;
}

}  // namespace nufi_gb300
