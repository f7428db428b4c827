// run_split_1d.cu — a whole FP32-split 1D simulation (steps n0..n1) in one
// cooperative launch.
//
// The per-step work outside the trace is small (Ns <= 256 nodes) but a
// chain of dependent phases: partial sums -> rho -> circulant solve ->
// slab, table and W_n.  As separate launches each phase costs a launch gap
// and a cold start (about 20 us per step in total, against ~100 us of trace
// at mid-run).  Here the grid stays resident (one CTA per SM, co-resident
// by the cooperative launch) and the phases are separated by a bounded grid
// barrier, two per step:
//   trace    each CTA: its velocity chains through slabs n-1..0, streamed
//            through the shared-memory ring (as trace_split_staged.cu);
//            the CTA's sum of f~ for each node is added into
//            rho_fix[n % 2][s] as a 64-bit fixed-point integer (scale 2^F,
//            chosen on the host so that no sum leaves the range): integer
//            sums are exact and independent of their order, so rho is
//            deterministic without a reduction phase of its own
//   barrier
//   solve    every CTA reads rho from the integers and computes its nodes'
//            circulant products c, phi, K(A,B,C) from the Green's kernels
//            held in shared memory for the whole run; writes slab n (FP64),
//            table n (store_kick_entry) and, per node, rho_i phi_i into row
//            n of epart; CTA 0 writes rho and clears rho_fix[(n+1) % 2]
//   barrier
// After the last step, W_n = L/(2N) sum_i epart[n][i] for all n at once
// (no per-step energy reduction on the critical path).
// The next step's trace reads table n through the async proxy (bulk
// copies) after the barrier; fence.proxy.async.global orders that read
// after the generic-proxy writes made visible by the barrier.
// All arithmetic is that of trace_split_staged.cu and field_solve.cu.
#include "split_device.cuh"

namespace nufi_gb300 {

using namespace split;

// Which of the five solve sums lane `lane` holds after the butterfly in
// the solve phase (lanes 4q..4q+3 share one; -1: none).
__device__ __forceinline__ int lane_sum_of(int lane)
{
    const int q = lane >> 2;
    return q < 3 ? q : (q == 4 || q == 5) ? q - 1 : -1;
}

template <int PPT, bool POW2, bool UNWRAP>
__global__ void __launch_bounds__(PPT > 4 ? 256 : 512, 1) run_split_1d_kernel(
    const Problem p, float *__restrict__ tables, double *__restrict__ hist, const SplitNode *__restrict__ nodes,
    const float2 *__restrict__ phase, const double *__restrict__ green, unsigned long long *__restrict__ rho_fix,
    double fix_scale, double fix_limit, double *__restrict__ rho, double *__restrict__ energy,
    double *__restrict__ epart, int n0, int n1, int S, int Nr, unsigned *sync, unsigned *err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long full_bar[kRing];
    __shared__ unsigned released[kRing];  // warps done with the slot's chunk
    __shared__ double wacc[16][5];
    __shared__ double combine[256];

    const int N = p.N[0];
    const int G = gridDim.x;
    const int W = blockDim.x >> 5;
    const int s = threadIdx.x % Nr;    // spatial node of this thread
    const int grp = threadIdx.x / Nr;  // its chain group
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int TS = int(p.table_stride);  // floats per slab table
    const int log2n = __ffs(N) - 1;      // UNWRAP: N is a power of two
    float *ring = reinterpret_cast<float *>(smem_raw);
    double *rs = reinterpret_cast<double *>(smem_raw + size_t(kRing) * S * TS * sizeof(float));  // rho' [N]
    double *gs = rs + N;                                                                       // green [5][N]
    unsigned *count = sync, *abort = sync + 1;

    // velocity nodes interleaved over the CTAs (chain j of CTA c: c + j G),
    // so every CTA holds a spread of velocities and the per-step barriers
    // wait less for the CTAs whose velocities filament most
    long long mv[PPT];
    int S0m[PPT];
    float shi[PPT], slo[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = blockIdx.x + (long long)(grp * PPT + q) * G;
        live[q] = (s < N) && (m < p.Nm);
        mv[q] = live[q] ? m : blockIdx.x;
        const SplitNode nd = nodes[mv[q]];
        S0m[q] = nd.S0 + kMagicBits;
        shi[q] = nd.sig_hi;
        slo[q] = nd.sig_lo;
    }
    // the FP64 part of this thread's f~ sum, constant over the run (chain order)
    double gsum = 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q)
        if (live[q]) gsum += nodes[mv[q]].g;

    for (int j = threadIdx.x; j < 5 * N; j += blockDim.x) gs[j] = green[j];
    if (threadIdx.x == 0) {
        for (int r = 0; r < kRing; ++r) {
            mbar_init(smem_addr(&full_bar[r]), 1);
            released[r] = 0;
        }
        mbar_fence_init();
    }
    __syncthreads();

    const F0 f = make_f0(p);
    const unsigned slab_bytes = unsigned(p.table_stride) * 4u;
    unsigned target = 0;
    // nodes of this CTA in the solve phase: blockIdx.x + k*G
    const int K = blockIdx.x < N ? (N - 1 - int(blockIdx.x)) / G + 1 : 0;
    int Kp = 1;
    while (Kp < K) Kp <<= 1;
    const int wpn = K > 0 ? W / Kp : W;  // warps per node in the solve
    const double Lfac = p.L[0] / (2.0 * double(N));

    // The ring as one stream of chunks over the whole run: chunk g (global
    // count from n0) sits in slot g % kRing, phase parity (g / kRing) & 1.
    // Chunk j of step n holds slabs [k_lo, k_hi], k_hi = n-1-j*S.  A slot
    // is refilled by the last warp to release it (a per-slot count in
    // shared memory), with chunk g + kRing: of this step, or of step n+1
    // (its chunk 0 without its newest slab n-1+1 = n, which the field solve
    // of step n has not written yet).  After the grid barriers of step n,
    // thread 0 issues that newest slab, and the first chunks of step n+1
    // whose predecessors were not in step n.  No warp waits for another in
    // the trace; it waits only for its data.
    auto nchunks_of = [&](int n) { return n > 0 ? (n + S - 1) / S : 0; };
    auto chunk_range = [&](int n, int j, int &k_lo, int &k_hi) {
        k_hi = n - 1 - j * S;
        k_lo = max(0, k_hi - S + 1);
    };
    // bulk copy of slabs k_from..k_to of chunk (n, j) in slot `slot`
    auto copy_part = [&](int n, int j, unsigned slot, int k_from, int k_to) {
        int k_lo, k_hi;
        chunk_range(n, j, k_lo, k_hi);
        bulk_g2s(smem_addr(ring + slot * S * TS + (k_from - k_lo) * TS), tables + (long long)k_from * p.table_stride,
                 unsigned(k_to - k_from + 1) * slab_bytes, smem_addr(&full_bar[slot]));
    };
    // arm slot for the whole chunk (n, j), then copy slabs k_lo..k_last
    auto issue = [&](int n, int j, unsigned slot, int k_last) {
        int k_lo, k_hi;
        chunk_range(n, j, k_lo, k_hi);
        mbar_expect_tx(smem_addr(&full_bar[slot]), unsigned(k_hi - k_lo + 1) * slab_bytes);
        if (k_last >= k_lo) copy_part(n, j, slot, k_lo, k_last);
    };
    // Thread 0 at the start of step m (after the barriers of step m-1, or
    // at launch): complete chunk 0's newest slab, issue the first chunks
    // whose predecessor chunk g - kRing is older than step m-1.
    unsigned gbase = 0, gbase_prev = 0;  // first chunk of this / the previous step
    auto start_step = [&](int m, bool first) {
        const int nch = nchunks_of(m);
        for (int j = 0; j < kRing && j < nch; ++j) {
            const unsigned g = gbase + j;
            const bool pred_prev = !first && g >= unsigned(kRing) && g - kRing >= gbase_prev;
            int k_lo, k_hi;
            chunk_range(m, j, k_lo, k_hi);
            if (!pred_prev)
                issue(m, j, g % kRing, k_hi);
            else if (j == 0)
                copy_part(m, 0, g % kRing, k_hi, k_hi);
        }
    };
    // The last warp to release chunk g of step n (local j) refills its slot.
    auto refill = [&](int n, int j, unsigned g) {
        const unsigned slot = g % kRing;
        const int nch = nchunks_of(n);
        const int jj = j + kRing;
        if (jj < nch) {
            int k_lo, k_hi;
            chunk_range(n, jj, k_lo, k_hi);
            issue(n, jj, slot, k_hi);
        } else if (n + 1 <= n1 && jj - nch < nchunks_of(n + 1)) {
            const int j1 = jj - nch;
            int k_lo, k_hi;
            chunk_range(n + 1, j1, k_lo, k_hi);
            issue(n + 1, j1, slot, j1 == 0 ? k_hi - 1 : k_hi);  // slab n comes after the barriers
        }
    };
    // Drain on a failed barrier during step n (gbase already advanced to
    // step n+1): copies of step n+1 issued by refill are completed (chunk
    // 0's newest slab issued too) and waited for.
    auto drain = [&](int n) {
        if (threadIdx.x != 0 || n + 1 > n1) return;
        const int nch1 = nchunks_of(n + 1);
        for (int j = 0; j < kRing && j < nch1; ++j) {
            const unsigned g = gbase + j;
            if (g < unsigned(kRing) || g - kRing < gbase_prev) continue;  // not issued by refill
            int k_lo, k_hi;
            chunk_range(n + 1, j, k_lo, k_hi);
            if (j == 0) copy_part(n + 1, 0, g % kRing, k_hi, k_hi);
            mbar_wait(smem_addr(&full_bar[g % kRing]), (g / kRing) & 1u);
        }
    };
    auto barrier = [&](int n) -> bool {
        if (grid_barrier(count, target, abort, err)) return true;
        drain(n);
        return false;
    };

    for (int n = n0; n <= n1; ++n) {
        // ---------------- trace of step n ----------------
        int I[PPT], Wr[PPT];
        float xi[PPT], dwT[PPT], dwTc[PPT];
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            I[q] = s < N ? s : 0;
            Wr[q] = 0;
            xi[q] = 0.0f;
            dwT[q] = slo[q];
            dwTc[q] = 0.0f;
        }
        const int nchunks = nchunks_of(n);
        if (threadIdx.x == 0 && nchunks > 0) {
            fence_proxy_async_global();
            start_step(n, n == n0);
        }
        if (nchunks > 0) {
            bool ok = true;
            for (int j = 0; j < nchunks; ++j) {
                const unsigned g = gbase + j, slot = g % kRing;
                ok &= mbar_wait(smem_addr(&full_bar[slot]), (g / kRing) & 1u);
                const float *__restrict__ chunk = ring + slot * S * TS;
                int k_lo, k_hi;
                chunk_range(n, j, k_lo, k_hi);
                trace_chunk<PPT, POW2, UNWRAP, 2>(chunk, TS, k_hi, k_lo, N, I, xi, dwT, dwTc, shi, S0m, err, &Wr,
                                                  log2n);
                __syncwarp();
                if (lane == 0 && atom_add_acq_rel_cta(&released[slot], 1u) == unsigned(W - 1)) {
                    released[slot] = 0;
                    fence_proxy_async_shared();
                    refill(n, j, g);
                }
            }
            if (!ok) atomicOr(err, kErrStageTimeout);
        }
        gbase_prev = gbase;
        gbase += nchunks;
        float ds = 0.f, dc = 0.f;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            if (!live[q]) continue;
            const SplitNode nd = nodes[mv[q]];
            float2 cs = __ldg(phase + I[q]);
            if constexpr (UNWRAP) cs = phase_unwrapped(cs, Wr[q] - n * ((nd.S0u - nd.S0) / N), p.phase_wrap[0]);
            two_sum_acc(ds, dc, delta_f0(f, nd, cs, xi[q], (dwT[q] - dwTc[q]) - slo[q]));
        }
        double acc = gsum + (double(ds) + double(dc));
        if (blockDim.x > unsigned(Nr)) {
            if (grp == 1) combine[s] = acc;
            __syncthreads();
            if (grp == 0) acc += combine[s];
        }
        unsigned long long *fix_n = rho_fix + (long long)(n & 1) * N;
        if (grp == 0 && s < N) {
            const double v = acc * fix_scale;
            if (!(fabs(v) < fix_limit)) atomicOr(err, kErrRhoRange);  // outside the host's bound: not expected
            red_global_add_u64(fix_n + s, (unsigned long long)__double2ll_rn(fmin(fmax(v, -fix_limit), fix_limit)));
        }
        if (!barrier(n)) return;

        // ---------------- field solve ----------------
        // rho from the exact integer sums.  rho itself, not rho - mean:
        // every circulant kernel sums to zero (the k = 0 mode is dropped),
        // so the mean only costs a block-wide sum per step; the rounding it
        // would remove is ~1e-13 of the field, far below the FP32-split
        // arithmetic
        const double to_rho = -p.wv / fix_scale;
        for (int j = threadIdx.x; j < N; j += blockDim.x) {
            rs[j] = double((long long)__ldcg(fix_n + j)) * to_rho;
            if (blockIdx.x == 0) {
                rho[j] = rs[j];
                rho_fix[(long long)((n + 1) & 1) * N + j] = 0ull;  // the next step's sums start from zero
            }
        }
        __syncthreads();
        // node slot warp % Kp, part warp / Kp: the slots' part-0 warps (which
        // finish the nodes) sit on different SM sub-partitions
        const int slotn = warp % Kp, pw = warp / Kp;
        double a[5] = {0, 0, 0, 0, 0};
        if (slotn < K) {
            const int node = int(blockIdx.x) + slotn * G;
            const int jlen = (N + wpn - 1) / wpn;
            const int jb = pw * jlen, je = min(N, jb + jlen);
            for (int j = jb + lane; j < je; j += 32) {
                int m = node - j;
                m += m < 0 ? N : 0;
                const double r = rs[j];
#pragma unroll
                for (int c = 0; c < 5; ++c) a[c] = fma(gs[c * N + m], r, a[c]);
            }
        }
        // the five lane sums by a reduce-scatter butterfly (8 FP64 adds per
        // warp instead of five shuffle trees' 25; FP64 issues at 1/64 of
        // the FP32 rate): after it, lanes 4c' hold sum c of lane_sum_of
        const int c_of_lane = lane_sum_of(lane);
        {
            const bool hi16 = lane & 16, hi8 = lane & 8, hi4 = lane & 4;
            // xor 16: the lower half keeps sums 0..2, the upper half 3, 4
            const double k0 = hi16 ? a[3] : a[0], k1 = hi16 ? a[4] : a[1], k2 = hi16 ? 0.0 : a[2];
            const double g0 = hi16 ? a[0] : a[3], g1 = hi16 ? a[1] : a[4], g2 = hi16 ? a[2] : 0.0;
            const double b0 = k0 + __shfl_xor_sync(0xffffffffu, g0, 16);
            const double b1 = k1 + __shfl_xor_sync(0xffffffffu, g1, 16);
            const double b2 = k2 + __shfl_xor_sync(0xffffffffu, g2, 16);
            // xor 8: slots 0, 1 or slot 2
            const double d0 = (hi8 ? b2 : b0) + __shfl_xor_sync(0xffffffffu, hi8 ? b0 : b2, 8);
            const double d1 = (hi8 ? 0.0 : b1) + __shfl_xor_sync(0xffffffffu, hi8 ? b1 : 0.0, 8);
            // xor 4: one slot; then xor 2, xor 1 over the four lanes that share it
            double e = (hi4 ? d1 : d0) + __shfl_xor_sync(0xffffffffu, hi4 ? d0 : d1, 4);
            e += __shfl_xor_sync(0xffffffffu, e, 2);
            e += __shfl_xor_sync(0xffffffffu, e, 1);
            if ((lane & 3) == 0 && c_of_lane >= 0) wacc[slotn * wpn + pw][c_of_lane] = e;
        }
        __syncthreads();
        if (pw == 0 && slotn < K) {  // uniform over the warp
            // lane c < 5: sum c over the node's parts in part order; lane 0 gathers the five
            double vc = 0;
            if (lane < 5) {
                vc = wacc[slotn * wpn][lane];
                for (int w = 1; w < wpn; ++w) vc += wacc[slotn * wpn + w][lane];
            }
            double v[5];
#pragma unroll
            for (int c = 0; c < 5; ++c) v[c] = __shfl_sync(0xffffffffu, vc, c);
            if (lane == 0) {
                const int node = int(blockIdx.x) + slotn * G;
                double *slab = hist + (long long)n * p.hist_stride;
                slab[node] = v[0];
                if (node + N < p.P[0]) slab[node + N] = v[0];
                store_kick_entry(tables + (long long)n * p.table_stride, N, node, float(v[2]), float(v[3]),
                                 float(v[4]));
                epart[(long long)(n - n0) * N + node] = rs[node] * v[1];
            }
        }
        if (!barrier(n)) return;
    }
    // refill issues nothing past step n1: no bulk copy is in flight here.
    // W_n = L/(2N) sum_i rho'_i phi_i for all steps at once, off the
    // per-step critical path: CTA c sums the steps n0 + c + j G, one warp,
    // lanes in fixed stride and a fixed shuffle tree.
    if (warp == 0)
        for (int n = n0 + int(blockIdx.x); n <= n1; n += G) {
            const double *e = epart + (long long)(n - n0) * N;
            double v = 0;
            for (int i = lane; i < N; i += 32) v += __ldcg(e + i);
            for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
            if (lane == 0) energy[n] = v * Lfac;
        }
}

namespace {

template <int PPT>
cudaError_t launch_run_ppt(const Problem &p, const PersistentRun &pr, const SolvePlan &plan, float *tables,
                           double *hist, const SplitNode *nodes, const float2 *phase, double *rho, double *energy,
                           int n0, int n1, unsigned *err, cudaStream_t st)
{
    const bool pow2 = (p.N[0] & (p.N[0] - 1)) == 0;
    void (*fn)(const Problem, float *, double *, const SplitNode *, const float2 *, const double *,
               unsigned long long *, double, double, double *, double *, double *, int, int, int, int, unsigned *,
               unsigned *) = pow2 ? run_split_1d_kernel<PPT, true, false> : run_split_1d_kernel<PPT, false, false>;
    if (phase_wraps(p)) {  // f0's phase at the unwrapped foot (admitted for N a power of two only)
        if (!pow2) return cudaErrorInvalidValue;
        fn = run_split_1d_kernel<PPT, true, true>;
    }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(pr.smem));
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(pr.ctas);
    cfg.blockDim = dim3(pr.threads);
    cfg.dynamicSmemBytes = pr.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaMemsetAsync(pr.sync, 0, 2 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(pr.rho_fix, 0, 2 * size_t(p.N[0]) * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, fn, p, tables, hist, nodes, phase, (const double *)plan.green, pr.rho_fix,
                              pr.fix_scale, pr.fix_limit, rho, energy, pr.epart, n0, n1, pr.slabs_per_chunk,
                              pr.threads / pr.tpn, pr.sync, err);
}

}  // namespace

PersistentRun persistent_shape_1d(const Problem &p, const StagedShape &sh, const SolvePlan &plan, int sms)
{
    PersistentRun pr;
    if (!sh.ok || p.dim != 1 || plan.nconv != 5 || sh.threads > 512 || sh.threads < 32) return pr;
    if (sh.ppt > 4 && sh.threads > 256) return pr;  // launch bounds of the PPT > 4 instances
    const int W = sh.threads / 32;
    const int K = (p.N[0] + sh.ctas - 1) / sh.ctas;  // nodes per CTA in the solve
    // at most two CTAs per SM (cooperative launch: all co-resident)
    if (K > W || sh.ctas > kMaxCtasPerSm * sms) return pr;
    pr.ctas = sh.ctas;
    pr.threads = sh.threads;
    pr.tpn = sh.tpn;
    pr.ppt = sh.ppt;
    pr.slabs_per_chunk = sh.slabs_per_chunk;
    const size_t ring = size_t(kRing) * sh.slabs_per_chunk * size_t(p.table_stride) * sizeof(float);
    pr.smem = std::max(ring + size_t(6) * p.N[0] * sizeof(double), sh.smem);
    if (pr.smem > 220 * 1024) return pr;
    if (!rho_fixed_point(p, sh.ctas, sh.ppt * sh.tpn, pr.fix_scale, pr.fix_limit)) return pr;
    pr.ok = true;
    return pr;
}

bool rho_fixed_point(const Problem &p, int ctas, int chains, double &scale, double &limit)
{
    // A CTA adds, per node, the f~ of its `chains` chains of that node; f~
    // is f0 at a foot, so each is at most max f0 over (x, u).  fmax bounds
    // that with a margin of 2; with `ctas` parts below 2^62 / ctas each, no
    // node's sum leaves int64.
    if (p.dim != 1 || ctas < 1 || chains < 1) return false;
    const double alpha = std::fabs(p.f0p[0]), inv_sqrt_2pi = 0.39894228040143267794;
    double fmax;
    switch (p.f0_kind) {
    case NUFI_F0_LANDAU: fmax = (1 + alpha) * inv_sqrt_2pi; break;                        // max exp(-u^2/2) = 1
    case NUFI_F0_TWO_STREAM: fmax = (1 + alpha) * 2.0 * std::exp(-1.0) * inv_sqrt_2pi; break;  // u^2 e^{-u^2/2} <= 2/e
    case NUFI_F0_BUMP_ON_TAIL: fmax = (1 + alpha) * (0.9 + 0.1 / p.f0p[3]) * inv_sqrt_2pi; break;
    default: return false;
    }
    const double part_max = 2.0 * double(chains) * fmax;
    const int F = std::min(60, int(std::floor(62.0 - std::log2(double(ctas) * part_max))));
    if (!(F >= 24)) return false;  // a bound this loose is not met by any real grid
    scale = std::ldexp(1.0, F);
    limit = std::ldexp(1.0, 62) / double(ctas);
    return true;
}

cudaError_t launch_run_split_1d(const Problem &p, const PersistentRun &pr, const SolvePlan &plan, float *tables,
                                double *hist, const SplitNode *nodes, const float2 *phase, double *rho,
                                double *energy, int n0, int n1, unsigned *err, cudaStream_t st)
{
    switch (pr.ppt) {
#define NUFI_CASE(K) \
    case K: return launch_run_ppt<K>(p, pr, plan, tables, hist, nodes, phase, rho, energy, n0, n1, err, st);
        NUFI_CASE(1) NUFI_CASE(2) NUFI_CASE(3) NUFI_CASE(4) NUFI_CASE(5) NUFI_CASE(6) NUFI_CASE(7) NUFI_CASE(8)
#undef NUFI_CASE
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace nufi_gb300
