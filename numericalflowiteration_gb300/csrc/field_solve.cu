// field_solve.cu — periodic Poisson solve fused with the B-spline
// collocation solve, as one diagonal in Fourier space, plus the small
// kernels around it (FP32 field tables).
//
// The reference (a) transforms rho with FFTW's separable DHT, scales mode
// k by 1/(N |k|^2), zeroes the mean and transforms back
// (nufi/poisson.cpp:66-89, 190-219, 328-362), returning
// W = prod L / 2 * sum_{k != 0} |k|^2 phi_k^2; then (b) solves the circulant
// collocation system sum_j N_j(0) c[(i+j) mod N] = phi_i by LSMR
// (nufi/fields.hpp:63-142, 186-300, 352-490) and writes the periodically
// padded slab c[i] = c~[i mod N].  Because the Poisson scaling depends only
// on the folded |k| per axis, the DHT sandwich equals a DFT sandwich, and
// the collocation matrix is circulant with symbol
// lambda(k) = prod_a sum_j N_j(0) exp(+2 pi i j k_a / N_a).  So
//     c^(k) = rho^(k) / (N_tot |k|^2 lambda(k)),  c^(0) = 0,
//     W     = prod L / 2 * sum_{k != 0} |rho^(k)|^2 / (N_tot^2 |k|^2)
// with rho^ the unnormalised DFT.  Everything here is FP64.
//
// One block does the whole solve in shared memory (N_tot <= 8192 complex
// values): radix-2 FFTs along each axis, then the diagonal, then the
// inverse.  FP64 throughput is low on this part, but the solve is
// O(N log N) per time step against O(N_points * n) for the trace.
#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-place radix-2 FFT of every line along axis a (length N = 2^lg,
// element stride S) of the N_tot-element array z.  sign = -1 forward
// (twiddles as stored), +1 inverse (conjugated twiddles).
__device__ void fft_axis(double2 *z, long long ntot, int N, int lg, long long S, const double2 *__restrict__ tw,
                         bool inverse)
{
    if (N <= 1) return;
    const long long lines = ntot / N;
    // bit reversal along the axis
    for (long long e = threadIdx.x; e < ntot; e += blockDim.x) {
        const long long line = e / N;
        const int i = int(e % N);
        const int r = int(__brev(unsigned(i)) >> (32 - lg));
        if (i < r) {
            const long long base = (line / S) * (S * N) + (line % S);
            const long long a = base + (long long)i * S, b = base + (long long)r * S;
            const double2 t = z[a];
            z[a] = z[b];
            z[b] = t;
        }
    }
    __syncthreads();
    const long long nb = lines * (N / 2);
    for (int len = 2; len <= N; len <<= 1) {
        const int half = len >> 1, step = N / len;
        for (long long b = threadIdx.x; b < nb; b += blockDim.x) {
            const long long line = b / (N / 2);
            const int j = int(b % (N / 2));
            const int pos = j % half;
            const int i0 = (j / half) * len + pos;
            const long long base = (line / S) * (S * N) + (line % S);
            const long long e0 = base + (long long)i0 * S, e1 = e0 + (long long)half * S;
            double2 w = tw[pos * step];
            if (inverse) w.y = -w.y;
            const double2 a = z[e0];
            const double2 t = cmul(z[e1], w);
            z[e0] = make_double2(a.x + t.x, a.y + t.y);
            z[e1] = make_double2(a.x - t.x, a.y - t.y);
        }
        __syncthreads();
    }
}

// K (A, B, C) of cell i from c[i..i+3]: the derivative of the cubic
// B-spline sum on [i, i+1) as a quadratic in xi, times K = -dt^2/dx^2.
__device__ __forceinline__ float4 cubic_kick_poly(double c0, double c1, double c2, double c3, double K)
{
    const double A = (c2 - c0) * 0.5;
    const double B = (c0 - 2.0 * c1) + c2;
    const double C = ((3.0 * (c1 - c2) - c0) + c3) * 0.5;
    return make_float4(float(K * A), float(K * B), float(K * C), 0.0f);
}

}  // namespace

struct SolveArgs {
    const double2 *tw[3];
    const double2 *isym[3];
    const double *ksq[3];
    int lg[3];
};

__global__ void __launch_bounds__(1024) field_solve_kernel(const Problem p, const SolveArgs a,
                                                           const double *__restrict__ rho, double *__restrict__ slab,
                                                           float *__restrict__ table, double *__restrict__ energy_out,
                                                           unsigned *err)
{
    extern __shared__ double2 z[];
    __shared__ double red[1024];
    const long long ntot = p.Ns;
    // 1. rho (written by the trace kernel, or copied in by the caller)
    for (long long s = threadIdx.x; s < ntot; s += blockDim.x) z[s] = make_double2(rho[s], 0.0);
    __syncthreads();
    // 2. forward DFT, axis by axis (x fastest)
    long long S = 1;
    for (int ax = 0; ax < p.dim; ++ax) {
        fft_axis(z, ntot, p.N[ax], a.lg[ax], S, a.tw[ax], false);
        S *= p.N[ax];
    }
    // 3. diagonal + energy
    double e = 0;
    const double inv_ntot = 1.0 / double(ntot);
    for (long long s = threadIdx.x; s < ntot; s += blockDim.x) {
        if (s == 0) {
            z[0] = make_double2(0.0, 0.0);
            continue;
        }
        long long r = s;
        double ksq = 0;
        double2 is = make_double2(1.0, 0.0);
        for (int ax = 0; ax < p.dim; ++ax) {
            const int k = int(r % p.N[ax]);
            r /= p.N[ax];
            ksq += a.ksq[ax][k];
            is = cmul(is, a.isym[ax][k]);
        }
        const double2 F = z[s];
        e += (F.x * F.x + F.y * F.y) / ksq;
        const double scale = inv_ntot / ksq;
        const double2 c = cmul(F, is);
        z[s] = make_double2(c.x * scale, c.y * scale);
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    // 4. inverse DFT
    S = 1;
    for (int ax = 0; ax < p.dim; ++ax) {
        fft_axis(z, ntot, p.N[ax], a.lg[ax], S, a.tw[ax], true);
        S *= p.N[ax];
    }
    // 5. padded slab (reference layout) and the FP32 field table
    const long long P0 = p.P[0], P1 = p.P[1], P2 = p.P[2];
    const long long npad = P0 * P1 * P2;
    for (long long idx = threadIdx.x; idx < npad; idx += blockDim.x) {
        const long long i = idx % P0, j = (idx / P0) % P1, k = idx / (P0 * P1);
        const long long src = ((k % p.N[2]) * p.N[1] + (j % p.N[1])) * p.N[0] + (i % p.N[0]);
        const double c = z[src].x;
        slab[idx] = c;
        if (table && p.dim > 1) table[idx] = float(c);
    }
    if (table && p.dim == 1) {
        const int N = p.N[0];
        const double K = -p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
        float4 *t4 = reinterpret_cast<float4 *>(table);
        for (int i = threadIdx.x; i < N; i += blockDim.x)
            t4[i] = cubic_kick_poly(z[i].x, z[(i + 1) % N].x, z[(i + 2) % N].x, z[(i + 3) % N].x, K);
    }
    if (threadIdx.x == 0 && energy_out) {
        double Lp = 1;
        for (int ax = 0; ax < p.dim; ++ax) Lp *= p.L[ax];
        energy_out[0] = red[0] * inv_ntot * inv_ntot * (Lp / 2);
    }
}

cudaError_t launch_field_solve(const Problem &p, const SolvePlan &plan, const double *rho, double *hist_slab,
                               float *table_slab, double *energy_out, unsigned *err, cudaStream_t st)
{
    SolveArgs a;
    for (int i = 0; i < 3; ++i) {
        a.tw[i] = plan.tw[i];
        a.isym[i] = plan.isym[i];
        a.ksq[i] = plan.ksq[i];
        a.lg[i] = plan.log2n[i];
    }
    field_solve_kernel<<<1, 1024, plan.smem, st>>>(p, a, rho, hist_slab, table_slab, energy_out, err);
    return cudaGetLastError();
}

__global__ void derive_table_kernel(const Problem p, const double *__restrict__ slab, float *__restrict__ table)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p.dim == 1) {
        if (idx >= p.N[0]) return;
        const double K = -p.dt * p.dt * p.dxinv[0] * p.dxinv[0];
        reinterpret_cast<float4 *>(table)[idx] =
            cubic_kick_poly(slab[idx], slab[idx + 1], slab[idx + 2], slab[idx + 3], K);
    } else {
        if (idx >= p.stride_t) return;
        table[idx] = float(slab[idx]);
    }
}

cudaError_t launch_derive_table(const Problem &p, const double *hist_slab, float *table_slab, cudaStream_t st)
{
    const long long n = p.dim == 1 ? p.N[0] : p.stride_t;
    derive_table_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(p, hist_slab, table_slab);
    return cudaGetLastError();
}

}  // namespace nufi_gb300

namespace nufi_gb300 {
cudaError_t field_solve_set_smem(size_t smem)
{
    return cudaFuncSetAttribute(field_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
}
}  // namespace nufi_gb300
