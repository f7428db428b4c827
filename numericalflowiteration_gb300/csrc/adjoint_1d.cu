// adjoint_1d.cu — reverse-mode gradient of the time-integrated field energy
//     J = 2 dt sum_{n=0}^{n1} W_n     (W_n = 1/2 int |E_n|^2 dx, the energy
//                                      poisson::solve returns at step n)
// with respect to the initial-condition parameters theta = (alpha, k, u_b,
// sigma_b) of f0 (1D1V, FP64).  The forward pass is the ordinary run; its
// coefficient history c_0..c_n1 is the only checkpoint.
//
// Forward, per step n: rho_n(s) = -w sum_j f0(foot_n(s, j); theta), the
// foot from the backward trace through c_{n-1}..c_0 (nufi/rho.hpp:31-61);
// c_n = G_c (rho_n - mean) and W_n = L/(2N) sum_i rho'_i phi_i, phi the
// potential at the nodes (field_solve.cu).  Reverse, for m = n1 .. 0:
//   lambda_m = dJ/drho_m = 2 dt L/N phi_m + G_c^T fold(mu_m)
// (mu_m = dJ/dc_m, complete once every step after m has been reversed;
// fold adds the periodic padding copies; G_c^T is the circulant with the
// reversed kernel; phi_m = sum_j N_j(0) c_m[i+j] from the stored slab).
// Then every point of step m is traced to its foot again, seeded with
// a = -w lambda_m(s):  xbar = a df0/dx, ubar = a df0/du, thetabar += a
// df0/dtheta, and walked forward in time through the substeps k = 0 ..
// m-1, each inverted exactly (Stormer-Verlet is reversible):
//   substep k (forward):  x' = x - dt u,  u' = u + h_k dt E_k(x')
//   adjoint:  xbar <- xbar + ubar h_k dt E_k'(x');  ubar <- ubar - dt xbar
//             mu_k[i + j] += ubar' h_k dt (-1/dx) N'_j(xi)
//   inverse:  u = u' - h_k dt E_k(x');  x = x' + dt u
// (h_k = 1/2 for k = 0, else 1).  mu contributions are summed per block in
// shared memory (FP64 atomics), a chunk of slabs at a time, then added to
// the global mu (FP64 atomics: the order of those additions is not fixed,
// so the gradient varies in the last bits from run to run).
#include <algorithm>

#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

struct F0Grad {
    double fx, fu, dth[4];
};

// Partial derivatives of the 1D initial conditions (nufi/config.hpp:82-83;
// the bump-on-tail of the batched configuration) at the foot (x unwrapped,
// as the reference evaluates f0 there).
__device__ __forceinline__ F0Grad f0_grad_1d(const Problem &p, double x, double u)
{
    const double alpha = p.f0p[0], k = p.f0p[1];
    const double c0 = 0.39894228040143267793994;
    double sk, ck;
    sincos(k * x, &sk, &ck);
    const double sp = 1. + alpha * ck;
    double g, gu, gub = 0, gsb = 0;
    if (p.f0_kind == NUFI_F0_LANDAU) {
        const double e = c0 * exp(-u * u / 2);
        g = e;
        gu = -u * e;
    } else if (p.f0_kind == NUFI_F0_TWO_STREAM) {
        const double e = c0 * exp(-u * u / 2.);
        g = e * u * u;
        gu = e * u * (2. - u * u);
    } else {
        const double ubv = p.f0p[2], sb = p.f0p[3];
        const double z = (u - ubv) / sb;
        const double e1 = c0 * exp(-u * u / 2), e2 = c0 / sb * exp(-z * z / 2);
        g = 0.9 * e1 + 0.1 * e2;
        gu = -0.9 * u * e1 - 0.1 * z / sb * e2;
        gub = 0.1 * z / sb * e2;
        gsb = 0.1 * (z * z - 1.) / sb * e2;
    }
    F0Grad r;
    r.fx = -alpha * k * sk * g;
    r.fu = sp * gu;
    r.dth[0] = ck * g;
    r.dth[1] = -alpha * x * sk * g;
    r.dth[2] = sp * gub;
    r.dth[3] = sp * gsb;
    return r;
}

// fields.hpp wrap + knot (as trace_fp64.cu's locate_fp64).
__device__ __forceinline__ int locate_adj(const Problem &p, double x, double &xi, unsigned *err)
{
    x -= p.xmin[0];
    x = x - p.L[0] * floor(x * p.Linv[0]);
    const double xk = floor(x * p.dxinv[0]);
    int ii = int(xk);
    xi = x * p.dxinv[0] - xk;
    if (ii >= p.N[0]) ii -= p.N[0];
    if (ii < 0 || ii >= p.N[0]) {
        atomicOr(err, kErrCellIndex);
        ii = 0;
    }
    return ii;
}

// E = -dS/dx at x with the primal's arithmetic (trace_fp64.cu field_1d).
template <int ORDER>
__device__ __forceinline__ double efield_primal(const Problem &p, const double *__restrict__ c, double x, unsigned *err)
{
    double xi;
    const int ii = locate_adj(p, x, xi, err);
    double w[ORDER];
#pragma unroll
    for (int j = 0; j < ORDER; ++j) w[j] = __ldg(c + ii + j);
    return -((1 * p.dxinv[0]) * deboor<double, ORDER, 1>(xi, w));
}

}  // namespace

// Per step m: rebuild the feet, seed, reverse through slabs 0..m-1.
// Block (T threads = spatial nodes blockIdx.x*T + t), PPT velocity nodes
// per thread from blockIdx.y*PPT.  theta_acc[i*blocks + block] += this
// block's share of dJ/dtheta_i (a fixed slot per block: deterministic).
template <int ORDER, int PPT>
__global__ void __launch_bounds__(256) adjoint_trace_1d_kernel(const Problem p, const double *__restrict__ hist,
                                                               const double *__restrict__ lambda, int m, int chunk,
                                                               double *__restrict__ mu, double *__restrict__ theta_acc,
                                                               unsigned *err)
{
    extern __shared__ double mu_s[];  // [chunk][P]
    __shared__ double red[4][8];
    const int P = p.P[0], N = p.N[0];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const long long mb = (long long)blockIdx.y * PPT;
    const double dt = p.dt, dxinv = p.dxinv[0];
    const long long hs = p.hist_stride;

    for (int i = threadIdx.x; i < chunk * P; i += blockDim.x) mu_s[i] = 0;

    double x[PPT], u[PPT], xb[PPT], ub[PPT];
    bool live[PPT];
    const double a = s < N ? -p.wv * lambda[s] : 0.0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long jm = mb + q;
        live[q] = s < N && jm < p.Nm;
        x[q] = p.xmin[0] + (s < N ? s : 0) * p.dx[0];
        u[q] = p.vmin[0] + (jm < p.Nm ? jm : 0) * p.dv[0] + p.dv[0] / 2;
    }
    // 1. the primal trace to the foot (eval_ftilda, same operations)
    for (int k = m - 1; k >= 1; --k) {
        const double *c = hist + k * hs;
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            if (!live[q]) continue;
            x[q] = x[q] - dt * u[q];
            u[q] = u[q] + dt * efield_primal<ORDER>(p, c, x[q], err);
        }
    }
    if (m > 0) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            if (!live[q]) continue;
            x[q] -= dt * u[q];
            u[q] += 0.5 * dt * efield_primal<ORDER>(p, hist, x[q], err);
        }
    }
    // 2. seed at the foot
    double th[4] = {0, 0, 0, 0};
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        xb[q] = 0;
        ub[q] = 0;
        if (!live[q]) continue;
        const F0Grad g = f0_grad_1d(p, x[q], u[q]);
        xb[q] = a * g.fx;
        ub[q] = a * g.fu;
#pragma unroll
        for (int i = 0; i < 4; ++i) th[i] += a * g.dth[i];
    }
    __syncthreads();
    // 3. reverse sweep, slabs 0..m-1 in chunks staged in shared memory
    for (int k0 = 0; k0 < m; k0 += chunk) {
        const int k1 = min(m, k0 + chunk);
        for (int k = k0; k < k1; ++k) {
            const double h = k == 0 ? 0.5 : 1.0;
            const double *c = hist + k * hs;
            double *ms = mu_s + (k - k0) * P;
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                if (!live[q]) continue;
                double xi;
                const int ii = locate_adj(p, x[q], xi, err);
                double N1[ORDER], N2[ORDER];
                bspline_basis<double, ORDER, 1>(xi, N1);
                bspline_basis<double, ORDER, 2>(xi, N2);
                double s1 = 0, s2 = 0;
#pragma unroll
                for (int j = 0; j < ORDER; ++j) {
                    const double w = __ldg(c + ii + j);
                    s1 = fma(w, N1[j], s1);
                    s2 = fma(w, N2[j], s2);
                }
                const double E = -dxinv * s1;
                const double Ep = -dxinv * dxinv * s2;
                const double coef = ub[q] * h * dt * (-dxinv);
#pragma unroll
                for (int j = 0; j < ORDER; ++j) atomicAdd(ms + ii + j, coef * N1[j]);
                const double xt = xb[q] + ub[q] * h * dt * Ep;
                xb[q] = xt;
                ub[q] = ub[q] - dt * xt;
                u[q] = u[q] - h * dt * E;
                x[q] = x[q] + dt * u[q];
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < (k1 - k0) * P; i += blockDim.x) {
            const double v = mu_s[i];
            if (v != 0) {
                atomicAdd(mu + (long long)(k0 + i / P) * P + i % P, v);
                mu_s[i] = 0;
            }
        }
        __syncthreads();
    }
    // 4. this block's dJ/dtheta (fixed-order shuffle tree, warps in order)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double v = th[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[i][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = red[threadIdx.x][0];
        for (int w = 1; w < int(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        const long long blocks = (long long)gridDim.x * gridDim.y;
        theta_acc[threadIdx.x * blocks + (long long)blockIdx.y * gridDim.x + blockIdx.x] += t;
    }
}

// lambda_m = scale * phi_m + G_c^T fold(mu_m), one thread per node.
template <int ORDER>
__global__ void adjoint_lambda_1d_kernel(const Problem p, const double *__restrict__ slab,
                                         const double *__restrict__ mu_m, const double *__restrict__ gc, double scale,
                                         double *__restrict__ lambda)
{
    extern __shared__ double mt[];  // fold(mu_m) [N]
    const int N = p.N[0], P = p.P[0];
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double v = mu_m[i];
        for (int q = i + N; q < P; q += N) v += mu_m[q];
        mt[i] = v;
    }
    __syncthreads();
    double b[ORDER];
    bspline_basis<double, ORDER, 0>(0.0, b);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double phi = 0;
#pragma unroll
        for (int j = 0; j < ORDER; ++j) phi += b[j] * slab[i + j];
        double t = 0;
        for (int j = 0; j < N; ++j) {
            int d = j - i;
            d += d < 0 ? N : 0;
            t = fma(gc[d], mt[j], t);
        }
        lambda[i] = scale * phi + t;
    }
}

namespace {

template <int ORDER>
cudaError_t launch_adjoint_order(const Problem &p, const AdjointPlan &ap, const double *hist, const double *gc,
                                 double *mu, double *lambda, double *theta_acc, int n1, unsigned *err,
                                 cudaStream_t st)
{
    const int N = p.N[0], P = p.P[0];
    const double scale = 2.0 * p.dt * p.L[0] / N;
    const dim3 block(ap.threads), grid(ap.grid_x, ap.grid_y);
    const size_t smem = size_t(ap.chunk) * P * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(adjoint_trace_1d_kernel<ORDER, kAdjointPPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    for (int m = n1; m >= 0; --m) {
        const int lb = (N + 255) / 256;
        adjoint_lambda_1d_kernel<ORDER><<<lb, 256, N * sizeof(double), st>>>(p, hist + m * p.hist_stride,
                                                                          mu + (long long)m * P, gc, scale, lambda);
        adjoint_trace_1d_kernel<ORDER, kAdjointPPT><<<grid, block, smem, st>>>(p, hist, lambda, m, ap.chunk, mu,
                                                                              theta_acc, err);
    }
    return cudaGetLastError();
}

}  // namespace

AdjointPlan adjoint_plan_1d(const Problem &p)
{
    AdjointPlan ap;
    // odd-degree splines only: phi_m = B c_m recovers the potential from the
    // stored slab when the collocation matrix B is invertible (orders 4, 6)
    if (p.dim != 1 || (p.order != 4 && p.order != 6)) return ap;
    const int N = p.N[0], P = p.P[0];
    ap.threads = std::min(256, (N + 31) / 32 * 32);
    ap.grid_x = (N + ap.threads - 1) / ap.threads;
    ap.grid_y = int((p.Nm + kAdjointPPT - 1) / kAdjointPPT);
    ap.chunk = int(std::max<long long>(1, std::min<long long>(16, (40 * 1024) / (8LL * P))));
    ap.ok = N <= 16384;
    return ap;
}

cudaError_t launch_adjoint_1d(const Problem &p, const AdjointPlan &ap, const double *hist, const double *gc,
                              double *mu, double *lambda, double *theta_acc, int n1, unsigned *err, cudaStream_t st)
{
    switch (p.order) {
    case 4: return launch_adjoint_order<4>(p, ap, hist, gc, mu, lambda, theta_acc, n1, err, st);
    case 6: return launch_adjoint_order<6>(p, ap, hist, gc, mu, lambda, theta_acc, n1, err, st);
    default: return cudaErrorNotSupported;
    }
}

}  // namespace nufi_gb300
