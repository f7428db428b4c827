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

#include "adjoint_device.cuh"

namespace nufi_gb300 {

using namespace adj;

// Per step m: rebuild the feet, seed, reverse through slabs 0..m-1.
// Block (T threads = spatial nodes blockIdx.x*T + t), PPT velocity nodes
// per thread from blockIdx.y*PPT.  theta_acc[i*blocks + block] += this
// block's share of dJ/dtheta_i (a fixed slot per block: deterministic).
template <int ORDER, int PPT>
__global__ void __launch_bounds__(256, 1) adjoint_trace_1d_kernel(const Problem p, const double *__restrict__ hist,
                                                               const double *__restrict__ lambda, int m, int chunk,
                                                               double *__restrict__ mu, double *__restrict__ theta_acc,
                                                               unsigned *err)
{
    extern __shared__ double mu_s[];  // [chunk][P]
    const int N = p.N[0];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const long long mb = (long long)blockIdx.y * PPT;
    double x[PPT], u[PPT];
    bool live[PPT];
    const double a = s < N ? -p.wv * lambda[s] : 0.0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long jm = mb + q;
        live[q] = s < N && jm < p.Nm;
        x[q] = p.xmin[0] + (s < N ? s : 0) * p.dx[0];
        u[q] = p.vmin[0] + (jm < p.Nm ? jm : 0) * p.dv[0] + p.dv[0] / 2;
    }
    double th[4] = {0, 0, 0, 0};
    adjoint_chains<ORDER, PPT>(p, hist, m, chunk, a, x, u, live, mu_s, mu, th, err);
    const long long blocks = (long long)gridDim.x * gridDim.y;
    block_theta_add(th, theta_acc, blocks, (long long)blockIdx.y * gridDim.x + blockIdx.x);
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
