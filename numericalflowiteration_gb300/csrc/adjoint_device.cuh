// adjoint_device.cuh — device pieces of the 1D FP64 adjoint shared by the
// single-handle and the batched kernels (adjoint_1d.cu, batch_1d.cu).  The
// mathematics is stated at the top of adjoint_1d.cu.
#pragma once

#include "nufi_kernels.cuh"

namespace nufi_gb300 {
namespace adj {

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
    if constexpr (ORDER == 4) {
        return -((1 * p.dxinv[0]) *
                 deboor4_d1(xi, __ldg(c + ii), __ldg(c + ii + 1), __ldg(c + ii + 2), __ldg(c + ii + 3)));
    } else {
        double w[ORDER];
#pragma unroll
        for (int j = 0; j < ORDER; ++j) w[j] = __ldg(c + ii + j);
        return -((1 * p.dxinv[0]) * deboor<double, ORDER, 1>(xi, w));
    }
}

// Phases of one block's points for step m: (1) the primal trace to the
// foot with the primal's operations, (2) the seed a * grad f0 (a = -w
// lambda_m at the thread's node), (3) the reverse sweep through slabs
// 0..m-1, slab adjoints summed in shared memory (mu_s, chunk x P doubles,
// zeroed here) and added to mu (slab k at mu + k*P).  th += a * df0/dtheta.
// Every thread of the block calls it (it holds __syncthreads).
template <int ORDER, int PPT>
__device__ __forceinline__ void adjoint_chains(const Problem &p, const double *__restrict__ hist, int m, int chunk,
                                               double a, double (&x)[PPT], double (&u)[PPT],
                                               const bool (&live)[PPT], double *mu_s, double *__restrict__ mu,
                                               double (&th)[4], unsigned *err)
{
    const int P = p.P[0];
    const double dt = p.dt, dxinv = p.dxinv[0];
    const long long hs = p.hist_stride;
    double xb[PPT], ub[PPT];
    for (int i = threadIdx.x; i < chunk * P; i += blockDim.x) mu_s[i] = 0;
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
            if constexpr (ORDER == 4) {
                // The cubic spline's derivatives from the window's first
                // differences D_j = w_{j+1} - w_j and the quadratic B-spline
                // values B0 = (1-xi)^2/2, B2 = xi^2/2, B1 = 1 - B0 - B2:
                //   S'  = D0 B0 + D1 B1 + D2 B2
                //   S'' = (D1 - D0) + xi ((D2 - D1) - (D1 - D0))
                //   dS'/dw = (-B0, B0 - B1, B1 - B2, B2)
                // (per cell, times dx^-1 and dx^-2); the same mathematics
                // as the basis loops below in fewer FP64 operations.
                const double hdt = h * dt, cscale = hdt * -dxinv;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    if (!live[q]) continue;
                    double xi;
                    const int ii = locate_adj(p, x[q], xi, err);
                    const double w0 = __ldg(c + ii), w1 = __ldg(c + ii + 1), w2 = __ldg(c + ii + 2),
                                 w3 = __ldg(c + ii + 3);
                    const double D0 = w1 - w0, D1 = w2 - w1, D2 = w3 - w2;
                    const double om = 1.0 - xi;
                    const double B0 = 0.5 * (om * om), B2 = 0.5 * (xi * xi), B1 = (1.0 - B0) - B2;
                    const double s1 = D0 * B0 + D1 * B1 + D2 * B2;
                    const double Da = D1 - D0, s2 = Da + xi * ((D2 - D1) - Da);
                    const double E = -dxinv * s1;
                    const double Ep = -dxinv * dxinv * s2;
                    const double coef = ub[q] * cscale;
                    const double g0 = coef * B0, g1 = coef * B1, g2 = coef * B2;
                    atomicAdd(ms + ii, -g0);
                    atomicAdd(ms + ii + 1, g0 - g1);
                    atomicAdd(ms + ii + 2, g1 - g2);
                    atomicAdd(ms + ii + 3, g2);
                    const double xt = xb[q] + ub[q] * hdt * Ep;
                    xb[q] = xt;
                    ub[q] = ub[q] - dt * xt;
                    u[q] = u[q] - hdt * E;
                    x[q] = x[q] + dt * u[q];
                }
            } else {
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
}

// Adds a block's four dJ/dtheta sums (fixed-order shuffle tree, warps in
// order) to theta_acc[i * slots + slot].
__device__ __forceinline__ void block_theta_add(const double (&th)[4], double *theta_acc, long long slots,
                                                long long slot)
{
    __shared__ double red[4][32];
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
        theta_acc[threadIdx.x * slots + slot] += t;
    }
}

}  // namespace adj
}  // namespace nufi_gb300
