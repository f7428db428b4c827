// trace_fp64.cu — FP64 plain form of the backward characteristic trace.
//
// Each thread owns PPT quadrature points with the same spatial node and
// consecutive velocity nodes; a warp spans 32 consecutive spatial nodes
// (x fastest), so at small and moderate n the lanes of a warp locate into
// neighbouring cells and the slab gathers stay coalesced.  The substep loop
// is outermost and the PPT points innermost, which gives PPT independent
// dependency chains per thread.
//
// Per point the arithmetic is the reference's eval_ftilda
// (nufi/rho.hpp:31-61, 191-232, 318-367) with dimN::eval
// (nufi/fields.hpp:36-61, 149-184, 308-350) and the spline kernels
// (nufi/splines.hpp:39-172): drift x -= dt u, periodic wrap
// x - L floor(x/L), knot floor(x/dx), de Boor / tensor contraction, kick
// u += dt E; the first half kick is omitted and the last kick is halved.
// In 2D/3D the components of E come from one gather of the order^d window
// and the shared partial contractions; each component is formed by exactly
// the operations of its own reference eval<> call.
//
// rho is reduced without atomics (the reference uses one atomicAdd per
// point, nufi/cuda_kernel.cu:50): per thread over its PPT points, in fixed
// order per block (write_partial_tiled) and across blocks (reduce_rho), so
// repeated runs are bitwise identical.
#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

// fields.hpp wrap + locate on one axis; the knot is remapped when the wrap
// rounds up to exactly L (the reference would read one value past the
// padded slab there).
__device__ __forceinline__ int locate_fp64(const Problem &p, int a, double x, double &xi, unsigned *err)
{
    x -= p.xmin[a];
    x = x - p.L[a] * floor(x * p.Linv[a]);
    const double xk = floor(x * p.dxinv[a]);
    int ii = int(xk);
    xi = x * p.dxinv[a] - xk;
    if (ii >= p.N[a]) ii -= p.N[a];
    if (ii < 0 || ii >= p.N[a]) {
        atomicOr(err, kErrCellIndex);
        ii = 0;
    }
    return ii;
}

template <int ORDER>
__device__ __forceinline__ void field_1d(const Problem &p, const double *__restrict__ c, const double *x, double *E,
                                         unsigned *err)
{
    double xi;
    const int ii = locate_fp64(p, 0, x[0], xi, err);
    const double factor = 1 * p.dxinv[0];
    if constexpr (ORDER == 4) {
        E[0] = -(factor * deboor4_d1(xi, __ldg(c + ii), __ldg(c + ii + 1), __ldg(c + ii + 2), __ldg(c + ii + 3)));
    } else {
        double w[ORDER];
#pragma unroll
        for (int j = 0; j < ORDER; ++j) w[j] = __ldg(c + ii + j);
        E[0] = -(factor * deboor<double, ORDER, 1>(xi, w));
    }
}

template <int ORDER>
__device__ __forceinline__ void field_2d(const Problem &p, const double *__restrict__ c, const double *x, double *E,
                                         unsigned *err)
{
    double xi, eta;
    const int ii = locate_fp64(p, 0, x[0], xi, err);
    const int jj = locate_fp64(p, 1, x[1], eta, err);
    const int sy = p.P[0];
    const double *__restrict__ w = c + (long long)jj * sy + ii;
    if constexpr (ORDER == 4) {
        // E_x = -dx^-1 sum_j (sum_i w_ji d_i(xi)) b_j(eta), E_y likewise with
        // the roles swapped: one pass over the 16 coefficients
        double bx[4], dx[4], by[4], dy[4];
        cubic_bd_fp64(xi, bx, dx);
        cubic_bd_fp64(eta, by, dy);
        double ex = 0, ey = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double r0 = 0, r1 = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const double v = __ldg(w + j * sy + i);
                r0 = fma(v, bx[i], r0);
                r1 = fma(v, dx[i], r1);
            }
            ex = fma(r1, by[j], ex);
            ey = fma(r0, dy[j], ey);
        }
        E[0] = -(p.dxinv[0] * ex);
        E[1] = -(p.dxinv[1] * ey);
        return;
    }
    double N0[ORDER], N1[ORDER], c0[ORDER], c1[ORDER];
    bspline_basis<double, ORDER, 0>(xi, N0);
    bspline_basis<double, ORDER, 1>(xi, N1);
#pragma unroll
    for (int j = 0; j < ORDER; ++j) {
        c0[j] = 0;
        c1[j] = 0;
#pragma unroll
        for (int i = 0; i < ORDER; ++i) {
            const double v = __ldg(w + j * sy + i);
            c1[j] += v * N1[i];
            c0[j] += v * N0[i];
        }
    }
    const double fx = 1 * p.dxinv[0], fy = 1 * p.dxinv[1];
    E[0] = -(fx * deboor<double, ORDER, 0>(eta, c1));
    E[1] = -(fy * deboor<double, ORDER, 1>(eta, c0));
}

template <int ORDER>
__device__ __forceinline__ void field_3d(const Problem &p, const double *__restrict__ c, const double *x, double *E,
                                         unsigned *err)
{
    double xi, eta, zeta;
    const int ii = locate_fp64(p, 0, x[0], xi, err);
    const int jj = locate_fp64(p, 1, x[1], eta, err);
    const int kk = locate_fp64(p, 2, x[2], zeta, err);
    const int sy = p.P[0], sz = p.P[0] * p.P[1];
    const double *__restrict__ w = c + (long long)kk * sz + (long long)jj * sy + ii;
    if constexpr (ORDER == 4) {
        // one pass over the 64 coefficients: per (k, j) the x-contractions
        // with the value and derivative bases, folded at once into the three
        // components' y-contractions, then the z-contractions per k
        double bx[4], dx[4], by[4], dy[4], bz[4], dz[4];
        cubic_bd_fp64(xi, bx, dx);
        cubic_bd_fp64(eta, by, dy);
        cubic_bd_fp64(zeta, bz, dz);
        double ex = 0, ey = 0, ez = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double sx = 0, s_y = 0, s_z = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                double r0 = 0, r1 = 0;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const double v = __ldg(w + k * sz + j * sy + i);
                    r0 = fma(v, bx[i], r0);
                    r1 = fma(v, dx[i], r1);
                }
                sx = fma(r1, by[j], sx);
                s_y = fma(r0, dy[j], s_y);
                s_z = fma(r0, by[j], s_z);
            }
            ex = fma(sx, bz[k], ex);
            ey = fma(s_y, bz[k], ey);
            ez = fma(s_z, dz[k], ez);
        }
        E[0] = -(p.dxinv[0] * ex);
        E[1] = -(p.dxinv[1] * ey);
        E[2] = -(p.dxinv[2] * ez);
        return;
    }
    double Nx0[ORDER], Nx1[ORDER];
    bspline_basis<double, ORDER, 0>(xi, Nx0);
    bspline_basis<double, ORDER, 1>(xi, Nx1);
    // czy contracted over x with the value basis (E_y, E_z) and with the
    // derivative basis (E_x).
    double czy0[ORDER][ORDER], czy1[ORDER][ORDER];
#pragma unroll
    for (int k = 0; k < ORDER; ++k)
#pragma unroll
        for (int j = 0; j < ORDER; ++j) {
            double a0 = 0, a1 = 0;
#pragma unroll
            for (int i = 0; i < ORDER; ++i) {
                const double v = __ldg(w + k * sz + j * sy + i);
                a1 += v * Nx1[i];
                a0 += v * Nx0[i];
            }
            czy0[k][j] = a0;
            czy1[k][j] = a1;
        }
    double Ny0[ORDER], Ny1[ORDER];
    bspline_basis<double, ORDER, 0>(eta, Ny0);
    bspline_basis<double, ORDER, 1>(eta, Ny1);
    double czx[ORDER], czy[ORDER], czz[ORDER];
#pragma unroll
    for (int k = 0; k < ORDER; ++k) {
        double ax = 0, ay = 0, az = 0;
#pragma unroll
        for (int j = 0; j < ORDER; ++j) {
            ax += czy1[k][j] * Ny0[j];
            ay += czy0[k][j] * Ny1[j];
            az += czy0[k][j] * Ny0[j];
        }
        czx[k] = ax;
        czy[k] = ay;
        czz[k] = az;
    }
    const double fx = 1 * p.dxinv[0], fy = 1 * p.dxinv[1], fz = 1 * p.dxinv[2];
    E[0] = -(fx * deboor<double, ORDER, 0>(zeta, czx));
    E[1] = -(fy * deboor<double, ORDER, 0>(zeta, czy));
    E[2] = -(fz * deboor<double, ORDER, 1>(zeta, czz));
}

template <int D, int ORDER>
__device__ __forceinline__ void field_fp64(const Problem &p, const double *__restrict__ c, const double *x, double *E,
                                           unsigned *err)
{
    if constexpr (D == 1) field_1d<ORDER>(p, c, x, E, err);
    else if constexpr (D == 2) field_2d<ORDER>(p, c, x, E, err);
    else field_3d<ORDER>(p, c, x, E, err);
}

template <int D>
__device__ __forceinline__ double f0_fp64(const Problem &p, const double *x, const double *u)
{
    if constexpr (D == 1) return f0_1d(p, x[0], u[0]);
    else if constexpr (D == 2) return f0_2d(p, x[0], x[1], u[0], u[1]);
    else return f0_3d(p, x[0], x[1], x[2], u[0], u[1], u[2]);
}

}  // namespace

// eval_ftilda (mode 0) or eval_f (mode 1, with the first half kick from
// slab n) of PPT points per thread; see the file comment.
template <int D, int ORDER, int PPT>
__global__ void __launch_bounds__(256) trace_fp64_kernel(const Problem p, const PointGrid g,
                                                         const double *__restrict__ hist, int n, long long q_begin,
                                                         long long q_end, int mode, int vblocks,
                                                         double *__restrict__ partial, unsigned *err)
{
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    const long long s = (long long)blockIdx.x * 32 + lane;
    const double dt = p.dt;
    // metrics of cuda_eval_metrics (nufi/cuda_kernel.cu:53-79, 239-271,
    // 428-466): weight * f, weight * f^2, weight * |u0|^2 f / 2 and
    // -weight f log f, u0 the point's initial velocity; weight du (dx) in
    // 1D, dx dy du dv in 2D, du dv dw in 3D (the reference's 3D kernel
    // leaves out dx dy dz).  The points and the weight come from g (the
    // handle's grid, or the metrics grid); the history and splines from p.
    const double w = g.w;
    double acc = 0;
    double m4[4] = {0, 0, 0, 0};

    // velocity blocks vb = blockIdx.y, blockIdx.y + gridDim.y, ...: one per
    // block unless the velocity grid has more blocks than the grid's y axis
    // holds; each block sums its points in this fixed order
    for (int vb = blockIdx.y; vb < vblocks; vb += gridDim.y) {
        const long long mb = ((long long)vb * W + warp) * PPT;
        double x[PPT][D], u[PPT][D];
        bool live[PPT];
        {
            long long rs = s < g.Ns ? s : 0;
            int is[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < D; ++a) {
                is[a] = int(rs % g.N[a]);
                rs /= g.N[a];
            }
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                const long long m = mb + q;
                const long long qq = s * g.Nm + m;
                live[q] = (s < g.Ns) && (m < g.Nm) && (qq >= q_begin) && (qq < q_end);
                long long rm = m < g.Nm ? m : 0;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    const int im = int(rm % g.M[a]);
                    rm /= g.M[a];
                    x[q][a] = g.xmin[a] + is[a] * g.dx[a];
                    u[q][a] = g.vmin[a] + im * g.dv[a] + g.dv[a] / 2;
                }
            }
        }

        if (n > 0) {
            double E[D];
            if (mode >= 1) {  // eval_f: initial half kick with slab n
                const double *c = hist + (long long)n * p.hist_stride;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    if (!live[q]) continue;
                    field_fp64<D, ORDER>(p, c, x[q], E, err);
#pragma unroll
                    for (int a = 0; a < D; ++a) u[q][a] += 0.5 * dt * E[a];
                }
            }
            for (int k = n - 1; k >= 1; --k) {
                const double *c = hist + (long long)k * p.hist_stride;
#pragma unroll
                for (int q = 0; q < PPT; ++q) {
                    if (!live[q]) continue;
#pragma unroll
                    for (int a = 0; a < D; ++a) x[q][a] = x[q][a] - dt * u[q][a];
                    field_fp64<D, ORDER>(p, c, x[q], E, err);
#pragma unroll
                    for (int a = 0; a < D; ++a) u[q][a] = u[q][a] + dt * E[a];
                }
            }
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                if (!live[q]) continue;
#pragma unroll
                for (int a = 0; a < D; ++a) x[q][a] -= dt * u[q][a];
                field_fp64<D, ORDER>(p, hist, x[q], E, err);
#pragma unroll
                for (int a = 0; a < D; ++a) u[q][a] += 0.5 * dt * E[a];
            }
        }
        if (mode == 2) {
#pragma unroll
            for (int q = 0; q < PPT; ++q) {
                if (!live[q]) continue;
                const double f = f0_fp64<D>(p, x[q], u[q]);
                long long rm = mb + q;
                double uu = 0;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    const double u0 = g.vmin[a] + int(rm % g.M[a]) * g.dv[a] + g.dv[a] / 2;
                    rm /= g.M[a];
                    uu += u0 * u0;
                }
                const double wf = w * f;
                m4[0] += wf;
                m4[1] += wf * f;
                m4[2] += w * (uu * f / 2);
                m4[3] += (f > 0) ? -wf * log(f) : 0.0;
            }
        } else {
#pragma unroll
            for (int q = 0; q < PPT; ++q)
                if (live[q]) acc += f0_fp64<D>(p, x[q], u[q]);
        }
    }
    if (mode == 2) {
        write_metrics_block(m4, partial);
        return;
    }
    write_partial_tiled(acc, s, g.Ns, partial);
}

// Launch table: dims x orders x points-per-thread.
template <int D, int ORDER>
static cudaError_t launch_fp64_order(const Problem &p, const PointGrid &g, const LaunchShape &ls, const double *hist,
                                     int n, long long qb, long long qe, int mode, double *partial, unsigned *err,
                                     cudaStream_t st)
{
    const dim3 block(32, ls.warps);
    const dim3 grid(unsigned((g.Ns + 31) / 32), unsigned(fp64_rows(ls)));
    const int vb = ls.vblocks;
    switch (ls.ppt) {
    case 1: trace_fp64_kernel<D, ORDER, 1><<<grid, block, 0, st>>>(p, g, hist, n, qb, qe, mode, vb, partial, err); break;
    case 2: trace_fp64_kernel<D, ORDER, 2><<<grid, block, 0, st>>>(p, g, hist, n, qb, qe, mode, vb, partial, err); break;
    case 4: trace_fp64_kernel<D, ORDER, 4><<<grid, block, 0, st>>>(p, g, hist, n, qb, qe, mode, vb, partial, err); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_fp64(const Problem &p, const LaunchShape &ls, const double *hist, int n, long long qb,
                              long long qe, int mode, double *partial, int *rows, unsigned *err, cudaStream_t st,
                              const PointGrid *grid)
{
    *rows = fp64_rows(ls);
    const PointGrid g = grid ? *grid : point_grid_of(p);
#define NUFI_CASE(D, O) \
    if (p.dim == D && p.order == O) return launch_fp64_order<D, O>(p, g, ls, hist, n, qb, qe, mode, partial, err, st);
    NUFI_CASE(1, 3) NUFI_CASE(1, 4) NUFI_CASE(1, 5) NUFI_CASE(1, 6) NUFI_CASE(1, 7) NUFI_CASE(1, 8)
    NUFI_CASE(2, 3) NUFI_CASE(2, 4) NUFI_CASE(2, 5) NUFI_CASE(2, 6)
    NUFI_CASE(3, 3) NUFI_CASE(3, 4) NUFI_CASE(3, 5)
#undef NUFI_CASE
    return cudaErrorNotSupported;
}

// f~ (mode 0, eval_ftilda), f (mode 1, eval_f, nufi/rho.hpp:63-96,
// 234-281, 369-426) or the phase flow (mode 2, 1D eval_phase_flow,
// nufi/rho.hpp:98-131: the eval_f trajectory only when n > 1, then x
// wrapped as x - L floor(x / L)) at arbitrary points, one thread per point.
// pts: [npts][2D] (x.., v..); f_out (modes 0, 1) may be null; feet
// (may be null) receives the final (x.., v..).
template <int D, int ORDER>
__global__ void eval_points_kernel(const Problem p, const double *__restrict__ hist, int n, int mode, long long npts,
                                   const double *__restrict__ pts, double *__restrict__ f_out,
                                   double *__restrict__ feet, unsigned *err)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    double x[D], u[D], E[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        x[a] = pts[i * 2 * D + a];
        u[a] = pts[i * 2 * D + D + a];
    }
    const double dt = p.dt;
    const bool trace = mode == 2 ? n > 1 : n > 0;
    if (trace) {
        int k = n;
        if (mode >= 1) {
            field_fp64<D, ORDER>(p, hist + (long long)n * p.hist_stride, x, E, err);
#pragma unroll
            for (int a = 0; a < D; ++a) u[a] += 0.5 * dt * E[a];
        }
        while (--k) {
#pragma unroll
            for (int a = 0; a < D; ++a) x[a] = x[a] - dt * u[a];
            field_fp64<D, ORDER>(p, hist + (long long)k * p.hist_stride, x, E, err);
#pragma unroll
            for (int a = 0; a < D; ++a) u[a] = u[a] + dt * E[a];
        }
#pragma unroll
        for (int a = 0; a < D; ++a) x[a] -= dt * u[a];
        field_fp64<D, ORDER>(p, hist, x, E, err);
#pragma unroll
        for (int a = 0; a < D; ++a) u[a] += 0.5 * dt * E[a];
    }
    if (mode == 2) {
#pragma unroll
        for (int a = 0; a < D; ++a) x[a] = x[a] - p.L[a] * floor(x[a] * p.Linv[a]);
    } else if (f_out) {
        f_out[i] = f0_fp64<D>(p, x, u);
    }
    if (feet)
#pragma unroll
        for (int a = 0; a < D; ++a) {
            feet[i * 2 * D + a] = x[a];
            feet[i * 2 * D + D + a] = u[a];
        }
}

cudaError_t launch_eval_points(const Problem &p, const double *hist, int n, int mode, long long npts,
                               const double *pts, double *f_out, double *feet, unsigned *err, cudaStream_t st)
{
    const unsigned blocks = unsigned((npts + 127) / 128);
#define NUFI_CASE(D, O)                                                                                       \
    if (p.dim == D && p.order == O) {                                                                        \
        eval_points_kernel<D, O><<<blocks, 128, 0, st>>>(p, hist, n, mode, npts, pts, f_out, feet, err); \
        return cudaGetLastError();                                                                           \
    }
    NUFI_CASE(1, 3) NUFI_CASE(1, 4) NUFI_CASE(1, 5) NUFI_CASE(1, 6) NUFI_CASE(1, 7) NUFI_CASE(1, 8)
    NUFI_CASE(2, 3) NUFI_CASE(2, 4) NUFI_CASE(2, 5) NUFI_CASE(2, 6)
    NUFI_CASE(3, 3) NUFI_CASE(3, 4) NUFI_CASE(3, 5)
#undef NUFI_CASE
    return cudaErrorNotSupported;
}

bool fp64_order_supported(int dim, int order)
{
    if (dim == 1) return order >= 3 && order <= 8;
    if (dim == 2) return order >= 3 && order <= 6;
    if (dim == 3) return order >= 3 && order <= 5;
    return false;
}

}  // namespace nufi_gb300
