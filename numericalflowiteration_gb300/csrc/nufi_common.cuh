// nufi_common.cuh — device-side problem descriptor and the B-spline
// arithmetic shared by the trace and field-solve kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nufi_gb300.h"

namespace nufi_gb300 {

constexpr int kMaxOrder = 8;
constexpr int kMaxVelocityTable = 4096;  // per-axis velocity nodes kept in tables
constexpr long long kMaxSteps = 1LL << 30;  // time steps per run (kernels take 32-bit step indices)
constexpr long long kMaxEvalPoints = 1LL << 36;  // points per nufi_eval_points call

// Bits of the device error word (checked by the host after each blocking
// call).  Kernels set a bit and skip the offending access; they never trap.
enum : unsigned {
    kErrCellIndex = 1u << 0,   // a located cell fell outside [0, N)
    kErrKickRange = 1u << 1,   // split mode: per-substep kick displacement too large
    kErrSolveSize = 1u << 2,   // field solve: grid larger than its shared-memory plan
    kErrStageTimeout = 1u << 3, // a bounded wait on a shared-memory staging barrier gave up
    kErrBarrierTimeout = 1u << 4, // a bounded wait on the persistent kernel's grid barrier gave up
    kErrAdjointRange = 1u << 5,   // FP32-split adjoint: a fixed-point table-adjoint sum left its range
    kErrRhoRange = 1u << 6,       // 1D split traces: a fixed-point part of rho left its range
};

// Everything a kernel needs to know about one configuration, by value.
// Mirrors the reference's config_t (nufi/config.hpp:33-53, 91-114, 167-193)
// with the derived quantities computed the same way (config.hpp:67-69).
struct Problem {
    int dim, order, f0_kind, precision;
    int N[3];            // spatial nodes per axis (1 when unused)
    int M[3];            // velocity nodes per axis (1 when unused)
    int P[3];            // padded slab extents N + order - 1 (1 when unused)
    long long Ns, Nm, Nq;
    long long stride_t;  // values per slab, reference layout
    long long hist_stride;  // doubles between slabs in the device FP64 history
    long long table_stride; // floats between slabs in the device FP32 tables
    int table_sx;           // 2D/3D FP32 table: floats per x row (>= P[0], see make_problem)
    int row_step;           // 2D/3D split trace with N[0] < 32: the 32 / N[0] x rows a warp
                            // spans are row_step rows apart (0: consecutive rows)
    double dt;
    double xmin[3], L[3], Linv[3], dx[3], dxinv[3];
    double vmin[3], dv[3];
    double f0p[8];
    double wv;           // prod_d dv_d, the quadrature weight of rho
    int split_plain_kick;  // split mode: 1 = uncompensated FP32 kick sum
                           // (nufi_options.split_plain_kick; for measuring
                           // what the compensation buys)
    double phase_wrap[3];  // split: k L_a reduced to [0, 2 pi), the phase f0 gains per wrap of the
                           // domain along axis a; 0 when k L_a is a multiple of 2 pi (the wrapped
                           // foot's phase is exact)
};

// Some axis of a split problem turns f0's phase per wrap (the traces count wraps)
__host__ __device__ inline bool phase_wraps(const Problem &p)
{
    return p.phase_wrap[0] != 0.0 || p.phase_wrap[1] != 0.0 || p.phase_wrap[2] != 0.0;
}

// The points an FP64 trace starts from and their metric weight: the
// handle's own grid (point_grid_of), or for nufi_compute_metrics the
// reference's metrics grid (conf_metrics, nufi/cuda_kernel.cu:53-79: x =
// x_min + ix dx, u = u_min + iu du + du / 2, weight du dx).
struct PointGrid {
    int N[3], M[3];
    long long Ns, Nm;
    double xmin[3], dx[3], vmin[3], dv[3];
    double w;  // prod_a dv_a, times prod_a dx_a below 3D (the reference's 3D metrics leave dx dy dz out)
};

inline PointGrid point_grid_of(const Problem &p)
{
    PointGrid g;
    g.Ns = p.Ns;
    g.Nm = p.Nm;
    g.w = p.wv;
    for (int a = 0; a < 3; ++a) {
        g.N[a] = p.N[a];
        g.M[a] = p.M[a];
        g.xmin[a] = p.xmin[a];
        g.dx[a] = p.dx[a];
        g.vmin[a] = p.vmin[a];
        g.dv[a] = p.dv[a];
        if (p.dim < 3 && a < p.dim) g.w *= p.dx[a];
    }
    return g;
}

// n!, evaluated at compile time where the spline kernels use it (a runtime
// call would recurse and divide in every spline evaluation)
__host__ __device__ constexpr double faculty(int n) { return (n > 1) ? double(n) * faculty(n - 1) : 1.0; }

// splines1d::N<real,order,derivative> (nufi/splines.hpp:39-79), restated:
// all `order` basis values (or their derivative) at reference coordinate x.
template <typename real, int ORDER, int DERIV>
__host__ __device__ __forceinline__ void bspline_basis(real x, real *result)
{
    constexpr int n = ORDER, d = DERIV;
    if (DERIV >= ORDER) {
#pragma unroll
        for (int i = 0; i < ORDER; ++i) result[i] = 0;
        return;
    }
    real v[ORDER];
    v[n - 1] = 1;
#pragma unroll
    for (int k = 1; k < n - d; ++k) {
        v[n - k - 1] = (1 - x) * v[n - k];
#pragma unroll
        for (int i = 1 - k; i < 0; ++i) v[n - 1 + i] = (x - i) * v[n - 1 + i] + (k + 1 + i - x) * v[n + i];
        v[n - 1] *= x;
    }
#pragma unroll
    for (int j = d - 1; j >= 0; --j) {
        v[j] = -v[j + 1];
#pragma unroll
        for (int i = j + 1; i < ORDER - 1; ++i) v[i] = v[i] - v[i + 1];
    }
    constexpr real factor = real(1) / real(faculty(ORDER - DERIV - 1));
#pragma unroll
    for (int i = 0; i < ORDER; ++i) result[i] = v[i] * factor;
}

// splines1d::eval<real,order,derivative> (nufi/splines.hpp:81-110) on a
// window already gathered into c[0..ORDER) (destroyed), x the local
// coordinate in [0, 1] (to a rounding).  The first factor of each de Boor
// update is ((x + n) - d - 1 - i) there, four adds in that order; with x in
// [0, 1] every subtraction after the first add is exact, so x + n rounded
// once and then minus the integer d + 1 + i gives the same bits with one
// add per update (the FP64 trace is bound by the FP64 pipe).
template <typename real, int ORDER, int DERIV>
__host__ __device__ __forceinline__ real deboor(real x, real *c)
{
    constexpr int n = ORDER, d = DERIV;
    if (d >= n) return 0;
#pragma unroll
    for (int j = 1; j <= d; ++j)
#pragma unroll
        for (int i = n - 1; i >= j; --i) c[i] = c[i] - c[i - 1];
    const real y = x + real(n);
#pragma unroll
    for (int j = 1; j < n - d; ++j)
#pragma unroll
        for (int i = n - d - 1; i >= j; --i)
            c[d + i] = (y - real(d + 1 + i)) * c[d + i] + (i - j + 1 - x) * c[d + i - 1];
    constexpr real factor = real(1) / real(faculty(ORDER - DERIV - 1));
    return factor * c[n - 1];
}

// deboor<double, 4, 1> on the window c0..c3 held in registers: the same
// operations in the same order (the differences, then the three de Boor
// updates), written out.  On the FP64 pipe this form compiles to about six
// fewer FP64 instructions per evaluation than the array loop.
__host__ __device__ __forceinline__ double deboor4_d1(double x, double c0, double c1, double c2, double c3)
{
    const double d3 = c3 - c2, d2 = c2 - c1, d1 = c1 - c0;
    const double y = x + 4.0;
    const double a4 = y - 4.0, a3 = y - 3.0, b2 = 2.0 - x, b1 = 1.0 - x;
    const double e3 = a4 * d3 + b2 * d2;
    const double e2 = a3 * d2 + b1 * d1;
    return 0.5 * (a4 * e3 + b1 * e2);
}

// Cubic (order-4) B-spline values b[0..3] and derivatives d[0..3] (d/dt)
// at the local coordinate t in [0, 1]: closed forms of splines1d::N<4,0>
// and N<4,1> (nufi/splines.hpp:39-79),
//   b0 = (1-t)^3/6, b3 = t^3/6, b1 = 2/3 - t^2 + t^3/2, b2 = 1 - b0 - b1 - b3,
//   d0 = -(1-t)^2/2, d3 = t^2/2, d1 = t (3t/2 - 2), d2 = -(d0 + d1 + d3),
// about 20 FP64 operations for both (the FP64 trace is bound by the FP64
// pipe; the results agree with the recurrence to rounding).
__device__ __forceinline__ void cubic_bd_fp64(double t, double (&b)[4], double (&d)[4])
{
    const double s = 1.0 - t, t2 = t * t, s2 = s * s;
    b[0] = (s2 * s) * (1.0 / 6.0);
    b[3] = (t2 * t) * (1.0 / 6.0);
    b[1] = fma(0.5 * t, t2, 2.0 / 3.0 - t2);
    b[2] = ((1.0 - b[0]) - b[1]) - b[3];
    d[0] = -0.5 * s2;
    d[3] = 0.5 * t2;
    d[1] = t * fma(1.5, t, -2.0);
    d[2] = -((d[0] + d[1]) + d[3]);
}

// Initial conditions in FP64, same expressions as the oracle's and the
// reference's f0 (nufi/config.hpp:82-83, 148-149, 233-234).
__device__ __forceinline__ double f0_1d(const Problem &p, double x, double u)
{
    const double alpha = p.f0p[0], k = p.f0p[1];
    if (p.f0_kind == NUFI_F0_LANDAU)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2);
    if (p.f0_kind == NUFI_F0_TWO_STREAM)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2.) * u * u;
    const double ub = p.f0p[2], sb = p.f0p[3];
    const double z = (u - ub) / sb;
    return (1. + alpha * cos(k * x)) *
           (0.9 * 0.39894228040143267793994 * exp(-u * u / 2) + 0.1 * 0.39894228040143267793994 / sb * exp(-z * z / 2));
}

__device__ __forceinline__ double f0_2d(const Problem &p, double x, double y, double u, double v)
{
    const double alpha = p.f0p[0], k = p.f0p[1];
    return 1.0 / (2.0 * 3.14159265358979323846) * exp(-0.5 * (u * u + v * v)) * (1 + alpha * (cos(k * x) + cos(k * y)));
}

__device__ __forceinline__ double f0_3d(const Problem &p, double x, double y, double z, double u, double v, double w)
{
    const double alpha = p.f0p[0], k = p.f0p[1];
    if (p.f0_kind == NUFI_F0_BUMP_ON_TAIL) {
        // the reference's compiled-in 3D f0 (nufi/config.hpp:80-82) with
        // runtime alpha, k, u_b, sigma_b, in its operation order
        const double ub = p.f0p[2], sb = p.f0p[3], a = 1 / (2 * sb * sb);
        return 0.06349363593424096978576330493464 *
               (0.9 * exp(-0.5 * u * u) + 0.1 / sb * exp(-a * (u - ub) * (u - ub))) *
               exp(-0.5 * (v * v + w * w)) * (1 + alpha * (cos(k * x) + cos(k * y) + cos(k * z)));
    }
    return 0.06349363593424096978576330493464 * (1. + alpha * cos(k * x) + alpha * cos(k * y) + alpha * cos(k * z)) *
           exp(-(u * u + v * v + w * w) / 2);
}

}  // namespace nufi_gb300
