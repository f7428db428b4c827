// trace_fp64_table.cu — FP64 plain form of the 1D cubic (order-4) trace in
// cell units, with the field of each slab held as a per-cell FP64 table of
// the spline derivative's quadratic.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so the FP64 trace is bound by
// FP64 instructions; the reference's substep (nufi/rho.hpp:31-61 with
// dim1::eval, nufi/fields.hpp:36-61, and de Boor, nufi/splines.hpp:81-110)
// takes about 23 of them.  Here a substep takes 7, all FP64:
//   state per point: unwrapped cell count U (int), fraction xi in [0, 1)
//   and V = u dt / dx, the velocity in cells per substep
//   drift (x -= dt u):  t = xi - V;  s = t + 1.5 * 2^52 rounded down, whose
//                       low word is floor(t);  U += floor(t);
//                       xi = t - (s - 1.5 * 2^52)                (4 DADD)
//   kick  (u += dt E):  V += a_J + xi (b_J + xi c_J),  J = U mod N  (2 DFMA,
//                       1 DADD; halved on slab 0 as in the reference)
// where (a, b, c)_J = -(dt/dx)^2 ((c2 - c0)/2, c0 - 2 c1 + c2,
// (3 (c1 - c2) - c0 + c3)/2) of the slab's coefficients c0..c3 = c[J..J+3]:
// the derivative of the cubic spline on cell J, dS/dxi = sum_j c_{J+j}
// N'_j(xi), times the kick in cells (derive_table64_kernel).  The same
// substeps in the same order as the reference, in exact FP64 arithmetic
// organised around the cell; the rounding differs from the reference's in
// the last bits of each operation.  f0 is evaluated at the unwrapped foot
// x = x_min + dx (U + xi), u = V dx / dt, as the reference evaluates it.
//
// 2D (order 4) the same way: per axis the cell count, fraction and velocity
// in cells per substep, and per cell the 24 monomial coefficients of the
// field's two components,
//   -(dt/dx)^2 dS/dxi  = sum_{p<=2, q<=3} P_pq xi^p eta^q,
//   -(dt/dy)^2 dS/deta = sum_{p<=3, q<=2} Q_pq xi^p eta^q,
// S the bicubic spline on the cell (derive_table64_2d_kernel), evaluated by
// Horner's rule: 22 DFMA for both components against about 80 FP64
// operations for the bases and the 4 x 4 contraction of trace_fp64.cu, and
// 4 DADD of drift per axis against about 8 of wrap and locate.  The
// reference's 2D substep is nufi/rho.hpp:191-232 with dim2::eval
// (nufi/fields.hpp:149-184).  The table holds 24 doubles per cell and slab
// (coefficient-major: each of the 24 loads of a warp is contiguous when its
// lanes sit in neighbouring cells).
//
// 3D (order 4): a per-cell table would hold 144 doubles per cell, 477 MB
// for the 16^3 x 32^3, 101-step run, beyond L2; the kernel keeps the 4^3
// window contraction of trace_fp64.cu on the slab (55 KB, L2-resident) and
// takes the cell-unit drift and locate (4 DADD per axis against about 9 for
// drift, wrap and locate) and the kick V += -(dt/dx)^2 dS/dxi (one DFMA per
// axis).  The contraction (188 multiply-adds) and the cubic bases run in
// double-float arithmetic on the FP32 pipe: each value a pair of floats
// (hi, lo), hi + lo its value to about 2^-48 relative, with Dekker's and
// Knuth's error-free sum and product (T. J. Dekker, "A floating-point
// technique for extending the available precision", Numer. Math. 18, 1971;
// the product's error term by one FMA).  The slab is read as such pairs
// (derive_ff3d_kernel writes them beside each FP64 slab), the fractions are
// split once per substep, and E goes back to FP64 for the kick: 36 FP64
// and about 3,300 FP32 operations per point-substep instead of about 240
// FP64 ones.  Each multiply-add's error is below 2^-47 of its operands'
// magnitudes (FP64: 2^-53), far below the 1e-12 parity bar.
//
// Thread mapping and the deterministic rho rows are trace_fp64.cu's: a warp
// is 32 consecutive spatial nodes at one velocity node, PPT velocity nodes
// per thread, write_partial_tiled then reduce_rho.
#include "double_float.cuh"
#include "nufi_kernels.cuh"

namespace nufi_gb300 {

namespace {

constexpr double kMagic64 = 6755399441055744.0;  // 1.5 * 2^52: unit ulp for |t| < 2^51

// Cubic B-spline bases on a cell as monomials, b_a(t) = sum_p kM[a][p] t^p
// (the closed forms of splines1d::N<4,0>, nufi/splines.hpp:39-79), and
// their derivatives b'_a(t) = sum_p kD[a][p] t^p.
__constant__ double kM[4][4] = {{1.0 / 6, -0.5, 0.5, -1.0 / 6},
                                {4.0 / 6, 0.0, -1.0, 0.5},
                                {1.0 / 6, 0.5, 0.5, -0.5},
                                {0.0, 0.0, 0.0, 1.0 / 6}};
__constant__ double kD[4][3] = {{-0.5, 1.0, -0.5}, {0.0, -2.0, 1.5}, {0.5, 1.0, -1.5}, {0.0, 0.0, 0.5}};

// The drift of one axis in cell units (see the file comment): 4 DADD.
__device__ __forceinline__ void drift_cells(int &U, double &xi, double V)
{
    const double t = xi - V;
    const double sm = __dadd_rd(t, kMagic64);
    U += __double2loint(sm);
    xi = t - (sm - kMagic64);
}

template <bool POW2>
__device__ __forceinline__ int cell_of(int U, int N)
{
    if constexpr (POW2) {
        return U & (N - 1);
    } else {
        const int J = U % N;
        return J + (J < 0 ? N : 0);
    }
}

// cubic_bd_fp64 (nufi_common.cuh) in double-float: the four cubic B-spline
// values and derivatives on a cell at fraction t; c6 = 1/6, c23 = 2/3.
__device__ __forceinline__ void cubic_bd_ff(ff t, ff c6, ff c23, ff (&b)[4], ff (&d)[4])
{
    const ff one = {1.0f, 0.0f};
    const ff s = ff_add(one, ff_neg(t));
    const ff t2 = ff_mul(t, t), s2 = ff_mul(s, s);
    const ff t3 = ff_mul(t2, t);
    b[0] = ff_mul(ff_mul(s2, s), c6);
    b[3] = ff_mul(t3, c6);
    b[1] = ff_add(ff_scale2(t3, 0.5f), ff_add(c23, ff_neg(t2)));
    b[2] = ff_add(ff_add(ff_add(one, ff_neg(b[0])), ff_neg(b[1])), ff_neg(b[3]));
    d[0] = ff_scale2(s2, -0.5f);
    d[3] = ff_scale2(t2, 0.5f);
    d[1] = ff_mul(t, ff_add(ff_mul(t, ff{1.5f, 0.0f}), ff{-2.0f, 0.0f}));
    d[2] = ff_neg(ff_add(ff_add(d[0], d[1]), d[3]));
}

}  // namespace

template <int PPT, bool POW2>
__global__ void __launch_bounds__(256) trace_fp64_1d_table_kernel(const Problem p, const double *__restrict__ tab,
                                                                  long long tstride, int n, long long q_begin,
                                                                  long long q_end, int vblocks,
                                                                  double *__restrict__ partial, unsigned *err)
{
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    const long long s = (long long)blockIdx.x * 32 + lane;
    const int N = p.N[0];
    const double vscale = p.dt * p.dxinv[0];  // V = u dt / dx
    double acc = 0;
    // velocity blocks strided over the grid's y axis (one each below 65536)
    for (int vb = blockIdx.y; vb < vblocks; vb += gridDim.y) {
    const long long mb = ((long long)vb * W + warp) * PPT;
    int U[PPT];
    double xi[PPT], V[PPT];
    bool live[PPT];
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = mb + q;
        const long long qq = s * p.Nm + m;
        live[q] = (s < p.Ns) && (m < p.Nm) && (qq >= q_begin) && (qq < q_end);
        U[q] = int(s < p.Ns ? s : 0);
        xi[q] = 0.0;
        V[q] = (p.vmin[0] + double(m < p.Nm ? m : 0) * p.dv[0] + p.dv[0] / 2) * vscale;
    }
    auto substep = [&](const double *__restrict__ tk, bool half) {
        const double2 *__restrict__ ab = reinterpret_cast<const double2 *>(tk);
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            drift_cells(U[q], xi[q], V[q]);
            const int J = cell_of<POW2>(U[q], N);
            const double2 v = __ldg(ab + J);
            const double poly = fma(xi[q], fma(xi[q], __ldg(tk + 2 * N + J), v.y), v.x);
            V[q] = half ? fma(0.5, poly, V[q]) : V[q] + poly;
        }
    };
    if (n > 0) {
        for (int k = n - 1; k >= 1; --k) substep(tab + (long long)k * tstride, false);
        substep(tab, true);
    }
    const double udx = p.dx[0] / p.dt;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        // a non-finite position (the cells stayed in range: J is U mod N)
        if (!isfinite(xi[q])) atomicOr(err, kErrCellIndex);
        acc += f0_1d(p, fma(p.dx[0], double(U[q]) + xi[q], p.xmin[0]), V[q] * udx);
    }
    }
    write_partial_tiled(acc, s, p.Ns, partial);
}

template <int PPT, bool POW2>
__global__ void __launch_bounds__(256) trace_fp64_2d_table_kernel(const Problem p, const double *__restrict__ tab,
                                                                  long long tstride, int n, long long q_begin,
                                                                  long long q_end, int vblocks,
                                                                  double *__restrict__ partial, unsigned *err)
{
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    const long long s = (long long)blockIdx.x * 32 + lane;
    const int N0 = p.N[0], N1 = p.N[1];
    const long long Ns = p.Ns;
    const double vs0 = p.dt * p.dxinv[0], vs1 = p.dt * p.dxinv[1];
    double acc = 0;
    for (int vb = blockIdx.y; vb < vblocks; vb += gridDim.y) {
    const long long mb = ((long long)vb * W + warp) * PPT;
    int U0[PPT], U1[PPT];
    double x0[PPT], x1[PPT], V0[PPT], V1[PPT];
    bool live[PPT];
    const long long sc = s < Ns ? s : 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = mb + q;
        const long long qq = s * p.Nm + m;
        live[q] = (s < Ns) && (m < p.Nm) && (qq >= q_begin) && (qq < q_end);
        const long long mc = m < p.Nm ? m : 0;
        U0[q] = int(sc % N0);
        U1[q] = int(sc / N0);
        x0[q] = 0.0;
        x1[q] = 0.0;
        V0[q] = (p.vmin[0] + double(mc % p.M[0]) * p.dv[0] + p.dv[0] / 2) * vs0;
        V1[q] = (p.vmin[1] + double(mc / p.M[0]) * p.dv[1] + p.dv[1] / 2) * vs1;
    }
    auto substep = [&](const double *__restrict__ tk, bool half) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
            drift_cells(U0[q], x0[q], V0[q]);
            drift_cells(U1[q], x1[q], V1[q]);
            const double *__restrict__ c = tk + cell_of<POW2>(U0[q], N0) + (long long)cell_of<POW2>(U1[q], N1) * N0;
            const double xi = x0[q], eta = x1[q];
            // dS/dxi: rows q = 3..0 of P_pq (coefficient p * 4 + q), Horner in eta
            double ex = fma(xi, fma(xi, __ldg(c + 11 * Ns), __ldg(c + 7 * Ns)), __ldg(c + 3 * Ns));
#pragma unroll
            for (int r = 2; r >= 0; --r)
                ex = fma(ex, eta, fma(xi, fma(xi, __ldg(c + (8 + r) * Ns), __ldg(c + (4 + r) * Ns)), __ldg(c + r * Ns)));
            // dS/deta: rows p = 3..0 of Q_pq (coefficient 12 + p * 3 + q), Horner in xi
            double ey = fma(eta, fma(eta, __ldg(c + 23 * Ns), __ldg(c + 22 * Ns)), __ldg(c + 21 * Ns));
#pragma unroll
            for (int r = 2; r >= 0; --r)
                ey = fma(ey, xi,
                         fma(eta, fma(eta, __ldg(c + (14 + 3 * r) * Ns), __ldg(c + (13 + 3 * r) * Ns)),
                             __ldg(c + (12 + 3 * r) * Ns)));
            V0[q] = half ? fma(0.5, ex, V0[q]) : V0[q] + ex;
            V1[q] = half ? fma(0.5, ey, V1[q]) : V1[q] + ey;
        }
    };
    if (n > 0) {
        for (int k = n - 1; k >= 1; --k) substep(tab + (long long)k * tstride, false);
        substep(tab, true);
    }
    const double u0 = p.dx[0] / p.dt, u1 = p.dx[1] / p.dt;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        if (!isfinite(x0[q]) || !isfinite(x1[q])) atomicOr(err, kErrCellIndex);
        acc += f0_2d(p, fma(p.dx[0], double(U0[q]) + x0[q], p.xmin[0]), fma(p.dx[1], double(U1[q]) + x1[q], p.xmin[1]),
                     V0[q] * u0, V1[q] * u1);
    }
    }
    write_partial_tiled(acc, s, Ns, partial);
}

template <int PPT, bool POW2>
__global__ void __launch_bounds__(256, 2) trace_fp64_3d_cells_kernel(const Problem p, const float2 *__restrict__ tff,
                                                                  long long tstride, int n, long long q_begin,
                                                                  long long q_end, int vblocks,
                                                                  double *__restrict__ partial, unsigned *err)
{
    const int lane = threadIdx.x, warp = threadIdx.y, W = blockDim.y;
    const long long s = (long long)blockIdx.x * 32 + lane;
    const long long Ns = p.Ns;
    const int sy = p.P[0], sz = p.P[0] * p.P[1];
    const ff c6 = ff_of(1.0 / 6.0), c23 = ff_of(2.0 / 3.0);
    double K[3], vs[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        vs[a] = p.dt * p.dxinv[a];
        K[a] = -vs[a] * vs[a];
    }
    double acc = 0;
    for (int vb = blockIdx.y; vb < vblocks; vb += gridDim.y) {
    const long long mb = ((long long)vb * W + warp) * PPT;
    int U[PPT][3];
    double X[PPT][3], V[PPT][3];
    bool live[PPT];
    const long long sc = s < Ns ? s : 0;
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        const long long m = mb + q;
        const long long qq = s * p.Nm + m;
        live[q] = (s < Ns) && (m < p.Nm) && (qq >= q_begin) && (qq < q_end);
        long long rs = sc, rm = m < p.Nm ? m : 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            U[q][a] = int(rs % p.N[a]);
            rs /= p.N[a];
            X[q][a] = 0.0;
            V[q][a] = (p.vmin[a] + double(rm % p.M[a]) * p.dv[a] + p.dv[a] / 2) * vs[a];
            rm /= p.M[a];
        }
    }
    auto substep = [&](const float2 *__restrict__ c, double h) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
#pragma unroll
            for (int a = 0; a < 3; ++a) drift_cells(U[q][a], X[q][a], V[q][a]);
            const float2 *__restrict__ w = c + (long long)cell_of<POW2>(U[q][2], p.N[2]) * sz +
                                           (long long)cell_of<POW2>(U[q][1], p.N[1]) * sy +
                                           cell_of<POW2>(U[q][0], p.N[0]);
            // the window contraction of trace_fp64.cu's field_3d<4>, in double-float
            ff bx[4], dx[4], by[4], dy[4], bz[4], dz[4];
            cubic_bd_ff(ff_of(X[q][0]), c6, c23, bx, dx);
            cubic_bd_ff(ff_of(X[q][1]), c6, c23, by, dy);
            cubic_bd_ff(ff_of(X[q][2]), c6, c23, bz, dz);
            const ff zero = {0.0f, 0.0f};
            ff ex = zero, ey = zero, ez = zero;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ff sx = zero, s_y = zero, s_z = zero;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    ff r0 = zero, r1 = zero;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float2 v2 = __ldg(w + k * sz + j * sy + i);
                        const ff v = {v2.x, v2.y};
                        r0 = ff_fma(v, bx[i], r0);
                        r1 = ff_fma(v, dx[i], r1);
                    }
                    sx = ff_fma(r1, by[j], sx);
                    s_y = ff_fma(r0, dy[j], s_y);
                    s_z = ff_fma(r0, by[j], s_z);
                }
                ex = ff_fma(sx, bz[k], ex);
                ey = ff_fma(s_y, bz[k], ey);
                ez = ff_fma(s_z, dz[k], ez);
            }
            V[q][0] = fma(h * K[0], ff_value(ex), V[q][0]);
            V[q][1] = fma(h * K[1], ff_value(ey), V[q][1]);
            V[q][2] = fma(h * K[2], ff_value(ez), V[q][2]);
        }
    };
    if (n > 0) {
        for (int k = n - 1; k >= 1; --k) substep(tff + (long long)k * tstride, 1.0);
        substep(tff, 0.5);
    }
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
        if (!live[q]) continue;
        double x[3], u[3];
        bool finite = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            finite = finite && isfinite(X[q][a]);
            x[a] = fma(p.dx[a], double(U[q][a]) + X[q][a], p.xmin[a]);
            u[a] = V[q][a] * (p.dx[a] / p.dt);
        }
        if (!finite) atomicOr(err, kErrCellIndex);
        acc += f0_3d(p, x[0], x[1], x[2], u[0], u[1], u[2]);
    }
    }
    write_partial_tiled(acc, s, Ns, partial);
}

// The double-float pairs of one 3D slab: (hi, lo) with hi the coefficient
// rounded to FP32 and lo the rest rounded to FP32 (see the file comment).
__global__ void derive_ff3d_kernel(const Problem p, const double *__restrict__ slab, float2 *__restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.stride_t) return;
    const ff v = ff_of(slab[i]);
    out[i] = make_float2(v.hi, v.lo);
}

// The 24 coefficients of every cell of one 2D slab (see the file comment):
// one thread per cell (i, j), from the 4 x 4 window w[b][a] =
// slab[(j + b) P0 + i + a] (a along x).
__global__ void derive_table64_2d_kernel(const Problem p, const double *__restrict__ slab, double *__restrict__ tab)
{
    const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= p.Ns) return;
    const int i = int(cell % p.N[0]), j = int(cell / p.N[0]);
    const int P0 = p.P[0];
    const double Kx = -(p.dt * p.dxinv[0]) * (p.dt * p.dxinv[0]);
    const double Ky = -(p.dt * p.dxinv[1]) * (p.dt * p.dxinv[1]);
    double T[4][4], S[4][3];  // per x index a: the y-monomials of the value and of the y-derivative
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        double w[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) w[b] = slab[(long long)(j + b) * P0 + i + a];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double t = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) t = fma(w[b], kM[b][q], t);
            T[a][q] = t;
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double t = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) t = fma(w[b], kD[b][q], t);
            S[a][q] = t;
        }
    }
    const long long Ns = p.Ns;
#pragma unroll
    for (int pp = 0; pp < 3; ++pp)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double t = 0;
#pragma unroll
            for (int a = 0; a < 4; ++a) t = fma(kD[a][pp], T[a][q], t);
            tab[(pp * 4 + q) * Ns + cell] = Kx * t;
        }
#pragma unroll
    for (int pp = 0; pp < 4; ++pp)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double t = 0;
#pragma unroll
            for (int a = 0; a < 4; ++a) t = fma(kM[a][pp], S[a][q], t);
            tab[(12 + pp * 3 + q) * Ns + cell] = Ky * t;
        }
}

// (a, b, c) of every cell of one slab (see the file comment): one thread
// per cell, from the padded FP64 slab.
__global__ void derive_table64_kernel(const Problem p, const double *__restrict__ slab, double *__restrict__ tab,
                                      double *__restrict__ hist_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = p.N[0];
    if (hist_out && i < p.stride_t) hist_out[i] = slab[i];  // the slab itself, when it comes from elsewhere
    if (i >= N) return;
    const double K = -(p.dt * p.dxinv[0]) * (p.dt * p.dxinv[0]);
    const double c0 = slab[i], c1 = slab[i + 1], c2 = slab[i + 2], c3 = slab[i + 3];
    reinterpret_cast<double2 *>(tab)[i] = make_double2(K * (0.5 * (c2 - c0)), K * ((c0 - 2.0 * c1) + c2));
    tab[2 * N + i] = K * (0.5 * ((3.0 * (c1 - c2) - c0) + c3));
}

// The table trace where it applies: 1D, order 4, and an unwrapped cell
// count that stays far inside int (|U| grows by at most |V| + 1 per
// substep; the margin of 4 covers the kicks' change of V).
// 2D: also a table of at most 4 GiB (24 doubles per cell and slab).  3D:
// the cell-unit trace on the slab's double-float pairs (the slab's size).
bool fp64_table_supported(const Problem &p, long long Nt)
{
    if (p.order != 4) return false;
    for (int a = 0; a < p.dim; ++a) {
        const double vmax = fmax(fabs(p.vmin[a]), fabs(p.vmin[a] + p.M[a] * p.dv[a]));
        if (!((double(Nt) + 1) * (vmax * p.dt * p.dxinv[a] + 1) * 4 + p.N[a] < 2147483647.0)) return false;
    }
    if (p.dim == 2 && (double(Nt) + 1) * 24.0 * double(p.Ns) * 8.0 > 4294967296.0) return false;
    return true;
}

long long fp64_table_stride(const Problem &p)
{
    // 3D: the slab's double-float pairs, one float2 (8 bytes) per coefficient
    return p.dim == 1 ? (3LL * p.N[0] + 1) / 2 * 2 : p.dim == 2 ? (24LL * p.Ns + 1) / 2 * 2 : p.hist_stride;
}

cudaError_t launch_derive_table64(const Problem &p, const double *hist_slab, double *table_slab, cudaStream_t st,
                                  double *hist_out)
{
    if (hist_out && p.dim != 1) return cudaErrorInvalidValue;  // the copy form is 1D only
    if (p.dim == 3) {
        derive_ff3d_kernel<<<unsigned((p.stride_t + 255) / 256), 256, 0, st>>>(p, hist_slab,
                                                                          reinterpret_cast<float2 *>(table_slab));
        return cudaGetLastError();
    }
    if (p.dim == 1) {
        const long long n = hist_out ? p.stride_t : p.N[0];
        derive_table64_kernel<<<unsigned((n + 127) / 128), 128, 0, st>>>(p, hist_slab, table_slab, hist_out);
    } else
        derive_table64_2d_kernel<<<unsigned((p.Ns + 127) / 128), 128, 0, st>>>(p, hist_slab, table_slab);
    return cudaGetLastError();
}

cudaError_t launch_trace_fp64_table(const Problem &p, const LaunchShape &ls, const double *tables,
                                    const double *hist, int n, long long qb, long long qe, double *partial,
                                    int *rows, unsigned *err, cudaStream_t st)
{
    *rows = fp64_rows(ls);
    const dim3 block(32, ls.warps);
    const dim3 grid(unsigned((p.Ns + 31) / 32), unsigned(fp64_rows(ls)));
    const int vb = ls.vblocks;
    const long long ts = fp64_table_stride(p);
    bool pow2 = true;
    for (int a = 0; a < p.dim; ++a) pow2 = pow2 && (p.N[a] & (p.N[a] - 1)) == 0;
    if (p.dim == 3) {  // the planner caps 3D at 2 points per thread
        const float2 *tff = reinterpret_cast<const float2 *>(tables);
#define NUFI_LAUNCH3(K)                                                                                        \
    if (pow2)                                                                                                  \
        trace_fp64_3d_cells_kernel<K, true><<<grid, block, 0, st>>>(p, tff, ts, n, qb, qe, vb, partial, err);  \
    else                                                                                                       \
        trace_fp64_3d_cells_kernel<K, false><<<grid, block, 0, st>>>(p, tff, ts, n, qb, qe, vb, partial, err);
        switch (ls.ppt) {
        case 1: NUFI_LAUNCH3(1) break;
        case 2: NUFI_LAUNCH3(2) break;
        default: return cudaErrorInvalidValue;
        }
#undef NUFI_LAUNCH3
        return cudaGetLastError();
    }
#define NUFI_LAUNCH(K)                                                                                         \
    if (p.dim == 2) {                                                                                          \
        if (pow2)                                                                                              \
            trace_fp64_2d_table_kernel<K, true><<<grid, block, 0, st>>>(p, tables, ts, n, qb, qe, vb, partial, err); \
        else                                                                                                   \
            trace_fp64_2d_table_kernel<K, false><<<grid, block, 0, st>>>(p, tables, ts, n, qb, qe, vb, partial, err); \
    } else if (pow2)                                                                                           \
        trace_fp64_1d_table_kernel<K, true><<<grid, block, 0, st>>>(p, tables, ts, n, qb, qe, vb, partial, err);   \
    else                                                                                                       \
        trace_fp64_1d_table_kernel<K, false><<<grid, block, 0, st>>>(p, tables, ts, n, qb, qe, vb, partial, err);
    switch (ls.ppt) {
    case 1: NUFI_LAUNCH(1) break;
    case 2: NUFI_LAUNCH(2) break;
    case 4: NUFI_LAUNCH(4) break;
    default: return cudaErrorInvalidValue;
    }
#undef NUFI_LAUNCH
    return cudaGetLastError();
}

}  // namespace nufi_gb300
