/*
 * nufi_oracle.c — CPU restatement of the NuFI hot path.  TEST
 * INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
 * baseline leg of bench.py call this library as the oracle.  The product
 * (numericalflowiteration_gb300/) never links, loads or calls it.
 *
 * Parity pin: the restatement follows the reference's operation order so
 * that, built with -ffp-contract=off, its rho agrees with the reference's
 * own header code (compiled from its sources by oracle/ref/Makefile) to the
 * last bit, and its field solve (direct solve instead of LSMR) to ~1e-15;
 * tests/golden/ holds vectors produced by that reference build.
 *
 * What is restated, with the reference lines it follows:
 *   config derived quantities      nufi/config.hpp:55-70, 117-138, 196-219
 *   f0 (runtime kinds)             nufi/config.hpp:72-84, 140-159, 221-247
 *   B-spline basis N<order,d>      nufi/splines.hpp:39-79
 *   de Boor eval<order,d>          nufi/splines.hpp:81-110
 *   2D / 3D tensor evaluation      nufi/splines.hpp:117-137, 144-172
 *   periodic wrap + knot locate    nufi/fields.hpp:36-61, 149-184, 308-350
 *   eval_ftilda (the trace)        nufi/rho.hpp:31-61, 191-232, 318-367
 *   eval_f (with first half kick)  nufi/rho.hpp:63-96, 234-281, 369-426
 *   GPU point convention + weights nufi/cuda_kernel.cu:31-51, 210-237, 392-426
 *   metrics                        nufi/cuda_kernel.cu:53-79, 239-271, 428-466
 *   Poisson via DHT                nufi/poisson.cpp:66-89, 190-219, 328-362
 *   collocation solve + padding    nufi/fields.hpp:63-142, 186-300, 352-490
 * The DHT is FFTW's r2r FFTW_DHT kind (separable in 2D/3D), restated from
 * its definition H_k = sum_j x_j cas(2 pi j k / N).  The reference solves
 * the circulant collocation system with LSMR to machine precision
 * (nufi/lsmr.tpp:65-222); the restatement solves the same system directly
 * per axis of its Kronecker factors, in the circulant's eigenbasis.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/nufi_gb300.h"
#include "nufi_f0.h"

#define OC_MAX_ORDER 8

typedef struct {
    int dim, order, f0_kind;
    size_t N[3];       /* Nx, Ny, Nz        */
    size_t M[3];       /* Nu, Nv, Nw        */
    size_t Nt;
    double dt;
    double xmin[3], L[3], Linv[3], dx[3], dxinv[3];
    double vmin[3], dv[3];
    double p[8];
    size_t sstride[3]; /* slab strides: 1, Nx+o-1, (Nx+o-1)(Ny+o-1) */
    size_t stride_t;   /* values per slab */
    size_t Ns, Nm;     /* spatial nodes, velocity nodes */
} oc_t;

static int oc_setup(const nufi_config *c, oc_t *o)
{
    int d;
    if (!c || c->dim < 1 || c->dim > 3 || c->order < 2 || c->order > OC_MAX_ORDER)
        return NUFI_ERR_INVALID;
    memset(o, 0, sizeof(*o));
    o->dim = c->dim; o->order = c->order; o->f0_kind = c->f0_kind;
    o->Nt = (size_t)c->Nt; o->dt = c->dt;
    for (d = 0; d < 8; ++d) o->p[d] = c->f0_params[d];
    o->Ns = 1; o->Nm = 1; o->stride_t = 1;
    for (d = 0; d < 3; ++d) {
        o->N[d] = 1; o->M[d] = 1; o->sstride[d] = 0;
    }
    for (d = 0; d < c->dim; ++d) {
        if (c->Nx[d] < 1 || c->Nv[d] < 1) return NUFI_ERR_INVALID;
        o->N[d] = (size_t)c->Nx[d];
        o->M[d] = (size_t)c->Nv[d];
        /* config.hpp:67-69 */
        o->xmin[d] = c->x_min[d];
        o->L[d] = c->x_max[d] - c->x_min[d];
        o->Linv[d] = 1 / o->L[d];
        o->dx[d] = o->L[d] / (double)o->N[d];
        o->dxinv[d] = 1 / o->dx[d];
        o->vmin[d] = c->v_min[d];
        o->dv[d] = (c->v_max[d] - c->v_min[d]) / (double)o->M[d];
        o->sstride[d] = o->stride_t;
        o->stride_t *= o->N[d] + (size_t)o->order - 1;
        o->Ns *= o->N[d];
        o->Nm *= o->M[d];
    }
    return NUFI_OK;
}

/* ---- f0 (nufi_f0.h) ----------------------------------------------------- */
static inline __attribute__((always_inline)) double oc_f0_dim(const oc_t *o, int dim, const double *x,
                                                              const double *u)
{
    nufi_f0_params f;
    int i;
    f.kind = o->f0_kind;
    for (i = 0; i < 8; ++i) f.p[i] = o->p[i];
    if (dim == 1) return nufi_f0_1d(&f, x[0], u[0]);
    if (dim == 2) return nufi_f0_2d(&f, x[0], x[1], u[0], u[1]);
    return nufi_f0_3d(&f, x[0], x[1], x[2], u[0], u[1], u[2]);
}

static double oc_f0(const oc_t *o, const double *x, const double *u) { return oc_f0_dim(o, o->dim, x, u); }

/* ---- B-splines (splines.hpp:33-110) ------------------------------------ */
/* 1 / k!: the reference's constexpr factor 1 / faculty<real>(order - d - 1)
 * (splines.hpp:33-37, 76, 108), folded by the compiler here too. */
static const double oc_inv_fac[OC_MAX_ORDER + 1] = {
    1.0 / 1.0, 1.0 / 1.0, 1.0 / 2.0, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0, 1.0 / 5040.0, 1.0 / 40320.0};

/* The trace's functions are written once with the dimension and the spline
 * order as parameters and inlined into one copy per (dimension, order)
 * (oc_trace below), so both are compile-time constants there, as in the
 * reference's templates; the operations and their order are the same in
 * every copy. */
#define OC_INLINE static inline __attribute__((always_inline))

/* splines1d::N<real,order,derivative>: all `order` basis values (or
 * derivatives) at reference coordinate x in [0,1). */
OC_INLINE void oc_N(int order, int deriv, double x, double *result)
{
    const int n = order, d = deriv;
    double v[OC_MAX_ORDER];
    int k, i, j;
    if (deriv >= order) {
        for (i = 0; i < order; ++i) result[i] = 0;
        return;
    }
    if (n == 1) { result[0] = 1; return; }
    v[n - 1] = 1;
    for (k = 1; k < n - d; ++k) {
        v[n - k - 1] = (1 - x) * v[n - k];
        for (i = 1 - k; i < 0; ++i)
            v[n - 1 + i] = (x - i) * v[n - 1 + i] + (k + 1 + i - x) * v[n + i];
        v[n - 1] *= x;
    }
    for (j = d - 1; j >= 0; --j) {
        v[j] = -v[j + 1];
        for (i = j + 1; i < order - 1; ++i) v[i] = v[i] - v[i + 1];
    }
    {
        const double factor = oc_inv_fac[order - deriv - 1];
        for (i = 0; i < order; ++i) result[i] = v[i] * factor;
    }
}

/* splines1d::eval<real,order,derivative> on an already gathered window. */
OC_INLINE double oc_eval1(int order, int deriv, double x, const double *coef, size_t stride)
{
    const int n = order, d = deriv;
    double c[OC_MAX_ORDER];
    int i, j;
    if (d >= n) return 0;
    if (n == 1) return coef[0];
    for (j = 0; j < n; ++j) c[j] = coef[stride * (size_t)j];
    for (j = 1; j <= d; ++j)
        for (i = n - 1; i >= j; --i) c[i] = c[i] - c[i - 1];
    for (j = 1; j < n - d; ++j)
        for (i = n - d - 1; i >= j; --i)
            c[d + i] = (x + n - d - 1 - i) * c[d + i] + (i - j + 1 - x) * c[d + i - 1];
    return oc_inv_fac[order - deriv - 1] * c[n - 1];
}

/* fields.hpp periodic wrap + knot (shared by all dims, per axis). */
OC_INLINE void oc_locate(const oc_t *o, int a, double x, size_t *knot, double *xi)
{
    double xk;
    x -= o->xmin[a];
    x = x - o->L[a] * floor(x * o->Linv[a]);
    xk = floor(x * o->dxinv[a]);
    *knot = (size_t)xk;
    *xi = x * o->dxinv[a] - xk;
}

/* dim1::eval<real,order,1> (fields.hpp:36-61) */
OC_INLINE double oc_eval_1d(const oc_t *o, int order, double x, const double *c, int deriv)
{
    size_t ii; double xi, factor = 1; int i;
    oc_locate(o, 0, x, &ii, &xi);
    for (i = 0; i < deriv; ++i) factor *= o->dxinv[0];
    return factor * oc_eval1(order, deriv, xi, c + ii, 1);
}

/* dim2::eval<real,order,dx,dy> (fields.hpp:149-184, splines.hpp:117-137) */
OC_INLINE double oc_eval_2d(const oc_t *o, int order, double x, double y, const double *coeffs, int ddx, int ddy)
{
    size_t ii, jj, i, j;
    double xi, eta, factor = 1, cc[OC_MAX_ORDER], Nb[OC_MAX_ORDER];
    const size_t sy = o->sstride[1];
    int q;
    oc_locate(o, 0, x, &ii, &xi);
    oc_locate(o, 1, y, &jj, &eta);
    for (q = 0; q < ddx; ++q) factor *= o->dxinv[0];
    for (q = 0; q < ddy; ++q) factor *= o->dxinv[1];
    coeffs += jj * sy + ii;
    if (ddx >= order || ddy >= order) return factor * 0;
    for (j = 0; j < (size_t)order; ++j) cc[j] = 0;
    oc_N(order, ddx, xi, Nb);
    for (j = 0; j < (size_t)order; ++j)
        for (i = 0; i < (size_t)order; ++i)
            cc[j] += coeffs[j * sy + i] * Nb[i];
    return factor * oc_eval1(order, ddy, eta, cc, 1);
}

/* dim3::eval<real,order,dx,dy,dz> (fields.hpp:308-350, splines.hpp:144-172) */
OC_INLINE double oc_eval_3d(const oc_t *o, int order, double x, double y, double z, const double *coeffs,
                            int ddx, int ddy, int ddz)
{
    size_t ii, jj, kk, i, j, k;
    double xi, eta, zeta, factor = 1;
    double czy[OC_MAX_ORDER * OC_MAX_ORDER], cz[OC_MAX_ORDER], Nb[OC_MAX_ORDER];
    const size_t sy = o->sstride[1], sz = o->sstride[2];
    int q;
    oc_locate(o, 0, x, &ii, &xi);
    oc_locate(o, 1, y, &jj, &eta);
    oc_locate(o, 2, z, &kk, &zeta);
    for (q = 0; q < ddx; ++q) factor *= o->dxinv[0];
    for (q = 0; q < ddy; ++q) factor *= o->dxinv[1];
    for (q = 0; q < ddz; ++q) factor *= o->dxinv[2];
    coeffs += kk * sz + jj * sy + ii;
    for (k = 0; k < (size_t)(order * order); ++k) czy[k] = 0;
    for (k = 0; k < (size_t)order; ++k) cz[k] = 0;
    oc_N(order, ddx, xi, Nb);
    for (k = 0; k < (size_t)order; ++k)
        for (j = 0; j < (size_t)order; ++j)
            for (i = 0; i < (size_t)order; ++i)
                czy[k * order + j] += coeffs[k * sz + j * sy + i] * Nb[i];
    oc_N(order, ddy, eta, Nb);
    for (k = 0; k < (size_t)order; ++k)
        for (j = 0; j < (size_t)order; ++j)
            cz[k] += czy[k * order + j] * Nb[j];
    return factor * oc_eval1(order, ddz, zeta, cz, 1);
}

/* E = -grad phi from one slab, component by component as the reference
 * does (two / three separate eval calls, rho.hpp:213-214, 343-345). */
OC_INLINE void oc_field(const oc_t *o, int dim, int order, const double *x, const double *c, double *E)
{
    if (dim == 1) {
        E[0] = -oc_eval_1d(o, order, x[0], c, 1);
    } else if (dim == 2) {
        E[0] = -oc_eval_2d(o, order, x[0], x[1], c, 1, 0);
        E[1] = -oc_eval_2d(o, order, x[0], x[1], c, 0, 1);
    } else {
        E[0] = -oc_eval_3d(o, order, x[0], x[1], x[2], c, 1, 0, 0);
        E[1] = -oc_eval_3d(o, order, x[0], x[1], x[2], c, 0, 1, 0);
        E[2] = -oc_eval_3d(o, order, x[0], x[1], x[2], c, 0, 0, 1);
    }
}

/* eval_ftilda (rho.hpp:31-61 / 191-232 / 318-367) when half_first == 0,
 * eval_f (rho.hpp:63-96 / 234-281 / 369-426) when half_first == 1.
 * x, u are updated in place to the foot of the characteristic. */
OC_INLINE double oc_trace_k(const oc_t *o, int D, int order, size_t n, double *x, double *u, const double *coeffs,
                            int half_first)
{
    const double dt = o->dt;
    double E[3];
    const double *c;
    int a;
    if (n == 0) return oc_f0_dim(o, D, x, u);
    if (half_first) {
        c = coeffs + n * o->stride_t;
        oc_field(o, D, order, x, c, E);
        for (a = 0; a < D; ++a) u[a] += 0.5 * dt * E[a];
    }
    while (--n) {
        for (a = 0; a < D; ++a) x[a] = x[a] - dt * u[a];
        c = coeffs + n * o->stride_t;
        oc_field(o, D, order, x, c, E);
        for (a = 0; a < D; ++a) u[a] = u[a] + dt * E[a];
    }
    for (a = 0; a < D; ++a) x[a] -= dt * u[a];
    c = coeffs + n * o->stride_t;
    oc_field(o, D, order, x, c, E);
    for (a = 0; a < D; ++a) u[a] += 0.5 * dt * E[a];
    return oc_f0_dim(o, D, x, u);
}

/* one copy of the trace per dimension and spline order (oc_setup admits
 * dim 1..3 and order 2..8) */
#define OC_TRACE_COPY(D, K)                                                                        \
    static double oc_trace_##D##_##K(const oc_t *o, size_t n, double *x, double *u, const double *c, \
                                     int half_first)                                               \
    {                                                                                              \
        return oc_trace_k(o, D, K, n, x, u, c, half_first);                                        \
    }
#define OC_TRACE_DIM(D) \
    OC_TRACE_COPY(D, 2) OC_TRACE_COPY(D, 3) OC_TRACE_COPY(D, 4) OC_TRACE_COPY(D, 5) OC_TRACE_COPY(D, 6) \
    OC_TRACE_COPY(D, 7) OC_TRACE_COPY(D, 8)
OC_TRACE_DIM(1)
OC_TRACE_DIM(2)
OC_TRACE_DIM(3)

typedef double (*oc_trace_fn)(const oc_t *, size_t, double *, double *, const double *, int);
static const oc_trace_fn oc_trace_copies[3][7] = {
    {oc_trace_1_2, oc_trace_1_3, oc_trace_1_4, oc_trace_1_5, oc_trace_1_6, oc_trace_1_7, oc_trace_1_8},
    {oc_trace_2_2, oc_trace_2_3, oc_trace_2_4, oc_trace_2_5, oc_trace_2_6, oc_trace_2_7, oc_trace_2_8},
    {oc_trace_3_2, oc_trace_3_3, oc_trace_3_4, oc_trace_3_5, oc_trace_3_6, oc_trace_3_7, oc_trace_3_8}};

static double oc_trace(const oc_t *o, size_t n, double *x, double *u, const double *coeffs, int half_first)
{
    return oc_trace_copies[o->dim - 1][o->order - 2](o, n, x, u, coeffs, half_first);
}

/* Point coordinates by the GPU kernels' convention (cuda_kernel.cu:43-44,
 * 227-230, 414-419): x on nodes, v on midpoints u_min + i*du + du/2. */
static void oc_point(const oc_t *o, size_t s, size_t m, double *x, double *u)
{
    int a;
    for (a = 0; a < o->dim; ++a) {
        const size_t is = s % o->N[a], im = m % o->M[a];
        s /= o->N[a]; m /= o->M[a];
        x[a] = o->xmin[a] + (double)is * o->dx[a];
        u[a] = o->vmin[a] + (double)im * o->dv[a] + o->dv[a] / 2;
    }
}

static double oc_weight_v(const oc_t *o)
{
    double w = 1; int a;
    for (a = 0; a < o->dim; ++a) w *= o->dv[a];
    return w;
}

/* Summation of rho over velocity: 0 = in q order in double, as the
 * reference's CPU loop (rho.hpp:140-143); 1 = Neumaier-compensated, which
 * removes the O(sqrt(Nm) eps) rounding of the plain sum (the reference's
 * GPU kernel sums with atomics in arbitrary order, so its own rho carries
 * that rounding as run-to-run noise). */
static int g_sum_mode = 0;
void oracle_set_summation(int mode) { g_sum_mode = mode; }

/* rho[s] = -(prod dv) * sum_{m : q_begin <= s*Nm+m < q_end} f~(n; s, m)
 * (cuda_kernel.cu:46-50 with the atomics replaced by an ordered sum). */
int oracle_rho(const nufi_config *cfg, int64_t n, const double *coeffs, int64_t q_begin,
               int64_t q_end, double *rho, int nthreads)
{
    oc_t o; long long s;
    int st = oc_setup(cfg, &o);
    if (st) return st;
    if (n < 0 || (size_t)n > o.Nt || q_begin < 0 || q_end < q_begin ||
        (size_t)q_end > o.Ns * o.Nm)
        return NUFI_ERR_RANGE;
    {
        const double w = oc_weight_v(&o);
        (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (s = 0; s < (long long)o.Ns; ++s) {
            double acc = 0, comp = 0;
            size_t m;
            for (m = 0; m < o.Nm; ++m) {
                const int64_t q = (int64_t)((size_t)s * o.Nm + m);
                double x[3], u[3], f;
                if (q < q_begin || q >= q_end) continue;
                oc_point(&o, (size_t)s, m, x, u);
                f = oc_trace(&o, (size_t)n, x, u, coeffs, 0);
                if (g_sum_mode == 1) {
                    const double t = acc + f;
                    comp += (fabs(acc) >= fabs(f)) ? (acc - t) + f : (f - t) + acc;
                    acc = t;
                } else {
                    acc += f;
                }
            }
            rho[s] = -w * (acc + comp);
        }
    }
    return NUFI_OK;
}

/* f~ (mode 0, eval_ftilda) or f (mode 1, eval_f) at arbitrary points;
 * pts holds 2*dim doubles per point (x.., v..); the feet are written back
 * into pts when feet != 0. */
int oracle_eval(const nufi_config *cfg, int64_t n, const double *coeffs, int64_t npts,
                double *pts, double *out, int mode, int feet, int nthreads)
{
    oc_t o; long long i;
    int st = oc_setup(cfg, &o);
    if (st) return st;
    if (n < 0 || (size_t)n > o.Nt) return NUFI_ERR_RANGE;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (i = 0; i < npts; ++i) {
        double x[3], u[3]; int a;
        for (a = 0; a < o.dim; ++a) { x[a] = pts[i * 2 * o.dim + a]; u[a] = pts[i * 2 * o.dim + o.dim + a]; }
        out[i] = oc_trace(&o, (size_t)n, x, u, coeffs, mode);
        if (feet)
            for (a = 0; a < o.dim; ++a) { pts[i * 2 * o.dim + a] = x[a]; pts[i * 2 * o.dim + o.dim + a] = u[a]; }
    }
    return NUFI_OK;
}

/* Metrics of cuda_eval_metrics (cuda_kernel.cu:53-79, 239-271, 428-466):
 * m[0] = sum w f, m[1] = sum w f^2, m[2] = sum w |v|^2 f / 2,
 * m[3] = -sum w f log f (f > 0), f = eval_f(n, .) at the quadrature
 * points; w = prod dv * prod dx in 1D/2D.  In 3D the reference uses
 * w = du dv dw only (cuda_kernel.cu:457); weight3d_full selects prod dx
 * too. */
int oracle_metrics(const nufi_config *cfg, int64_t n, const double *coeffs, int64_t q_begin,
                   int64_t q_end, double *metrics, int weight3d_full, int nthreads)
{
    oc_t o; long long s;
    double m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    int st = oc_setup(cfg, &o);
    if (st) return st;
    if (n < 0 || (size_t)n > o.Nt || q_begin < 0 || q_end < q_begin ||
        (size_t)q_end > o.Ns * o.Nm)
        return NUFI_ERR_RANGE;
    {
        double w = oc_weight_v(&o);
        /* per-node sums in q order, then over the nodes in order: the same
         * result for any thread count or schedule */
        double *part = (double *)malloc(sizeof(double) * 4 * o.Ns);
        int a;
        if (!part) return NUFI_ERR_INVALID;
        if (o.dim < 3 || weight3d_full)
            for (a = 0; a < o.dim; ++a) w *= o.dx[a];
        (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (s = 0; s < (long long)o.Ns; ++s) {
            size_t m;
            double p0 = 0, p1 = 0, p2 = 0, p3 = 0;
            for (m = 0; m < o.Nm; ++m) {
                const int64_t q = (int64_t)((size_t)s * o.Nm + m);
                double x[3], u[3], u0[3], f, uu = 0;
                int b;
                if (q < q_begin || q >= q_end) continue;
                oc_point(&o, (size_t)s, m, x, u);
                for (b = 0; b < o.dim; ++b) { u0[b] = u[b]; uu += u0[b] * u0[b]; }
                f = oc_trace(&o, (size_t)n, x, u, coeffs, 1);
                p0 += w * f;
                p1 += w * f * f;
                p2 += w * (uu * f / 2);
                p3 += (f > 0) ? -w * f * log(f) : 0;
            }
            part[4 * s] = p0; part[4 * s + 1] = p1; part[4 * s + 2] = p2; part[4 * s + 3] = p3;
        }
        for (s = 0; s < (long long)o.Ns; ++s) {
            m0 += part[4 * s]; m1 += part[4 * s + 1]; m2 += part[4 * s + 2]; m3 += part[4 * s + 3];
        }
        free(part);
    }
    metrics[0] = m0; metrics[1] = m1; metrics[2] = m2; metrics[3] = m3;
    return NUFI_OK;
}

/* ---- field solve -------------------------------------------------------- */

/* cas(2 pi j k / N) with the angle reduced exactly in integers.  The DHT
 * sums are formed in long double: with rho ~ -1 + O(alpha) the non-zero
 * modes are small differences of O(1) terms, and the oracle should sit
 * closer to the exact transform than any FP64 FFT. */
static long double oc_cas(size_t r, size_t N)
{
    const long double a = 6.283185307179586476925286766559005768L * (long double)r / (long double)N;
    return cosl(a) + sinl(a);
}

/* In-place separable DHT over the axes of a dim-D array (x fastest). */
static void oc_dht(const oc_t *o, double *data)
{
    int a;
    size_t total = o->Ns;
    for (a = 0; a < o->dim; ++a) {
        const size_t N = o->N[a];
        size_t stride = 1, b, lines, l, j, k;
        long double *cas_t = (long double *)malloc(sizeof(long double) * N * N);
        long double *cas_r = (long double *)malloc(sizeof(long double) * N);
        double *tmp = (double *)malloc(sizeof(double) * N);
        for (b = 0; b < (size_t)a; ++b) stride *= o->N[b];
        lines = total / N;
        /* cas(2 pi j k / N) takes N distinct values, one per (j k) mod N */
        for (j = 0; j < N; ++j) cas_r[j] = oc_cas(j, N);
        for (j = 0; j < N; ++j)
            for (k = 0; k < N; ++k) cas_t[j * N + k] = cas_r[(j * k) % N];
        free(cas_r);
        for (l = 0; l < lines; ++l) {
            const size_t lo = l % stride, hi = l / stride;
            double *line = data + hi * stride * N + lo;
            for (k = 0; k < N; ++k) {
                long double acc = 0;
                for (j = 0; j < N; ++j) acc += (long double)line[j * stride] * cas_t[j * N + k];
                tmp[k] = (double)acc;
            }
            for (k = 0; k < N; ++k) line[k * stride] = tmp[k];
        }
        free(cas_t); free(tmp);
    }
}

/* poisson<double>::solve (poisson.cpp:66-89, 190-219, 328-362): in place,
 * returns the electric energy 1/2 int |E|^2. */
static double oc_poisson(const oc_t *o, double *data)
{
    double energy = 0;
    size_t i, j, k;
    const size_t Nx = o->N[0], Ny = o->N[1], Nz = o->N[2];
    const double fac_N = 1.0 / (double)(Nx * Ny * Nz);
    const double fac_x = 2 * M_PI * o->Linv[0];
    const double fac_y = o->dim > 1 ? 2 * M_PI * o->Linv[1] : 0;
    const double fac_z = o->dim > 2 ? 2 * M_PI * o->Linv[2] : 0;
    oc_dht(o, data);
    for (k = 0; k < Nz; ++k)
        for (j = 0; j < Ny; ++j)
            for (i = 0; i < Nx; ++i) {
                const size_t l = (k * Ny + j) * Nx + i;
                double ii, jj, kk, fac;
                if (i == 0 && j == 0 && k == 0) continue;
                ii = (2 * i < Nx) ? (double)i : (double)(Nx - i);
                jj = (2 * j < Ny) ? (double)j : (double)(Ny - j);
                kk = (2 * k < Nz) ? (double)k : (double)(Nz - k);
                if (o->dim == 1) {
                    fac = fac_N / (ii * ii * fac_x * fac_x);
                    data[l] *= fac;
                    { const double Ex = ii * fac_x * data[l]; energy += Ex * Ex; }
                } else if (o->dim == 2) {
                    fac = fac_N / (ii * ii * fac_x * fac_x + jj * jj * fac_y * fac_y);
                    data[l] *= fac;
                    {
                        const double Ex = ii * fac_x * data[l], Ey = jj * fac_y * data[l];
                        energy += Ex * Ex + Ey * Ey;
                    }
                } else {
                    fac = fac_N / (ii * ii * fac_x * fac_x + jj * jj * fac_y * fac_y + kk * kk * fac_z * fac_z);
                    data[l] *= fac;
                    {
                        const double Ex = ii * fac_x * data[l], Ey = jj * fac_y * data[l],
                                     Ez = kk * fac_z * data[l];
                        energy += Ex * Ex + Ey * Ey + Ez * Ez;
                    }
                }
            }
    data[0] = 0;
    oc_dht(o, data);
    {
        double Lprod = 1; int a;
        for (a = 0; a < o->dim; ++a) Lprod *= o->L[a];
        energy *= Lprod / 2;
    }
    return energy;
}

/* Solve the circulant collocation system along one axis:
 *   sum_j N_j(0) c[(i+j) mod N] = phi[i]   (fields.hpp:81-99)
 * for every line.  The reference runs LSMR from a zero start
 * (fields.hpp:133-135, lsmr.tpp:65-222), which converges to the
 * minimum-norm least-squares solution; for even-degree splines (order 3,
 * 5) the system is singular at the Nyquist mode.  Restated here in the
 * eigenbasis of the circulant: direct DFT sums with exactly reduced angles,
 * division by the symbol lambda(k) = sum_j N_j(0) exp(+2 pi i j k / N),
 * modes with |lambda| <= 1e-12 max|lambda| set to zero, inverse DFT. */
static int oc_collocation_axis(const oc_t *o, int a, double *data)
{
    const size_t N = o->N[a];
    const int order = o->order;
    size_t stride = 1, b, lines, l, j, k;
    double Nb[OC_MAX_ORDER], lmax = 0;
    double *cs = (double *)malloc(sizeof(double) * N * 2);
    double *lre = (double *)malloc(sizeof(double) * N * 2);
    double *fre = (double *)malloc(sizeof(double) * N * 2);
    double *lim, *fim, *sn;
    if (!cs || !lre || !fre) { free(cs); free(lre); free(fre); return NUFI_ERR_INVALID; }
    sn = cs + N; lim = lre + N; fim = fre + N;
    for (j = 0; j < N; ++j) {
        const double ang = 2 * M_PI * (double)j / (double)N;
        cs[j] = cos(ang); sn[j] = sin(ang);
    }
    oc_N(order, 0, 0.0, Nb);
    for (k = 0; k < N; ++k) {
        double re = 0, im = 0, m;
        for (j = 0; j < (size_t)order; ++j) {
            const size_t t = (j * k) % N;
            re += Nb[j] * cs[t]; im += Nb[j] * sn[t];
        }
        lre[k] = re; lim[k] = im;
        m = sqrt(re * re + im * im);
        if (m > lmax) lmax = m;
    }
    for (b = 0; b < (size_t)a; ++b) stride *= o->N[b];
    lines = o->Ns / N;
    for (l = 0; l < lines; ++l) {
        const size_t lo = l % stride, hi = l / stride;
        double *line = data + hi * stride * N + lo;
        for (k = 0; k < N; ++k) {  /* forward DFT, exp(-2 pi i j k / N) */
            double re = 0, im = 0;
            for (j = 0; j < N; ++j) {
                const size_t t = (j * k) % N;
                re += line[j * stride] * cs[t];
                im -= line[j * stride] * sn[t];
            }
            {
                const double den = lre[k] * lre[k] + lim[k] * lim[k];
                if (sqrt(den) <= 1e-12 * lmax) { fre[k] = 0; fim[k] = 0; }
                else {
                    fre[k] = (re * lre[k] + im * lim[k]) / den;
                    fim[k] = (im * lre[k] - re * lim[k]) / den;
                }
            }
        }
        for (j = 0; j < N; ++j) {  /* inverse DFT, real part */
            double acc = 0;
            for (k = 0; k < N; ++k) {
                const size_t t = (j * k) % N;
                acc += fre[k] * cs[t] - fim[k] * sn[t];
            }
            line[j * stride] = acc / (double)N;
        }
    }
    free(cs); free(lre); free(fre);
    return NUFI_OK;
}

/* dimN::interpolate (fields.hpp:63-142, 186-300, 352-490): values -> padded
 * slab c[k][j][i] = c~[k mod Nz][j mod Ny][i mod Nx]. */
static int oc_interpolate(const oc_t *o, const double *values, double *slab)
{
    double *tmp = (double *)malloc(sizeof(double) * o->Ns);
    size_t i, j, k;
    const size_t o1 = (size_t)o->order - 1;
    const size_t Px = o->N[0] + o1;
    const size_t Py = o->dim > 1 ? o->N[1] + o1 : 1;
    const size_t Pz = o->dim > 2 ? o->N[2] + o1 : 1;
    int a, st = NUFI_OK;
    if (!tmp) return NUFI_ERR_INVALID;
    memcpy(tmp, values, sizeof(double) * o->Ns);
    for (a = 0; a < o->dim && !st; ++a) st = oc_collocation_axis(o, a, tmp);
    for (k = 0; k < Pz; ++k)
        for (j = 0; j < Py; ++j)
            for (i = 0; i < Px; ++i)
                slab[(k * Py + j) * Px + i] =
                    tmp[((k % o->N[2]) * o->N[1] + (j % o->N[1])) * o->N[0] + (i % o->N[0])];
    free(tmp);
    return st;
}

/* Poisson + interpolation on a copy of rho; returns W via *energy. */
int oracle_field_solve(const nufi_config *cfg, const double *rho, double *slab, double *energy)
{
    oc_t o; double *work; int st;
    st = oc_setup(cfg, &o);
    if (st) return st;
    work = (double *)malloc(sizeof(double) * o.Ns);
    if (!work) return NUFI_ERR_INVALID;
    memcpy(work, rho, sizeof(double) * o.Ns);
    *energy = oc_poisson(&o, work);
    st = oc_interpolate(&o, work, slab);
    free(work);
    return st;
}

/* Poisson alone (for the reference's test_poisson known-answer check). */
int oracle_poisson(const nufi_config *cfg, double *data, double *energy)
{
    oc_t o; int st = oc_setup(cfg, &o);
    if (st) return st;
    *energy = oc_poisson(&o, data);
    return NUFI_OK;
}

/* Interpolation alone (test_fields known-answer check). */
int oracle_interpolate(const nufi_config *cfg, const double *values, double *slab)
{
    oc_t o; int st = oc_setup(cfg, &o);
    if (st) return st;
    return oc_interpolate(&o, values, slab);
}

/* Field value or derivative of one slab at points (fields.hpp eval). */
int oracle_eval_field(const nufi_config *cfg, const double *slab, int64_t npts, const double *pts,
                      const int *deriv, double *out)
{
    oc_t o; int64_t i;
    int st = oc_setup(cfg, &o);
    if (st) return st;
    for (i = 0; i < npts; ++i) {
        const double *x = pts + i * o.dim;
        if (o.dim == 1) out[i] = oc_eval_1d(&o, o.order, x[0], slab, deriv[0]);
        else if (o.dim == 2) out[i] = oc_eval_2d(&o, o.order, x[0], x[1], slab, deriv[0], deriv[1]);
        else out[i] = oc_eval_3d(&o, o.order, x[0], x[1], x[2], slab, deriv[0], deriv[1], deriv[2]);
    }
    return NUFI_OK;
}

/* The driver loop of bin/test_nufi_gpu_{1d,2d,3d}.cpp (1d:241-252,
 * 2d:145-158, 3d:150-162): for n = n0..n1, rho(n) from slabs 0..n-1, then
 * the field solve writes slab n.  rho_hist (optional) gets rho(n) before
 * the solve, Ns values per step, indexed from n0. */
int oracle_run(const nufi_config *cfg, int64_t n0, int64_t n1, double *coeffs, double *energy,
               double *rho_hist, int nthreads)
{
    oc_t o; int64_t n; double *rho; int st = oc_setup(cfg, &o);
    if (st) return st;
    if (n0 < 0 || n1 < n0 || (size_t)n1 > o.Nt) return NUFI_ERR_RANGE;
    rho = (double *)malloc(sizeof(double) * o.Ns);
    if (!rho) return NUFI_ERR_INVALID;
    for (n = n0; n <= n1 && !st; ++n) {
        st = oracle_rho(cfg, n, coeffs, 0, (int64_t)(o.Ns * o.Nm), rho, nthreads);
        if (st) break;
        if (rho_hist) memcpy(rho_hist + (size_t)(n - n0) * o.Ns, rho, sizeof(double) * o.Ns);
        st = oracle_field_solve(cfg, rho, coeffs + (size_t)n * o.stride_t, energy + (n - n0));
    }
    free(rho);
    return st;
}

/* ---- forward-mode derivative of J = 2 dt sum_{n<=n1} W_n (1D) ------------
 * The check of the GPU adjoint: every quantity of the 1D loop carries its
 * derivative with respect to theta = (alpha, k, u_b, sigma_b) (4 tangent
 * directions at once):  per point (x, u) and (dx_i, du_i) through the trace,
 *   x -= dt u              dx_i -= dt du_i
 *   E = -S'_k(x)/dx        dE_i = -S''_k(x)/dx^2 dx_i - dS'_k[dc_k,i](x)/dx
 *   u += h dt E            du_i += h dt dE_i
 * then df~_i = f0_x dx_i + f0_u du_i + df0/dtheta_i at the foot,
 * drho_i = -w sum df~_i, dc_n,i = the (linear) field solve of drho_i, and
 * dW_n,i = L/N sum_s (drho_i - mean drho_i) phi_n (W = L/(2N) rho'.G rho'
 * with G symmetric).  The foot derivatives of f0 are those of nufi_f0.h
 * (k inside f0 only, the domain fixed; x unwrapped, as the reference
 * evaluates f0). */
static void oc_f0_grad_1d(const oc_t *o, double x, double u, double *fx, double *fu, double *dth)
{
    const double alpha = o->p[0], k = o->p[1], c0 = 0.39894228040143267793994;
    const double ck = cos(k * x), sk = sin(k * x), sp = 1. + alpha * ck;
    double g, gu, gub = 0, gsb = 0;
    if (o->f0_kind == NUFI_F0_LANDAU) {
        g = c0 * exp(-u * u / 2); gu = -u * g;
    } else if (o->f0_kind == NUFI_F0_TWO_STREAM) {
        const double e = c0 * exp(-u * u / 2.);
        g = e * u * u; gu = e * u * (2. - u * u);
    } else {
        const double ub = o->p[2], sb = o->p[3], z = (u - ub) / sb;
        const double e1 = c0 * exp(-u * u / 2), e2 = c0 / sb * exp(-z * z / 2);
        g = 0.9 * e1 + 0.1 * e2;
        gu = -0.9 * u * e1 - 0.1 * z / sb * e2;
        gub = 0.1 * z / sb * e2;
        gsb = 0.1 * (z * z - 1.) / sb * e2;
    }
    *fx = -alpha * k * sk * g;
    *fu = sp * gu;
    dth[0] = ck * g; dth[1] = -alpha * x * sk * g; dth[2] = sp * gub; dth[3] = sp * gsb;
}

int oracle_objective_tangent(const nufi_config *cfg, int64_t n1, double *J, double *dJ, int nthreads)
{
    oc_t o; int st = oc_setup(cfg, &o); int64_t n; int i;
    double *coeffs, *dco[4], *rho, *drho[4], *phi, *work;
    if (st) return st;
    if (o.dim != 1) return NUFI_ERR_UNSUPPORTED;
    if (n1 < 0 || (size_t)n1 > o.Nt) return NUFI_ERR_RANGE;
    coeffs = (double *)calloc((o.Nt + 1) * o.stride_t, sizeof(double));
    rho = (double *)malloc(sizeof(double) * o.Ns);
    phi = (double *)malloc(sizeof(double) * o.Ns);
    work = (double *)malloc(sizeof(double) * o.stride_t);
    for (i = 0; i < 4; ++i) {
        dco[i] = (double *)calloc((o.Nt + 1) * o.stride_t, sizeof(double));
        drho[i] = (double *)malloc(sizeof(double) * o.Ns);
    }
    *J = 0;
    for (i = 0; i < 4; ++i) dJ[i] = 0;
    for (n = 0; n <= n1 && !st; ++n) {
        const double w = oc_weight_v(&o);
        long long s;
        double W, mean[4] = {0, 0, 0, 0};
        (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (s = 0; s < (long long)o.Ns; ++s) {
            double acc = 0, dacc[4] = {0, 0, 0, 0};
            size_t m;
            for (m = 0; m < o.Nm; ++m) {
                double x, u, dx[4] = {0, 0, 0, 0}, du[4] = {0, 0, 0, 0}, fx, fu, dth[4];
                size_t k;
                int a;
                { double xx[3], uu[3]; oc_point(&o, (size_t)s, m, xx, uu); x = xx[0]; u = uu[0]; }
                for (k = (size_t)n; k-- > 0;) {
                    const double h = k == 0 ? 0.5 : 1.0;
                    const double *c = coeffs + k * o.stride_t;
                    size_t ii; double xi, w1[OC_MAX_ORDER], w2[OC_MAX_ORDER], S1 = 0, S2 = 0, E, Ep;
                    int j;
                    x = x - o.dt * u;
                    for (a = 0; a < 4; ++a) dx[a] = dx[a] - o.dt * du[a];
                    oc_locate(&o, 0, x, &ii, &xi);
                    oc_N(o.order, 1, xi, w1);
                    oc_N(o.order, 2, xi, w2);
                    for (j = 0; j < o.order; ++j) { S1 += c[ii + j] * w1[j]; S2 += c[ii + j] * w2[j]; }
                    E = -o.dxinv[0] * S1;
                    Ep = -o.dxinv[0] * o.dxinv[0] * S2;
                    for (a = 0; a < 4; ++a) {
                        const double *dc = dco[a] + k * o.stride_t;
                        double dS1 = 0;
                        for (j = 0; j < o.order; ++j) dS1 += dc[ii + j] * w1[j];
                        du[a] = du[a] + h * o.dt * (Ep * dx[a] - o.dxinv[0] * dS1);
                    }
                    u = u + h * o.dt * E;
                }
                { double xx[3] = {x, 0, 0}, uu[3] = {u, 0, 0}; acc += oc_f0(&o, xx, uu); }
                oc_f0_grad_1d(&o, x, u, &fx, &fu, dth);
                for (a = 0; a < 4; ++a) dacc[a] += fx * dx[a] + fu * du[a] + dth[a];
            }
            rho[s] = -w * acc;
            for (i = 0; i < 4; ++i) drho[i][s] = -w * dacc[i];
        }
        /* primal: phi (Poisson in place on a copy) and slab n */
        memcpy(phi, rho, sizeof(double) * o.Ns);
        W = oc_poisson(&o, phi);
        st = oc_interpolate(&o, phi, coeffs + (size_t)n * o.stride_t);
        *J += 2.0 * o.dt * W;
        for (i = 0; i < 4 && !st; ++i) {
            double dW = 0; long long l;
            for (l = 0; l < (long long)o.Ns; ++l) mean[i] += drho[i][l];
            mean[i] /= (double)o.Ns;
            for (l = 0; l < (long long)o.Ns; ++l) dW += (drho[i][l] - mean[i]) * phi[l];
            dJ[i] += 2.0 * o.dt * o.L[0] / (double)o.Ns * dW;
            /* tangent slab: the same linear solve of drho */
            {
                double e;
                memcpy(work, drho[i], sizeof(double) * o.Ns);
                e = oc_poisson(&o, work);
                (void)e;
                st = oc_interpolate(&o, work, dco[i] + (size_t)n * o.stride_t);
            }
        }
    }
    free(coeffs); free(rho); free(phi); free(work);
    for (i = 0; i < 4; ++i) { free(dco[i]); free(drho[i]); }
    return st;
}

int oracle_sizes(const nufi_config *cfg, int64_t *stride_t, int64_t *ns, int64_t *nq)
{
    oc_t o; int st = oc_setup(cfg, &o);
    if (st) return st;
    *stride_t = (int64_t)o.stride_t; *ns = (int64_t)o.Ns; *nq = (int64_t)(o.Ns * o.Nm);
    return NUFI_OK;
}
