// ref_driver.cpp — runs the REFERENCE's own hot-path code (nufi/rho.hpp,
// nufi/fields.hpp, nufi/splines.hpp, nufi/lsmr.tpp, nufi/poisson.cpp,
// included and compiled where they lie) on a runtime configuration, to pin
// the oracle and to produce the golden vectors under tests/golden/.
// Test infrastructure only; built by oracle/ref/Makefile into oracle/_ref/.
//
// The reference hard-codes f0 as config_t<real>::f0 (nufi/config.hpp:72-84,
// 140-159, 221-247).  This driver supplies the configured f0 through an
// explicit specialisation of that member for real = double, declared
// before any use; everything else is the reference's code unchanged.
//
// NUFI_REF_SUMMATION=1 in the environment sums rho compensated (see
// rho_sum); the default is the reference's in-order sum.
// Usage:
//   ref_driver run   <cfg.bin> <n0> <n1> <out_prefix> [threads]
//       steps n0..n1 of the loop of bin/test_nufi_gpu_{1d,2d,3d}.cpp with
//       rho formed by the GPU kernels' point convention
//       (nufi/cuda_kernel.cu:31-51, 210-237, 392-426); writes
//       <out>.energy (n1-n0+1 doubles), <out>.rho ((n1-n0+1)*Ns doubles),
//       <out>.coeffs ((Nt+1)*stride_t doubles).
//   ref_driver solve <cfg.bin> <rho.bin> <out_prefix>
//       poisson<double>::solve + interpolate<double,order>; writes
//       <out>.slab and <out>.energy.
//   ref_driver metrics <cfg.bin> <coeffs.bin> <n> <out_prefix>
//       the four sums of cuda_eval_metrics (nufi/cuda_kernel.cu:53-79,
//       239-271, 428-466) over all q, f from the reference's eval_f
//       (nufi/rho.hpp:63-93, 234-, 369-); per-node sums in q order, nodes
//       summed in order; writes <out>.metrics (4 doubles).
//   ref_driver rho <cfg.bin> <coeffs.bin> <n> <out_prefix> <reps>
//       rho of step n (as in run), reps times; writes <out>.rho and prints
//       the best wall time of the trace in seconds.
//   ref_driver points <cfg.bin> <coeffs.bin> <n> <mode> <pts.bin> <out_prefix>
//       eval_ftilda (mode 0), eval_f (1) or the 1D eval_phase_flow (2) at
//       points (x.., v..); writes <out>.f and <out>.pts (moved by mode 2).
//   ref_driver poisson_kat        bin/test_poisson.cpp's analytic check
//   ref_driver fields_kat         bin/test_fields.cpp's checks at nodes
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <nufi/config.hpp>

#include "../../include/nufi_gb300.h"
#include "../nufi_f0.h"

static nufi_f0_params g_f0;
// 0: rho summed in q order (as the reference's CPU loop); 1: Neumaier
// compensated, i.e. the same f~ values summed to ~1 ulp.
static int g_sum_mode = 0;

struct rho_sum {
    double acc = 0, comp = 0;
    void add(double f)
    {
        if (g_sum_mode == 1) {
            const double t = acc + f;
            comp += (std::abs(acc) >= std::abs(f)) ? (acc - t) + f : (f - t) + acc;
            acc = t;
        } else {
            acc += f;
        }
    }
    double value() const { return acc + comp; }
};

// Built with NUFI_REF_NATIVE_F0 (ref_driver_native), the driver keeps the
// reference's own compiled-in f0 of each dimension instead (config.hpp:
// 1D u^2 M two-stream, 2D Landau alpha = k = 0.5, 3D bump-on-tail), and the
// configured f0 is ignored.
#ifndef NUFI_REF_NATIVE_F0
namespace nufi {
namespace dim1 {
template <> __host__ __device__ double config_t<double>::f0(double x, double u) noexcept
{ return nufi_f0_1d(&g_f0, x, u); }
}  // namespace dim1
namespace dim2 {
template <> __host__ __device__ double config_t<double>::f0(double x, double y, double u, double v) noexcept
{ return nufi_f0_2d(&g_f0, x, y, u, v); }
}  // namespace dim2
namespace dim3 {
template <> __host__ __device__ double config_t<double>::f0(double x, double y, double z, double u, double v,
                                                          double w) noexcept
{ return nufi_f0_3d(&g_f0, x, y, z, u, v, w); }
}  // namespace dim3
}  // namespace nufi
#endif

#include <nufi/fields.hpp>
#include <nufi/poisson.hpp>
#include <nufi/rho.hpp>

namespace {

bool read_file(const char *path, void *dst, size_t bytes)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    const size_t got = std::fread(dst, 1, bytes, f);
    std::fclose(f);
    return got == bytes;
}

void write_file(const std::string &path, const void *src, size_t bytes)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    std::fwrite(src, 1, bytes, f);
    std::fclose(f);
}

// config_t setup exactly as the constructors derive the grid quantities
// (nufi/config.hpp:67-69, 132-137, 210-218).
void fill(nufi::dim1::config_t<double> &c, const nufi_config &k)
{
    c.Nx = k.Nx[0]; c.Nu = k.Nv[0]; c.Nt = k.Nt; c.dt = k.dt;
    c.x_min = k.x_min[0]; c.x_max = k.x_max[0]; c.u_min = k.v_min[0]; c.u_max = k.v_max[0];
    c.Lx = c.x_max - c.x_min; c.Lx_inv = 1 / c.Lx;
    c.dx = c.Lx / c.Nx; c.dx_inv = 1 / c.dx;
    c.du = (c.u_max - c.u_min) / c.Nu;
}
void fill(nufi::dim2::config_t<double> &c, const nufi_config &k)
{
    c.Nx = k.Nx[0]; c.Ny = k.Nx[1]; c.Nu = k.Nv[0]; c.Nv = k.Nv[1]; c.Nt = k.Nt; c.dt = k.dt;
    c.x_min = k.x_min[0]; c.x_max = k.x_max[0]; c.y_min = k.x_min[1]; c.y_max = k.x_max[1];
    c.u_min = k.v_min[0]; c.u_max = k.v_max[0]; c.v_min = k.v_min[1]; c.v_max = k.v_max[1];
    c.Lx = c.x_max - c.x_min; c.Lx_inv = 1 / c.Lx;
    c.Ly = c.y_max - c.y_min; c.Ly_inv = 1 / c.Ly;
    c.dx = c.Lx / c.Nx; c.dx_inv = 1 / c.dx;
    c.dy = c.Ly / c.Ny; c.dy_inv = 1 / c.dy;
    c.du = (c.u_max - c.u_min) / c.Nu;
    c.dv = (c.v_max - c.v_min) / c.Nv;
}
void fill(nufi::dim3::config_t<double> &c, const nufi_config &k)
{
    c.Nx = k.Nx[0]; c.Ny = k.Nx[1]; c.Nz = k.Nx[2];
    c.Nu = k.Nv[0]; c.Nv = k.Nv[1]; c.Nw = k.Nv[2]; c.Nt = k.Nt; c.dt = k.dt;
    c.x_min = k.x_min[0]; c.x_max = k.x_max[0]; c.y_min = k.x_min[1]; c.y_max = k.x_max[1];
    c.z_min = k.x_min[2]; c.z_max = k.x_max[2];
    c.u_min = k.v_min[0]; c.u_max = k.v_max[0]; c.v_min = k.v_min[1]; c.v_max = k.v_max[1];
    c.w_min = k.v_min[2]; c.w_max = k.v_max[2];
    c.Lx = c.x_max - c.x_min; c.Lx_inv = 1 / c.Lx;
    c.Ly = c.y_max - c.y_min; c.Ly_inv = 1 / c.Ly;
    c.Lz = c.z_max - c.z_min; c.Lz_inv = 1 / c.Lz;
    c.dx = c.Lx / c.Nx; c.dx_inv = 1 / c.dx;
    c.dy = c.Ly / c.Ny; c.dy_inv = 1 / c.dy;
    c.dz = c.Lz / c.Nz; c.dz_inv = 1 / c.dz;
    c.du = (c.u_max - c.u_min) / c.Nu;
    c.dv = (c.v_max - c.v_min) / c.Nv;
    c.dw = (c.w_max - c.w_min) / c.Nw;
}

// rho by the GPU kernels' point convention, summed in q order per node.
template <size_t order>
void rho_1d(size_t n, const double *coeffs, const nufi::dim1::config_t<double> &conf, double *rho)
{
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t ix = 0; ix < conf.Nx; ++ix) {
        rho_sum acc;
        for (size_t iu = 0; iu < conf.Nu; ++iu) {
            const double x = conf.x_min + ix * conf.dx;
            const double u = conf.u_min + iu * conf.du + conf.du / 2;
            acc.add(nufi::dim1::eval_ftilda<double, order>(n, x, u, coeffs, conf));
        }
        rho[ix] = -conf.du * acc.value();
    }
}

template <size_t order>
void rho_2d(size_t n, const double *coeffs, const nufi::dim2::config_t<double> &conf, double *rho)
{
    const size_t Ns = conf.Nx * conf.Ny;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t s = 0; s < Ns; ++s) {
        const size_t ix = s % conf.Nx, iy = s / conf.Nx;
        rho_sum acc;
        for (size_t iv = 0; iv < conf.Nv; ++iv)
            for (size_t iu = 0; iu < conf.Nu; ++iu) {
                const double x = conf.x_min + ix * conf.dx;
                const double y = conf.y_min + iy * conf.dy;
                const double u = conf.u_min + iu * conf.du + conf.du / 2;
                const double v = conf.v_min + iv * conf.dv + conf.dv / 2;
                acc.add(nufi::dim2::eval_ftilda<double, order>(n, x, y, u, v, coeffs, conf));
            }
        rho[s] = -(conf.du * conf.dv) * acc.value();
    }
}

template <size_t order>
void rho_3d(size_t n, const double *coeffs, const nufi::dim3::config_t<double> &conf, double *rho)
{
    const size_t Ns = conf.Nx * conf.Ny * conf.Nz;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t s = 0; s < Ns; ++s) {
        const size_t ix = s % conf.Nx, iy = (s / conf.Nx) % conf.Ny, iz = s / (conf.Nx * conf.Ny);
        rho_sum acc;
        for (size_t iw = 0; iw < conf.Nw; ++iw)
            for (size_t iv = 0; iv < conf.Nv; ++iv)
                for (size_t iu = 0; iu < conf.Nu; ++iu) {
                    const double x = conf.x_min + ix * conf.dx;
                    const double y = conf.y_min + iy * conf.dy;
                    const double z = conf.z_min + iz * conf.dz;
                    const double u = conf.u_min + iu * conf.du + conf.du / 2;
                    const double v = conf.v_min + iv * conf.dv + conf.dv / 2;
                    const double w = conf.w_min + iw * conf.dw + conf.dw / 2;
                    acc.add(nufi::dim3::eval_ftilda<double, order>(n, x, y, z, u, v, w, coeffs, conf));
                }
        rho[s] = -(conf.du * conf.dv * conf.dw) * acc.value();
    }
}

void rho_any(const nufi_config &k, size_t n, const double *coeffs, double *rho)
{
#define NUFI_REF_ORDER_CASE(O)                                               \
    case O:                                                                   \
        if (k.dim == 1) { nufi::dim1::config_t<double> c; fill(c, k); rho_1d<O>(n, coeffs, c, rho); } \
        else if (k.dim == 2) { nufi::dim2::config_t<double> c; fill(c, k); rho_2d<O>(n, coeffs, c, rho); } \
        else { nufi::dim3::config_t<double> c; fill(c, k); rho_3d<O>(n, coeffs, c, rho); } \
        return;
    switch (k.order) {
        NUFI_REF_ORDER_CASE(3)
        NUFI_REF_ORDER_CASE(4)
        NUFI_REF_ORDER_CASE(5)
        NUFI_REF_ORDER_CASE(6)
        NUFI_REF_ORDER_CASE(7)
        NUFI_REF_ORDER_CASE(8)
    default: std::fprintf(stderr, "order %d not built\n", k.order); std::exit(2);
    }
#undef NUFI_REF_ORDER_CASE
}

// Metrics by the GPU kernels' point order, weights and expressions.
struct metric_sums {
    double m[4] = {0, 0, 0, 0};
    void add(double weight, double f, double uu)
    {
        m[0] += weight * f;
        m[1] += weight * f * f;
        m[2] += weight * (uu * f / 2);
        m[3] += (f > 0) ? -weight * f * std::log(f) : 0;
    }
};

template <size_t order>
void metrics_1d(size_t n, const double *coeffs, const nufi::dim1::config_t<double> &conf, double *out)
{
    std::vector<metric_sums> per(conf.Nx);
    const double weight = conf.du * conf.dx;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t ix = 0; ix < conf.Nx; ++ix)
        for (size_t iu = 0; iu < conf.Nu; ++iu) {
            const double x = conf.x_min + ix * conf.dx;
            const double u = conf.u_min + iu * conf.du + conf.du / 2;
            per[ix].add(weight, nufi::dim1::eval_f<double, order>(n, x, u, coeffs, conf), u * u);
        }
    for (auto &p : per)
        for (int k = 0; k < 4; ++k) out[k] += p.m[k];
}

template <size_t order>
void metrics_2d(size_t n, const double *coeffs, const nufi::dim2::config_t<double> &conf, double *out)
{
    const size_t Ns = conf.Nx * conf.Ny;
    std::vector<metric_sums> per(Ns);
    const double weight = conf.dx * conf.dy * conf.du * conf.dv;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t s = 0; s < Ns; ++s) {
        const size_t ix = s % conf.Nx, iy = s / conf.Nx;
        for (size_t iv = 0; iv < conf.Nv; ++iv)
            for (size_t iu = 0; iu < conf.Nu; ++iu) {
                const double x = conf.x_min + ix * conf.dx, y = conf.y_min + iy * conf.dy;
                const double u = conf.u_min + iu * conf.du + conf.du / 2;
                const double v = conf.v_min + iv * conf.dv + conf.dv / 2;
                per[s].add(weight, nufi::dim2::eval_f<double, order>(n, x, y, u, v, coeffs, conf), u * u + v * v);
            }
    }
    for (auto &p : per)
        for (int k = 0; k < 4; ++k) out[k] += p.m[k];
}

template <size_t order>
void metrics_3d(size_t n, const double *coeffs, const nufi::dim3::config_t<double> &conf, double *out)
{
    const size_t Ns = conf.Nx * conf.Ny * conf.Nz;
    std::vector<metric_sums> per(Ns);
    const double weight = conf.du * conf.dv * conf.dw;
#pragma omp parallel for schedule(dynamic, 1)
    for (size_t s = 0; s < Ns; ++s) {
        const size_t ix = s % conf.Nx, iy = (s / conf.Nx) % conf.Ny, iz = s / (conf.Nx * conf.Ny);
        for (size_t iw = 0; iw < conf.Nw; ++iw)
            for (size_t iv = 0; iv < conf.Nv; ++iv)
                for (size_t iu = 0; iu < conf.Nu; ++iu) {
                    const double x = conf.x_min + ix * conf.dx, y = conf.y_min + iy * conf.dy;
                    const double z = conf.z_min + iz * conf.dz;
                    const double u = conf.u_min + iu * conf.du + conf.du / 2;
                    const double v = conf.v_min + iv * conf.dv + conf.dv / 2;
                    const double w = conf.w_min + iw * conf.dw + conf.dw / 2;
                    per[s].add(weight, nufi::dim3::eval_f<double, order>(n, x, y, z, u, v, w, coeffs, conf),
                               u * u + v * v + w * w);
                }
    }
    for (auto &p : per)
        for (int k = 0; k < 4; ++k) out[k] += p.m[k];
}

void metrics_any(const nufi_config &k, size_t n, const double *coeffs, double *out)
{
#define NUFI_REF_ORDER_CASE(O)                                               \
    case O:                                                                   \
        if (k.dim == 1) { nufi::dim1::config_t<double> c; fill(c, k); metrics_1d<O>(n, coeffs, c, out); } \
        else if (k.dim == 2) { nufi::dim2::config_t<double> c; fill(c, k); metrics_2d<O>(n, coeffs, c, out); } \
        else { nufi::dim3::config_t<double> c; fill(c, k); metrics_3d<O>(n, coeffs, c, out); } \
        return;
    switch (k.order) {
        NUFI_REF_ORDER_CASE(3)
        NUFI_REF_ORDER_CASE(4)
        NUFI_REF_ORDER_CASE(5)
        NUFI_REF_ORDER_CASE(6)
        NUFI_REF_ORDER_CASE(7)
        NUFI_REF_ORDER_CASE(8)
    default: std::fprintf(stderr, "order %d not built\n", k.order); std::exit(2);
    }
#undef NUFI_REF_ORDER_CASE
}

// poisson<double>::solve then interpolate<double,order>, as the drivers do
// (bin/test_nufi_gpu_1d.cpp:248-249; _2d.cpp:156-157; _3d.cpp:160-161).
double solve_any(const nufi_config &k, double *rho, double *slab)
{
#define NUFI_REF_ORDER_CASE(O)                                                          \
    case O:                                                                              \
        if (k.dim == 1) { nufi::dim1::config_t<double> c; fill(c, k);                    \
            nufi::dim1::poisson<double> p(c); double e = p.solve(rho);                   \
            nufi::dim1::interpolate<double, O>(slab, rho, c); return e; }                 \
        else if (k.dim == 2) { nufi::dim2::config_t<double> c; fill(c, k);               \
            nufi::dim2::poisson<double> p(c); double e = p.solve(rho);                   \
            nufi::dim2::interpolate<double, O>(slab, rho, c); return e; }                 \
        else { nufi::dim3::config_t<double> c; fill(c, k);                               \
            nufi::dim3::poisson<double> p(c); double e = p.solve(rho);                   \
            nufi::dim3::interpolate<double, O>(slab, rho, c); return e; }
    switch (k.order) {
        NUFI_REF_ORDER_CASE(3)
        NUFI_REF_ORDER_CASE(4)
        NUFI_REF_ORDER_CASE(5)
        NUFI_REF_ORDER_CASE(6)
        NUFI_REF_ORDER_CASE(7)
        NUFI_REF_ORDER_CASE(8)
    default: std::fprintf(stderr, "order %d not built\n", k.order); std::exit(2);
    }
#undef NUFI_REF_ORDER_CASE
}

size_t slab_size(const nufi_config &k)
{
    size_t s = 1;
    for (int d = 0; d < k.dim; ++d) s *= size_t(k.Nx[d] + k.order - 1);
    return s;
}

size_t spatial_size(const nufi_config &k)
{
    size_t s = 1;
    for (int d = 0; d < k.dim; ++d) s *= size_t(k.Nx[d]);
    return s;
}

int cmd_run(int argc, char **argv)
{
    if (argc < 6) return 2;
    nufi_config k;
    if (!read_file(argv[2], &k, sizeof(k))) { std::fprintf(stderr, "bad config\n"); return 2; }
    const size_t n0 = std::strtoull(argv[3], nullptr, 10), n1 = std::strtoull(argv[4], nullptr, 10);
    const std::string out = argv[5];
    g_f0.kind = k.f0_kind;
    for (int i = 0; i < 8; ++i) g_f0.p[i] = k.f0_params[i];
    const size_t st = slab_size(k), Ns = spatial_size(k);
    std::vector<double> coeffs((k.Nt + 1) * st, 0.0), rho(Ns), energy, rho_hist;
    if (n0 > 0) {  // continue from a given history
        if (!read_file((out + ".coeffs_in").c_str(), coeffs.data(), sizeof(double) * coeffs.size())) {
            std::fprintf(stderr, "n0 > 0 needs <out>.coeffs_in\n"); return 2;
        }
    }
    for (size_t n = n0; n <= n1; ++n) {
        rho_any(k, n, coeffs.data(), rho.data());
        rho_hist.insert(rho_hist.end(), rho.begin(), rho.end());
        energy.push_back(solve_any(k, rho.data(), coeffs.data() + n * st));
    }
    write_file(out + ".energy", energy.data(), sizeof(double) * energy.size());
    write_file(out + ".rho", rho_hist.data(), sizeof(double) * rho_hist.size());
    write_file(out + ".coeffs", coeffs.data(), sizeof(double) * coeffs.size());
    return 0;
}

int cmd_solve(int argc, char **argv)
{
    if (argc < 5) return 2;
    nufi_config k;
    if (!read_file(argv[2], &k, sizeof(k))) return 2;
    const size_t st = slab_size(k), Ns = spatial_size(k);
    std::vector<double> rho(Ns), slab(st, 0.0);
    if (!read_file(argv[3], rho.data(), sizeof(double) * Ns)) return 2;
    double e = solve_any(k, rho.data(), slab.data());
    write_file(std::string(argv[4]) + ".slab", slab.data(), sizeof(double) * st);
    write_file(std::string(argv[4]) + ".energy", &e, sizeof(double));
    return 0;
}

int cmd_metrics(int argc, char **argv)
{
    if (argc < 6) return 2;
    nufi_config k;
    if (!read_file(argv[2], &k, sizeof(k))) return 2;
    g_f0.kind = k.f0_kind;
    for (int i = 0; i < 8; ++i) g_f0.p[i] = k.f0_params[i];
    std::vector<double> coeffs((k.Nt + 1) * slab_size(k));
    if (!read_file(argv[3], coeffs.data(), sizeof(double) * coeffs.size())) return 2;
    const size_t n = std::strtoull(argv[4], nullptr, 10);
    double m[4] = {0, 0, 0, 0};
    metrics_any(k, n, coeffs.data(), m);
    write_file(std::string(argv[5]) + ".metrics", m, sizeof(m));
    return 0;
}

// The reference's point functions at arbitrary points (x.., v..) of step n:
// mode 0 eval_ftilda, 1 eval_f (nufi/rho.hpp:31-96, 191-281, 318-426),
// 2 the 1D eval_phase_flow (rho.hpp:98-131), which moves the point.
template <size_t order>
void points_order(const nufi_config &k, size_t n, int mode, const double *coeffs, double *pts, size_t npts,
                  double *f)
{
    const int D = k.dim;
    if (D == 1) {
        nufi::dim1::config_t<double> c;
        fill(c, k);
        for (size_t i = 0; i < npts; ++i) {
            double &x = pts[2 * i], &u = pts[2 * i + 1];
            if (mode == 0) f[i] = nufi::dim1::eval_ftilda<double, order>(n, x, u, coeffs, c);
            else if (mode == 1) f[i] = nufi::dim1::eval_f<double, order>(n, x, u, coeffs, c);
            else nufi::dim1::eval_phase_flow<double, order>(n, x, u, coeffs, c);
        }
    } else if (D == 2) {
        nufi::dim2::config_t<double> c;
        fill(c, k);
        for (size_t i = 0; i < npts; ++i) {
            const double *q = pts + 4 * i;
            f[i] = mode == 0 ? nufi::dim2::eval_ftilda<double, order>(n, q[0], q[1], q[2], q[3], coeffs, c)
                             : nufi::dim2::eval_f<double, order>(n, q[0], q[1], q[2], q[3], coeffs, c);
        }
    } else {
        nufi::dim3::config_t<double> c;
        fill(c, k);
        for (size_t i = 0; i < npts; ++i) {
            const double *q = pts + 6 * i;
            f[i] = mode == 0
                       ? nufi::dim3::eval_ftilda<double, order>(n, q[0], q[1], q[2], q[3], q[4], q[5], coeffs, c)
                       : nufi::dim3::eval_f<double, order>(n, q[0], q[1], q[2], q[3], q[4], q[5], coeffs, c);
        }
    }
}

// ref_driver points <cfg> <hist> <n> <mode> <pts file> <out>: writes
// <out>.f (f per point) and <out>.pts (the points, moved by mode 2).
int cmd_points(int argc, char **argv)
{
    if (argc < 8) return 2;
    nufi_config k;
    if (!read_file(argv[2], &k, sizeof(k))) return 2;
    g_f0.kind = k.f0_kind;
    for (int i = 0; i < 8; ++i) g_f0.p[i] = k.f0_params[i];
    std::vector<double> coeffs((k.Nt + 1) * slab_size(k));
    if (!read_file(argv[3], coeffs.data(), sizeof(double) * coeffs.size())) return 2;
    const size_t n = std::strtoull(argv[4], nullptr, 10);
    const int mode = std::atoi(argv[5]);
    if (mode == 2 && k.dim != 1) return 2;
    FILE *fp = std::fopen(argv[6], "rb");
    if (!fp) return 2;
    std::vector<double> pts;
    double v;
    while (std::fread(&v, sizeof(double), 1, fp) == 1) pts.push_back(v);
    std::fclose(fp);
    const size_t npts = pts.size() / size_t(2 * k.dim);
    std::vector<double> f(npts, 0.0);
    switch (k.order) {
#define NUFI_REF_ORDER_CASE(O) \
    case O: points_order<O>(k, n, mode, coeffs.data(), pts.data(), npts, f.data()); break;
        NUFI_REF_ORDER_CASE(3)
        NUFI_REF_ORDER_CASE(4)
        NUFI_REF_ORDER_CASE(5)
        NUFI_REF_ORDER_CASE(6)
        NUFI_REF_ORDER_CASE(7)
        NUFI_REF_ORDER_CASE(8)
#undef NUFI_REF_ORDER_CASE
    default: return 2;
    }
    write_file(std::string(argv[7]) + ".f", f.data(), sizeof(double) * f.size());
    write_file(std::string(argv[7]) + ".pts", pts.data(), sizeof(double) * pts.size());
    return 0;
}

// rho of step n from a given history, `reps` times: writes rho and prints
// the best wall time in seconds (the trace alone, for timing the
// reference's own CPU trace beside the oracle's on the same cores).
int cmd_rho(int argc, char **argv)
{
    if (argc < 7) return 2;
    nufi_config k;
    if (!read_file(argv[2], &k, sizeof(k))) return 2;
    g_f0.kind = k.f0_kind;
    for (int i = 0; i < 8; ++i) g_f0.p[i] = k.f0_params[i];
    std::vector<double> coeffs((k.Nt + 1) * slab_size(k)), rho(spatial_size(k));
    if (!read_file(argv[3], coeffs.data(), sizeof(double) * coeffs.size())) return 2;
    const size_t n = std::strtoull(argv[4], nullptr, 10);
    const int reps = std::atoi(argv[6]);
    double best = 1e300;
    for (int r = 0; r < reps; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        rho_any(k, n, coeffs.data(), rho.data());
        best = std::min(best, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    write_file(std::string(argv[5]) + ".rho", rho.data(), sizeof(double) * rho.size());
    std::printf("%.9f\n", best);
    return 0;
}

// bin/test_poisson.cpp:36-119: rho = cos2z + sin8y + cos42x on 128x64x32.
template <typename real>
double poisson_kat()
{
    nufi::dim3::config_t<real> conf;
    conf.Nx = 128; conf.x_min = 0; conf.x_max = 2 * M_PI;
    conf.Lx = conf.x_max - conf.x_min; conf.Lx_inv = 1 / conf.Lx;
    conf.dx = conf.Lx / conf.Nx; conf.dx_inv = 1 / conf.dx;
    conf.Ny = 64; conf.y_min = 0; conf.y_max = 2 * M_PI;
    conf.Ly = conf.y_max - conf.y_min; conf.Ly_inv = 1 / conf.Ly;
    conf.dy = conf.Ly / conf.Ny; conf.dy_inv = 1 / conf.dy;
    conf.Nz = 32; conf.z_min = 0; conf.z_max = 2 * M_PI;
    conf.Lz = conf.z_max - conf.z_min; conf.Lz_inv = 1 / conf.Lz;
    conf.dz = conf.Lz / conf.Nz; conf.dz_inv = 1 / conf.dz;
    nufi::dim3::poisson<real> pois(conf);
    std::vector<real> data(conf.Nx * conf.Ny * conf.Nz);
    for (size_t k = 0; k < conf.Nz; ++k)
        for (size_t j = 0; j < conf.Ny; ++j)
            for (size_t i = 0; i < conf.Nx; ++i) {
                real x = conf.x_min + i * conf.dx, y = conf.y_min + j * conf.dy, z = conf.z_min + k * conf.dz;
                data[i + j * conf.Nx + k * conf.Nx * conf.Ny] = std::cos(2 * z) + std::sin(8 * y) + std::cos(42 * x);
            }
    pois.solve(data.data());
    real l1_err = 0, l1_norm = 0;
    for (size_t k = 0; k < conf.Nz; ++k)
        for (size_t j = 0; j < conf.Ny; ++j)
            for (size_t i = 0; i < conf.Nx; ++i) {
                real x = conf.x_min + i * conf.dx, y = conf.y_min + j * conf.dy, z = conf.z_min + k * conf.dz;
                real exact = std::cos(2 * z) / 4 + std::sin(8 * y) / 64 + std::cos(42 * x) / (42 * 42);
                l1_err += std::abs(data[i + j * conf.Nx + k * conf.Nx * conf.Ny] - exact);
                l1_norm += std::abs(exact);
            }
    return double(l1_err / l1_norm);
}

// bin/test_fields.cpp:129-204 (2D part, nodes only): interpolate
// sin3x + sin3y on 128x128 and evaluate back at the nodes.
double fields_kat_2d()
{
    nufi::dim2::config_t<double> conf;
    conf.Nx = 128; conf.x_min = 0; conf.x_max = 4 * M_PI;
    conf.Lx = conf.x_max - conf.x_min; conf.Lx_inv = 1 / conf.Lx;
    conf.dx = double(conf.Lx) / conf.Nx; conf.dx_inv = 1 / conf.dx;
    conf.Ny = 128; conf.y_min = -M_PI; conf.y_max = M_PI;
    conf.Ly = conf.y_max - conf.y_min; conf.Ly_inv = 1 / conf.Ly;
    conf.dy = double(conf.Ly) / conf.Ny; conf.dy_inv = 1 / conf.dy;
    std::vector<double> values(conf.Nx * conf.Ny), coeffs((conf.Nx + 3) * (conf.Ny + 3));
    for (size_t l = 0; l < conf.Nx * conf.Ny; ++l) {
        size_t j = l / conf.Nx, i = l % conf.Nx;
        values[l] = std::sin(3 * (conf.x_min + i * conf.dx)) + std::sin(3 * (conf.y_min + j * conf.dy));
    }
    nufi::dim2::interpolate<double, 4>(coeffs.data(), values.data(), conf);
    double max_err = 0;
    for (size_t l = 0; l < conf.Nx * conf.Ny; ++l) {
        size_t j = l / conf.Nx, i = l % conf.Nx;
        double val = nufi::dim2::eval<double, 4>(conf.x_min + i * conf.dx, conf.y_min + j * conf.dy, coeffs.data(), conf);
        max_err = std::max(max_err, std::abs(val - values[l]));
    }
    return max_err;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_driver run|solve|metrics|rho|points|poisson_kat|fields_kat ...\n");
        return 2;
    }
    if (const char *m = std::getenv("NUFI_REF_SUMMATION")) g_sum_mode = std::atoi(m);
    const std::string cmd = argv[1];
    if (cmd == "run") return cmd_run(argc, argv);
    if (cmd == "solve") return cmd_solve(argc, argv);
    if (cmd == "metrics") return cmd_metrics(argc, argv);
    if (cmd == "rho") return cmd_rho(argc, argv);
    if (cmd == "points") return cmd_points(argc, argv);
    if (cmd == "poisson_kat") {
        std::printf("{\"float\": %.17g, \"double\": %.17g}\n", poisson_kat<float>(), poisson_kat<double>());
        return 0;
    }
    if (cmd == "fields_kat") {
        std::printf("{\"max_node_error_2d\": %.17g}\n", fields_kat_2d());
        return 0;
    }
    return 2;
}
