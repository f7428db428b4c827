/*
 * nufi_f0.h — initial conditions f0 of the NuFI configurations, shared by
 * the oracle (nufi_oracle.c) and the reference build's driver
 * (oracle/ref/ref_driver.cpp) so both evaluate f0 with the same operations.
 * TEST INFRASTRUCTURE ONLY (see nufi_oracle.c).
 *
 * The reference hard-codes f0 as a static member of config_t
 * (nufi/config.hpp:72-84, 140-159, 221-247); the expressions below keep
 * its operation order and constants and take alpha, k (and u_b, sigma_b
 * for the bump-on-tail) at run time:
 *   1D Landau      config.hpp:83   0.398942.. (1 + a cos kx) exp(-u u/2)
 *   1D two-stream  config.hpp:82   0.398942.. (1 + a cos kx) exp(-u u/2.) u u
 *   2D Landau      config.hpp:148  1/(2 pi) exp(-(u u + v v)/2) (1 + a (cos kx + cos ky))
 *   3D Landau      config.hpp:233-234 (2 pi)^-3/2 (1 + a cos kx + a cos ky + a cos kz) exp(-|v|^2/2)
 */
#ifndef NUFI_F0_H
#define NUFI_F0_H

#include <math.h>
#include "../include/nufi_gb300.h"

typedef struct {
    int kind;
    double p[8];
} nufi_f0_params;

static inline double nufi_f0_1d(const nufi_f0_params *f, double x, double u)
{
    const double alpha = f->p[0], k = f->p[1];
    if (f->kind == NUFI_F0_LANDAU)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2);
    if (f->kind == NUFI_F0_TWO_STREAM)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2.) * u * u;
    if (f->kind == NUFI_F0_BUMP_ON_TAIL) {
        const double ub = f->p[2], sb = f->p[3];
        const double z = (u - ub) / sb;
        return (1. + alpha * cos(k * x)) *
               (0.9 * 0.39894228040143267793994 * exp(-u * u / 2) +
                0.1 * 0.39894228040143267793994 / sb * exp(-z * z / 2));
    }
    return NAN;
}

static inline double nufi_f0_2d(const nufi_f0_params *f, double x, double y, double u, double v)
{
    const double alpha = f->p[0], k = f->p[1];
    if (f->kind == NUFI_F0_LANDAU)
        return 1.0 / (2.0 * M_PI) * exp(-0.5 * (u * u + v * v)) *
               (1 + alpha * (cos(k * x) + cos(k * y)));
    return NAN;
}

static inline double nufi_f0_3d(const nufi_f0_params *f, double x, double y, double z, double u,
                                double v, double w)
{
    const double alpha = f->p[0], k = f->p[1];
    if (f->kind == NUFI_F0_LANDAU)
        return 0.06349363593424096978576330493464 *
               (1. + alpha * cos(k * x) + alpha * cos(k * y) + alpha * cos(k * z)) *
               exp(-(u * u + v * v + w * w) / 2);
    if (f->kind == NUFI_F0_BUMP_ON_TAIL) {
        /* the reference's compiled-in 3D f0 (config.hpp:80-82), with
         * alpha, k, u_b, sigma_b at run time: 0.1 / sigma_b = 0.2 and
         * 1 / (2 sigma_b^2) = 2 there, in the same operation order */
        const double ub = f->p[2], sb = f->p[3], a = 1 / (2 * sb * sb);
        return 0.06349363593424096978576330493464 *
               (0.9 * exp(-0.5 * u * u) + 0.1 / sb * exp(-a * (u - ub) * (u - ub))) *
               exp(-0.5 * (v * v + w * w)) * (1 + alpha * (cos(k * x) + cos(k * y) + cos(k * z)));
    }
    return NAN;
}

#endif
