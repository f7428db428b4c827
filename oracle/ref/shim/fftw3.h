/*
 * fftw3.h stand-in for building the reference's nufi/poisson.cpp here.
 * FFTW3 is a third-party dependency of the reference (linked as -lfftw3
 * -lfftw3f, bin/makefile.am:7; version not pinned there) and is not
 * installed.  Only the calls poisson.cpp makes are provided, restated from
 * FFTW's documented definition of the r2r FFTW_DHT kind:
 *   Y_k = sum_j X_j [cos(2 pi j k / n) + sin(2 pi j k / n)]   (unnormalised)
 * applied separably along each dimension for the multi-dimensional plans
 * (FFTW documents multi-dimensional r2r transforms as separable products of
 * the 1D kinds).  Test infrastructure only.
 */
#ifndef NUFI_REF_SHIM_FFTW3_H
#define NUFI_REF_SHIM_FFTW3_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2 } fftw_r2r_kind;
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

typedef struct nufi_shim_dht_plan *fftw_plan;
typedef struct nufi_shim_dht_plan *fftwf_plan;

fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out, fftw_r2r_kind kind, unsigned flags);
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double *in, double *out, fftw_r2r_kind k0,
                           fftw_r2r_kind k1, unsigned flags);
fftw_plan fftw_plan_r2r_3d(int n0, int n1, int n2, double *in, double *out, fftw_r2r_kind k0,
                           fftw_r2r_kind k1, fftw_r2r_kind k2, unsigned flags);
void fftw_execute_r2r(const fftw_plan p, double *in, double *out);
void fftw_destroy_plan(fftw_plan p);

fftwf_plan fftwf_plan_r2r_1d(int n, float *in, float *out, fftw_r2r_kind kind, unsigned flags);
fftwf_plan fftwf_plan_r2r_2d(int n0, int n1, float *in, float *out, fftw_r2r_kind k0,
                             fftw_r2r_kind k1, unsigned flags);
fftwf_plan fftwf_plan_r2r_3d(int n0, int n1, int n2, float *in, float *out, fftw_r2r_kind k0,
                             fftw_r2r_kind k1, fftw_r2r_kind k2, unsigned flags);
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif

#endif
