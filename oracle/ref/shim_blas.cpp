// Level-1 BLAS behind the reference's nufi::blas wrappers (nufi/blas.hpp),
// which LSMR uses (nufi/lsmr.tpp:47-50, 74-76).  The reference forwards
// them to CBLAS (nufi/blas.cpp:30-116, OpenBLAS 0.3.20 headers vendored,
// library absent); these are plain loops with the documented semantics
// (dot = sum x_i y_i, axpy y += a x, scal x *= a, copy y = x).
// Test infrastructure only.
#include <nufi/blas.hpp>

namespace nufi {
namespace blas {

template <typename real>
static real dot_t(size_t n, const real *x, size_t incx, const real *y, size_t incy)
{
    real r = 0;
    for (size_t i = 0; i < n; ++i) r += x[i * incx] * y[i * incy];
    return r;
}

double dot(const size_t n, const double *x, size_t incx, const double *y, size_t incy)
{ return dot_t(n, x, incx, y, incy); }
float dot(const size_t n, const float *x, size_t incx, const float *y, size_t incy)
{ return dot_t(n, x, incx, y, incy); }

void axpy(size_t n, double a, const double *x, size_t incx, double *y, size_t incy)
{ for (size_t i = 0; i < n; ++i) y[i * incy] += a * x[i * incx]; }
void axpy(size_t n, float a, const float *x, size_t incx, float *y, size_t incy)
{ for (size_t i = 0; i < n; ++i) y[i * incy] += a * x[i * incx]; }

void scal(size_t n, double a, double *x, size_t incx)
{ for (size_t i = 0; i < n; ++i) x[i * incx] *= a; }
void scal(size_t n, float a, float *x, size_t incx)
{ for (size_t i = 0; i < n; ++i) x[i * incx] *= a; }

void copy(size_t n, const double *x, size_t incx, double *y, size_t incy)
{ for (size_t i = 0; i < n; ++i) y[i * incy] = x[i * incx]; }
void copy(size_t n, const float *x, size_t incx, float *y, size_t incy)
{ for (size_t i = 0; i < n; ++i) y[i * incy] = x[i * incx]; }

}  // namespace blas
}  // namespace nufi
