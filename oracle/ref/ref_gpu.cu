// ref_gpu.cu — the REFERENCE's own GPU kernels (nufi/cuda_kernel.cu,
// included where it lies and compiled unchanged) built for sm_103a as a
// device-code-only cubin, so that the reference's GPU path can be timed and
// checked beside the new kernels on the same GB300 (ref_gpu.py launches it
// through the CUDA driver API).  Test infrastructure only; built by
// oracle/ref/Makefile into oracle/_ref/.
//
// The reference hard-codes f0 as config_t<real>::f0 (nufi/config.hpp:72-84,
// 140-159, 221-247).  As ref_driver.cpp does for the host code, f0 is
// supplied here by explicit specialisations of that member (1D, 2D, 3D;
// float and double), declared before any use; they read the configured kind
// and parameters from __constant__ memory (set by the launcher) and evaluate
// nufi_f0.h's expressions in double.  Everything else is the reference's
// code.
#include <nufi/config.hpp>

#include "../nufi_f0.h"

extern "C" __constant__ nufi_f0_params nufi_ref_f0;

namespace nufi {
namespace dim1 {

__device__ inline double ref_f0_1d(double x, double u)
{
    const double alpha = nufi_ref_f0.p[0], k = nufi_ref_f0.p[1];
    if (nufi_ref_f0.kind == NUFI_F0_LANDAU)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2);
    if (nufi_ref_f0.kind == NUFI_F0_TWO_STREAM)
        return 0.39894228040143267793994 * (1. + alpha * cos(k * x)) * exp(-u * u / 2.) * u * u;
    const double ub = nufi_ref_f0.p[2], sb = nufi_ref_f0.p[3];
    const double z = (u - ub) / sb;
    return (1. + alpha * cos(k * x)) * (0.9 * 0.39894228040143267793994 * exp(-u * u / 2) +
                                        0.1 * 0.39894228040143267793994 / sb * exp(-z * z / 2));
}

template <>
__host__ __device__ float config_t<float>::f0(float x, float u) noexcept
{
#ifdef __CUDA_ARCH__
    return float(ref_f0_1d(x, u));
#else
    return 0.0f;
#endif
}

template <>
__host__ __device__ double config_t<double>::f0(double x, double u) noexcept
{
#ifdef __CUDA_ARCH__
    return ref_f0_1d(x, u);
#else
    return 0.0;
#endif
}

}  // namespace dim1

namespace dim2 {

__device__ inline double ref_f0_2d(double x, double y, double u, double v)
{
    const double alpha = nufi_ref_f0.p[0], k = nufi_ref_f0.p[1];
    return 1.0 / (2.0 * M_PI) * exp(-0.5 * (u * u + v * v)) * (1 + alpha * (cos(k * x) + cos(k * y)));
}

template <>
__host__ __device__ float config_t<float>::f0(float x, float y, float u, float v) noexcept
{
#ifdef __CUDA_ARCH__
    return float(ref_f0_2d(x, y, u, v));
#else
    return 0.0f;
#endif
}

template <>
__host__ __device__ double config_t<double>::f0(double x, double y, double u, double v) noexcept
{
#ifdef __CUDA_ARCH__
    return ref_f0_2d(x, y, u, v);
#else
    return 0.0;
#endif
}

}  // namespace dim2

namespace dim3 {

__device__ inline double ref_f0_3d(double x, double y, double z, double u, double v, double w)
{
    const double alpha = nufi_ref_f0.p[0], k = nufi_ref_f0.p[1];
    return 0.06349363593424096978576330493464 * (1. + alpha * cos(k * x) + alpha * cos(k * y) + alpha * cos(k * z)) *
           exp(-(u * u + v * v + w * w) / 2);
}

template <>
__host__ __device__ float config_t<float>::f0(float x, float y, float z, float u, float v, float w) noexcept
{
#ifdef __CUDA_ARCH__
    return float(ref_f0_3d(x, y, z, u, v, w));
#else
    return 0.0f;
#endif
}

template <>
__host__ __device__ double config_t<double>::f0(double x, double y, double z, double u, double v, double w) noexcept
{
#ifdef __CUDA_ARCH__
    return ref_f0_3d(x, y, z, u, v, w);
#else
    return 0.0;
#endif
}

}  // namespace dim3
}  // namespace nufi

#include <nufi/cuda_kernel.cu>
