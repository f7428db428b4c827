/*
 * Drop-in replacement of the reference's nufi/cuda_kernel.hpp, backed by
 * the C ABI of include/nufi_gb300.h (libnufi_gb300.so).
 *
 * Put include/nufi_gb300 ahead of the reference's tree on the include path,
 * drop nufi/cuda_kernel.cu from the build and link libnufi_gb300.so: the
 * reference's nufi/cuda_scheduler.hpp (which includes this header) and the
 * drivers bin/test_nufi_gpu_{1d,2d,3d}.cpp then compile unchanged.
 *
 * Same class names, constructors and member functions as the reference
 * (nufi/cuda_kernel.hpp:33-56, 75-100, 117-142), same semantics:
 * compute_rho(n, q_begin, q_end) throws std::range_error for n > Nt and
 * returns early for an empty range; download_rho / download_metrics
 * accumulate (+=) into the caller's buffer; upload_phi(n, base) copies
 * slab n of the caller's history.  CUDA failures throw nufi::cuda::exception
 * (nufi/cuda_runtime.hpp:46-51).
 *
 * The reference hard-codes f0 in config_t<real>::f0; the device side needs
 * it as data.  nufi_gb300::set_initial_condition() selects it (kind +
 * parameters, see NUFI_F0_* in nufi_gb300.h); the default per dimension is
 * the reference's compiled-in f0 (1D: the u^2 M(u) form with alpha = 0.01,
 * k = 0.5; 2D: Landau with alpha = 0.5, k = 0.5; 3D: bump-on-tail with
 * alpha = 0.03, k = 0.3, u_b = 4.5, sigma_b = 0.5; nufi/config.hpp), each
 * reproduced to the last bit by the matching f0 kind.  real = double runs
 * the FP64 plain form, real = float the FP32-split form (built for order 4;
 * float kernels of other orders run the FP64 plain form).
 */
#ifndef NUFI_CUDA_KERNEL_HPP
#define NUFI_CUDA_KERNEL_HPP

#include <array>
#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <nufi/config.hpp>
#include <nufi/cuda_runtime.hpp>

#include "../../nufi_gb300.h"

namespace nufi_gb300 {

struct initial_condition {
    int kind;
    double params[8];
};

inline initial_condition &initial_condition_slot(int dim)
{
    static initial_condition slots[3] = {
        {NUFI_F0_TWO_STREAM, {0.01, 0.5, 0, 0, 0, 0, 0, 0}},
        {NUFI_F0_LANDAU, {0.5, 0.5, 0, 0, 0, 0, 0, 0}},
        {NUFI_F0_BUMP_ON_TAIL, {0.03, 0.3, 4.5, 0.5, 0, 0, 0, 0}},
    };
    return slots[dim - 1];
}

// Select f0 for the kernels created afterwards in dimension `dim`.
inline void set_initial_condition(int dim, int kind, const double *params, int nparams)
{
    initial_condition &ic = initial_condition_slot(dim);
    ic.kind = kind;
    for (int i = 0; i < 8; ++i) ic.params[i] = i < nparams ? params[i] : 0.0;
}

inline void throw_status(const nufi_handle *h, int st)
{
    if (st == NUFI_OK) return;
    const std::string msg = nufi_last_error(h);
    switch (st) {
    case NUFI_ERR_RANGE: throw std::range_error(msg);
    case NUFI_ERR_INVALID: throw std::invalid_argument(msg);
    case NUFI_ERR_CUDA: throw nufi::cuda::exception(cudaErrorUnknown, msg + " ");
    default: throw std::runtime_error(msg);
    }
}

struct handle_deleter {
    void operator()(nufi_handle *h) const noexcept { nufi_destroy(h); }
};

// real = float runs the FP32-split form, which is built for cubic splines
// (order 4); cuda_kernel<float, order> of any other order runs the FP64
// plain form instead (results at FP64 accuracy, at the FP64 rate), so that
// every <real, order> the reference instantiates has a kernel here.
template <typename real>
int precision_of(int order)
{
    return (std::is_same<real, float>::value && order == 4) ? NUFI_PREC_FP32_SPLIT : NUFI_PREC_FP64;
}

// config_t -> nufi_config, per dimension (members of nufi/config.hpp).
template <typename real>
nufi_config to_c(const nufi::dim1::config_t<real> &c, int order)
{
    nufi_config k{};
    k.dim = 1; k.order = order; k.precision = precision_of<real>(order);
    k.Nx[0] = (int64_t)c.Nx; k.Nv[0] = (int64_t)c.Nu; k.Nx[1] = k.Nx[2] = k.Nv[1] = k.Nv[2] = 1;
    k.Nt = (int64_t)c.Nt; k.dt = c.dt;
    k.x_min[0] = c.x_min; k.x_max[0] = c.x_max; k.v_min[0] = c.u_min; k.v_max[0] = c.u_max;
    k.x_max[1] = k.x_max[2] = k.v_max[1] = k.v_max[2] = 1;
    const initial_condition &ic = initial_condition_slot(1);
    k.f0_kind = ic.kind;
    for (int i = 0; i < 8; ++i) k.f0_params[i] = ic.params[i];
    return k;
}

template <typename real>
nufi_config to_c(const nufi::dim2::config_t<real> &c, int order)
{
    nufi_config k{};
    k.dim = 2; k.order = order; k.precision = precision_of<real>(order);
    k.Nx[0] = (int64_t)c.Nx; k.Nx[1] = (int64_t)c.Ny; k.Nx[2] = 1;
    k.Nv[0] = (int64_t)c.Nu; k.Nv[1] = (int64_t)c.Nv; k.Nv[2] = 1;
    k.Nt = (int64_t)c.Nt; k.dt = c.dt;
    k.x_min[0] = c.x_min; k.x_max[0] = c.x_max; k.x_min[1] = c.y_min; k.x_max[1] = c.y_max;
    k.v_min[0] = c.u_min; k.v_max[0] = c.u_max; k.v_min[1] = c.v_min; k.v_max[1] = c.v_max;
    k.x_max[2] = k.v_max[2] = 1;
    const initial_condition &ic = initial_condition_slot(2);
    k.f0_kind = ic.kind;
    for (int i = 0; i < 8; ++i) k.f0_params[i] = ic.params[i];
    return k;
}

template <typename real>
nufi_config to_c(const nufi::dim3::config_t<real> &c, int order)
{
    nufi_config k{};
    k.dim = 3; k.order = order; k.precision = precision_of<real>(order);
    k.Nx[0] = (int64_t)c.Nx; k.Nx[1] = (int64_t)c.Ny; k.Nx[2] = (int64_t)c.Nz;
    k.Nv[0] = (int64_t)c.Nu; k.Nv[1] = (int64_t)c.Nv; k.Nv[2] = (int64_t)c.Nw;
    k.Nt = (int64_t)c.Nt; k.dt = c.dt;
    k.x_min[0] = c.x_min; k.x_max[0] = c.x_max; k.x_min[1] = c.y_min; k.x_max[1] = c.y_max;
    k.x_min[2] = c.z_min; k.x_max[2] = c.z_max;
    k.v_min[0] = c.u_min; k.v_max[0] = c.u_max; k.v_min[1] = c.v_min; k.v_max[1] = c.v_max;
    k.v_min[2] = c.w_min; k.v_max[2] = c.w_max;
    const initial_condition &ic = initial_condition_slot(3);
    k.f0_kind = ic.kind;
    for (int i = 0; i < 8; ++i) k.f0_params[i] = ic.params[i];
    return k;
}

// The body shared by dim1/dim2/dim3::cuda_kernel.
template <typename conf_t, typename real, size_t order>
class kernel_impl {
public:
    kernel_impl(const conf_t &conf, int dev)
    {
        const nufi_config k = to_c<real>(conf, int(order));
        nufi_handle *h = nullptr;
        throw_status(nullptr, nufi_create(&k, dev, &h));
        handle.reset(h);
    }

    void compute_rho(size_t n, size_t q_min, size_t q_max)
    {
        throw_status(handle.get(), nufi_compute_rho(handle.get(), (int64_t)n, (int64_t)q_min, (int64_t)q_max));
    }

    void download_rho(real *rho)
    {
        if (std::is_same<real, float>::value)
            throw_status(handle.get(), nufi_download_rho_f32(handle.get(), reinterpret_cast<float *>(rho)));
        else
            throw_status(handle.get(), nufi_download_rho(handle.get(), reinterpret_cast<double *>(rho)));
    }

    void upload_phi(size_t n, const real *coeffs)
    {
        if (std::is_same<real, float>::value)
            throw_status(handle.get(), nufi_upload_phi_f32(handle.get(), (int64_t)n, reinterpret_cast<const float *>(coeffs)));
        else
            throw_status(handle.get(), nufi_upload_phi(handle.get(), (int64_t)n, reinterpret_cast<const double *>(coeffs)));
    }

    // The reference's metrics points lie on conf_metrics's grid
    // (nufi/cuda_kernel.cu:53-79, 96-108): nufi_set_metrics_grid.
    void set_metrics_grid(const conf_t &conf_metrics)
    {
        const nufi_config k = to_c<real>(conf_metrics, int(order));
        throw_status(handle.get(), nufi_set_metrics_grid(handle.get(), &k));
    }

    void compute_metrics(size_t n, size_t q_min, size_t q_max)
    {
        throw_status(handle.get(), nufi_compute_metrics(handle.get(), (int64_t)n, (int64_t)q_min, (int64_t)q_max));
    }

    void download_metrics(real *metrics)
    {
        double m[4] = {0, 0, 0, 0};
        throw_status(handle.get(), nufi_download_metrics(handle.get(), m));
        for (int i = 0; i < 4; ++i) metrics[i] += real(m[i]);
    }

    // Not in the reference: J = 2 dt sum_{n<=n1} W_n after running steps
    // 0..n1 on the device, and dJ/d(alpha, k, u_b, sigma_b) by the adjoint.
    double forward(size_t n1)
    {
        double J = 0;
        throw_status(handle.get(), nufi_forward(handle.get(), (int64_t)n1, &J));
        return J;
    }

    std::array<double, 4> backward(size_t n1)
    {
        std::array<double, 4> g{};
        throw_status(handle.get(), nufi_backward(handle.get(), (int64_t)n1, g.data()));
        return g;
    }

    nufi_handle *get() const noexcept { return handle.get(); }

private:
    std::unique_ptr<nufi_handle, handle_deleter> handle;
};

}  // namespace nufi_gb300

namespace nufi {

#define NUFI_GB300_DECLARE_KERNEL(DIM)                                                              \
    namespace DIM {                                                                                 \
    template <typename real, size_t order>                                                          \
    class cuda_kernel {                                                                             \
    public:                                                                                         \
        cuda_kernel(const config_t<real> &conf, int dev = cuda::get_device()) : impl(conf, dev) {} \
        cuda_kernel(const config_t<real> &conf, const config_t<real> &conf_metrics,                \
                    int dev = cuda::get_device())                                                   \
            : impl(conf, dev)                                                                       \
        {                                                                                           \
            impl.set_metrics_grid(conf_metrics);                                                    \
        }                                                                                           \
        cuda_kernel(const cuda_kernel &rhs) = delete;                                               \
        cuda_kernel(cuda_kernel &&rhs) = default;                                                   \
        cuda_kernel &operator=(const cuda_kernel &rhs) = delete;                                    \
        cuda_kernel &operator=(cuda_kernel &&rhs) = default;                                        \
        void compute_rho(size_t n, size_t q_min, size_t q_max) { impl.compute_rho(n, q_min, q_max); } \
        void download_rho(real *rho) { impl.download_rho(rho); }                                    \
        void upload_phi(size_t n, const real *coeffs) { impl.upload_phi(n, coeffs); }              \
        void compute_metrics(size_t n, size_t q_min, size_t q_max) { impl.compute_metrics(n, q_min, q_max); } \
        void download_metrics(real *metrics) { impl.download_metrics(metrics); }                    \
        double forward(size_t n1) { return impl.forward(n1); }                                      \
        std::array<double, 4> backward(size_t n1) { return impl.backward(n1); }                     \
        nufi_handle *native_handle() const noexcept { return impl.get(); }                          \
                                                                                                    \
    private:                                                                                        \
        nufi_gb300::kernel_impl<config_t<real>, real, order> impl;                                  \
    };                                                                                              \
    }

NUFI_GB300_DECLARE_KERNEL(dim1)
NUFI_GB300_DECLARE_KERNEL(dim2)
NUFI_GB300_DECLARE_KERNEL(dim3)

#undef NUFI_GB300_DECLARE_KERNEL

}  // namespace nufi

#endif
