/*
 * Interface-only stand-in for the reference's nufi/config.hpp, for
 * compiling the drop-in include/nufi_gb300/nufi/cuda_kernel.hpp where the
 * reference sources are absent (the GPU machine).  It declares the members of
 * nufi::dimN::config_t<real> that the drop-in reads (nufi/config.hpp:34-51,
 * 92-113, 168-192: node counts, Nt, dt, domain bounds) plus the derived
 * grid quantities, filled by derive() from those; there are no defaults and
 * no f0 (the drop-in takes f0 as data).  Test infrastructure only.
 */
#ifndef NUFI_CONFIG_HPP
#define NUFI_CONFIG_HPP

#include <cstddef>

namespace nufi {
namespace dim1 {
template <typename real>
struct config_t {
    size_t Nx = 0, Nu = 0, Nt = 0;
    real dt = 0;
    real x_min = 0, x_max = 0, u_min = 0, u_max = 0;
    real dx = 0, dx_inv = 0, Lx = 0, Lx_inv = 0, du = 0;
    void derive()
    {
        Lx = x_max - x_min; Lx_inv = 1 / Lx;
        dx = Lx / Nx; dx_inv = 1 / dx;
        du = (u_max - u_min) / Nu;
    }
};
}  // namespace dim1

namespace dim2 {
template <typename real>
struct config_t {
    size_t Nx = 0, Ny = 0, Nu = 0, Nv = 0, Nt = 0;
    real dt = 0;
    real x_min = 0, x_max = 0, y_min = 0, y_max = 0;
    real u_min = 0, u_max = 0, v_min = 0, v_max = 0;
    real dx = 0, dx_inv = 0, Lx = 0, Lx_inv = 0;
    real dy = 0, dy_inv = 0, Ly = 0, Ly_inv = 0;
    real du = 0, dv = 0;
    void derive()
    {
        Lx = x_max - x_min; Lx_inv = 1 / Lx; dx = Lx / Nx; dx_inv = 1 / dx;
        Ly = y_max - y_min; Ly_inv = 1 / Ly; dy = Ly / Ny; dy_inv = 1 / dy;
        du = (u_max - u_min) / Nu; dv = (v_max - v_min) / Nv;
    }
};
}  // namespace dim2

namespace dim3 {
template <typename real>
struct config_t {
    size_t Nx = 0, Ny = 0, Nz = 0, Nu = 0, Nv = 0, Nw = 0, Nt = 0;
    real dt = 0;
    real x_min = 0, x_max = 0, y_min = 0, y_max = 0, z_min = 0, z_max = 0;
    real u_min = 0, u_max = 0, v_min = 0, v_max = 0, w_min = 0, w_max = 0;
    real dx = 0, dx_inv = 0, Lx = 0, Lx_inv = 0;
    real dy = 0, dy_inv = 0, Ly = 0, Ly_inv = 0;
    real dz = 0, dz_inv = 0, Lz = 0, Lz_inv = 0;
    real du = 0, dv = 0, dw = 0;
    void derive()
    {
        Lx = x_max - x_min; Lx_inv = 1 / Lx; dx = Lx / Nx; dx_inv = 1 / dx;
        Ly = y_max - y_min; Ly_inv = 1 / Ly; dy = Ly / Ny; dy_inv = 1 / dy;
        Lz = z_max - z_min; Lz_inv = 1 / Lz; dz = Lz / Nz; dz_inv = 1 / dz;
        du = (u_max - u_min) / Nu; dv = (v_max - v_min) / Nv; dw = (w_max - w_min) / Nw;
    }
};
}  // namespace dim3
}  // namespace nufi

#endif
