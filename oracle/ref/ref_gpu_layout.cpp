// ref_gpu_layout.cpp — prints, as JSON, the byte layout of the reference's
// nufi::dim{1,2,3}::config_t<float> / <double> (nufi/config.hpp:33-50,
// 91-114, 167-193) and of nufi_f0_params, compiled against the reference's
// own header.  The launcher of the reference GPU kernels (ref_gpu.py) packs
// the by-value kernel argument from this layout.  Test infrastructure only;
// built and run by oracle/ref/Makefile into oracle/_ref/.
#include <cstddef>
#include <cstdio>
#include <string>

#include <nufi/config.hpp>

#include "../nufi_f0.h"

#define NUFI_FIELD(C, f)                                                                              \
    do {                                                                                               \
        std::printf("%s\"%s\": %zu", first ? "" : ", ", #f, offsetof(C, f));                           \
        first = false;                                                                                 \
    } while (0)

template <typename real>
static void layout1(const char *name)
{
    using C = nufi::dim1::config_t<real>;
    bool first = true;
    std::printf("  \"%s\": {\"size\": %zu, \"real\": %zu, \"fields\": {", name, sizeof(C), sizeof(real));
    NUFI_FIELD(C, Nx); NUFI_FIELD(C, Nu); NUFI_FIELD(C, Nt); NUFI_FIELD(C, dt);
    NUFI_FIELD(C, x_min); NUFI_FIELD(C, x_max); NUFI_FIELD(C, u_min); NUFI_FIELD(C, u_max);
    NUFI_FIELD(C, dx); NUFI_FIELD(C, dx_inv); NUFI_FIELD(C, Lx); NUFI_FIELD(C, Lx_inv); NUFI_FIELD(C, du);
    std::printf("}},\n");
}

template <typename real>
static void layout2(const char *name)
{
    using C = nufi::dim2::config_t<real>;
    bool first = true;
    std::printf("  \"%s\": {\"size\": %zu, \"real\": %zu, \"fields\": {", name, sizeof(C), sizeof(real));
    NUFI_FIELD(C, Nx); NUFI_FIELD(C, Ny); NUFI_FIELD(C, Nu); NUFI_FIELD(C, Nv); NUFI_FIELD(C, Nt);
    NUFI_FIELD(C, dt); NUFI_FIELD(C, x_min); NUFI_FIELD(C, x_max); NUFI_FIELD(C, y_min); NUFI_FIELD(C, y_max);
    NUFI_FIELD(C, u_min); NUFI_FIELD(C, u_max); NUFI_FIELD(C, v_min); NUFI_FIELD(C, v_max);
    NUFI_FIELD(C, dx); NUFI_FIELD(C, dx_inv); NUFI_FIELD(C, Lx); NUFI_FIELD(C, Lx_inv);
    NUFI_FIELD(C, dy); NUFI_FIELD(C, dy_inv); NUFI_FIELD(C, Ly); NUFI_FIELD(C, Ly_inv);
    NUFI_FIELD(C, du); NUFI_FIELD(C, dv);
    std::printf("}},\n");
}

template <typename real>
static void layout3(const char *name)
{
    using C = nufi::dim3::config_t<real>;
    bool first = true;
    std::printf("  \"%s\": {\"size\": %zu, \"real\": %zu, \"fields\": {", name, sizeof(C), sizeof(real));
    NUFI_FIELD(C, Nx); NUFI_FIELD(C, Ny); NUFI_FIELD(C, Nz); NUFI_FIELD(C, Nu); NUFI_FIELD(C, Nv);
    NUFI_FIELD(C, Nw); NUFI_FIELD(C, Nt); NUFI_FIELD(C, dt);
    NUFI_FIELD(C, x_min); NUFI_FIELD(C, x_max); NUFI_FIELD(C, y_min); NUFI_FIELD(C, y_max);
    NUFI_FIELD(C, z_min); NUFI_FIELD(C, z_max); NUFI_FIELD(C, u_min); NUFI_FIELD(C, u_max);
    NUFI_FIELD(C, v_min); NUFI_FIELD(C, v_max); NUFI_FIELD(C, w_min); NUFI_FIELD(C, w_max);
    NUFI_FIELD(C, dx); NUFI_FIELD(C, dx_inv); NUFI_FIELD(C, Lx); NUFI_FIELD(C, Lx_inv);
    NUFI_FIELD(C, dy); NUFI_FIELD(C, dy_inv); NUFI_FIELD(C, Ly); NUFI_FIELD(C, Ly_inv);
    NUFI_FIELD(C, dz); NUFI_FIELD(C, dz_inv); NUFI_FIELD(C, Lz); NUFI_FIELD(C, Lz_inv);
    NUFI_FIELD(C, du); NUFI_FIELD(C, dv); NUFI_FIELD(C, dw);
    std::printf("}},\n");
}

int main()
{
    std::printf("{\n");
    layout1<float>("dim1::config_t<float>");
    layout1<double>("dim1::config_t<double>");
    layout2<float>("dim2::config_t<float>");
    layout2<double>("dim2::config_t<double>");
    layout3<float>("dim3::config_t<float>");
    layout3<double>("dim3::config_t<double>");
    std::printf("  \"nufi_f0_params\": {\"size\": %zu, \"kind\": %zu, \"p\": %zu}\n}\n", sizeof(nufi_f0_params),
                offsetof(nufi_f0_params, kind), offsetof(nufi_f0_params, p));
    return 0;
}
