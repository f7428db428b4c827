// ref_gpu_layout.cpp — prints, as JSON, the byte layout of the reference's
// nufi::dim1::config_t<float> / <double> (nufi/config.hpp:33-50) and of
// nufi_f0_params, compiled against the reference's own header.  The
// launcher of the reference GPU kernels (ref_gpu.py) packs the by-value
// kernel argument from this layout.  Test infrastructure only; built and
// run by oracle/ref/Makefile into oracle/_ref/.
#include <cstddef>
#include <cstdio>

#include <nufi/config.hpp>

#include "../nufi_f0.h"

template <typename real>
static void print_conf(const char *name, bool last)
{
    using C = nufi::dim1::config_t<real>;
    std::printf("  \"%s\": {\"size\": %zu, \"real\": %zu, \"fields\": {", name, sizeof(C), sizeof(real));
    std::printf("\"Nx\": %zu, \"Nu\": %zu, \"Nt\": %zu, \"dt\": %zu, \"x_min\": %zu, \"x_max\": %zu, "
                "\"u_min\": %zu, \"u_max\": %zu, \"dx\": %zu, \"dx_inv\": %zu, \"Lx\": %zu, \"Lx_inv\": %zu, "
                "\"du\": %zu}}%s\n",
                offsetof(C, Nx), offsetof(C, Nu), offsetof(C, Nt), offsetof(C, dt), offsetof(C, x_min),
                offsetof(C, x_max), offsetof(C, u_min), offsetof(C, u_max), offsetof(C, dx), offsetof(C, dx_inv),
                offsetof(C, Lx), offsetof(C, Lx_inv), offsetof(C, du), last ? "" : ",");
}

int main()
{
    std::printf("{\n");
    print_conf<float>("config_t<float>", false);
    print_conf<double>("config_t<double>", false);
    std::printf("  \"nufi_f0_params\": {\"size\": %zu, \"kind\": %zu, \"p\": %zu}\n}\n", sizeof(nufi_f0_params),
                offsetof(nufi_f0_params, kind), offsetof(nufi_f0_params, p));
    return 0;
}
