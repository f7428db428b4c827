// Uses the C++ interface (include/nufi_gb300/nufi_gb300.hpp): a 1D run,
// the forward/backward pair and a small batch.  Prints one line per
// result; with no usable GPU it prints the exception it caught.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "nufi_gb300/nufi_gb300.hpp"

static nufi_config landau(int64_t nx, int64_t nv, int64_t nt)
{
    nufi_config c;
    std::memset(&c, 0, sizeof(c));
    c.dim = 1;
    c.order = 4;
    c.precision = NUFI_PREC_FP64;
    c.f0_kind = NUFI_F0_LANDAU;
    c.Nx[0] = nx; c.Nx[1] = c.Nx[2] = 1;
    c.Nv[0] = nv; c.Nv[1] = c.Nv[2] = 1;
    c.Nt = nt;
    c.dt = 1.0 / 16;
    c.x_min[0] = 0; c.x_max[0] = 4 * 3.14159265358979323846;
    c.v_min[0] = -10; c.v_max[0] = 10;
    c.x_max[1] = c.x_max[2] = c.v_max[1] = c.v_max[2] = 1;
    c.f0_params[0] = 0.01;
    c.f0_params[1] = 0.5;
    return c;
}

int main()
{
    nufi_config bad = landau(32, 64, 10);
    bad.Nx[0] = 0;
    try {
        nufi_gb300::simulation s(bad);
        std::printf("invalid: accepted\n");
    } catch (const std::invalid_argument &) {
        std::printf("invalid: invalid_argument\n");
    }
    try {
        nufi_gb300::simulation s(landau(32, 64, 40));
        const double J = s.forward();
        const std::array<double, 4> g = s.backward();
        std::printf("J %.17g\ngrad %.17g %.17g %.17g %.17g\n", J, g[0], g[1], g[2], g[3]);
        nufi_gb300::batch b({landau(32, 64, 40), landau(16, 32, 20)});
        const std::vector<double> Jb = b.forward();
        const auto gb = b.backward();
        std::printf("batch J %.17g %.17g\nbatch grad0 %.17g %.17g\n", Jb[0], Jb[1], gb[0][0], gb[0][1]);
    } catch (const std::runtime_error &e) {
        std::printf("runtime_error: %s\n", e.what());
    }
    return 0;
}
