// The drop-in nufi::dimN::cuda_kernel<real, 4> (include/nufi_gb300/nufi/
// cuda_kernel.hpp) driven the way the reference's drivers drive theirs
// (bin/test_nufi_gpu_1d.cpp:241-252): upload_phi of every slab of a given
// history, then per step compute_rho over a q range split in parts and
// download_rho (which accumulates) into a zeroed buffer.  Built against
// the interface-only stand-ins in tests/cpp/dropin_stubs/ where the
// reference's headers are absent.
//
//   dropin_gpu <dim> <real: f|d> <N> <Nv> <Nt> <history file> <rho out>
//
// The history file holds (Nt+1) slabs of doubles in the reference layout;
// rho out gets rho(n) for n = 0..Nt, Ns doubles each.  Exit 0 after the
// error checks below passed; the caller compares rho with the golden one.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include <nufi/cuda_kernel.hpp>

namespace {

constexpr double kPi = 3.14159265358979323846;

template <typename conf_t>
void set_common(conf_t &c, size_t Nt)
{
    c.Nt = Nt;
    c.dt = 1.0 / 16.0;
}

template <typename real>
nufi::dim1::config_t<real> conf1(size_t N, size_t Nv, size_t Nt)
{
    nufi::dim1::config_t<real> c;
    c.Nx = N; c.Nu = Nv;
    c.x_min = 0; c.x_max = real(4 * kPi); c.u_min = -10; c.u_max = 10;
    set_common(c, Nt);
    c.derive();
    return c;
}

template <typename real>
nufi::dim2::config_t<real> conf2(size_t N, size_t Nv, size_t Nt)
{
    nufi::dim2::config_t<real> c;
    c.Nx = c.Ny = N; c.Nu = c.Nv = Nv;
    c.x_min = c.y_min = 0; c.x_max = c.y_max = real(4 * kPi);
    c.u_min = c.v_min = -8; c.u_max = c.v_max = 8;
    set_common(c, Nt);
    c.dt = 1.0 / 8.0;
    c.derive();
    return c;
}

template <typename real>
nufi::dim3::config_t<real> conf3(size_t N, size_t Nv, size_t Nt)
{
    nufi::dim3::config_t<real> c;
    c.Nx = c.Ny = c.Nz = N; c.Nu = c.Nv = c.Nw = Nv;
    c.x_min = c.y_min = c.z_min = 0; c.x_max = c.y_max = c.z_max = real(4 * kPi);
    c.u_min = c.v_min = c.w_min = -6; c.u_max = c.v_max = c.w_max = 6;
    set_common(c, Nt);
    c.dt = 0.1;
    c.derive();
    return c;
}

template <typename kernel_t, typename real>
int drive(kernel_t &k, size_t Ns, size_t Nq, size_t Nt, const std::vector<double> &hist64, const char *out)
{
    std::vector<real> hist(hist64.begin(), hist64.end());
    // the drivers' errors: a step past Nt is std::range_error
    try {
        k.compute_rho(Nt + 1, 0, Nq);
        std::puts("no range_error for n > Nt");
        return 3;
    } catch (const std::range_error &) {
    }
    std::vector<double> all;
    std::vector<real> rho(Ns);
    for (size_t n = 0; n <= Nt; ++n) k.upload_phi(n, hist.data());
    for (size_t n = 0; n <= Nt; ++n) {
        for (auto &r : rho) r = 0;
        const size_t cuts[4] = {0, Nq / 3, Nq / 3 + 1, Nq};
        for (int p = 0; p < 3; ++p) {
            k.compute_rho(n, cuts[p], cuts[p + 1]);
            k.download_rho(rho.data());
        }
        all.insert(all.end(), rho.begin(), rho.end());
    }
    FILE *f = std::fopen(out, "wb");
    if (!f) return 2;
    std::fwrite(all.data(), sizeof(double), all.size(), f);
    std::fclose(f);
    return 0;
}

template <typename real>
int run(int dim, size_t N, size_t Nv, size_t Nt, const std::vector<double> &hist, const char *out)
{
    const double landau[2] = {0.01, 0.5};
    nufi_gb300::set_initial_condition(dim, NUFI_F0_LANDAU, landau, 2);
    if (dim == 1) {
        nufi::dim1::cuda_kernel<real, 4> k(conf1<real>(N, Nv, Nt));
        return drive<decltype(k), real>(k, N, N * Nv, Nt, hist, out);
    }
    if (dim == 2) {
        nufi::dim2::cuda_kernel<real, 4> k(conf2<real>(N, Nv, Nt));
        return drive<decltype(k), real>(k, N * N, N * N * Nv * Nv, Nt, hist, out);
    }
    nufi::dim3::cuda_kernel<real, 4> k(conf3<real>(N, Nv, Nt), 0);
    return drive<decltype(k), real>(k, N * N * N, N * N * N * Nv * Nv * Nv, Nt, hist, out);
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 8) {
        std::fprintf(stderr, "usage: dropin_gpu dim f|d N Nv Nt history rho_out\n");
        return 2;
    }
    const int dim = std::atoi(argv[1]);
    const bool single = argv[2][0] == 'f';
    const size_t N = std::strtoull(argv[3], nullptr, 10), Nv = std::strtoull(argv[4], nullptr, 10),
                 Nt = std::strtoull(argv[5], nullptr, 10);
    std::vector<double> hist;
    FILE *f = std::fopen(argv[6], "rb");
    if (!f) return 2;
    double v;
    while (std::fread(&v, sizeof(double), 1, f) == 1) hist.push_back(v);
    std::fclose(f);
    try {
        return single ? run<float>(dim, N, Nv, Nt, hist, argv[7]) : run<double>(dim, N, Nv, Nt, hist, argv[7]);
    } catch (const nufi::cuda::exception &e) {
        std::fprintf(stderr, "nufi::cuda::exception: %s\n", e.what());
        return 4;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 5;
    }
}
