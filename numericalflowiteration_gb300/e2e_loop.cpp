// e2e_loop.cpp — the reference drivers' time loop through the C ABI with
// host buffers, timed end to end (bin/test_nufi_gpu_1d.cpp:241-252): per
// step n = 0..Nt
//     rho = 0;  compute_rho(n, 0, Nq);  download_rho(rho)     (+=, host)
//     field solve of the host rho -> host slab n and W_n     (nufi_field_solve)
//     copy the slab into the host history;  upload_phi(n, history)
// Every host<->device copy of the loop is inside the timed region.  This is
// what a C or C++ caller of the library runs; bench.py reports its rate as
// the end-to-end number.
//
//   e2e_loop <config file (struct nufi_config, raw bytes)> <repeats> [device]
//
// Prints one JSON object: the median seconds of a whole run over `repeats`
// timed runs (after one untimed run), the bytes copied per run, and the
// host time inside each call per time step (microseconds, mean over the
// timed runs; a blocking call's time includes its wait for the device).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "nufi_gb300.h"

namespace {

int check(nufi_handle *h, int st, const char *what)
{
    if (st != NUFI_OK) std::fprintf(stderr, "%s failed (%d): %s\n", what, st, nufi_last_error(h));
    return st;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: e2e_loop <config bytes> <repeats> [device]\n");
        return 2;
    }
    nufi_config cfg;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f || std::fread(&cfg, sizeof(cfg), 1, f) != 1) {
        std::fprintf(stderr, "cannot read the configuration\n");
        if (f) std::fclose(f);
        return 2;
    }
    std::fclose(f);
    const int repeats = std::max(1, std::atoi(argv[2]));
    const int device = argc > 3 ? std::atoi(argv[3]) : 0;
    nufi_handle *h = nullptr;
    if (check(nullptr, nufi_create(&cfg, device, &h), "nufi_create")) return 3;
    int64_t stride_t = 0, ns = 0, nq = 0;
    nufi_sizes(h, &stride_t, &ns, &nq);
    const int64_t Nt = cfg.Nt;
    std::vector<double> rho(static_cast<size_t>(ns)), coeffs(static_cast<size_t>((Nt + 1) * stride_t)),
        energy(static_cast<size_t>(Nt + 1));
    using clk = std::chrono::steady_clock;
    double call_s[4] = {0, 0, 0, 0};  // compute_rho, download_rho, field_solve, upload_phi
    auto run = [&]() -> int {
        for (int64_t n = 0; n <= Nt; ++n) {
            std::fill(rho.begin(), rho.end(), 0.0);
            const auto t0 = clk::now();
            if (check(h, nufi_compute_rho(h, n, 0, nq), "compute_rho")) return 1;
            const auto t1 = clk::now();
            if (check(h, nufi_download_rho(h, rho.data()), "download_rho")) return 1;
            const auto t2 = clk::now();
            if (check(h, nufi_field_solve(h, rho.data(), coeffs.data() + n * stride_t, &energy[size_t(n)]),
                      "field_solve"))
                return 1;
            const auto t3 = clk::now();
            if (check(h, nufi_upload_phi(h, n, coeffs.data()), "upload_phi")) return 1;
            const auto t4 = clk::now();
            call_s[0] += std::chrono::duration<double>(t1 - t0).count();
            call_s[1] += std::chrono::duration<double>(t2 - t1).count();
            call_s[2] += std::chrono::duration<double>(t3 - t2).count();
            call_s[3] += std::chrono::duration<double>(t4 - t3).count();
        }
        return check(h, nufi_synchronize(h), "synchronize");
    };
    if (run()) return 4;
    for (double &c : call_s) c = 0;
    std::vector<double> secs;
    for (int r = 0; r < repeats; ++r) {
        const auto t0 = std::chrono::steady_clock::now();
        if (run()) return 4;
        secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    std::sort(secs.begin(), secs.end());
    const double med = secs[secs.size() / 2];
    const long long steps = Nt + 1;
    // per step: slab H2D (upload_phi) and rho H2D (field solve); rho D2H,
    // slab + W D2H (field solve)
    const long long h2d = steps * 8LL * (stride_t + ns), d2h = steps * 8LL * (ns + stride_t + 1);
    const double per = 1e6 / (double(repeats) * double(steps));
    std::printf("{\"seconds\": %.9f, \"repeats\": %d, \"h2d_bytes\": %lld, \"d2h_bytes\": %lld, "
                "\"energy_last\": %.17g, \"call_us_per_step\": {\"compute_rho\": %.3f, \"download_rho\": %.3f, "
                "\"field_solve\": %.3f, \"upload_phi\": %.3f}}\n",
                med, repeats, h2d, d2h, energy[size_t(Nt)], call_s[0] * per, call_s[1] * per, call_s[2] * per,
                call_s[3] * per);
    nufi_destroy(h);
    return 0;
}
