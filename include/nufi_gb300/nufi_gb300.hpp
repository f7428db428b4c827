/*
 * nufi_gb300.hpp — C++ interface over the C ABI (nufi_gb300.h) for what the
 * reference has no class for: the device-resident run, the gradient of the
 * time-integrated field energy (forward / backward pair) and batches of 1D
 * instances.  Header only; link libnufi_gb300.so.  No reference headers
 * needed (the drop-in classes live in nufi/cuda_kernel.hpp).
 *
 * Errors become exceptions: std::range_error (NUFI_ERR_RANGE),
 * std::invalid_argument (NUFI_ERR_INVALID), std::logic_error
 * (NUFI_ERR_UNSUPPORTED), std::runtime_error (CUDA and device checks).
 */
#ifndef NUFI_GB300_HPP
#define NUFI_GB300_HPP

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../nufi_gb300.h"

namespace nufi_gb300 {

inline void check_status(int st, const char *msg)
{
    if (st == NUFI_OK) return;
    const std::string m = msg ? msg : "";
    switch (st) {
    case NUFI_ERR_RANGE: throw std::range_error(m);
    case NUFI_ERR_INVALID: throw std::invalid_argument(m);
    case NUFI_ERR_UNSUPPORTED: throw std::logic_error(m);
    default: throw std::runtime_error(m);
    }
}

// One configuration on one GPU.
class simulation {
public:
    explicit simulation(const nufi_config &cfg, int device = 0) : nt_(cfg.Nt)
    {
        nufi_handle *h = nullptr;
        const int st = nufi_create(&cfg, device, &h);
        check_status(st, nufi_last_error(nullptr));
        h_.reset(h);
    }

    // Steps n0..n1 on the device; returns W_n0..W_n1.
    std::vector<double> run(int64_t n0, int64_t n1)
    {
        std::vector<double> e(size_t(n1 - n0 + 1));
        check(nufi_run(h_.get(), n0, n1, e.data()));
        return e;
    }
    std::vector<double> run() { return run(0, nt_); }

    // J = 2 dt sum_{n <= n1} W_n after running steps 0..n1.
    double forward(int64_t n1)
    {
        double J = 0;
        check(nufi_forward(h_.get(), n1, &J));
        return J;
    }
    double forward() { return forward(nt_); }

    // dJ/d(alpha, k, u_b, sigma_b) by the adjoint of the forward run.
    std::array<double, 4> backward(int64_t n1)
    {
        std::array<double, 4> g{};
        check(nufi_backward(h_.get(), n1, g.data()));
        return g;
    }
    std::array<double, 4> backward() { return backward(nt_); }

    nufi_handle *get() const noexcept { return h_.get(); }

private:
    struct deleter {
        void operator()(nufi_handle *h) const noexcept { nufi_destroy(h); }
    };
    void check(int st) { check_status(st, nufi_last_error(h_.get())); }
    std::unique_ptr<nufi_handle, deleter> h_;
    int64_t nt_;
};

// Many 1D instances of uneven grid sizes advanced together.
class batch {
public:
    explicit batch(const std::vector<nufi_config> &cfgs, int device = 0) : nt_(cfgs.size())
    {
        for (size_t i = 0; i < cfgs.size(); ++i) nt_[i] = cfgs[i].Nt;
        nufi_batch *b = nullptr;
        const int st = nufi_batch_create(cfgs.data(), int32_t(cfgs.size()), device, &b);
        check_status(st, nufi_batch_last_error(nullptr));
        b_.reset(b);
    }

    size_t size() const noexcept { return nt_.size(); }

    // All steps of every instance; J_i = 2 dt sum_n W_n.
    std::vector<double> forward()
    {
        std::vector<double> J(size());
        check(nufi_batch_forward(b_.get(), J.data()));
        return J;
    }

    // dJ_i/d(alpha, k, u_b, sigma_b) of every instance.
    std::vector<std::array<double, 4>> backward()
    {
        std::vector<std::array<double, 4>> g(size());
        check(nufi_batch_backward(b_.get(), g.empty() ? nullptr : g[0].data()));
        return g;
    }

    std::vector<double> energy(int32_t i)
    {
        std::vector<double> e(size_t(nt_.at(size_t(i)) + 1));
        check(nufi_batch_energy(b_.get(), i, e.data()));
        return e;
    }

    // The autotuner's choice and the work decomposition, as JSON.
    std::string describe() const
    {
        std::string s(1 << 16, '\0');
        check_status(nufi_batch_describe(b_.get(), &s[0], s.size()), nufi_batch_last_error(b_.get()));
        s.resize(s.find('\0'));
        return s;
    }

private:
    struct deleter {
        void operator()(nufi_batch *b) const noexcept { nufi_batch_destroy(b); }
    };
    void check(int st) { check_status(st, nufi_batch_last_error(b_.get())); }
    std::unique_ptr<nufi_batch, deleter> b_;
    std::vector<int64_t> nt_;
};

}  // namespace nufi_gb300

#endif
