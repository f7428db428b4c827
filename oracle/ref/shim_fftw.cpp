// Separable DHT behind the fftw3.h stand-in (see shim/fftw3.h).  Sums are
// formed in long double with exactly reduced angles.  Test infrastructure.
#include <fftw3.h>

#include <cmath>
#include <vector>

struct nufi_shim_dht_plan {
    std::vector<int> dims;  // slowest first, as FFTW takes them
};

namespace {

template <typename real>
void dht_inplace(const nufi_shim_dht_plan *p, real *in, real *out)
{
    size_t total = 1;
    for (int d : p->dims) total *= size_t(d);
    std::vector<long double> a(in, in + total), tmp;
    const size_t nd = p->dims.size();
    // axis index ax counts from the fastest (last) dimension.
    size_t inner = 1;
    for (size_t ax = 0; ax < nd; ++ax) {
        const size_t N = size_t(p->dims[nd - 1 - ax]);
        std::vector<long double> cas(N * N);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (size_t j = 0; j < N; ++j)
            for (size_t k = 0; k < N; ++k) {
                const long double ang = two_pi * (long double)((j * k) % N) / (long double)N;
                cas[j * N + k] = cosl(ang) + sinl(ang);
            }
        tmp.assign(N, 0.0L);
        const size_t outer = total / (N * inner);
        for (size_t o = 0; o < outer; ++o)
            for (size_t i = 0; i < inner; ++i) {
                long double *line = a.data() + o * N * inner + i;
                for (size_t k = 0; k < N; ++k) {
                    long double acc = 0;
                    for (size_t j = 0; j < N; ++j) acc += line[j * inner] * cas[j * N + k];
                    tmp[k] = acc;
                }
                for (size_t k = 0; k < N; ++k) line[k * inner] = tmp[k];
            }
        inner *= N;
    }
    for (size_t i = 0; i < total; ++i) out[i] = (real)a[i];
}

}  // namespace

extern "C" {

fftw_plan fftw_plan_r2r_1d(int n, double *, double *, fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n}}; }
fftw_plan fftw_plan_r2r_2d(int n0, int n1, double *, double *, fftw_r2r_kind, fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n0, n1}}; }
fftw_plan fftw_plan_r2r_3d(int n0, int n1, int n2, double *, double *, fftw_r2r_kind, fftw_r2r_kind,
                           fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n0, n1, n2}}; }
void fftw_execute_r2r(const fftw_plan p, double *in, double *out) { dht_inplace(p, in, out); }
void fftw_destroy_plan(fftw_plan p) { delete p; }

fftwf_plan fftwf_plan_r2r_1d(int n, float *, float *, fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n}}; }
fftwf_plan fftwf_plan_r2r_2d(int n0, int n1, float *, float *, fftw_r2r_kind, fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n0, n1}}; }
fftwf_plan fftwf_plan_r2r_3d(int n0, int n1, int n2, float *, float *, fftw_r2r_kind, fftw_r2r_kind,
                             fftw_r2r_kind, unsigned)
{ return new nufi_shim_dht_plan{{n0, n1, n2}}; }
void fftwf_execute_r2r(const fftwf_plan p, float *in, float *out) { dht_inplace(p, in, out); }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }

}
