// peaks.cu — measured denominators for the roofline of the trace kernels,
// which are bound by FP32 / FP64 FMA issue (not by HBM or tensor cores).
// Each thread runs 8 independent FMA chains for `iters` rounds; the peak
// is 2 flop per FMA over the kernel's CUDA-event time.  Built into
// libnufi_probes.so, used by bench.py only.
#include <cuda_runtime.h>
#include <cstdio>

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T *out, int iters, T a, T b)
{
    T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == T(-12345.678)) out[threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
int run(double *tflops, double *ms_out, int iters)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    T *out = nullptr;
    if (cudaMalloc(&out, 256 * sizeof(T)) != cudaSuccess) return 1;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<blocks, 256>>>(out, iters / 8 + 1, T(0.999999), T(1e-7));  // warm-up
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, 256>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double fmas = double(blocks) * 256.0 * double(iters) * 16.0 * 8.0;
    *tflops = 2.0 * fmas / (double(ms) * 1e-3) / 1e12;
    *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

extern "C" int nufi_probe_fma_peak(int fp64, int iters, double *tflops, double *ms)
{
    return fp64 ? run<double>(tflops, ms, iters) : run<float>(tflops, ms, iters);
}
