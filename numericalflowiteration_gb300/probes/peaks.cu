// peaks.cu — measured denominators for the roofline of the trace kernels,
// which are bound by FP32 / FP64 FMA issue and shared-memory load
// bandwidth (not by HBM or tensor cores).
//   nufi_probe_fma_peak: each thread runs 8 independent FMA chains for
//     `iters` rounds; 2 flop per FMA over the kernel's CUDA-event time.
//   nufi_probe_smem_bw: every warp reads 32 consecutive float4 (512 B,
//     conflict-free) of a 64 KB shared buffer per load, `iters` x 16 loads
//     per thread; bytes read over the kernel's CUDA-event time.
// Built into libnufi_probes.so, used by bench.py only.
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

__global__ void __launch_bounds__(1024) smem_reads(float *out, int iters)
{
    extern __shared__ float4 buf[];  // 4096 float4
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) buf[i] = make_float4(i, i + 1, i + 2, i + 3);
    __syncthreads();
    float4 acc = make_float4(0, 0, 0, 0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int base = warp * 32;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const float4 v = buf[((base + r * 256) & 4095) + lane];
            acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
        }
        base = (base + 32 * 33) & 4095;
    }
    const float s = (acc.x + acc.y) + (acc.z + acc.w);
    if (s == -12345.678f) out[threadIdx.x] = s;
}

int run_smem(double *gbs, double *ms_out, int iters)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, 1024 * sizeof(float)) != cudaSuccess) return 1;
    const size_t smem = 4096 * sizeof(float4);
    cudaFuncSetAttribute(smem_reads, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    const int blocks = sms * 2, threads = 1024;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    smem_reads<<<blocks, threads, smem>>>(out, iters / 8 + 1);  // warm-up
    cudaEventRecord(e0);
    smem_reads<<<blocks, threads, smem>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double bytes = double(blocks) * threads * double(iters) * 16.0 * 16.0;
    *gbs = bytes / (double(ms) * 1e-3) / 1e9;
    *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace

extern "C" int nufi_probe_smem_bw(int iters, double *gbs, double *ms) { return run_smem(gbs, ms, iters); }

extern "C" int nufi_probe_fma_peak(int fp64, int iters, double *tflops, double *ms)
{
    return fp64 ? run<double>(tflops, ms, iters) : run<float>(tflops, ms, iters);
}
