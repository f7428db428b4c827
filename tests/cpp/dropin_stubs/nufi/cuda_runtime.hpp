/*
 * Interface-only stand-in for the reference's nufi/cuda_runtime.hpp, for
 * compiling the drop-in include/nufi_gb300/nufi/cuda_kernel.hpp where the
 * reference sources are absent: the exception type the drop-in throws for
 * CUDA failures (nufi::cuda::exception, a std::runtime_error carrying the
 * CUDA error; nufi/cuda_runtime.hpp:46-51) and get_device(), the default
 * device argument of the kernels' constructors.  Test infrastructure only.
 */
#ifndef NUFI_CUDA_RUNTIME_HPP
#define NUFI_CUDA_RUNTIME_HPP

#include <stdexcept>
#include <string>

#include <cuda_runtime_api.h>

namespace nufi {
namespace cuda {

class exception : public std::runtime_error {
public:
    exception(cudaError_t code, const std::string &msg)
        : std::runtime_error(msg + cudaGetErrorName(code)), code_(code) {}
    cudaError_t code() const noexcept { return code_; }

private:
    cudaError_t code_;
};

inline int get_device()
{
    int d = 0;
    const cudaError_t e = cudaGetDevice(&d);
    if (e != cudaSuccess) throw exception(e, "cudaGetDevice: ");
    return d;
}

}  // namespace cuda
}  // namespace nufi

#endif
