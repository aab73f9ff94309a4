// cuda_context.hpp - the host's GPU context for the CUDA backend: the counterpart of the
// Metal context the reference host builds for libquasi_metal (src/quasi/gpu/metal). It
// fills Q_gpu_context (src/quasi/gpu/types.hpp:37-42) with backend = Q_GPU_BACKEND_CUDA,
// device = pointer to the device ordinal, queue = a cudaStream_t owned by the host.
#pragma once

#include "quasi_cuda.h"

#include <cuda_runtime.h>

#include <string>

namespace quasi::host {

class cuda_context {
public:
    cuda_context() = default;
    ~cuda_context() {
        if (stream_) {
            cudaStreamSynchronize(stream_);
            cudaStreamDestroy(stream_);
        }
    }
    cuda_context(const cuda_context&) = delete;
    cuda_context& operator=(const cuda_context&) = delete;

    bool init(int device, std::string& error) {
        ordinal_ = device;
        cudaError_t e = cudaSetDevice(ordinal_);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            error = cudaGetErrorString(e);
            return false;
        }
        gpu_.backend = Q_GPU_BACKEND_CUDA;
        gpu_.device = &ordinal_;
        gpu_.queue = stream_;
        gpu_.layer = nullptr;
        return true;
    }

    Q_gpu_context* gpu() { return &gpu_; }
    cudaStream_t stream() const { return stream_; }

private:
    int ordinal_ = 0;
    cudaStream_t stream_ = nullptr;
    Q_gpu_context gpu_{};
};

}  // namespace quasi::host
