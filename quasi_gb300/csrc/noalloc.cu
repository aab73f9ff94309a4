// noalloc.cu - a radix sort entry point that allocates no memory.
//
// Some callers of this library cannot let it allocate device memory. A real-time frame loop
// cannot afford cudaMalloc/cudaFree, which may synchronise the whole device and stall
// the other streams in the middle of a frame. A host may also reserve all device memory up
// front in its own pool and forbid its plugins to allocate. For them,
// Q_cuda_radix_sort_pairs_noalloc sorts with the same kernels as Q_cuda_radix_sort_pairs,
// but takes its scratch space (the ping-pong key/value buffers and the digit histograms)
// from one fixed array in device global memory, declared below. Every GPU that loads this
// library holds that array (QUASI_NOALLOC_SORT_SCRATCH_BYTES, about 8.5 MB) until the process exits.
#include "../../include/quasi_cuda.h"
#include "bvh.cuh"

#include <cuda_runtime.h>

#include <mutex>

namespace quasi {
namespace {

constexpr uint32_t k_max_keys = QUASI_NOALLOC_SORT_MAX_KEYS;
constexpr uint32_t k_tile = 2048;  // keys per sort block (k_sort_block * k_sort_items in bvh.cu)
constexpr uint32_t k_hist_words = 256u * ((k_max_keys + k_tile - 1) / k_tile);
constexpr size_t k_scratch_words = 2ull * k_max_keys + k_hist_words;
static_assert(k_scratch_words * 4 == QUASI_NOALLOC_SORT_SCRATCH_BYTES, "header and scratch size disagree");

// The scratch: [k_max_keys] alternate keys, [k_max_keys] alternate values, then histograms.
// Every sort writes each word it later reads, so nothing here has to start at zero.
static __device__ __align__(256) uint32_t g_sort_scratch[k_scratch_words];

constexpr int k_max_devices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_addr[k_max_devices] = {};

// Device address of g_sort_scratch on the current device. In host code the name
// g_sort_scratch is only a host-side stand-in, so the address is looked up once per device
// (with that device current) and cached for the life of the process. A cudaDeviceReset of
// that device after the first call would reload the module and leave the cached address
// stale, which is why callers must not reset the primary context after it.
cudaError_t scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= k_max_devices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace quasi

extern "C" Q_CUDA_EXPORT int Q_cuda_radix_sort_pairs_noalloc(uint32_t* device_keys, uint32_t* device_values,
                                                             uint32_t n, uint32_t key_bits, void* stream) {
    if (n > QUASI_NOALLOC_SORT_MAX_KEYS) return QUASI_ERR_TOO_LARGE;
    if (n == 0) return QUASI_OK;
    if (!device_keys || !device_values || key_bits == 0 || key_bits > 32) return QUASI_ERR_INVALID;
    uint32_t* base = nullptr;
    cudaError_t e = quasi::scratch_for_current_device(&base);
    if (e != cudaSuccess) return QUASI_ERR_CUDA;
    quasi::RadixSortScratch scratch;
    scratch.keys_alt = base;
    scratch.vals_alt = base + quasi::k_max_keys;
    scratch.hist = base + 2ull * quasi::k_max_keys;
    scratch.capacity = quasi::k_max_keys;
    scratch.hist_capacity = quasi::k_hist_words;
    quasi::KernelProfiler prof;  // disabled: counts launches only, creates no events
    e = quasi::radix_sort_pairs(device_keys, device_values, n, static_cast<int>(key_bits), scratch,
                                static_cast<cudaStream_t>(stream), prof);
    return e == cudaSuccess ? QUASI_OK : QUASI_ERR_CUDA;
}
