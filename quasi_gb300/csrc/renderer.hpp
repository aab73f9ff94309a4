// renderer.hpp - host side of the CUDA path tracer: scene buffers, the per-frame LBVH,
// the wavefront loop and the progressive Kahan accumulation. One Renderer per plugin
// handle; every call comes from the host's main thread (single-threaded plugin ABI).
#pragma once

#include "../../include/quasi_cuda.h"
#include "bvh.cuh"
#include "launch.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace quasi {

struct FrameParams;  // device launch parameters (wavefront_kernels.cuh)

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes && ptr) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, n > 0 ? n : 16);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(ptr); }
};

class Renderer {
public:
    Renderer(int device, cudaStream_t stream, bool own_stream);
    ~Renderer();
    Renderer(const Renderer&) = delete;
    Renderer& operator=(const Renderer&) = delete;

    int init();
    int set_scene(const Q_cuda_scene& scene);
    int update_vertices(const float* vertices, uint32_t tri_count);
    int set_materials(const float* albedo, const float* emission, uint32_t tri_count);
    int set_options(const Q_cuda_options& o);
    Q_cuda_options options() const { return opt_; }
    int render(const Q_render_frame& frame);
    int reset();
    int synchronize();
    int resolve_host(float* rgba_beauty, float* rgba_albedo, float* rgba_normal, float* rgba_depth);
    int resolve_device(float* device_rgba);
    int read_samples(float* radiance, uint32_t* signatures);
    int read_bvh(uint32_t* morton, uint32_t* order, int32_t* children, float* boxes, float* bounds);
    int read_wide_bvh(uint32_t* words);
    int stats(Q_cuda_stats* out);
    int kernel_times(Q_cuda_kernel_time* out, uint32_t capacity, uint32_t* count);
    int autotune(double budget_ms);
    // Device materials (3 floats per triangle); the set of emitters stays as last set from
    // host arrays.
    int set_materials_device(const float* albedo, const float* emission, uint32_t tri_count);
    // Path-replay adjoint of samples [sample_base, sample_base + spp) of the current frame.
    int backward(const float* grad_image, uint32_t spp, uint32_t sample_base, float* grad_albedo,
                 float* grad_emission, cudaStream_t stream);
    uint32_t tri_count() const { return n_tris_; }
    uint32_t samples() const { return samples_; }

    uint32_t width() const { return width_; }
    uint32_t height() const { return height_; }
    bool has_scene() const { return has_scene_; }
    cudaStream_t stream() const { return stream_; }
    int device() const { return device_; }
    int sm_count() const { return sm_count_; }
    const std::string& last_error() const { return error_; }
    int fail(int code, const std::string& msg) {
        error_ = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* where);

private:
    int ensure_frame_buffers(uint32_t w, uint32_t h);
    int ensure_wave_buffers(uint32_t paths);
    int upload_materials_host(const float* albedo, const float* emission, uint32_t n);
    int render_wavefront(cudaStream_t s, uint32_t spp);
    int render_megakernel(cudaStream_t s, uint32_t spp);
    int render_reference(cudaStream_t s, uint32_t spp);
    uint32_t effective_wave_spp(uint32_t spp) const;
    FrameParams frame_params(uint32_t spp, uint32_t slots, uint32_t tiles_x) const;
    bool last_frame_megakernel_ = false;
    uint64_t mk_paths_ = 0;

    int device_ = 0;
    cudaStream_t stream_ = nullptr;        // stream of the most recent call
    cudaStream_t owned_stream_ = nullptr;  // created by init() when the host gave none
    bool own_stream_ = false;
    int sm_count_ = 0;
    std::string error_;
    Q_cuda_options opt_{};

    // scene (original triangle order)
    bool has_scene_ = false;
    bool bvh_dirty_ = true;
    uint32_t n_tris_ = 0;
    uint32_t n_emit_ = 0;
    uint32_t n_quads_ = 0;
    DeviceBuffer raw_vertices_;   // 9 floats per triangle (upload staging)
    DeviceBuffer tri_in_;         // 3 float4 per triangle
    DeviceBuffer albedo_;         // float4 per triangle
    DeviceBuffer emission_;       // float4 per triangle
    DeviceBuffer emitters_;       // int per emitter (original index)
    DeviceBuffer quads_;          // reference integrator: 3 float4 + 2 float4 material per quad
    Q_camera scene_camera_{};
    LbvhBuilder bvh_;

    // frame
    uint32_t width_ = 0, height_ = 0;
    uint32_t samples_ = 0;        // samples accumulated so far
    uint32_t frame_index_ = 0;    // frames since the last reset (reference integrator seeding)
    Q_camera camera_{};
    DeviceBuffer accum_;          // float4 per pixel: Kahan sum (rgb)
    DeviceBuffer comp_;           // float4 per pixel: Kahan compensation
    DeviceBuffer aov_albedo_;     // float4 per pixel: sum of albedo (rgb), depth (w)
    DeviceBuffer aov_normal_;     // float4 per pixel: sum of remapped normal
    DeviceBuffer record_rad_;     // per-sample radiance (record_samples)
    DeviceBuffer record_sig_;     // per-sample signatures (record_samples)
    DeviceBuffer resolve_;        // float4 per pixel: the image a readback copies to the host
    uint32_t record_spp_ = 0;

    // wavefront
    DeviceBuffer queue_[2];       // 2 float4 per ray
    DeviceBuffer hits_;           // float4 per ray: t, prim, u, v
    DeviceBuffer shadow_;         // 4 float4 per shadow ray
    DeviceBuffer beta_, lpath_, aov_a_, aov_n_, sig_;
    DeviceBuffer ray_ff_;         // 3 float4 per path: double-float ray of the next segment
    DeviceBuffer defer_;          // int2 per path slot: rays deferred to the fixup kernels
    DeviceBuffer counters_;       // int counters of the current frame
    DeviceBuffer stats_dev_;      // uint64 stats
    DeviceBuffer err_dev_;        // uint32 error bits
    uint32_t wave_capacity_ = 0;
    uint32_t counter_capacity_ = 0;
    int* counters_host_ = nullptr;            // pinned
    unsigned long long* stats_host_ = nullptr;// pinned
    uint32_t* err_host_ = nullptr;            // pinned
    uint32_t counters_used_ = 0;
    bool stats_pending_ = false;
    Q_cuda_stats last_stats_{};
    uint64_t total_samples_ = 0;

    KernelProfiler prof_;
    cudaEvent_t ev_frame0_ = nullptr, ev_frame1_ = nullptr, ev_bvh0_ = nullptr, ev_bvh1_ = nullptr;
    bool bvh_timed_ = false;
    bool frame_timed_ = false;
};

}  // namespace quasi
