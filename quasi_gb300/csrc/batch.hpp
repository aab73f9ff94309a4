// batch.hpp - host side of the multi-scene batch renderer (Q_cuda_batch_*): scene pools,
// one LBVH per scene, the work-item plan, the captured frame and adjoint graphs and the
// autotuner. The device kernels are in batch_kernels.cuh.
#pragma once

#include "../../include/quasi_cuda.h"
#include "bvh.cuh"
#include "launch.hpp"
#include "renderer.hpp"

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace quasi {

class BatchRenderer {
public:
    explicit BatchRenderer(Renderer& owner);
    ~BatchRenderer();
    BatchRenderer(const BatchRenderer&) = delete;
    BatchRenderer& operator=(const BatchRenderer&) = delete;

    int create(const Q_cuda_batch_scene* scenes, uint32_t count, const Q_cuda_batch_options* options);
    int set_options(const Q_cuda_batch_options& o);
    Q_cuda_batch_options options() const { return opt_; }
    int render(cudaStream_t stream);
    int reset();
    int set_seed(uint32_t seed, cudaStream_t stream);
    int synchronize();
    int stats(Q_cuda_batch_stats* out);
    int readback(uint32_t index, float* host_rgba);
    int resolve_device(float* device_rgb, cudaStream_t stream);
    int offsets(uint32_t index, uint64_t* tri_offset, uint64_t* px_offset) const;
    int set_materials_device(const float* albedo, const float* emission, cudaStream_t stream);
    int backward(const float* grad_image, float* grad_albedo, float* grad_emission, cudaStream_t stream);
    int autotune(double budget_ms, Q_cuda_batch_options* chosen);
    const std::string& last_error() const { return error_; }

private:
    struct HostScene {
        uint32_t tri_offset, n_tris, width, height, spp, px_offset, emit_offset, n_emit;
        Q_camera camera;
    };
    struct Item {
        uint32_t scene, j0, nj, slots, pid_base, acc_base;
    };
    struct Wave {
        uint32_t item0, n_items, paths, acc_threads;
    };

    int fail(int code, const std::string& msg) {
        error_ = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* where);
    int validate(Q_cuda_batch_options& o) const;
    int upload_table();
    int plan(uint32_t spp_cap);
    int ensure_buffers();
    int record_frame(cudaStream_t s, uint32_t& launches);
    int record_adjoint(cudaStream_t s);
    int ensure_graphs();
    void drop_graphs();
    cudaStream_t pick(cudaStream_t s) {
        if (s) stream_ = s;
        return stream_;
    }
    void compute_grids();
    int time_frame(float& ms);

    Renderer& owner_;
    cudaStream_t stream_ = nullptr;  // stream of the most recent call (initially the plugin's)
    std::string error_;
    Q_cuda_batch_options opt_{};
    std::vector<HostScene> scenes_;
    uint64_t tri_total_ = 0, px_total_ = 0, camera_rays_ = 0;
    uint32_t max_slots_ = 0;

    // pools (scene after scene)
    DeviceBuffer tri_in_, albedo_, emission_, emitters_;
    DeviceBuffer accum_, comp_, aov_a_, aov_n_;
    std::vector<std::unique_ptr<LbvhBuilder>> bvh_;
    DeviceBuffer table_;    // BatchSceneDev per scene
    DeviceBuffer items_;    // BatchItem per item
    // wave buffers
    DeviceBuffer queue_[2], hits_, shadow_, beta_, lpath_, pa_, pn_, ray_ff_, meta_;
    DeviceBuffer defer_;  // rays deferred to the fixup kernels
    uint32_t wave_capacity_ = 0;
    DeviceBuffer counters_, adj_counters_, stats_dev_, err_dev_;
    // adjoint staging (the adjoint graph reads and writes these fixed buffers)
    DeviceBuffer grad_image_, grad_albedo_, grad_emission_;

    std::vector<Item> items_host_;
    std::vector<Wave> waves_;
    uint32_t plan_cap_ = 0xffffffffu;
    uint32_t plan_wave_paths_ = 0;
    uint32_t kernels_per_frame_ = 0;
    uint64_t frames_since_reset_ = 0;
    int grid_c_ = 0, grid_s_ = 0, grid_m_ = 0, grid_adj_ = 0;  // persistent grids (SMs x occupancy)
    size_t smem_c_ = 0, smem_s_ = 0;  // dynamic shared memory of a trace block (8-wide stacks)

    cudaStream_t capture_ = nullptr;
    cudaGraphExec_t frame_exec_ = nullptr, adjoint_exec_ = nullptr;
    bool graphs_dirty_ = true;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    bool timed_ = false;
    unsigned long long* stats_host_ = nullptr;  // pinned
    uint32_t* err_host_ = nullptr;              // pinned
    KernelProfiler prof_;                       // launch counting only
};

}  // namespace quasi
