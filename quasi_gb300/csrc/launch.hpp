// launch.hpp - kernel launch bookkeeping: error checks, a launch counter and optional
// per-kernel CUDA-event timing on the launching stream.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

namespace quasi {

// Path slots of a wave that fit in device memory: at most `want`, leaving a sixteenth of
// the device free; `held` is what the wave buffers already occupy (freed when they grow).
// A device with less free memory gets smaller waves (slower, same images) instead of an
// allocation failure.
inline uint64_t wave_paths_fitting(uint64_t want, size_t bytes_per_path, size_t held) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return want;
    }
    const size_t margin = total_b / 16;
    const size_t avail = free_b + held > margin ? free_b + held - margin : 0;
    const uint64_t fit = avail / bytes_per_path;
    return fit < want ? fit : want;
}

// Resident blocks per SM of `kernel` launched with `threads` threads and `smem` bytes of
// dynamic shared memory, at least 1. The persistent kernels size their grids with it; they
// loop over their work, so a grid of one block per SM (the answer if the query itself fails,
// whose error is then cleared so a later launch check does not report it) is slower, never
// wrong.
template <class Kernel>
int resident_blocks(Kernel kernel, int threads, size_t smem) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return occ > 1 ? occ : 1;
}

// NVTX range over a host scope (frame, LBVH build, wave): lets a profiler attribute and
// filter the launches inside it (ncu --nvtx --nvtx-include "quasi.wave/"). Without an
// attached tool the calls return at once.
class NvtxRange {
public:
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

class KernelProfiler {
public:
    ~KernelProfiler() {
        for (auto& r : pending_) { pool_.push_back(r.a); pool_.push_back(r.b); }
        for (cudaEvent_t e : pool_) cudaEventDestroy(e);
    }

    void set_enabled(bool on) { enabled_ = on; }
    bool enabled() const { return enabled_; }

    // Brackets one launch on `stream`; returns false if an event could not be created.
    void begin(const char* name, cudaStream_t stream) {
        ++launches_;
        if (!enabled_) return;
        Rec r{name, take(), take()};
        if (r.a && r.b) cudaEventRecord(r.a, stream);
        pending_.push_back(r);
    }
    void end(cudaStream_t stream) {
        if (!enabled_ || pending_.empty()) return;
        Rec& r = pending_.back();
        if (r.a && r.b) cudaEventRecord(r.b, stream);
    }

    // Call after the stream has been synchronised: folds pending events into totals.
    void collect() {
        for (auto& r : pending_) {
            float ms = 0.f;
            if (r.a && r.b && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
                auto& t = totals_[r.name];
                t.first += 1;
                t.second += ms;
            }
            if (r.a) pool_.push_back(r.a);
            if (r.b) pool_.push_back(r.b);
        }
        pending_.clear();
    }

    void reset_totals() { totals_.clear(); }
    uint32_t launches() const { return launches_; }
    void reset_launches() { launches_ = 0; }
    const std::map<std::string, std::pair<uint32_t, double>>& totals() const { return totals_; }

private:
    struct Rec { const char* name; cudaEvent_t a; cudaEvent_t b; };
    cudaEvent_t take() {
        if (!pool_.empty()) { cudaEvent_t e = pool_.back(); pool_.pop_back(); return e; }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        return e;
    }
    bool enabled_ = false;
    uint32_t launches_ = 0;
    std::vector<Rec> pending_;
    std::vector<cudaEvent_t> pool_;
    std::map<std::string, std::pair<uint32_t, double>> totals_;
};

}  // namespace quasi

// Launches `call` (a <<<>>> expression) on `stream`, counting and optionally timing it.
// Evaluates to a cudaError_t from cudaGetLastError().
#define QUASI_LAUNCH(prof, name, stream, call) \
    ([&]() -> cudaError_t {                    \
        (prof).begin(name, stream);            \
        call;                                  \
        (prof).end(stream);                    \
        return cudaGetLastError();             \
    }())

#define QUASI_TRY_CUDA(expr)                                       \
    do {                                                           \
        cudaError_t quasi_err_ = (expr);                           \
        if (quasi_err_ != cudaSuccess) return quasi_err_;          \
    } while (0)
