// wavefront_kernels.cuh - device kernels of the single-scene NEE path tracer (included by
// wavefront.cu).
//
// One wave = wave_spp samples of every pixel. Per wave:
//   k_camera          camera rays for every (sample, pixel) -> ray queue
//   for bounce k = 1..D:
//     k_trace_closest persistent, warp-fetched closest-hit traversal of the queue (FP32),
//                     over the 8-wide records (wide.cuh) or the binary LBVH nodes
//     k_fixup         re-traces the rays the trace kernel could not decide for certain,
//                     with exact (double-float) re-decisions (robust.cuh)
//     k_shade         emission (k == 1), AOVs (k == 1), light sample -> shadow queue,
//                     cosine-weighted continuation -> next ray queue; both queues are
//                     compacted with one atomic per warp (ballot + popc)
//     k_trace_shadow  persistent any-hit traversal (FP32); unoccluded rays add their
//                     contribution to the owning path's radiance
//     k_fixup         the same for the shadow rays
//   k_accumulate      per pixel, Kahan-adds the wave's samples in sample order
// Paths are addressed by a stable id (sample-in-wave * slots + tile-ordered pixel slot); a
// path has at most one ray in each queue, so no two threads ever update the same path.
//
// Precision: traversal tests triangles in FP32 with a rigorous error bound per test; the
// few rays that meet a candidate the bound cannot decide are re-traced with double-float
// decisions, so every hit decision agrees with exact arithmetic. The path geometry (ray
// origins and directions, the hit point, the light sample and the shading frame) is
// carried in double-float (ffmath.cuh): each vertex re-intersects the hit triangle's plane
// with the double-float ray, so a path's radiance matches the FP64 oracle to ~1e-7 even
// where short segments in a corner would amplify FP32 rounding by 1e4.
#pragma once

#include "path.cuh"

#include <type_traits>

namespace quasi {

__global__ void __launch_bounds__(256) k_pack_tris(const float* __restrict__ raw, uint32_t n, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = raw + 9ull * i;
    out[3 * i + 0] = make_float4(v[0], v[1], v[2], 0.f);
    out[3 * i + 1] = make_float4(v[3], v[4], v[5], 0.f);
    out[3 * i + 2] = make_float4(v[6], v[7], v[8], 0.f);
}

__global__ void __launch_bounds__(256) k_camera(FrameParams f, SceneDev s, PathDev p, float4* __restrict__ q,
                                                int* __restrict__ q_count) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    float3 o = mk3(0.f, 0.f, 0.f), d = o;
    const bool valid = gid < f.wave_spp * f.slots && begin_path(f, p, gid, gid, s.nodes, s.n_tris, o, d);
    const int pos = block_append(valid, q_count);
    if (valid) {
        q[2 * pos] = make_float4(o.x, o.y, o.z, __int_as_float(static_cast<int>(gid)));
        q[2 * pos + 1] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    }
}

constexpr int trace_min_blocks(int mode) { return mode >= k_mode_wide ? QUASI_WIDE_MIN_BLOCKS : 1; }

// Persistent closest-hit traversal.
template <bool STATS, int MODE>
__global__ void __launch_bounds__(256, trace_min_blocks(MODE)) k_trace_closest(SceneDev s, ClosestJob job,
                                                       const int* __restrict__ count, int capacity,
                                                       int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                       unsigned long long* __restrict__ stats) {
    __shared__ int s_pid[256];
    job.slot_pid = s_pid;
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    if (MODE == k_mode_wide)
        trace_batches_wide<false, STATS>(job, s.wide, s.tris, s.n_tris, n, fetch, e, c);
    else if (MODE == k_mode_wide_refill)
        trace_wide_refill<false, STATS>(job, s.wide, s.tris, s.n_tris, n, s.refill, fetch, e, c);
    else if (MODE == k_mode_refill)
        trace_persistent<false, STATS>(job, s.nodes, s.tris, s.n_tris, n, s.refill, s.steps, fetch, e, c);
    else if (MODE == k_mode_batch_tree)
        trace_batches<false, STATS, true>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, stage_treelet(s), s.tree_n);
    else
        trace_batches<false, STATS, false>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, nullptr, 0);
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats);
}

// Persistent any-hit traversal of the shadow queue.
template <bool STATS, int MODE>
__global__ void __launch_bounds__(256, trace_min_blocks(MODE)) k_trace_shadow(SceneDev s, ShadowJob job,
                                                      const int* __restrict__ count, int capacity,
                                                      int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                      unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    if (MODE == k_mode_wide)
        trace_batches_wide<true, STATS>(job, s.wide, s.tris, s.n_tris, n, fetch, e, c);
    else if (MODE == k_mode_wide_refill)
        trace_wide_refill<true, STATS>(job, s.wide, s.tris, s.n_tris, n, s.refill, fetch, e, c);
    else if (MODE == k_mode_refill)
        trace_persistent<true, STATS>(job, s.nodes, s.tris, s.n_tris, n, s.refill, s.steps, fetch, e, c);
    else if (MODE == k_mode_batch_tree)
        trace_batches<true, STATS, true>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, stage_treelet(s), s.tree_n);
    else
        trace_batches<true, STATS, false>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, nullptr, 0);
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats + 2);
}

// Completes the rays a closest-hit or shadow trace kernel deferred (robust.cuh): re-decides
// each ray's recorded candidate exactly against its certain result, or re-traces a ray that
// met more than one (over the 8-wide records when the scene has them: a third of the
// binary LBVH's dependent node fetches), and stores the final results. The list lengths are
// read on the device, so the launch needs no host synchronisation; a persistent grid takes
// one chunk of 32 entries per warp (resolve_deferred).
template <class Job>
__global__ void __launch_bounds__(128) k_fixup(SceneDev s, Job job, int* __restrict__ fetch,
                                               uint32_t* __restrict__ err) {
    constexpr bool any = std::is_same<Job, ShadowJob>::value;
    uint32_t e = 0;
    const float pad = s.n_tris && !s.wide ? scene_box_pad(s.nodes) : 0.0f;
    auto retrace = [&](int i, float3 o, float3 d, float tmax, int exclude) {
        if (s.wide) return trace_wide_exact<any>(s.wide, s.tris, s.tri_in, s.n_tris, o, d, tmax, exclude, job.exact(i), e);
        TraceCounters cnt;
        return trace_bvh<any, false, false, true>(s.nodes, s.tris, s.tri_in, s.n_tris, make_ray(o, d, pad), tmax,
                                                  exclude, e, cnt, job.exact(i));
    };
    resolve_deferred<any>(job, [&](int) { return s.tri_in; }, job.deferred, fetch, retrace);
    if (e) atomicOr(err, e);
}

// Per-wave frame counters, k_counters_per_bounce per bounce: [0, D) closest-hit queue
// lengths, [D, 2D) shadow queue lengths, [2D, 3D) and [3D, 4D) their trace fetch counters,
// [4D, 5D) and [5D, 6D) the rays each deferred with one undecided candidate, [6D, 8D) the
// fixup kernels' fetch counters, [8D, 9D) and [9D, 10D) the rays each deferred to be
// re-traced whole.
constexpr uint32_t k_counters_per_bounce = 10;

// Adds the frame's queue lengths (rays traced) to the cumulative counter stats[4]; one
// warp, so the timed loop needs no host synchronisation to know how many rays it traced.
__global__ void k_tally(const int* __restrict__ counters, uint32_t waves, uint32_t depth,
                        unsigned long long* __restrict__ stats) {
    unsigned long long sum = 0;
    for (uint32_t i = threadIdx.x; i < waves * 2 * depth; i += 32) {
        const uint32_t w = i / (2 * depth), k = i - w * 2 * depth;
        sum += static_cast<unsigned long long>(max(counters[w * k_counters_per_bounce * depth + k], 0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (threadIdx.x == 0) stats[4] += sum;
}

__global__ void __launch_bounds__(256, QUASI_SHADE_MIN_BLOCKS) k_shade(FrameParams f, SceneDev s, PathDev p, uint32_t bounce,
                                               const float4* __restrict__ hits,
                                               const int* __restrict__ count, int capacity, float4* __restrict__ next_q,
                                               int* __restrict__ next_count, float4* __restrict__ shadow_q,
                                               int* __restrict__ shadow_count) {
    const int n = min(*count, capacity);
    const int stride = gridDim.x * blockDim.x;
    // One warp-aggregated atomic per queue and warp: aggregating over the block instead (two
    // barriers per append) made this kernel 9 % slower; the camera kernel, one short pass per
    // thread, gained from it (block_append).
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const int i = base + static_cast<int>(threadIdx.x);
        int pid = 0;
        float4 h = make_float4(0.f, __int_as_float(-1), 0.f, 0.f);
        if (i < n) {
            h = hits[i];
            pid = __float_as_int(h.z);
            if (__float_as_int(h.y) < 0) miss_at_bounce(p, bounce, pid);
        }
        shade_and_enqueue(i < n && __float_as_int(h.y) >= 0, f, s, p, bounce, pid, static_cast<uint32_t>(pid), h,
                          shadow_q, shadow_count, next_q, next_count);
    }
}

__global__ void __launch_bounds__(256) k_accumulate(FrameParams f, PathDev p, float4* __restrict__ accum,
                                                    float4* __restrict__ comp, float4* __restrict__ aov_a,
                                                    float4* __restrict__ aov_n, float* __restrict__ rec_rad,
                                                    uint32_t* __restrict__ rec_sig) {
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= f.width * f.height) return;
    const uint32_t y = pixel / f.width, x = pixel - y * f.width;
    const uint32_t slot = xy_to_slot(x, y, f.tiles_x);
    accumulate_pixel(p, slot, f.slots, f.wave_spp, &accum[pixel], &comp[pixel], &aov_a[pixel], &aov_n[pixel], rec_rad,
                     rec_sig, static_cast<size_t>(pixel) * f.frame_spp + f.wave_offset);
}

// Mean image (RGBA, alpha 1) from the accumulation: mode 0 beauty, 1 albedo, 2 normal, 3 depth.
__global__ void __launch_bounds__(256) k_resolve(const float4* __restrict__ accum, const float4* __restrict__ aov_a,
                                                 const float4* __restrict__ aov_n, uint32_t n_px, float count,
                                                 int mode, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_px) return;
    float4 v;
    if (mode == 0) v = accum[i];
    else if (mode == 1 || mode == 3) v = aov_a[i];
    else v = aov_n[i];
    float4 o;
    if (count <= 0.0f) o = make_float4(0.f, 0.f, 0.f, 1.f);
    else if (mode == 3) { const float d = v.w / count; o = make_float4(d, d, d, 1.f); }
    else o = make_float4(v.x / count, v.y / count, v.z / count, 1.f);
    out[i] = o;
}

// plugin.mm:334-350: Reinhard then gamma 1/2.2, written as RGBA8 into a device buffer.
__global__ void __launch_bounds__(256) k_tonemap(const float4* __restrict__ accum, uint32_t n_px, float count,
                                                 uchar4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_px) return;
    const float4 s = accum[i];
    const float inv = count > 0.f ? 1.0f / count : 0.f;
    float c[3] = {s.x * inv, s.y * inv, s.z * inv};
    unsigned char b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float m = c[k] / (c[k] + 1.0f);
        const float g = powf(fmaxf(m, 0.0f), 1.0f / 2.2f);
        b[k] = static_cast<unsigned char>(fminf(g * 255.0f + 0.5f, 255.0f));
    }
    out[i] = make_uchar4(b[0], b[1], b[2], 255);
}

}  // namespace quasi
