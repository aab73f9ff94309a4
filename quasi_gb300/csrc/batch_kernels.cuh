// batch_kernels.cuh - device kernels of the multi-scene batch renderer (included by batch.cu).
//
// A batch frame renders spp_s samples of every pixel of every scene s. The host cuts each
// scene's samples into items (runs of whole sample planes: nj samples x slots_s pixel
// slots) and packs the items into waves of at most wave_paths path slots, in scene order;
// a scene appears at most once per wave. The item table is the device work queue: every
// kernel of a wave maps its path slot or pixel thread to an item by binary search, and the
// persistent kernels take paths or rays from it with one atomic per warp.
//
// Per wave (wavefront form):
//   k_batch_camera           path slots -> (scene, local path id) table, camera rays -> queue
//   for bounce k = 1..D:     (D = the largest max_depth of the batch)
//     k_batch_trace_closest  persistent closest-hit traversal; each ray uses its scene's BVH
//     k_batch_shade          the single-scene shading code with the ray's scene parameters
//     k_batch_trace_shadow   persistent any-hit traversal
//   k_batch_accumulate       per (scene, pixel) Kahan adds of the wave's samples, in order
// or (megakernel form) k_batch_megakernel + k_batch_accumulate. Because items keep whole
// sample planes in sample order and a scene's samples are accumulated in the same order as
// the single-scene renderer's, every image of the batch is bit-identical to rendering that
// scene alone with the same seed.
//
// The first sample of the current frame of every scene lives in the device scene table
// (f.sample_base) and k_batch_advance moves it on at the end of the frame, so the whole
// frame is a fixed launch sequence that is captured once as a CUDA graph and replayed.
#pragma once

#include "path.cuh"

#include <type_traits>

namespace quasi {

struct BatchSceneDev {
    FrameParams f;          // camera, size, seed, depth, eps; f.sample_base = first sample of this frame
    SceneDev s;             // geometry and materials (pointers into the batch pools)
    uint32_t px_offset;     // first pixel of the scene in the batch image pools
    uint32_t tri_offset;    // first triangle of the scene in the batch material pools
    uint32_t spp;           // samples per frame
    uint32_t pad;
};

// A run of whole sample planes [j0, j0 + nj) of one scene inside one wave.
struct BatchItem {
    uint32_t scene;
    uint32_t j0, nj;
    uint32_t slots;         // pixel slots of the scene (multiple of 32)
    uint32_t pid_base;      // first path slot of the item in the wave
    uint32_t acc_base;      // first accumulate thread of the item in the wave
};

// Index of the last item whose `base` (pid_base or acc_base) is <= key; items are sorted.
template <bool ACC>
__device__ __forceinline__ int find_item(const BatchItem* __restrict__ items, int n_items, uint32_t key) {
    int lo = 0, hi = n_items - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const uint32_t b = ACC ? __ldg(&items[mid].acc_base) : __ldg(&items[mid].pid_base);
        if (b <= key) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Scene-local path id of wave path slot `pid` (which lies inside item `it`).
__device__ __forceinline__ uint32_t item_local(const BatchItem& it, uint32_t pid) {
    return it.j0 * it.slots + (pid - it.pid_base);
}

__global__ void __launch_bounds__(256) k_batch_camera(const BatchSceneDev* __restrict__ scenes,
                                                      const BatchItem* __restrict__ items, int n_items, uint32_t paths,
                                                      PathDev p, uint2* __restrict__ meta, float4* __restrict__ q,
                                                      int* __restrict__ q_count) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    float3 o = mk3(0.f, 0.f, 0.f), d = o;
    bool valid = false;
    if (gid < paths) {
        const BatchItem it = items[find_item<false>(items, n_items, gid)];
        const uint32_t local = item_local(it, gid);
        meta[gid] = make_uint2(it.scene, local);
        const BatchSceneDev& b = scenes[it.scene];
        valid = begin_path(b.f, p, gid, local, b.s.nodes, b.s.n_tris, o, d);
    }
    const int pos = block_append(valid, q_count);
    if (valid) {
        q[2 * pos] = make_float4(o.x, o.y, o.z, __int_as_float(static_cast<int>(gid)));
        q[2 * pos + 1] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    }
}

// Warp-batch persistent traversal over rays of several scenes: a warp takes `chunk` rays
// (a multiple of 32) with one atomic; each ray traverses the BVH of its path's scene.
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_batches_multi(Job& job, const BatchSceneDev* __restrict__ scenes,
                                                    const uint2* __restrict__ meta, int n, int chunk,
                                                    int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        for (int r = 0; r < chunk; r += 32) {
            const int i = base + r + lane;
            if (i < n) {
                const SceneDev& s = scenes[meta[job.pid(i)].x].s;
                float3 o, d;
                float tmax;
                int exclude;
                job.load(i, o, d, tmax, exclude);
                const RayInv r = make_ray(o, d, s.n_tris ? scene_box_pad(s.nodes) : 0.0f);
                finish_ray(job, i, trace_result(trace_bvh<ANY, STATS>(s.nodes, s.tris, nullptr, s.n_tris, r, tmax,
                                                                      exclude, err, cnt)));
            }
        }
    }
}

// Persistent traversal over rays of several scenes with per-lane refill on the 8-wide
// records: once `refill` lanes of a warp are idle they take the next rays with one atomic;
// each lane traverses the records of its own ray's scene. Blocks are launched with
// wide_stack_smem_bytes<ANY>(blockDim.x) of dynamic shared memory (the stacks' shared part).
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_wide_refill_multi(Job& job, const BatchSceneDev* __restrict__ scenes,
                                                        const uint2* __restrict__ meta, int n, int refill,
                                                        int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
    WideRay q;
    WideStack<wide_smem_stack<ANY>()> stack;
    stack.slot = wide_stack_slot<ANY>();
    const float4* wide = nullptr;
    const float4* tris = nullptr;
    bool active = false, exhausted = false;
    int idx = 0;
    while (true) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(idle) >= refill) {
            const int leader = __ffs(idle) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + __popc(idle) >= n;
            if (!active) {
                idx = base + __popc(idle & lanemask_lt());
                if (idx < n) {
                    const SceneDev& s = scenes[meta[job.pid(idx)].x].s;
                    wide = s.wide;
                    tris = s.tris;
                    float3 o, d;
                    float tmax;
                    int exclude;
                    job.load(idx, o, d, tmax, exclude);
                    wide_begin(q, o, d, tmax, exclude, s.n_tris);
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        bool done = false;
        if (active) {
#pragma unroll 1
            for (int i = 0; i < wide_visits_per_check<ANY>(); ++i) {
                done = wide_visit<ANY, STATS>(wide, tris, q, stack, err, cnt);
                if (done) break;
            }
        }
        if (done) {
            finish_ray(job, idx, trace_result(q.b));
            active = false;
        }
    }
}

// WIDE: per-lane refill over the 8-wide records (refill = idle lanes that trigger a fetch);
// otherwise warp chunks over the scenes' binary LBVHs.
template <bool STATS, bool WIDE>
__global__ void __launch_bounds__(256, WIDE ? QUASI_WIDE_MIN_BLOCKS : 1) k_batch_trace_closest(const BatchSceneDev* __restrict__ scenes,
                                                             const uint2* __restrict__ meta, ClosestJob job,
                                                             const int* __restrict__ count,
                                                             int capacity, int chunk, int refill, int* __restrict__ fetch,
                                                             uint32_t* __restrict__ err,
                                                             unsigned long long* __restrict__ stats) {
    __shared__ int s_pid[256];
    job.slot_pid = s_pid;
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    if (WIDE)
        trace_wide_refill_multi<false, STATS>(job, scenes, meta, n, refill, fetch, e, c);
    else
        trace_batches_multi<false, STATS>(job, scenes, meta, n, chunk, fetch, e, c);
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats);
}

template <bool STATS, bool WIDE>
__global__ void __launch_bounds__(256, WIDE ? QUASI_WIDE_MIN_BLOCKS : 1) k_batch_trace_shadow(const BatchSceneDev* __restrict__ scenes,
                                                            const uint2* __restrict__ meta, ShadowJob job,
                                                            const int* __restrict__ count,
                                                            int capacity, int chunk, int refill,
                                                            int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                            unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    if (WIDE)
        trace_wide_refill_multi<true, STATS>(job, scenes, meta, n, refill, fetch, e, c);
    else
        trace_batches_multi<true, STATS>(job, scenes, meta, n, chunk, fetch, e, c);
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats + 2);
}

// Completes the rays a batch trace kernel deferred (robust.cuh) with each ray's scene:
// re-decides its recorded candidate exactly against its certain result, or re-traces a ray
// that met more than one over the scene's 8-wide records or binary LBVH (resolve_deferred).
template <class Job>
__global__ void __launch_bounds__(128) k_batch_fixup(const BatchSceneDev* __restrict__ scenes,
                                                     const uint2* __restrict__ meta, Job job,
                                                     int* __restrict__ fetch, uint32_t* __restrict__ err) {
    constexpr bool any = std::is_same<Job, ShadowJob>::value;
    uint32_t e = 0;
    auto scene = [&](int i) -> const SceneDev& { return scenes[meta[job.pid(i)].x].s; };
    auto retrace = [&](int i, float3 o, float3 d, float tmax, int exclude) {
        const SceneDev& s = scene(i);
        if (s.wide) return trace_wide_exact<any>(s.wide, s.tris, s.tri_in, s.n_tris, o, d, tmax, exclude, job.exact(i), e);
        TraceCounters cnt;
        const RayInv r = make_ray(o, d, s.n_tris ? scene_box_pad(s.nodes) : 0.0f);
        return trace_bvh<any, false, false, true>(s.nodes, s.tris, s.tri_in, s.n_tris, r, tmax, exclude, e, cnt,
                                                  job.exact(i));
    };
    resolve_deferred<any>(job, [&](int i) { return scene(i).tri_in; }, job.deferred, fetch, retrace);
    if (e) atomicOr(err, e);
}

__global__ void __launch_bounds__(256, QUASI_SHADE_MIN_BLOCKS) k_batch_shade(const BatchSceneDev* __restrict__ scenes,
                                                     const uint2* __restrict__ meta, PathDev p, uint32_t bounce,
                                                     const float4* __restrict__ hits,
                                                     const int* __restrict__ count, int capacity,
                                                     float4* __restrict__ next_q, int* __restrict__ next_count,
                                                     float4* __restrict__ shadow_q, int* __restrict__ shadow_count) {
    const int n = min(*count, capacity);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
        const int i = base + lane;
        int pid = 0;
        uint2 m = make_uint2(0u, 0u);  // scene 0 stands in for lanes without a hit (not read)
        float4 h = make_float4(0.f, __int_as_float(-1), 0.f, 0.f);
        if (i < n) {
            h = hits[i];
            pid = __float_as_int(h.z);
            if (__float_as_int(h.y) < 0) {
                miss_at_bounce(p, bounce, pid);
            } else {
                m = meta[pid];
            }
        }
        const BatchSceneDev& b = scenes[m.x];
        shade_and_enqueue(i < n && __float_as_int(h.y) >= 0, b.f, b.s, p, bounce, pid, m.y, h, shadow_q,
                          shadow_count, next_q, next_count);
    }
}

// One thread per (item, pixel slot): Kahan-adds the item's nj samples of that pixel.
__global__ void __launch_bounds__(256) k_batch_accumulate(const BatchSceneDev* __restrict__ scenes,
                                                          const BatchItem* __restrict__ items, int n_items,
                                                          uint32_t threads, PathDev p, float4* __restrict__ accum,
                                                          float4* __restrict__ comp, float4* __restrict__ aov_a,
                                                          float4* __restrict__ aov_n) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= threads) return;
    const BatchItem it = items[find_item<true>(items, n_items, t)];
    const uint32_t slot = t - it.acc_base;
    const BatchSceneDev& b = scenes[it.scene];
    uint32_t x, y;
    slot_to_xy(slot, b.f.tiles_x, x, y);
    if (x >= b.f.width || y >= b.f.height) return;
    const size_t px = static_cast<size_t>(b.px_offset) + y * b.f.width + x;
    accumulate_pixel(p, it.pid_base + slot, it.slots, it.nj, &accum[px], &comp[px], &aov_a[px], &aov_n[px], nullptr,
                     nullptr, 0);
}

// Megakernel form: warps take `chunk` paths of the wave per atomic and trace each to the end.
// Ray counts go to stats[5] (closest-hit) and stats[6] (shadow), both cumulative.
template <bool STATS>
__global__ void __launch_bounds__(128) k_batch_megakernel(const BatchSceneDev* __restrict__ scenes,
                                                          const BatchItem* __restrict__ items, int n_items,
                                                          uint32_t paths, PathDev p, int chunk, int* __restrict__ fetch,
                                                          uint32_t* __restrict__ err,
                                                          unsigned long long* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int total = static_cast<int>(paths);
    uint32_t e = 0;
    TraceCounters c;
    int rays = 0, shadow_rays = 0;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        for (int r = 0; r < chunk; r += 32) {
            const int gid = base + r + lane;
            if (gid >= total) continue;
            const BatchItem it = items[find_item<false>(items, n_items, static_cast<uint32_t>(gid))];
            const uint32_t local = item_local(it, static_cast<uint32_t>(gid));
            const BatchSceneDev& b = scenes[it.scene];
            const uint32_t j = local / b.f.slots;
            uint32_t x, y;
            slot_to_xy(local - j * b.f.slots, b.f.tiles_x, x, y);
            if (x >= b.f.width || y >= b.f.height) continue;
            int nv = 0;
            float4 aa = make_float4(0.f, 0.f, 0.f, 0.f), an = aa;
            const float pad = b.s.n_tris ? scene_box_pad(b.s.nodes) : 0.0f;
            const float3 L = trace_path<STATS>(b.f, b.s, x, y, b.f.sample_base + j, nullptr, nv, &aa, &an, nullptr, e,
                                               c, rays, shadow_rays, pad);
            p.lpath[gid] = make_float4(L.x, L.y, L.z, 0.f);
            p.aov_a[gid] = aa;
            p.aov_n[gid] = an;
        }
    }
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats);
    unsigned long long rc = static_cast<unsigned long long>(rays), sr = static_cast<unsigned long long>(shadow_rays);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rc += __shfl_xor_sync(0xffffffffu, rc, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
    }
    if (lane == 0) {
        atomicAdd(&stats[5], rc);
        atomicAdd(&stats[6], sr);
    }
}

// Path-replay adjoint of the batch's last frame (samples [f.sample_base - spp, f.sample_base)
// of every scene). grad_image: 3 floats per pixel of the batch image pool; grads are += into
// 3 floats per triangle of the batch material pools. Rays replayed are added to stats[7].
__global__ void __launch_bounds__(128) k_batch_adjoint(const BatchSceneDev* __restrict__ scenes,
                                                       const BatchItem* __restrict__ items, int n_items, uint32_t paths,
                                                       const float* __restrict__ grad_image,
                                                       float* __restrict__ grad_albedo,
                                                       float* __restrict__ grad_emission, int chunk,
                                                       int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                       unsigned long long* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int total = static_cast<int>(paths);
    uint32_t e = 0;
    TraceCounters c;
    int rays = 0;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        for (int r = 0; r < chunk; r += 32) {
            const int gid = base + r + lane;
            if (gid >= total) continue;
            const BatchItem it = items[find_item<false>(items, n_items, static_cast<uint32_t>(gid))];
            const uint32_t local = item_local(it, static_cast<uint32_t>(gid));
            const BatchSceneDev& b = scenes[it.scene];
            const uint32_t j = local / b.f.slots;
            uint32_t x, y;
            slot_to_xy(local - j * b.f.slots, b.f.tiles_x, x, y);
            if (x >= b.f.width || y >= b.f.height) continue;
            const size_t px = static_cast<size_t>(b.px_offset) + y * b.f.width + x;
            const float inv_spp = 1.0f / static_cast<float>(b.spp);
            const float3 d = mk3(grad_image[3 * px] * inv_spp, grad_image[3 * px + 1] * inv_spp,
                                 grad_image[3 * px + 2] * inv_spp);
            if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) continue;
            const float pad = b.s.n_tris ? scene_box_pad(b.s.nodes) : 0.0f;
            adjoint_path(b.f, b.s, x, y, b.f.sample_base - b.spp + j, d, grad_albedo + 3ull * b.tri_offset,
                         grad_emission + 3ull * b.tri_offset, e, c, rays, pad);
        }
    }
    if (e) atomicOr(err, e);
    warp_add_count(rays, &stats[7]);
}

// Per-wave counters of the wavefront form, k_batch_counters_per_bounce per bounce: queue
// lengths [0, 2D), trace fetch counters [2D, 4D), rays deferred with one undecided
// candidate [4D, 6D), fixup fetch counters [6D, 8D), rays deferred to be re-traced whole
// [8D, 10D).
constexpr uint32_t k_batch_counters_per_bounce = 10;

// Adds the frame's closest-hit and shadow queue lengths to stats[5] and stats[6] and the
// rays re-traced by the fixup kernels to stats[8]. One warp.
__global__ void k_batch_tally(const int* __restrict__ counters, uint32_t waves, uint32_t depth,
                              unsigned long long* __restrict__ stats) {
    unsigned long long closest = 0, shadow = 0, redecided = 0;
    for (uint32_t i = threadIdx.x; i < waves * 2 * depth; i += 32) {
        const uint32_t w = i / (2 * depth), k = i - w * 2 * depth;
        const int* c = counters + w * k_batch_counters_per_bounce * depth;
        const unsigned long long v = static_cast<unsigned long long>(max(c[k], 0));
        if (k < depth) closest += v;
        else shadow += v;
        redecided += static_cast<unsigned long long>(max(c[4 * depth + k], 0)) +
                     static_cast<unsigned long long>(max(c[8 * depth + k], 0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        closest += __shfl_xor_sync(0xffffffffu, closest, o);
        shadow += __shfl_xor_sync(0xffffffffu, shadow, o);
        redecided += __shfl_xor_sync(0xffffffffu, redecided, o);
    }
    if (threadIdx.x == 0) {
        stats[5] += closest;
        stats[6] += shadow;
        stats[8] += redecided;
    }
}

// End of a frame: every scene's next frame starts spp samples later; stats[4] counts frames.
__global__ void k_batch_advance(BatchSceneDev* __restrict__ scenes, uint32_t n, unsigned long long* __restrict__ stats) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) scenes[i].f.sample_base += scenes[i].spp;
    if (threadIdx.x == 0) stats[4] += 1;
}

// Clears the accumulation of a reset: sample bases back to 0.
__global__ void k_batch_rewind(BatchSceneDev* __restrict__ scenes, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) scenes[i].f.sample_base = 0;
}

// A new RNG seed for every scene, and sample bases back to 0.
__global__ void k_batch_reseed(BatchSceneDev* __restrict__ scenes, uint32_t n, uint32_t seed) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        scenes[i].f.seed = seed;
        scenes[i].f.sample_base = 0;
    }
}

// Mean beauty image over pixels [px_begin, px_begin + px_count) of the batch image pool, as
// RGBA (alpha 1) or, with rgb, 3 floats per pixel. Each pixel's scene is found by binary
// search over the scenes' px_offset (scenes are stored in pool order).
__global__ void __launch_bounds__(256) k_batch_resolve(const BatchSceneDev* __restrict__ scenes, int n_scenes,
                                                       const float4* __restrict__ accum, uint32_t px_begin,
                                                       uint32_t px_count, bool rgb, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= px_count) return;
    const uint32_t px = px_begin + i;
    int lo = 0, hi = n_scenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&scenes[mid].px_offset) <= px) lo = mid;
        else hi = mid - 1;
    }
    const float count = static_cast<float>(scenes[lo].f.sample_base);
    const float4 v = accum[px];
    const float r = count > 0.0f ? v.x / count : 0.0f;
    const float g = count > 0.0f ? v.y / count : 0.0f;
    const float b = count > 0.0f ? v.z / count : 0.0f;
    if (rgb) {
        out[3ull * i] = r;
        out[3ull * i + 1] = g;
        out[3ull * i + 2] = b;
    } else {
        out[4ull * i] = r;
        out[4ull * i + 1] = g;
        out[4ull * i + 2] = b;
        out[4ull * i + 3] = 1.0f;
    }
}

// Packs device materials of the whole batch (3 floats per triangle, scenes back to back).
__global__ void __launch_bounds__(256) k_batch_pack_materials(const float* __restrict__ albedo,
                                                              const float* __restrict__ emission, uint32_t n,
                                                              float4* __restrict__ a4, float4* __restrict__ e4) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (albedo) a4[i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.f);
    if (emission) e4[i] = make_float4(emission[3 * i], emission[3 * i + 1], emission[3 * i + 2], 0.f);
}

__global__ void __launch_bounds__(256) k_batch_pack_tris(const float* __restrict__ raw, uint32_t n,
                                                         float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = raw + 9ull * i;
    out[3 * i + 0] = make_float4(v[0], v[1], v[2], 0.f);
    out[3 * i + 1] = make_float4(v[3], v[4], v[5], 0.f);
    out[3 * i + 2] = make_float4(v[6], v[7], v[8], 0.f);
}

}  // namespace quasi
