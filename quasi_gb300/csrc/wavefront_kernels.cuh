// wavefront_kernels.cuh - device kernels of the NEE path tracer (included by wavefront.cu).
//
// One wave = wave_spp samples of every pixel. Per wave:
//   k_camera          camera rays for every (sample, pixel) -> ray queue
//   for bounce k = 1..D:
//     k_trace_closest persistent, warp-fetched closest-hit traversal of the queue (FP32)
//     k_shade         emission (k == 1), AOVs (k == 1), light sample -> shadow queue,
//                     cosine-weighted continuation -> next ray queue; both queues are
//                     compacted with one atomic per warp (ballot + popc)
//     k_trace_shadow  persistent any-hit traversal (FP32); unoccluded rays add their
//                     contribution to the owning path's radiance
//   k_accumulate      per pixel, Kahan-adds the wave's samples in sample order
// Paths are addressed by a stable id (sample-in-wave * slots + tile-ordered pixel slot); a
// path has at most one ray in each queue, so no two threads ever update the same path.
//
// Precision: traversal decides which triangle a ray hits in FP32. The path geometry (ray
// origins and directions, the hit point, the light sample and the shading frame) is
// carried in double-float (ffmath.cuh): each vertex re-intersects the hit triangle's plane
// with the double-float ray, so a path's radiance matches the FP64 oracle to ~1e-7 even
// where short segments in a corner would amplify FP32 rounding by 1e4.
#pragma once

#include "common.cuh"
#include "ffmath.cuh"
#include "shading.cuh"
#include "trace.cuh"

namespace quasi {

// Camera basis (plugin.mm:134-147) as double-float vectors, split on the host from double.
struct CameraFF {
    float3 origin;
    float3 ll_hi, ll_lo, h_hi, h_lo, v_hi, v_lo;
};

struct FrameParams {
    CameraFF cam;
    uint32_t width, height, tiles_x, slots;
    uint32_t wave_spp, sample_base;
    uint32_t seed, max_depth;
    float eps;
    uint32_t frame_spp, wave_offset;
};

struct SceneDev {
    const float4* tri_in;   // original order, v0 v1 v2
    const float4* albedo;
    const float4* emission;
    const int* emitters;
    const float4* nodes;
    const float4* tris;     // leaf order, v0+orig, e1, e2
    uint32_t n_tris, n_emit;
    int refill;             // idle lanes that trigger a ray refill in the trace kernels
    int steps;              // node visits per lane between refill checks
    const float4* tree;     // top BVH levels, breadth first, staged in shared memory
    int tree_n;             // nodes in `tree` (0 = no staging)
};

// Copies the treelet into the block's shared memory (dynamic size tree_n * 64 bytes).
__device__ __forceinline__ const float4* stage_treelet(const SceneDev& s) {
    extern __shared__ float4 s_tree[];
    for (int i = threadIdx.x; i < 4 * s.tree_n; i += blockDim.x) s_tree[i] = __ldg(&s.tree[i]);
    __syncthreads();
    return s_tree;
}

struct PathDev {
    float4* beta;
    float4* lpath;
    float4* aov_a;   // first-hit albedo (rgb) + depth (w)
    float4* aov_n;   // first-hit remapped normal
    float4* ray_ff;  // 3 float4 per path: the double-float ray of the path's next segment
    uint32_t* sig;   // path signatures (record mode) or null
};

// Pixel slots are ordered in 8x4 tiles so a warp's camera rays cover a compact patch.
__device__ __forceinline__ void slot_to_xy(uint32_t slot, uint32_t tiles_x, uint32_t& x, uint32_t& y) {
    const uint32_t tile = slot >> 5, in = slot & 31u;
    const uint32_t ty = tile / tiles_x, tx = tile - ty * tiles_x;
    x = tx * 8u + (in & 7u);
    y = ty * 4u + (in >> 3);
}
__device__ __forceinline__ uint32_t xy_to_slot(uint32_t x, uint32_t y, uint32_t tiles_x) {
    return ((((y >> 2) * tiles_x) + (x >> 3)) << 5) | ((y & 3u) << 3) | (x & 7u);
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float x) {
    const float y = x - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

__device__ __forceinline__ ff3 ff3_pair(float3 hi, float3 lo) {
    return ff3{ff{hi.x, lo.x}, ff{hi.y, lo.y}, ff{hi.z, lo.z}};
}

__global__ void __launch_bounds__(256) k_pack_tris(const float* __restrict__ raw, uint32_t n, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = raw + 9ull * i;
    out[3 * i + 0] = make_float4(v[0], v[1], v[2], 0.f);
    out[3 * i + 1] = make_float4(v[3], v[4], v[5], 0.f);
    out[3 * i + 2] = make_float4(v[6], v[7], v[8], 0.f);
}

__global__ void __launch_bounds__(256) k_camera(FrameParams f, PathDev p, float4* __restrict__ q, int* __restrict__ q_count) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= f.wave_spp * f.slots) return;  // slots is a multiple of 32: whole warps leave
    const uint32_t j = gid / f.slots, slot = gid - j * f.slots;
    uint32_t x, y;
    slot_to_xy(slot, f.tiles_x, x, y);
    const bool valid = x < f.width && y < f.height;
    float3 d = mk3(0.f, 0.f, 0.f);
    if (valid) {
        const uint32_t pixel = y * f.width + x;
        uint32_t st = path_key(f.seed, pixel, f.sample_base + j, 0u);
        const float jx = rng_next(st);
        const float jy = rng_next(st);
        // u = (x + jx) / W, v = 1 - (y + jy) / H, direction = normalize(ll + u h + v v' - o)
        const ff u = ff_div(two_sum(static_cast<float>(x), jx), ffv(static_cast<float>(f.width)));
        const ff v = ff_sub(ffv(1.0f), ff_div(two_sum(static_cast<float>(y), jy), ffv(static_cast<float>(f.height))));
        const ff3 dir = ff3_normalize(ff3_sub(ff3_add(ff3_add(ff3_pair(f.cam.ll_hi, f.cam.ll_lo),
                                                              ff3_scale(ff3_pair(f.cam.h_hi, f.cam.h_lo), u)),
                                                      ff3_scale(ff3_pair(f.cam.v_hi, f.cam.v_lo), v)),
                                              ff3v(f.cam.origin)));
        ff_ray_store(&p.ray_ff[3ull * gid], ff3v(f.cam.origin), dir);
        d = ff3_f(dir);
        p.beta[gid] = make_float4(1.f, 1.f, 1.f, 0.f);
        p.lpath[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.aov_a[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.aov_n[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p.sig) p.sig[gid] = 0u;
    }
    const int pos = warp_append(0xffffffffu, valid, q_count);
    if (valid) {
        q[2 * pos] = make_float4(f.cam.origin.x, f.cam.origin.y, f.cam.origin.z, __int_as_float(static_cast<int>(gid)));
        q[2 * pos + 1] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    }
}

template <bool STATS>
__device__ __forceinline__ void flush_counters(const TraceCounters& c, unsigned long long* stats) {
    if (!STATS) return;
    uint32_t a = c.nodes, b = c.tris;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[0], static_cast<unsigned long long>(a));
        atomicAdd(&stats[1], static_cast<unsigned long long>(b));
    }
}

// Closest-hit queue: ray i is q[2i] = (origin, path id), q[2i+1] = (direction, excluded
// triangle); the result is hits[i] = (t, triangle or -1, u, v).
struct ClosestJob {
    const float4* __restrict__ q;
    float4* __restrict__ hits;
    __device__ __forceinline__ void load(int i, float3& o, float3& d, float& tmax, int& exclude) const {
        const float4 r0 = q[2 * i], r1 = q[2 * i + 1];
        o = xyz(r0);
        d = xyz(r1);
        tmax = __int_as_float(0x7f800000);
        exclude = __float_as_int(r1.w);
    }
    __device__ __forceinline__ void store(int i, const TraceState& s) const {
        hits[i] = make_float4(s.best_t, __int_as_float(s.best), s.bu, s.bv);
    }
};

// Shadow queue: sq[3i] = (origin, path id), sq[3i+1] = (direction, t_max), sq[3i+2] =
// (contribution); an unoccluded ray adds its contribution to the path's radiance.
struct ShadowJob {
    const float4* __restrict__ sq;
    PathDev p;
    __device__ __forceinline__ void load(int i, float3& o, float3& d, float& tmax, int& exclude) const {
        const float4 r0 = sq[3 * i], r1 = sq[3 * i + 1];
        o = xyz(r0);
        d = xyz(r1);
        tmax = r1.w;
        exclude = -1;
    }
    __device__ __forceinline__ void store(int i, const TraceState& s) const {
        const int pid = __float_as_int(sq[3 * i].w);
        if (s.best < 0) {
            const float4 c = sq[3 * i + 2];
            float4 L = p.lpath[pid];
            L.x += c.x;
            L.y += c.y;
            L.z += c.z;
            p.lpath[pid] = L;
        }
        if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], s.best < 0 ? k_sig_lit : k_sig_shadowed);
    }
};

// Traversal modes of the persistent trace kernels.
constexpr int k_mode_batch = 0;       // warp batches of 32 rays, nodes from global memory
constexpr int k_mode_batch_tree = 1;  // warp batches, top levels from shared memory
constexpr int k_mode_refill = 2;      // per-lane refill (trace_persistent)

// Persistent closest-hit traversal.
template <bool STATS, int MODE>
__global__ void __launch_bounds__(256) k_trace_closest(SceneDev s, const float4* __restrict__ q,
                                                       float4* __restrict__ hits, const int* __restrict__ count,
                                                       int capacity, int* __restrict__ fetch,
                                                       uint32_t* __restrict__ err, unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    ClosestJob job{q, hits};
    if (MODE == k_mode_refill)
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
__global__ void __launch_bounds__(256) k_trace_shadow(SceneDev s, PathDev p, const float4* __restrict__ sq,
                                                      const int* __restrict__ count, int capacity,
                                                      int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                      unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    uint32_t e = 0;
    TraceCounters c;
    ShadowJob job{sq, p};
    if (MODE == k_mode_refill)
        trace_persistent<true, STATS>(job, s.nodes, s.tris, s.n_tris, n, s.refill, s.steps, fetch, e, c);
    else if (MODE == k_mode_batch_tree)
        trace_batches<true, STATS, true>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, stage_treelet(s), s.tree_n);
    else
        trace_batches<true, STATS, false>(job, s.nodes, s.tris, s.n_tris, n, fetch, e, c, nullptr, 0);
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats + 2);
}

// Adds the frame's queue lengths (rays traced) to the cumulative counter stats[4]; one
// warp, so the timed loop needs no host synchronisation to know how many rays it traced.
__global__ void k_tally(const int* __restrict__ counters, uint32_t waves, uint32_t depth,
                        unsigned long long* __restrict__ stats) {
    unsigned long long sum = 0;
    for (uint32_t i = threadIdx.x; i < waves * 2 * depth; i += 32) {
        const uint32_t w = i / (2 * depth), k = i - w * 2 * depth;
        sum += static_cast<unsigned long long>(max(counters[w * 4 * depth + k], 0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (threadIdx.x == 0) stats[4] += sum;
}

__global__ void __launch_bounds__(256) k_shade(FrameParams f, SceneDev s, PathDev p, uint32_t bounce,
                                               const float4* __restrict__ q, const float4* __restrict__ hits,
                                               const int* __restrict__ count, int capacity, float4* __restrict__ next_q,
                                               int* __restrict__ next_count, float4* __restrict__ shadow_q,
                                               int* __restrict__ shadow_count) {
    const int n = min(*count, capacity);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const VertexScene vs{s.tri_in, s.albedo, s.emission, s.emitters, s.n_emit, f.eps};
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
        const int i = base + lane;
        bool want_shadow = false, want_next = false;
        float3 contrib = mk3(0.f, 0.f, 0.f), norg = contrib, nd = contrib;
        VertexResult v;
        v.so = v.sd = contrib;
        v.stmax = 0.f;
        int pid = 0, prim = -1;
        if (i < n) {
            const float4 h = hits[i];
            pid = __float_as_int(q[2 * i].w);
            prim = __float_as_int(h.y);
            if (prim < 0) {
                if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], k_sig_miss);
            } else {
                ff3 ro, rd;
                ff_ray_load(&p.ray_ff[3ull * pid], ro, rd);
                const uint32_t j = static_cast<uint32_t>(pid) / f.slots;
                uint32_t px, py;
                slot_to_xy(static_cast<uint32_t>(pid) - j * f.slots, f.tiles_x, px, py);
                const uint32_t key = path_key(f.seed, py * f.width + px, f.sample_base + j, bounce);
                const float3 alb = xyz(__ldg(&s.albedo[prim]));
                float3 beta = xyz(p.beta[pid]);
                const float3 nb = beta * alb;
                const bool cont = bounce < f.max_depth && max3(nb) > 0.0f;
                shade_vertex(vs, key, prim, h, ro, rd, cont, v);
                uint32_t sig = p.sig ? sig_mix(p.sig[pid], static_cast<uint32_t>(prim)) : 0u;
                if (bounce == 1) {
                    const float3 em = xyz(__ldg(&s.emission[prim]));
                    p.lpath[pid] = make_float4(em.x, em.y, em.z, 0.f);
                    first_hit_aovs(alb, em, h.x, v.nrm, p.aov_a[pid], p.aov_n[pid]);
                }
                if (v.nee) {
                    contrib = beta * alb * xyz(__ldg(&s.emission[v.light])) * v.g;
                    want_shadow = true;
                } else {
                    sig = sig_mix(sig, k_sig_no_nee);
                }
                p.beta[pid] = make_float4(nb.x, nb.y, nb.z, 0.f);
                if (p.sig) p.sig[pid] = sig;
                want_next = cont;
                if (want_next) {
                    ff_ray_store(&p.ray_ff[3ull * pid], v.org, v.dir);
                    norg = ff3_f(v.org);
                    nd = ff3_f(v.dir);
                }
            }
        }
        const int ps = warp_append(0xffffffffu, want_shadow, shadow_count);
        if (want_shadow) {
            shadow_q[3 * ps] = make_float4(v.so.x, v.so.y, v.so.z, __int_as_float(pid));
            shadow_q[3 * ps + 1] = make_float4(v.sd.x, v.sd.y, v.sd.z, v.stmax);
            shadow_q[3 * ps + 2] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
        }
        const int pn = warp_append(0xffffffffu, want_next, next_count);
        if (want_next) {
            next_q[2 * pn] = make_float4(norg.x, norg.y, norg.z, __int_as_float(pid));
            next_q[2 * pn + 1] = make_float4(nd.x, nd.y, nd.z, __int_as_float(prim));
        }
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
    float4 sum = accum[pixel], c = comp[pixel], A = aov_a[pixel], N = aov_n[pixel];
    for (uint32_t j = 0; j < f.wave_spp; ++j) {
        const uint32_t pid = j * f.slots + slot;
        const float4 L = p.lpath[pid];
        kahan_add(sum.x, c.x, L.x);
        kahan_add(sum.y, c.y, L.y);
        kahan_add(sum.z, c.z, L.z);
        const float4 a = p.aov_a[pid], nn = p.aov_n[pid];
        A.x += a.x; A.y += a.y; A.z += a.z; A.w += a.w;
        N.x += nn.x; N.y += nn.y; N.z += nn.z;
        if (rec_rad) {
            const size_t idx = static_cast<size_t>(pixel) * f.frame_spp + f.wave_offset + j;
            rec_rad[3 * idx] = L.x;
            rec_rad[3 * idx + 1] = L.y;
            rec_rad[3 * idx + 2] = L.z;
            rec_sig[idx] = p.sig ? p.sig[pid] : 0u;
        }
    }
    accum[pixel] = sum;
    comp[pixel] = c;
    aov_a[pixel] = A;
    aov_n[pixel] = N;
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
