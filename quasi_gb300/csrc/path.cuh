// path.cuh - per-path device code shared by every form of the NEE path tracer: the
// single-scene wavefront (wavefront_kernels.cuh), the one-thread-per-path megakernel and
// adjoint (megakernel.cuh) and the multi-scene batch (batch_kernels.cuh).
//
// A path is addressed by its scene-local id `local` = j * slots + slot: sample
// f.sample_base + j of the pixel at `slot` (pixel slots are ordered in 8x4 tiles). Its state
// lives at a path-state index `pid` of the current wave's buffers; the single-scene renderer
// uses pid == local (per wave), the batch maps pid -> (scene, local) through a table.
// Every form calls the same functions here with the same keys, so a path sample gets the
// same radiance bit for bit whichever form traced it.
#pragma once

#include "common.cuh"
#include "ffmath.cuh"
#include "shading.cuh"
#include "trace.cuh"
#include "wide.cuh"

namespace quasi {

// Camera basis (plugin.mm:134-147) as double-float vectors, split on the host from double.
// Camera basis as double-float vectors (hi, lo): the unnormalised direction of pixel
// position (x + jx, y + jy) is base + step_x (x + jx) - step_y (y + jy), with
// base = lower-left corner + vertical - origin, step_x = horizontal / width and
// step_y = vertical / height (plugin.mm:134-153 with u = (x + jx) / W, v = 1 - (y + jy) / H).
struct CameraFF {
    float3 origin;
    float3 base_hi, base_lo, sx_hi, sx_lo, sy_hi, sy_lo;
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
    const float4* nodes;
    const float4* tris;     // leaf order, v0+orig, e1, e2
    uint32_t n_tris, n_emit;
    int refill;             // idle lanes that trigger a ray refill in the trace kernels
    int steps;              // node visits per lane between refill checks
    const float4* tree;     // top BVH levels, breadth first, staged in shared memory
    int tree_n;             // nodes in `tree` (0 = no staging)
    const float4* wide;     // 8-wide traversal records (wide.cuh) for the wavefront trace
                            // kernels, or null: they traverse `nodes`
    const float4* tri_plane;  // per triangle: unit normal and plane offset n.v0, double-float
    const float4* emit_tab;   // per emitter slot: light-sampling record, 5 float4 (k_emit_table)
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
    float4* aov_a;      // first-hit albedo (rgb) + depth (w)
    float4* aov_n;      // first-hit remapped normal
    float4* ray_ff;     // 3 float4 per path: the double-float ray of the path's next segment
    uint32_t* sig;      // path signatures (record mode) or null
};

// Rays a fast trace kernel could not decide for certain (robust.cuh): entries (ray index,
// undecided candidate) for the fixup kernel.
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

// Adds a per-thread count to *out with one atomic per warp (all lanes must call).
__device__ __forceinline__ void warp_add_count(int v, unsigned long long* out) {
    unsigned long long x = static_cast<unsigned long long>(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(out, x);
}

// Camera ray of (pixel x,y; sample) in double-float: jitter (r1, r2) inside the pixel,
// u = (x + r1) / W, v = 1 - (y + r2) / H, direction = normalize(ll + u h + v v' - o), as
// base + step_x (x + r1) - step_y (y + r2) with the per-frame vectors of CameraFF.
__device__ __forceinline__ void camera_ray_ff(const FrameParams& f, uint32_t x, uint32_t y, uint32_t sample, ff3& o,
                                              ff3& d) {
    uint32_t st = path_key(f.seed, y * f.width + x, sample, 0u);
    const float jx = rng_next(st);
    const float jy = rng_next(st);
    const ff px = two_sum(static_cast<float>(x), jx), py = two_sum(static_cast<float>(y), jy);
    d = ff3_normalize(ff3_sub_fast(ff3_add_fast(ff3_pair(f.cam.base_hi, f.cam.base_lo),
                                                ff3_scale(ff3_pair(f.cam.sx_hi, f.cam.sx_lo), px)),
                                   ff3_scale(ff3_pair(f.cam.sy_hi, f.cam.sy_lo), py)));
    o = ff3v(f.cam.origin);
}

// Distance along the ray (o, d) to just before where it enters the scene's bounding box (the
// union of the binary LBVH root's child boxes), or 0 when it starts inside or misses it.
__device__ __forceinline__ float scene_entry(const float4* __restrict__ nodes, float3 o, float3 d) {
    const float4 n0 = __ldg(&nodes[0]), n1 = __ldg(&nodes[1]), n2 = __ldg(&nodes[2]);
    const float lo[3] = {fminf(n0.x, n1.x), fminf(n0.z, n1.z), fminf(n2.x, n2.z)};
    const float hi[3] = {fmaxf(n0.y, n1.y), fmaxf(n0.w, n1.w), fmaxf(n2.y, n2.w)};
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    float t0 = 0.0f, t1 = __int_as_float(0x7f800000);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float inv = 1.0f / dd[a];
        float ta = (lo[a] - oo[a]) * inv, tb = (hi[a] - oo[a]) * inv;
        if (ta > tb) { const float x = ta; ta = tb; tb = x; }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
    }
    return t0 <= t1 ? t0 * (1.0f - 0x1p-8f) : 0.0f;
}

// Starts path `local` in state slot `pid`: returns false for a slot outside the image;
// otherwise initialises the state and returns the FP32 camera ray in (o, d). The FP32 ray
// starts where the exact (double-float) camera ray enters the scene's bounding box (nodes:
// the binary LBVH; no shift when n_tris is 0): the error bound of an FP32 triangle test
// grows with the distance from the ray's origin (robust.cuh), and camera rays otherwise
// cross the empty space between the camera and the scene first. The shift te is kept in
// lpath.w for the exact geometry of a re-decision (ExactShifted); the stored double-float ray
// keeps the camera origin, from which shading measures the first hit's depth.
__device__ __forceinline__ bool begin_path(const FrameParams& f, const PathDev& p, uint32_t pid, uint32_t local,
                                           const float4* __restrict__ nodes, uint32_t n_tris, float3& o, float3& d) {
    const uint32_t j = local / f.slots;
    uint32_t x, y;
    slot_to_xy(local - j * f.slots, f.tiles_x, x, y);
    if (x >= f.width || y >= f.height) return false;
    ff3 ro, rd;
    camera_ray_ff(f, x, y, f.sample_base + j, ro, rd);
    ff_ray_store(&p.ray_ff[3ull * pid], ro, rd);
    d = ff3_f(rd);
    const float te = n_tris ? scene_entry(nodes, f.cam.origin, d) : 0.0f;
    o = te > 0.0f ? ff3_f(ff3_add(ro, ff3_scale(rd, te))) : f.cam.origin;  // as ExactShifted
    // beta starts at 1 and the first-hit AOVs at 0 without being stored: shading at bounce 1
    // takes beta as 1 and writes the AOVs of every path, hit or missed (miss_at_bounce)
    p.lpath[pid] = make_float4(0.f, 0.f, 0.f, te);
    if (p.sig) p.sig[pid] = 0u;
    return true;
}

// Closest-hit queue: ray i is q[2i] = (origin, path id), q[2i+1] = (direction, excluded
// triangle); the result is hits[i] = (t, triangle or -1, path id, 0), so shading reads the
// path id with the hit. The exact ray of path pid is ray_ff[3 pid] (the path's double-float
// segment). A deferred ray leaves its certain result in hits[i] for the fixup kernel.
// The exact geometry of a closest-hit ray: the path's double-float ray, started te along
// its direction (te: the shift of a camera ray's FP32 start, begin_path; 0 for the other
// rays), the same point the FP32 ray was rounded from, so exact and FP32 distances agree.
struct ExactShifted {
    const float4* ray;
    float te;
    __device__ __forceinline__ void get(ff3& o, ff3& d) const {
        ff_ray_load(ray, o, d);
        if (te > 0.0f) o = ff3_add(o, ff3_scale(d, te));
    }
};

struct ClosestJob {
    const float4* __restrict__ q;
    float4* __restrict__ hits;
    const float4* __restrict__ ray_ff;
    const float4* __restrict__ lpath;  // .w: the camera ray's FP32 start shift (begin_path)
    DeferList deferred;
    // Set by the trace kernels: one shared-memory word per thread that carries the path id of
    // the thread's ray from load() to store(); null: store() reads it from the queue.
    int* slot_pid;
    __device__ __forceinline__ int pid(int i) const { return __float_as_int(q[2 * i].w); }
    __device__ __forceinline__ ExactShifted exact(int i) const {
        const int id = pid(i);
        return ExactShifted{ray_ff + 3ull * id, lpath[id].w};
    }
    __device__ __forceinline__ void defer(int i, const TraceResult& r) const {
        store(i, r);
        deferred.push(i, r.undec);
    }
    __device__ __forceinline__ HitBest partial(int i) const {
        const float4 h = hits[i];
        HitBest b;
        b.lo = b.hi = h.x;
        b.prim = __float_as_int(h.y);
        b.undec = k_undec_none;
        return b;
    }
    __device__ __forceinline__ void load(int i, float3& o, float3& d, float& tmax, int& exclude) const {
        const float4 r0 = q[2 * i], r1 = q[2 * i + 1];
        o = xyz(r0);
        d = xyz(r1);
        tmax = __int_as_float(0x7f800000);
        exclude = __float_as_int(r1.w);
        if (slot_pid) slot_pid[threadIdx.x] = __float_as_int(r0.w);
    }
    __device__ __forceinline__ void store(int i, const TraceResult& s) const {
        const int id = slot_pid ? slot_pid[threadIdx.x] : pid(i);
        hits[i] = make_float4(s.t, __int_as_float(s.prim), __int_as_float(id), 0.f);
    }
};

// The exact segment of a shadow ray, for re-decisions: its start (the lifted light sample,
// double-float: the hi parts are the queue's FP32 origin, the lo parts ride in the queue
// entry) and its end, the lifted shading point, which is the origin of the path's stored
// double-float ray (shading writes it whether or not the path continues).
struct ExactSeg {
    ff3 start;
    const float4* ray;
    __device__ __forceinline__ void get(ff3& o, ff3& d) const {
        ff3 end, unused;
        ff_ray_load(ray, end, unused);
        o = start;
        d = ff3_sub(end, start);
    }
};

// Shadow queue, 4 float4 per ray: sq[4i] = (origin, path id), sq[4i+1] = (direction, t_max),
// sq[4i+2] = (contribution, origin lo.x), sq[4i+3] = (origin lo.y, origin lo.z, -, -); an
// unoccluded ray adds its contribution to the path's radiance. A deferred ray found no
// certain occluder (it would have stopped there), so its certain result is "unoccluded".
struct ShadowJob {
    const float4* __restrict__ sq;
    PathDev p;
    DeferList deferred;
    __device__ __forceinline__ int pid(int i) const { return __float_as_int(sq[4 * i].w); }
    __device__ __forceinline__ ExactSeg exact(int i) const {
        const float4 a = sq[4 * i], c = sq[4 * i + 2], e = sq[4 * i + 3];
        return ExactSeg{ff3{ff{a.x, c.w}, ff{a.y, e.x}, ff{a.z, e.y}}, p.ray_ff + 3ull * __float_as_int(a.w)};
    }
    __device__ __forceinline__ void defer(int i, const TraceResult& r) const { deferred.push(i, r.undec); }
    __device__ __forceinline__ HitBest partial(int i) const {
        HitBest b;
        b.lo = b.hi = sq[4 * i + 1].w;
        b.prim = -1;
        b.undec = k_undec_none;
        return b;
    }
    __device__ __forceinline__ void load(int i, float3& o, float3& d, float& tmax, int& exclude) const {
        const float4 r0 = sq[4 * i], r1 = sq[4 * i + 1];
        o = xyz(r0);
        d = xyz(r1);
        tmax = r1.w;
        exclude = -1;
    }
    __device__ __forceinline__ void store(int i, const TraceResult& s) const {
        const int pid = __float_as_int(sq[4 * i].w);
        if (s.prim < 0) {
            const float4 c = sq[4 * i + 2];
            float4 L = p.lpath[pid];
            L.x += c.x;
            L.y += c.y;
            L.z += c.z;
            p.lpath[pid] = L;
        }
        if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], s.prim < 0 ? k_sig_lit : k_sig_shadowed);
    }
};

// Traversal modes of the persistent trace kernels.
constexpr int k_mode_batch = 0;       // warp batches of 32 rays, nodes from global memory
constexpr int k_mode_batch_tree = 1;  // warp batches, top levels from shared memory
constexpr int k_mode_refill = 2;      // per-lane refill (trace_persistent)
constexpr int k_mode_wide = 3;        // warp batches over the 8-wide records (trace_batches_wide)
constexpr int k_mode_wide_refill = 4; // per-lane refill over the 8-wide records (trace_wide_refill)

// A path whose closest-hit ray of bounce `bounce` missed: its signature, and at bounce 1 the
// zero first-hit AOVs the camera kernel leaves unwritten.
__device__ __forceinline__ void miss_at_bounce(const PathDev& p, uint32_t bounce, int pid) {
    if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], k_sig_miss);
    if (bounce == 1) {
        p.aov_a[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.aov_n[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Minimum resident 256-thread blocks per SM asked of the compiler for k_shade and
// k_batch_shade (a register cap). Before the shading table k_shade took 141 registers
// uncapped and the 1080p frame's shading cost 138 ms; 2 blocks (128 registers) or 4 (64,
// with spills) cost 101 ms on GB300. With the continuation finished before the light sample
// (shade_and_enqueue) it fits 78 registers without spills at 3 blocks; 4 blocks (64
// registers, 36 bytes spilled) cost 20 % more (33.6 vs 40.2 ms per 1080p frame).
#ifndef QUASI_SHADE_MIN_BLOCKS
#define QUASI_SHADE_MIN_BLOCKS 3
#endif

// Shades the closest hit h = (t, prim, u, v) at bounce `bounce` of path `local` (state slot
// `pid`) and enqueues the rays it asks for; all lanes of the warp call it, `active` lanes
// hold a hit (prim >= 0), and f and s are only read for them. In order: the hit point,
// first-hit emission and AOVs, beta; the continuation ray (stored double-float ray and next
// queue); then the NEE sample (shadow queue) and the signature. Finishing the continuation
// before the light triangle is loaded keeps fewer values live at once than computing both
// from one set of loads; the values are those of shade_vertex.
__device__ __forceinline__ void shade_and_enqueue(bool active, const FrameParams& f, const SceneDev& s,
                                                  const PathDev& p, uint32_t bounce, int pid, uint32_t local,
                                                  float4 h, float4* __restrict__ shadow_q,
                                                  int* __restrict__ shadow_count, float4* __restrict__ next_q,
                                                  int* __restrict__ next_count) {
    const int prim = __float_as_int(h.y);
    ff3 x{}, nrm{}, org{};
    float3 nb = mk3(0.f, 0.f, 0.f);
    bool cont = false;
    VertexRandom r{};
    if (active) {
        const VertexScene vs{s.tri_plane, s.emit_tab, s.n_emit, f.eps};
        ff3 ro, rd;
        ff_ray_load(&p.ray_ff[3ull * pid], ro, rd);
        const uint32_t j = local / f.slots;
        uint32_t px, py;
        slot_to_xy(local - j * f.slots, f.tiles_x, px, py);
        r = vertex_random(path_key(f.seed, py * f.width + px, f.sample_base + j, bounce));
        const float3 alb = xyz(__ldg(&s.albedo[prim]));
        nb = bounce == 1 ? alb : xyz(p.beta[pid]) * alb;  // beta is 1 at the first hit (1 * a = a)
        cont = bounce < f.max_depth && max3(nb) > 0.0f;
        float t_hit;
        vertex_point(vs, prim, ro, rd, x, nrm, t_hit);
        org = vertex_origin(vs, x, nrm);
        if (bounce == 1) {
            const float3 em = xyz(__ldg(&s.emission[prim]));
            p.lpath[pid] = make_float4(em.x, em.y, em.z, 0.f);
            // the depth from the camera: the plane's t along the (unshifted) double-float ray
            first_hit_aovs(alb, em, t_hit, ff3_f(nrm), p.aov_a[pid], p.aov_n[pid]);
        }
        p.beta[pid] = make_float4(nb.x, nb.y, nb.z, 0.f);
    }
    // The continuation ray.
    float3 nd = mk3(0.f, 0.f, 0.f);
    if (active && cont) {
        const ff3 dir = vertex_dir(nrm, r.r3, r.r4);
        ff_ray_store(&p.ray_ff[3ull * pid], org, dir);
        nd = ff3_f(dir);
    }
    const bool want_next = active && cont && next_count != nullptr;
    const int pn = warp_append(0xffffffffu, want_next, next_count);
    if (want_next) {
        const float3 no = ff3_f(org);
        next_q[2 * pn] = make_float4(no.x, no.y, no.z, __int_as_float(pid));
        next_q[2 * pn + 1] = make_float4(nd.x, nd.y, nd.z, __int_as_float(prim));
    }
    // The NEE sample.
    VertexResult v;
    v.nee = false;
    if (active) {
        const VertexScene vs{s.tri_plane, s.emit_tab, s.n_emit, f.eps};
        const LightTri lt = load_light(vs, r.sel);
        vertex_light(vs, prim, lt, r.r1, r.r2, x, nrm, org, v);
        // without a continuation the stored ray keeps only the shadow segment's end (ExactSeg)
        if (v.nee && !cont) ff_ray_store(&p.ray_ff[3ull * pid], org, ff3{});
    }
    const int ps = warp_append(0xffffffffu, v.nee, shadow_count);
    if (v.nee) {
        const float3 contrib = nb * xyz(__ldg(&s.emission[v.light])) * v.g;
        shadow_q[4 * ps] = make_float4(v.so.x, v.so.y, v.so.z, __int_as_float(pid));
        shadow_q[4 * ps + 1] = make_float4(v.sd.x, v.sd.y, v.sd.z, v.stmax);
        shadow_q[4 * ps + 2] = make_float4(contrib.x, contrib.y, contrib.z, v.seg_o.x.lo);
        shadow_q[4 * ps + 3] = make_float4(v.seg_o.y.lo, v.seg_o.z.lo, 0.f, 0.f);
    }
    if (active && p.sig) {
        uint32_t sig = sig_mix(p.sig[pid], static_cast<uint32_t>(prim));
        if (!v.nee) sig = sig_mix(sig, k_sig_no_nee);
        p.sig[pid] = sig;
    }
}

// Kahan-adds samples pid0, pid0 + stride, ... (n of them, in sample order) of one pixel to
// its accumulators; records per-sample radiance and signatures when rec_rad is set.
__device__ __forceinline__ void accumulate_pixel(const PathDev& p, uint32_t pid0, uint32_t stride, uint32_t n,
                                                 float4* accum, float4* comp, float4* aov_a, float4* aov_n,
                                                 float* rec_rad, uint32_t* rec_sig, size_t rec_idx) {
    float4 sum = *accum, c = *comp, A = *aov_a, N = *aov_n;
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t pid = pid0 + j * stride;
        const float4 L = p.lpath[pid];
        kahan_add(sum.x, c.x, L.x);
        kahan_add(sum.y, c.y, L.y);
        kahan_add(sum.z, c.z, L.z);
        const float4 a = p.aov_a[pid], nn = p.aov_n[pid];
        A.x += a.x; A.y += a.y; A.z += a.z; A.w += a.w;
        N.x += nn.x; N.y += nn.y; N.z += nn.z;
        if (rec_rad) {
            const size_t idx = rec_idx + j;
            rec_rad[3 * idx] = L.x;
            rec_rad[3 * idx + 1] = L.y;
            rec_rad[3 * idx + 2] = L.z;
            rec_sig[idx] = p.sig ? p.sig[pid] : 0u;
        }
    }
    *accum = sum;
    *comp = c;
    *aov_a = A;
    *aov_n = N;
}

// ------------------------------------------------------------------ one thread per path

constexpr int k_adjoint_max_depth = 16;

struct PathVertex {
    int prim;
    int light;
    float gv;
};

// Traces one path sample; fills up to k_adjoint_max_depth vertices when `verts` is given.
// One thread follows one path here, so no lane can take new work while the others finish
// their rays; the binary LBVH traversal (fewer registers) is the faster one in that form:
// the 10k-triangle adjoint took 5.5 ms with it and 7.2 ms with the 8-wide records on GB300.
// Returns the radiance; writes first-hit AOVs and the signature when the pointers are set.
// rays / shadow_rays are incremented per closest-hit / shadow ray traced. Hit decisions are
// exact (robust traversal, re-deciding undecided candidates inline from the path's
// double-float geometry); pad is the scene's box padding (scene_box_pad).
template <bool STATS>
__device__ __forceinline__ float3 trace_path(const FrameParams& f, const SceneDev& s, uint32_t x, uint32_t y,
                                             uint32_t sample, PathVertex* verts, int& n_verts, float4* aov_a,
                                             float4* aov_n, uint32_t* sig_out, uint32_t& err, TraceCounters& cnt,
                                             int& rays, int& shadow_rays, float pad) {
    const VertexScene vs{s.tri_plane, s.emit_tab, s.n_emit, f.eps};
    ff3 ro, rd;
    camera_ray_ff(f, x, y, sample, ro, rd);
    float3 beta = mk3(1.f, 1.f, 1.f), L = mk3(0.f, 0.f, 0.f);
    uint32_t sig = 0;
    int exclude = -1;
    n_verts = 0;
    for (uint32_t k = 1; k <= f.max_depth; ++k) {
        const RayInv r = make_ray(ff3_f(ro), ff3_f(rd), pad);
        ++rays;
        const HitBest hb = trace_bvh<false, STATS, false, true>(s.nodes, s.tris, s.tri_in, s.n_tris, r,
                                                                __int_as_float(0x7f800000), exclude, err, cnt,
                                                                ExactRegs{ro, rd});
        const int prim = hb.prim;
        const float t = hit_t(hb);
        if (prim < 0) {
            sig = sig_mix(sig, k_sig_miss);
            break;
        }
        const float3 alb = xyz(__ldg(&s.albedo[prim]));
        const float3 nb = beta * alb;
        const bool cont = k < f.max_depth && max3(nb) > 0.0f;
        VertexResult v;
        shade_vertex(vs, path_key(f.seed, y * f.width + x, sample, k), prim, make_float4(t, 0.f, 0.f, 0.f), ro, rd,
                     cont, v);
        sig = sig_mix(sig, static_cast<uint32_t>(prim));
        if (k == 1) {
            const float3 em = xyz(__ldg(&s.emission[prim]));
            L = em;
            if (aov_a) first_hit_aovs(alb, em, v.t, v.nrm, *aov_a, *aov_n);
        }
        float gv = 0.0f;
        if (v.nee) {
            const RayInv sr = make_ray(v.so, v.sd, pad);
            ++shadow_rays;
            const int occ = trace_bvh<true, STATS, false, true>(s.nodes, s.tris, s.tri_in, s.n_tris, sr, v.stmax, -1,
                                                                err, cnt, ExactRegs{v.seg_o, v.seg_d})
                                .prim;
            if (occ < 0) {
                // The same product and the same unfused add as the wavefront's shadow kernel.
                const float3 cb = beta * alb * xyz(__ldg(&s.emission[v.light])) * v.g;
                L = mk3(__fadd_rn(L.x, cb.x), __fadd_rn(L.y, cb.y), __fadd_rn(L.z, cb.z));
                gv = v.g;
                sig = sig_mix(sig, k_sig_lit);
            } else {
                sig = sig_mix(sig, k_sig_shadowed);
            }
        } else {
            sig = sig_mix(sig, k_sig_no_nee);
        }
        if (verts && n_verts < k_adjoint_max_depth) verts[n_verts] = PathVertex{prim, v.nee ? v.light : -1, gv};
        ++n_verts;
        beta = nb;
        if (!cont) break;
        ro = v.org;
        rd = v.dir;
        exclude = prim;
    }
    if (sig_out) *sig_out = sig;
    return L;
}

// Path-replay adjoint of one path sample with pixel adjoint d (= dLoss/dI_pixel / spp).
// With vertices k = 1..K on triangles h_k (albedo rho_k), NEE lights l_k with factors gv_k
// (g times visibility, 0 without an unoccluded light sample) and throughput
// beta_k = prod_{j<k} rho_j:
//   radiance = Le(h_1) + sum_k beta_k rho_k Le(l_k) gv_k
//   dL/dLe(h_1)  += d
//   dL/dLe(l_k)  += d beta_k rho_k gv_k
//   dL/drho(h_k) += d beta_k H_k,  H_k = Le(l_k) gv_k + rho_{k+1} H_{k+1},  H_{K+1} = 0
// (all products per colour channel). H_k needs no division by albedo, so zero albedos are
// exact. The vertex records of the path (at most k_adjoint_max_depth) live in local memory.
// `rays` is incremented by the rays the replay traces.
__device__ __forceinline__ void adjoint_path(const FrameParams& f, const SceneDev& s, uint32_t x, uint32_t y,
                                             uint32_t sample, float3 d, float* __restrict__ grad_albedo,
                                             float* __restrict__ grad_emission, uint32_t& err, TraceCounters& cnt,
                                             int& rays, float pad) {
    PathVertex verts[k_adjoint_max_depth];
    float3 H[k_adjoint_max_depth];
    int nv = 0, shadow_rays = 0;
    trace_path<false>(f, s, x, y, sample, verts, nv, nullptr, nullptr, nullptr, err, cnt, rays, shadow_rays, pad);
    rays += shadow_rays;
    nv = min(nv, k_adjoint_max_depth);
    if (nv == 0) return;
    atomicAdd(&grad_emission[3 * verts[0].prim + 0], d.x);
    atomicAdd(&grad_emission[3 * verts[0].prim + 1], d.y);
    atomicAdd(&grad_emission[3 * verts[0].prim + 2], d.z);
    float3 next = mk3(0.f, 0.f, 0.f);
    for (int k = nv - 1; k >= 0; --k) {
        float3 h = mk3(0.f, 0.f, 0.f);
        if (verts[k].light >= 0 && verts[k].gv != 0.0f) h = xyz(__ldg(&s.emission[verts[k].light])) * verts[k].gv;
        if (k + 1 < nv) h += xyz(__ldg(&s.albedo[verts[k + 1].prim])) * next;
        H[k] = h;
        next = h;
    }
    float3 beta = mk3(1.f, 1.f, 1.f);
    for (int k = 0; k < nv; ++k) {
        const int h = verts[k].prim;
        const float3 rho = xyz(__ldg(&s.albedo[h]));
        const float3 ga = d * beta * H[k];
        atomicAdd(&grad_albedo[3 * h + 0], ga.x);
        atomicAdd(&grad_albedo[3 * h + 1], ga.y);
        atomicAdd(&grad_albedo[3 * h + 2], ga.z);
        if (verts[k].light >= 0 && verts[k].gv != 0.0f) {
            const float3 ge = d * beta * rho * verts[k].gv;
            atomicAdd(&grad_emission[3 * verts[k].light + 0], ge.x);
            atomicAdd(&grad_emission[3 * verts[k].light + 1], ge.y);
            atomicAdd(&grad_emission[3 * verts[k].light + 2], ge.z);
        }
        beta = beta * rho;
    }
}

}  // namespace quasi
