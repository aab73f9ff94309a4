// trace.cuh - stack-based LBVH traversal with Moller-Trumbore triangle tests (FP32).
//
// Rays never store more than one stack entry per tree level (nearest child first, the far
// child is pushed), so the stack bound is the tree depth; a ray that would overflow the
// k_stack_size entries stops, reports a miss and raises QUASI_DEVERR_STACK. A traversal
// also stops after 2n + 64 node visits (a tree of n leaves has n - 1 internal nodes), which
// only a malformed hierarchy could reach (QUASI_DEVERR_TRAVERSAL).
//
// Closest hit is defined independently of traversal order: the smallest t wins and an
// exact tie goes to the smaller original triangle index. The oracle uses the same rule.
// Hit decisions agree with exact arithmetic (robust.cuh): every FP32 triangle test carries
// an error bound, boxes are padded by more than the slab planes' rounding, and box tests
// cull beyond the closest hit's t plus its error bound. Undecided candidates are either
// recorded for the fixup kernel (fast mode) or re-decided in double-float (ROBUST).
//
// Traversal is written as a resumable step (one node visit) so persistent kernels can keep
// every lane of a warp busy: a lane whose ray finishes takes a new ray from the queue while
// the other lanes continue (trace_persistent).
#pragma once

#include "common.cuh"
#include "robust.cuh"

namespace quasi {

constexpr int k_stack_size = 64;
// Persistent kernels refill a warp once at least this many of its lanes are idle (default).
constexpr int k_refill_lanes = 32;
// Node visits per lane between two refill checks (default).
constexpr int k_trace_steps = 8;
// BVH levels staged in shared memory by default (2^5 - 1 = 31 nodes, 2 KB per block).
// Measured on GB300 (soup 1M, 1080p): 5 levels is neutral, 7 slightly slower, 9 (32 KB per
// block) 22% slower; the top levels are L1-resident either way.
constexpr int k_default_smem_levels = 5;

// Spatial box padding Delta of the scene whose binary LBVH is `nodes`: 2^-16 times the
// largest absolute vertex coordinate S (the root's child boxes hold every vertex). The
// 8-wide records are padded by the same Delta when they are built (k_collapse8); the binary
// traversal pads its slab planes per ray.
__device__ __forceinline__ float scene_box_pad(const float4* __restrict__ nodes) {
    const float4 n0 = __ldg(&nodes[0]), n1 = __ldg(&nodes[1]), n2 = __ldg(&nodes[2]);
    const float sxy = fmaxf(fmaxf(fmaxf(fabsf(n0.x), fabsf(n0.y)), fmaxf(fabsf(n0.z), fabsf(n0.w))),
                            fmaxf(fmaxf(fabsf(n1.x), fabsf(n1.y)), fmaxf(fabsf(n1.z), fabsf(n1.w))));
    const float sz = fmaxf(fmaxf(fabsf(n2.x), fabsf(n2.y)), fmaxf(fabsf(n2.z), fabsf(n2.w)));
    return __fmul_rn(fmaxf(fmaxf(sxy, sz), 0x1p-100f), k_box_pad_rel);
}

struct RayInv {
    float3 o;
    float3 d;
    float3 inv;     // 1/d with tiny components clamped away from zero
    float3 oinv_lo; // (o + pad) * inv: lower slab planes moved out by pad
    float3 oinv_hi; // (o - pad) * inv: upper slab planes moved out by pad
};

__device__ __forceinline__ float safe_inv(float x) {
    const float ax = fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x);
    return 1.0f / ax;
}

// pad: spatial box padding (scene_box_pad); 0 for the 8-wide records, which carry it.
__device__ __forceinline__ RayInv make_ray(float3 o, float3 d, float pad = 0.0f) {
    RayInv r;
    r.o = o;
    r.d = d;
    r.inv = mk3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    r.oinv_lo = mk3((o.x + pad) * r.inv.x, (o.y + pad) * r.inv.y, (o.z + pad) * r.inv.z);
    r.oinv_hi = mk3((o.x - pad) * r.inv.x, (o.y - pad) * r.inv.y, (o.z - pad) * r.inv.z);
    return r;
}

// Slab test of one child box padded by the ray's pad; returns entry distance, or +inf.
__device__ __forceinline__ float box_entry(const RayInv& r, float lox, float hix, float loy, float hiy, float loz,
                                           float hiz, float tmax) {
    const float tx0 = fmaf(lox, r.inv.x, -r.oinv_lo.x), tx1 = fmaf(hix, r.inv.x, -r.oinv_hi.x);
    const float ty0 = fmaf(loy, r.inv.y, -r.oinv_lo.y), ty1 = fmaf(hiy, r.inv.y, -r.oinv_hi.y);
    const float tz0 = fmaf(loz, r.inv.z, -r.oinv_lo.z), tz1 = fmaf(hiz, r.inv.z, -r.oinv_hi.z);
    const float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float tfar = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    // no relative slack is needed: where the exact ray touches the unpadded box its padded
    // slabs overlap by 2 pad, far above the planes' rounding (robust.cuh)
    return tmin <= tfar ? tmin : __int_as_float(0x7f800000);
}

// Start of a closest-hit (t_max = inf) or any-hit (t_max of the segment) query.
__device__ __forceinline__ HitBest hit_begin(float tmax) {
    HitBest b;
    // t_max of a shadow segment is FP32 (its length times 1 - 1e-4, a few roundings)
    const float dt = tmax < __int_as_float(0x7f800000) ? 8.0f * k_ulp * tmax : 0.0f;
    b.lo = tmax - dt;
    b.hi = tmax + dt;
    b.prim = -1;
    b.undec = k_undec_none;
    return b;
}

// Tests the triangle at leaf position `pos` (tris: leaf order {v0, orig}, {e1, K1},
// {e2, K2}) and updates `b`. Returns true when the traversal ends: an any-hit query is
// answered, or (fast mode) a second undecided candidate was met.
// Fast mode: an undecided candidate is recorded in b.undec and the traversal goes on with
// the certain decisions (it culls only beyond the certain closest hit, so every triangle
// that could beat it is still tested); the fixup kernel re-decides the record.
// ROBUST: undecided candidates are re-decided inline from xr (the ray's exact geometry) and
// tri_in (original-order vertices).
template <bool ANY, bool ROBUST, class X>
__device__ __forceinline__ bool leaf_test(const float4* __restrict__ tris, const float4* __restrict__ tri_in,
                                          const X& xr, const RayInv& r, uint32_t pos, int exclude, HitBest& b) {
    const float4* p = tris + 3ull * pos;
    const float4 a = __ldg(p), e1 = __ldg(p + 1), e2 = __ldg(p + 2);
    const int orig = __float_as_int(a.w);
    // (a triangle met again through another of its leaf references, split boxes, gives the
    // same result as the first time: nothing to do if it is the closest hit already)
    if (orig == exclude || orig == b.prim) return false;
    float t, dt;
    const int c = tri_classify<ANY>(r.o, r.d, a, e1, e2, t, dt);
    if (c == k_tri_miss) return false;
    if (c == k_tri_hit) {
        if (t + dt < b.lo) {  // certainly closer than the closest so far (inside t_max)
            b.lo = t - dt;
            b.hi = t + dt;
            b.prim = orig;
            if (ANY) b.undec = k_undec_none;  // a certain occluder answers the query
            return ANY;
        }
        if (t - dt > b.hi) return false;  // certainly farther
    }
    if constexpr (ROBUST) {
        return redecide<ANY>(tri_in, xr, orig, b);
    } else {
        if (b.undec == orig) return false;  // recorded through another leaf reference
        if (b.undec == k_undec_none) {
            b.undec = orig;
            return false;
        }
        b.undec = k_undec_many;
        return true;
    }
}

// No exact geometry (fast mode never re-decides).
struct ExactNone {
    __device__ __forceinline__ void get(ff3&, ff3&) const {}
};

struct TraceCounters {
    uint32_t nodes = 0;
    uint32_t tris = 0;
};

// Result of one traversal: prim = original index of the closest certain hit or -1; undec =
// the undecided candidate the fixup kernel must re-decide (k_undec_none: the result is final;
// k_undec_many: re-trace the ray whole).
struct TraceResult {
    float t;
    int prim;
    int undec;
};
__device__ __forceinline__ TraceResult trace_result(const HitBest& b) { return TraceResult{hit_t(b), b.prim, b.undec}; }

// Per-ray traversal state of the resumable binary traversal (the stack lives beside it).
struct TraceState {
    RayInv r;
    int exclude;
    HitBest b;
    int node;
    int sp;
    uint32_t budget;
};

__device__ __forceinline__ void trace_begin(TraceState& s, float3 o, float3 d, float tmax, int exclude,
                                            uint32_t n_tris, float pad) {
    s.r = make_ray(o, d, pad);
    s.exclude = exclude;
    s.b = hit_begin(tmax);
    s.node = n_tris == 0 ? -1 : 0;
    s.sp = 0;
    s.budget = 2u * n_tris + 64u;
}

// One node visit (fast mode). Returns true when the traversal has finished.
template <bool ANY, bool STATS>
__device__ __forceinline__ bool trace_step(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                           TraceState& s, int* stack, uint32_t& err, TraceCounters& cnt) {
    if (s.node < 0) return true;
    if (--s.budget == 0u) {
        err |= k_deverr_traversal;
        return true;
    }
    if (STATS) ++cnt.nodes;
    const float4 n0 = __ldg(&nodes[4 * s.node + 0]);
    const float4 n1 = __ldg(&nodes[4 * s.node + 1]);
    const float4 n2 = __ldg(&nodes[4 * s.node + 2]);
    const float4 n3 = __ldg(&nodes[4 * s.node + 3]);
    const float tcull = s.b.hi;
    const float t0 = box_entry(s.r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, tcull);
    const float t1 = box_entry(s.r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, tcull);
    const int c0 = __float_as_int(n3.x);
    const int c1 = __float_as_int(n3.y);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int c = k == 0 ? c0 : c1;
        const float tb = k == 0 ? t0 : t1;
        if (c < 0 && tb < s.b.hi) {
            if (STATS) ++cnt.tris;
            if (leaf_test<ANY, false>(tris, nullptr, ExactNone{}, s.r, ~c, s.exclude, s.b)) {
                s.node = -1;
                return true;
            }
        }
    }
    const float tc = s.b.hi;
    const bool h0 = c0 >= 0 && t0 < tc;
    const bool h1 = c1 >= 0 && t1 < tc;
    if (h0 && h1) {
        const bool swap = t1 < t0;
        if (s.sp >= k_stack_size) {
            err |= k_deverr_stack;
            s.node = -1;
            return true;
        }
        stack[s.sp++] = swap ? c0 : c1;
        s.node = swap ? c1 : c0;
    } else if (h0) {
        s.node = c0;
    } else if (h1) {
        s.node = c1;
    } else {
        if (s.sp == 0) {
            s.node = -1;
            return true;
        }
        s.node = stack[--s.sp];
    }
    return false;
}

// Whole-ray traversal for kernels that trace one ray at a time.
// ANY = true: stops at the first hit with t in (0, tmax) and returns a prim >= 0.
// Returns the traversal's final state: the closest (certain) hit and, in fast mode, the
// undecided candidate it recorded. ROBUST: undecided candidates are re-decided exactly from
// xr (the exact ray) and tri_in, so the result is final.
// Treelet nodes (the top levels copied to shared memory) are addressed as k_tree_flag | i.
constexpr int k_tree_flag = 0x40000000;

// This monolithic loop keeps the whole traversal state in registers and is ~20% faster on
// GB300 than driving trace_step in a loop, so the batch-fetch kernels use it. With tree_n > 0
// the traversal starts in `tree` (shared memory), whose child links point into the treelet
// (k_tree_flag) or out to global nodes.
template <bool ANY, bool STATS, bool TREE = false, bool ROBUST = false, class X = ExactNone>
__device__ __forceinline__ HitBest trace_bvh(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                             const float4* __restrict__ tri_in, uint32_t n_tris, const RayInv& r,
                                             float tmax, int exclude, uint32_t& err, TraceCounters& cnt,
                                             const X& xr = X{}, const float4* tree = nullptr, int tree_n = 0) {
    HitBest b = hit_begin(tmax);
    if (n_tris == 0) return b;
    int stack[k_stack_size];
    int sp = 0;
    int node = (TREE && tree_n > 0) ? k_tree_flag : 0;
    uint32_t budget = 2u * n_tris + 64u;
    while (true) {
        if (--budget == 0u) {
            err |= k_deverr_traversal;
            break;
        }
        if (STATS) ++cnt.nodes;
        float4 n0, n1, n2, n3;
        if (TREE && (node & k_tree_flag)) {
            const float4* p = tree + 4 * (node & ~k_tree_flag);
            n0 = p[0];
            n1 = p[1];
            n2 = p[2];
            n3 = p[3];
        } else {
            n0 = __ldg(&nodes[4 * node + 0]);
            n1 = __ldg(&nodes[4 * node + 1]);
            n2 = __ldg(&nodes[4 * node + 2]);
            n3 = __ldg(&nodes[4 * node + 3]);
        }
        const float tcull = b.hi;
        float t0 = box_entry(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, tcull);
        float t1 = box_entry(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, tcull);
        int c0 = __float_as_int(n3.x);
        int c1 = __float_as_int(n3.y);
        bool ended = false;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int c = k == 0 ? c0 : c1;
            const float tb = k == 0 ? t0 : t1;
            if (!ended && c < 0 && tb < b.hi) {
                if (STATS) ++cnt.tris;
                ended = leaf_test<ANY, ROBUST>(tris, tri_in, xr, r, ~c, exclude, b);
            }
        }
        if (ended) break;
        const float tc = b.hi;
        const bool h0 = c0 >= 0 && t0 < tc;
        const bool h1 = c1 >= 0 && t1 < tc;
        if (h0 && h1) {
            int near_c = c0, far_c = c1;
            if (t1 < t0) {
                near_c = c1;
                far_c = c0;
            }
            if (sp >= k_stack_size) {
                err |= k_deverr_stack;
                break;
            }
            stack[sp++] = far_c;
            node = near_c;
        } else if (h0) {
            node = c0;
        } else if (h1) {
            node = c1;
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return b;
}

// Hands one finished ray to the job: a ray with an undecided candidate goes to the fixup
// list (with its certain result), others store their final result.
// The rays a trace kernel leaves to its fixup kernel, as (ray, recorded candidate) pairs: rays
// with one undecided candidate from the front of the list, rays to re-trace whole
// (k_undec_many) from the back, so the fixup kernel can spread the long re-traces one per
// warp.
struct DeferList {
    int2* list;
    int* count;       // entries at the front
    int* count_many;  // entries at the back
    int capacity;     // entries the list holds (one per ray of the launch)
    __device__ __forceinline__ void push(int i, int undec) const {
        if (undec == k_undec_many)
            list[capacity - 1 - atomicAdd(count_many, 1)] = make_int2(i, undec);
        else
            list[atomicAdd(count, 1)] = make_int2(i, undec);
    }
    // Entry of lane `lane` in chunk c of the fixup order (n_many re-traces, n_single single
    // re-decisions): while re-traces last, lane 0 of each chunk takes one and lanes 1..31 take
    // single entries; later chunks hold 32 single entries. Returns false past the end.
    __device__ __forceinline__ bool entry(int c, int lane, int n_many, int n_single, int2& e) const {
        int k;
        if (c < n_many) {
            if (lane == 0) {
                e = list[capacity - 1 - c];
                return true;
            }
            k = 31 * c + lane - 1;
        } else {
            k = 31 * n_many + 32 * (c - n_many) + lane;
        }
        if (k >= n_single) return false;
        e = list[k];
        return true;
    }
    // Chunks of the fixup order.
    __device__ __forceinline__ static int chunks(int n_many, int n_single) {
        const int rest = n_single - 31 * n_many;
        return n_many + (rest > 0 ? (rest + 31) / 32 : 0);
    }
};

template <class Job>
__device__ __forceinline__ void finish_ray(Job& job, int i, const TraceResult& res) {
    if (res.undec != k_undec_none)
        job.defer(i, res);
    else
        job.store(i, res);
}

// Warp-batch persistent traversal: a warp takes 32 consecutive rays with one atomic and
// traces them to completion before taking more (coherent node fetches within a batch).
// tree/tree_n: the treelet in shared memory (used when TREE). Job supplies
//   void load(int i, float3& o, float3& d, float& tmax, int& exclude)
//   void store(int i, const TraceResult& r)
//   void defer(int i, const TraceResult& r)   (r.undec needs an exact re-decision)
template <bool ANY, bool STATS, bool TREE, class Job>
__device__ __forceinline__ void trace_batches(Job& job, const float4* __restrict__ nodes,
                                              const float4* __restrict__ tris, uint32_t n_tris, int n,
                                              int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt,
                                              const float4* tree, int tree_n) {
    const int lane = threadIdx.x & 31;
    const float pad = n_tris ? scene_box_pad(nodes) : 0.0f;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i < n) {
            float3 o, d;
            float tmax;
            int exclude;
            job.load(i, o, d, tmax, exclude);
            const RayInv r = make_ray(o, d, pad);
            finish_ray(job, i,
                       trace_result(trace_bvh<ANY, STATS, TREE>(nodes, tris, nullptr, n_tris, r, tmax, exclude, err,
                                                                cnt, ExactNone{}, tree, tree_n)));
        }
    }
}

// Persistent traversal of a queue of n rays with per-lane refill: once `refill` lanes of a
// warp are idle they take the next rays with one atomic (refill = 32 takes 32 rays at a
// time and waits for all of them). Job as in trace_batches. Every lane of the warp must call
// this (it uses full-warp votes). Between refills each lane runs up to `steps` node visits
// without warp votes.
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_persistent(Job& job, const float4* __restrict__ nodes,
                                                 const float4* __restrict__ tris, uint32_t n_tris, int n, int refill,
                                                 int steps, int* __restrict__ fetch, uint32_t& err,
                                                 TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
    const float pad = n_tris ? scene_box_pad(nodes) : 0.0f;
    TraceState s;
    int stack[k_stack_size];
    bool active = false;
    bool exhausted = false;
    int idx = 0;
    while (true) {
        const uint32_t need = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(need) >= refill) {
            const int leader = __ffs(need) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + __popc(need) >= n;
            if (!active) {
                idx = base + __popc(need & lanemask_lt());
                if (idx < n) {
                    float3 o, d;
                    float tmax;
                    int exclude;
                    job.load(idx, o, d, tmax, exclude);
                    trace_begin(s, o, d, tmax, exclude, n_tris, pad);
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        for (int k = 0; k < steps && active; ++k) {
            if (trace_step<ANY, STATS>(nodes, tris, s, stack, err, cnt)) {
                finish_ray(job, idx, trace_result(s.b));
                active = false;
            }
        }
    }
}

// Completes the rays a trace kernel deferred. List entries are (ray i, its undecided
// candidate); each warp takes one chunk of 32 per atomic (DeferList::entry): a ray to
// re-trace whole in lane 0 while they last, single re-decisions in the other lanes. A
// re-trace makes its own exact re-decisions one lane at a time, so spreading re-traces one
// per warp keeps those from queueing behind each other. A candidate is re-decided against
// the ray's certain result (job.partial(i)); a ray that met more than one is re-traced whole
// with inline re-decisions by `retrace(i, o, d, tmax, exclude)` (over the 8-wide records or
// the binary LBVH). Job supplies load, store, partial(i) and exact(i); tri_in(i) gives the
// original triangles of ray i's scene.
template <bool ANY, class Job, class TriIn, class Retrace>
__device__ __forceinline__ void resolve_deferred(Job& job, const TriIn& tri_in, const DeferList& dl,
                                                 int* __restrict__ fetch, const Retrace& retrace) {
    const int lane = threadIdx.x & 31;
    const int n_many = *dl.count_many;
    const int n_single = *dl.count;
    const int n_chunks = DeferList::chunks(n_many, n_single);
    while (true) {
        int c = 0;
        if (lane == 0) c = atomicAdd(fetch, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= n_chunks) break;
        int2 e;
        if (dl.entry(c, lane, n_many, n_single, e)) {
            const int i = e.x;
            HitBest b;
            if (e.y == k_undec_many) {
                float3 o, d;
                float tmax;
                int exclude;
                job.load(i, o, d, tmax, exclude);
                b = retrace(i, o, d, tmax, exclude);
            } else {
                b = job.partial(i);
                redecide<ANY>(tri_in(i), job.exact(i), e.y, b);
            }
            b.undec = k_undec_none;
            job.store(i, trace_result(b));
        }
    }
}

}  // namespace quasi
