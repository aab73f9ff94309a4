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
//
// Traversal is written as a resumable step (one node visit) so persistent kernels can keep
// every lane of a warp busy: a lane whose ray finishes takes a new ray from the queue while
// the other lanes continue (trace_persistent).
#pragma once

#include "common.cuh"

namespace quasi {

constexpr int k_stack_size = 64;
// Box tests widen t_max by a few ulps so FP32 rounding never culls a box the ray touches.
constexpr float k_box_pad = 1.0000004f;
// Persistent kernels refill a warp once at least this many of its lanes are idle (default).
constexpr int k_refill_lanes = 32;
// Node visits per lane between two refill checks (default).
constexpr int k_trace_steps = 8;
// BVH levels staged in shared memory by default (2^5 - 1 = 31 nodes, 2 KB per block).
// Measured on GB300 (soup 1M, 1080p): 5 levels is neutral, 7 slightly slower, 9 (32 KB per
// block) 22% slower; the top levels are L1-resident either way.
constexpr int k_default_smem_levels = 5;

struct RayInv {
    float3 o;
    float3 d;
    float3 inv;  // 1/d with tiny components clamped away from zero
    float3 oinv; // o * inv
};

__device__ __forceinline__ float safe_inv(float x) {
    const float ax = fabsf(x) > 1e-20f ? x : copysignf(1e-20f, x);
    return 1.0f / ax;
}

__device__ __forceinline__ RayInv make_ray(float3 o, float3 d) {
    RayInv r;
    r.o = o;
    r.d = d;
    r.inv = mk3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    r.oinv = mk3(o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z);
    return r;
}

// Slab test of one child box; returns entry distance, or +inf on a miss.
__device__ __forceinline__ float box_entry(const RayInv& r, float lox, float hix, float loy, float hiy, float loz,
                                           float hiz, float tmax) {
    const float tx0 = fmaf(lox, r.inv.x, -r.oinv.x), tx1 = fmaf(hix, r.inv.x, -r.oinv.x);
    const float ty0 = fmaf(loy, r.inv.y, -r.oinv.y), ty1 = fmaf(hiy, r.inv.y, -r.oinv.y);
    const float tz0 = fmaf(loz, r.inv.z, -r.oinv.z), tz1 = fmaf(hiz, r.inv.z, -r.oinv.z);
    const float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float tfar = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    return tmin <= tfar * k_box_pad ? tmin : __int_as_float(0x7f800000);
}

// Moller & Trumbore (1997) with precomputed edges. Returns t or +inf, and the barycentrics
// (u, v) of the hit, from which the hit point is rebuilt as v0 + u e1 + v e2 (on the
// triangle's plane to within vertex rounding, unlike o + t d).
__device__ __forceinline__ float tri_t(const RayInv& r, float4 a, float4 e1, float4 e2, float& u, float& v) {
    const float3 E1 = xyz(e1), E2 = xyz(e2);
    const float3 p = cross(r.d, E2);
    const float det = dot(E1, p);
    const float inv = 1.0f / det;  // det == 0 gives inf/nan and fails the tests below
    const float3 tv = r.o - xyz(a);
    u = dot(tv, p) * inv;
    const float3 q = cross(tv, E1);
    v = dot(r.d, q) * inv;
    const float t = dot(E2, q) * inv;
    const bool ok = (u >= 0.0f) && (v >= 0.0f) && (u + v <= 1.0f) && (t > 0.0f) && (det != 0.0f);
    return ok ? t : __int_as_float(0x7f800000);
}

struct TraceCounters {
    uint32_t nodes = 0;
    uint32_t tris = 0;
};

// Per-ray traversal state; the stack lives beside it (thread-local array).
struct TraceState {
    RayInv r;
    float tmax;
    int exclude;
    float best_t;
    int best;  // original index of the closest hit so far, or -1
    float bu, bv;
    int node;
    int sp;
    uint32_t budget;
};

__device__ __forceinline__ void trace_begin(TraceState& s, float3 o, float3 d, float tmax, int exclude,
                                            uint32_t n_tris) {
    s.r = make_ray(o, d);
    s.tmax = tmax;
    s.exclude = exclude;
    s.best_t = tmax;
    s.best = -1;
    s.bu = s.bv = 0.0f;
    s.node = n_tris == 0 ? -1 : 0;
    s.sp = 0;
    s.budget = 2u * n_tris + 64u;
}

// One node visit. Returns true when the traversal has finished (state holds the result).
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
    const float t0 = box_entry(s.r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, s.best_t);
    const float t1 = box_entry(s.r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, s.best_t);
    const int c0 = __float_as_int(n3.x);
    const int c1 = __float_as_int(n3.y);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int c = k == 0 ? c0 : c1;
        const float tb = k == 0 ? t0 : t1;
        if (c < 0 && tb < s.best_t) {
            const int pos = ~c;
            if (STATS) ++cnt.tris;
            const float4 a = __ldg(&tris[3 * pos]);
            const float4 e1 = __ldg(&tris[3 * pos + 1]);
            const float4 e2 = __ldg(&tris[3 * pos + 2]);
            const int orig = __float_as_int(a.w);
            float u, v;
            const float t = tri_t(s.r, a, e1, e2, u, v);
            if (orig != s.exclude && (t < s.best_t || (t == s.best_t && orig < s.best && t < s.tmax))) {
                s.best_t = t;
                s.best = orig;
                s.bu = u;
                s.bv = v;
                if (ANY) {
                    s.node = -1;
                    return true;
                }
            }
        }
    }
    const bool h0 = c0 >= 0 && t0 < s.best_t;
    const bool h1 = c1 >= 0 && t1 < s.best_t;
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
// Returns the original index of the hit triangle (or -1), its distance in t_out and its
// barycentrics in bu, bv.
// Treelet nodes (the top levels copied to shared memory) are addressed as k_tree_flag | i.
constexpr int k_tree_flag = 0x40000000;

// This monolithic loop keeps the whole traversal state in registers and is ~20% faster on
// GB300 than driving trace_step in a loop, so the batch-fetch kernels use it. With tree_n > 0
// the traversal starts in `tree` (shared memory), whose child links point into the treelet
// (k_tree_flag) or out to global nodes.
template <bool ANY, bool STATS, bool TREE = false>
__device__ __forceinline__ int trace_bvh(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                         uint32_t n_tris, const RayInv& r, float tmax, int exclude, float& t_out,
                                         float& bu, float& bv, uint32_t& err, TraceCounters& cnt,
                                         const float4* tree = nullptr, int tree_n = 0) {
    float best_t = tmax;
    int best = -1;
    bu = bv = 0.0f;
    if (n_tris == 0) {
        t_out = best_t;
        return -1;
    }
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
        float t0 = box_entry(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best_t);
        float t1 = box_entry(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best_t);
        int c0 = __float_as_int(n3.x);
        int c1 = __float_as_int(n3.y);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int c = k == 0 ? c0 : c1;
            const float tb = k == 0 ? t0 : t1;
            if (c < 0 && tb < best_t) {
                const int pos = ~c;
                if (STATS) ++cnt.tris;
                const float4 a = __ldg(&tris[3 * pos]);
                const float4 e1 = __ldg(&tris[3 * pos + 1]);
                const float4 e2 = __ldg(&tris[3 * pos + 2]);
                const int orig = __float_as_int(a.w);
                float u, v;
                const float t = tri_t(r, a, e1, e2, u, v);
                if (orig != exclude && (t < best_t || (t == best_t && orig < best && t < tmax))) {
                    best_t = t;
                    best = orig;
                    bu = u;
                    bv = v;
                    if (ANY) {
                        t_out = best_t;
                        return best;
                    }
                }
            }
        }
        const bool h0 = c0 >= 0 && t0 < best_t;
        const bool h1 = c1 >= 0 && t1 < best_t;
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
    t_out = best_t;
    return best;
}

// Warp-batch persistent traversal: a warp takes 32 consecutive rays with one atomic and
// traces them to completion before taking more (coherent node fetches within a batch).
// tree/tree_n: the treelet in shared memory (used when TREE).
template <bool ANY, bool STATS, bool TREE, class Job>
__device__ __forceinline__ void trace_batches(Job& job, const float4* __restrict__ nodes,
                                              const float4* __restrict__ tris, uint32_t n_tris, int n,
                                              int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt,
                                              const float4* tree, int tree_n) {
    const int lane = threadIdx.x & 31;
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
            TraceState s;
            s.r = make_ray(o, d);
            s.tmax = tmax;
            s.best = trace_bvh<ANY, STATS, TREE>(nodes, tris, n_tris, s.r, tmax, exclude, s.best_t, s.bu, s.bv, err,
                                                 cnt, tree, tree_n);
            job.store(i, s);
        }
    }
}

// Persistent traversal of a queue of n rays with per-lane refill: once `refill` lanes of a
// warp are idle they take the next rays with one atomic (refill = 32 takes 32 rays at a
// time and waits for all of them). Job supplies
//   void load(int i, float3& o, float3& d, float& tmax, int& exclude)
//   void store(int i, const TraceState& s)
// Every lane of the warp must call this (it uses full-warp votes).
// Between refills each lane runs up to `steps` node visits without warp votes.
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_persistent(Job& job, const float4* __restrict__ nodes,
                                                 const float4* __restrict__ tris, uint32_t n_tris, int n, int refill,
                                                 int steps, int* __restrict__ fetch, uint32_t& err,
                                                 TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
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
                    trace_begin(s, o, d, tmax, exclude, n_tris);
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        for (int k = 0; k < steps && active; ++k) {
            if (trace_step<ANY, STATS>(nodes, tris, s, stack, err, cnt)) {
                job.store(idx, s);
                active = false;
            }
        }
    }
}

}  // namespace quasi
