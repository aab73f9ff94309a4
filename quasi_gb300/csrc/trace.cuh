// trace.cuh - stack-based LBVH traversal with Moller-Trumbore triangle tests (FP32).
//
// Rays never store more than one stack entry per tree level (nearest child first, the far
// child is pushed), so the stack bound is the tree depth; a ray that would overflow the
// k_stack_size entries stops, reports a miss and raises QUASI_DEVERR_STACK.
//
// Closest hit is defined independently of traversal order: the smallest t wins and an
// exact tie goes to the smaller original triangle index. The oracle uses the same rule.
#pragma once

#include "common.cuh"

namespace quasi {

constexpr int k_stack_size = 64;
// Box tests widen t_max by a few ulps so FP32 rounding never culls a box the ray touches.
constexpr float k_box_pad = 1.0000004f;

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

// ANY = true: stops at the first hit with t in (0, tmax) and returns a prim >= 0.
// Returns the original index of the hit triangle (or -1), its distance in t_out and its
// barycentrics in bu, bv. err receives k_deverr_stack on stack overflow.
template <bool ANY, bool STATS>
__device__ __forceinline__ int trace_bvh(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                         uint32_t n_tris, const RayInv& r, float tmax, int exclude, float& t_out,
                                         float& bu, float& bv, uint32_t& err, TraceCounters& cnt) {
    float best_t = tmax;
    int best = -1;
    bu = bv = 0.0f;
    if (n_tris == 0) {
        t_out = best_t;
        return -1;
    }
    int stack[k_stack_size];
    int sp = 0;
    int node = 0;
    // A tree of n leaves has at most n internal nodes to visit; anything beyond that means a
    // malformed hierarchy, so the ray stops instead of looping.
    uint32_t budget = 2u * n_tris + 64u;
    while (true) {
        if (--budget == 0u) {
            err |= k_deverr_traversal;
            break;
        }
        if (STATS) ++cnt.nodes;
        const float4 n0 = __ldg(&nodes[4 * node + 0]);
        const float4 n1 = __ldg(&nodes[4 * node + 1]);
        const float4 n2 = __ldg(&nodes[4 * node + 2]);
        const float4 n3 = __ldg(&nodes[4 * node + 3]);
        float t0 = box_entry(r, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best_t);
        float t1 = box_entry(r, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best_t);
        int c0 = __float_as_int(n3.x);
        int c1 = __float_as_int(n3.y);
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int c = s == 0 ? c0 : c1;
            const float tb = s == 0 ? t0 : t1;
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
            if (t1 < t0) { near_c = c1; far_c = c0; }
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

}  // namespace quasi
