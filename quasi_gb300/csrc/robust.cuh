// robust.cuh - hit decisions that agree with exact (FP64) arithmetic.
//
// Traversal tests triangles in FP32 (Moller & Trumbore 1997). A ray that passes within a
// few FP32 rounding errors of a triangle edge, or meets two triangles at almost the same
// distance, can get a different answer in FP32 than in FP64. Every FP32 test here therefore
// also computes a rigorous bound on its own rounding error and classifies the candidate:
//
//   certain miss   some barycentric coordinate is below -M (M = the error bound)
//   certain hit    every barycentric coordinate is above M and t > dt (t's error bound)
//   undecided      otherwise, or a certain hit whose t lies within dt + dt_best of the
//                  current closest hit (a near tie), or of t_max for a shadow segment
//
// Undecided candidates are re-decided in double-float arithmetic (ffmath.cuh, ~48 bits)
// from the exact path geometry: the double-float ray or shadow segment the path carries and
// the triangle's original vertices (their differences are exact in double-float). The
// re-decision agrees with FP64 except where the exact answer lies within ~1e-14 of a
// boundary. Exact re-decisions are rare (~1% of rays meet one undecided candidate); the
// wavefront trace kernels do not make them inline (one lane would hold up its warp for ~1000
// instructions) but record the undecided candidate and finish the traversal on the certain
// decisions, culling only beyond the certain closest hit; a fixup kernel then re-decides the
// recorded candidates with all lanes in step. A ray that meets a second undecided candidate
// is re-traced whole with inline re-decisions.
//
// Error bound of the FP32 test (u = 2^-24; first order, each operation rounding once, FMA
// contraction only removes roundings). Inputs: the FP32 ray (o, d) rounds the exact ray per
// component by u (origin) and by u (closest-hit rays) or up to 6u (the shadow ray's
// normalised direction); the stored edges E1, E2 round v1 - v0, v2 - v0 by u. With
// A = |E1|_1, B = |E2|_1, |d|_1 <= 1.74, T = |o - v0|_inf and sigma = |o|_inf + 13 T
// (shadow rays) or |o|_inf + 8 T (closest-hit rays: the direction's error is 1u, not 6u):
//   |dUd| <= 1.74 u B sigma,  |dVd| <= 2 u A sigma,  |dDet| <= 22.7 u A B,
//   |dTd| <= 2 u A B sigma
// where Ud = (o - v0).p, Vd = d.q, Td = E2.q, det = E1.p, p = d x E2, q = (o - v0) x E1.
// 1/det is the hardware reciprocal approximation (relative error <= 2^-23 = 2u), so u, v and
// t carry 3u of relative rounding from their normalisation. For |u|, |v| <= 4 the computed
// u = Ud/det, v = Vd/det and w = 1 - u - v are each within
//   M = u (sigma (1.74 B + 2 A) + 363.2 A B) / |det| + 48 u
// of their exact values (48 u >= 5 u (|u| + |v|) + 2 u), and t = Td/det within
//   dt = u A B (2 sigma + 45.4 |t|) / |det| + 4 u |t|.
// A coordinate with |u| or |v| > 4 is a certain miss whenever M < 1 (the relative error of
// det is then below 1/16). The per-triangle factors K1 = 1.01 u (1.74 B + 2 A) and
// K2 = 1.01 * 363.2 u A B are stored with the leaf triangles (e1.w, e2.w).
#pragma once

#include "common.cuh"
#include "ffmath.cuh"

namespace quasi {

constexpr float k_ulp = 0x1p-24f;
// Per-triangle error factors (written with the leaf triangles by the LBVH build).
__host__ __device__ __forceinline__ float robust_k1(float a, float b) { return 1.01f * k_ulp * (1.74f * b + 2.0f * a); }
__host__ __device__ __forceinline__ float robust_k2(float a, float b) { return 1.01f * 363.2f * k_ulp * a * b; }
// dt = K2 (sigma / 181.6 + |t| / 8) / |det| + 4 u |t| (from u A B = K2 / (1.01 * 363.2)).
constexpr float k_dt_sigma = 1.0f / 181.6f;
constexpr float k_dt_t = 0.125f;

// Spatial padding of every box the traversal tests, as a multiple of the scene's largest
// absolute coordinate S: 2^-16 S is far above the FP32 error of a slab-plane distance
// (~16 u S for ray origins within ~50 S of the scene), so a box whose exact extent the exact
// ray touches is never culled by rounding. The LBVH build stores S and the pad on the device.
constexpr float k_box_pad_rel = 0x1p-16f;

// The smallest t of a shadow segment that counts as its far end: the segment runs from the
// light sample towards the lifted shading point and stops at 1 - 1e-4 of its length (as a
// double, 1e-4 is not a float: hi + lo below).
constexpr float k_seg_end_hi = 0.99989998340606689453125f;  // float nearest 1 - 1e-4
constexpr float k_seg_end_lo = 1.6593933338526767e-08f;     // (1 - 1e-4) - hi, rounded

// Reciprocal by the hardware approximation (rcp.approx.ftz.f32: relative error <= 2^-23;
// subnormal inputs flush to zero and give inf, which the error bound turns into undecided).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Largest absolute component.
__device__ __forceinline__ float max_abs3(float3 v) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(fabsf(v.x)), "f"(fabsf(v.y)), "f"(fabsf(v.z)));
    return r;
}

// Outcome of one FP32 triangle test.
enum : int { k_tri_miss = 0, k_tri_hit = 1, k_tri_undecided = 2 };

// FP32 Moller-Trumbore with its error bound. a = (v0, orig), e1 = (E1, K1), e2 = (E2, K2).
// ANY: a shadow segment (its direction carries more rounding). Returns the class; t and dt
// (t's error bound) are set on every path.
template <bool ANY>
__device__ __forceinline__ int tri_classify(float3 o, float3 d, float4 a, float4 e1, float4 e2, float& t,
                                            float& dt) {
    const float3 E1 = xyz(e1), E2 = xyz(e2);
    const float3 p = cross(d, E2);
    const float det = dot(E1, p);
    const float inv = rcp_approx(det);  // det == 0 gives inf/nan: the bound is then inf/nan, undecided
    const float3 tv = o - xyz(a);
    const float u = dot(tv, p) * inv;
    const float3 q = cross(tv, E1);
    const float v = dot(d, q) * inv;
    t = dot(E2, q) * inv;
    const float w = 1.0f - u - v;
    const float ainv = fabsf(inv);
    const float sigma = fmaf(ANY ? 13.0f : 8.0f, max_abs3(tv), max_abs3(o));
    const float m = fmaf(fmaf(e1.w, sigma, e2.w), ainv, 48.0f * k_ulp);
    const float at = fabsf(t);
    dt = fmaf(e2.w * ainv, fmaf(at, k_dt_t, sigma * k_dt_sigma), 4.0f * k_ulp * at);
    const float mn = fminf(u, fminf(v, w));
    if (mn > m && t > dt) return k_tri_hit;
    if ((mn < -m && m < 1.0f) || (mn > m && t < -dt)) return k_tri_miss;
    return k_tri_undecided;
}

// Double-float Moller-Trumbore of the exact ray o + t d against the triangle with float
// vertices v0, v1, v2 (its edges are exact in double-float). SEG: the ray is a shadow
// segment (d = end - start) that counts only for t < 1 - 1e-4. Returns true on a hit with
// t > 0 (and, SEG, t < 1 - 1e-4); t is then set. The signs decide, as the FP64 oracle's
// u < 0, u + v > 1, ... tests do.
template <bool SEG>
__device__ __noinline__ bool exact_tri(ff3 o, ff3 d, float3 v0, float3 v1, float3 v2, ff& t) {
    const ff3 E1 = ff3_diff(v1, v0), E2 = ff3_diff(v2, v0);
    const ff3 p = ff3_cross(d, E2);
    const ff det = ff3_dot(E1, p);
    if (det.hi == 0.0f) return false;
    const ff3 tv = ff3_sub(o, ff3v(v0));
    const ff ud = ff3_dot(tv, p);
    const ff3 q = ff3_cross(tv, E1);
    const ff vd = ff3_dot(d, q);
    const ff td = ff3_dot(E2, q);
    const ff wd = ff_sub(ff_sub(det, ud), vd);
    if (det.hi < 0.0f) {
        if (ud.hi > 0.0f || vd.hi > 0.0f || wd.hi > 0.0f || !(td.hi < 0.0f)) return false;
    } else {
        if (ud.hi < 0.0f || vd.hi < 0.0f || wd.hi < 0.0f || !(td.hi > 0.0f)) return false;
    }
    t = ff_div(td, det);
    if (SEG) {
        const ff end{k_seg_end_hi, k_seg_end_lo};
        const ff diff = ff_sub(t, end);
        if (!(diff.hi < 0.0f)) return false;
    }
    return true;
}

// ff comparison (both normalised): a < b.
__device__ __forceinline__ bool ff_less(ff a, ff b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// The exact geometry of the ray being traced, for re-decisions: a double-float origin and
// direction (closest-hit rays) or start and end - start (shadow segments) packed as
// ff_ray_store does, read through a pointer.
struct ExactPtr {
    const float4* p;
    __device__ __forceinline__ void get(ff3& o, ff3& d) const { ff_ray_load(p, o, d); }
};
// The same held in registers (one-thread-per-path kernels).
struct ExactRegs {
    ff3 o, d;
    __device__ __forceinline__ void get(ff3& oo, ff3& dd) const {
        oo = o;
        dd = d;
    }
};

// The undecided candidate a fast traversal recorded: none, or more than one (the ray is
// then re-traced whole with inline re-decisions).
constexpr int k_undec_none = -1;
constexpr int k_undec_many = -2;

// Closest-hit state of one ray (or the any-hit state of a shadow segment).
struct HitBest {
    float lo, hi;  // the exact t of the closest certain hit so far lies in [lo, hi] (t_max's
                   // interval before any); box tests cull beyond hi
    int prim;      // original index, or -1
    int undec;     // fast traversal: the undecided candidate met (orig), k_undec_none or _many
};
// The closest hit's t (the middle of its interval).
__device__ __forceinline__ float hit_t(const HitBest& b) { return 0.5f * (b.lo + b.hi); }

// Re-decides candidate `orig` (vertices from the original-order triangle array) exactly and
// updates `b`. Returns true when an any-hit query is answered (the segment is blocked).
// When the candidate wins, its t comes from the exact computation; when the incumbent stays,
// its stored t is kept, so the result does not depend on the order in which candidates are
// met.
template <bool ANY, class X>
__device__ __noinline__ bool redecide(const float4* __restrict__ tri_in, const X& xr, int orig, HitBest& b) {
    ff3 o, d;
    xr.get(o, d);
    const float3 a = xyz(__ldg(&tri_in[3 * orig])), bb = xyz(__ldg(&tri_in[3 * orig + 1])),
                 c = xyz(__ldg(&tri_in[3 * orig + 2]));
    ff t;
    if (!exact_tri<ANY>(o, d, a, bb, c, t)) return false;
    if (ANY) {
        b.prim = orig;
        return true;
    }
    if (b.prim >= 0) {
        const float3 a2 = xyz(__ldg(&tri_in[3 * b.prim])), b2 = xyz(__ldg(&tri_in[3 * b.prim + 1])),
                     c2 = xyz(__ldg(&tri_in[3 * b.prim + 2]));
        ff tb;
        // The incumbent was decided as a hit; an exact miss here can only be a boundary case
        // within ~1e-14, where either answer is as good as FP64's.
        if (exact_tri<false>(o, d, a2, b2, c2, tb)) {
            if (ff_less(tb, t) || (tb.hi == t.hi && tb.lo == t.lo && b.prim < orig)) return false;
        }
    }
    const float tf = ff_f(t);
    const float dtf = 2.0f * k_ulp * fabsf(tf);
    b.lo = tf - dtf;
    b.hi = tf + dtf;
    b.prim = orig;
    return false;
}

}  // namespace quasi
