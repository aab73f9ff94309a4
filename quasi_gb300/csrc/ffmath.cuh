// ffmath.cuh - double-float arithmetic for the path geometry.
//
// A value is the unevaluated sum hi + lo of two floats (about 48 significant bits), built
// from error-free transformations that run at FP32 rate: Knuth's TwoSum, Dekker's
// FastTwoSum, TwoProd through a fused multiply-add, and Dekker's (1971) double-length
// add / multiply / divide / square root as organised in the QD library (Hida, Li and
// Bailey, 2001). sin and cos come from their Taylor series after reduction to |x| <= pi/4.
//
// Why: FP32 coordinates near 1.0 carry 6e-8 of absolute rounding. A path that bounces in a
// corner (segments of 1e-4) turns that into 1e-3 of relative error in its radiance, far
// above the 1e-4 bound against the FP64 oracle, while GB300's FP64 rate is a small fraction
// of its FP32 rate. Traversal stays in FP32; only positions, directions and the shading
// geometry of each path vertex use these types. Every operation uses the _rn intrinsics so
// the compiler can neither contract nor reassociate them.
#pragma once

#include <cuda_runtime.h>

namespace quasi {

struct ff {
    float hi, lo;
};
struct ff3 {
    ff x, y, z;
};

__device__ __forceinline__ ff ffv(float a) { return ff{a, 0.0f}; }

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

// Requires |a| >= |b| (or a == 0).
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return ff{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.hi, b.hi);
    const ff t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_mul(ff a, float b) {
    ff p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    ff r = ff_sub(a, ff_mul(b, q1));
    const float q2 = __fdiv_rn(r.hi, b.hi);
    r = ff_sub(r, ff_mul(b, q2));
    const float q3 = __fdiv_rn(r.hi, b.hi);
    return ff_add(fast_two_sum(q1, q2), ffv(q3));
}

__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return ff{0.0f, 0.0f};
    const float s = __fsqrt_rn(a.hi);
    const ff r = ff_sub(a, two_prod(s, s));
    return fast_two_sum(s, __fdiv_rn(r.hi, __fmul_rn(2.0f, s)));
}

__device__ __forceinline__ float ff_f(ff a) { return __fadd_rn(a.hi, a.lo); }

// sin(pi x) and cos(pi x) for a float x: x = k/2 + y with |y| <= 1/4 exactly, then Taylor
// series of sin and cos at pi*y to degree 15 and 14: the first omitted terms are below
// 5e-17 and 1.1e-15 for |pi y| <= pi/4, under the ~1e-14 of double-float arithmetic.
__device__ __forceinline__ void ff_sincospi(float x, ff& s, ff& c) {
    const float k = rintf(__fmul_rn(2.0f, x));
    const float y = __fsub_rn(x, __fmul_rn(0.5f, k));
    const int q = static_cast<int>(k) & 3;
    const ff t = ff_mul(ff{3.14159274101257324f, -8.742277657347586e-08f}, y);
    const ff t2 = ff_mul(t, t);
    // (-1)^k / (2k+1)! and (-1)^k / (2k)!, as hi + lo float pairs, highest order first.
    const float sin_c[8][2] = {{-7.647163609812713e-13f, -1.2200710471178288e-20f},
                               {1.6059044372074283e-10f, -5.352526511562726e-18f},
                               {-2.5052107943679403e-08f, -4.4176230446483665e-16f},
                               {2.7557318844628753e-06f, 3.793571224297229e-14f},
                               {-0.00019841270113829523f, 2.725596874933456e-12f},
                               {0.008333333767950535f, -4.34617203337595e-10f},
                               {-0.1666666716337204f, 4.967053879312289e-09f},
                               {1.0f, 0.0f}};
    const float cos_c[8][2] = {{-1.147074536050896e-11f, -2.372207689231238e-19f},
                               {2.0876755879584152e-09f, 1.1082839809204342e-16f},
                               {-2.755731998149713e-07f, 7.575112209051195e-15f},
                               {2.4801587642286904e-05f, -3.40699609366682e-13f},
                               {-0.0013888889225199819f, 3.3631094437103215e-11f},
                               {0.0416666679084301f, -1.2417634698280722e-09f},
                               {-0.5f, 0.0f},
                               {1.0f, 0.0f}};
    ff ps = ff{sin_c[0][0], sin_c[0][1]};
    ff pc = ff{cos_c[0][0], cos_c[0][1]};
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        ps = ff_add(ff_mul(ps, t2), ff{sin_c[i][0], sin_c[i][1]});
        pc = ff_add(ff_mul(pc, t2), ff{cos_c[i][0], cos_c[i][1]});
    }
    const ff sv = ff_mul(ps, t);
    const ff cv = pc;
    switch (q) {
        case 0: s = sv; c = cv; break;
        case 1: s = cv; c = ff_neg(sv); break;
        case 2: s = ff_neg(sv); c = ff_neg(cv); break;
        default: s = ff_neg(cv); c = sv; break;
    }
}

// ------------------------------------------------------------------------ 3-vectors

__device__ __forceinline__ ff3 ff3v(float3 a) { return ff3{ffv(a.x), ffv(a.y), ffv(a.z)}; }
__device__ __forceinline__ float3 ff3_f(const ff3& a) { return make_float3(a.x.hi, a.y.hi, a.z.hi); }
// Exact difference of two float vectors.
__device__ __forceinline__ ff3 ff3_diff(float3 a, float3 b) {
    return ff3{two_sum(a.x, -b.x), two_sum(a.y, -b.y), two_sum(a.z, -b.z)};
}
__device__ __forceinline__ ff3 ff3_add(const ff3& a, const ff3& b) {
    return ff3{ff_add(a.x, b.x), ff_add(a.y, b.y), ff_add(a.z, b.z)};
}
__device__ __forceinline__ ff3 ff3_sub(const ff3& a, const ff3& b) {
    return ff3{ff_sub(a.x, b.x), ff_sub(a.y, b.y), ff_sub(a.z, b.z)};
}
__device__ __forceinline__ ff3 ff3_scale(const ff3& a, ff s) { return ff3{ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)}; }
__device__ __forceinline__ ff3 ff3_scale(const ff3& a, float s) {
    return ff3{ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)};
}
__device__ __forceinline__ ff3 ff3_neg(const ff3& a) { return ff3{ff_neg(a.x), ff_neg(a.y), ff_neg(a.z)}; }
__device__ __forceinline__ ff ff3_dot(const ff3& a, const ff3& b) {
    return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
__device__ __forceinline__ ff3 ff3_cross(const ff3& a, const ff3& b) {
    return ff3{ff_sub(ff_mul(a.y, b.z), ff_mul(a.z, b.y)), ff_sub(ff_mul(a.z, b.x), ff_mul(a.x, b.z)),
               ff_sub(ff_mul(a.x, b.y), ff_mul(a.y, b.x))};
}
__device__ __forceinline__ ff ff3_length(const ff3& a) { return ff_sqrt(ff3_dot(a, a)); }
// One double-float division (the reciprocal of the length) and three products: a third of
// the cost of three divisions, and the same ~1e-14 relative accuracy.
__device__ __forceinline__ ff3 ff3_normalize(const ff3& a) {
    return ff3_scale(a, ff_div(ffv(1.0f), ff3_length(a)));
}

// Packed storage of a double-float ray (origin, direction) in 3 float4.
__device__ __forceinline__ void ff_ray_store(float4* p, const ff3& o, const ff3& d) {
    p[0] = make_float4(o.x.hi, o.y.hi, o.z.hi, o.x.lo);
    p[1] = make_float4(o.y.lo, o.z.lo, d.x.hi, d.y.hi);
    p[2] = make_float4(d.z.hi, d.x.lo, d.y.lo, d.z.lo);
}
__device__ __forceinline__ void ff_ray_load(const float4* p, ff3& o, ff3& d) {
    const float4 a = p[0], b = p[1], c = p[2];
    o = ff3{ff{a.x, a.w}, ff{a.y, b.x}, ff{a.z, b.y}};
    d = ff3{ff{b.z, c.y}, ff{b.w, c.z}, ff{c.x, c.w}};
}

}  // namespace quasi
