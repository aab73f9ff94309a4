// ffmath.cuh - double-float arithmetic for the path geometry.
//
// A value is the unevaluated sum hi + lo of two floats (about 48 significant bits), built
// from error-free transformations that run at FP32 rate: Knuth's TwoSum, Dekker's
// FastTwoSum, TwoProd through a fused multiply-add, and Dekker's (1971) double-length
// add / multiply / divide / square root as organised in the QD library (Hida, Li and
// Bailey, 2001). sin and cos come from a table of 33 angles and short Taylor series.
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

// a + b with an error below ~2^-47 (|a| + |b|) rather than 2^-47 |a + b| (the QD library's
// "sloppy" addition: one TwoSum instead of two, 11 operations instead of 20). For operands
// that already carry rounding of that size (products, rounded positions) the two agree; the
// exact re-decisions of hit tests keep the accurate form.
__device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
    const ff s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_sub_fast(ff a, ff b) { return ff_add_fast(a, ff_neg(b)); }

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

// a + b for a float b (one TwoSum fewer than ff_add; the same ~2^-48 relative accuracy).
__device__ __forceinline__ ff ff_add(ff a, float b) {
    ff s = two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return fast_two_sum(s.hi, s.lo);
}

// Three quotient digits, each the running remainder times one float reciprocal of b.hi; the
// exact remainders absorb the reciprocal's rounding, so the result keeps ~2^-47 relative
// accuracy with one reciprocal instead of three divisions.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    const float rb = __frcp_rn(b.hi);
    const float q1 = __fmul_rn(a.hi, rb);
    ff r = ff_sub(a, ff_mul(b, q1));
    const float q2 = __fmul_rn(r.hi, rb);
    r = ff_sub(r, ff_mul(b, q2));
    const float q3 = __fmul_rn(r.hi, rb);
    return ff_add(fast_two_sum(q1, q2), q3);
}

__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return ff{0.0f, 0.0f};
    const float s = __fsqrt_rn(a.hi);
    const ff r = ff_sub(a, two_prod(s, s));
    return fast_two_sum(s, __fmul_rn(r.hi, __frcp_rn(__fmul_rn(2.0f, s))));
}

__device__ __forceinline__ float ff_f(ff a) { return __fadd_rn(a.hi, a.lo); }

// sin(pi j / 128) and cos(pi j / 128) for j = 0..32 as double-float pairs
// (sin.hi, sin.lo, cos.hi, cos.lo): the exact values rounded to ~48 bits, computed from their
// Taylor series in 60-digit decimal arithmetic (tests/test_ffmath.py recomputes them).
namespace {
__device__ const float k_sincospi_tab[33][4] = {
    {0.0f, 0.0f, 1.0f, 0.0f},
    {0.024541229009628296f, -4.867160008359406e-10f, 0.99969881772995f, 9.66254298795377e-10f},
    {0.049067676067352295f, -1.7399343077428853e-09f, 0.9987954497337341f, 6.471438052102485e-09f},
    {0.0735645666718483f, -3.0721809540779077e-09f, 0.9972904324531555f, 2.4225535355526517e-08f},
    {0.0980171412229538f, -8.933931927579408e-10f, 0.9951847195625305f, 7.109666189109021e-09f},
    {0.12241067737340927f, -2.1741930478214044e-09f, 0.9924795627593994f, -2.8160689780065695e-08f},
    {0.1467304676771164f, 6.778245520422388e-09f, 0.9891765117645264f, -1.7997453527485163e-09f},
    {0.1709618866443634f, 2.115937869362483e-09f, 0.9852776527404785f, -1.0351537405028921e-08f},
    {0.19509032368659973f, -1.670471427850373e-09f, 0.9807852506637573f, 2.9739473106360492e-08f},
    {0.21910123527050018f, 4.88636953122068e-09f, 0.9757021069526672f, 2.3085862110860944e-08f},
    {0.24298018217086792f, -2.267604104488896e-09f, 0.9700312614440918f, -8.249547711614014e-09f},
    {0.2667127549648285f, 2.5100699296842777e-09f, 0.9637760519981384f, 1.3797301079421231e-08f},
    {0.290284663438797f, 1.3815665056426951e-08f, 0.9569403529167175f, -1.7184508038781132e-08f},
    {0.3136817514896393f, -1.1090747875641682e-08f, 0.949528157711029f, 2.288200739997137e-08f},
    {0.3368898630142212f, -9.622000973763534e-09f, 0.9415440559387207f, 9.244300436250796e-09f},
    {0.3598950505256653f, -1.3990677061315182e-08f, 0.9329928159713745f, -1.7136635221959295e-08f},
    {0.3826834261417389f, 6.2233507236442165e-09f, 0.9238795042037964f, 2.830748968563057e-08f},
    {0.40524131059646606f, 3.4085239075665186e-09f, 0.91420978307724f, -2.7373708633149363e-08f},
    {0.4275550842285156f, 9.201766459909777e-09f, 0.903989315032959f, -2.1909515979245953e-08f},
    {0.4496113359928131f, -6.338206404166158e-09f, 0.89322429895401f, 2.241505203670613e-09f},
    {0.4713967442512512f, -7.425253745196869e-09f, 0.8819212913513184f, -2.7002963420841297e-08f},
    {0.49289819598197937f, -3.75219544324068e-09f, 0.8700869679450989f, 2.3163613249721493e-08f},
    {0.5141027569770813f, -1.2783859304477119e-08f, 0.8577286005020142f, 9.498258179974073e-09f},
    {0.5349976420402527f, -2.2153155754267573e-08f, 0.8448535799980164f, -1.4748309240530943e-08f},
    {0.5555702447891235f, -1.1769521357507529e-08f, 0.8314695954322815f, 1.687026340846387e-08f},
    {0.5758081674575806f, 2.396026488327152e-08f, 0.8175848126411438f, 5.104399125599457e-10f},
    {0.5956993103027344f, -5.810301129116624e-09f, 0.803207516670227f, 1.4810417781063734e-08f},
    {0.6152315735816956f, 1.6998932039768988e-08f, 0.7883464097976685f, 1.7828938325692434e-08f},
    {0.6343932747840881f, 9.37955757507325e-09f, 0.7730104327201843f, 2.0642552556182636e-08f},
    {0.6531728506088257f, -7.655049039101414e-09f, 0.7572088241577148f, 2.2348769945779168e-08f},
    {0.6715589761734009f, -2.1326382437791835e-08f, 0.7409511208534241f, 4.501535144640911e-09f},
    {0.6895405650138855f, -2.027681844651852e-08f, 0.7242470979690552f, -1.5017588950172467e-08f},
    {0.7071067690849304f, 1.2101617485882343e-08f, 0.7071067690849304f, 1.2101617485882343e-08f},
};
}  // namespace

// sin(pi x) and cos(pi x) for a float x: x = k/2 + j/128 + z exactly, with |j| <= 32 and
// |z| <= 1/256; sin and cos of pi z from their Taylor series (degree 5 and 6: the first
// omitted terms are below 1e-16 of the result for |pi z| <= pi/256, the double-float terms
// are the ones above 1e-9), then the angle-sum formulas with the table entry for |j| and the
// quadrant k.
__device__ __forceinline__ void ff_sincospi(float x, ff& s, ff& c) {
    const float k = rintf(__fmul_rn(2.0f, x));
    const float y = __fsub_rn(x, __fmul_rn(0.5f, k));          // |y| <= 1/4, exact
    const int q = static_cast<int>(k) & 3;
    const float jf = rintf(__fmul_rn(128.0f, y));
    const float z = __fsub_rn(y, __fmul_rn(jf, 0.0078125f));   // |z| <= 1/256, exact (Sterbenz)
    const ff b = ff_mul(ff{3.14159274101257324f, -8.742277657347586e-08f}, z);
    const ff b2 = ff_mul(b, b);
    const float f2 = b2.hi;
    // sin b = b + b^3 (-1/6 + b^2 (1/120 - b^2 / 5040)), cos b = 1 + b^2 (-1/2 + b^2 (1/24 - b^2 / 720))
    const ff ps = ff_add(ff{-0.1666666716337204f, 4.967053879312289e-09f},
                         __fmul_rn(f2, __fmaf_rn(f2, -1.984127e-4f, 8.333333e-3f)));
    const ff pc = ff_add(ffv(-0.5f), __fmul_rn(f2, __fmaf_rn(f2, -1.3888889e-3f, 4.1666668e-2f)));
    const ff sb = ff_add_fast(b, ff_mul(ff_mul(b, b2), ps));
    const ff cb = ff_add_fast(ffv(1.0f), ff_mul(b2, pc));
    const int j = abs(static_cast<int>(jf));
    ff sa{k_sincospi_tab[j][0], k_sincospi_tab[j][1]};
    const ff ca{k_sincospi_tab[j][2], k_sincospi_tab[j][3]};
    if (jf < 0.0f) sa = ff_neg(sa);
    const ff sv = ff_add_fast(ff_mul(sa, cb), ff_mul(ca, sb));
    const ff cv = ff_sub_fast(ff_mul(ca, cb), ff_mul(sa, sb));
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
__device__ __forceinline__ ff3 ff3_add_fast(const ff3& a, const ff3& b) {
    return ff3{ff_add_fast(a.x, b.x), ff_add_fast(a.y, b.y), ff_add_fast(a.z, b.z)};
}
__device__ __forceinline__ ff3 ff3_sub_fast(const ff3& a, const ff3& b) {
    return ff3{ff_sub_fast(a.x, b.x), ff_sub_fast(a.y, b.y), ff_sub_fast(a.z, b.z)};
}
__device__ __forceinline__ ff3 ff3_scale(const ff3& a, ff s) { return ff3{ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)}; }
__device__ __forceinline__ ff3 ff3_scale(const ff3& a, float s) {
    return ff3{ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)};
}
__device__ __forceinline__ ff3 ff3_neg(const ff3& a) { return ff3{ff_neg(a.x), ff_neg(a.y), ff_neg(a.z)}; }
__device__ __forceinline__ ff ff3_dot(const ff3& a, const ff3& b) {
    return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
__device__ __forceinline__ ff ff3_dot_fast(const ff3& a, const ff3& b) {
    return ff_add_fast(ff_add_fast(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
// a . b - c rounded to float. The products of the high parts and their sums are formed exactly
// (TwoProd, TwoSum); only the low-order terms (product and sum errors, cross terms with the
// low parts) are added in FP32. The absolute error stays near 2^-48 (|a||b| + |c|) however much
// the terms cancel, so a result near zero keeps its relative accuracy.
__device__ __forceinline__ float ff3_dot_sub(const ff3& a, const ff3& b, float c) {
    const ff px = two_prod(a.x.hi, b.x.hi), py = two_prod(a.y.hi, b.y.hi), pz = two_prod(a.z.hi, b.z.hi);
    const ff s1 = two_sum(px.hi, py.hi);
    const ff s2 = two_sum(s1.hi, pz.hi);
    const ff s3 = two_sum(s2.hi, -c);
    float lo = __fadd_rn(__fadd_rn(__fadd_rn(px.lo, py.lo), __fadd_rn(pz.lo, s1.lo)), __fadd_rn(s2.lo, s3.lo));
    lo = __fmaf_rn(a.x.hi, b.x.lo, __fmaf_rn(a.x.lo, b.x.hi, lo));
    lo = __fmaf_rn(a.y.hi, b.y.lo, __fmaf_rn(a.y.lo, b.y.hi, lo));
    lo = __fmaf_rn(a.z.hi, b.z.lo, __fmaf_rn(a.z.lo, b.z.hi, lo));
    return __fadd_rn(s3.hi, lo);
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
