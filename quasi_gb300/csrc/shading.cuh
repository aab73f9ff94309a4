// shading.cuh - one path vertex of the NEE integrator, shared by the wavefront shade kernel,
// the one-thread-per-path megakernel and the adjoint replay so all three take identical
// decisions and produce identical values for a given (seed, pixel, sample, bounce).
//
// Per vertex k of a path (hit triangle h, incoming double-float ray ro + t rd):
//   x   = plane(h) intersected with the double-float ray        (hit point)
//   n   = normalize(cross(e1, e2)) flipped to face the ray       (plugin.mm:192); the unit
//         normal and the plane offset n.v0 come from a per-triangle table built with the
//         LBVH, the light triangle's data from a per-emitter record built with it
//   key = path_key(seed, pixel, sample, k);  sel = pcg(key); r1, r2, r3, r4 chained
//   NEE: light l = emitters[(sel * n_emit) >> 32], point y = v0 + su(1-r2) e1 + su r2 e2,
//        su = sqrt(r1); g = cos_x cos_l / d^2 * area * n_emit / pi, skipped when l == h or a
//        cosine or d^2 is not positive; the shadow ray runs from y (lifted along the light
//        normal towards x) to just short of x + eps n.
//   continuation: cosine-weighted direction from (r3, r4) about n (plugin.mm:111-125),
//        origin x + eps n.
// The contribution of the NEE sample is beta * albedo(h) * emission(l) * g when unoccluded.
#pragma once

#include "common.cuh"
#include "ffmath.cuh"
#include "trace.cuh"

namespace quasi {

struct VertexScene {
    const float4* tri_plane;  // original order: unit normal of cross(e1, e2) and the plane offset n.v0
    const float4* emit_tab;   // per emitter slot: (v0, l), (v1, |ng|.hi), (v2, |ng|.lo), (n.x, n.y), (n.z)
    uint32_t n_emit;
    float eps;
};

struct VertexResult {
    float3 nrm;        // shading normal (float), facing the incoming ray
    bool nee;          // a shadow ray is wanted
    int light;         // emitter triangle of the NEE sample
    float g;           // NEE factor: contribution = beta * albedo * emission(light) * g
    float3 so, sd;     // shadow ray origin and unit direction (float)
    float stmax;       // shadow ray t_max
    ff3 seg_o, seg_d;  // the exact shadow segment: start and end - start (double-float)
    ff3 org;           // continuation origin x + eps n (double-float)
    ff3 dir;           // continuation direction (valid when want_dir)
    float t;           // distance of the hit along the ray (the plane's, rounded to float)
};

// FP32 dot product with a fixed operation order (no contraction choices left to the
// compiler), so every kernel that inlines the shading code computes the same bits.
__device__ __forceinline__ float fdot3(float3 a, float3 b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}

// The random numbers of one vertex, from its path key: sel picks the light, (r1, r2) the
// point on it, (r3, r4) the continuation direction.
struct VertexRandom {
    uint32_t sel;
    float r1, r2, r3, r4;
};

__device__ __forceinline__ VertexRandom vertex_random(uint32_t key) {
    VertexRandom r;
    uint32_t st = key;
    r.sel = pcg_hash(st);
    st = r.sel;
    r.r1 = rng_next(st);
    r.r2 = rng_next(st);
    r.r3 = rng_next(st);
    r.r4 = rng_next(st);
    return r;
}

// The light-sampling record of the emitter a vertex's NEE sample picked (l = -1 without
// emitters): the triangle's vertices, |cross(e1, e2)| and unit normal (k_emit_table).
struct LightTri {
    int l;
    float4 v0, v1, v2, n0, n1;
};

__device__ __forceinline__ LightTri load_light(const VertexScene& s, uint32_t sel) {
    LightTri t;
    t.l = -1;
    t.v0 = t.v1 = t.v2 = t.n0 = t.n1 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (s.n_emit > 0) {
        const float4* r = s.emit_tab + 5ull * static_cast<uint32_t>((static_cast<uint64_t>(sel) * s.n_emit) >> 32);
        t.v0 = __ldg(&r[0]);
        t.v1 = __ldg(&r[1]);
        t.v2 = __ldg(&r[2]);
        t.n0 = __ldg(&r[3]);
        t.n1 = __ldg(&r[4]);
        t.l = __float_as_int(t.v0.w);
    }
    return t;
}

// The hit point x (the hit triangle's plane n.x = n.v0 intersected with the double-float ray
// ro + t rd, t = (n.v0 - n.ro) / n.rd) and the unit normal facing the ray.
// t_hit: the hit's distance along the ray, the plane's t rounded to float (the first-hit
// depth). It depends only on the ray and the triangle, whereas the traversal's t depends on
// whether the hit was decided by the FP32 test or re-decided exactly, and so on the order in
// which a hierarchy presents the candidates.
__device__ __forceinline__ void vertex_point(const VertexScene& s, int prim, const ff3& ro, const ff3& rd, ff3& x,
                                             ff3& nrm, float& t_hit) {
    const float4 p = __ldg(&s.tri_plane[2 * prim]), q = __ldg(&s.tri_plane[2 * prim + 1]);
    nrm = ff3{ff{p.x, p.y}, ff{p.z, p.w}, ff{q.x, q.y}};
    const ff den = ff3_dot_fast(nrm, rd);
    if (den.hi != 0.0f) {
        const ff t = ff_div(ff_sub_fast(ff{q.z, q.w}, ff3_dot_fast(nrm, ro)), den);
        x = ff3_add_fast(ro, ff3_scale(rd, t));
        t_hit = ff_f(t);
    } else {
        // A ray parallel to the plane cannot hit the triangle (an exact hit needs
        // det = -d.(e1 x e2) != 0); kept only so that x is defined.
        x = ro;
        t_hit = 0.0f;
    }
    if (den.hi > 0.0f) nrm = ff3_neg(nrm);
}

// Continuation origin x + eps n.
__device__ __forceinline__ ff3 vertex_origin(const VertexScene& s, const ff3& x, const ff3& nrm) {
    return ff3_add_fast(x, ff3_scale(nrm, s.eps));
}

// Cosine-weighted continuation direction about n = nrm (plugin.mm:111-125) in double-float:
// phi = 2 pi r3, cos = sqrt(1 - r4), sin = sqrt(r4), in the basis (u, v, n) with
// v = normalize(cross(n, a)), a = (0,1,0) if |n.x| > 0.9 else (1,0,0), u = cross(n, v).
// With c = cross(n, a): v = c / |c| and u = cross(n, c) / |c|, whose components are single
// products (|c|^2 is the sum of the other two squares), so
//   dir = (cross(n, c) cos(phi) + c sin(phi)) sin / |c| + n cos
// with one division and no normalised basis vectors. The basis is orthonormal to ~1e-14 and
// cos^2 + sin^2 = 1, so dir is a unit vector to that accuracy without the final
// normalisation of plugin.mm:124.
__device__ __forceinline__ ff3 vertex_dir(const ff3& nrm, float r3, float r4) {
    ff sphi, cphi;
    ff_sincospi(2.0f * r3, sphi, cphi);
    const ff cos_t = ff_sqrt(two_sum(1.0f, -r4));
    const ff sin_t = ff_sqrt(ffv(r4));
    const ff &x = nrm.x, &y = nrm.y, &z = nrm.z;
    ff3 c, nc;  // c = cross(n, a), nc = cross(n, c)
    ff cc;      // |c|^2
    if (fabsf(x.hi) > 0.9f) {
        cc = ff_add_fast(ff_mul(x, x), ff_mul(z, z));
        c = ff3{ff_neg(z), ffv(0.0f), x};
        nc = ff3{ff_mul(x, y), ff_neg(cc), ff_mul(y, z)};
    } else {
        cc = ff_add_fast(ff_mul(y, y), ff_mul(z, z));
        c = ff3{ffv(0.0f), z, ff_neg(y)};
        nc = ff3{ff_neg(cc), ff_mul(x, y), ff_mul(x, z)};
    }
    const ff g = ff_div(sin_t, ff_sqrt(cc));
    const ff wu = ff_mul(cphi, g), wv = ff_mul(sphi, g);
    return ff3_add_fast(ff3_add_fast(ff3_scale(nc, wu), ff3_scale(c, wv)), ff3_scale(nrm, cos_t));
}

// The NEE sample of a vertex at x (normal nrm, continuation origin org) towards the light
// triangle lt: sets nee, light, g, the FP32 shadow ray and the exact segment.
__device__ __forceinline__ void vertex_light(const VertexScene& s, int prim, const LightTri& lt, float r1, float r2,
                                             const ff3& x, const ff3& nrm, const ff3& org, VertexResult& out) {
    out.nee = false;
    out.light = -1;
    out.g = 0.0f;
    if (s.n_emit == 0 || lt.l == prim) return;
    const float3 la = xyz(lt.v0);
    const ff3 le1 = ff3_diff(xyz(lt.v1), la);
    const ff3 le2 = ff3_diff(xyz(lt.v2), la);
    const ff su = ff_sqrt(ffv(r1));
    const ff3 yl = ff3_add_fast(ff3_add_fast(ff3v(la), ff3_scale(le1, ff_mul(su, two_sum(1.0f, -r2)))),
                                ff3_scale(le2, ff_mul(su, r2)));
    // (y - x) first, in double-float: both lie on their planes, so a small surface-to-light
    // gap keeps its digits; subtracting the rounded offset origin would not. The light sample
    // only weights this vertex (nothing of it carries to the next bounce), so once that
    // difference is formed the eps offset and the length are FP32 (relative errors ~1e-7).
    const ff3 dxy = ff3_sub_fast(yl, x);
    const float3 d0 = ff3_f(dxy);
    const float3 nf = ff3_f(nrm);
    const float3 dv = mk3(__fsub_rn(d0.x, __fmul_rn(s.eps, nf.x)), __fsub_rn(d0.y, __fmul_rn(s.eps, nf.y)),
                          __fsub_rn(d0.z, __fmul_rn(s.eps, nf.z)));
    const float d2 = fdot3(dv, dv);
    const float inv_dist = __fdiv_rn(1.0f, __fsqrt_rn(d2));
    // The cosines are not: an FP32 dot of unit vectors keeps an absolute error of ~1e-7, a
    // relative error above 1e-4 once a grazing light sample brings a cosine below ~1e-3. Both
    // come from the double-float difference with exact products and sums instead:
    // n.dv = n.(y - x) - eps (n is a unit vector) and nl.dv = nl.(y - x) - eps (nl.n).
    const ff area2 = ff{lt.v1.w, lt.v2.w};
    const ff3 nl = ff3{ff{lt.n0.x, lt.n0.y}, ff{lt.n0.z, lt.n0.w}, ff{lt.n1.x, lt.n1.y}};
    const float cos_x = __fmul_rn(ff3_dot_sub(nrm, dxy, s.eps), inv_dist);
    const float cl = __fmul_rn(ff3_dot_sub(nl, dxy, __fmul_rn(s.eps, fdot3(ff3_f(nl), nf))), inv_dist);
    const float cos_l = fabsf(cl);
    if (cos_x > 0.0f && cos_l > 0.0f && d2 > 0.0f) {
        out.g = cos_x * cos_l / d2 * (0.5f * ff_f(area2)) * static_cast<float>(s.n_emit) * k_inv_pi;
        // The shadow ray runs from the light sample, lifted by eps along the light's
        // normal towards the shading side, to just short of the lifted shading point:
        // neither end's plane (nor a coplanar neighbour) can be crossed.
        const float side = cl < 0.0f ? s.eps : -s.eps;
        const ff3 so = ff3_add_fast(yl, ff3_scale(nl, side));
        out.seg_o = so;
        out.seg_d = ff3_sub_fast(org, so);
        const float3 sd = ff3_f(out.seg_d);
        const float sdist = __fsqrt_rn(fdot3(sd, sd));
        const float inv_s = __fdiv_rn(1.0f, sdist);
        out.so = ff3_f(so);
        out.sd = mk3(__fmul_rn(sd.x, inv_s), __fmul_rn(sd.y, inv_s), __fmul_rn(sd.z, inv_s));
        out.stmax = sdist * (1.0f - 1e-4f);
        out.light = lt.l;
        out.nee = true;
    }
}

// hit: (t, prim, -, -) from the traversal; ro, rd: the double-float ray that found it. The
// light choice depends only on the path key: its dependent loads (emitter index, then the
// light triangle and its table entry) start before the hit-point arithmetic so their latency
// overlaps it.
__device__ __forceinline__ void shade_vertex(const VertexScene& s, uint32_t key, int prim, float4 /*hit*/,
                                             const ff3& ro, const ff3& rd, bool want_dir, VertexResult& out) {
    const VertexRandom r = vertex_random(key);
    const LightTri lt = load_light(s, r.sel);
    ff3 x, nrm;
    vertex_point(s, prim, ro, rd, x, nrm, out.t);
    out.nrm = ff3_f(nrm);
    out.org = vertex_origin(s, x, nrm);
    vertex_light(s, prim, lt, r.r1, r.r2, x, nrm, out.org, out);
    if (want_dir) out.dir = vertex_dir(nrm, r.r3, r.r4);
}

// First-hit AOVs (plugin.mm:242-249, 301): albedo (emission for emitters), depth, normal.
__device__ __forceinline__ void first_hit_aovs(float3 alb, float3 em, float t, float3 nrm, float4& aov_a, float4& aov_n) {
    const float3 aa = max3(em) > 0.1f ? em : alb;
    const float depth = fminf(fmaxf((t - 1.0f) * 0.25f, 0.0f), 1.0f);
    aov_a = make_float4(aa.x, aa.y, aa.z, depth);
    aov_n = make_float4(nrm.x * 0.5f + 0.5f, nrm.y * 0.5f + 0.5f, nrm.z * 0.5f + 0.5f, 0.f);
}

}  // namespace quasi
