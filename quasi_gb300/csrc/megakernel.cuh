// megakernel.cuh - one-thread-per-path forms of the NEE path tracer (included by wavefront.cu):
//   k_megakernel  the forward renderer as a single persistent kernel (the wavefront's
//                 alternative; same per-vertex code, so bit-identical per-sample radiance)
//   k_adjoint     path-replay backpropagation: regenerates every path of a frame from its RNG
//                 key and accumulates dLoss/dalbedo and dLoss/demission per triangle.
//
// Adjoint of one path sample with vertices k = 1..K on triangles h_k (albedo rho_k), NEE
// lights l_k with factors gv_k (g times visibility, 0 without an unoccluded light sample),
// throughput beta_k = prod_{j<k} rho_j and the pixel's adjoint d = dLoss/dI_p / spp:
//   radiance = Le(h_1) + sum_k beta_k rho_k Le(l_k) gv_k
//   dL/dLe(h_1)  += d
//   dL/dLe(l_k)  += d beta_k rho_k gv_k
//   dL/drho(h_k) += d beta_k H_k,  H_k = Le(l_k) gv_k + rho_{k+1} H_{k+1},  H_{K+1} = 0
// (all products per colour channel). H_k needs no division by albedo, so zero albedos are
// exact. The per-vertex records of one path (at most k_adjoint_max_depth) live in local
// memory; nothing of the forward pass is stored.
#pragma once

#include "wavefront_kernels.cuh"

namespace quasi {

constexpr int k_adjoint_max_depth = 16;

// Camera ray of (pixel x,y; sample) in double-float, as k_camera builds it.
__device__ __forceinline__ void camera_ray_ff(const FrameParams& f, uint32_t x, uint32_t y, uint32_t sample, ff3& o,
                                              ff3& d) {
    uint32_t st = path_key(f.seed, y * f.width + x, sample, 0u);
    const float jx = rng_next(st);
    const float jy = rng_next(st);
    const ff u = ff_div(two_sum(static_cast<float>(x), jx), ffv(static_cast<float>(f.width)));
    const ff v = ff_sub(ffv(1.0f), ff_div(two_sum(static_cast<float>(y), jy), ffv(static_cast<float>(f.height))));
    d = ff3_normalize(ff3_sub(ff3_add(ff3_add(ff3_pair(f.cam.ll_hi, f.cam.ll_lo), ff3_scale(ff3_pair(f.cam.h_hi, f.cam.h_lo), u)),
                                      ff3_scale(ff3_pair(f.cam.v_hi, f.cam.v_lo), v)),
                              ff3v(f.cam.origin)));
    o = ff3v(f.cam.origin);
}

struct PathVertex {
    int prim;
    int light;
    float gv;
};

// Traces one path sample; fills up to k_adjoint_max_depth vertices when `verts` is given.
// Returns the radiance; writes first-hit AOVs and the signature when the pointers are set.
// rays / shadow_rays are incremented per closest-hit / shadow ray traced.
template <bool STATS>
__device__ __forceinline__ float3 trace_path(const FrameParams& f, const SceneDev& s, uint32_t x, uint32_t y,
                                             uint32_t sample, PathVertex* verts, int& n_verts, float4* aov_a,
                                             float4* aov_n, uint32_t* sig_out, uint32_t& err, TraceCounters& cnt,
                                             int& rays, int& shadow_rays) {
    const VertexScene vs{s.tri_in, s.albedo, s.emission, s.emitters, s.n_emit, f.eps};
    ff3 ro, rd;
    camera_ray_ff(f, x, y, sample, ro, rd);
    float3 beta = mk3(1.f, 1.f, 1.f), L = mk3(0.f, 0.f, 0.f);
    uint32_t sig = 0;
    int exclude = -1;
    n_verts = 0;
    for (uint32_t k = 1; k <= f.max_depth; ++k) {
        const RayInv r = make_ray(ff3_f(ro), ff3_f(rd));
        float t, bu, bv;
        ++rays;
        const int prim = trace_bvh<false, STATS>(s.nodes, s.tris, s.n_tris, r, __int_as_float(0x7f800000), exclude, t,
                                                 bu, bv, err, cnt);
        if (prim < 0) {
            sig = sig_mix(sig, k_sig_miss);
            break;
        }
        const float3 alb = xyz(__ldg(&s.albedo[prim]));
        const float3 nb = beta * alb;
        const bool cont = k < f.max_depth && max3(nb) > 0.0f;
        VertexResult v;
        shade_vertex(vs, path_key(f.seed, y * f.width + x, sample, k), prim, make_float4(t, 0.f, bu, bv), ro, rd, cont,
                     v);
        sig = sig_mix(sig, static_cast<uint32_t>(prim));
        if (k == 1) {
            const float3 em = xyz(__ldg(&s.emission[prim]));
            L = em;
            if (aov_a) first_hit_aovs(alb, em, t, v.nrm, *aov_a, *aov_n);
        }
        float gv = 0.0f;
        if (v.nee) {
            const RayInv sr = make_ray(v.so, v.sd);
            float st2, su, sv;
            ++shadow_rays;
            const int occ = trace_bvh<true, STATS>(s.nodes, s.tris, s.n_tris, sr, v.stmax, -1, st2, su, sv, err, cnt);
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

// Forward megakernel: warps take 32 paths of the wave at a time (persistent). Ray counts go
// to stats[4] (cumulative), stats[5] (closest-hit, this frame), stats[6] (shadow, this frame).
template <bool STATS>
__global__ void __launch_bounds__(128) k_megakernel(FrameParams f, SceneDev s, PathDev p, int* __restrict__ fetch,
                                                    uint32_t* __restrict__ err, unsigned long long* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int total = static_cast<int>(f.wave_spp * f.slots);
    uint32_t e = 0;
    TraceCounters c;
    int rays = 0, shadow_rays = 0;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const int gid = base + lane;
        if (gid >= total) continue;
        const uint32_t j = static_cast<uint32_t>(gid) / f.slots;
        uint32_t x, y;
        slot_to_xy(static_cast<uint32_t>(gid) - j * f.slots, f.tiles_x, x, y);
        if (x >= f.width || y >= f.height) continue;
        int nv = 0;
        float4 aa = make_float4(0.f, 0.f, 0.f, 0.f), an = aa;
        uint32_t sig = 0;
        const float3 L =
            trace_path<STATS>(f, s, x, y, f.sample_base + j, nullptr, nv, &aa, &an, &sig, e, c, rays, shadow_rays);
        p.lpath[gid] = make_float4(L.x, L.y, L.z, 0.f);
        p.aov_a[gid] = aa;
        p.aov_n[gid] = an;
        if (p.sig) p.sig[gid] = sig;
    }
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats);
    unsigned long long r = static_cast<unsigned long long>(rays), sr = static_cast<unsigned long long>(shadow_rays);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_xor_sync(0xffffffffu, r, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
    }
    if (lane == 0) {
        atomicAdd(&stats[4], r + sr);
        atomicAdd(&stats[5], r);
        atomicAdd(&stats[6], sr);
    }
}

// Path-replay adjoint over samples [sample_base, sample_base + wave_spp) of every pixel.
// grad_image: dLoss/dI per pixel (3 floats, row-major, top row first); grads are += into
// grad_albedo / grad_emission (3 floats per triangle, original order).
__global__ void __launch_bounds__(128) k_adjoint(FrameParams f, SceneDev s, const float* __restrict__ grad_image,
                                                 float inv_spp, float* __restrict__ grad_albedo,
                                                 float* __restrict__ grad_emission, int* __restrict__ fetch,
                                                 uint32_t* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int total = static_cast<int>(f.wave_spp * f.slots);
    uint32_t e = 0;
    TraceCounters c;
    PathVertex verts[k_adjoint_max_depth];
    float3 H[k_adjoint_max_depth];
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const int gid = base + lane;
        if (gid >= total) continue;
        const uint32_t j = static_cast<uint32_t>(gid) / f.slots;
        uint32_t x, y;
        slot_to_xy(static_cast<uint32_t>(gid) - j * f.slots, f.tiles_x, x, y);
        if (x >= f.width || y >= f.height) continue;
        const size_t px = static_cast<size_t>(y) * f.width + x;
        const float3 d = mk3(grad_image[3 * px] * inv_spp, grad_image[3 * px + 1] * inv_spp,
                             grad_image[3 * px + 2] * inv_spp);
        if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) continue;
        int nv = 0, rays = 0, shadow_rays = 0;
        trace_path<false>(f, s, x, y, f.sample_base + j, verts, nv, nullptr, nullptr, nullptr, e, c, rays, shadow_rays);
        nv = min(nv, k_adjoint_max_depth);
        if (nv == 0) continue;
        // camera-ray emission
        atomicAdd(&grad_emission[3 * verts[0].prim + 0], d.x);
        atomicAdd(&grad_emission[3 * verts[0].prim + 1], d.y);
        atomicAdd(&grad_emission[3 * verts[0].prim + 2], d.z);
        // suffix sums H_k, back to front
        float3 next = mk3(0.f, 0.f, 0.f);
        for (int k = nv - 1; k >= 0; --k) {
            float3 h = mk3(0.f, 0.f, 0.f);
            if (verts[k].light >= 0 && verts[k].gv != 0.0f) h = xyz(__ldg(&s.emission[verts[k].light])) * verts[k].gv;
            if (k + 1 < nv) h += xyz(__ldg(&s.albedo[verts[k + 1].prim])) * next;
            H[k] = h;
            next = h;
        }
        // front to back with the throughput
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
    if (e) atomicOr(err, e);
}

// Packs device materials (3 floats per triangle) into the float4 arrays the kernels read.
__global__ void __launch_bounds__(256) k_pack_materials(const float* __restrict__ albedo, const float* __restrict__ emission,
                                                        uint32_t n, float4* __restrict__ a4, float4* __restrict__ e4) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (albedo) a4[i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.f);
    if (emission) e4[i] = make_float4(emission[3 * i], emission[3 * i + 1], emission[3 * i + 2], 0.f);
}

}  // namespace quasi
