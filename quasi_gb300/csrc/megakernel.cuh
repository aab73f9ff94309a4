// megakernel.cuh - one-thread-per-path forms of the NEE path tracer (included by wavefront.cu):
//   k_megakernel  the forward renderer as a single persistent kernel (the wavefront's
//                 alternative; same per-vertex code, so bit-identical per-sample radiance)
//   k_adjoint     path-replay backpropagation: regenerates every path of a frame from its RNG
//                 key and accumulates dLoss/dalbedo and dLoss/demission per triangle
//                 (the per-path recursion is adjoint_path in path.cuh).
#pragma once

#include "path.cuh"

namespace quasi {

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
    const float pad = s.n_tris ? scene_box_pad(s.nodes) : 0.0f;
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
            trace_path<STATS>(f, s, x, y, f.sample_base + j, nullptr, nv, &aa, &an, &sig, e, c, rays, shadow_rays, pad);
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
// Rays replayed are added to stats[7].
__global__ void __launch_bounds__(128) k_adjoint(FrameParams f, SceneDev s, const float* __restrict__ grad_image,
                                                 float inv_spp, float* __restrict__ grad_albedo,
                                                 float* __restrict__ grad_emission, int* __restrict__ fetch,
                                                 uint32_t* __restrict__ err, unsigned long long* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int total = static_cast<int>(f.wave_spp * f.slots);
    uint32_t e = 0;
    TraceCounters c;
    int rays = 0;
    const float pad = s.n_tris ? scene_box_pad(s.nodes) : 0.0f;
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
        adjoint_path(f, s, x, y, f.sample_base + j, d, grad_albedo, grad_emission, e, c, rays, pad);
    }
    if (e) atomicOr(err, e);
    warp_add_count(rays, &stats[7]);
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
