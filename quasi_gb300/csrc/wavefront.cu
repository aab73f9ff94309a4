// wavefront.cu - the NEE path tracer as a wavefront of kernels, plus the Renderer host code.
//
// One wave = wave_spp samples of every pixel. Per wave:
//   k_camera                 camera rays for every (sample, pixel) -> ray queue
//   for bounce k = 1..D:
//     k_trace_closest        persistent, warp-fetched closest-hit traversal of the queue
//     k_shade                emission (k == 1), AOVs (k == 1), light sample -> shadow queue,
//                            cosine-weighted continuation -> next ray queue; both queues are
//                            compacted with one atomic per warp (ballot + popc)
//     k_trace_shadow         persistent any-hit traversal; unoccluded rays add their
//                            contribution to the owning path's radiance
//   k_accumulate             per pixel, Kahan-adds the wave's samples in sample order
// Paths are addressed by a stable id (sample-in-wave * slots + tile-ordered pixel slot); a
// path has at most one ray in each queue, so no two threads ever update the same path.
#include "common.cuh"
#include "renderer.hpp"
#include "trace.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace quasi {

// ---------------------------------------------------------------------------- kernels

struct FrameParams {
    CameraBasis cam;
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
    const int* emitters;
    const float4* nodes;
    const float4* tris;     // leaf order, v0+orig, e1, e2
    uint32_t n_tris, n_emit;
};

struct PathDev {
    float4* beta;
    float4* lpath;
    float4* aov_a;   // first-hit albedo (rgb) + depth (w)
    float4* aov_n;   // first-hit remapped normal
    uint32_t* sig;   // path signatures (record mode) or null
};

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

__global__ void __launch_bounds__(256) k_pack_tris(const float* __restrict__ raw, uint32_t n, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = raw + 9ull * i;
    out[3 * i + 0] = make_float4(v[0], v[1], v[2], 0.f);
    out[3 * i + 1] = make_float4(v[3], v[4], v[5], 0.f);
    out[3 * i + 2] = make_float4(v[6], v[7], v[8], 0.f);
}

__global__ void __launch_bounds__(256) k_camera(FrameParams f, PathDev p, float4* __restrict__ q, int* __restrict__ q_count) {
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= f.wave_spp * f.slots) return;  // slots is a multiple of 32: whole warps leave
    const uint32_t j = gid / f.slots, slot = gid - j * f.slots;
    uint32_t x, y;
    slot_to_xy(slot, f.tiles_x, x, y);
    const bool valid = x < f.width && y < f.height;
    float3 d = mk3(0.f, 0.f, 0.f);
    if (valid) {
        const uint32_t pixel = y * f.width + x;
        uint32_t st = path_key(f.seed, pixel, f.sample_base + j, 0u);
        const float jx = rng_next(st);
        const float jy = rng_next(st);
        const float u = (static_cast<float>(x) + jx) / static_cast<float>(f.width);
        const float v = 1.0f - (static_cast<float>(y) + jy) / static_cast<float>(f.height);
        d = camera_dir(f.cam, u, v);
        p.beta[gid] = make_float4(1.f, 1.f, 1.f, 0.f);
        p.lpath[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.aov_a[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        p.aov_n[gid] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p.sig) p.sig[gid] = 0u;
    }
    const int pos = warp_append(0xffffffffu, valid, q_count);
    if (valid) {
        q[2 * pos] = make_float4(f.cam.origin.x, f.cam.origin.y, f.cam.origin.z, __int_as_float(static_cast<int>(gid)));
        q[2 * pos + 1] = make_float4(d.x, d.y, d.z, __int_as_float(-1));
    }
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

// Persistent closest-hit traversal: warps grab 32 rays at a time from the queue.
template <bool STATS>
__global__ void __launch_bounds__(256) k_trace_closest(SceneDev s, const float4* __restrict__ q,
                                                       float4* __restrict__ hits, const int* __restrict__ count,
                                                       int capacity, int* __restrict__ fetch,
                                                       uint32_t* __restrict__ err, unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    const int lane = threadIdx.x & 31;
    uint32_t e = 0;
    TraceCounters c;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i < n) {
            const float4 r0 = q[2 * i], r1 = q[2 * i + 1];
            const RayInv r = make_ray(xyz(r0), xyz(r1));
            float t, bu, bv;
            const int prim = trace_bvh<false, STATS>(s.nodes, s.tris, s.n_tris, r, __int_as_float(0x7f800000),
                                                     __float_as_int(r1.w), t, bu, bv, e, c);
            hits[i] = make_float4(t, __int_as_float(prim), bu, bv);
        }
    }
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats);
}

template <bool STATS>
__global__ void __launch_bounds__(256) k_trace_shadow(SceneDev s, PathDev p, const float4* __restrict__ sq,
                                                      const int* __restrict__ count, int capacity,
                                                      int* __restrict__ fetch, uint32_t* __restrict__ err,
                                                      unsigned long long* __restrict__ stats) {
    const int n = min(*count, capacity);
    const int lane = threadIdx.x & 31;
    uint32_t e = 0;
    TraceCounters c;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i < n) {
            const float4 r0 = sq[3 * i], r1 = sq[3 * i + 1], r2 = sq[3 * i + 2];
            const RayInv r = make_ray(xyz(r0), xyz(r1));
            float t, bu, bv;
            const int hit = trace_bvh<true, STATS>(s.nodes, s.tris, s.n_tris, r, r1.w, -1, t, bu, bv, e, c);
            const int pid = __float_as_int(r0.w);
            if (hit < 0) {
                float4 L = p.lpath[pid];
                L.x += r2.x;
                L.y += r2.y;
                L.z += r2.z;
                p.lpath[pid] = L;
            }
            if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], hit < 0 ? k_sig_lit : k_sig_shadowed);
        }
    }
    if (e) atomicOr(err, e);
    flush_counters<STATS>(c, stats + 2);
}

// Adds the frame's queue lengths (rays traced) to the cumulative counter stats[4]; one
// warp, so the timed loop needs no host synchronisation to know how many rays it traced.
__global__ void k_tally(const int* __restrict__ counters, uint32_t waves, uint32_t depth,
                        unsigned long long* __restrict__ stats) {
    unsigned long long sum = 0;
    for (uint32_t i = threadIdx.x; i < waves * 2 * depth; i += 32) {
        const uint32_t w = i / (2 * depth), k = i - w * 2 * depth;
        sum += static_cast<unsigned long long>(max(counters[w * 4 * depth + k], 0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (threadIdx.x == 0) stats[4] += sum;
}

__global__ void __launch_bounds__(256) k_shade(FrameParams f, SceneDev s, PathDev p, uint32_t bounce,
                                               const float4* __restrict__ q, const float4* __restrict__ hits,
                                               const int* __restrict__ count, int capacity, float4* __restrict__ next_q,
                                               int* __restrict__ next_count, float4* __restrict__ shadow_q,
                                               int* __restrict__ shadow_count) {
    const int n = min(*count, capacity);
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
        const int i = base + lane;
        bool want_shadow = false, want_next = false;
        float3 org = mk3(0.f, 0.f, 0.f), wi = org, contrib = org, nd = org;
        float tmax_s = 0.f;
        int pid = 0, prim = -1;
        if (i < n) {
            const float4 r0 = q[2 * i], r1 = q[2 * i + 1];
            const float4 h = hits[i];
            pid = __float_as_int(r0.w);
            prim = __float_as_int(h.y);
            if (prim < 0) {
                if (p.sig) p.sig[pid] = sig_mix(p.sig[pid], k_sig_miss);
            } else {
                const float3 d = xyz(r1);
                const float3 a = xyz(__ldg(&s.tri_in[3 * prim]));
                const float3 e1 = xyz(__ldg(&s.tri_in[3 * prim + 1])) - a;
                const float3 e2 = xyz(__ldg(&s.tri_in[3 * prim + 2])) - a;
                const float3 x = a + e1 * h.z + e2 * h.w;  // barycentric hit point, on the plane
                float3 nrm = normalize(cross(e1, e2));
                if (dot(nrm, d) > 0.0f) nrm = -nrm;
                const float3 alb = xyz(__ldg(&s.albedo[prim]));
                float3 beta = xyz(p.beta[pid]);
                uint32_t sig = p.sig ? sig_mix(p.sig[pid], static_cast<uint32_t>(prim)) : 0u;
                if (bounce == 1) {
                    const float3 em = xyz(__ldg(&s.emission[prim]));
                    p.lpath[pid] = make_float4(em.x, em.y, em.z, 0.f);
                    const float3 aa = max3(em) > 0.1f ? em : alb;
                    const float depth = fminf(fmaxf((h.x - 1.0f) * 0.25f, 0.0f), 1.0f);
                    p.aov_a[pid] = make_float4(aa.x, aa.y, aa.z, depth);
                    p.aov_n[pid] = make_float4(nrm.x * 0.5f + 0.5f, nrm.y * 0.5f + 0.5f, nrm.z * 0.5f + 0.5f, 0.f);
                }
                const uint32_t j = static_cast<uint32_t>(pid) / f.slots;
                uint32_t px, py;
                slot_to_xy(static_cast<uint32_t>(pid) - j * f.slots, f.tiles_x, px, py);
                uint32_t st = path_key(f.seed, py * f.width + px, f.sample_base + j, bounce);
                const uint32_t sel = pcg_hash(st);
                st = sel;
                const float r1 = rng_next(st);
                const float r2 = rng_next(st);
                org = x + nrm * f.eps;
                if (s.n_emit > 0) {
                    const int l = __ldg(&s.emitters[static_cast<uint32_t>((static_cast<uint64_t>(sel) * s.n_emit) >> 32)]);
                    if (l != prim) {
                        const float3 la = xyz(__ldg(&s.tri_in[3 * l]));
                        const float3 e1 = xyz(__ldg(&s.tri_in[3 * l + 1])) - la;
                        const float3 e2 = xyz(__ldg(&s.tri_in[3 * l + 2])) - la;
                        const float su = sqrtf(r1);
                        const float3 yl = la + e1 * (su * (1.0f - r2)) + e2 * (su * r2);
                        // (y - x) first: both lie on their planes, so a small surface-to-light gap
                        // keeps its digits; subtracting the rounded offset origin would not.
                        const float3 dv = (yl - x) - nrm * f.eps;
                        const float d2 = dot(dv, dv);
                        const float dist = sqrtf(d2);
                        wi = dv * (1.0f / dist);
                        const float cos_x = dot(nrm, wi);
                        const float3 nl = cross(e1, e2);
                        const float area2 = sqrtf(dot(nl, nl));
                        const float cos_l = fabsf(dot(nl, wi)) / area2;
                        if (cos_x > 0.0f && cos_l > 0.0f && d2 > 0.0f) {
                            const float g = cos_x * cos_l / d2 * (0.5f * area2) * static_cast<float>(s.n_emit) * k_inv_pi;
                            contrib = beta * alb * xyz(__ldg(&s.emission[l])) * g;
                            tmax_s = dist * (1.0f - 1e-4f);
                            want_shadow = true;
                        }
                    }
                }
                if (!want_shadow) sig = sig_mix(sig, k_sig_no_nee);
                const float r3 = rng_next(st);
                const float r4 = rng_next(st);
                nd = cosine_sample(nrm, r3, r4);
                beta = beta * alb;
                p.beta[pid] = make_float4(beta.x, beta.y, beta.z, 0.f);
                if (p.sig) p.sig[pid] = sig;
                want_next = bounce < f.max_depth && max3(beta) > 0.0f;
            }
        }
        const int ps = warp_append(0xffffffffu, want_shadow, shadow_count);
        if (want_shadow) {
            shadow_q[3 * ps] = make_float4(org.x, org.y, org.z, __int_as_float(pid));
            shadow_q[3 * ps + 1] = make_float4(wi.x, wi.y, wi.z, tmax_s);
            shadow_q[3 * ps + 2] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
        }
        const int pn = warp_append(0xffffffffu, want_next, next_count);
        if (want_next) {
            next_q[2 * pn] = make_float4(org.x, org.y, org.z, __int_as_float(pid));
            next_q[2 * pn + 1] = make_float4(nd.x, nd.y, nd.z, __int_as_float(prim));
        }
    }
}

__global__ void __launch_bounds__(256) k_accumulate(FrameParams f, PathDev p, float4* __restrict__ accum,
                                                    float4* __restrict__ comp, float4* __restrict__ aov_a,
                                                    float4* __restrict__ aov_n, float* __restrict__ rec_rad,
                                                    uint32_t* __restrict__ rec_sig) {
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= f.width * f.height) return;
    const uint32_t y = pixel / f.width, x = pixel - y * f.width;
    const uint32_t slot = xy_to_slot(x, y, f.tiles_x);
    float4 sum = accum[pixel], c = comp[pixel], A = aov_a[pixel], N = aov_n[pixel];
    for (uint32_t j = 0; j < f.wave_spp; ++j) {
        const uint32_t pid = j * f.slots + slot;
        const float4 L = p.lpath[pid];
        kahan_add(sum.x, c.x, L.x);
        kahan_add(sum.y, c.y, L.y);
        kahan_add(sum.z, c.z, L.z);
        const float4 a = p.aov_a[pid], nn = p.aov_n[pid];
        A.x += a.x; A.y += a.y; A.z += a.z; A.w += a.w;
        N.x += nn.x; N.y += nn.y; N.z += nn.z;
        if (rec_rad) {
            const size_t idx = static_cast<size_t>(pixel) * f.frame_spp + f.wave_offset + j;
            rec_rad[3 * idx] = L.x;
            rec_rad[3 * idx + 1] = L.y;
            rec_rad[3 * idx + 2] = L.z;
            rec_sig[idx] = p.sig ? p.sig[pid] : 0u;
        }
    }
    accum[pixel] = sum;
    comp[pixel] = c;
    aov_a[pixel] = A;
    aov_n[pixel] = N;
}

// Mean image (RGBA, alpha 1) from the accumulation: mode 0 beauty, 1 albedo, 2 normal, 3 depth.
__global__ void __launch_bounds__(256) k_resolve(const float4* __restrict__ accum, const float4* __restrict__ aov_a,
                                                 const float4* __restrict__ aov_n, uint32_t n_px, float count,
                                                 int mode, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_px) return;
    float4 v;
    if (mode == 0) v = accum[i];
    else if (mode == 1 || mode == 3) v = aov_a[i];
    else v = aov_n[i];
    float4 o;
    if (count <= 0.0f) o = make_float4(0.f, 0.f, 0.f, 1.f);
    else if (mode == 3) { const float d = v.w / count; o = make_float4(d, d, d, 1.f); }
    else o = make_float4(v.x / count, v.y / count, v.z / count, 1.f);
    out[i] = o;
}

// plugin.mm:334-350: Reinhard then gamma 1/2.2, written as RGBA8 into a device buffer.
__global__ void __launch_bounds__(256) k_tonemap(const float4* __restrict__ accum, uint32_t n_px, float count,
                                                 uchar4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_px) return;
    const float4 s = accum[i];
    const float inv = count > 0.f ? 1.0f / count : 0.f;
    float c[3] = {s.x * inv, s.y * inv, s.z * inv};
    unsigned char b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float m = c[k] / (c[k] + 1.0f);
        const float g = powf(fmaxf(m, 0.0f), 1.0f / 2.2f);
        b[k] = static_cast<unsigned char>(fminf(g * 255.0f + 0.5f, 255.0f));
    }
    out[i] = make_uchar4(b[0], b[1], b[2], 255);
}

// ---------------------------------------------------------------------------- host

namespace {

inline uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

CameraBasis make_camera_basis(const Q_camera& c, uint32_t w, uint32_t h) {
    // plugin.mm:649-674 (host direction) and plugin.mm:134-147 (shader basis), in double.
    double dir[3] = {double(c.target[0]) - c.position[0], double(c.target[1]) - c.position[1],
                     double(c.target[2]) - c.position[2]};
    double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (len > 0) for (double& v : dir) v /= len;
    double wv[3] = {-dir[0], -dir[1], -dir[2]};
    len = std::sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
    if (len > 0) for (double& v : wv) v /= len;
    const double up[3] = {c.up[0], c.up[1], c.up[2]};
    double r[3] = {up[1] * wv[2] - up[2] * wv[1], up[2] * wv[0] - up[0] * wv[2], up[0] * wv[1] - up[1] * wv[0]};
    len = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (len > 0) for (double& v : r) v /= len;
    const double u2[3] = {wv[1] * r[2] - wv[2] * r[1], wv[2] * r[0] - wv[0] * r[2], wv[0] * r[1] - wv[1] * r[0]};
    const double theta = double(c.fov) * 3.14159265358979323846 / 180.0;
    const double vh = 2.0 * std::tan(theta / 2.0);
    const double vw = (double(w) / double(h)) * vh;
    CameraBasis b;
    b.origin = make_float3(c.position[0], c.position[1], c.position[2]);
    double H[3], V[3], LL[3];
    for (int k = 0; k < 3; ++k) {
        H[k] = vw * r[k];
        V[k] = vh * u2[k];
        LL[k] = double(c.position[k]) - H[k] * 0.5 - V[k] * 0.5 - wv[k];
    }
    b.horizontal = make_float3(float(H[0]), float(H[1]), float(H[2]));
    b.vertical = make_float3(float(V[0]), float(V[1]), float(V[2]));
    b.lower_left = make_float3(float(LL[0]), float(LL[1]), float(LL[2]));
    return b;
}

}  // namespace

// Reference-integrator entry point (refmode.cu).
cudaError_t launch_reference_frame(const float4* quads, uint32_t n_quads, const Q_camera& cam, uint32_t width,
                                   uint32_t height, uint32_t sample_base, uint32_t spp, float4* accum, float4* comp,
                                   float4* aov_a, float4* aov_n, cudaStream_t s, KernelProfiler& prof);

Renderer::Renderer(int device, cudaStream_t stream, bool own_stream)
    : device_(device), stream_(stream), own_stream_(own_stream) {
    opt_.spp_per_frame = 1;
    opt_.max_depth = 4;
    opt_.rebuild_each_frame = 1;
    opt_.ray_eps = 1e-4f;
}

Renderer::~Renderer() {
    if (stream_) cudaStreamSynchronize(stream_);
    bvh_.release();
    for (DeviceBuffer* b : {&raw_vertices_, &tri_in_, &albedo_, &emission_, &emitters_, &quads_, &accum_, &comp_,
                            &aov_albedo_, &aov_normal_, &record_rad_, &record_sig_, &queue_[0], &queue_[1], &hits_,
                            &shadow_, &beta_, &lpath_, &aov_a_, &aov_n_, &sig_, &counters_, &stats_dev_, &err_dev_})
        b->release();
    if (counters_host_) cudaFreeHost(counters_host_);
    if (stats_host_) cudaFreeHost(stats_host_);
    if (err_host_) cudaFreeHost(err_host_);
    for (cudaEvent_t e : {ev_frame0_, ev_frame1_, ev_bvh0_, ev_bvh1_})
        if (e) cudaEventDestroy(e);
    if (own_stream_ && stream_) cudaStreamDestroy(stream_);
}

int Renderer::cuda_fail(cudaError_t e, const char* where) {
    error_ = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QUASI_ERR_OOM : QUASI_ERR_CUDA;
}

#define R_TRY(expr, where)                                  \
    do {                                                    \
        cudaError_t r_err_ = (expr);                        \
        if (r_err_ != cudaSuccess) return cuda_fail(r_err_, where); \
    } while (0)

int Renderer::init() {
    R_TRY(cudaSetDevice(device_), "cudaSetDevice");
    R_TRY(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "sm count");
    if (!stream_) {
        R_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
        own_stream_ = true;
    }
    R_TRY(cudaEventCreate(&ev_frame0_), "event");
    R_TRY(cudaEventCreate(&ev_frame1_), "event");
    R_TRY(cudaEventCreate(&ev_bvh0_), "event");
    R_TRY(cudaEventCreate(&ev_bvh1_), "event");
    R_TRY(stats_dev_.reserve(sizeof(unsigned long long) * 8), "stats");
    R_TRY(err_dev_.reserve(sizeof(uint32_t)), "err");
    R_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, stats_dev_.bytes, stream_), "memset");
    R_TRY(cudaMemsetAsync(err_dev_.ptr, 0, err_dev_.bytes, stream_), "memset");
    R_TRY(cudaMallocHost(&stats_host_, sizeof(unsigned long long) * 8), "pinned");
    R_TRY(cudaMallocHost(&err_host_, sizeof(uint32_t)), "pinned");
    std::memset(stats_host_, 0, sizeof(unsigned long long) * 8);
    *err_host_ = 0;
    return QUASI_OK;
}

int Renderer::upload_materials_host(const float* albedo, const float* emission, uint32_t n) {
    std::vector<float4> a(n), e(n);
    std::vector<int> emit;
    for (uint32_t i = 0; i < n; ++i) {
        a[i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.f);
        e[i] = make_float4(emission[3 * i], emission[3 * i + 1], emission[3 * i + 2], 0.f);
        if (e[i].x > 0.f || e[i].y > 0.f || e[i].z > 0.f) emit.push_back(static_cast<int>(i));
    }
    R_TRY(albedo_.reserve(sizeof(float4) * n), "albedo");
    R_TRY(emission_.reserve(sizeof(float4) * n), "emission");
    R_TRY(emitters_.reserve(sizeof(int) * std::max<size_t>(emit.size(), 1)), "emitters");
    if (n) {
        R_TRY(cudaMemcpyAsync(albedo_.ptr, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream_), "h2d");
        R_TRY(cudaMemcpyAsync(emission_.ptr, e.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream_), "h2d");
    }
    if (!emit.empty())
        R_TRY(cudaMemcpyAsync(emitters_.ptr, emit.data(), sizeof(int) * emit.size(), cudaMemcpyHostToDevice, stream_),
              "h2d");
    n_emit_ = static_cast<uint32_t>(emit.size());
    // The staging vectors die at return: wait for the copies.
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    return QUASI_OK;
}

int Renderer::set_scene(const Q_cuda_scene& sc) {
    if (sc.tri_count > 0 && (!sc.vertices || !sc.albedo || !sc.emission))
        return fail(QUASI_ERR_INVALID, "scene arrays missing");
    if (sc.quad_count > 0 && (!sc.quads || !sc.quad_albedo || !sc.quad_emission))
        return fail(QUASI_ERR_INVALID, "quad arrays missing");
    if (sc.tri_count > (1u << 28)) return fail(QUASI_ERR_INVALID, "too many triangles");
    n_tris_ = sc.tri_count;
    R_TRY(raw_vertices_.reserve(sizeof(float) * 9ull * n_tris_), "vertices");
    R_TRY(tri_in_.reserve(sizeof(float4) * 3ull * n_tris_), "tri_in");
    int rc = update_vertices(sc.vertices, sc.tri_count);
    if (rc) return rc;
    rc = upload_materials_host(sc.albedo, sc.emission, n_tris_);
    if (rc) return rc;
    n_quads_ = sc.quad_count;
    if (n_quads_) {
        std::vector<float4> q(5ull * n_quads_);
        for (uint32_t i = 0; i < n_quads_; ++i) {
            const float* g = sc.quads + 9ull * i;
            q[5 * i + 0] = make_float4(g[0], g[1], g[2], 0.f);
            q[5 * i + 1] = make_float4(g[3], g[4], g[5], 0.f);
            q[5 * i + 2] = make_float4(g[6], g[7], g[8], 0.f);
            q[5 * i + 3] = make_float4(sc.quad_albedo[3 * i], sc.quad_albedo[3 * i + 1], sc.quad_albedo[3 * i + 2], 0.f);
            q[5 * i + 4] = make_float4(sc.quad_emission[3 * i], sc.quad_emission[3 * i + 1], sc.quad_emission[3 * i + 2], 0.f);
        }
        R_TRY(quads_.reserve(sizeof(float4) * q.size()), "quads");
        R_TRY(cudaMemcpy(quads_.ptr, q.data(), sizeof(float4) * q.size(), cudaMemcpyHostToDevice), "h2d");
    }
    scene_camera_ = sc.camera;
    has_scene_ = true;
    bvh_dirty_ = true;
    return reset();
}

int Renderer::update_vertices(const float* vertices, uint32_t tri_count) {
    if (tri_count != n_tris_) return fail(QUASI_ERR_INVALID, "vertex count differs from the scene");
    if (tri_count == 0) return QUASI_OK;
    if (!vertices) return fail(QUASI_ERR_INVALID, "null vertices");
    R_TRY(cudaMemcpyAsync(raw_vertices_.ptr, vertices, sizeof(float) * 9ull * tri_count, cudaMemcpyHostToDevice, stream_),
          "h2d vertices");
    R_TRY(QUASI_LAUNCH(prof_, "pack_tris", stream_,
                       (k_pack_tris<<<ceil_div(tri_count, 256), 256, 0, stream_>>>(raw_vertices_.as<float>(), tri_count,
                                                                                 tri_in_.as<float4>()))),
          "pack_tris");
    bvh_dirty_ = true;
    return QUASI_OK;
}

int Renderer::set_materials(const float* albedo, const float* emission, uint32_t tri_count) {
    if (tri_count != n_tris_) return fail(QUASI_ERR_INVALID, "material count differs from the scene");
    if (tri_count && (!albedo || !emission)) return fail(QUASI_ERR_INVALID, "null materials");
    int rc = upload_materials_host(albedo, emission, tri_count);
    if (rc) return rc;
    return reset();
}

int Renderer::set_options(const Q_cuda_options& o) {
    Q_cuda_options n = o;
    if (n.spp_per_frame == 0) n.spp_per_frame = 1;
    if (n.max_depth == 0) n.max_depth = 4;
    if (n.max_depth > 64) return fail(QUASI_ERR_INVALID, "max_depth above 64");
    if (n.integrator > QUASI_INTEGRATOR_REFERENCE) return fail(QUASI_ERR_INVALID, "unknown integrator");
    if (!(n.ray_eps > 0.f)) n.ray_eps = 1e-4f;
    if (n.trace_block != 0 && (n.trace_block % 32 != 0 || n.trace_block > 256))
        return fail(QUASI_ERR_INVALID, "trace_block must be a multiple of 32 up to 256");
    const bool changed = n.seed != opt_.seed || n.max_depth != opt_.max_depth || n.integrator != opt_.integrator ||
                         n.ray_eps != opt_.ray_eps;
    opt_ = n;
    prof_.set_enabled(opt_.profile != 0);
    if (changed) return reset();
    return QUASI_OK;
}

int Renderer::reset() {
    samples_ = 0;
    frame_index_ = 0;
    if (accum_.ptr) {
        R_TRY(cudaMemsetAsync(accum_.ptr, 0, accum_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(comp_.ptr, 0, comp_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(aov_albedo_.ptr, 0, aov_albedo_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(aov_normal_.ptr, 0, aov_normal_.bytes, stream_), "memset");
    }
    return QUASI_OK;
}

int Renderer::ensure_frame_buffers(uint32_t w, uint32_t h) {
    if (w == width_ && h == height_ && accum_.ptr) return QUASI_OK;
    const size_t px = static_cast<size_t>(w) * h;
    accum_.release(); comp_.release(); aov_albedo_.release(); aov_normal_.release();
    R_TRY(accum_.reserve(sizeof(float4) * px), "accum");
    R_TRY(comp_.reserve(sizeof(float4) * px), "accum");
    R_TRY(aov_albedo_.reserve(sizeof(float4) * px), "accum");
    R_TRY(aov_normal_.reserve(sizeof(float4) * px), "accum");
    width_ = w;
    height_ = h;
    return reset();
}

int Renderer::ensure_wave_buffers(uint32_t paths) {
    if (paths <= wave_capacity_) return QUASI_OK;
    R_TRY(queue_[0].reserve(sizeof(float4) * 2ull * paths), "queue");
    R_TRY(queue_[1].reserve(sizeof(float4) * 2ull * paths), "queue");
    R_TRY(hits_.reserve(sizeof(float4) * paths), "hits");
    R_TRY(shadow_.reserve(sizeof(float4) * 3ull * paths), "shadow");
    R_TRY(beta_.reserve(sizeof(float4) * paths), "beta");
    R_TRY(lpath_.reserve(sizeof(float4) * paths), "lpath");
    R_TRY(aov_a_.reserve(sizeof(float4) * paths), "aov");
    R_TRY(aov_n_.reserve(sizeof(float4) * paths), "aov");
    R_TRY(sig_.reserve(sizeof(uint32_t) * paths), "sig");
    wave_capacity_ = paths;
    return QUASI_OK;
}

uint32_t Renderer::effective_wave_spp(uint32_t spp) const {
    if (opt_.wave_spp > 0) return std::min(opt_.wave_spp, spp);
    const uint32_t tiles = ceil_div(width_, 8) * ceil_div(height_, 4);
    const uint32_t slots = tiles * 32;
    const uint32_t target = 8u << 20;  // ~8M paths per wave
    return std::max<uint32_t>(1, std::min<uint32_t>(spp, target / std::max<uint32_t>(slots, 1)));
}

int Renderer::render(const Q_render_frame& fr) {
    error_.clear();
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (fr.width == 0 || fr.height == 0) return fail(QUASI_ERR_INVALID, "zero-sized frame");
    if (static_cast<uint64_t>(fr.width) * fr.height > (1ull << 26)) return fail(QUASI_ERR_INVALID, "frame too large");
    if (fr.command_buffer) stream_ = static_cast<cudaStream_t>(fr.command_buffer);
    cudaStream_t s = stream_;
    int rc = ensure_frame_buffers(fr.width, fr.height);
    if (rc) return rc;
    if (fr.camera_dirty) {
        rc = reset();
        if (rc) return rc;
    }
    camera_ = fr.camera;
    prof_.reset_launches();
    R_TRY(cudaEventRecord(ev_frame0_, s), "event");
    bvh_timed_ = false;
    if (opt_.integrator == QUASI_INTEGRATOR_NEE && (bvh_dirty_ || opt_.rebuild_each_frame)) {
        R_TRY(cudaEventRecord(ev_bvh0_, s), "event");
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, s, prof_, err_dev_.as<uint32_t>()), "lbvh build");
        R_TRY(cudaEventRecord(ev_bvh1_, s), "event");
        bvh_timed_ = true;
        bvh_dirty_ = false;
    }
    const uint32_t spp = opt_.spp_per_frame;
    if (opt_.record_samples) {
        const size_t n = static_cast<size_t>(width_) * height_ * spp;
        R_TRY(record_rad_.reserve(sizeof(float) * 3 * n), "record");
        R_TRY(record_sig_.reserve(sizeof(uint32_t) * n), "record");
        record_spp_ = spp;
    }
    if (opt_.integrator == QUASI_INTEGRATOR_REFERENCE) rc = render_reference(s, spp);
    else rc = render_wavefront(s, spp);
    if (rc) return rc;
    samples_ += spp;
    total_samples_ += spp;
    ++frame_index_;
    R_TRY(cudaEventRecord(ev_frame1_, s), "event");
    frame_timed_ = true;
    if (fr.drawable) {
        const uint32_t px = width_ * height_;
        R_TRY(QUASI_LAUNCH(prof_, "tonemap", s,
                           (k_tonemap<<<ceil_div(px, 256), 256, 0, s>>>(accum_.as<float4>(), px, float(samples_),
                                                                       static_cast<uchar4*>(fr.drawable)))),
              "tonemap");
    }
    return QUASI_OK;
}

int Renderer::render_wavefront(cudaStream_t s, uint32_t spp) {
    const uint32_t D = opt_.max_depth;
    const uint32_t tiles_x = ceil_div(width_, 8), tiles_y = ceil_div(height_, 4);
    const uint32_t slots = tiles_x * tiles_y * 32;
    const uint32_t S = effective_wave_spp(spp);
    const uint32_t waves = ceil_div(spp, S);
    int rc = ensure_wave_buffers(slots * S);
    if (rc) return rc;
    const uint32_t per_wave = 4 * D;
    const uint32_t need = per_wave * waves;
    if (need > counter_capacity_) {
        R_TRY(counters_.reserve(sizeof(int) * need), "counters");
        if (counters_host_) cudaFreeHost(counters_host_);
        R_TRY(cudaMallocHost(&counters_host_, sizeof(int) * need), "pinned");
        counter_capacity_ = need;
    }
    counters_used_ = need;
    R_TRY(cudaMemsetAsync(counters_.ptr, 0, sizeof(int) * need, s), "memset");
    if (opt_.collect_stats) R_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, sizeof(unsigned long long) * 4, s), "memset");

    const LbvhView bv = bvh_.view();
    SceneDev sd{tri_in_.as<float4>(), albedo_.as<float4>(), emission_.as<float4>(), emitters_.as<int>(),
                bv.nodes, bv.tris, n_tris_, n_emit_};
    PathDev pd{beta_.as<float4>(), lpath_.as<float4>(), aov_a_.as<float4>(), aov_n_.as<float4>(),
               opt_.record_samples ? sig_.as<uint32_t>() : nullptr};
    FrameParams f{};
    f.cam = make_camera_basis(camera_, width_, height_);
    f.width = width_;
    f.height = height_;
    f.tiles_x = tiles_x;
    f.slots = slots;
    f.seed = opt_.seed;
    f.max_depth = D;
    f.eps = opt_.ray_eps;
    f.frame_spp = spp;

    const int tb = opt_.trace_block ? static_cast<int>(opt_.trace_block) : 128;
    int occ_c = 0, occ_s = 0;
    if (opt_.collect_stats) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, k_trace_closest<true>, tb, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_trace_shadow<true>, tb, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, k_trace_closest<false>, tb, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_trace_shadow<false>, tb, 0);
    }
    const int grid_c = sm_count_ * std::max(occ_c, 1);
    const int grid_s = sm_count_ * std::max(occ_s, 1);
    const int grid_shade = sm_count_ * 8;
    uint32_t* err = err_dev_.as<uint32_t>();
    unsigned long long* st = stats_dev_.as<unsigned long long>();
    const uint32_t px = width_ * height_;
    const int cap = static_cast<int>(slots * S);

    for (uint32_t w = 0; w < waves; ++w) {
        const uint32_t Sw = std::min(S, spp - w * S);
        f.wave_spp = Sw;
        f.sample_base = samples_ + w * S;
        f.wave_offset = w * S;
        int* cnt = counters_.as<int>() + w * per_wave;
        R_TRY(QUASI_LAUNCH(prof_, "camera", s,
                           (k_camera<<<ceil_div(Sw * slots, 256), 256, 0, s>>>(f, pd, queue_[0].as<float4>(), cnt))),
              "camera");
        for (uint32_t k = 1; k <= D; ++k) {
            float4* qcur = queue_[(k - 1) & 1].as<float4>();
            float4* qnext = queue_[k & 1].as<float4>();
            int* c_cur = cnt + (k - 1);
            int* c_next = cnt + k;  // unused when k == D (index D is the first shadow counter, never appended)
            int* c_shadow = cnt + D + (k - 1);
            int* f_cur = cnt + 2 * D + (k - 1);
            int* f_shadow = cnt + 3 * D + (k - 1);
            if (opt_.collect_stats)
                R_TRY(QUASI_LAUNCH(prof_, "trace_closest", s,
                                   (k_trace_closest<true><<<grid_c, tb, 0, s>>>(sd, qcur, hits_.as<float4>(), c_cur,
                                                                                cap, f_cur, err, st))),
                      "trace_closest");
            else
                R_TRY(QUASI_LAUNCH(prof_, "trace_closest", s,
                                   (k_trace_closest<false><<<grid_c, tb, 0, s>>>(sd, qcur, hits_.as<float4>(), c_cur,
                                                                                 cap, f_cur, err, st))),
                      "trace_closest");
            R_TRY(QUASI_LAUNCH(prof_, "shade", s,
                               (k_shade<<<grid_shade, 256, 0, s>>>(f, sd, pd, k, qcur, hits_.as<float4>(), c_cur, cap, qnext,
                                                                  k < D ? c_next : nullptr, shadow_.as<float4>(),
                                                                  c_shadow))),
                  "shade");
            if (opt_.collect_stats)
                R_TRY(QUASI_LAUNCH(prof_, "trace_shadow", s,
                                   (k_trace_shadow<true><<<grid_s, tb, 0, s>>>(sd, pd, shadow_.as<float4>(), c_shadow,
                                                                               cap, f_shadow, err, st))),
                      "trace_shadow");
            else
                R_TRY(QUASI_LAUNCH(prof_, "trace_shadow", s,
                                   (k_trace_shadow<false><<<grid_s, tb, 0, s>>>(sd, pd, shadow_.as<float4>(), c_shadow,
                                                                                cap, f_shadow, err, st))),
                      "trace_shadow");
        }
        R_TRY(QUASI_LAUNCH(prof_, "accumulate", s,
                           (k_accumulate<<<ceil_div(px, 256), 256, 0, s>>>(
                               f, pd, accum_.as<float4>(), comp_.as<float4>(), aov_albedo_.as<float4>(),
                               aov_normal_.as<float4>(), opt_.record_samples ? record_rad_.as<float>() : nullptr,
                               opt_.record_samples ? record_sig_.as<uint32_t>() : nullptr))),
              "accumulate");
    }
    R_TRY(QUASI_LAUNCH(prof_, "tally", s, (k_tally<<<1, 32, 0, s>>>(counters_.as<int>(), waves, D, st))), "tally");
    R_TRY(cudaMemcpyAsync(counters_host_, counters_.ptr, sizeof(int) * need, cudaMemcpyDeviceToHost, s), "d2h");
    R_TRY(cudaMemcpyAsync(stats_host_, stats_dev_.ptr, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost, s), "d2h");
    R_TRY(cudaMemcpyAsync(err_host_, err_dev_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "d2h");
    stats_pending_ = true;
    return QUASI_OK;
}

int Renderer::render_megakernel(cudaStream_t, uint32_t) { return fail(QUASI_ERR_INVALID, "megakernel not built"); }

int Renderer::render_reference(cudaStream_t s, uint32_t spp) {
    if (n_quads_ == 0) return fail(QUASI_ERR_STATE, "reference integrator needs quads");
    R_TRY(launch_reference_frame(quads_.as<float4>(), n_quads_, camera_, width_, height_, samples_, spp,
                                 accum_.as<float4>(), comp_.as<float4>(), aov_albedo_.as<float4>(),
                                 aov_normal_.as<float4>(), s, prof_),
          "reference frame");
    counters_used_ = 0;
    stats_pending_ = false;
    return QUASI_OK;
}

int Renderer::synchronize() {
    R_TRY(cudaStreamSynchronize(stream_), "synchronize");
    return QUASI_OK;
}

int Renderer::resolve_device(float* device_rgba) {
    if (!accum_.ptr) return fail(QUASI_ERR_STATE, "nothing rendered");
    const uint32_t px = width_ * height_;
    R_TRY(QUASI_LAUNCH(prof_, "resolve", stream_,
                       (k_resolve<<<ceil_div(px, 256), 256, 0, stream_>>>(accum_.as<float4>(), aov_albedo_.as<float4>(),
                                                                         aov_normal_.as<float4>(), px, float(samples_), 0,
                                                                         reinterpret_cast<float4*>(device_rgba)))),
          "resolve");
    return QUASI_OK;
}

int Renderer::resolve_host(float* beauty, float* albedo, float* normal, float* depth) {
    if (!accum_.ptr) return fail(QUASI_ERR_STATE, "nothing rendered");
    const uint32_t px = width_ * height_;
    DeviceBuffer tmp;
    R_TRY(tmp.reserve(sizeof(float4) * px), "resolve buffer");
    float* outs[4] = {beauty, albedo, normal, depth};
    for (int mode = 0; mode < 4; ++mode) {
        if (!outs[mode]) continue;
        cudaError_t e = QUASI_LAUNCH(prof_, "resolve", stream_,
                                     (k_resolve<<<ceil_div(px, 256), 256, 0, stream_>>>(
                                         accum_.as<float4>(), aov_albedo_.as<float4>(), aov_normal_.as<float4>(), px,
                                         float(samples_), mode, tmp.as<float4>())));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(outs[mode], tmp.ptr, sizeof(float4) * px, cudaMemcpyDeviceToHost, stream_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
        if (e != cudaSuccess) {
            tmp.release();
            return cuda_fail(e, "resolve");
        }
    }
    tmp.release();
    return QUASI_OK;
}

int Renderer::read_samples(float* radiance, uint32_t* signatures) {
    if (!opt_.record_samples || !record_rad_.ptr) return fail(QUASI_ERR_STATE, "record_samples was off");
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    const size_t n = static_cast<size_t>(width_) * height_ * record_spp_;
    if (radiance) R_TRY(cudaMemcpy(radiance, record_rad_.ptr, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost), "d2h");
    if (signatures) R_TRY(cudaMemcpy(signatures, record_sig_.ptr, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost), "d2h");
    return QUASI_OK;
}

int Renderer::read_bvh(uint32_t* morton, uint32_t* order, int32_t* children, float* boxes, float* bounds) {
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (bvh_dirty_) {
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, stream_, prof_, err_dev_.as<uint32_t>()), "lbvh build");
        bvh_dirty_ = false;
    }
    R_TRY(bvh_.read(morton, order, children, boxes, bounds, stream_), "read bvh");
    return QUASI_OK;
}

int Renderer::stats(Q_cuda_stats* out) {
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    Q_cuda_stats st{};
    if (stats_pending_) {
        const uint32_t D = opt_.max_depth;
        const uint32_t per_wave = 4 * D;
        const uint32_t waves = per_wave ? counters_used_ / per_wave : 0;
        for (uint32_t w = 0; w < waves; ++w) {
            const int* c = counters_host_ + w * per_wave;
            st.camera_rays += static_cast<uint64_t>(c[0]);
            for (uint32_t k = 1; k < D; ++k) st.extension_rays += static_cast<uint64_t>(c[k]);
            for (uint32_t k = 0; k < D; ++k) st.shadow_rays += static_cast<uint64_t>(c[D + k]);
        }
        if (opt_.collect_stats) {
            st.node_visits = stats_host_[0];
            st.tri_tests = stats_host_[1];
            st.shadow_node_visits = stats_host_[2];
            st.shadow_tri_tests = stats_host_[3];
        }
        last_stats_ = st;
    } else {
        st = last_stats_;
    }
    st.total_rays = stats_host_[4];
    st.samples_accumulated = samples_;
    st.kernel_launches = prof_.launches();
    st.error_flags = err_host_ ? *err_host_ : 0u;
    float ms = 0.f;
    if (frame_timed_ && cudaEventElapsedTime(&ms, ev_frame0_, ev_frame1_) == cudaSuccess) st.frame_ms = ms;
    if (bvh_timed_ && cudaEventElapsedTime(&ms, ev_bvh0_, ev_bvh1_) == cudaSuccess) st.bvh_ms = ms;
    prof_.collect();
    *out = st;
    return QUASI_OK;
}

int Renderer::kernel_times(Q_cuda_kernel_time* out, uint32_t capacity, uint32_t* count) {
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    prof_.collect();
    const auto& t = prof_.totals();
    uint32_t i = 0;
    for (const auto& kv : t) {
        if (out && i < capacity) {
            std::memset(out[i].name, 0, sizeof(out[i].name));
            std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
            out[i].launches = kv.second.first;
            out[i].total_ms = kv.second.second;
        }
        ++i;
    }
    if (count) *count = i;
    if (!out && !count) prof_.reset_totals();  // (NULL, 0, NULL) clears the totals
    return QUASI_OK;
}

int Renderer::autotune(double) { return fail(QUASI_ERR_INVALID, "autotuner not built"); }

}  // namespace quasi
