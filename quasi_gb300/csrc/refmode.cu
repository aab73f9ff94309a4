// refmode.cu - the reference integrator: backends/metal/plugin.mm:98-309 restated in CUDA.
//
// Brute-force quads (at most 32, plugin.mm:21), the reference's seeding
// rng = pcg_hash(px + py*1920 + frame*1920*1080) (plugin.mm:295) where `frame` is the
// global sample index, uv jitter of +-0.0005 (plugin.mm:131-132), at most 5 bounces,
// emission added then the path stops at an emitter (plugin.mm:252-258), Russian roulette
// after bounce 2 (plugin.mm:264-268) and the first-hit AOVs (plugin.mm:242-249, 301-307).
// Per pixel the kernel Kahan-adds its samples in order, so the mean equals the reference's
// running mix() average up to FP32 rounding.
#include "common.cuh"
#include "launch.hpp"
#include "../../include/quasi_cuda.h"

#include <cmath>

namespace quasi {

constexpr uint32_t k_ref_max_quads = 32;
constexpr int k_ref_max_bounces = 5;

struct RefCamera {  // plugin.mm:48-55 (direction normalised on the host, plugin.mm:653-659)
    float3 position;
    float fov;
    float3 direction;
    float aspect;
    float3 up;
};

struct RefHit {
    float t;
    float3 point;
    float3 normal;
    int index;
};

__device__ __forceinline__ float ref_random(uint32_t& s) {  // plugin.mm:104-107
    s = pcg_hash(s);
    return __uint2float_rn(s) / 4294967296.0f;
}

__device__ __forceinline__ float3 ref_normalize(float3 v) { return v * rsqrtf(dot(v, v)); }

__device__ float3 ref_cosine_sample(float3 normal, uint32_t& rng) {  // plugin.mm:111-125
    const float r1 = ref_random(rng);
    const float r2 = ref_random(rng);
    const float phi = 2.0f * k_pi * r1;
    const float cos_theta = sqrtf(1.0f - r2);
    const float sin_theta = sqrtf(r2);
    const float3 w = ref_normalize(normal);
    const float3 a = (fabsf(w.x) > 0.9f) ? mk3(0.f, 1.f, 0.f) : mk3(1.f, 0.f, 0.f);
    const float3 v = ref_normalize(cross(w, a));
    const float3 u = cross(w, v);
    return ref_normalize(u * cosf(phi) * sin_theta + v * sinf(phi) * sin_theta + w * cos_theta);
}

__device__ void ref_camera_ray(const RefCamera& cam, float ux, float uy, uint32_t& rng, float3& o,
                               float3& d) {  // plugin.mm:129-153
    const float jx = ref_random(rng) - 0.5f;  // the reference builds float2(r(), r()) left to right
    const float jy = ref_random(rng) - 0.5f;
    ux += jx * 0.001f;
    uy += jy * 0.001f;
    const float theta = cam.fov * k_pi / 180.0f;
    const float h = tanf(theta / 2.0f);
    const float vh = 2.0f * h;
    const float vw = cam.aspect * vh;
    const float3 w = ref_normalize(-cam.direction);
    const float3 right = ref_normalize(cross(cam.up, w));
    const float3 up = cross(w, right);
    const float3 horizontal = right * vw;
    const float3 vertical = up * vh;
    const float3 lower_left = cam.position - horizontal * 0.5f - vertical * 0.5f - w;
    const float3 target = lower_left + horizontal * ux + vertical * uy;
    o = cam.position;
    d = ref_normalize(target - cam.position);
}

// plugin.mm:157-195
__device__ __forceinline__ bool ref_intersect_quad(float3 ro, float3 rd, float3 qo, float3 qu, float3 qv, float tmin,
                                                   float tmax, RefHit& rec, int idx) {
    const float3 n = cross(qu, qv);
    const float area_sq = dot(n, n);
    if (area_sq < 1e-8f) return false;
    const float3 normal = n * rsqrtf(area_sq);
    const float dd = dot(normal, qo);
    const float denom = dot(normal, rd);
    if (fabsf(denom) < 1e-8f) return false;
    const float t = (dd - dot(normal, ro)) / denom;
    if (t < tmin || t > tmax) return false;
    const float3 p = ro + rd * t;
    const float3 planar = p - qo;
    const float3 w = n * (1.0f / area_sq);
    const float alpha = dot(w, cross(planar, qv));
    const float beta = dot(w, cross(qu, planar));
    if (alpha < 0.0f || alpha > 1.0f || beta < 0.0f || beta > 1.0f) return false;
    rec.t = t;
    rec.point = p;
    rec.index = idx;
    rec.normal = (denom < 0.0f) ? normal : -normal;
    return true;
}

__global__ void __launch_bounds__(128) k_reference(const float4* __restrict__ quads, uint32_t n_quads, RefCamera cam,
                                                   uint32_t width, uint32_t height, uint32_t sample_base, uint32_t spp,
                                                   float4* __restrict__ accum, float4* __restrict__ comp,
                                                   float4* __restrict__ aov_a, float4* __restrict__ aov_n) {
    __shared__ float4 sq[5 * k_ref_max_quads];
    const uint32_t nq = min(n_quads, k_ref_max_quads);
    for (uint32_t i = threadIdx.x; i < 5 * nq; i += blockDim.x) sq[i] = quads[i];
    __syncthreads();
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= width * height) return;
    const uint32_t py = pixel / width, px = pixel - py * width;
    float4 sum = accum[pixel], c = comp[pixel], A = aov_a[pixel], N = aov_n[pixel];
    const float ux = (static_cast<float>(px) + 0.5f) / static_cast<float>(width);
    const float uy = 1.0f - (static_cast<float>(py) + 0.5f) / static_cast<float>(height);
    for (uint32_t s = 0; s < spp; ++s) {
        const uint32_t frame = sample_base + s;
        uint32_t rng = pcg_hash(px + py * 1920u + frame * 1920u * 1080u);
        float3 ro, rd;
        ref_camera_ray(cam, ux, uy, rng, ro, rd);
        float3 color = mk3(0.f, 0.f, 0.f), tp = mk3(1.f, 1.f, 1.f);
        float3 fa = color, fn = color;
        float fd = 0.f;
        for (int bounce = 0; bounce < k_ref_max_bounces; ++bounce) {
            RefHit closest;
            closest.t = 1e30f;
            bool hit = false;
            for (uint32_t i = 0; i < nq; ++i) {
                RefHit h;
                if (ref_intersect_quad(ro, rd, xyz(sq[5 * i]), xyz(sq[5 * i + 1]), xyz(sq[5 * i + 2]), 0.001f,
                                       closest.t, h, static_cast<int>(i))) {
                    closest = h;
                    hit = true;
                }
            }
            if (!hit) break;
            const float3 alb = xyz(sq[5 * closest.index + 3]);
            const float3 em = xyz(sq[5 * closest.index + 4]);
            const float es = fmaxf(em.x, fmaxf(em.y, em.z));
            if (bounce == 0) {
                fa = es > 0.1f ? em : alb;
                fn = closest.normal * 0.5f + mk3(0.5f, 0.5f, 0.5f);
                fd = closest.t;
            }
            color = color + tp * em;
            if (es > 0.1f) break;
            tp = tp * alb;
            if (bounce > 2) {
                const float p = fmaxf(0.05f, fmaxf(tp.x, fmaxf(tp.y, tp.z)));
                if (ref_random(rng) > p) break;
                tp = tp * (1.0f / p);
            }
            ro = closest.point + closest.normal * 0.001f;
            rd = ref_cosine_sample(closest.normal, rng);
        }
        const float depth = fminf(fmaxf((fd - 1.0f) / 4.0f, 0.0f), 1.0f);
        float y = color.x - c.x, t = sum.x + y; c.x = (t - sum.x) - y; sum.x = t;
        y = color.y - c.y; t = sum.y + y; c.y = (t - sum.y) - y; sum.y = t;
        y = color.z - c.z; t = sum.z + y; c.z = (t - sum.z) - y; sum.z = t;
        A.x += fa.x; A.y += fa.y; A.z += fa.z; A.w += depth;
        N.x += fn.x; N.y += fn.y; N.z += fn.z;
    }
    accum[pixel] = sum;
    comp[pixel] = c;
    aov_a[pixel] = A;
    aov_n[pixel] = N;
}

cudaError_t launch_reference_frame(const float4* quads, uint32_t n_quads, const Q_camera& qc, uint32_t width,
                                   uint32_t height, uint32_t sample_base, uint32_t spp, float4* accum, float4* comp,
                                   float4* aov_a, float4* aov_n, cudaStream_t s, KernelProfiler& prof) {
    // plugin.mm:649-674: direction = normalize(target - position) in float on the host.
    float dx = qc.target[0] - qc.position[0];
    float dy = qc.target[1] - qc.position[1];
    float dz = qc.target[2] - qc.position[2];
    const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (len > 0.0f) {
        dx /= len;
        dy /= len;
        dz /= len;
    }
    RefCamera cam;
    cam.position = make_float3(qc.position[0], qc.position[1], qc.position[2]);
    cam.fov = qc.fov;
    cam.direction = make_float3(dx, dy, dz);
    cam.aspect = static_cast<float>(width) / static_cast<float>(height);
    cam.up = make_float3(qc.up[0], qc.up[1], qc.up[2]);
    const uint32_t px = width * height;
    return QUASI_LAUNCH(prof, "reference_pathtrace", s,
                        (k_reference<<<(px + 127) / 128, 128, 0, s>>>(quads, n_quads, cam, width, height, sample_base,
                                                                     spp, accum, comp, aov_a, aov_n)));
}

}  // namespace quasi
