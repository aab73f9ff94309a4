// common.cuh - device math, RNG and sampling conventions shared by every kernel.
//
// Conventions (the oracle restates each of them independently):
//  * pcg_hash / rng_next follow backends/metal/plugin.mm:98-107: a 32-bit PCG output hash,
//    and float(state)/float(0xFFFFFFFF) which equals float(state)*2^-32 (it may be 1.0).
//  * A path vertex's random stream is keyed on (seed, pixel, sample, bounce):
//    key = pcg(pcg(pcg(seed ^ pixel) + sample) + bounce); draws then chain with pcg.
//  * cosine_sample follows plugin.mm:111-125 including its orthonormal-basis choice.
//  * The pinhole camera follows plugin.mm:129-153 / src/quasi/scene/camera.hpp:36-52; its
//    basis is precomputed on the host (in double) instead of per ray.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace quasi {

constexpr float k_pi = 3.14159265358979323846f;
constexpr float k_inv_pi = 0.318309886183790671538f;

__host__ __device__ __forceinline__ float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__host__ __device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize(float3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__device__ __forceinline__ float max3(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
__device__ __forceinline__ float3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }

// plugin.mm:98-102 (PCG output permutation, O'Neill 2014; constants as in the reference).
__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// plugin.mm:104-107. float(0xFFFFFFFFu) rounds to 2^32, so the quotient is exact scaling.
__device__ __forceinline__ float rng_next(uint32_t& state) {
    state = pcg_hash(state);
    return __uint2float_rn(state) * 0x1p-32f;
}

__host__ __device__ __forceinline__ uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample,
                                                      uint32_t bounce) {
    return pcg_hash(pcg_hash(pcg_hash(seed ^ pixel) + sample) + bounce);
}

// Path signature: a running hash of the primitives hit and the shadow-ray outcomes. The
// oracle computes the same value, which identifies paths whose branch decisions differ.
__host__ __device__ __forceinline__ uint32_t sig_mix(uint32_t sig, uint32_t v) { return pcg_hash(sig ^ v) + v; }
constexpr uint32_t k_sig_miss = 0xFFFFFFFFu;
constexpr uint32_t k_sig_lit = 0xFFFFFFF1u;
constexpr uint32_t k_sig_shadowed = 0xFFFFFFF2u;
constexpr uint32_t k_sig_no_nee = 0xFFFFFFF3u;

// plugin.mm:111-125: cosine-weighted direction about `normal`.
__device__ __forceinline__ float3 cosine_sample(float3 normal, float r1, float r2) {
    float sphi, cphi;
    sincospif(2.0f * r1, &sphi, &cphi);
    const float cos_theta = sqrtf(1.0f - r2);
    const float sin_theta = sqrtf(r2);
    const float3 w = normalize(normal);
    const float3 a = (fabsf(w.x) > 0.9f) ? mk3(0.f, 1.f, 0.f) : mk3(1.f, 0.f, 0.f);
    const float3 v = normalize(cross(w, a));
    const float3 u = cross(w, v);
    return normalize(u * (cphi * sin_theta) + v * (sphi * sin_theta) + w * cos_theta);
}

// Pinhole camera, plugin.mm:129-153 with the per-ray basis hoisted to the host.
struct CameraBasis {
    float3 origin;
    float3 lower_left;   // position - horizontal/2 - vertical/2 - w
    float3 horizontal;   // viewport_width * right
    float3 vertical;     // viewport_height * up'
};

__device__ __forceinline__ float3 camera_dir(const CameraBasis& c, float u, float v) {
    return normalize(c.lower_left + c.horizontal * u + c.vertical * v - c.origin);
}

// Device-side error bits (mirrors QUASI_DEVERR_* in quasi_cuda.h).
constexpr uint32_t k_deverr_stack = 1u;
constexpr uint32_t k_deverr_timeout = 2u;
constexpr uint32_t k_deverr_traversal = 4u;  // a traversal or tree climb exceeded its bound

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Appends one element per participating lane to a queue whose length lives at *counter;
// one atomic per warp (ballot + popc). All lanes of `mask` must call it.
__device__ __forceinline__ int warp_append(uint32_t mask, bool want, int* counter) {
    const uint32_t ballot = __ballot_sync(mask, want);
    if (ballot == 0) return -1;
    const int leader = __ffs(ballot) - 1;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return want ? base + __popc(ballot & lanemask_lt()) : -1;
}

// Reserves queue slots for the threads of a block that want one, with one atomic per block:
// warp counts by ballot, a scan over the warps in warp 0, one atomicAdd. Every thread of the
// block calls it (it has two barriers); the block size is a multiple of 32. Returns the
// thread's slot, or -1 when it wants none. One atomic per block instead of one per warp:
// every block of a launch appends to the same counter, and same-address atomics are served
// one at a time by the L2 slice that holds the address.
__device__ __forceinline__ int block_append(bool want, int* counter) {
    __shared__ int s_count[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ballot = __ballot_sync(0xffffffffu, want);
    if (lane == 0) s_count[warp] = __popc(ballot);
    __syncthreads();
    if (warp == 0) {
        const int nw = static_cast<int>(blockDim.x >> 5);
        const int c = lane < nw ? s_count[lane] : 0;
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int base = 0;
        if (lane == 0 && total > 0) base = atomicAdd(counter, total);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (lane < nw) s_count[lane] = base + incl - c;
    }
    __syncthreads();
    return want ? s_count[warp] + __popc(ballot & lanemask_lt()) : -1;
}

}  // namespace quasi
