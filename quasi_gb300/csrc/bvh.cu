// bvh.cu - GPU LBVH construction: leaf references (split triangle boxes), centroid bounds,
// Morton-30 codes, stable LSD radix sort, Karras (2012) hierarchy and bottom-up child boxes.
// All FP32 arithmetic feeding integer results uses round-to-nearest intrinsics so the
// compiler cannot contract it, which keeps Morton codes, the sort order and the topology
// bit-exact against the oracle when no triangle is split.
#include "bvh.cuh"
#include "common.cuh"
#include "ffmath.cuh"
#include "wide.cuh"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

namespace quasi {
namespace {

constexpr int k_sort_block = 256;
constexpr int k_sort_items = 8;
constexpr int k_sort_tile = k_sort_block * k_sort_items;
constexpr int k_sort_warps = k_sort_block / 32;

// ---------------------------------------------------------------- radix sort (8-bit digits)

__global__ void __launch_bounds__(k_sort_block)
k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift, uint32_t* __restrict__ hist,
             uint32_t nblocks) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += k_sort_block) h[i] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * k_sort_tile;
#pragma unroll
    for (int r = 0; r < k_sort_items; ++r) {
        const uint32_t i = base + r * k_sort_block + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += k_sort_block) hist[d * nblocks + blockIdx.x] = h[d];
}

// Exclusive scan of m entries in one block of 1024 threads (m is at most a few million).
__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t* data, uint32_t m) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t per = (m + 1023u) / 1024u;
    const uint32_t begin = min(threadIdx.x * per, m);
    const uint32_t end = min(begin + per, m);
    uint32_t sum = 0;
    for (uint32_t i = begin; i < end; ++i) sum += data[i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        warp_sums[lane] = v;
    }
    __syncthreads();
    uint32_t prefix = x - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
    for (uint32_t i = begin; i < end; ++i) {
        const uint32_t t = data[i];
        data[i] = prefix;
        prefix += t;
    }
}

// Stable scatter. Warp w of a block owns the contiguous sub-tile [w*256, (w+1)*256) of the
// block's 2048 keys and walks it in 8 rounds of 32; ranks inside a round come from
// __match_any_sync, ranks across rounds from per-warp digit counters, and ranks across
// warps from a per-digit prefix over the warps' counters.
__global__ void __launch_bounds__(k_sort_block)
k_radix_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n, int shift,
                const uint32_t* __restrict__ hist, uint32_t nblocks) {
    __shared__ uint32_t warp_cnt[k_sort_warps][256];
    __shared__ uint32_t block_off[256];
    for (int i = threadIdx.x; i < k_sort_warps * 256; i += k_sort_block) (&warp_cnt[0][0])[i] = 0;
    for (int d = threadIdx.x; d < 256; d += k_sort_block) block_off[d] = hist[d * nblocks + blockIdx.x];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    const uint32_t warp_base = blockIdx.x * k_sort_tile + warp * 32 * k_sort_items;
    uint32_t key[k_sort_items], val[k_sort_items], rank[k_sort_items];
#pragma unroll
    for (int r = 0; r < k_sort_items; ++r) {
        const uint32_t i = warp_base + r * 32 + lane;
        const bool valid = i < n;
        key[r] = valid ? keys_in[i] : 0u;
        val[r] = valid ? vals_in[i] : 0u;
        const uint32_t d = (key[r] >> shift) & 255u;
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 256u + lane);
        const uint32_t before = __popc(peers & lt);
        uint32_t cnt = 0;
        if (valid) cnt = warp_cnt[warp][d];
        __syncwarp();
        if (valid && before == 0) warp_cnt[warp][d] = cnt + __popc(peers);
        __syncwarp();
        rank[r] = valid ? cnt + before : 0xffffffffu;
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += k_sort_block) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < k_sort_warps; ++w) {
            const uint32_t c = warp_cnt[w][d];
            warp_cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < k_sort_items; ++r) {
        if (rank[r] == 0xffffffffu) continue;
        const uint32_t d = (key[r] >> shift) & 255u;
        const uint32_t pos = block_off[d] + warp_cnt[warp][d] + rank[r];
        keys_out[pos] = key[r];
        vals_out[pos] = val[r];
    }
}

// ---------------------------------------------------------------- bounds and Morton codes

__device__ __forceinline__ float3 centroid(float4 a, float4 b, float4 c) {
    const float third = 1.0f / 3.0f;
    return mk3(__fmul_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), third),
               __fmul_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), third),
               __fmul_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), third));
}

// ---------------------------------------------------------------- leaf references
//
// The hierarchy's leaves are references to triangles. Without splitting, reference i is
// triangle i: its box is the bounds of its vertices and its Morton point is its centroid, bit
// for bit as the oracle builds them. With splitting (Ernst and Greiner 2007, "Early split
// clipping"), the S triangles whose boxes hold the most empty surface area are each cut in
// two at the middle of their box's longest axis: reference i keeps triangle i with the bounds
// of its part below the cut, reference n + k the part above it for the k-th of them. Every
// reference carries a box that contains its part of the triangle, so together they cover the
// whole triangle, and its Morton point is the centre of that box.

struct RefView {
    const uint32_t* tri = nullptr;  // reference -> triangle; null: reference i is triangle i
    const float4* box = nullptr;    // 2 float4 per reference: (lo, -), (hi, -)
};

__device__ __forceinline__ void tri_bounds(float4 a, float4 b, float4 c, float3& lo, float3& hi) {
    lo = mk3(fminf(a.x, fminf(b.x, c.x)), fminf(a.y, fminf(b.y, c.y)), fminf(a.z, fminf(b.z, c.z)));
    hi = mk3(fmaxf(a.x, fmaxf(b.x, c.x)), fmaxf(a.y, fmaxf(b.y, c.y)), fmaxf(a.z, fmaxf(b.z, c.z)));
}

// Triangle of reference r and the reference's box.
__device__ __forceinline__ uint32_t ref_geometry(const float4* __restrict__ tri_in, const RefView& rv, uint32_t r,
                                                 float3& lo, float3& hi) {
    if (!rv.tri) {
        tri_bounds(__ldg(&tri_in[3 * r]), __ldg(&tri_in[3 * r + 1]), __ldg(&tri_in[3 * r + 2]), lo, hi);
        return r;
    }
    const float4 l = __ldg(&rv.box[2 * r]), h = __ldg(&rv.box[2 * r + 1]);
    lo = mk3(l.x, l.y, l.z);
    hi = mk3(h.x, h.y, h.z);
    return __ldg(&rv.tri[r]);
}

// Morton point of reference r: the triangle's centroid, or the centre of a split reference's box.
__device__ __forceinline__ float3 ref_point(const float4* __restrict__ tri_in, const RefView& rv, uint32_t r) {
    if (!rv.tri) return centroid(__ldg(&tri_in[3 * r]), __ldg(&tri_in[3 * r + 1]), __ldg(&tri_in[3 * r + 2]));
    const float4 l = __ldg(&rv.box[2 * r]), h = __ldg(&rv.box[2 * r + 1]);
    return mk3(__fmul_rn(__fadd_rn(l.x, h.x), 0.5f), __fmul_rn(__fadd_rn(l.y, h.y), 0.5f),
               __fmul_rn(__fadd_rn(l.z, h.z), 0.5f));
}

// Sort key of triangle i for choosing the ones to split: the surface area of its box that
// the triangle leaves empty, 2 (dx dy + dy dz + dz dx) - 2 area, as the bits of a non-negative
// float (which order like the floats).
__global__ void __launch_bounds__(256) k_split_keys(const float4* __restrict__ tri_in, uint32_t n,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = __ldg(&tri_in[3 * i]), b = __ldg(&tri_in[3 * i + 1]), c = __ldg(&tri_in[3 * i + 2]);
    float3 lo, hi;
    tri_bounds(a, b, c, lo, hi);
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    const float3 e1 = mk3(b.x - a.x, b.y - a.y, b.z - a.z), e2 = mk3(c.x - a.x, c.y - a.y, c.z - a.z);
    const float3 cr = cross(e1, e2);
    const float empty = 2.0f * (dx * dy + dy * dz + dz * dx) - sqrtf(dot(cr, cr));
    keys[i] = __float_as_uint(empty > 0.0f ? empty : 0.0f);
    vals[i] = i;
}

// The part of triangle (a, b, c) on one side of the plane x_axis = cut (below: x <= cut):
// the bounds of its vertices on that side and of the points where its edges cross the plane,
// computed in FP64 and rounded outwards one float step beyond the directed rounding, so the
// box contains the part whatever the rounding of the crossing points.
__device__ void half_bounds(const float3 (&v)[3], int axis, float cut, bool below, float3& lo, float3& hi) {
    double l[3] = {1e300, 1e300, 1e300}, h[3] = {-1e300, -1e300, -1e300};
    auto grow = [&](double x, double y, double z) {
        l[0] = fmin(l[0], x); l[1] = fmin(l[1], y); l[2] = fmin(l[2], z);
        h[0] = fmax(h[0], x); h[1] = fmax(h[1], y); h[2] = fmax(h[2], z);
    };
    auto coord = [&](const float3& p) { return axis == 0 ? p.x : (axis == 1 ? p.y : p.z); };
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float3 p = v[k], q = v[(k + 1) % 3];
        const float cp = coord(p), cq = coord(q);
        if (below ? cp <= cut : cp >= cut) grow(p.x, p.y, p.z);
        if ((cp < cut && cq > cut) || (cp > cut && cq < cut)) {
            const double s = (static_cast<double>(cut) - cp) / (static_cast<double>(cq) - cp);
            double x = p.x + s * (static_cast<double>(q.x) - p.x);
            double y = p.y + s * (static_cast<double>(q.y) - p.y);
            double z = p.z + s * (static_cast<double>(q.z) - p.z);
            if (axis == 0) x = cut;
            else if (axis == 1) y = cut;
            else z = cut;
            grow(x, y, z);
        }
    }
    const float inf = __int_as_float(0x7f800000);
    lo = mk3(nextafterf(__double2float_rd(l[0]), -inf), nextafterf(__double2float_rd(l[1]), -inf),
             nextafterf(__double2float_rd(l[2]), -inf));
    hi = mk3(nextafterf(__double2float_ru(h[0]), inf), nextafterf(__double2float_ru(h[1]), inf),
             nextafterf(__double2float_ru(h[2]), inf));
}

// One thread per triangle in the order of k_split_keys' sort (ascending empty area): the last
// s of them are split, the others become one reference each (see RefView).
__global__ void __launch_bounds__(256) k_make_refs(const float4* __restrict__ tri_in, uint32_t n, uint32_t s,
                                                   const uint32_t* __restrict__ sorted_tris,
                                                   uint32_t* __restrict__ ref_tri, float4* __restrict__ ref_box) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t t = sorted_tris[p];
    const float4 a = __ldg(&tri_in[3 * t]), b = __ldg(&tri_in[3 * t + 1]), c = __ldg(&tri_in[3 * t + 2]);
    float3 lo, hi;
    tri_bounds(a, b, c, lo, hi);
    ref_tri[t] = t;
    if (p < n - s) {
        ref_box[2 * t] = make_float4(lo.x, lo.y, lo.z, 0.f);
        ref_box[2 * t + 1] = make_float4(hi.x, hi.y, hi.z, 0.f);
        return;
    }
    const uint32_t r2 = n + (p - (n - s));
    ref_tri[r2] = t;
    const float ext[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    const int axis = ext[0] >= ext[1] && ext[0] >= ext[2] ? 0 : (ext[1] >= ext[2] ? 1 : 2);
    const float l = axis == 0 ? lo.x : (axis == 1 ? lo.y : lo.z), h = axis == 0 ? hi.x : (axis == 1 ? hi.y : hi.z);
    const float cut = __fmul_rn(__fadd_rn(l, h), 0.5f);
    float3 lo1 = lo, hi1 = hi, lo2 = lo, hi2 = hi;
    if (cut > l && cut < h) {  // else (a box too thin to cut) both references keep the whole box
        const float3 v[3] = {mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z)};
        half_bounds(v, axis, cut, true, lo1, hi1);
        half_bounds(v, axis, cut, false, lo2, hi2);
        // never beyond the triangle's own box, nor across the cut
        lo1 = mk3(fmaxf(lo1.x, lo.x), fmaxf(lo1.y, lo.y), fmaxf(lo1.z, lo.z));
        hi1 = mk3(fminf(hi1.x, hi.x), fminf(hi1.y, hi.y), fminf(hi1.z, hi.z));
        lo2 = mk3(fmaxf(lo2.x, lo.x), fmaxf(lo2.y, lo.y), fmaxf(lo2.z, lo.z));
        hi2 = mk3(fminf(hi2.x, hi.x), fminf(hi2.y, hi.y), fminf(hi2.z, hi.z));
        if (axis == 0) { hi1.x = fminf(hi1.x, cut); lo2.x = fmaxf(lo2.x, cut); }
        else if (axis == 1) { hi1.y = fminf(hi1.y, cut); lo2.y = fmaxf(lo2.y, cut); }
        else { hi1.z = fminf(hi1.z, cut); lo2.z = fmaxf(lo2.z, cut); }
    }
    ref_box[2 * t] = make_float4(lo1.x, lo1.y, lo1.z, 0.f);
    ref_box[2 * t + 1] = make_float4(hi1.x, hi1.y, hi1.z, 0.f);
    ref_box[2 * r2] = make_float4(lo2.x, lo2.y, lo2.z, 0.f);
    ref_box[2 * r2 + 1] = make_float4(hi2.x, hi2.y, hi2.z, 0.f);
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(256) k_bounds_partial(const float4* __restrict__ tri, RefView rv, uint32_t n,
                                                        float* __restrict__ partial) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float3 c = ref_point(tri, rv, i);
        lo[0] = fminf(lo[0], c.x); lo[1] = fminf(lo[1], c.y); lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x); hi[1] = fmaxf(hi[1], c.y); hi[2] = fmaxf(hi[2], c.z);
    }
    __shared__ float s[8][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < 3; ++a) { lo[a] = warp_min(lo[a]); hi[a] = warp_max(hi[a]); }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) { s[warp][a] = lo[a]; s[warp][3 + a] = hi[a]; }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        float v = s[0][threadIdx.x];
        for (int w = 1; w < 8; ++w) v = threadIdx.x < 3 ? fminf(v, s[w][threadIdx.x]) : fmaxf(v, s[w][threadIdx.x]);
        partial[blockIdx.x * 6 + threadIdx.x] = v;
    }
}

__global__ void k_bounds_final(const float* __restrict__ partial, int nparts, float* __restrict__ bounds) {
    const int lane = threadIdx.x;
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int p = lane; p < nparts; p += 32) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], partial[p * 6 + a]);
            hi[a] = fmaxf(hi[a], partial[p * 6 + 3 + a]);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) { lo[a] = warp_min(lo[a]); hi[a] = warp_max(hi[a]); }
    if (lane == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            bounds[a] = lo[a];
            bounds[3 + a] = hi[a];
            const float ext = __fsub_rn(hi[a], lo[a]);
            bounds[6 + a] = ext > 0.0f ? __fdiv_rn(1.0f, ext) : 0.0f;
        }
        bounds[9] = bounds[10] = bounds[11] = 0.0f;
    }
}

// Spreads the low 10 bits of v to every third bit (bit k -> bit 3k).
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t quantize10(float c, float lo, float inv) {
    const float q = fminf(fmaxf(__fmul_rn(__fmul_rn(__fsub_rn(c, lo), inv), 1024.0f), 0.0f), 1023.0f);
    return static_cast<uint32_t>(q);
}

__global__ void __launch_bounds__(256) k_morton(const float4* __restrict__ tri, RefView rv, uint32_t n,
                                                const float* __restrict__ bounds, uint32_t* __restrict__ morton,
                                                uint32_t* __restrict__ keys, uint32_t* __restrict__ order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 c = ref_point(tri, rv, i);
    const uint32_t qx = quantize10(c.x, bounds[0], bounds[6]);
    const uint32_t qy = quantize10(c.y, bounds[1], bounds[7]);
    const uint32_t qz = quantize10(c.z, bounds[2], bounds[8]);
    const uint32_t code = (spread3(qx) << 2) | (spread3(qy) << 1) | spread3(qz);
    morton[i] = code;
    keys[i] = code;
    order[i] = i;
}

// ---------------------------------------------------------------- Karras hierarchy

// Common-prefix length of sorted keys i and j, index-augmented for equal keys; -1 outside.
__device__ __forceinline__ int prefix_len(const uint32_t* __restrict__ keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = __ldg(&keys[i]), b = __ldg(&keys[j]);
    if (a == b) return 32 + __clz(i ^ j);
    return __clz(a ^ b);
}

__global__ void __launch_bounds__(256) k_karras(const uint32_t* __restrict__ keys, int n,
                                                float4* __restrict__ nodes, int* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int dl = prefix_len(keys, n, i, i - 1);
    const int dr = prefix_len(keys, n, i, i + 1);
    const int d = dr > dl ? 1 : -1;
    const int dmin = min(dl, dr);
    int lmax = 2;
    while (prefix_len(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (prefix_len(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = prefix_len(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (prefix_len(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int left = (min(i, j) == gamma) ? ~gamma : gamma;
    const int right = (max(i, j) == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    // n3 = (left, right, first leaf, last leaf): the node covers leaves min(i, j) .. max(i, j)
    nodes[4 * i + 3] = make_float4(__int_as_float(left), __int_as_float(right), __int_as_float(min(i, j)),
                                   __int_as_float(max(i, j)));
    parent[left >= 0 ? left : (n - 1) + ~left] = i;
    parent[right >= 0 ? right : (n - 1) + ~right] = i;
    if (i == 0) parent[0] = -1;
}

// One thread per leaf: gathers the triangle into leaf order and climbs to the root,
// writing each child's box into its parent's slot. The second thread to arrive at a node
// (arrival counter) owns the union and continues upwards.
__global__ void __launch_bounds__(256) k_leaf_boxes(const float4* __restrict__ tri_in, RefView rv,
                                                    const uint32_t* __restrict__ order, int n,
                                                    const int* __restrict__ parent, float4* nodes,
                                                    uint32_t* flags, float4* __restrict__ tris,
                                                    uint32_t* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 lo, hi;
    const uint32_t o = ref_geometry(tri_in, rv, order[i], lo, hi);  // the reference's triangle and box
    const float4 a = __ldg(&tri_in[3 * o]), b = __ldg(&tri_in[3 * o + 1]), c = __ldg(&tri_in[3 * o + 2]);
    {
        // edges rounded to FP32, and the per-triangle factors of the test's error bound
        // (robust.cuh) from their 1-norms
        const float3 e1 = mk3(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z));
        const float3 e2 = mk3(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z));
        const float n1 = fabsf(e1.x) + fabsf(e1.y) + fabsf(e1.z), n2 = fabsf(e2.x) + fabsf(e2.y) + fabsf(e2.z);
        tris[3 * i] = make_float4(a.x, a.y, a.z, __int_as_float(static_cast<int>(o)));
        tris[3 * i + 1] = make_float4(e1.x, e1.y, e1.z, robust_k1(n1, n2));
        tris[3 * i + 2] = make_float4(e2.x, e2.y, e2.z, robust_k2(n1, n2));
    }
    if (n == 1) {
        nodes[0] = make_float4(lo.x, hi.x, lo.y, hi.y);
        nodes[1] = make_float4(lo.x, hi.x, lo.y, hi.y);
        nodes[2] = make_float4(lo.z, hi.z, lo.z, hi.z);
        nodes[3] = make_float4(__int_as_float(~0), __int_as_float(~0), __int_as_float(0), __int_as_float(0));
        return;
    }
    int child = ~i;
    int p = parent[(n - 1) + i];
    // Depth is bounded by the 64 bits of the index-augmented keys; a longer climb means a
    // malformed parent array.
    for (int depth = 0;; ++depth) {
        if (depth > 128 || p < 0 || p >= n - 1) {
            atomicOr(err, k_deverr_traversal);
            return;
        }
        const float4 meta = __ldcg(&nodes[4 * p + 3]);
        const int slot = (__float_as_int(meta.x) == child) ? 0 : 1;
        nodes[4 * p + slot] = make_float4(lo.x, hi.x, lo.y, hi.y);
        reinterpret_cast<float2*>(&nodes[4 * p + 2])[slot] = make_float2(lo.z, hi.z);
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0u) return;
        __threadfence();
        const float4 n0 = __ldcg(&nodes[4 * p]);
        const float4 n1 = __ldcg(&nodes[4 * p + 1]);
        const float4 n2 = __ldcg(&nodes[4 * p + 2]);
        lo = mk3(fminf(n0.x, n1.x), fminf(n0.z, n1.z), fminf(n2.x, n2.z));
        hi = mk3(fmaxf(n0.y, n1.y), fmaxf(n0.w, n1.w), fmaxf(n2.y, n2.w));
        if (p == 0) return;
        child = p;
        p = parent[p];
    }
}

// ---------------------------------------------------------------- 8-wide collapse (wide.cuh)

struct WideEntry {
    int ref;     // binary child: >= 0 internal node, < 0 leaf ~pos
    int first;   // first leaf of the subtree
    int size;    // leaves in the subtree
    float lo[3], hi[3];
};

__device__ __forceinline__ float half_area(const float lo[3], const float hi[3]) {
    const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]), dz = __fsub_rn(hi[2], lo[2]);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}

// Child k (0/1) of binary node c as a collapse entry; reads c's record (and, for an internal
// child, that child's leaf range).
__device__ __forceinline__ void wide_entry(const float4* __restrict__ nodes, int c, int k, WideEntry& e) {
    const float4 nb = __ldg(&nodes[4 * c + k]);
    const float4 n2 = __ldg(&nodes[4 * c + 2]);
    const float4 n3 = __ldg(&nodes[4 * c + 3]);
    e.ref = __float_as_int(k == 0 ? n3.x : n3.y);
    e.lo[0] = nb.x;
    e.hi[0] = nb.y;
    e.lo[1] = nb.z;
    e.hi[1] = nb.w;
    e.lo[2] = k == 0 ? n2.x : n2.z;
    e.hi[2] = k == 0 ? n2.y : n2.w;
    if (e.ref < 0) {
        e.first = ~e.ref;
        e.size = 1;
    } else {
        const float4 m3 = __ldg(&nodes[4 * e.ref + 3]);
        e.first = __float_as_int(m3.z);
        e.size = __float_as_int(m3.w) - e.first + 1;
    }
}

// Smallest e (clamped to [-100, 126]) with 255 * 2^e >= hi - lo, as the biased exponent byte.
__device__ __forceinline__ uint32_t wide_exponent(float lo, float hi) {
    const float x = __fdiv_ru(__fsub_ru(hi, lo), 255.0f);
    const uint32_t bits = __float_as_uint(x);
    const int ebits = static_cast<int>((bits >> 23) & 0xffu);
    int e = ebits == 0 ? -100 : ebits - 127 + ((bits & 0x7fffffu) != 0u ? 1 : 0);
    e = max(-100, min(126, e));
    return static_cast<uint32_t>(e + 127);
}

// ---------------------------------------------------------------- SAH refinement of small subtrees
//
// The Morton order places a subtree's leaves well at large scale but splits small groups of
// triangles by their code bits, not by their boxes. Each maximal subtree of 3..cluster leaves
// (cluster <= 32: one warp lane per leaf) is rebuilt top-down with the split of least
// surface-area cost (areas of the two child boxes times their leaf counts) over every
// position of the leaves sorted along each axis by box centre; the subtree keeps its root
// node, its set of node indices and its leaves, so the rest of the tree is untouched. On the
// 1M soup this cuts the 8-wide records a ray visits by 2-3 % (a full top-down SAH build:
// 5 %).

// Roots of the maximal subtrees with 3..cluster leaves (their parent covers more).
__global__ void __launch_bounds__(256) k_sah_roots(const float4* __restrict__ nodes, const int* __restrict__ parent,
                                                   int n, int cluster, int* __restrict__ roots,
                                                   int* __restrict__ count) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n - 1) return;
    const float4 m = __ldg(&nodes[4 * c + 3]);
    const int size = __float_as_int(m.w) - __float_as_int(m.z) + 1;
    if (size < 3 || size > cluster) return;
    if (c != 0) {
        const float4 pm = __ldg(&nodes[4 * __ldg(&parent[c]) + 3]);
        if (__float_as_int(pm.w) - __float_as_int(pm.z) + 1 <= cluster) return;
    }
    roots[atomicAdd(count, 1)] = c;
}

// Inclusive scan over the warp's lanes of a box (min of lo, max of hi) and a count; reverse
// = true scans from lane 31 down.
template <bool REVERSE>
__device__ __forceinline__ void warp_box_scan(float (&lo)[3], float (&hi)[3], int& cnt, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float l[3], h[3];
        int c;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            l[a] = REVERSE ? __shfl_down_sync(0xffffffffu, lo[a], o) : __shfl_up_sync(0xffffffffu, lo[a], o);
            h[a] = REVERSE ? __shfl_down_sync(0xffffffffu, hi[a], o) : __shfl_up_sync(0xffffffffu, hi[a], o);
        }
        c = REVERSE ? __shfl_down_sync(0xffffffffu, cnt, o) : __shfl_up_sync(0xffffffffu, cnt, o);
        if (REVERSE ? lane + o < 32 : lane >= o) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], l[a]);
                hi[a] = fmaxf(hi[a], h[a]);
            }
            cnt += c;
        }
    }
}

// One warp per subtree root from k_sah_roots.
__global__ void __launch_bounds__(256) k_sah_rebuild(const float4* __restrict__ tri_in, RefView rv,
                                                     const uint32_t* __restrict__ order, float4* nodes,
                                                     int* __restrict__ parent, int n_leaves,
                                                     const int* __restrict__ roots, const int* __restrict__ count,
                                                     uint32_t* __restrict__ err) {
    constexpr int W = 8;  // warps per block
    __shared__ int s_pool[W][32];       // the subtree's node indices, root first
    __shared__ uint2 s_task[W][32];     // pending (leaf mask, node index)
    __shared__ float s_box[W][3][32][6];  // leaf boxes in centre order along each axis
    __shared__ int s_lane[W][3][32];    // lane (leaf) at each rank along each axis
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_roots = *count;
    for (int ci = blockIdx.x * W + warp; ci < n_roots; ci += gridDim.x * W) {
        const int r0 = roots[ci];
        const float4 m3 = nodes[4 * r0 + 3];
        const int f = __float_as_int(m3.z), m = __float_as_int(m3.w) - f + 1;  // 3..32 leaves
        int np = 0;
        if (lane == 0) {  // the subtree's internal nodes, depth first (m - 1 of them)
            int st[32], sp = 0;
            st[sp++] = r0;
            while (sp > 0 && np < 32) {
                const int c = st[--sp];
                s_pool[warp][np++] = c;
                const float4 q = nodes[4 * c + 3];
                const int a = __float_as_int(q.x), b = __float_as_int(q.y);
                if (a >= 0 && sp < 32) st[sp++] = a;
                if (b >= 0 && sp < 32) st[sp++] = b;
            }
        }
        np = __shfl_sync(0xffffffffu, np, 0);
        if (np != m - 1) {  // not the subtree the leaf range says: leave it as it is
            if (lane == 0) atomicOr(err, k_deverr_traversal);
            continue;
        }
        // this lane's leaf: box and centre
        const bool have = lane < m;
        float lo[3], hi[3], ce[3];
        if (have) {
            float3 l3, h3;
            ref_geometry(tri_in, rv, order[f + lane], l3, h3);
            lo[0] = l3.x;
            lo[1] = l3.y;
            lo[2] = l3.z;
            hi[0] = h3.x;
            hi[1] = h3.y;
            hi[2] = h3.z;
#pragma unroll
            for (int k = 0; k < 3; ++k) ce[k] = __fadd_rn(lo[k], hi[k]);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lo[k] = __int_as_float(0x7f800000);
                hi[k] = -__int_as_float(0x7f800000);
                ce[k] = __int_as_float(0x7f800000);
            }
        }
        // rank of this leaf along each axis (centre, then lane), and the boxes in rank order
        int rank[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            int r = 0;
            for (int j = 0; j < 32; ++j) {
                const float cj = __shfl_sync(0xffffffffu, ce[k], j);
                r += (cj < ce[k] || (cj == ce[k] && j < lane)) ? 1 : 0;
            }
            rank[k] = r;
            s_box[warp][k][r][0] = lo[0];
            s_box[warp][k][r][1] = lo[1];
            s_box[warp][k][r][2] = lo[2];
            s_box[warp][k][r][3] = hi[0];
            s_box[warp][k][r][4] = hi[1];
            s_box[warp][k][r][5] = hi[2];
            s_lane[warp][k][r] = lane;
        }
        if (lane == 0) s_task[warp][0] = make_uint2(m == 32 ? 0xffffffffu : (1u << m) - 1u, static_cast<uint32_t>(r0));
        __syncwarp();
        int n_task = 1, n_used = 1;  // warp-uniform: pending tasks, pool entries handed out
        for (int it = 0; n_task > 0; ++it) {
            if (it >= 64) {
                if (lane == 0) atomicOr(err, k_deverr_traversal);
                break;
            }
            const uint2 task = s_task[warp][--n_task];
            const uint32_t mask = task.x;
            float bl[6], br[6];
            uint32_t left;
            if (__popc(mask) == 2) {
                // two leaves: one split, no search (half the nodes of a subtree)
                const int l0 = __ffs(mask) - 1, l1 = __ffs(mask & (mask - 1u)) - 1;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    bl[a] = __shfl_sync(0xffffffffu, lo[a], l0);
                    bl[3 + a] = __shfl_sync(0xffffffffu, hi[a], l0);
                    br[a] = __shfl_sync(0xffffffffu, lo[a], l1);
                    br[3 + a] = __shfl_sync(0xffffffffu, hi[a], l1);
                }
                left = 1u << l0;
            } else {
            // best split over the three axes: leaves of rank <= r go left
            float best = __int_as_float(0x7f800000);
            int best_axis = 0, best_r = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const bool member = (mask >> s_lane[warp][k][lane]) & 1u;
                float pl[3], ph[3], sl[3], sh[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    pl[a] = member ? s_box[warp][k][lane][a] : __int_as_float(0x7f800000);
                    ph[a] = member ? s_box[warp][k][lane][3 + a] : -__int_as_float(0x7f800000);
                    sl[a] = pl[a];
                    sh[a] = ph[a];
                }
                int pc = member ? 1 : 0, sc = pc;
                warp_box_scan<false>(pl, ph, pc, lane);
                warp_box_scan<true>(sl, sh, sc, lane);
                // split after rank `lane`: left = prefix(lane), right = suffix(lane + 1)
                float rl[3], rh[3];
                int rc = __shfl_down_sync(0xffffffffu, sc, 1);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    rl[a] = __shfl_down_sync(0xffffffffu, sl[a], 1);
                    rh[a] = __shfl_down_sync(0xffffffffu, sh[a], 1);
                }
                if (lane == 31) rc = 0;
                float cost = __int_as_float(0x7f800000);
                if (member && pc > 0 && rc > 0) {
                    const float al = half_area(pl, ph), ar = half_area(rl, rh);
                    cost = __fadd_rn(__fmul_rn(al, static_cast<float>(pc)), __fmul_rn(ar, static_cast<float>(rc)));
                }
                // warp argmin (cost, rank)
                float c = cost;
                int r = lane;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
                    const int r2 = __shfl_xor_sync(0xffffffffu, r, o);
                    if (c2 < c || (c2 == c && r2 < r)) {
                        c = c2;
                        r = r2;
                    }
                }
                if (c < best) {
                    best = c;
                    best_axis = k;
                    best_r = r;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        bl[a] = __shfl_sync(0xffffffffu, pl[a], r);
                        bl[3 + a] = __shfl_sync(0xffffffffu, ph[a], r);
                        br[a] = __shfl_sync(0xffffffffu, rl[a], r);
                        br[3 + a] = __shfl_sync(0xffffffffu, rh[a], r);
                    }
                }
            }
            if (!(best < __int_as_float(0x7f800000))) {  // no split found: keep the old tree shape
                if (lane == 0) atomicOr(err, k_deverr_traversal);
                break;
            }
            const bool mine = (mask >> lane) & 1u;
            left = __ballot_sync(0xffffffffu, mine && rank[best_axis] <= best_r);
            }
            const uint32_t right = mask & ~left;
            const uint32_t side[2] = {left, right};
            const int need = (__popc(left) > 1 ? 1 : 0) + (__popc(right) > 1 ? 1 : 0);
            if (left == 0u || right == 0u || n_used + need > m - 1 || n_task + need > 32) {
                if (lane == 0) atomicOr(err, k_deverr_traversal);
                break;
            }
            int ref[2];
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2) {
                if (__popc(side[s2]) == 1) {
                    ref[s2] = ~(f + __ffs(side[s2]) - 1);
                } else {
                    ref[s2] = s_pool[warp][n_used];
                    if (lane == 0) s_task[warp][n_task] = make_uint2(side[s2], static_cast<uint32_t>(ref[s2]));
                    ++n_used;
                    ++n_task;
                }
            }
            if (lane == 0) {
                for (int s2 = 0; s2 < 2; ++s2)
                    parent[ref[s2] >= 0 ? ref[s2] : (n_leaves - 1) + ~ref[s2]] = static_cast<int>(task.y);
                float4* nd = nodes + 4 * static_cast<size_t>(task.y);
                nd[0] = make_float4(bl[0], bl[3], bl[1], bl[4]);
                nd[1] = make_float4(br[0], br[3], br[1], br[4]);
                nd[2] = make_float4(bl[2], bl[5], br[2], br[5]);
                // (z, w): a leaf range of the node's leaf count (the collapse reads only the count)
                nd[3] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), __int_as_float(f),
                                    __int_as_float(f + __popc(mask) - 1));
            }
            __syncwarp();
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- SAH-optimal 8-wide collapse
//
// Ylitie, Karras and Laine (2017): the cheapest way to spread a binary subtree over the at
// most 8 child slots of a wide record, by dynamic programming over the binary nodes, bottom
// up. cost(n, i) is the least surface-area cost of subtree n given i slots: with one slot n
// becomes a wide record of its own (cost half_area(n) plus the best spread of its two
// children over 8 slots); with i > 1 slots also cost(n, i - 1) or k slots to the left child
// and i - k to the right. One-triangle leaves take a slot each at a cost that does not depend
// on the spread, so it is left out. The decisions are stored per node: dec[0] = the best k for
// n's own record, dec[i - 1] = 0 (as with i - 1 slots) or k for i > 1. On the 1M soup this
// records 4-6 % fewer visits per ray than opening the largest child greedily.

constexpr float k_dp_inf = 3.0e38f;

__device__ __forceinline__ float dp_child_cost(const float* __restrict__ cost, int c, int slots) {
    return c < 0 ? 0.0f : __ldcg(&cost[8 * c + slots - 1]);
}

// One thread per leaf climbs to the root; the second thread to arrive at a node computes its
// table from its children's (arrival counters as in k_leaf_boxes).
__global__ void __launch_bounds__(256) k_collapse_dp(const float4* __restrict__ nodes, const int* __restrict__ parent,
                                                     int n, uint32_t* flags, float* cost, uint8_t* dec,
                                                     uint32_t* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || n < 2) return;
    int p = parent[(n - 1) + i];
    for (int depth = 0;; ++depth) {
        if (depth > 4096 || p < 0 || p >= n - 1) {
            atomicOr(err, k_deverr_traversal);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0u) return;
        __threadfence();
        const float4 n0 = __ldg(&nodes[4 * p]), n1 = __ldg(&nodes[4 * p + 1]), n2 = __ldg(&nodes[4 * p + 2]);
        const float4 n3 = __ldg(&nodes[4 * p + 3]);
        const int l = __float_as_int(n3.x), r = __float_as_int(n3.y);
        float cl[8], cr[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cl[k] = dp_child_cost(cost, l, k + 1);
            cr[k] = dp_child_cost(cost, r, k + 1);
        }
        const float lo[3] = {fminf(n0.x, n1.x), fminf(n0.z, n1.z), fminf(n2.x, n2.z)};
        const float hi[3] = {fmaxf(n0.y, n1.y), fmaxf(n0.w, n1.w), fmaxf(n2.y, n2.w)};
        float c_int = k_dp_inf;
        int k_int = 1;
#pragma unroll
        for (int k = 1; k <= 7; ++k) {
            const float v = __fadd_rn(cl[k - 1], cr[8 - k - 1]);
            if (v < c_int) {
                c_int = v;
                k_int = k;
            }
        }
        float c[8];
        uint8_t d[8];
        c[0] = __fadd_rn(half_area(lo, hi), c_int);
        d[0] = static_cast<uint8_t>(k_int);
#pragma unroll
        for (int s = 2; s <= 8; ++s) {
            float best = c[s - 2];
            int bk = 0;
#pragma unroll
            for (int k = 1; k < s; ++k) {
                const float v = __fadd_rn(cl[k - 1], cr[s - k - 1]);
                if (v < best) {
                    best = v;
                    bk = k;
                }
            }
            c[s - 1] = best;
            d[s - 1] = static_cast<uint8_t>(bk);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            cost[8 * p + k] = c[k];
            dec[8 * p + k] = d[k];
        }
        if (p == 0) return;
        p = parent[p];
    }
}

// One thread per binary internal node b: the wide record of b's subtree (layout in wide.cuh).
// DP: the children come from the decisions of k_collapse_dp; otherwise the internal child of
// largest surface area is opened greedily (ties to the lower entry) until 8 entries.
template <bool DP>
__global__ void __launch_bounds__(128) k_collapse8(const float4* __restrict__ nodes, int n_internal,
                                                   const uint8_t* __restrict__ dec, float4* __restrict__ wide) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_internal) return;
    WideEntry e[8];
    int count;
    if (DP) {
        // entries with their slot budgets; an internal entry with budget > 1 is replaced by
        // its children as its decisions say, until every entry is final
        int slots[8];
        const int k0 = max(1, min(7, static_cast<int>(__ldg(&dec[8 * b]))));
        wide_entry(nodes, b, 0, e[0]);
        wide_entry(nodes, b, 1, e[1]);
        slots[0] = k0;
        slots[1] = 8 - k0;
        count = 2;
        for (int it = 0; it < 16; ++it) {
            int pick = -1, ii = 1;
            for (int j = 0; j < count && pick < 0; ++j) {
                if (e[j].ref < 0 || slots[j] <= 1) continue;
                int s = slots[j];
                while (s > 1 && __ldg(&dec[8 * e[j].ref + s - 1]) == 0) --s;
                if (s > 1) {
                    pick = j;
                    ii = s;
                } else {
                    slots[j] = 1;
                }
            }
            if (pick < 0 || count >= 8) break;
            const int c = e[pick].ref;
            const int k = max(1, min(ii - 1, static_cast<int>(__ldg(&dec[8 * c + ii - 1]))));
            wide_entry(nodes, c, 1, e[count]);
            slots[count] = ii - k;
            wide_entry(nodes, c, 0, e[pick]);
            slots[pick] = k;
            ++count;
        }
    } else {
        wide_entry(nodes, b, 0, e[0]);
        wide_entry(nodes, b, 1, e[1]);
        count = 2;
        while (count < 8) {
            int pick = -1;
            float best = 0.0f;
            for (int i = 0; i < count; ++i) {
                if (e[i].ref < 0) continue;
                const float a = half_area(e[i].lo, e[i].hi);
                if (pick < 0 || a > best) {
                    pick = i;
                    best = a;
                }
            }
            if (pick < 0) break;
            const int c = e[pick].ref;
            wide_entry(nodes, c, 1, e[count]);
            wide_entry(nodes, c, 0, e[pick]);
            ++count;
        }
    }
    // node box; the grid covers it padded by the scene's Delta (every child box is quantised
    // padded by Delta, lower planes rounded down and upper planes up), so a ray's FP32 slab
    // test never culls a child box the exact ray touches (robust.cuh)
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = e[0].lo[a];
        hi[a] = e[0].hi[a];
        for (int i = 1; i < count; ++i) {
            lo[a] = fminf(lo[a], e[i].lo[a]);
            hi[a] = fmaxf(hi[a], e[i].hi[a]);
        }
    }
    const float pad = scene_box_pad(nodes);
    float glo[3];
    uint32_t ex[3];
    float inv_s[3];
    for (int a = 0; a < 3; ++a) {
        glo[a] = __fsub_rd(lo[a], pad);
        ex[a] = wide_exponent(glo[a], __fadd_ru(hi[a], pad));
        inv_s[a] = __uint_as_float((254u - ex[a]) << 23);  // 2^-e for e in [-100, 126]
    }
    // slots by direction: child i goes to the free slot s maximising sum_a sign_s(a) * c_i(a),
    // c_i = child centre - node centre, sign negative where bit a of s is set; greedy over
    // (child, slot) pairs in descending score, ties to the lower child, then the lower slot
    float cx[8], cy[8], cz[8];
    const float mx = __fmul_rn(__fadd_rn(lo[0], hi[0]), 0.5f), my = __fmul_rn(__fadd_rn(lo[1], hi[1]), 0.5f),
                mz = __fmul_rn(__fadd_rn(lo[2], hi[2]), 0.5f);
    for (int i = 0; i < count; ++i) {
        cx[i] = __fsub_rn(__fmul_rn(__fadd_rn(e[i].lo[0], e[i].hi[0]), 0.5f), mx);
        cy[i] = __fsub_rn(__fmul_rn(__fadd_rn(e[i].lo[1], e[i].hi[1]), 0.5f), my);
        cz[i] = __fsub_rn(__fmul_rn(__fadd_rn(e[i].lo[2], e[i].hi[2]), 0.5f), mz);
    }
    int slot_of[8];
    uint32_t used_slots = 0, placed = 0;
    for (int it = 0; it < count; ++it) {
        int bi = -1, bs = -1;
        float bsc = 0.0f;
        for (int i = 0; i < count; ++i) {
            if (placed & (1u << i)) continue;
            for (int s = 0; s < 8; ++s) {
                if (used_slots & (1u << s)) continue;
                const float sc = __fadd_rn(__fadd_rn((s & 1) ? -cx[i] : cx[i], (s & 2) ? -cy[i] : cy[i]),
                                           (s & 4) ? -cz[i] : cz[i]);
                if (bi < 0 || sc > bsc) {
                    bi = i;
                    bs = s;
                    bsc = sc;
                }
            }
        }
        slot_of[bi] = bs;
        placed |= 1u << bi;
        used_slots |= 1u << bs;
    }
    uint32_t qb[3][2][2] = {};  // [axis][lo/hi][word]: bytes of slots 0..3 and 4..7
    int refs[8];
    uint32_t imask = 0;
    for (int s = 0; s < 8; ++s) {
        refs[s] = k_wide_empty_ref;
        for (int a = 0; a < 3; ++a) qb[a][0][s >> 2] |= 255u << (8 * (s & 3));
    }
    for (int i = 0; i < count; ++i) {
        const int s = slot_of[i];
        for (int a = 0; a < 3; ++a) {
            const float ql = floorf(__fmul_rd(__fsub_rd(__fsub_rd(e[i].lo[a], pad), glo[a]), inv_s[a]));
            const float qh = ceilf(__fmul_ru(__fsub_ru(__fadd_ru(e[i].hi[a], pad), glo[a]), inv_s[a]));
            const uint32_t bl = static_cast<uint32_t>(fminf(fmaxf(ql, 0.0f), 255.0f));
            const uint32_t bh = static_cast<uint32_t>(fminf(fmaxf(qh, 0.0f), 255.0f));
            qb[a][0][s >> 2] = (qb[a][0][s >> 2] & ~(255u << (8 * (s & 3)))) | (bl << (8 * (s & 3)));
            qb[a][1][s >> 2] |= bh << (8 * (s & 3));
        }
        if (e[i].ref >= 0 && e[i].size > k_wide_leaf_max) {
            refs[s] = e[i].ref;
            imask |= 1u << s;
        } else {
            refs[s] = ~((e[i].first << 2) | (e[i].size - 1));
        }
    }
    float4* w = wide + k_wide_node_f4 * static_cast<size_t>(b);
    w[0] = make_float4(glo[0], glo[1], glo[2], __uint_as_float(ex[0] | (ex[1] << 8) | (ex[2] << 16) | (imask << 24)));
    for (int a = 0; a < 3; ++a)
        w[1 + a] = make_float4(__uint_as_float(qb[a][0][0]), __uint_as_float(qb[a][0][1]), __uint_as_float(qb[a][1][0]),
                               __uint_as_float(qb[a][1][1]));
    w[4] = make_float4(__int_as_float(refs[0]), __int_as_float(refs[1]), __int_as_float(refs[2]), __int_as_float(refs[3]));
    w[5] = make_float4(__int_as_float(refs[4]), __int_as_float(refs[5]), __int_as_float(refs[6]), __int_as_float(refs[7]));
}

// Unit normal u = ng / |ng| of the triangle (a, b, c), ng = cross(e1, e2) in double-float from
// the exact edge differences (one reciprocal); len = |ng| (twice the area). Shared by the
// plane and emitter tables so both hold the same bits.
__device__ __forceinline__ ff3 tri_unit_normal_ff(float3 a, float3 b, float3 c, ff& len) {
    const ff3 e1 = ff3_diff(b, a), e2 = ff3_diff(c, a);
    const ff3 ng = ff3_cross(e1, e2);
    len = ff3_length(ng);
    return ff3_scale(ng, ff_div(ffv(1.0f), len));
}

// Shading plane of triangle i (original order): the unit normal u and the plane offset u.v0,
// double-float; 32 bytes, one sector per hit.
__global__ void __launch_bounds__(256) k_tri_planes(const float4* __restrict__ tri_in, uint32_t n,
                                                    float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 a = xyz(__ldg(&tri_in[3 * i]));
    ff len;
    const ff3 u = tri_unit_normal_ff(a, xyz(__ldg(&tri_in[3 * i + 1])), xyz(__ldg(&tri_in[3 * i + 2])), len);
    const ff off = ff3_dot(u, ff3v(a));
    out[2 * i] = make_float4(u.x.hi, u.x.lo, u.y.hi, u.y.lo);
    out[2 * i + 1] = make_float4(u.z.hi, u.z.lo, off.hi, off.lo);
}

// Light-sampling record of emitter slot k (triangle l = emitters[k]), 5 float4:
// (v0, l), (v1, |ng|.hi), (v2, |ng|.lo), (u.x, u.y), (u.z, -, -) with u and |ng| as in
// k_tri_planes. One record per light sample replaces the emitter index and the light
// triangle's vertex and table loads that depend on it.
__global__ void __launch_bounds__(256) k_emit_table(const float4* __restrict__ tri_in, const int* __restrict__ emitters,
                                                    uint32_t n_emit, float4* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_emit) return;
    const int l = __ldg(&emitters[k]);
    const float3 a = xyz(__ldg(&tri_in[3 * l])), b = xyz(__ldg(&tri_in[3 * l + 1])), c = xyz(__ldg(&tri_in[3 * l + 2]));
    ff len;
    const ff3 u = tri_unit_normal_ff(a, b, c, len);
    out[5 * k] = make_float4(a.x, a.y, a.z, __int_as_float(l));
    out[5 * k + 1] = make_float4(b.x, b.y, b.z, len.hi);
    out[5 * k + 2] = make_float4(c.x, c.y, c.z, len.lo);
    out[5 * k + 3] = make_float4(u.x.hi, u.x.lo, u.y.hi, u.y.lo);
    out[5 * k + 4] = make_float4(u.z.hi, u.z.lo, 0.f, 0.f);
}

// Copies the first `count` internal nodes in breadth-first order (the top levels of the
// tree) into `tree`, rewriting child links that stay inside the copy to k_tree_flag | slot.
// One thread: count is at most a few hundred. The queue of global indices lives in the
// (not yet written) n3.z words of the output slots.
__global__ void k_treelet(const float4* __restrict__ nodes, int count, float4* __restrict__ tree) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    constexpr int flag = 0x40000000;
    tree[3] = make_float4(0.f, 0.f, __int_as_float(0), 0.f);
    int tail = 1;
    for (int head = 0; head < tail; ++head) {
        const int g = __float_as_int(tree[4 * head + 3].z);
        const float4 n3 = nodes[4 * g + 3];
        int c[2] = {__float_as_int(n3.x), __float_as_int(n3.y)};
        for (int k = 0; k < 2; ++k) {
            if (c[k] >= 0 && tail < count) {
                tree[4 * tail + 3] = make_float4(0.f, 0.f, __int_as_float(c[k]), 0.f);
                c[k] = flag | tail;
                ++tail;
            }
        }
        tree[4 * head + 0] = nodes[4 * g + 0];
        tree[4 * head + 1] = nodes[4 * g + 1];
        tree[4 * head + 2] = nodes[4 * g + 2];
        tree[4 * head + 3] = make_float4(__int_as_float(c[0]), __int_as_float(c[1]), __int_as_float(g), 0.f);
    }
}

inline uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace

cudaError_t LbvhBuilder::build_treelet(int max_nodes, cudaStream_t stream, KernelProfiler& prof) {
    tree_n_ = 0;
    if (n_ == 0 || max_nodes <= 0) return cudaSuccess;
    const int internal = static_cast<int>(n_ > 1 ? n_ - 1 : 1);
    const int count = std::min(max_nodes, internal);
    if (count > tree_capacity_) {
        if (tree_) cudaFree(tree_);
        tree_ = nullptr;
        tree_capacity_ = 0;
        QUASI_TRY_CUDA(cudaMalloc(&tree_, sizeof(float4) * 4 * count));
        tree_capacity_ = count;
    }
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_treelet", stream, (k_treelet<<<1, 32, 0, stream>>>(nodes_, count, tree_))));
    tree_n_ = count;
    return cudaSuccess;
}

// ---------------------------------------------------------------- host: radix sort

size_t radix_sort_hist_entries(uint32_t n) { return 256ull * ceil_div(n > 0 ? n : 1, k_sort_tile); }

cudaError_t radix_sort_reserve(RadixSortScratch& s, uint32_t n) {
    if (n <= s.capacity && radix_sort_hist_entries(n) <= s.hist_capacity) return cudaSuccess;
    radix_sort_release(s);
    QUASI_TRY_CUDA(cudaMalloc(&s.keys_alt, sizeof(uint32_t) * std::max<uint32_t>(n, 1)));
    QUASI_TRY_CUDA(cudaMalloc(&s.vals_alt, sizeof(uint32_t) * std::max<uint32_t>(n, 1)));
    const size_t h = radix_sort_hist_entries(n);
    QUASI_TRY_CUDA(cudaMalloc(&s.hist, sizeof(uint32_t) * h));
    s.capacity = n;
    s.hist_capacity = static_cast<uint32_t>(h);
    return cudaSuccess;
}

void radix_sort_release(RadixSortScratch& s) {
    if (s.keys_alt) cudaFree(s.keys_alt);
    if (s.vals_alt) cudaFree(s.vals_alt);
    if (s.hist) cudaFree(s.hist);
    s = RadixSortScratch{};
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int key_bits,
                             RadixSortScratch& s, cudaStream_t stream, KernelProfiler& prof) {
    if (n <= 1) return cudaSuccess;
    if (n > s.capacity) return cudaErrorInvalidValue;
    const uint32_t nblocks = ceil_div(n, k_sort_tile);
    const int passes = (key_bits + 7) / 8;
    uint32_t *ki = keys, *vi = vals, *ko = s.keys_alt, *vo = s.vals_alt;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "radix_hist", stream,
                                    (k_radix_hist<<<nblocks, k_sort_block, 0, stream>>>(ki, n, shift, s.hist, nblocks))));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "radix_scan", stream,
                                    (k_scan_exclusive<<<1, 1024, 0, stream>>>(s.hist, 256u * nblocks))));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "radix_scatter", stream,
                                    (k_radix_scatter<<<nblocks, k_sort_block, 0, stream>>>(ki, vi, ko, vo, n, shift,
                                                                                           s.hist, nblocks))));
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    if (ki != keys) {
        QUASI_TRY_CUDA(cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream));
        QUASI_TRY_CUDA(cudaMemcpyAsync(vals, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream));
    }
    return cudaSuccess;
}

// ---------------------------------------------------------------- host: LBVH builder

cudaError_t LbvhBuilder::reserve(uint32_t n) {
    if (n <= capacity_ && bounds_) return cudaSuccess;
    release();
    const uint32_t m = std::max<uint32_t>(n, 2);
    QUASI_TRY_CUDA(cudaMalloc(&bounds_, sizeof(float) * 12));
    QUASI_TRY_CUDA(cudaMalloc(&partial_, sizeof(float) * 6 * k_bounds_blocks));
    QUASI_TRY_CUDA(cudaMalloc(&morton_, sizeof(uint32_t) * m));
    QUASI_TRY_CUDA(cudaMalloc(&keys_, sizeof(uint32_t) * m));
    QUASI_TRY_CUDA(cudaMalloc(&order_, sizeof(uint32_t) * m));
    QUASI_TRY_CUDA(cudaMalloc(&parent_, sizeof(int) * (2 * m)));
    QUASI_TRY_CUDA(cudaMalloc(&flags_, sizeof(uint32_t) * m));
    QUASI_TRY_CUDA(cudaMalloc(&nodes_, sizeof(float4) * 4 * m));
    QUASI_TRY_CUDA(cudaMalloc(&tris_, sizeof(float4) * 3 * m));
    QUASI_TRY_CUDA(cudaMalloc(&wide_, sizeof(float4) * k_wide_node_f4 * m));
    QUASI_TRY_CUDA(cudaMalloc(&tri_plane_, sizeof(float4) * 2 * m));
    QUASI_TRY_CUDA(cudaMalloc(&sah_roots_, sizeof(int) * m));
    QUASI_TRY_CUDA(cudaMalloc(&dp_cost_, sizeof(float) * 8 * m));
    QUASI_TRY_CUDA(cudaMalloc(&dp_dec_, 8 * static_cast<size_t>(m)));
    QUASI_TRY_CUDA(cudaMalloc(&sah_count_, sizeof(int)));
    QUASI_TRY_CUDA(radix_sort_reserve(sort_, m));
    capacity_ = m;
    return cudaSuccess;
}

void LbvhBuilder::release() {
    for (void* p : {static_cast<void*>(bounds_), static_cast<void*>(partial_), static_cast<void*>(morton_),
                    static_cast<void*>(keys_), static_cast<void*>(order_), static_cast<void*>(parent_),
                    static_cast<void*>(flags_), static_cast<void*>(nodes_), static_cast<void*>(tris_),
                    static_cast<void*>(wide_), static_cast<void*>(tri_plane_), static_cast<void*>(emit_tab_),
                    static_cast<void*>(sah_roots_), static_cast<void*>(sah_count_), static_cast<void*>(dp_cost_),
                    static_cast<void*>(dp_dec_)})
        if (p) cudaFree(p);
    bounds_ = partial_ = nullptr;
    morton_ = keys_ = order_ = flags_ = nullptr;
    parent_ = nullptr;
    nodes_ = tris_ = wide_ = tri_plane_ = emit_tab_ = nullptr;
    sah_roots_ = sah_count_ = nullptr;
    dp_cost_ = nullptr;
    dp_dec_ = nullptr;
    emit_capacity_ = 0;
    if (tree_) cudaFree(tree_);
    tree_ = nullptr;
    tree_n_ = tree_capacity_ = 0;
    if (ref_tri_) cudaFree(ref_tri_);
    if (ref_box_) cudaFree(ref_box_);
    ref_tri_ = nullptr;
    ref_box_ = nullptr;
    ref_capacity_ = 0;
    radix_sort_release(sort_);
    capacity_ = 0;
    n_ = 0;
    n_tris_ = 0;
}

cudaError_t LbvhBuilder::reserve_refs(uint32_t m) {
    if (m <= ref_capacity_ && ref_tri_) return cudaSuccess;
    if (ref_tri_) cudaFree(ref_tri_);
    if (ref_box_) cudaFree(ref_box_);
    ref_tri_ = nullptr;
    ref_box_ = nullptr;
    ref_capacity_ = 0;
    QUASI_TRY_CUDA(cudaMalloc(&ref_tri_, sizeof(uint32_t) * m));
    QUASI_TRY_CUDA(cudaMalloc(&ref_box_, sizeof(float4) * 2 * m));
    ref_capacity_ = m;
    return cudaSuccess;
}

cudaError_t LbvhBuilder::build(const float4* tri_in, uint32_t n, const int* emitters, uint32_t n_emit,
                               cudaStream_t stream, KernelProfiler& prof, uint32_t* err) {
    // triangles split into two leaf references: a fixed share, so the leaf count is known here
    const uint32_t split =
        n >= k_split_min_tris ? static_cast<uint32_t>(uint64_t(n) * uint32_t(split_percent_) / 100u) : 0u;
    QUASI_TRY_CUDA(reserve(n + split));
    n_ = n + split;
    n_tris_ = n;
    if (n == 0) return cudaSuccess;
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "tri_planes", stream,
                                (k_tri_planes<<<ceil_div(n, 256), 256, 0, stream>>>(tri_in, n, tri_plane_))));
    if (n_emit > 0) {
        if (n_emit > emit_capacity_) {
            if (emit_tab_) cudaFree(emit_tab_);
            emit_tab_ = nullptr;
            emit_capacity_ = 0;
            QUASI_TRY_CUDA(cudaMalloc(&emit_tab_, sizeof(float4) * 5 * n_emit));
            emit_capacity_ = n_emit;
        }
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "emit_table", stream,
                                    (k_emit_table<<<ceil_div(n_emit, 256), 256, 0, stream>>>(tri_in, emitters, n_emit,
                                                                                             emit_tab_))));
    }
    RefView rv;
    if (split > 0) {
        QUASI_TRY_CUDA(reserve_refs(n + split));
        // triangles in ascending order of the empty area of their boxes (keys_ and order_ are
        // free until the Morton sort); the last `split` of them are cut
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_split_keys", stream,
                                    (k_split_keys<<<ceil_div(n, 256), 256, 0, stream>>>(tri_in, n, keys_, order_))));
        QUASI_TRY_CUDA(radix_sort_pairs(keys_, order_, n, 32, sort_, stream, prof));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_make_refs", stream,
                                    (k_make_refs<<<ceil_div(n, 256), 256, 0, stream>>>(tri_in, n, split, order_,
                                                                                       ref_tri_, ref_box_))));
        rv = RefView{ref_tri_, ref_box_};
    }
    n = n_;  // from here on the leaves
    const int parts = static_cast<int>(std::min<uint32_t>(k_bounds_blocks, ceil_div(n, 256)));
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_bounds", stream,
                                (k_bounds_partial<<<parts, 256, 0, stream>>>(tri_in, rv, n, partial_))));
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_bounds_final", stream,
                                (k_bounds_final<<<1, 32, 0, stream>>>(partial_, parts, bounds_))));
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_morton", stream,
                                (k_morton<<<ceil_div(n, 256), 256, 0, stream>>>(tri_in, rv, n, bounds_, morton_,
                                                                                keys_, order_))));
    QUASI_TRY_CUDA(radix_sort_pairs(keys_, order_, n, 30, sort_, stream, prof));
    if (n > 1) {
        QUASI_TRY_CUDA(cudaMemsetAsync(flags_, 0, sizeof(uint32_t) * (n - 1), stream));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_karras", stream,
                                    (k_karras<<<ceil_div(n - 1, 256), 256, 0, stream>>>(keys_, static_cast<int>(n),
                                                                                        nodes_, parent_))));
    }
    QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_leaf_boxes", stream,
                                (k_leaf_boxes<<<ceil_div(n, 256), 256, 0, stream>>>(
                                    tri_in, rv, order_, static_cast<int>(n), parent_, nodes_, flags_, tris_, err))));
    if (sah_cluster_ >= 3 && n >= 3) {
        QUASI_TRY_CUDA(cudaMemsetAsync(sah_count_, 0, sizeof(int), stream));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_sah_roots", stream,
                                    (k_sah_roots<<<ceil_div(n - 1, 256), 256, 0, stream>>>(
                                        nodes_, parent_, static_cast<int>(n), sah_cluster_, sah_roots_, sah_count_))));
        // at most one root per 3 leaves; 8 per block, a block per 24 leaves up to a full GPU
        const uint32_t blocks = std::max<uint32_t>(1, std::min<uint32_t>(ceil_div(n, 24), 152u * 8u));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_sah_rebuild", stream,
                                    (k_sah_rebuild<<<blocks, 256, 0, stream>>>(tri_in, rv, order_, nodes_, parent_,
                                                                               static_cast<int>(n), sah_roots_,
                                                                               sah_count_, err))));
    }
    const uint32_t internal = n > 1 ? n - 1 : 1;
    if (dp_collapse_ && n >= 2) {
        QUASI_TRY_CUDA(cudaMemsetAsync(flags_, 0, sizeof(uint32_t) * (n - 1), stream));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_collapse_dp", stream,
                                    (k_collapse_dp<<<ceil_div(n, 256), 256, 0, stream>>>(
                                        nodes_, parent_, static_cast<int>(n), flags_, dp_cost_, dp_dec_, err))));
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_collapse8", stream,
                                    (k_collapse8<true><<<ceil_div(internal, 128), 128, 0, stream>>>(
                                        nodes_, static_cast<int>(internal), dp_dec_, wide_))));
    } else {
        QUASI_TRY_CUDA(QUASI_LAUNCH(prof, "bvh_collapse8", stream,
                                    (k_collapse8<false><<<ceil_div(internal, 128), 128, 0, stream>>>(
                                        nodes_, static_cast<int>(internal), nullptr, wide_))));
    }
    return cudaSuccess;
}

cudaError_t LbvhBuilder::read(uint32_t* morton, uint32_t* order, int32_t* children, float* boxes, float* bounds,
                              cudaStream_t stream) const {
    QUASI_TRY_CUDA(cudaStreamSynchronize(stream));
    if (n_ == 0) return cudaSuccess;
    if (morton) QUASI_TRY_CUDA(cudaMemcpy(morton, morton_, sizeof(uint32_t) * n_, cudaMemcpyDeviceToHost));
    if (order) QUASI_TRY_CUDA(cudaMemcpy(order, order_, sizeof(uint32_t) * n_, cudaMemcpyDeviceToHost));
    if (bounds) QUASI_TRY_CUDA(cudaMemcpy(bounds, bounds_, sizeof(float) * 6, cudaMemcpyDeviceToHost));
    const uint32_t nodes = n_ > 1 ? n_ - 1 : 1;
    if (children || boxes) {
        std::vector<float4> host(4 * nodes);
        QUASI_TRY_CUDA(cudaMemcpy(host.data(), nodes_, sizeof(float4) * 4 * nodes, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < nodes; ++i) {
            const float4 n0 = host[4 * i], n1 = host[4 * i + 1], n2 = host[4 * i + 2], n3 = host[4 * i + 3];
            if (children) {
                int32_t c0, c1;
                std::memcpy(&c0, &n3.x, 4);
                std::memcpy(&c1, &n3.y, 4);
                children[2 * i] = c0;
                children[2 * i + 1] = c1;
            }
            if (boxes) {
                float* b = boxes + 12 * i;
                b[0] = n0.x; b[1] = n0.z; b[2] = n2.x; b[3] = n0.y; b[4] = n0.w; b[5] = n2.y;
                b[6] = n1.x; b[7] = n1.z; b[8] = n2.z; b[9] = n1.y; b[10] = n1.w; b[11] = n2.w;
            }
        }
    }
    return cudaSuccess;
}

cudaError_t LbvhBuilder::read_wide(uint32_t* words, cudaStream_t stream) const {
    QUASI_TRY_CUDA(cudaStreamSynchronize(stream));
    if (n_ == 0 || !words) return cudaSuccess;
    const uint32_t nodes = n_ > 1 ? n_ - 1 : 1;
    QUASI_TRY_CUDA(cudaMemcpy(words, wide_, sizeof(float4) * k_wide_node_f4 * nodes, cudaMemcpyDeviceToHost));
    return cudaSuccess;
}

}  // namespace quasi

// Standalone sort entry point (allocates its own scratch for the call).
extern "C" __attribute__((visibility("default"))) int Q_cuda_radix_sort_pairs(uint32_t* device_keys,
                                                                              uint32_t* device_values, uint32_t n,
                                                                              uint32_t key_bits, void* stream) {
    if (n == 0) return 0;
    if (!device_keys || !device_values || key_bits == 0 || key_bits > 32) return -1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    quasi::RadixSortScratch scratch;
    quasi::KernelProfiler prof;
    cudaError_t e = quasi::radix_sort_reserve(scratch, n);
    if (e == cudaSuccess) e = quasi::radix_sort_pairs(device_keys, device_values, n, static_cast<int>(key_bits), scratch, s, prof);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    quasi::radix_sort_release(scratch);
    return e == cudaSuccess ? 0 : (e == cudaErrorMemoryAllocation ? -3 : -2);
}
