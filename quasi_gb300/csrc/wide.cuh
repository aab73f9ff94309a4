// wide.cuh - 8-wide BVH collapsed from the binary LBVH, and its traversal (FP32).
//
// The binary LBVH (bvh.cuh) is the bit-exact structure; this is a derived traversal
// structure built from it in one kernel (k_collapse8, bvh.cu) after every LBVH build:
//
//   * Every binary internal node b gets a wide record at index b, computed from b's subtree
//     alone: start from b's two children and repeatedly open the internal child of largest
//     surface area (ties to the lower entry) until 8 children or none left to open.
//     Children whose subtree holds at most k_wide_leaf_max triangles become leaves: a
//     leaf is a run of consecutive triangles of the leaf-order array (a binary subtree
//     covers a contiguous Morton range), so the triangle array is shared with the binary
//     BVH. Larger internal children refer to their own wide record by binary index.
//     Only records reachable from record 0 are ever visited; the others are never read.
//   * Child boxes are quantised to 8 bits per plane on a per-node power-of-two grid with
//     the lower planes rounded down and the upper planes rounded up, so each decoded box
//     contains the exact child box (Ylitie, Karras and Laine 2017, "Efficient incoherent
//     ray traversal on GPUs through compressed wide BVHs").
//   * Children are placed in slots by direction: slot bit a set means "on the negative
//     side of axis a" (x = bit 0, y = 1, z = 2). A ray whose direction octant is `oct`
//     ranks slot s by s ^ oct, so the children it reaches first are taken first.
//
// Record layout, 96 bytes (6 x float4):
//   w0 = (p.x, p.y, p.z, ex | ey << 8 | ez << 16 | imask << 24)
//        p = grid origin, scale per axis 2^(e - 127), imask = slots holding internal children
//   w1 = x planes: lo[0..3], lo[4..7], hi[0..3], hi[4..7] (one byte per slot)
//   w2 = y planes, w3 = z planes (same packing)
//   w4 = refs[0..3], w5 = refs[4..7]
//        ref >= 0: internal child, the wide record of binary node `ref`
//        ref < 0:  leaf, ~ref = pos << 2 | code, triangles pos .. pos + ((code + 1) & 3) - 1
//                  (code 3 = an empty slot: lo planes 255, hi planes 0, no triangles)
//
// Closest hit is the smallest t, and an exact tie goes to the smaller original index, as in
// the binary traversal (trace.cuh), so both return the same triangle. Child boxes are padded
// by the scene's Delta (scene_box_pad) before quantisation, and triangle tests classify
// their candidates (robust.cuh): an undecided candidate is recorded for the fixup kernel.
#pragma once

#include "trace.cuh"

namespace quasi {

// Triangles per leaf. Runs of 2-3 triangles save record visits, but the union box of a
// Morton run is much larger than its triangles' boxes. On the 1M soup (1080p frame),
// closest-hit visits / triangle tests per ray and Mrays/s: one triangle 24.0 / 5.3, 1442;
// up to two 23.0 / 6.7, 1381; up to three 21.4 / 10.8, 1264. Every leaf holds one triangle.
constexpr int k_wide_leaf_max = 1;
constexpr int k_wide_stack = 96;      // (ref, t_near) entries per ray
constexpr int k_wide_node_f4 = 6;     // float4 per wide record
constexpr int k_wide_empty_ref = ~3;  // leaf with code 3: no triangles
// Minimum resident 256-thread blocks per SM asked of the compiler for the 8-wide trace
// kernels, a register cap (4 -> 64 registers per thread). Uncapped, they take 93 registers
// and 5 blocks of 128 threads fit an SM; at 64 registers (no spills) 8 fit, and the
// 1M-triangle frame renders 18% faster on GB300. Tighter caps spill: 56 registers (9 blocks
// of 128) cost 3%, 51 (10 blocks) 11%.
#ifndef QUASI_WIDE_MIN_BLOCKS
#define QUASI_WIDE_MIN_BLOCKS 4
#endif

// Stack entries per ray that the refill traversal keeps in shared memory, for closest-hit
// and for any-hit rays; deeper entries go to a thread-local array. Local-memory stack
// traffic shares L1 with the records, and a pop is a dependent load before the next record
// fetch. On the 1M soup 99% of rays never stack more than 15 entries. Measured per frame
// (1080p, 64 spp, 128-thread blocks), closest-hit kernel time by entries: none 334.6 ms,
// 10: 317.3, 12: 314.1, 16: 310.4, 20: 312.9; any-hit: none 142.4, 10: 138.7, 12: 136.0,
// 16: 130.7, 20: 128.0, 24: 134.9 (deeper shared stacks take L1 capacity the records use).
// With 16 and 20 the frame renders at 1389 Mrays/s against 1289 with local stacks only.
#ifndef QUASI_WIDE_SMEM_STACK
#define QUASI_WIDE_SMEM_STACK 16
#endif
#ifndef QUASI_WIDE_SMEM_STACK_ANY
#define QUASI_WIDE_SMEM_STACK_ANY 20
#endif
template <bool ANY>
__host__ __device__ constexpr int wide_smem_stack() {
    return ANY ? QUASI_WIDE_SMEM_STACK_ANY : QUASI_WIDE_SMEM_STACK;
}
static_assert(wide_smem_stack<false>() >= 0 && wide_smem_stack<false>() < k_wide_stack &&
                  wide_smem_stack<true>() >= 0 && wide_smem_stack<true>() < k_wide_stack,
              "shared stack entries (the thread-local part keeps at least one)");
static_assert(sizeof(int2) * wide_smem_stack<false>() * 256 <= 48 * 1024 &&
                  sizeof(int2) * wide_smem_stack<true>() * 256 <= 48 * 1024,
              "a 256-thread trace block stays within the default dynamic shared memory limit");

// Dynamic shared memory a refill trace block of `threads` threads needs for its stacks.
template <bool ANY>
constexpr size_t wide_stack_smem_bytes(int threads) {
    return sizeof(int2) * static_cast<size_t>(wide_smem_stack<ANY>()) * static_cast<size_t>(threads);
}

// Traversal stack of one ray: entries below Sh in shared memory, warp-major (entry i of a
// lane at slot[32 i], so the lanes of a warp touch 32 consecutive int2 whatever their
// depths: no bank conflicts), the rest in a thread-local array.
template <int Sh>
struct WideStack {
    int2* slot;
    int2 loc[k_wide_stack - Sh];
    __device__ __forceinline__ void put(int i, int2 e) {
        if (Sh > 0 && i < Sh)
            slot[32 * i] = e;
        else
            loc[i - Sh] = e;
    }
    __device__ __forceinline__ int2 get(int i) const {
        if (Sh > 0 && i < Sh) return slot[32 * i];
        return loc[i - Sh];
    }
};

// This thread's shared slots in a block launched with wide_stack_smem_bytes<ANY>(blockDim.x)
// of dynamic shared memory.
template <bool ANY>
__device__ __forceinline__ int2* wide_stack_slot() {
    extern __shared__ int2 s_wide_stack[];
    return s_wide_stack + (threadIdx.x >> 5) * (32 * wide_smem_stack<ANY>()) + (threadIdx.x & 31);
}

// Record visits a lane makes between two refill checks of its warp (ballot, fetch, vote),
// for closest-hit and for any-hit rays. Checking after every visit spends issue slots on the
// votes; after every k-th visit a lane whose ray ended idles for at most k - 1 visits. 1080p
// frame of the 1M soup, both kinds alike: 1 visit 1420 Mrays/s, 2: 1444, 3: 1429, 4: 1437.
// With the refined hierarchy and closest-hit at 2, any-hit at 1, 2, 3, 4, 5, 6: shadow traces
// of 113.5, 111.5, 109.9, 108.4, 109.5 and 110.5 ms per frame (1547.5 Mrays/s at 4);
// closest-hit at 3 (any-hit 3) took 299.4 instead of 296.5 ms.
#ifndef QUASI_WIDE_VISITS_PER_CHECK
#define QUASI_WIDE_VISITS_PER_CHECK 2
#endif
#ifndef QUASI_WIDE_VISITS_PER_CHECK_ANY
#define QUASI_WIDE_VISITS_PER_CHECK_ANY 4
#endif
template <bool ANY>
__host__ __device__ constexpr int wide_visits_per_check() {
    return ANY ? QUASI_WIDE_VISITS_PER_CHECK_ANY : QUASI_WIDE_VISITS_PER_CHECK;
}

// Marks a finished traversal in WideRay::node (no record index is negative).
constexpr int k_wide_done = static_cast<int>(0x80000000u);

// Idle lanes that make a warp of the 8-wide trace kernels fetch new rays (default).
constexpr int k_wide_refill_lanes = 4;

// Selects a[k] of eight values held in registers (k in 0..7) without local memory.
template <class T>
__device__ __forceinline__ T sel8(const T (&a)[8], uint32_t k) {
    const bool b0 = k & 1u, b1 = k & 2u, b2 = k & 4u;
    const T c0 = b0 ? a[1] : a[0], c1 = b0 ? a[3] : a[2], c2 = b0 ? a[5] : a[4], c3 = b0 ? a[7] : a[6];
    const T d0 = b1 ? c1 : c0, d1 = b1 ? c3 : c2;
    return b2 ? d1 : d0;
}

// Maps an 8-bit mask in slot space to rank space (bit s -> bit s ^ oct).
__device__ __forceinline__ uint32_t mask_xor_permute(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

// Byte k of w as the float 2^23 + byte: one byte permute into the mantissa of 2^23, exact.
__device__ __forceinline__ float byte_f23(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7650u | static_cast<uint32_t>(k)));
}

// Two FP32 lanes in one 64-bit register and the paired arithmetic of sm_100 and later
// (sub/fma .rn.f32x2): each lane rounds exactly as the scalar instruction does.
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Three-input minimum and maximum (one instruction each on sm_100 and later).
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Tests the triangle of one leaf (one-triangle leaves: a leaf that passed its box test
// holds exactly one triangle, empty slots never pass); returns true when the traversal ends
// (an any-hit query answered, or an undecided candidate flagged the ray).
// ROBUST: undecided candidates are re-decided exactly (tri_in: original-order vertices, xr:
// the ray's exact geometry).
template <bool ANY, bool STATS, bool ROBUST = false, class X = ExactNone>
__device__ __forceinline__ bool wide_leaf(const float4* __restrict__ tris, const RayInv& r, int ref, int exclude,
                                          HitBest& b, TraceCounters& cnt, const float4* __restrict__ tri_in = nullptr,
                                          const X& xr = X{}) {
    static_assert(k_wide_leaf_max == 1, "wide_leaf tests one triangle per leaf");
    if (STATS) ++cnt.tris;
    return leaf_test<ANY, ROBUST>(tris, tri_in, xr, r, static_cast<uint32_t>(~ref) >> 2, exclude, b);
}

// Traversal state of one ray over the 8-wide records (the stack lives beside it).
struct WideRay {
    RayInv r;
    uint32_t oct;   // direction octant: bit a set where component a is negative
    int exclude;
    HitBest b;      // closest certain hit so far and the undecided candidate met, if any
    int node;       // record to visit next, or k_wide_done
    int sp;
    uint32_t budget;
};

__device__ __forceinline__ void wide_begin(WideRay& q, float3 o, float3 d, float tmax, int exclude, uint32_t n_tris) {
    q.r = make_ray(o, d);
    // octant from the reciprocals, which carry the sign of a zero component (-0 -> -1e20)
    q.oct = (q.r.inv.x < 0.0f ? 1u : 0u) | (q.r.inv.y < 0.0f ? 2u : 0u) | (q.r.inv.z < 0.0f ? 4u : 0u);
    q.exclude = exclude;
    q.b = hit_begin(tmax);
    q.node = n_tris == 0 ? k_wide_done : 0;
    q.sp = 0;
    q.budget = 2u * n_tris + 64u;
}

// Pops the nearest stacked entry entered before the closest hit's t plus its error bound,
// or k_wide_done.
template <class Stack>
__device__ __forceinline__ int wide_pop(WideRay& q, const Stack& stack) {
    const float tcull = q.b.hi;
    while (q.sp > 0) {
        const int2 e = stack.get(--q.sp);
        if (__int_as_float(e.y) < tcull) return e.x;
    }
    return k_wide_done;
}

// One record visit: tests the 8 child boxes, the triangles of the leaves hit, pushes the
// internal children hit but the first-ranked, and moves to the next record. Returns true
// when the traversal has finished (q holds the result). Testing at most one triangle per
// visit and stacking the other leaves (each loop turn then costs one triangle test, not the
// busiest lane's count) was measured 7% slower on the 1M soup: the extra stack traffic and
// loop turns cost more than the divergence they remove.
template <bool ANY, bool STATS, class Stack, bool ROBUST = false, class X = ExactNone>
__device__ __forceinline__ bool wide_visit(const float4* __restrict__ wide, const float4* __restrict__ tris,
                                           WideRay& q, Stack& stack, uint32_t& err, TraceCounters& cnt,
                                           const float4* __restrict__ tri_in = nullptr, const X& xr = X{}) {
    if (q.node == k_wide_done) return true;
    if (--q.budget == 0u) {
        err |= k_deverr_traversal;
        q.node = k_wide_done;
        return true;
    }
    if (STATS) ++cnt.nodes;
    const RayInv& r = q.r;
    const bool nx = q.oct & 1u, ny = q.oct & 2u, nz = q.oct & 4u;
    const float4* w = wide + k_wide_node_f4 * static_cast<size_t>(q.node);
    const float4 w0 = __ldg(w), w1 = __ldg(w + 1), w2 = __ldg(w + 2), w3 = __ldg(w + 3);
    const int4 w4 = __ldg(reinterpret_cast<const int4*>(w + 4));
    const int4 w5 = __ldg(reinterpret_cast<const int4*>(w + 5));
    const uint32_t hdr = __float_as_uint(w0.w);
    const float sx = __uint_as_float((hdr & 0xffu) << 23);
    const float sy = __uint_as_float(((hdr >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((hdr >> 16) & 0xffu) << 23);
    const uint32_t imask = hdr >> 24;
    const float az = sz * r.inv.z, bz = (w0.z - r.o.z) * r.inv.z;
    const uint64_t azz = f2_pack(az, az), bzz = f2_pack(bz, bz);
    const uint64_t axy = f2_pack(sx * r.inv.x, sy * r.inv.y);
    const uint64_t bxy = f2_pack((w0.x - r.o.x) * r.inv.x, (w0.y - r.o.y) * r.inv.y);
    // near planes are the lower ones along a positive direction component
    const uint32_t wx[4] = {__float_as_uint(w1.x), __float_as_uint(w1.y), __float_as_uint(w1.z), __float_as_uint(w1.w)};
    const uint32_t wy[4] = {__float_as_uint(w2.x), __float_as_uint(w2.y), __float_as_uint(w2.z), __float_as_uint(w2.w)};
    const uint32_t wz[4] = {__float_as_uint(w3.x), __float_as_uint(w3.y), __float_as_uint(w3.z), __float_as_uint(w3.w)};
    const uint32_t nx0 = nx ? wx[2] : wx[0], nx1 = nx ? wx[3] : wx[1], fx0 = nx ? wx[0] : wx[2], fx1 = nx ? wx[1] : wx[3];
    const uint32_t ny0 = ny ? wy[2] : wy[0], ny1 = ny ? wy[3] : wy[1], fy0 = ny ? wy[0] : wy[2], fy1 = ny ? wy[1] : wy[3];
    const uint32_t nz0 = nz ? wz[2] : wz[0], nz1 = nz ? wz[3] : wz[1], fz0 = nz ? wz[0] : wz[2], fz1 = nz ? wz[1] : wz[3];
    float tn[8];
    uint32_t hit = 0;
    // any-hit rays: the internal child whose box covers the longest stretch of the segment
    float best_ov = -1.0f;
    uint32_t best_slot = 0;
    const float tcull = q.b.hi;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t nxw = k < 4 ? nx0 : nx1, fxw = k < 4 ? fx0 : fx1;
        const uint32_t nyw = k < 4 ? ny0 : ny1, fyw = k < 4 ? fy0 : fy1;
        const uint32_t nzw = k < 4 ? nz0 : nz1, fzw = k < 4 ? fz0 : fz1;
        const int b = k & 3;
        // plane distance q * a + b with q = (2^23 + q) - 2^23 (exact), two planes per paired
        // subtract and FMA (near x and y, far x and y, near and far z): the same bits as
        // fmaf(q, a, b) per plane, in fewer instructions than integer-to-float conversions
        // and scalar FMAs (1288 vs 1281 Mrays/s on the 1M soup, before the shared stacks)
        float tnx, tny, tfx, tfy;
        const uint64_t c23 = 0x4B0000004B000000ull;  // (2^23, 2^23)
        f2_unpack(f2_fma(f2_sub(f2_pack(byte_f23(nxw, b), byte_f23(nyw, b)), c23), axy, bxy), tnx, tny);
        f2_unpack(f2_fma(f2_sub(f2_pack(byte_f23(fxw, b), byte_f23(fyw, b)), c23), axy, bxy), tfx, tfy);
        float tnz, tfz;
        f2_unpack(f2_fma(f2_sub(f2_pack(byte_f23(nzw, b), byte_f23(fzw, b)), c23), azz, bzz), tnz, tfz);
        const float tnear = fmax3(tnx, tny, fmaxf(tnz, 0.0f));
        const float tfar = fmin3(tfx, tfy, fminf(tfz, tcull));
        tn[k] = tnear;
        // the decoded boxes carry the scene's spatial padding: no relative slack needed
        const bool h = tnear <= tfar;
        hit |= (h ? 1u : 0u) << k;
        if (ANY) {
            const float ov = tfar - tnear;
            if (h && ((imask >> k) & 1u) && ov > best_ov) {
                best_ov = ov;
                best_slot = k;
            }
        }
    }
    const int refs[8] = {w4.x, w4.y, w4.z, w4.w, w5.x, w5.y, w5.z, w5.w};
    uint32_t im = mask_xor_permute(hit & imask, q.oct);
    // leaves first: a hit found here shortens every interval tested after it. Every leaf hit
    // is tested (no culling by entry distance) and the closest-hit rule does not depend on
    // the order, so they go in slot order, without the rank permutation.
    uint32_t lm = hit & ~imask;
    while (lm) {
        const uint32_t s = __ffs(lm) - 1;
        lm &= lm - 1u;
        if (wide_leaf<ANY, STATS, ROBUST>(tris, r, sel8(refs, s), q.exclude, q.b, cnt, tri_in, xr)) {
            q.node = k_wide_done;
            return true;
        }
    }
    int next = k_wide_done;
    if (ANY && im) {
        // Any-hit: visit next the internal child whose box covers the longest stretch of the
        // segment (where an occluder is likeliest), push the others lowest rank first. On
        // occluded shadow segments through the 1M soup this visits 17% fewer records than
        // nearest-first. Also stacking the runner-up on top saved 3% more visits but its
        // bookkeeping in the eight-child loop cost more (frame 1% slower).
        next = sel8(refs, best_slot);
        im &= ~(1u << (best_slot ^ q.oct));
        while (im) {
            const uint32_t p = __ffs(im) - 1;
            im &= im - 1u;
            const uint32_t s = p ^ q.oct;
            if (q.sp >= k_wide_stack) {
                err |= k_deverr_stack;
                q.node = k_wide_done;
                return true;
            }
            stack.put(q.sp++, make_int2(sel8(refs, s), __float_as_int(sel8(tn, s))));
        }
    }
    // internal children: push all but the first-ranked, lowest rank first
    while (im) {
        const uint32_t p = __ffs(im) - 1;
        im &= im - 1u;
        const uint32_t s = p ^ q.oct;
        const float t = sel8(tn, s);
        if (t >= q.b.hi) continue;
        const int ref = sel8(refs, s);
        if (im) {
            if (q.sp >= k_wide_stack) {
                err |= k_deverr_stack;
                q.node = k_wide_done;
                return true;
            }
            stack.put(q.sp++, make_int2(ref, __float_as_int(t)));
        } else {
            next = ref;
        }
    }
    if (next == k_wide_done) next = wide_pop(q, stack);
    q.node = next;
    return next == k_wide_done;
}

// Whole-ray traversal of the 8-wide BVH (fast mode); same contract as trace_bvh
// (trace.cuh): ANY = true stops at the first certain hit with t in (0, tmax); the result
// carries the undecided candidate met, if any.
template <bool ANY, bool STATS>
__device__ __forceinline__ TraceResult trace_wide(const float4* __restrict__ wide, const float4* __restrict__ tris,
                                                  uint32_t n_tris, float3 o, float3 d, float tmax, int exclude,
                                                  uint32_t& err, TraceCounters& cnt) {
    WideRay q;
    wide_begin(q, o, d, tmax, exclude, n_tris);
    WideStack<0> stack;
    while (!wide_visit<ANY, STATS>(wide, tris, q, stack, err, cnt)) {
    }
    return trace_result(q.b);
}

// Whole-ray traversal of the 8-wide BVH with exact re-decisions of undecided candidates
// (xr: the ray's exact geometry, tri_in: original-order vertices); the result is final.
template <bool ANY, class X>
__device__ __forceinline__ HitBest trace_wide_exact(const float4* __restrict__ wide, const float4* __restrict__ tris,
                                                    const float4* __restrict__ tri_in, uint32_t n_tris, float3 o,
                                                    float3 d, float tmax, int exclude, const X& xr, uint32_t& err) {
    WideRay q;
    wide_begin(q, o, d, tmax, exclude, n_tris);
    WideStack<0> stack;
    TraceCounters cnt;
    while (!wide_visit<ANY, false, WideStack<0>, true>(wide, tris, q, stack, err, cnt, tri_in, xr)) {
    }
    return q.b;
}

// Warp-batch persistent traversal of a ray queue over the 8-wide records: a warp takes 32
// consecutive rays with one atomic and traces each to completion (Job as in trace_batches).
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_batches_wide(Job& job, const float4* __restrict__ wide,
                                                   const float4* __restrict__ tris, uint32_t n_tris, int n,
                                                   int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
    while (true) {
        int base = 0;
        if (lane == 0) base = atomicAdd(fetch, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int i = base + lane;
        if (i < n) {
            float3 o, d;
            float tmax;
            int exclude;
            job.load(i, o, d, tmax, exclude);
            finish_ray(job, i, trace_wide<ANY, STATS>(wide, tris, n_tris, o, d, tmax, exclude, err, cnt));
        }
    }
}

// Persistent traversal of a ray queue with per-lane refill: once `refill` lanes of a warp
// are idle they take the next rays with one atomic, while the other lanes carry on with
// their own rays (refill = 32 waits for the whole warp). Job as in trace_batches. Every
// lane of the warp must call this (it uses full-warp votes), and the block must be launched
// with wide_stack_smem_bytes<ANY>(blockDim.x) of dynamic shared memory.
template <bool ANY, bool STATS, class Job>
__device__ __forceinline__ void trace_wide_refill(Job& job, const float4* __restrict__ wide,
                                                  const float4* __restrict__ tris, uint32_t n_tris, int n, int refill,
                                                  int* __restrict__ fetch, uint32_t& err, TraceCounters& cnt) {
    const int lane = threadIdx.x & 31;
    WideRay q;
    WideStack<wide_smem_stack<ANY>()> stack;
    stack.slot = wide_stack_slot<ANY>();
    bool active = false, exhausted = false;
    int idx = 0;
    while (true) {
        const uint32_t idle = __ballot_sync(0xffffffffu, !active);
        if (!exhausted && __popc(idle) >= refill) {
            const int leader = __ffs(idle) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(fetch, __popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            exhausted = base + __popc(idle) >= n;
            if (!active) {
                idx = base + __popc(idle & lanemask_lt());
                if (idx < n) {
                    float3 o, d;
                    float tmax;
                    int exclude;
                    job.load(idx, o, d, tmax, exclude);
                    wide_begin(q, o, d, tmax, exclude, n_tris);
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        bool done = false;
        if (active) {
#pragma unroll 1
            for (int i = 0; i < wide_visits_per_check<ANY>(); ++i) {
                done = wide_visit<ANY, STATS>(wide, tris, q, stack, err, cnt);
                if (done) break;
            }
        }
        if (done) {
            finish_ray(job, idx, trace_result(q.b));
            active = false;
        }
    }
}

}  // namespace quasi
