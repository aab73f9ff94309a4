// bvh.cuh - linear BVH (LBVH) built on the GPU every frame.
//
// Pipeline (one scene of n triangles, all integer steps bit-exact against the oracle):
//   1. centroid bounds   c = ((v0 + v1) + v2) * (1/3) in FP32, min/max reduction
//   2. Morton-30 codes    q = min(max((c - lo) * (1/(hi - lo)) * 1024, 0), 1023) per axis,
//                         code = (expand(qx) << 2) | (expand(qy) << 1) | expand(qz)
//   3. stable LSD radix sort of (code, index) on 8-bit digits
//   4. Karras 2012 hierarchy (index-augmented common-prefix for duplicate codes)
//   5. bottom-up child boxes with per-node arrival counters; triangles gathered into
//      leaf order as {v0, orig index}, {e1}, {e2}
//   6. the 8-wide traversal records collapsed from the binary nodes (wide.cuh)
//   7. per-triangle shading geometry: the unit normal of cross(e1, e2) and its length in
//      double-float, read by every shading step instead of recomputing them
// The leaves are references to triangles. By default the triangles whose boxes leave the
// most surface area empty are first split in two (early split clipping, bvh.cu), so a scene
// of n triangles has more than n leaves; with splitting off (set_split_percent(0)) leaf i
// of the Morton order is a triangle and steps 1-5 are the oracle's, bit for bit.
//
// Node layout, 64 bytes (4 x float4), child boxes stored in the parent:
//   n0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   n1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   n2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   n3 = (child0, child1, first, last) as ints; child >= 0 internal node, child < 0 leaf ~pos;
//        the node covers leaves first .. last (a contiguous Morton range).
// A scene of one triangle gets a single node whose second child has an empty box.
#pragma once

#include "launch.hpp"

#include <cuda_runtime.h>
#include <cstdint>

namespace quasi {

// Sorts (keys, values) by the low key_bits of keys; stable. keys/values and the alt
// buffers are swapped internally; on return the sorted data is in keys/values.
struct RadixSortScratch {
    uint32_t* keys_alt = nullptr;
    uint32_t* vals_alt = nullptr;
    uint32_t* hist = nullptr;
    uint32_t capacity = 0;
    uint32_t hist_capacity = 0;
};

size_t radix_sort_hist_entries(uint32_t n);
cudaError_t radix_sort_reserve(RadixSortScratch& s, uint32_t n);
void radix_sort_release(RadixSortScratch& s);
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int key_bits,
                             RadixSortScratch& s, cudaStream_t stream, KernelProfiler& prof);

// Percentage of a scene's triangles whose boxes are split in two before the hierarchy is
// built (the ones whose boxes leave the most surface area empty). Benchmark frame (1M soup,
// 1080p, 64 spp), Mrays/s by share: 0 %: 1539.3, 10 %: 1584.9, 20 %: 1593.7, 30 %: 1597.1,
// 40 %: 1597.5, 50 %: 1592.5, 70 %: 1582.5 (triangle tests per closest-hit ray 5.54, 5.12,
// 4.92, 4.77, 4.66, 4.57, 4.43; the build 2.4 ms at 0 %, 3.8 ms at 30 %).
#ifndef QUASI_BVH_SPLIT_PERCENT
#define QUASI_BVH_SPLIT_PERCENT 30
#endif
// Scenes below this many triangles are not split: their builds are launch-bound, and the
// split's key sort and references (14 more launches) cost the 10k-triangle soup's frame
// (512^2, 16 spp, LBVH rebuilt every frame) 2.69 -> 2.82 ms, more than its traversal gained.
constexpr uint32_t k_split_min_tris = 1u << 17;

struct LbvhView {
    const float4* nodes = nullptr;  // 4 float4 per internal node
    const float4* tris = nullptr;   // 3 float4 per leaf (triangle reference) in leaf order
    uint32_t tri_count = 0;         // leaves
    uint32_t node_count = 0;
    const float4* tree = nullptr;   // top levels in breadth-first order (for shared memory)
    int tree_n = 0;                 // nodes in `tree`
    const float4* wide = nullptr;   // 8-wide records (wide.cuh), one per internal node
    const float4* tri_plane = nullptr; // per triangle (original order), 2 float4: the unit normal
                                       // of cross(e1, e2) and the plane offset n.v0, double-float
    const float4* emit_tab = nullptr;  // per emitter slot, 5 float4 (k_emit_table)
};

class LbvhBuilder {
public:
    LbvhBuilder() = default;
    ~LbvhBuilder() { release(); }
    LbvhBuilder(const LbvhBuilder&) = delete;
    LbvhBuilder& operator=(const LbvhBuilder&) = delete;

    cudaError_t reserve(uint32_t n);
    void release();

    // tri_in: 3 float4 per triangle (v0, v1, v2; w ignored), original order, device.
    // emitters: the n_emit emitting triangles (indices into tri_in), device; their
    // light-sampling records are rebuilt with the hierarchy.
    // err: device word that receives QUASI_DEVERR_* bits if the hierarchy is malformed.
    cudaError_t build(const float4* tri_in, uint32_t n, const int* emitters, uint32_t n_emit, cudaStream_t stream,
                      KernelProfiler& prof, uint32_t* err);

    // Leaves of the largest subtrees rebuilt with the surface-area split after the Morton
    // hierarchy (3..32; below 3: the plain LBVH).
    void set_sah_cluster(int leaves) { sah_cluster_ = leaves < 3 ? 0 : (leaves > 32 ? 32 : leaves); }
    // The 8-wide records' children from the surface-area-optimal spread (true) or by opening
    // the largest child greedily (false).
    void set_dp_collapse(bool on) { dp_collapse_ = on; }
    // Percentage (0..100) of the triangles split into two leaf references before the build,
    // in scenes of at least k_split_min_tris triangles.
    void set_split_percent(int p) { split_percent_ = p < 0 ? 0 : (p > 100 ? 100 : p); }
    // Whether the last build split triangles (its leaves then outnumber the triangles).
    bool split_active() const { return n_ != n_tris_; }

    // Copies the top max_nodes internal nodes (breadth first) for staging in shared memory.
    cudaError_t build_treelet(int max_nodes, cudaStream_t stream, KernelProfiler& prof);

    LbvhView view() const {
        return LbvhView{nodes_, tris_, n_, n_ == 0 ? 0u : (n_ > 1 ? n_ - 1 : 1u), tree_, tree_n_, wide_, tri_plane_,
                        emit_tab_};
    }

    // Debug copies to host (stream-synchronous).
    cudaError_t read(uint32_t* morton, uint32_t* order, int32_t* children, float* boxes,
                     float* bounds, cudaStream_t stream) const;
    // The 8-wide records as 24 words per internal node (stream-synchronous).
    cudaError_t read_wide(uint32_t* words, cudaStream_t stream) const;

private:
    cudaError_t reserve_refs(uint32_t m);

    uint32_t n_ = 0;                 // leaves (triangle references)
    uint32_t n_tris_ = 0;            // triangles
    uint32_t capacity_ = 0;
    float* bounds_ = nullptr;        // 12 floats: lo.xyz hi.xyz inv.xyz pad
    float* partial_ = nullptr;       // per-block partial bounds
    uint32_t* morton_ = nullptr;     // original order
    uint32_t* keys_ = nullptr;       // sorted keys
    uint32_t* order_ = nullptr;      // sorted original indices
    int* parent_ = nullptr;          // [n-1 internal][n leaves]
    uint32_t* flags_ = nullptr;      // arrival counters, n-1
    float4* nodes_ = nullptr;
    float4* tris_ = nullptr;
    float4* wide_ = nullptr;         // 8-wide records, 96 bytes per internal node
    float4* tri_plane_ = nullptr;    // 32 bytes per triangle (shading normal and plane offset)
    float4* emit_tab_ = nullptr;     // 80 bytes per emitter (light-sampling records)
    uint32_t emit_capacity_ = 0;
    int sah_cluster_ = 32;           // leaves of the subtrees rebuilt with the SAH split (0: none)
    int* sah_roots_ = nullptr;       // roots of those subtrees
    int* sah_count_ = nullptr;
    bool dp_collapse_ = true;
    int split_percent_ = QUASI_BVH_SPLIT_PERCENT;
    uint32_t* ref_tri_ = nullptr;    // per reference: its triangle (split builds only)
    float4* ref_box_ = nullptr;      // per reference: its box, 2 float4
    uint32_t ref_capacity_ = 0;
    float* dp_cost_ = nullptr;       // 8 costs per internal node (k_collapse_dp)
    uint8_t* dp_dec_ = nullptr;      // 8 decisions per internal node
    float4* tree_ = nullptr;
    int tree_n_ = 0;
    int tree_capacity_ = 0;
    RadixSortScratch sort_;
};

constexpr int k_bounds_blocks = 304;  // 2 x 152 SMs

}  // namespace quasi
