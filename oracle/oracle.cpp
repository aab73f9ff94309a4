// oracle.cpp - CPU oracle for the CUDA path tracer. TEST INFRASTRUCTURE ONLY.
//
// Only the tests, __graft_entry__.smoke() and bench.py's cpu_baseline / reference leg load
// this library, and only as a checker or as the timed CPU baseline; the product
// (libquasi_cuda.so) never links or calls it.
//
// It is an independent scalar restatement, templated on the real type (double = the
// correctness oracle, float = a timing/diagnosis twin), of:
//   backends/metal/plugin.mm:98-102   pcg_hash
//   backends/metal/plugin.mm:104-107  random_float
//   backends/metal/plugin.mm:111-125  cosine_sample_hemisphere
//   backends/metal/plugin.mm:129-153  get_camera_ray (= src/quasi/scene/camera.hpp:36-52 + jitter)
//   backends/metal/plugin.mm:157-212  intersect_quad, trace_scene
//   backends/metal/plugin.mm:223-309  path_trace and the per-pixel seeding / AOVs
// and of the parts the reference does not have (their published sources are named):
//   Morton-30 codes and a stable sort (std::stable_sort), the Karras 2012 hierarchy built
//   top-down, bottom-up boxes, Moller & Trumbore 1997 triangle tests, Lambertian
//   next-event estimation with uniform emitter selection.
// The conventions (RNG keying, emitter choice, ray offsets, signatures) are stated once in
// the project's design notes and restated here without sharing code with the product.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <cstdlib>
#include <thread>
#include <vector>

#define ORACLE_API extern "C" __attribute__((visibility("default")))

namespace oracle {

template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline V3<R> normalize(V3<R> v) { return v / std::sqrt(dot(v, v)); }
template <class R> inline R maxc(V3<R> v) { return std::max(v.x, std::max(v.y, v.z)); }
template <class R> inline V3<R> load3(const float* p) { return {R(p[0]), R(p[1]), R(p[2])}; }

// plugin.mm:98-102
inline uint32_t pcg_hash(uint32_t input) {
    const uint32_t state = input * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

// plugin.mm:104-107
inline float random_float(uint32_t& state) {
    state = pcg_hash(state);
    return static_cast<float>(state) / static_cast<float>(0xFFFFFFFFu);
}

inline uint32_t path_key(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t bounce) {
    return pcg_hash(pcg_hash(pcg_hash(seed ^ pixel) + sample) + bounce);
}

inline uint32_t sig_mix(uint32_t sig, uint32_t v) { return pcg_hash(sig ^ v) + v; }
constexpr uint32_t k_sig_miss = 0xFFFFFFFFu, k_sig_lit = 0xFFFFFFF1u, k_sig_shadowed = 0xFFFFFFF2u,
                   k_sig_no_nee = 0xFFFFFFF3u;

// plugin.mm:111-125 (cos/sin products grouped as the CUDA path groups them; order does not
// matter beyond rounding).
template <class R> V3<R> cosine_sample(V3<R> normal, float r1f, float r2f) {
    const R r1 = R(r1f), r2 = R(r2f);
    const R phi = R(2) * R(3.14159265358979323846) * r1;
    const R cos_theta = std::sqrt(R(1) - r2);
    const R sin_theta = std::sqrt(r2);
    const V3<R> w = normalize(normal);
    const V3<R> a = (std::fabs(w.x) > R(0.9)) ? V3<R>{0, 1, 0} : V3<R>{1, 0, 0};
    const V3<R> v = normalize(cross(w, a));
    const V3<R> u = cross(w, v);
    return normalize(u * (std::cos(phi) * sin_theta) + v * (std::sin(phi) * sin_theta) + w * cos_theta);
}

// Pinhole basis (plugin.mm:134-147 with the host normalisation of plugin.mm:653-659) in double.
struct CamBasis {
    double o[3], ll[3], h[3], v[3];
};
inline CamBasis camera_basis(const float* pos, const float* target, const float* up, float fov, uint32_t w,
                             uint32_t h) {
    double dir[3] = {double(target[0]) - pos[0], double(target[1]) - pos[1], double(target[2]) - pos[2]};
    double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (len > 0) for (double& x : dir) x /= len;
    double wv[3] = {-dir[0], -dir[1], -dir[2]};
    len = std::sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
    if (len > 0) for (double& x : wv) x /= len;
    double r[3] = {up[1] * wv[2] - up[2] * wv[1], up[2] * wv[0] - up[0] * wv[2], up[0] * wv[1] - up[1] * wv[0]};
    len = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (len > 0) for (double& x : r) x /= len;
    const double u2[3] = {wv[1] * r[2] - wv[2] * r[1], wv[2] * r[0] - wv[0] * r[2], wv[0] * r[1] - wv[1] * r[0]};
    const double vh = 2.0 * std::tan(double(fov) * 3.14159265358979323846 / 360.0);
    const double vw = (double(w) / double(h)) * vh;
    CamBasis b;
    for (int k = 0; k < 3; ++k) {
        b.o[k] = pos[k];
        b.h[k] = vw * r[k];
        b.v[k] = vh * u2[k];
        b.ll[k] = double(pos[k]) - b.h[k] * 0.5 - b.v[k] * 0.5 - wv[k];
    }
    return b;
}

// ------------------------------------------------------------------------------ LBVH

struct Lbvh {
    uint32_t n = 0;
    float bounds[9] = {};           // centroid lo, hi, 1/extent
    std::vector<uint32_t> morton;   // original order
    std::vector<uint32_t> order;    // sorted position -> original index
    std::vector<int32_t> child;     // 2 per internal node
    std::vector<float> box;         // 12 per internal node: c0 lo hi, c1 lo hi
    std::vector<int32_t> range;     // 2 per internal node: first and last leaf covered
};

inline uint32_t spread_bits(uint32_t q) {
    uint32_t out = 0;
    for (int b = 0; b < 10; ++b) out |= ((q >> b) & 1u) << (3 * b);
    return out;
}

inline int common_prefix(const std::vector<uint32_t>& keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (keys[i] == keys[j]) return 32 + __builtin_clz(static_cast<uint32_t>(i ^ j));
    return __builtin_clz(keys[i] ^ keys[j]);
}

// Builds the LBVH of n triangles (9 floats each). All float arithmetic here is FP32 with
// no contraction, matching the GPU build bit for bit.
void build_lbvh(uint32_t n, const float* v, Lbvh& b) {
    b.n = n;
    b.morton.assign(n, 0);
    b.order.resize(n);
    if (n == 0) return;
    std::vector<float> cen(3ull * n);
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    const float third = 1.0f / 3.0f;
    for (uint32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            const float* t = v + 9ull * i;
            const float c = ((t[a] + t[3 + a]) + t[6 + a]) * third;
            cen[3ull * i + a] = c;
            lo[a] = std::min(lo[a], c);
            hi[a] = std::max(hi[a], c);
        }
    float inv[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        inv[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
        b.bounds[a] = lo[a];
        b.bounds[3 + a] = hi[a];
        b.bounds[6 + a] = inv[a];
    }
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            float t = ((cen[3ull * i + a] - lo[a]) * inv[a]) * 1024.0f;
            t = std::min(std::max(t, 0.0f), 1023.0f);
            q[a] = static_cast<uint32_t>(t);
        }
        b.morton[i] = (spread_bits(q[0]) << 2) | (spread_bits(q[1]) << 1) | spread_bits(q[2]);
    }
    for (uint32_t i = 0; i < n; ++i) b.order[i] = i;
    std::stable_sort(b.order.begin(), b.order.end(),
                     [&](uint32_t x, uint32_t y) { return b.morton[x] < b.morton[y]; });
    std::vector<uint32_t> keys(n);
    for (uint32_t i = 0; i < n; ++i) keys[i] = b.morton[b.order[i]];

    const uint32_t nodes = n > 1 ? n - 1 : 1;
    b.child.assign(2ull * nodes, 0);
    b.box.assign(12ull * nodes, 0.f);
    b.range.assign(2ull * nodes, 0);
    auto leaf_box = [&](int pos, float* out) {
        const float* t = v + 9ull * b.order[pos];
        for (int a = 0; a < 3; ++a) {
            out[a] = std::min(t[a], std::min(t[3 + a], t[6 + a]));
            out[3 + a] = std::max(t[a], std::max(t[3 + a], t[6 + a]));
        }
    };
    if (n == 1) {
        b.child[0] = ~0;
        b.child[1] = ~0;
        leaf_box(0, &b.box[0]);
        leaf_box(0, &b.box[6]);
        return;
    }
    // Top-down: the node covering sorted range [lo, hi] splits after the last key that still
    // shares the range's common prefix plus one bit (binary search); its children are
    // internal node gamma ([lo, gamma]) and gamma + 1 ([gamma + 1, hi]), or leaves.
    struct Item {
        int idx, lo, hi;
    };
    std::vector<Item> stack{{0, 0, static_cast<int>(n) - 1}};
    std::vector<int> post;  // internal nodes in pre-order; boxes are filled in reverse
    while (!stack.empty()) {
        const Item it = stack.back();
        stack.pop_back();
        const int dnode = common_prefix(keys, n, it.lo, it.hi);
        int a = it.lo, z = it.hi - 1;  // find max k in [lo, hi-1] with prefix(lo, k) > dnode
        while (a < z) {
            const int mid = (a + z + 1) / 2;
            if (common_prefix(keys, n, it.lo, mid) > dnode) a = mid;
            else z = mid - 1;
        }
        const int gamma = a;
        const int left = (it.lo == gamma) ? ~gamma : gamma;
        const int right = (it.hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
        b.child[2ull * it.idx] = left;
        b.child[2ull * it.idx + 1] = right;
        b.range[2ull * it.idx] = it.lo;
        b.range[2ull * it.idx + 1] = it.hi;
        post.push_back(it.idx);
        if (left >= 0) stack.push_back({left, it.lo, gamma});
        if (right >= 0) stack.push_back({right, gamma + 1, it.hi});
    }
    // Children are always visited after their parent, so reverse order is bottom-up.
    for (auto itr = post.rbegin(); itr != post.rend(); ++itr) {
        const int i = *itr;
        for (int s = 0; s < 2; ++s) {
            const int c = b.child[2ull * i + s];
            float* out = &b.box[12ull * i + 6 * s];
            if (c < 0) {
                leaf_box(~c, out);
            } else {
                const float* cb = &b.box[12ull * c];
                for (int a = 0; a < 3; ++a) {
                    out[a] = std::min(cb[a], cb[6 + a]);
                    out[3 + a] = std::max(cb[3 + a], cb[9 + a]);
                }
            }
        }
    }
}

// ------------------------------------------------------------------------------ 8-wide collapse

// Directed roundings of FP32 operations, exact for all finite inputs: the rounding error
// of a - b comes from TwoSum, that of x / 255 from an FMA remainder.
inline float sub_round(float a, float b, bool up) {
    const float s = a - b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (-b - bb);  // a - b = s + e exactly
    if (up && e > 0.0f) return std::nextafter(s, std::numeric_limits<float>::infinity());
    if (!up && e < 0.0f) return std::nextafter(s, -std::numeric_limits<float>::infinity());
    return s;
}

inline float div255_up(float x) {
    const float q = x / 255.0f;
    const float r = std::fma(-q, 255.0f, x);  // x - 255 q exactly
    return r > 0.0f ? std::nextafter(q, std::numeric_limits<float>::infinity()) : q;
}

struct WideEntryO {
    int ref, first, size;
    float lo[3], hi[3];
};

inline float half_area_o(const float lo[3], const float hi[3]) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return (dx * dy + dy * dz) + dz * dx;
}

// 8-wide record of every internal node of b, 24 words each, restating k_collapse8
// (quasi_gb300/csrc/bvh.cu): greedy opening of the largest child by surface area, leaves of
// one triangle, child boxes padded by the scene's Delta and put on an 8-bit power-of-two grid
// rounded outwards, children placed in slots by direction (Ylitie, Karras and Laine 2017).
void collapse8(const Lbvh& b, std::vector<uint32_t>& out) {
    const uint32_t nodes = b.n > 1 ? b.n - 1 : (b.n == 1 ? 1 : 0);
    out.assign(24ull * nodes, 0u);
    auto entry = [&](int c, int k, WideEntryO& e) {
        e.ref = b.child[2ull * c + k];
        const float* bx = &b.box[12ull * c + 6 * k];
        for (int a = 0; a < 3; ++a) {
            e.lo[a] = bx[a];
            e.hi[a] = bx[3 + a];
        }
        if (e.ref < 0) {
            e.first = ~e.ref;
            e.size = 1;
        } else {
            e.first = b.range[2ull * e.ref];
            e.size = b.range[2ull * e.ref + 1] - e.first + 1;
        }
    };
    // Delta = 2^-16 S, S the largest absolute coordinate of the root's child boxes (every
    // vertex): the spatial box padding of the FP32 traversal (CUDA scene_box_pad)
    float smax = 0.0f;
    for (size_t k = 0; k < std::min<size_t>(12, b.box.size()); ++k) smax = std::max(smax, std::fabs(b.box[k]));
    const float pad = std::ldexp(std::max(smax, std::ldexp(1.0f, -100)), -16);
    for (uint32_t nb = 0; nb < nodes; ++nb) {
        WideEntryO e[8];
        entry(static_cast<int>(nb), 0, e[0]);
        entry(static_cast<int>(nb), 1, e[1]);
        int count = 2;
        while (count < 8) {
            int pick = -1;
            float best = 0.0f;
            for (int i = 0; i < count; ++i) {
                if (e[i].ref < 0) continue;
                const float a = half_area_o(e[i].lo, e[i].hi);
                if (pick < 0 || a > best) {
                    pick = i;
                    best = a;
                }
            }
            if (pick < 0) break;
            const int c = e[pick].ref;
            entry(c, 1, e[count]);
            entry(c, 0, e[pick]);
            ++count;
        }
        float lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = e[0].lo[a];
            hi[a] = e[0].hi[a];
            for (int i = 1; i < count; ++i) {
                lo[a] = std::fmin(lo[a], e[i].lo[a]);
                hi[a] = std::fmax(hi[a], e[i].hi[a]);
            }
        }
        // grid over the node box padded by the scene's Delta (padded child boxes, lower planes
        // rounded down, upper planes up)
        float glo[3];
        uint32_t ex[3];
        double inv_s[3];
        for (int a = 0; a < 3; ++a) {
            glo[a] = sub_round(lo[a], pad, false);
            const float x = div255_up(sub_round(sub_round(hi[a], -pad, true), glo[a], true));
            uint32_t bits;
            std::memcpy(&bits, &x, 4);
            const int eb = static_cast<int>((bits >> 23) & 0xffu);
            int ee = eb == 0 ? -100 : eb - 127 + ((bits & 0x7fffffu) != 0u ? 1 : 0);
            ee = std::max(-100, std::min(126, ee));
            ex[a] = static_cast<uint32_t>(ee + 127);
            inv_s[a] = std::ldexp(1.0, -ee);
        }
        const float mx = (lo[0] + hi[0]) * 0.5f, my = (lo[1] + hi[1]) * 0.5f, mz = (lo[2] + hi[2]) * 0.5f;
        float cx[8], cy[8], cz[8];
        for (int i = 0; i < count; ++i) {
            cx[i] = (e[i].lo[0] + e[i].hi[0]) * 0.5f - mx;
            cy[i] = (e[i].lo[1] + e[i].hi[1]) * 0.5f - my;
            cz[i] = (e[i].lo[2] + e[i].hi[2]) * 0.5f - mz;
        }
        int slot_of[8] = {};
        uint32_t used = 0, placed = 0;
        for (int it = 0; it < count; ++it) {
            int bi = -1, bs = -1;
            float bsc = 0.0f;
            for (int i = 0; i < count; ++i) {
                if (placed & (1u << i)) continue;
                for (int s = 0; s < 8; ++s) {
                    if (used & (1u << s)) continue;
                    const float sc = (((s & 1) ? -cx[i] : cx[i]) + ((s & 2) ? -cy[i] : cy[i])) + ((s & 4) ? -cz[i] : cz[i]);
                    if (bi < 0 || sc > bsc) {
                        bi = i;
                        bs = s;
                        bsc = sc;
                    }
                }
            }
            slot_of[bi] = bs;
            placed |= 1u << bi;
            used |= 1u << bs;
        }
        uint32_t* w = &out[24ull * nb];
        uint32_t qlo[3][2] = {}, qhi[3][2] = {};
        int32_t refs[8];
        uint32_t imask = 0;
        for (int s = 0; s < 8; ++s) {
            refs[s] = ~3;
            for (int a = 0; a < 3; ++a) qlo[a][s >> 2] |= 255u << (8 * (s & 3));
        }
        for (int i = 0; i < count; ++i) {
            const int s = slot_of[i];
            for (int a = 0; a < 3; ++a) {
                const double ql =
                    std::floor(double(sub_round(sub_round(e[i].lo[a], pad, false), glo[a], false)) * inv_s[a]);
                const double qh =
                    std::ceil(double(sub_round(sub_round(e[i].hi[a], -pad, true), glo[a], true)) * inv_s[a]);
                const uint32_t bl = static_cast<uint32_t>(std::min(std::max(ql, 0.0), 255.0));
                const uint32_t bh = static_cast<uint32_t>(std::min(std::max(qh, 0.0), 255.0));
                qlo[a][s >> 2] = (qlo[a][s >> 2] & ~(255u << (8 * (s & 3)))) | (bl << (8 * (s & 3)));
                qhi[a][s >> 2] |= bh << (8 * (s & 3));
            }
            if (e[i].ref >= 0 && e[i].size > 1) {  // leaves of one triangle (k_wide_leaf_max)
                refs[s] = e[i].ref;
                imask |= 1u << s;
            } else {
                refs[s] = ~((e[i].first << 2) | (e[i].size - 1));
            }
        }
        std::memcpy(&w[0], &glo[0], 4);
        std::memcpy(&w[1], &glo[1], 4);
        std::memcpy(&w[2], &glo[2], 4);
        w[3] = ex[0] | (ex[1] << 8) | (ex[2] << 16) | (imask << 24);
        for (int a = 0; a < 3; ++a) {
            w[4 + 4 * a] = qlo[a][0];
            w[5 + 4 * a] = qlo[a][1];
            w[6 + 4 * a] = qhi[a][0];
            w[7 + 4 * a] = qhi[a][1];
        }
        for (int s = 0; s < 8; ++s) std::memcpy(&w[16 + s], &refs[s], 4);
    }
}

// ------------------------------------------------------------------------------ tracing

template <class R> struct SceneR {
    uint32_t n = 0;
    const float* v = nullptr;
    const float* albedo = nullptr;
    const float* emission = nullptr;
    std::vector<int> emitters;
    const Lbvh* bvh = nullptr;
    std::vector<R> padded;  // 12 per node, boxes widened so a rounding never culls a hit
};

// Moller-Trumbore in R; returns t or +inf and the barycentrics (u, w) of e1, e2.
template <class R> inline R tri_hit(const float* t, V3<R> o, V3<R> d, R& u, R& w) {
    const V3<R> v0 = load3<R>(t), e1 = load3<R>(t + 3) - v0, e2 = load3<R>(t + 6) - v0;
    const V3<R> p = cross(d, e2);
    const R det = dot(e1, p);
    const R inf = std::numeric_limits<R>::infinity();
    if (det == R(0)) return inf;
    const R inv = R(1) / det;
    const V3<R> tv = o - v0;
    u = dot(tv, p) * inv;
    if (u < R(0) || u > R(1)) return inf;
    const V3<R> q = cross(tv, e1);
    w = dot(d, q) * inv;
    if (w < R(0) || u + w > R(1)) return inf;
    const R tt = dot(e2, q) * inv;
    return tt > R(0) ? tt : inf;
}

template <class R> inline bool box_hit(const R* b, V3<R> o, V3<R> inv, R tmax, R& tnear) {
    R t0 = R(0), t1 = tmax;
    const R oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    for (int a = 0; a < 3; ++a) {
        R lo = (b[a] - oo[a]) * ii[a], hi = (b[3 + a] - oo[a]) * ii[a];
        if (lo > hi) std::swap(lo, hi);
        t0 = std::max(t0, lo);
        t1 = std::min(t1, hi);
    }
    tnear = t0;
    return t0 <= t1;
}

struct Counters {
    uint64_t camera = 0, extension = 0, shadow = 0;
};

// Closest hit (any = false) or any hit (any = true) with t in (0, tmax), skipping `exclude`.
// Closest-hit ties go to the smaller original index. bu, bw receive the hit's barycentrics.
template <class R> int trace(const SceneR<R>& s, V3<R> o, V3<R> d, R tmax, int exclude, bool any, R& t_out,
                             R& bu, R& bw) {
    R best_t = tmax;
    int best = -1;
    bu = bw = R(0);
    if (s.n == 0) {
        t_out = best_t;
        return -1;
    }
    auto inv1 = [](R x) { return R(1) / (std::fabs(x) > R(1e-30) ? x : std::copysign(R(1e-30), x)); };
    const V3<R> inv{inv1(d.x), inv1(d.y), inv1(d.z)};
    int stack[128];
    R stack_t[128];
    int sp = 0;
    stack[sp] = 0;
    stack_t[sp++] = R(0);
    while (sp > 0) {
        --sp;
        const int node = stack[sp];
        if (stack_t[sp] > best_t) continue;  // entered beyond the current closest hit
        // Visit the nearer child first (it is pushed last).
        R tn[2];
        bool hit[2];
        for (int c = 0; c < 2; ++c) hit[c] = box_hit(&s.padded[12ull * node + 6 * c], o, inv, best_t, tn[c]);
        const int first = (hit[0] && hit[1] && tn[1] < tn[0]) ? 1 : 0;
        for (int k = 1; k >= 0; --k) {
            const int c = k == 0 ? first : 1 - first;
            const int ch = s.bvh->child[2ull * node + c];
            if (!hit[c]) continue;
            if (ch < 0) {
                const uint32_t orig = s.bvh->order[~ch];
                if (static_cast<int>(orig) == exclude) continue;
                R u = R(0), w = R(0);
                const R t = tri_hit<R>(s.v + 9ull * orig, o, d, u, w);
                if (t < best_t || (t == best_t && best >= 0 && static_cast<int>(orig) < best)) {
                    best_t = t;
                    best = static_cast<int>(orig);
                    bu = u;
                    bw = w;
                    if (any) {
                        t_out = best_t;
                        return best;
                    }
                }
            } else if (sp < 128) {
                stack[sp] = ch;
                stack_t[sp++] = tn[c];
            }
        }
    }
    t_out = best_t;
    return best;
}

struct PixelOut {
    double mean[3];
    double aov[7];
};

struct NeeConfig {
    uint32_t width, height, spp, sample_base, max_depth, seed;
    float eps;
};

// One vertex of a path as the adjoint needs it: the triangle hit, the NEE light (or -1) and
// the NEE factor g times visibility.
template <class R> struct PathVtx {
    int prim;
    int light;
    R gv;
};

// One path sample of the NEE integrator (the conventions the CUDA kernels implement). With
// `verts`, records every vertex for the adjoint.
template <class R> void nee_sample(const SceneR<R>& s, const CamBasis& cb, const NeeConfig& c, uint32_t x,
                                   uint32_t y, uint32_t sample, R L[3], uint32_t& sig, double aov[7], Counters& cnt,
                                   std::vector<PathVtx<R>>* verts = nullptr) {
    const uint32_t pixel = y * c.width + x;
    uint32_t st = path_key(c.seed, pixel, sample, 0);
    const float jx = random_float(st), jy = random_float(st);
    const R u = (R(x) + R(jx)) / R(c.width);
    const R vv = R(1) - (R(y) + R(jy)) / R(c.height);
    V3<R> o{R(cb.o[0]), R(cb.o[1]), R(cb.o[2])};
    V3<R> d;
    {
        const V3<R> ll{R(cb.ll[0]), R(cb.ll[1]), R(cb.ll[2])}, hh{R(cb.h[0]), R(cb.h[1]), R(cb.h[2])},
            vt{R(cb.v[0]), R(cb.v[1]), R(cb.v[2])};
        d = normalize(ll + hh * u + vt * vv - o);
    }
    V3<R> beta{1, 1, 1}, Lr{0, 0, 0};
    sig = 0;
    int exclude = -1;
    cnt.camera++;
    for (uint32_t k = 1; k <= c.max_depth; ++k) {
        if (k > 1) cnt.extension++;
        R t, bu, bw;
        const int h = trace(s, o, d, std::numeric_limits<R>::infinity(), exclude, false, t, bu, bw);
        if (h < 0) {
            sig = sig_mix(sig, k_sig_miss);
            break;
        }
        const float* tv = s.v + 9ull * h;
        const V3<R> a = load3<R>(tv);
        const V3<R> e1h = load3<R>(tv + 3) - a, e2h = load3<R>(tv + 6) - a;
        V3<R> n = normalize(cross(e1h, e2h));
        if (dot(n, d) > R(0)) n = -n;
        // The hit point from the barycentrics lies on the triangle's plane (in FP64 it equals
        // o + t d to ~1e-16; in FP32 it avoids the rounding of o + t d).
        const V3<R> x_hit = a + e1h * bu + e2h * bw;
        const V3<R> alb = load3<R>(s.albedo + 3ull * h);
        sig = sig_mix(sig, static_cast<uint32_t>(h));
        if (k == 1) {
            const V3<R> em = load3<R>(s.emission + 3ull * h);
            Lr = Lr + em;
            const V3<R> aa = maxc(em) > R(0.1) ? em : alb;
            const R depth = std::min(std::max((t - R(1)) / R(4), R(0)), R(1));
            aov[0] = double(aa.x); aov[1] = double(aa.y); aov[2] = double(aa.z); aov[3] = double(depth);
            aov[4] = double(n.x * R(0.5) + R(0.5)); aov[5] = double(n.y * R(0.5) + R(0.5));
            aov[6] = double(n.z * R(0.5) + R(0.5));
        }
        uint32_t rs = path_key(c.seed, pixel, sample, k);
        const uint32_t sel = pcg_hash(rs);
        rs = sel;
        const float r1 = random_float(rs), r2 = random_float(rs);
        const V3<R> org = x_hit + n * R(c.eps);
        bool nee = false;
        int vtx_light = -1;
        R vtx_gv = R(0);
        if (!s.emitters.empty()) {
            const uint32_t ne = static_cast<uint32_t>(s.emitters.size());
            const int l = s.emitters[static_cast<uint32_t>((static_cast<uint64_t>(sel) * ne) >> 32)];
            if (l != h) {
                const float* lt = s.v + 9ull * l;
                const V3<R> la = load3<R>(lt), e1 = load3<R>(lt + 3) - la, e2 = load3<R>(lt + 6) - la;
                const R su = std::sqrt(R(r1));
                const V3<R> yl = la + e1 * (su * (R(1) - R(r2))) + e2 * (su * R(r2));
                const V3<R> dv = (yl - x_hit) - n * R(c.eps);
                const R d2 = dot(dv, dv);
                const R dist = std::sqrt(d2);
                const V3<R> wi = dv / dist;
                const R cos_x = dot(n, wi);
                const V3<R> nl = cross(e1, e2);
                const R area2 = std::sqrt(dot(nl, nl));
                const R cl = dot(nl, wi);
                const R cos_l = std::fabs(cl) / area2;
                if (cos_x > R(0) && cos_l > R(0) && d2 > R(0)) {
                    nee = true;
                    cnt.shadow++;
                    // Visibility from the light sample lifted by eps along the light normal
                    // towards the shading side, to just short of the lifted shading point.
                    const R side = cl < R(0) ? R(c.eps) : -R(c.eps);
                    const V3<R> so = yl + nl * (side / area2);
                    const V3<R> sd = org - so;
                    const R sdist = std::sqrt(dot(sd, sd));
                    R ts, su2, sw2;
                    const int occ = trace(s, so, sd / sdist, sdist * (R(1) - R(1e-4)), -1, true, ts, su2, sw2);
                    if (occ < 0) {
                        const R g = cos_x * cos_l / d2 * (R(0.5) * area2) * R(ne) / R(3.14159265358979323846);
                        const V3<R> le = load3<R>(s.emission + 3ull * l);
                        Lr = Lr + beta * alb * le * g;
                        sig = sig_mix(sig, k_sig_lit);
                        vtx_light = l;
                        vtx_gv = g;
                    } else {
                        sig = sig_mix(sig, k_sig_shadowed);
                    }
                }
            }
        }
        if (!nee) sig = sig_mix(sig, k_sig_no_nee);
        if (verts) verts->push_back(PathVtx<R>{h, vtx_light, vtx_gv});
        const float r3 = random_float(rs), r4 = random_float(rs);
        const V3<R> nd = cosine_sample<R>(n, r3, r4);
        beta = beta * alb;
        if (k >= c.max_depth || !(maxc(beta) > R(0))) break;
        o = org;
        d = nd;
        exclude = h;
    }
    L[0] = Lr.x;
    L[1] = Lr.y;
    L[2] = Lr.z;
}

template <class R> void prepare(SceneR<R>& s, uint32_t n, const float* v, const float* albedo, const float* emission,
                                const Lbvh& b) {
    s.n = n;
    s.v = v;
    s.albedo = albedo;
    s.emission = emission;
    s.bvh = &b;
    for (uint32_t i = 0; i < n; ++i)
        if (emission[3 * i] > 0.f || emission[3 * i + 1] > 0.f || emission[3 * i + 2] > 0.f)
            s.emitters.push_back(static_cast<int>(i));
    s.padded.resize(b.box.size());
    for (size_t i = 0; i < b.box.size(); i += 6) {
        for (int a = 0; a < 3; ++a) {
            const R lo = R(b.box[i + a]), hi = R(b.box[i + 3 + a]);
            const R pad = R(1e-6) * (R(1) + std::max(std::fabs(lo), std::fabs(hi)));
            s.padded[i + a] = lo - pad;
            s.padded[i + 3 + a] = hi + pad;
        }
    }
}

template <class Fn> void parallel_for(uint32_t count, uint32_t threads, Fn fn) {
    if (threads <= 1 || count < 64) {
        for (uint32_t i = 0; i < count; ++i) fn(i, 0u);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    const uint32_t chunk = 16;
    for (uint32_t t = 0; t < threads; ++t)
        pool.emplace_back([&, t]() {
            while (true) {
                const uint32_t b = next.fetch_add(chunk);
                if (b >= count) break;
                for (uint32_t i = b; i < std::min(count, b + chunk); ++i) fn(i, t);
            }
        });
    for (auto& th : pool) th.join();
}

// ------------------------------------------------------------------------ reference mode

// backends/metal/plugin.mm:157-195
template <class R> bool ref_intersect_quad(V3<R> ro, V3<R> rd, const float* q, R tmin, R tmax, R& t_out,
                                           V3<R>& p_out, V3<R>& n_out) {
    const V3<R> qo = load3<R>(q), qu = load3<R>(q + 3), qv = load3<R>(q + 6);
    const V3<R> n = cross(qu, qv);
    const R area_sq = dot(n, n);
    if (area_sq < R(1e-8)) return false;
    const V3<R> normal = n * (R(1) / std::sqrt(area_sq));
    const R dd = dot(normal, qo);
    const R denom = dot(normal, rd);
    if (std::fabs(denom) < R(1e-8)) return false;
    const R t = (dd - dot(normal, ro)) / denom;
    if (t < tmin || t > tmax) return false;
    const V3<R> p = ro + rd * t;
    const V3<R> planar = p - qo;
    const V3<R> w = n / area_sq;
    const R alpha = dot(w, cross(planar, qv));
    const R beta = dot(w, cross(qu, planar));
    if (alpha < R(0) || alpha > R(1) || beta < R(0) || beta > R(1)) return false;
    t_out = t;
    p_out = p;
    n_out = (denom < R(0)) ? normal : -normal;
    return true;
}

// backends/metal/plugin.mm:223-276 plus the per-pixel seeding and camera of :129-153,
// :287-309. `frame` is the reference's frame_count for this sample.
template <class R> void ref_sample(uint32_t nq, const float* quads, const float* qalb, const float* qem,
                                   const float* cam_pos, const float* cam_dir, const float* cam_up, float fov,
                                   float aspect, uint32_t w, uint32_t h, uint32_t px, uint32_t py, uint32_t frame,
                                   R color[3], R aov[7]) {
    uint32_t rng = pcg_hash(px + py * 1920u + frame * 1920u * 1080u);
    R ux = (R(px) + R(0.5)) / R(w);
    R uy = R(1) - (R(py) + R(0.5)) / R(h);
    const R jx = R(random_float(rng)) - R(0.5);
    const R jy = R(random_float(rng)) - R(0.5);
    ux = ux + jx * R(0.001);
    uy = uy + jy * R(0.001);
    const R pi = R(3.14159265358979323846);
    const R theta = R(fov) * pi / R(180);
    const R hh = std::tan(theta / R(2));
    const R vh = R(2) * hh;
    const R vw = R(aspect) * vh;
    const V3<R> pos = load3<R>(cam_pos), dir = load3<R>(cam_dir), up = load3<R>(cam_up);
    const V3<R> wv = normalize(-dir);
    const V3<R> right = normalize(cross(up, wv));
    const V3<R> up2 = cross(wv, right);
    const V3<R> horizontal = right * vw, vertical = up2 * vh;
    const V3<R> lower_left = pos - horizontal * R(0.5) - vertical * R(0.5) - wv;
    const V3<R> target = lower_left + horizontal * ux + vertical * uy;
    V3<R> ro = pos, rd = normalize(target - pos);
    V3<R> col{0, 0, 0}, tp{1, 1, 1};
    for (int k = 0; k < 7; ++k) aov[k] = R(0);
    for (int bounce = 0; bounce < 5; ++bounce) {
        R best = R(1e30);
        int idx = -1;
        V3<R> bp{0, 0, 0}, bn{0, 0, 0};
        for (uint32_t i = 0; i < nq && i < 32; ++i) {
            R t;
            V3<R> p, n;
            if (ref_intersect_quad<R>(ro, rd, quads + 9ull * i, R(0.001), best, t, p, n)) {
                best = t;
                idx = static_cast<int>(i);
                bp = p;
                bn = n;
            }
        }
        if (idx < 0) break;
        const V3<R> alb = load3<R>(qalb + 3ull * idx), em = load3<R>(qem + 3ull * idx);
        const R es = maxc(em);
        if (bounce == 0) {
            const V3<R> aa = es > R(0.1) ? em : alb;
            aov[0] = aa.x; aov[1] = aa.y; aov[2] = aa.z;
            aov[3] = best;
            aov[4] = bn.x * R(0.5) + R(0.5); aov[5] = bn.y * R(0.5) + R(0.5); aov[6] = bn.z * R(0.5) + R(0.5);
        }
        col = col + tp * em;
        if (es > R(0.1)) break;
        tp = tp * alb;
        if (bounce > 2) {
            const R p = std::max(R(0.05), maxc(tp));
            if (R(random_float(rng)) > p) break;
            tp = tp / p;
        }
        ro = bp + bn * R(0.001);
        // plugin.mm:111-125 evaluated in the reference's operation order.
        const R r1 = R(random_float(rng)), r2 = R(random_float(rng));
        const R phi = R(2) * pi * r1;
        const R ct = std::sqrt(R(1) - r2), stt = std::sqrt(r2);
        const V3<R> w2 = normalize(bn);
        const V3<R> a = (std::fabs(w2.x) > R(0.9)) ? V3<R>{0, 1, 0} : V3<R>{1, 0, 0};
        const V3<R> vv = normalize(cross(w2, a));
        const V3<R> uu = cross(w2, vv);
        rd = normalize(uu * std::cos(phi) * stt + vv * std::sin(phi) * stt + w2 * ct);
    }
    aov[3] = std::min(std::max((aov[3] - R(1)) / R(4), R(0)), R(1));
    color[0] = col.x;
    color[1] = col.y;
    color[2] = col.z;
}

}  // namespace oracle

using namespace oracle;

// ------------------------------------------------------------------------------ C API

struct OracleConfig {
    uint32_t width, height, spp, sample_base, max_depth, seed;
    float cam_pos[3], cam_target[3], cam_up[3], cam_fov;
    float ray_eps;
    uint32_t precision;  // 64 = double, 32 = float
    uint32_t threads;
};

ORACLE_API uint32_t oracle_pcg_hash(uint32_t x) { return pcg_hash(x); }

ORACLE_API float oracle_random_float(uint32_t* state) { return random_float(*state); }

ORACLE_API uint32_t oracle_path_key(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t bounce) {
    return path_key(seed, pixel, sample, bounce);
}

ORACLE_API void oracle_cosine_sample(const double* n, float r1, float r2, double* out) {
    const V3<double> d = cosine_sample<double>({n[0], n[1], n[2]}, r1, r2);
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

// Pinhole direction of the NEE integrator's camera (no jitter) at (u, v), in double; this is
// src/quasi/scene/camera.hpp:36-52 evaluated on a position/target camera.
ORACLE_API void oracle_camera_dir(const float* pos, const float* target, const float* up, float fov, uint32_t w,
                                  uint32_t h, double u, double v, double* out) {
    const CamBasis b = camera_basis(pos, target, up, fov, w, h);
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = b.ll[k] + u * b.h[k] + v * b.v[k] - b.o[k];
    const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int k = 0; k < 3; ++k) out[k] = d[k] / len;
}

// Reference-convention camera ray (plugin.mm:129-153) for one uv and rng state, in double.
ORACLE_API void oracle_ref_camera_ray(const float* pos, const float* dir, const float* up, float fov, float aspect,
                                      double ux, double uy, uint32_t* rng, double* o, double* d) {
    const double jx = double(random_float(*rng)) - 0.5, jy = double(random_float(*rng)) - 0.5;
    ux += jx * 0.001;
    uy += jy * 0.001;
    const double h = std::tan(double(fov) * 3.14159265358979323846 / 180.0 / 2.0);
    const double vh = 2.0 * h, vw = double(aspect) * vh;
    const V3<double> p = load3<double>(pos), dd = load3<double>(dir), u = load3<double>(up);
    const V3<double> w = normalize(-dd), right = normalize(cross(u, w)), up2 = cross(w, right);
    const V3<double> hz = right * vw, vt = up2 * vh;
    const V3<double> ll = p - hz * 0.5 - vt * 0.5 - w;
    const V3<double> dir2 = normalize(ll + hz * ux + vt * uy - p);
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
    d[0] = dir2.x; d[1] = dir2.y; d[2] = dir2.z;
}

// Quad intersection (plugin.mm:157-195 / src/quasi/scene/quad.hpp:51-109) in double.
ORACLE_API int oracle_intersect_quad(const double* ro, const double* rd, const float* quad, double tmin, double tmax,
                                     double* t, double* p, double* n) {
    V3<double> pp, nn;
    double tt;
    if (!ref_intersect_quad<double>({ro[0], ro[1], ro[2]}, {rd[0], rd[1], rd[2]}, quad, tmin, tmax, tt, pp, nn))
        return 0;
    *t = tt;
    p[0] = pp.x; p[1] = pp.y; p[2] = pp.z;
    n[0] = nn.x; n[1] = nn.y; n[2] = nn.z;
    return 1;
}

ORACLE_API int oracle_collapse8(uint32_t n, const float* v, uint32_t* words) {
    Lbvh b;
    build_lbvh(n, v, b);
    std::vector<uint32_t> w;
    collapse8(b, w);
    if (words && !w.empty()) std::memcpy(words, w.data(), sizeof(uint32_t) * w.size());
    return 0;
}

ORACLE_API int oracle_lbvh(uint32_t n, const float* v, uint32_t* morton, uint32_t* order, int32_t* children,
                           float* boxes, float* bounds) {
    Lbvh b;
    build_lbvh(n, v, b);
    if (n == 0) return 0;
    if (morton) std::memcpy(morton, b.morton.data(), sizeof(uint32_t) * n);
    if (order) std::memcpy(order, b.order.data(), sizeof(uint32_t) * n);
    if (children) std::memcpy(children, b.child.data(), sizeof(int32_t) * b.child.size());
    if (boxes) std::memcpy(boxes, b.box.data(), sizeof(float) * b.box.size());
    if (bounds) std::memcpy(bounds, b.bounds, sizeof(float) * 6);
    return 0;
}

template <class R>
static int render_nee(uint32_t n, const float* v, const float* albedo, const float* emission, const OracleConfig* cfg,
                      const uint32_t* pixels, uint32_t npix, double* out_mean, double* out_samples, uint32_t* out_sig,
                      double* out_aov, uint64_t* out_rays) {
    Lbvh b;
    build_lbvh(n, v, b);
    SceneR<R> s;
    prepare(s, n, v, albedo, emission, b);
    const CamBasis cb = camera_basis(cfg->cam_pos, cfg->cam_target, cfg->cam_up, cfg->cam_fov, cfg->width, cfg->height);
    const NeeConfig c{cfg->width, cfg->height, cfg->spp, cfg->sample_base, cfg->max_depth, cfg->seed,
                      cfg->ray_eps > 0.f ? cfg->ray_eps : 1e-4f};
    const uint32_t count = pixels ? npix : cfg->width * cfg->height;
    const uint32_t threads = std::max<uint32_t>(1, cfg->threads);
    std::vector<Counters> cnt(threads);
    parallel_for(count, threads, [&](uint32_t i, uint32_t tid) {
        const uint32_t pix = pixels ? pixels[i] : i;
        const uint32_t x = pix % c.width, y = pix / c.width;
        double sum[3] = {0, 0, 0}, aov[7] = {0, 0, 0, 0, 0, 0, 0}, aov_sum[7] = {0, 0, 0, 0, 0, 0, 0};
        for (uint32_t sIdx = 0; sIdx < c.spp; ++sIdx) {
            R L[3];
            uint32_t sig;
            for (double& a : aov) a = 0;
            nee_sample<R>(s, cb, c, x, y, c.sample_base + sIdx, L, sig, aov, cnt[tid]);
            for (int k = 0; k < 3; ++k) sum[k] += double(L[k]);
            for (int k = 0; k < 7; ++k) aov_sum[k] += aov[k];
            if (out_samples)
                for (int k = 0; k < 3; ++k) out_samples[(size_t(i) * c.spp + sIdx) * 3 + k] = double(L[k]);
            if (out_sig) out_sig[size_t(i) * c.spp + sIdx] = sig;
        }
        for (int k = 0; k < 3; ++k) out_mean[3ull * i + k] = sum[k] / double(c.spp);
        if (out_aov)
            for (int k = 0; k < 7; ++k) out_aov[7ull * i + k] = aov_sum[k] / double(c.spp);
    });
    if (out_rays) {
        out_rays[0] = out_rays[1] = out_rays[2] = 0;
        for (const Counters& k : cnt) {
            out_rays[0] += k.camera;
            out_rays[1] += k.extension;
            out_rays[2] += k.shadow;
        }
    }
    return 0;
}

// Renders the NEE integrator. pixels = NULL renders every pixel (npix ignored). Outputs per
// listed pixel: mean rgb [3], per-sample rgb [spp*3], signatures [spp], AOVs [7] (albedo
// rgb, depth, normal xyz); any output but out_mean may be NULL. out_rays: camera,
// extension, shadow ray counts.
ORACLE_API int oracle_render_nee(uint32_t n, const float* v, const float* albedo, const float* emission,
                                 const OracleConfig* cfg, const uint32_t* pixels, uint32_t npix, double* out_mean,
                                 double* out_samples, uint32_t* out_sig, double* out_aov, uint64_t* out_rays) {
    if (!cfg || !out_mean || cfg->width == 0 || cfg->height == 0 || cfg->spp == 0) return -1;
    if (n > 0 && (!v || !albedo || !emission)) return -1;
    if (cfg->precision == 32)
        return render_nee<float>(n, v, albedo, emission, cfg, pixels, npix, out_mean, out_samples, out_sig, out_aov,
                                 out_rays);
    return render_nee<double>(n, v, albedo, emission, cfg, pixels, npix, out_mean, out_samples, out_sig, out_aov,
                              out_rays);
}

// Analytic gradient of Loss with respect to per-triangle albedo and emission (FP64), for the
// image I = mean over samples [sample_base, sample_base + spp) and grad_image = dLoss/dI
// (w*h*3, top row first). For each path with vertices k on triangles h_k, NEE lights l_k and
// factors gv_k (g times visibility), beta_k = prod_{j<k} rho_j, d = grad_image(p) / spp:
//   dLoss/dLe(h_1) += d;  dLoss/dLe(l_k) += d beta_k rho_k gv_k;
//   dLoss/drho(h_k) += d beta_k H_k with H_k = Le(l_k) gv_k + rho_{k+1} H_{k+1}.
ORACLE_API int oracle_backward(uint32_t n, const float* v, const float* albedo, const float* emission,
                               const OracleConfig* cfg, const double* grad_image, double* grad_albedo,
                               double* grad_emission) {
    if (!cfg || !grad_image || !grad_albedo || !grad_emission || cfg->spp == 0) return -1;
    Lbvh b;
    build_lbvh(n, v, b);
    SceneR<double> s;
    prepare(s, n, v, albedo, emission, b);
    const CamBasis cb = camera_basis(cfg->cam_pos, cfg->cam_target, cfg->cam_up, cfg->cam_fov, cfg->width, cfg->height);
    const NeeConfig c{cfg->width, cfg->height, cfg->spp, cfg->sample_base, cfg->max_depth, cfg->seed,
                      cfg->ray_eps > 0.f ? cfg->ray_eps : 1e-4f};
    const uint32_t threads = std::max<uint32_t>(1, cfg->threads);
    std::vector<std::vector<double>> ga(threads, std::vector<double>(3ull * n, 0.0)), ge = ga;
    std::vector<Counters> cnt(threads);
    parallel_for(c.width * c.height, threads, [&](uint32_t pix, uint32_t tid) {
        const uint32_t x = pix % c.width, y = pix / c.width;
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = grad_image[3ull * pix + k] / double(c.spp);
        if (d[0] == 0.0 && d[1] == 0.0 && d[2] == 0.0) return;
        std::vector<PathVtx<double>> verts;
        for (uint32_t si = 0; si < c.spp; ++si) {
            verts.clear();
            double L[3], aov[7];
            uint32_t sig;
            nee_sample<double>(s, cb, c, x, y, c.sample_base + si, L, sig, aov, cnt[tid], &verts);
            if (verts.empty()) continue;
            for (int k = 0; k < 3; ++k) ge[tid][3ull * verts[0].prim + k] += d[k];
            const size_t nv = verts.size();
            std::vector<double> H(3 * nv, 0.0);
            for (size_t k = nv; k-- > 0;) {
                for (int ch = 0; ch < 3; ++ch) {
                    double h = 0.0;
                    if (verts[k].light >= 0) h = double(emission[3ull * verts[k].light + ch]) * verts[k].gv;
                    if (k + 1 < nv) h += double(albedo[3ull * verts[k + 1].prim + ch]) * H[3 * (k + 1) + ch];
                    H[3 * k + ch] = h;
                }
            }
            double beta[3] = {1.0, 1.0, 1.0};
            for (size_t k = 0; k < nv; ++k) {
                const int hprim = verts[k].prim;
                for (int ch = 0; ch < 3; ++ch) {
                    const double rho = albedo[3ull * hprim + ch];
                    ga[tid][3ull * hprim + ch] += d[ch] * beta[ch] * H[3 * k + ch];
                    if (verts[k].light >= 0) ge[tid][3ull * verts[k].light + ch] += d[ch] * beta[ch] * rho * verts[k].gv;
                    beta[ch] *= rho;
                }
            }
        }
    });
    for (size_t i = 0; i < 3ull * n; ++i) {
        double sa = 0.0, se = 0.0;
        for (uint32_t t = 0; t < threads; ++t) {
            sa += ga[t][i];
            se += ge[t][i];
        }
        grad_albedo[i] = sa;
        grad_emission[i] = se;
    }
    return 0;
}

// Renders the reference integrator (plugin.mm:223-309) over quads for frames
// [sample_base, sample_base + spp): out_mean [w*h*3] is the mean over those frames, out_aov
// [w*h*7] the mean AOVs (albedo rgb, depth, normal xyz). The camera direction is
// normalize(target - position) in float, as the host computes it (plugin.mm:649-674).
ORACLE_API int oracle_render_reference(uint32_t nq, const float* quads, const float* qalb, const float* qem,
                                       const OracleConfig* cfg, double* out_mean, double* out_aov) {
    if (!cfg || !out_mean || cfg->width == 0 || cfg->height == 0) return -1;
    const uint32_t w = cfg->width, h = cfg->height;
    const float aspect = static_cast<float>(w) / static_cast<float>(h);
    float dir[3] = {cfg->cam_target[0] - cfg->cam_pos[0], cfg->cam_target[1] - cfg->cam_pos[1],
                    cfg->cam_target[2] - cfg->cam_pos[2]};
    const float len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (len > 0.0f)
        for (float& x : dir) x /= len;
    parallel_for(w * h, std::max<uint32_t>(1, cfg->threads), [&](uint32_t i, uint32_t) {
        const uint32_t px = i % w, py = i / w;
        double sum[3] = {0, 0, 0}, as[7] = {0, 0, 0, 0, 0, 0, 0};
        for (uint32_t f = 0; f < cfg->spp; ++f) {
            if (cfg->precision == 32) {
                float col[3], aov[7];
                ref_sample<float>(nq, quads, qalb, qem, cfg->cam_pos, dir, cfg->cam_up, cfg->cam_fov, aspect,
                                  w, h, px, py, cfg->sample_base + f, col, aov);
                for (int k = 0; k < 3; ++k) sum[k] += col[k];
                for (int k = 0; k < 7; ++k) as[k] += aov[k];
            } else {
                double col[3], aov[7];
                ref_sample<double>(nq, quads, qalb, qem, cfg->cam_pos, dir, cfg->cam_up, cfg->cam_fov,
                                   aspect, w, h, px, py, cfg->sample_base + f, col, aov);
                for (int k = 0; k < 3; ++k) sum[k] += col[k];
                for (int k = 0; k < 7; ++k) as[k] += aov[k];
            }
        }
        for (int k = 0; k < 3; ++k) out_mean[3ull * i + k] = sum[k] / cfg->spp;
        if (out_aov)
            for (int k = 0; k < 7; ++k) out_aov[7ull * i + k] = as[k] / cfg->spp;
    });
    return 0;
}

// ---------------------------------------------------------------- benchmark scenes
//
// The library's built-in scenes (quasi_gb300/csrc/scene.cpp, Q_cuda_make_scene) restated so
// the CPU baseline and the tests can build them without loading the product library. The
// values must be bit-identical, so every step is the same double-precision operation in the
// same order: std::mt19937_64 draws (the C++ standard fixes its output), uniforms as the top
// 53 bits times 2^-53, exp/log/sin/cos by the same truncated series (not libm, which differs
// between machines), and one rounding to float at the end.

namespace gen {

constexpr double kLn2 = 0.69314718055994530941723212145818;
constexpr double kPi = 3.14159265358979323846264338327950;

// e^x as 2^k e^r, r = x - k ln2 in [-ln2/2, ln2/2], e^r by its Taylor series through r^20.
double exp_series(double x) {
    const double k = std::floor(x / kLn2 + 0.5);
    const double r = x - k * kLn2;
    double term = 1.0, acc = 1.0;
    for (int i = 1; i <= 20; ++i) {
        term = term * r / i;
        acc += term;
    }
    return std::ldexp(acc, static_cast<int>(k));
}

// ln x = e ln2 + ln m with m in [1/sqrt2, sqrt2); ln m = 2 atanh(s), s = (m-1)/(m+1), the
// atanh series through s^41.
double log_series(double x) {
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double power = s, acc = 0.0;
    for (int i = 1; i <= 41; i += 2) {
        acc += power / i;
        power *= s2;
    }
    return 2.0 * acc + e * kLn2;
}

// sin x and cos x by their Taylor series (14 terms after the first).
void sincos_series(double x, double& sn, double& cs) {
    double ts = x, tc = 1.0;
    sn = x;
    cs = 1.0;
    for (int i = 1; i <= 14; ++i) {
        ts = -ts * x * x / ((2 * i) * (2 * i + 1));
        tc = -tc * x * x / ((2 * i - 1) * (2 * i));
        sn += ts;
        cs += tc;
    }
}

struct Out {
    std::vector<float> v, alb, em;
    float cam[10] = {};  // position, target, up, fov
    void push_tri(const double* a, const double* b, const double* c, const float* albedo, const float* emission) {
        for (const double* q : {a, b, c})
            for (int k = 0; k < 3; ++k) v.push_back(static_cast<float>(q[k]));
        for (int k = 0; k < 3; ++k) {
            alb.push_back(albedo[k]);
            em.push_back(emission[k]);
        }
    }
    // corner o and edges u, w: triangles (o, o+u, o+u+w) and (o, o+u+w, o+w), each sum
    // formed left to right
    void push_quad(const double* o, const double* u, const double* w, const float* albedo, const float* emission) {
        double b[3], c[3], d[3];
        for (int k = 0; k < 3; ++k) {
            b[k] = o[k] + u[k];
            c[k] = o[k] + u[k] + w[k];
            d[k] = o[k] + w[k];
        }
        push_tri(o, b, c, albedo, emission);
        push_tri(o, c, d, albedo, emission);
    }
    void camera(float px, float py, float pz, float tx, float ty, float tz, float fov) {
        const float c[10] = {px, py, pz, tx, ty, tz, 0.f, 1.f, 0.f, fov};
        std::memcpy(cam, c, sizeof(c));
    }
};

void cornell36(Out& o) {
    const float wht[3] = {0.73f, 0.73f, 0.73f}, red[3] = {0.63f, 0.065f, 0.05f}, grn[3] = {0.14f, 0.45f, 0.09f};
    const float none[3] = {0.f, 0.f, 0.f}, lamp[3] = {17.f, 12.f, 4.f};
    const double X[3] = {1, 0, 0}, Y[3] = {0, 1, 0}, Z[3] = {0, 0, 1}, zero[3] = {0, 0, 0};
    const double ceil_o[3] = {0, 1, 0}, back_o[3] = {0, 0, 1}, right_o[3] = {1, 0, 0};
    o.push_quad(zero, X, Z, wht, none);      // floor
    o.push_quad(ceil_o, X, Z, wht, none);    // ceiling
    o.push_quad(back_o, X, Y, wht, none);    // back wall
    o.push_quad(right_o, Z, Y, red, none);   // x = 1
    o.push_quad(zero, Z, Y, grn, none);      // x = 0
    const double lo[3] = {0.375, 0.999, 0.375}, lu[3] = {0.25, 0, 0}, lw[3] = {0, 0, 0.25};
    o.push_quad(lo, lu, lw, none, lamp);     // ceiling light
    auto box = [&](const double base[3], const double size[3], double degrees) {
        double sn, cs;
        sincos_series(degrees * kPi / 180.0, sn, cs);
        double c[8][3];
        for (int i = 0; i < 8; ++i) {
            const double lx = (i & 1) ? size[0] * 0.5 : -size[0] * 0.5;
            const double ly = (i & 4) ? size[1] : 0.0;
            const double lz = (i & 2) ? size[2] * 0.5 : -size[2] * 0.5;
            c[i][0] = lx * cs + lz * sn + base[0];
            c[i][1] = ly + base[1];
            c[i][2] = -lx * sn + lz * cs + base[2];
        }
        const int faces[6][3] = {{4, 5, 6}, {0, 2, 1}, {0, 1, 4}, {3, 2, 7}, {2, 0, 6}, {1, 3, 5}};
        for (const auto& f : faces) {
            double u[3], w[3];
            for (int k = 0; k < 3; ++k) {
                u[k] = c[f[1]][k] - c[f[0]][k];
                w[k] = c[f[2]][k] - c[f[0]][k];
            }
            o.push_quad(c[f[0]], u, w, wht, none);
        }
    };
    const double b1[3] = {0.66, 0.0, 0.34}, s1[3] = {0.3, 0.3, 0.3};
    const double b2[3] = {0.34, 0.0, 0.64}, s2[3] = {0.3, 0.6, 0.3};
    box(b1, s1, -18.0);
    box(b2, s2, 18.0);
    o.camera(0.5f, 0.5f, -1.4f, 0.5f, 0.5f, 0.5f, 40.f);
}

// centres (optional): receives the drawn centre of every triangle (3 doubles each).
void soup(Out& o, uint32_t n, uint64_t seed, double* centres = nullptr) {
    std::mt19937_64 eng(seed);
    auto uniform = [&]() { return static_cast<double>(eng() >> 11) * 0x1p-53; };
    auto gaussian = [&]() {  // Marsaglia's polar method, first variate
        double a, b, r;
        do {
            a = 2.0 * uniform() - 1.0;
            b = 2.0 * uniform() - 1.0;
            r = a * a + b * b;
        } while (r >= 1.0 || r == 0.0);
        return a * std::sqrt(-2.0 * log_series(r) / r);
    };
    const double mu = log_series(0.005);
    o.v.assign(9ull * n, 0.f);
    o.alb.assign(3ull * n, 0.f);
    o.em.assign(3ull * n, 0.f);
    for (uint32_t i = 0; i < n; ++i) {
        const double centre[3] = {uniform(), uniform(), uniform()};
        if (centres) std::memcpy(centres + 3ull * i, centre, sizeof(centre));
        for (int k = 0; k < 3; ++k) {
            double d[3], r2;
            do {
                for (double& x : d) x = 2.0 * uniform() - 1.0;
                r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            } while (r2 > 1.0 || r2 < 1e-12);
            const double scale = 1.0 / std::sqrt(r2);
            const double len = exp_series(mu + 0.5 * gaussian());
            for (int a = 0; a < 3; ++a) o.v[9ull * i + 3 * k + a] = static_cast<float>(centre[a] + d[a] * scale * len);
        }
        for (int k = 0; k < 3; ++k) o.alb[3ull * i + k] = static_cast<float>(0.2 + 0.6 * uniform());
    }
    // round(n / 100) emitters drawn without replacement (partial Fisher-Yates), emission
    // drawn per emitter in ascending index order
    const uint32_t count = (n + 50) / 100;
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    std::vector<uint8_t> lit(n, 0);
    for (uint32_t k = 0; k < count && k < n; ++k) {
        const uint32_t j = k + static_cast<uint32_t>(eng() % (n - k));
        std::swap(perm[k], perm[j]);
        lit[perm[k]] = 1;
    }
    for (uint32_t i = 0; i < n; ++i)
        if (lit[i])
            for (int k = 0; k < 3; ++k) o.em[3ull * i + k] = static_cast<float>(1.0 + 9.0 * uniform());
    o.camera(0.5f, 0.5f, -1.0f, 0.5f, 0.5f, 0.5f, 40.f);
}

}  // namespace gen

// Builds "cornell36" or "soup:n=N,seed=S" (defaults n = 1000000, seed = 0). On success the
// three arrays are malloc'd (release with oracle_free) and cam receives position, target, up
// and fov. Returns 0, or -1 for an unknown spec.
ORACLE_API int oracle_make_scene(const char* spec, uint32_t* tri_count, float** vertices, float** albedo,
                                 float** emission, float* cam) {
    if (!spec || !tri_count || !vertices || !albedo || !emission || !cam) return -1;
    const std::string sp(spec);
    gen::Out o;
    if (sp == "cornell36") {
        gen::cornell36(o);
    } else if (sp.rfind("soup", 0) == 0) {
        auto field = [&](const char* key, uint64_t dflt) {
            const std::string k = std::string(key) + "=";
            const size_t at = sp.find(k);
            return at == std::string::npos ? dflt : std::strtoull(sp.c_str() + at + k.size(), nullptr, 10);
        };
        const uint64_t n = field("n", 1000000), seed = field("seed", 0);
        if (n == 0 || n > (1ull << 26)) return -1;
        gen::soup(o, static_cast<uint32_t>(n), seed);
    } else {
        return -1;
    }
    auto dup = [](const std::vector<float>& a) {
        float* p = static_cast<float*>(std::malloc(sizeof(float) * std::max<size_t>(a.size(), 1)));
        if (p && !a.empty()) std::memcpy(p, a.data(), sizeof(float) * a.size());
        return p;
    };
    *tri_count = static_cast<uint32_t>(o.v.size() / 9);
    *vertices = dup(o.v);
    *albedo = dup(o.alb);
    *emission = dup(o.em);
    std::memcpy(cam, o.cam, sizeof(o.cam));
    return 0;
}

ORACLE_API void oracle_free(void* p) { std::free(p); }

// The centres the soup generator draws for "soup:n=N,seed=S" (3 doubles per triangle), for
// tests of its edge-length distribution.
ORACLE_API int oracle_soup_centres(uint32_t n, uint64_t seed, double* centres) {
    if (!centres || n == 0) return -1;
    gen::Out o;
    gen::soup(o, n, seed, centres);
    return 0;
}

ORACLE_API uint32_t oracle_hardware_threads(void) { return std::max(1u, std::thread::hardware_concurrency()); }
