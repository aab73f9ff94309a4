// scene.cpp - the built-in scenes, generated on the host.
//
// Generators use std::mt19937_64 (fully specified by the C++ standard) and only +,-,*,/,
// sqrt, frexp and ldexp (correctly rounded everywhere). exp, log and sin/cos are evaluated
// by the series below instead of libm, so a scene is bit-identical on x86 and on Arm. The
// translation unit is compiled with -ffp-contract=off for the same reason.
#include "../../include/quasi_cuda.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace quasi {
namespace {

constexpr double k_ln2 = 0.69314718055994530941723212145818;
constexpr double k_pi_d = 3.14159265358979323846264338327950;

// exp(x): x = k ln2 + r with |r| <= ln2/2, Taylor series of e^r to degree 20.
double series_exp(double x) {
    const double k = std::floor(x / k_ln2 + 0.5);
    const double r = x - k * k_ln2;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i <= 20; ++i) {
        term = term * r / i;
        sum += term;
    }
    return std::ldexp(sum, static_cast<int>(k));
}

// log(x), x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh((m-1)/(m+1)).
double series_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0.70710678118654752440) {
        m *= 2.0;
        e -= 1;
    }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double pw = s, sum = 0.0;
    for (int i = 1; i <= 41; i += 2) {
        sum += pw / i;
        pw *= s2;
    }
    return 2.0 * sum + e * k_ln2;
}

// sin and cos of |x| <= pi by Taylor series (used only for fixed box rotations).
void series_sincos(double x, double& s, double& c) {
    double term_s = x, term_c = 1.0;
    s = x;
    c = 1.0;
    for (int i = 1; i <= 14; ++i) {
        term_s = -term_s * x * x / ((2 * i) * (2 * i + 1));
        term_c = -term_c * x * x / ((2 * i - 1) * (2 * i));
        s += term_s;
        c += term_c;
    }
}

struct Vec {
    double x, y, z;
};

struct Builder {
    std::vector<float> v, alb, em, quads, qalb, qem;
    Q_camera cam{};

    void tri(Vec a, Vec b, Vec c, const float* albedo, const float* emission) {
        const Vec p[3] = {a, b, c};
        for (const Vec& q : p) {
            v.push_back(static_cast<float>(q.x));
            v.push_back(static_cast<float>(q.y));
            v.push_back(static_cast<float>(q.z));
        }
        for (int k = 0; k < 3; ++k) {
            alb.push_back(albedo[k]);
            em.push_back(emission[k]);
        }
    }
    // Parallelogram (o, u, v) as two triangles (o, o+u, o+u+v) and (o, o+u+v, o+v).
    void quad_tris(Vec o, Vec u, Vec w, const float* albedo, const float* emission) {
        const Vec a = o, b = {o.x + u.x, o.y + u.y, o.z + u.z};
        const Vec c = {o.x + u.x + w.x, o.y + u.y + w.y, o.z + u.z + w.z}, d = {o.x + w.x, o.y + w.y, o.z + w.z};
        tri(a, b, c, albedo, emission);
        tri(a, c, d, albedo, emission);
    }
};

void fill(const Builder& b, Q_cuda_scene* out) {
    auto dup = [](const std::vector<float>& src) -> float* {
        if (src.empty()) return nullptr;
        float* p = static_cast<float*>(std::malloc(sizeof(float) * src.size()));
        if (p) std::memcpy(p, src.data(), sizeof(float) * src.size());
        return p;
    };
    std::memset(out, 0, sizeof(*out));
    out->tri_count = static_cast<uint32_t>(b.v.size() / 9);
    out->vertices = dup(b.v);
    out->albedo = dup(b.alb);
    out->emission = dup(b.em);
    out->quad_count = static_cast<uint32_t>(b.quads.size() / 9);
    out->quads = dup(b.quads);
    out->quad_albedo = dup(b.qalb);
    out->quad_emission = dup(b.qem);
    out->camera = b.cam;
}

void set_camera(Q_camera& c, float px, float py, float pz, float tx, float ty, float tz, float fov) {
    c.position[0] = px; c.position[1] = py; c.position[2] = pz;
    c.target[0] = tx; c.target[1] = ty; c.target[2] = tz;
    c.up[0] = 0.f; c.up[1] = 1.f; c.up[2] = 0.f;
    c.fov = fov;
}

// The Cornell box of 36 triangles: unit box open towards -z, red and green side walls,
// a 0.25 x 0.25 ceiling light with emission (17, 12, 4), a 0.3 cube and a 0.3 x 0.6 x 0.3
// box rotated by -18 and +18 degrees about y. Camera at (0.5, 0.5, -1.4) looking +z.
void make_cornell36(Builder& b) {
    const float white[3] = {0.73f, 0.73f, 0.73f}, red[3] = {0.63f, 0.065f, 0.05f};
    const float green[3] = {0.14f, 0.45f, 0.09f}, black[3] = {0.f, 0.f, 0.f};
    const float light[3] = {17.f, 12.f, 4.f};
    b.quad_tris({0, 0, 0}, {1, 0, 0}, {0, 0, 1}, white, black);   // floor y = 0
    b.quad_tris({0, 1, 0}, {1, 0, 0}, {0, 0, 1}, white, black);   // ceiling y = 1
    b.quad_tris({0, 0, 1}, {1, 0, 0}, {0, 1, 0}, white, black);   // back z = 1
    b.quad_tris({1, 0, 0}, {0, 0, 1}, {0, 1, 0}, red, black);     // x = 1, image left
    b.quad_tris({0, 0, 0}, {0, 0, 1}, {0, 1, 0}, green, black);   // x = 0, image right
    b.quad_tris({0.375, 0.999, 0.375}, {0.25, 0, 0}, {0, 0, 0.25}, black, light);
    auto box = [&](Vec base, Vec size, double deg) {
        double s, c;
        series_sincos(deg * k_pi_d / 180.0, s, c);
        Vec p[8];
        for (int i = 0; i < 8; ++i) {
            const double lx = (i & 1) ? size.x * 0.5 : -size.x * 0.5;
            const double ly = (i & 4) ? size.y : 0.0;
            const double lz = (i & 2) ? size.z * 0.5 : -size.z * 0.5;
            p[i] = {lx * c + lz * s + base.x, ly + base.y, -lx * s + lz * c + base.z};
        }
        auto face = [&](int o, int u, int w) {
            b.quad_tris(p[o], {p[u].x - p[o].x, p[u].y - p[o].y, p[u].z - p[o].z},
                        {p[w].x - p[o].x, p[w].y - p[o].y, p[w].z - p[o].z}, white, black);
        };
        face(4, 5, 6);  // top
        face(0, 2, 1);  // bottom
        face(0, 1, 4);  // -z
        face(3, 2, 7);  // +z
        face(2, 0, 6);  // -x
        face(1, 3, 5);  // +x
    };
    box({0.66, 0.0, 0.34}, {0.3, 0.3, 0.3}, -18.0);
    box({0.34, 0.0, 0.64}, {0.3, 0.6, 0.3}, 18.0);
    set_camera(b.cam, 0.5f, 0.5f, -1.4f, 0.5f, 0.5f, 0.5f, 40.f);
}

// src/quasi/scene/cornell_box.hpp:95-134, evaluated in float with the same operation order
// (rotate_y at cornell_box.hpp:32-37, add_box at :45-90), as 16 quads and as 32 triangles.
void make_refcornell(Builder& b) {
    struct V3f {
        float x, y, z;
    };
    auto add = [](V3f a, V3f c) { return V3f{a.x + c.x, a.y + c.y, a.z + c.z}; };
    auto sub = [](V3f a, V3f c) { return V3f{a.x - c.x, a.y - c.y, a.z - c.z}; };
    auto quad = [&](V3f o, V3f u, V3f v, const float* albedo, const float* emission) {
        const float g[9] = {o.x, o.y, o.z, u.x, u.y, u.z, v.x, v.y, v.z};
        b.quads.insert(b.quads.end(), g, g + 9);
        b.qalb.insert(b.qalb.end(), albedo, albedo + 3);
        b.qem.insert(b.qem.end(), emission, emission + 3);
        const V3f p1 = add(o, u), p2 = add(add(o, u), v), p3 = add(o, v);
        b.tri({o.x, o.y, o.z}, {p1.x, p1.y, p1.z}, {p2.x, p2.y, p2.z}, albedo, emission);
        b.tri({o.x, o.y, o.z}, {p2.x, p2.y, p2.z}, {p3.x, p3.y, p3.z}, albedo, emission);
    };
    const float white[3] = {0.73f, 0.73f, 0.73f}, red[3] = {0.65f, 0.05f, 0.05f};
    const float green[3] = {0.12f, 0.45f, 0.15f}, zero[3] = {0.f, 0.f, 0.f};
    const float light[3] = {15.f, 15.f, 15.f};
    quad({-1, 0, -1}, {2, 0, 0}, {0, 0, 2}, white, zero);
    quad({-1, 2, 1}, {2, 0, 0}, {0, 0, -2}, white, zero);
    quad({-1, 0, -1}, {2, 0, 0}, {0, 2, 0}, white, zero);
    quad({-1, 0, 1}, {0, 0, -2}, {0, 2, 0}, red, zero);
    quad({1, 0, -1}, {0, 0, 2}, {0, 2, 0}, green, zero);
    quad({-0.25f, 1.99f, -0.25f}, {0.5f, 0, 0}, {0, 0, 0.5f}, zero, light);
    auto box = [&](V3f center, V3f size, float angle) {
        const float hw = size.x * 0.5f, h = size.y, hd = size.z * 0.5f;
        const V3f local[8] = {{-hw, 0, -hd}, {hw, 0, -hd}, {-hw, 0, hd}, {hw, 0, hd},
                              {-hw, h, -hd}, {hw, h, -hd}, {-hw, h, hd}, {hw, h, hd}};
        // The angle in radians is formed in float as in the reference; its sine and cosine
        // are the correctly rounded float values of the double series.
        const float rad = angle * 3.14159265359f / 180.0f;
        double sd, cd;
        series_sincos(static_cast<double>(rad), sd, cd);
        const float c = static_cast<float>(cd), s = static_cast<float>(sd);
        V3f p[8];
        for (int i = 0; i < 8; ++i) {
            const V3f r{local[i].x * c + local[i].z * s, local[i].y, -local[i].x * s + local[i].z * c};
            p[i] = add(r, center);
        }
        quad(p[4], sub(p[5], p[4]), sub(p[6], p[4]), white, zero);
        quad(p[0], sub(p[1], p[0]), sub(p[4], p[0]), white, zero);
        quad(p[3], sub(p[2], p[3]), sub(p[7], p[3]), white, zero);
        quad(p[2], sub(p[0], p[2]), sub(p[6], p[2]), white, zero);
        quad(p[1], sub(p[3], p[1]), sub(p[5], p[1]), white, zero);
    };
    box({-0.35f, 0.0f, 0.3f}, {0.5f, 1.2f, 0.5f}, 15.0f);
    box({0.35f, 0.0f, -0.3f}, {0.55f, 0.55f, 0.55f}, -18.0f);
    set_camera(b.cam, 0.f, 1.f, 3.5f, 0.f, 1.f, 0.f, 40.f);
}

// Seeded triangle soup. Per triangle, in order: a centre uniform in [0,1)^3; per vertex a
// direction uniform on the sphere (rejection from the cube) and a length
// exp(ln 0.005 + 0.5 N(0,1)) (Marsaglia polar normal); the albedo uniform in [0.2,0.8)^3.
// Then round(n/100) distinct emitters by a partial Fisher-Yates shuffle, and for each
// emitter in ascending index order an emission uniform in [1,10)^3.
void make_soup(Builder& b, uint32_t n, uint64_t seed) {
    std::mt19937_64 rng(seed);
    auto u01 = [&]() { return static_cast<double>(rng() >> 11) * 0x1p-53; };
    auto normal = [&]() {
        double a, c, s;
        do {
            a = 2.0 * u01() - 1.0;
            c = 2.0 * u01() - 1.0;
            s = a * a + c * c;
        } while (s >= 1.0 || s == 0.0);
        return a * std::sqrt(-2.0 * series_log(s) / s);
    };
    const double log_median = series_log(0.005);
    b.v.resize(9ull * n);
    b.alb.resize(3ull * n);
    b.em.assign(3ull * n, 0.f);
    for (uint32_t i = 0; i < n; ++i) {
        const double cx = u01(), cy = u01(), cz = u01();
        for (int k = 0; k < 3; ++k) {
            double dx, dy, dz, r2;
            do {
                dx = 2.0 * u01() - 1.0;
                dy = 2.0 * u01() - 1.0;
                dz = 2.0 * u01() - 1.0;
                r2 = dx * dx + dy * dy + dz * dz;
            } while (r2 > 1.0 || r2 < 1e-12);
            const double inv = 1.0 / std::sqrt(r2);
            const double len = series_exp(log_median + 0.5 * normal());
            b.v[9ull * i + 3 * k + 0] = static_cast<float>(cx + dx * inv * len);
            b.v[9ull * i + 3 * k + 1] = static_cast<float>(cy + dy * inv * len);
            b.v[9ull * i + 3 * k + 2] = static_cast<float>(cz + dz * inv * len);
        }
        for (int k = 0; k < 3; ++k) b.alb[3ull * i + k] = static_cast<float>(0.2 + 0.6 * u01());
    }
    const uint32_t n_emit = (n + 50) / 100;
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::vector<char> is_emit(n, 0);
    for (uint32_t k = 0; k < n_emit && k < n; ++k) {
        const uint32_t j = k + static_cast<uint32_t>(rng() % (n - k));
        std::swap(idx[k], idx[j]);
        is_emit[idx[k]] = 1;
    }
    for (uint32_t i = 0; i < n; ++i)
        if (is_emit[i])
            for (int k = 0; k < 3; ++k) b.em[3ull * i + k] = static_cast<float>(1.0 + 9.0 * u01());
    set_camera(b.cam, 0.5f, 0.5f, -1.0f, 0.5f, 0.5f, 0.5f, 40.f);
}

bool parse_kv(const std::string& spec, const char* key, uint64_t& value) {
    const std::string k = std::string(key) + "=";
    const size_t p = spec.find(k);
    if (p == std::string::npos) return false;
    char* end = nullptr;
    value = std::strtoull(spec.c_str() + p + k.size(), &end, 10);
    return end != spec.c_str() + p + k.size();
}

}  // namespace
}  // namespace quasi

extern "C" Q_CUDA_EXPORT int Q_cuda_make_scene(const char* spec, Q_cuda_scene* out) {
    if (!spec || !out) return QUASI_ERR_INVALID;
    const std::string s(spec);
    quasi::Builder b;
    if (s == "cornell36") {
        quasi::make_cornell36(b);
    } else if (s == "refcornell") {
        quasi::make_refcornell(b);
    } else if (s.rfind("soup", 0) == 0) {
        uint64_t n = 1000000, seed = 0;
        quasi::parse_kv(s, "n", n);
        quasi::parse_kv(s, "seed", seed);
        if (n == 0 || n > (1ull << 26)) return QUASI_ERR_INVALID;
        quasi::make_soup(b, static_cast<uint32_t>(n), seed);
    } else {
        return QUASI_ERR_INVALID;
    }
    quasi::fill(b, out);
    if (out->tri_count && (!out->vertices || !out->albedo || !out->emission)) {
        Q_cuda_free_scene(out);
        return QUASI_ERR_OOM;
    }
    return QUASI_OK;
}

extern "C" Q_CUDA_EXPORT void Q_cuda_free_scene(Q_cuda_scene* sc) {
    if (!sc) return;
    std::free(sc->vertices);
    std::free(sc->albedo);
    std::free(sc->emission);
    std::free(sc->quads);
    std::free(sc->quad_albedo);
    std::free(sc->quad_emission);
    std::memset(sc, 0, sizeof(*sc));
}
