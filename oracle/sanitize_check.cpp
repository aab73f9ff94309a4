// sanitize_check.cpp - runs the CPU oracle (test infrastructure) under AddressSanitizer and
// UndefinedBehaviorSanitizer: LBVH, 8-wide collapse, the NEE integrator in FP64 and FP32,
// the adjoint and the reference integrator, on seeded scenes including the edge cases
// (0, 1, 2 triangles, coincident and flat triangles). Built by `make -C oracle sanitize`;
// exits non-zero on the first failing call (the sanitizers abort on any report).
#include "oracle.cpp"

#include <cstdio>
#include <random>

namespace {

int check(const char* what, int rc) {
    if (rc != 0) std::fprintf(stderr, "%s failed: %d\n", what, rc);
    return rc != 0;
}

int run_scene(const char* name, std::vector<float> v, uint32_t threads) {
    const uint32_t n = static_cast<uint32_t>(v.size() / 9);
    std::vector<float> albedo(3ull * n, 0.6f), emission(3ull * n, 0.0f);
    for (uint32_t i = 0; i < n; i += 7) emission[3ull * i] = emission[3ull * i + 1] = emission[3ull * i + 2] = 4.0f;
    const uint32_t nodes = n > 1 ? n - 1 : 1;
    std::vector<uint32_t> morton(n + 1), order(n + 1), words(24ull * nodes);
    std::vector<int32_t> children(2ull * nodes);
    std::vector<float> boxes(12ull * nodes), bounds(6);
    int bad = 0;
    bad |= check("lbvh", oracle_lbvh(n, v.data(), morton.data(), order.data(), children.data(), boxes.data(),
                                     bounds.data()));
    bad |= check("collapse8", oracle_collapse8(n, v.data(), words.data()));
    OracleConfig c{};
    c.width = 16;
    c.height = 12;
    c.spp = 2;
    c.max_depth = 4;
    c.seed = 3;
    const float pos[3] = {0.5f, 0.5f, -1.0f}, tgt[3] = {0.5f, 0.5f, 0.5f}, up[3] = {0.0f, 1.0f, 0.0f};
    std::memcpy(c.cam_pos, pos, sizeof pos);
    std::memcpy(c.cam_target, tgt, sizeof tgt);
    std::memcpy(c.cam_up, up, sizeof up);
    c.cam_fov = 40.0f;
    c.ray_eps = 1e-4f;
    c.threads = threads;
    const size_t px = size_t(c.width) * c.height;
    std::vector<double> mean(3 * px), samples(3 * px * c.spp), aov(7 * px), grad(3 * px, 1e-3);
    std::vector<uint32_t> sig(px * c.spp);
    uint64_t rays[3] = {};
    for (uint32_t precision : {64u, 32u}) {
        c.precision = precision;
        bad |= check("render_nee", oracle_render_nee(n, v.data(), albedo.data(), emission.data(), &c, nullptr, 0,
                                                     mean.data(), samples.data(), sig.data(), aov.data(), rays));
    }
    c.precision = 64;
    std::vector<double> ga(3ull * n + 3), ge(3ull * n + 3);
    bad |= check("backward", oracle_backward(n, v.data(), albedo.data(), emission.data(), &c, grad.data(), ga.data(),
                                             ge.data()));
    std::printf("%-12s n=%-6u %s\n", name, n, bad ? "FAILED" : "ok");
    return bad;
}

}  // namespace

int main() {
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    auto soup = [&](uint32_t n) {
        std::vector<float> v(9ull * n);
        for (uint32_t i = 0; i < n; ++i) {
            const float cx = u(rng), cy = u(rng), cz = u(rng);
            for (int k = 0; k < 3; ++k) {
                v[9ull * i + 3 * k + 0] = cx + 0.05f * (u(rng) - 0.5f);
                v[9ull * i + 3 * k + 1] = cy + 0.05f * (u(rng) - 0.5f);
                v[9ull * i + 3 * k + 2] = cz + 0.05f * (u(rng) - 0.5f);
            }
        }
        return v;
    };
    int bad = 0;
    bad |= run_scene("empty", {}, 2);
    bad |= run_scene("one", soup(1), 2);
    bad |= run_scene("two", soup(2), 2);
    bad |= run_scene("soup", soup(3000), 4);
    std::vector<float> same = soup(1);
    for (int i = 0; i < 6; ++i) same.insert(same.end(), same.begin(), same.begin() + 9);  // 7 coincident
    bad |= run_scene("coincident", same, 2);
    std::vector<float> flat = soup(500);
    for (size_t i = 1; i < flat.size(); i += 3) flat[i] = 0.25f;  // zero extent on y
    bad |= run_scene("flat", flat, 2);
    // the reference integrator on two quads (origin, u, v)
    const float quads[18] = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 0, 0, 0, 0, -1};
    const float qa[6] = {0.7f, 0.7f, 0.7f, 0.5f, 0.5f, 0.5f}, qe[6] = {0, 0, 0, 3, 3, 3};
    OracleConfig c{};
    c.width = 8;
    c.height = 8;
    c.spp = 1;
    c.max_depth = 5;
    const float pos[3] = {0.5f, 0.5f, 2.0f}, tgt[3] = {0.5f, 0.5f, 0.0f}, up[3] = {0.0f, 1.0f, 0.0f};
    std::memcpy(c.cam_pos, pos, sizeof pos);
    std::memcpy(c.cam_target, tgt, sizeof tgt);
    std::memcpy(c.cam_up, up, sizeof up);
    c.cam_fov = 40.0f;
    c.threads = 2;
    std::vector<double> mean(3 * 64), aov(7 * 64);
    bad |= check("render_reference", oracle_render_reference(2, quads, qa, qe, &c, mean.data(), aov.data()));
    std::printf("%s\n", bad ? "FAILED" : "all ok");
    return bad;
}
