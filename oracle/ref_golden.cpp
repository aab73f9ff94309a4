// ref_golden.cpp - runs the reference's own code on the CPU and prints golden vectors as
// JSON. TEST INFRASTRUCTURE ONLY; built by `make -C oracle ref` into oracle/_ref/ from the
// sources under the reference checkout (it is never part of the product).
//
// It includes, unmodified:
//   src/quasi/scene/cornell_box.hpp, camera.hpp, quad.hpp, math/*.hpp   (C++ headers)
//   the shader source of backends/metal/plugin.mm:30-31,46-276 (extracted by the Makefile
//   into _ref/msl_pathtrace.inc and compiled through msl_shim.hpp)
// and drives them the way plugin.mm's host code and fragment stage do (seeding at :295,
// pixel-centre uv from the fullscreen triangle at :39-44, running-mean accumulation at
// :313-330, AOV depth normalisation at :301).
#include <quasi/scene/cornell_box.hpp>

#include "msl_shim.hpp"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace msl {
#include "msl_pathtrace.inc"
}  // namespace msl

namespace {

std::string f9(float v) {
    char b[48];
    std::snprintf(b, sizeof b, "%.9g", static_cast<double>(v));
    return b;
}

void arr(std::string& out, const float* v, size_t n) {
    out += "[";
    for (size_t i = 0; i < n; ++i) {
        if (i) out += ",";
        out += f9(v[i]);
    }
    out += "]";
}

int order_probe_counter = 0;
float order_probe(int expect) {
    const int got = order_probe_counter++;
    return got == expect ? 1.0f : 0.0f;
}

msl::Camera make_msl_camera(const float pos[3], const float target[3], const float up[3], float fov, float aspect) {
    // plugin.mm:649-674: the host normalises target - position in float.
    float dx = target[0] - pos[0], dy = target[1] - pos[1], dz = target[2] - pos[2];
    const float len = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (len > 0.0f) {
        dx /= len;
        dy /= len;
        dz /= len;
    }
    msl::Camera c{};
    c.position = {pos[0], pos[1], pos[2]};
    c.fov = fov;
    c.direction = {dx, dy, dz};
    c.aspect = aspect;
    c.up = {up[0], up[1], up[2]};
    return c;
}

}  // namespace

int main() {
    // C++20 evaluates parenthesised aggregate initialisers left to right, as Metal does for
    // float2(random_float(rng), random_float(rng)); refuse to emit vectors otherwise.
    const msl::float2 probe(order_probe(0), order_probe(1));
    if (probe.x != 1.0f || probe.y != 1.0f) {
        std::fprintf(stderr, "float2 initialisers not evaluated left to right\n");
        return 2;
    }

    std::string js = "{\n";

    // pcg_hash (plugin.mm:98-102)
    std::vector<uint32_t> ins = {0u, 1u, 2u, 3u, 7u, 255u, 256u, 65535u, 65536u, 1920u, 2073600u,
                                 0x7fffffffu, 0x80000000u, 0xfffffff0u, 0xffffffffu, 123456789u};
    for (uint32_t i = 0; i < 48; ++i) ins.push_back(i * 2654435761u + 12345u);
    js += "\"pcg_hash\": {\"in\": [";
    for (size_t i = 0; i < ins.size(); ++i) js += (i ? "," : "") + std::to_string(ins[i]);
    js += "], \"out\": [";
    for (size_t i = 0; i < ins.size(); ++i) js += (i ? "," : "") + std::to_string(msl::pcg_hash(ins[i]));
    js += "]},\n";

    // random_float chains (plugin.mm:104-107), including states whose hash is near 2^32.
    js += "\"random_float\": [";
    const uint32_t seeds[] = {0u, 1u, 42u, 0xdeadbeefu, 2073599u};
    for (size_t s = 0; s < 5; ++s) {
        uint32_t st = seeds[s];
        float v[16];
        for (float& x : v) x = msl::random_float(st);
        js += std::string(s ? "," : "") + "{\"seed\": " + std::to_string(seeds[s]) + ", \"values\": ";
        arr(js, v, 16);
        js += ", \"final_state\": " + std::to_string(st) + "}";
    }
    js += "],\n";

    // cosine_sample_hemisphere (plugin.mm:111-125)
    const float normals[][3] = {{0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {0, 0, 1}, {0.6f, 0.8f, 0}, {0.95f, 0.1f, 0.2f},
                                {-0.3f, 0.4f, -0.866f}, {0.91f, -0.41f, 0.05f}};
    js += "\"cosine_sample\": [";
    for (int i = 0; i < 8; ++i) {
        for (uint32_t k = 0; k < 4; ++k) {
            const uint32_t state0 = 977u * static_cast<uint32_t>(i) + 31u * k + 5u;
            uint32_t st = state0;
            const msl::float3 d = msl::cosine_sample_hemisphere(msl::float3(normals[i][0], normals[i][1], normals[i][2]), st);
            const float dv[3] = {d.x, d.y, d.z};
            js += std::string(i || k ? "," : "") + "{\"normal\": ";
            arr(js, normals[i], 3);
            js += ", \"state\": " + std::to_string(state0) + ", \"dir\": ";
            arr(js, dv, 3);
            js += "}";
        }
    }
    js += "],\n";

    // Reference scene (cornell_box.hpp:95-134) and its camera.
    const Q::scene::cornell_box_scene scene = Q::scene::make_cornell_box(1.0f);
    js += "\"cornell\": {\"light_index\": " + std::to_string(scene.light_index) + ", \"quads\": [";
    for (size_t i = 0; i < scene.quads.size(); ++i) {
        const auto& q = scene.quads[i];
        const float g[15] = {q.geometry.origin.x, q.geometry.origin.y, q.geometry.origin.z, q.geometry.u.x,
                             q.geometry.u.y,      q.geometry.u.z,      q.geometry.v.x,      q.geometry.v.y,
                             q.geometry.v.z,      q.mat.albedo.x,      q.mat.albedo.y,      q.mat.albedo.z,
                             q.mat.emission.x,    q.mat.emission.y,    q.mat.emission.z};
        if (i) js += ",";
        arr(js, g, 15);
    }
    const float cam[11] = {scene.cam.position.x, scene.cam.position.y, scene.cam.position.z, scene.cam.direction.x,
                           scene.cam.direction.y, scene.cam.direction.z, scene.cam.up.x, scene.cam.up.y, scene.cam.up.z,
                           scene.cam.fov, scene.cam.aspect};
    js += "], \"camera\": ";
    arr(js, cam, 11);
    js += "},\n";

    // camera::get_ray (camera.hpp:36-52) on a uv grid, no jitter.
    js += "\"camera_get_ray\": [";
    for (int iy = 0; iy < 5; ++iy)
        for (int ix = 0; ix < 5; ++ix) {
            const float u = 0.1f + 0.2f * ix, v = 0.05f + 0.225f * iy;
            const Q::math::ray r = scene.cam.get_ray(u, v);
            const float g[8] = {u, v, r.origin.x, r.origin.y, r.origin.z, r.direction.x, r.direction.y, r.direction.z};
            js += std::string(iy || ix ? "," : "");
            arr(js, g, 8);
        }
    js += "],\n";

    // get_camera_ray of the shader (plugin.mm:129-153), jittered, host camera of main.cpp.
    const float host_pos[3] = {0.f, 1.f, 3.5f}, host_target[3] = {0.f, 1.f, 0.f}, host_up[3] = {0.f, 1.f, 0.f};
    const msl::Camera mcam = make_msl_camera(host_pos, host_target, host_up, 40.0f, 1.0f);
    js += "\"msl_camera_ray\": [";
    for (int i = 0; i < 16; ++i) {
        const uint32_t state0 = msl::pcg_hash(static_cast<uint32_t>(i) * 7919u);
        uint32_t st = state0;
        const msl::float2 uv{(static_cast<float>(i % 4) + 0.5f) / 4.0f, 1.0f - (static_cast<float>(i / 4) + 0.5f) / 4.0f};
        const msl::Ray r = msl::get_camera_ray(mcam, uv, st);
        const float g[8] = {uv.x, uv.y, r.origin.x, r.origin.y, r.origin.z, r.direction.x, r.direction.y, r.direction.z};
        js += std::string(i ? "," : "") + "{\"state\": " + std::to_string(state0) + ", \"ray\": ";
        arr(js, g, 8);
        js += "}";
    }
    js += "],\n";

    // Quad intersection: quad.hpp:51-109 and the shader's intersect_quad, same rays.
    js += "\"quad_hits\": [";
    bool first = true;
    for (int i = 0; i < 24; ++i) {
        uint32_t st = 1000u + static_cast<uint32_t>(i);
        const msl::float2 uv{msl::random_float(st), msl::random_float(st)};
        const msl::Ray r = msl::get_camera_ray(mcam, uv, st);
        for (size_t q = 0; q < scene.quads.size(); ++q) {
            const auto& g = scene.quads[q].geometry;
            const Q::math::ray cr{{r.origin.x, r.origin.y, r.origin.z}, {r.direction.x, r.direction.y, r.direction.z}};
            const auto hit = Q::scene::intersect(cr, g, 0.001f, 1e30f);
            msl::Quad mq{};
            mq.origin = {g.origin.x, g.origin.y, g.origin.z};
            mq.u = {g.u.x, g.u.y, g.u.z};
            mq.v = {g.v.x, g.v.y, g.v.z};
            const msl::HitRecord mh = msl::intersect_quad(r, mq, static_cast<msl::uint>(q), 0.001f, 1e30f);
            const float ray[6] = {r.origin.x, r.origin.y, r.origin.z, r.direction.x, r.direction.y, r.direction.z};
            js += std::string(first ? "" : ",") + "{\"ray\": ";
            first = false;
            arr(js, ray, 6);
            js += ", \"quad\": " + std::to_string(q) + ", \"cpp_hit\": " + (hit ? "true" : "false");
            js += ", \"msl_hit\": " + std::string(mh.hit ? "true" : "false");
            if (hit) {
                const float h[7] = {hit->t, hit->point.x, hit->point.y, hit->point.z, hit->normal.x, hit->normal.y,
                                    hit->normal.z};
                js += ", \"cpp\": ";
                arr(js, h, 7);
            }
            if (mh.hit) {
                const float h[7] = {mh.t, mh.point.x, mh.point.y, mh.point.z, mh.normal.x, mh.normal.y, mh.normal.z};
                js += ", \"msl\": ";
                arr(js, h, 7);
            }
            js += "}";
        }
    }
    js += "],\n";

    // Whole frames: the shader's path_trace per pixel with the reference's seeding and the
    // running-mean accumulation of plugin.mm:313-330 over `frames` frames.
    const uint32_t W = 24, H = 24, frames = 16;
    msl::SceneUniforms su{};
    su.camera = make_msl_camera(host_pos, host_target, host_up, 40.0f, static_cast<float>(W) / static_cast<float>(H));
    su.quad_count = static_cast<msl::uint>(std::min<size_t>(scene.quads.size(), 32));
    su.light_index = static_cast<msl::uint>(scene.light_index);
    for (uint32_t i = 0; i < su.quad_count; ++i) {
        const auto& q = scene.quads[i];
        su.quads[i].origin = {q.geometry.origin.x, q.geometry.origin.y, q.geometry.origin.z};
        su.quads[i].u = {q.geometry.u.x, q.geometry.u.y, q.geometry.u.z};
        su.quads[i].v = {q.geometry.v.x, q.geometry.v.y, q.geometry.v.z};
        su.materials[i].albedo = {q.mat.albedo.x, q.mat.albedo.y, q.mat.albedo.z};
        su.materials[i].roughness = q.mat.roughness;
        su.materials[i].emission = {q.mat.emission.x, q.mat.emission.y, q.mat.emission.z};
        su.materials[i].metallic = q.mat.metallic;
    }
    std::vector<float> acc(W * H * 4 * 4, 0.0f);  // beauty, albedo, normal, depth (RGBA each)
    for (uint32_t f = 0; f < frames; ++f) {
        su.frame_count = f;
        const float weight = 1.0f / static_cast<float>(f + 1);
        for (uint32_t py = 0; py < H; ++py)
            for (uint32_t px = 0; px < W; ++px) {
                const msl::float2 uv{(static_cast<float>(px) + 0.5f) / static_cast<float>(W),
                                     1.0f - (static_cast<float>(py) + 0.5f) / static_cast<float>(H)};
                msl::uint rng = msl::pcg_hash(px + py * 1920u + su.frame_count * 1920u * 1080u);
                const msl::Ray ray = msl::get_camera_ray(su.camera, uv, rng);
                const msl::PathTraceResult pt = msl::path_trace(ray, su, rng);
                const float nd = std::min(std::max((pt.first_hit_depth - 1.0f) / 4.0f, 0.0f), 1.0f);
                const float vals[4][4] = {{pt.color.x, pt.color.y, pt.color.z, 1.0f},
                                          {pt.first_hit_albedo.x, pt.first_hit_albedo.y, pt.first_hit_albedo.z, 1.0f},
                                          {pt.first_hit_normal.x, pt.first_hit_normal.y, pt.first_hit_normal.z, 1.0f},
                                          {nd, nd, nd, 1.0f}};
                for (int a = 0; a < 4; ++a)
                    for (int c = 0; c < 4; ++c) {
                        float& dst = acc[((a * H + py) * W + px) * 4 + c];
                        dst = dst + (vals[a][c] - dst) * weight;  // mix(history, new, weight)
                    }
            }
    }
    js += "\"render\": {\"width\": " + std::to_string(W) + ", \"height\": " + std::to_string(H) +
          ", \"frames\": " + std::to_string(frames) + ", \"camera\": {\"position\": ";
    arr(js, host_pos, 3);
    js += ", \"target\": ";
    arr(js, host_target, 3);
    js += ", \"up\": ";
    arr(js, host_up, 3);
    js += ", \"fov\": 40}";
    const char* names[4] = {"beauty", "albedo", "normal", "depth"};
    for (int a = 0; a < 4; ++a) {
        js += std::string(", \"") + names[a] + "\": ";
        arr(js, &acc[a * W * H * 4], W * H * 4);
    }
    js += "}\n}\n";
    std::fwrite(js.data(), 1, js.size(), stdout);
    return 0;
}
