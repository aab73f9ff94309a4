// quasi_headless.cpp - headless C++ host for libquasi_cuda.so.
//
// Does what the reference host's frame loop does (src/quasi/host/main.cpp:265-300) without a
// window: builds a CUDA GPU context, loads the plugin through the C ABI (plugin_loader.hpp),
// calls update + render per frame with the scene camera, reads the image back (ABI v2) and
// the AOVs (ABI v3), and writes them as OpenEXR files (exr_writer.hpp). With --reload it
// then hot-reloads the library (destroy, dlclose, copy, dlopen, create) and renders the
// same frames again; a reloaded plugin must reproduce the image bit for bit.
//
//   quasi_headless [--lib PATH] [--scene SPEC] [--width W] [--height H] [--spp N]
//                  [--depth D] [--frames F] [--device N] [--exr PATH] [--aov-exr PATH] [--reload]
//
// Prints one JSON line; exit status 0 on success, 2 on a load error, 1 otherwise.
#include "cuda_context.hpp"
#include "exr_writer.hpp"
#include "plugin_loader.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct args_t {
    std::string lib = "quasi_gb300/_build/libquasi_cuda.so";
    std::string scene = "cornell36";
    uint32_t width = 256, height = 256, spp = 16, depth = 4, frames = 1;
    int device = 0;
    std::string exr, aov_exr;
    bool reload = false;
};

bool parse(int argc, char** argv, args_t& a) {
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        auto next = [&](const char*& v) {
            if (i + 1 >= argc) return false;
            v = argv[++i];
            return true;
        };
        const char* v = nullptr;
        if (k == "--reload") {
            a.reload = true;
        } else if (!next(v)) {
            return false;
        } else if (k == "--lib") {
            a.lib = v;
        } else if (k == "--scene") {
            a.scene = v;
        } else if (k == "--width") {
            a.width = static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
        } else if (k == "--height") {
            a.height = static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
        } else if (k == "--spp") {
            a.spp = static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
        } else if (k == "--depth") {
            a.depth = static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
        } else if (k == "--frames") {
            a.frames = static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
        } else if (k == "--device") {
            a.device = std::atoi(v);
        } else if (k == "--exr") {
            a.exr = v;
        } else if (k == "--aov-exr") {
            a.aov_exr = v;
        } else {
            return false;
        }
    }
    return a.width > 0 && a.height > 0 && a.frames > 0;
}

std::string json_escape(const std::string& s) {
    std::string o;
    for (char c : s) {
        if (c == '"' || c == '\\') o += '\\';
        if (static_cast<unsigned char>(c) >= 0x20) o += c;
    }
    return o;
}

struct host_state {
    std::vector<std::string> logs;
    bool shutdown = false;
};

void log_cb(void* host_data, const char* msg) { static_cast<host_state*>(host_data)->logs.emplace_back(msg); }
void shutdown_cb(void* host_data) { static_cast<host_state*>(host_data)->shutdown = true; }

struct frame_result {
    uint64_t checksum = 0;  // FNV-1a over the float bits of the RGBA readback
    double mean[3] = {0, 0, 0};
    double ms_per_frame = 0;
    bool ok = false;
};

// Sets the scene and options through the optional extensions (when the plugin has them),
// renders `frames` frames, reads back, optionally writes EXR files.
frame_result run_frames(quasi::host::plugin& p, const args_t& a, cudaStream_t stream, bool write, std::string& err) {
    frame_result r;
    auto make_scene = p.extension<int (*)(const char*, Q_cuda_scene*)>("Q_cuda_make_scene");
    auto free_scene = p.extension<void (*)(Q_cuda_scene*)>("Q_cuda_free_scene");
    auto set_scene = p.extension<int (*)(Q_plugin_handle*, const Q_cuda_scene*)>("Q_cuda_set_scene");
    auto get_options = p.extension<int (*)(Q_plugin_handle*, Q_cuda_options*)>("Q_cuda_get_options");
    auto set_options = p.extension<int (*)(Q_plugin_handle*, const Q_cuda_options*)>("Q_cuda_set_options");
    auto last_error = p.extension<const char* (*)(Q_plugin_handle*)>("Q_cuda_last_error");
    Q_camera cam{{0.5f, 0.5f, -1.4f}, {0.5f, 0.5f, 0.5f}, {0.f, 1.f, 0.f}, 40.f};
    if (make_scene && set_scene && free_scene) {
        Q_cuda_scene sc{};
        if (make_scene(a.scene.c_str(), &sc) != QUASI_OK) {
            err = "unknown scene " + a.scene;
            return r;
        }
        const int rc = set_scene(p.handle, &sc);
        cam = sc.camera;
        free_scene(&sc);
        if (rc != QUASI_OK) {
            err = last_error ? last_error(p.handle) : "Q_cuda_set_scene failed";
            return r;
        }
    }
    if (get_options && set_options) {
        Q_cuda_options o{};
        get_options(p.handle, &o);
        o.spp_per_frame = a.spp;
        o.max_depth = a.depth;
        if (set_options(p.handle, &o) != QUASI_OK) {
            err = last_error ? last_error(p.handle) : "Q_cuda_set_options failed";
            return r;
        }
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t f = 0; f < a.frames; ++f) {
        Q_render_frame fr{};
        fr.drawable = nullptr;
        fr.command_buffer = stream;
        fr.width = a.width;
        fr.height = a.height;
        fr.camera = cam;
        fr.camera_dirty = f == 0 ? 1u : 0u;
        p.update(p.handle, 1.0f / 60.0f);
        p.render(p.handle, &fr);
        if (last_error) {
            const char* e = last_error(p.handle);
            if (e && *e) {
                err = e;
                return r;
            }
        }
    }
    cudaStreamSynchronize(stream);
    const auto t1 = std::chrono::steady_clock::now();
    r.ms_per_frame = std::chrono::duration<double, std::milli>(t1 - t0).count() / a.frames;
    if (!p.readback || !p.readback_free) {
        err = "plugin has no readback (ABI < 2)";
        return r;
    }
    Q_readback_result img = p.readback(p.handle);
    if (!img.data) {
        err = "readback returned no data";
        return r;
    }
    uint64_t h = 1469598103934665603ull;
    const size_t n = static_cast<size_t>(img.width) * img.height * img.channels;
    for (size_t i = 0; i < n; ++i) {
        uint32_t bits;
        std::memcpy(&bits, &img.data[i], 4);
        for (int k = 0; k < 4; ++k) {
            h ^= (bits >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
        if (img.channels >= 3 && i % img.channels < 3) r.mean[i % img.channels] += img.data[i];
    }
    for (double& m : r.mean) m /= static_cast<double>(img.width) * img.height;
    r.checksum = h;
    if (write && !a.exr.empty()) {
        if (auto w = quasi::io::write_exr(a.exr, img); !w) {
            err = quasi::io::to_string(w.error());
            p.readback_free(&img);
            return r;
        }
    }
    p.readback_free(&img);
    if (write && !a.aov_exr.empty()) {
        if (!p.readback_aov || !p.readback_aov_free) {
            err = "plugin has no AOV readback (ABI < 3)";
            return r;
        }
        Q_readback_aov_result aov = p.readback_aov(p.handle);
        auto w = quasi::io::write_exr(a.aov_exr, aov);
        p.readback_aov_free(&aov);
        if (!w) {
            err = quasi::io::to_string(w.error());
            return r;
        }
    }
    r.ok = true;
    return r;
}

}  // namespace

int main(int argc, char** argv) {
    args_t a;
    if (!parse(argc, argv, a)) {
        std::fprintf(stderr, "usage: quasi_headless [--lib PATH] [--scene SPEC] [--width W] [--height H] [--spp N] "
                             "[--depth D] [--frames F] [--device N] [--exr PATH] [--aov-exr PATH] [--reload]\n");
        return 1;
    }
    quasi::host::cuda_context cuda;
    std::string err;
    if (!cuda.init(a.device, err)) {
        std::printf("{\"ok\": false, \"error\": \"cuda: %s\"}\n", json_escape(err).c_str());
        return 1;
    }
    host_state hs;
    Q_plugin_context ctx{};
    ctx.viewport_width = a.width;
    ctx.viewport_height = a.height;
    ctx.host_data = &hs;
    ctx.gpu = cuda.gpu();
    ctx.log = log_cb;
    ctx.request_shutdown = shutdown_cb;

    quasi::host::plugin p;
    quasi::host::load_error le = p.load(a.lib, &ctx, true);
    if (le != quasi::host::load_error::none) {
        std::printf("{\"ok\": false, \"load_error\": \"%s\", \"detail\": \"%s\"}\n", quasi::host::to_string(le),
                    json_escape(p.error()).c_str());
        return 2;
    }
    const Q_plugin_info info = p.get_info();
    frame_result first = run_frames(p, a, cuda.stream(), true, err);
    bool reload_ok = true, identical = true;
    frame_result second;
    if (first.ok && a.reload) {
        p.unload();
        le = p.load(a.lib, &ctx, true);
        reload_ok = le == quasi::host::load_error::none;
        if (reload_ok) {
            second = run_frames(p, a, cuda.stream(), false, err);
            identical = second.ok && second.checksum == first.checksum;
        }
    }
    const bool ok = first.ok && reload_ok && (!a.reload || identical);
    std::printf("{\"ok\": %s, \"abi\": %u, \"name\": \"%s\", \"version\": \"%u.%u.%u\", \"scene\": \"%s\", "
                "\"width\": %u, \"height\": %u, \"spp\": %u, \"frames\": %u, \"ms_per_frame\": %.3f, "
                "\"checksum\": \"%016llx\", \"mean\": [%.9g, %.9g, %.9g]",
                ok ? "true" : "false", p.abi, json_escape(info.name ? info.name : "").c_str(), info.version.major,
                info.version.minor, info.version.patch, json_escape(a.scene).c_str(), a.width, a.height, a.spp,
                a.frames, first.ms_per_frame, static_cast<unsigned long long>(first.checksum), first.mean[0],
                first.mean[1], first.mean[2]);
    if (a.reload)
        std::printf(", \"reload\": {\"loaded\": %s, \"identical\": %s, \"checksum\": \"%016llx\"}",
                    reload_ok ? "true" : "false", identical ? "true" : "false",
                    static_cast<unsigned long long>(second.checksum));
    if (!err.empty()) std::printf(", \"error\": \"%s\"", json_escape(err).c_str());
    std::printf(", \"logs\": %zu}\n", hs.logs.size());
    p.unload();
    return ok ? 0 : 1;
}
