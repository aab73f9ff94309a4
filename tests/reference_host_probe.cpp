// reference_host_probe.cpp - drives libquasi_cuda.so through the reference host's own plugin
// code, unchanged: Q::plugin::loader (src/quasi/plugin/loader.hpp) and the hot-reloading
// Q::plugin::manager (src/quasi/plugin/manager.hpp) on the reference's cooperative
// Q::async::scheduler. Built by tests/test_gpu_reference_host.py against those headers.
//
//   probe loader <plugin.so> <frames> <width> <height> <out.bin>
//       loader::load with a CUDA context on a host-created stream, `frames` renders
//       (the first camera_dirty), then readback and readback_aov (and their *_free);
//       writes the beauty then the albedo, normal and depth AOVs as raw RGBA float.
//   probe manager <plugin.so> <frames> <width> <height> <out.bin>
//       manager::load_sync, `frames` renders into a device RGBA8 drawable, touch of the
//       library file, scheduler ticks until the manager's watch loop has reloaded it (the
//       pre_unload hook synchronises the stream), `frames` renders again; writes both
//       tonemapped images and prints the manager's reload statistics.
// The plugin's scene and options come from QUASI_SCENE / QUASI_SPP / QUASI_DEPTH /
// QUASI_SEED (read by Q_plugin_create). Exit status 0 on success.
#include <quasi/async/scheduler.hpp>
#include <quasi/plugin/loader.hpp>
#include <quasi/plugin/manager.hpp>

#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <string>
#include <thread>
#include <vector>

namespace {

void log_fn(void*, const char* m) { std::printf("log: %s\n", m); }

bool write_all(const char* path, const std::vector<std::vector<unsigned char>>& parts) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    bool ok = true;
    for (const auto& p : parts) ok = ok && std::fwrite(p.data(), 1, p.size(), f) == p.size();
    return std::fclose(f) == 0 && ok;
}

std::vector<unsigned char> bytes_of(const float* data, size_t count) {
    std::vector<unsigned char> out(sizeof(float) * count);
    if (data && count) std::memcpy(out.data(), data, out.size());
    return out;
}

// The camera of the built-in 36-triangle Cornell box (and the soups): looking at the box
// from -z; the same values the Python host takes from the scene.
Q::gpu::camera_data scene_camera() {
    Q::gpu::camera_data c{};
    const char* spec = std::getenv("QUASI_SCENE");
    const bool cornell = spec && std::strcmp(spec, "cornell36") == 0;
    const float pos[3] = {0.5f, 0.5f, cornell ? -1.4f : -1.0f}, tgt[3] = {0.5f, 0.5f, 0.5f}, up[3] = {0.f, 1.f, 0.f};
    std::memcpy(c.position, pos, sizeof(pos));
    std::memcpy(c.target, tgt, sizeof(tgt));
    std::memcpy(c.up, up, sizeof(up));
    c.fov = 40.f;
    return c;
}

int run_loader(const char* lib_path, int frames, uint32_t w, uint32_t h, const char* out) {
    auto lib = Q::plugin::dynamic_library::open(lib_path);
    if (!lib) {
        std::printf("open_failed\n");
        return 1;
    }
    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return 1;
    int ordinal = 0;
    Q::gpu::gpu_context gpu{};
    gpu.backend = static_cast<Q::gpu::gpu_backend>(4);  // Q_GPU_BACKEND_CUDA
    gpu.device = &ordinal;
    gpu.queue = stream;
    Q::plugin::plugin_context ctx{};
    ctx.viewport_width = w;
    ctx.viewport_height = h;
    ctx.gpu = &gpu;
    ctx.log = log_fn;
    auto p = Q::plugin::loader::load(*lib, &ctx);
    if (!p) {
        std::printf("load_failed: %s\n", Q::plugin::to_string(p.error()));
        return 2;
    }
    std::printf("loaded abi=%u readback=%d aov=%d\n", p->abi_version(), int(p->supports_readback()),
                int(p->supports_readback_aov()));
    for (int i = 0; i < frames; ++i) {
        Q::gpu::render_frame f{};
        f.command_buffer = stream;
        f.width = w;
        f.height = h;
        f.camera = scene_camera();
        f.camera_dirty = i == 0 ? 1u : 0u;
        p->render(&f);
    }
    cudaStreamSynchronize(stream);
    auto rb = p->readback();
    auto aov = p->readback_aov();
    std::vector<std::vector<unsigned char>> parts;
    parts.push_back(bytes_of(rb.data, size_t(rb.width) * rb.height * rb.channels));
    for (int k = 1; k < 4; ++k) {
        const auto& b = aov.buffers[k];
        parts.push_back(bytes_of(b.data, size_t(b.width) * b.height * b.channels));
    }
    const bool shape_ok = rb.width == w && rb.height == h && rb.channels == 4;
    p->readback_free(&rb);
    p->readback_aov_free(&aov);
    p->destroy();
    cudaStreamDestroy(stream);
    if (!shape_ok || !write_all(out, parts)) return 3;
    std::printf("ok\n");
    return 0;
}

int run_manager(const char* lib_path, int frames, uint32_t w, uint32_t h, const char* out) {
    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return 1;
    unsigned char* drawable = nullptr;
    if (cudaMalloc(&drawable, size_t(w) * h * 4) != cudaSuccess) return 1;
    std::vector<unsigned char> before, after;
    int rc = 0;
    {
        // The manager (and the plugin it holds) is destroyed at the end of this scope, before
        // the stream and the drawable it renders with.
        int pre_unload_calls = 0;
        Q::plugin::reload_hooks hooks;
        hooks.pre_unload = [&]() -> Q::async::task<void> {
            // the plugin's work on the host's stream must finish before its library goes away
            cudaStreamSynchronize(stream);
            ++pre_unload_calls;
            co_return;
        };
        hooks.on_error = [](const std::string& m) { std::printf("reload error: %s\n", m.c_str()); };
        int ordinal = 0;
        Q::gpu::gpu_context gpu{};
        gpu.backend = static_cast<Q::gpu::gpu_backend>(4);
        gpu.device = &ordinal;
        gpu.queue = stream;
        Q::plugin::manager mgr{lib_path, hooks};
        mgr.set_viewport(w, h);
        mgr.set_gpu_context(&gpu);
        mgr.set_log_callback(log_fn);
        if (!mgr.load_sync()) {
            std::printf("load_sync failed\n");
            return 2;
        }
        auto render_frames = [&](std::vector<unsigned char>& img) {
            for (int i = 0; i < frames; ++i) {
                Q::gpu::render_frame f{};
                f.drawable = drawable;
                f.command_buffer = stream;
                f.width = w;
                f.height = h;
                f.camera = scene_camera();
                f.camera_dirty = i == 0 ? 1u : 0u;
                mgr.render(&f);
            }
            img.resize(size_t(w) * h * 4);
            cudaStreamSynchronize(stream);
            return cudaMemcpy(img.data(), drawable, img.size(), cudaMemcpyDeviceToHost) == cudaSuccess;
        };
        if (!render_frames(before)) return 3;
        std::fflush(stdout);
        Q::async::scheduler sched;
        sched.spawn(mgr.watch_and_reload_loop());
        sched.tick();  // the loop starts polling
        // a rebuilt library: a newer modification time on the watched file
        std::filesystem::last_write_time(lib_path, std::filesystem::file_time_type::clock::now() +
                                                       std::chrono::seconds(2));
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::seconds(30);
        while (mgr.stats().success_count + mgr.stats().failure_count == 0 &&
               std::chrono::steady_clock::now() < deadline) {
            sched.tick();
            std::this_thread::sleep_for(std::chrono::milliseconds(5));
        }
        const auto st = mgr.stats();
        std::printf("reloads=%llu success=%llu failure=%llu pre_unload=%d loaded=%d\n",
                    static_cast<unsigned long long>(st.reload_count),
                    static_cast<unsigned long long>(st.success_count),
                    static_cast<unsigned long long>(st.failure_count), pre_unload_calls, int(mgr.is_loaded()));
        std::fflush(stdout);
        if (st.success_count != 1 || !mgr.is_loaded()) rc = 4;
        else if (!render_frames(after)) rc = 3;
    }
    cudaFree(drawable);
    cudaStreamDestroy(stream);
    if (rc) return rc;
    if (!write_all(out, {before, after})) return 3;
    std::printf("ok\n");
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: %s loader|manager <plugin.so> <frames> <width> <height> <out.bin>\n", argv[0]);
        return 64;
    }
    const int frames = std::atoi(argv[3]);
    const uint32_t w = static_cast<uint32_t>(std::atoi(argv[4])), h = static_cast<uint32_t>(std::atoi(argv[5]));
    if (std::strcmp(argv[1], "loader") == 0) return run_loader(argv[2], frames, w, h, argv[6]);
    if (std::strcmp(argv[1], "manager") == 0) return run_manager(argv[2], frames, w, h, argv[6]);
    return 64;
}
