// plugin.cpp - the exported C ABI of libquasi_cuda.so.
//
// Q_plugin_* mirror backends/metal/plugin.mm:541-904 for a CUDA device:
//  * create checks ctx->gpu->backend == Q_GPU_BACKEND_CUDA (plugin.mm:561 checks METAL),
//    logs through ctx->log and returns NULL on failure;
//  * render draws one progressive frame; a camera_dirty frame restarts accumulation
//    (plugin.mm:643-646) and a resize reallocates (plugin.mm:638-640);
//  * readback / readback_aov return malloc'd RGBA float images, top row first, freed by the
//    matching *_free (plugin.mm:797-902).
// The scene and options come from the environment at create time (QUASI_SCENE,
// QUASI_INTEGRATOR, QUASI_SPP, QUASI_DEPTH, QUASI_SEED) or later from Q_cuda_set_*.
#include "../../include/quasi_cuda.h"
#include "batch.hpp"
#include "renderer.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

namespace {

constexpr const char* k_name = "CUDA Path Tracer";
constexpr const char* k_description = "LBVH + wavefront NEE path tracer for NVIDIA GB300 (sm_103a)";
constexpr const char* k_author = "Quasi";

struct PluginState {
    Q_plugin_context* ctx = nullptr;
    quasi::Renderer* renderer = nullptr;
    int device = 0;
    bool reported_error = false;
};

void log_msg(PluginState* st, const std::string& msg) {
    if (st && st->ctx && st->ctx->log) st->ctx->log(st->ctx->host_data, msg.c_str());
}

void log_ctx(Q_plugin_context* ctx, const char* msg) {
    if (ctx && ctx->log) ctx->log(ctx->host_data, msg);
}

uint32_t env_u32(const char* name, uint32_t fallback) {
    const char* v = std::getenv(name);
    if (!v || !*v) return fallback;
    char* end = nullptr;
    const unsigned long x = std::strtoul(v, &end, 10);
    return end != v ? static_cast<uint32_t>(x) : fallback;
}

PluginState* state_of(Q_plugin_handle* h) { return reinterpret_cast<PluginState*>(h); }

Q_aov_buffer alloc_buffer(uint32_t w, uint32_t h) {
    Q_aov_buffer b{};
    const size_t bytes = sizeof(float) * 4ull * w * h;
    b.data = static_cast<float*>(std::malloc(bytes ? bytes : 16));
    if (b.data) {
        b.width = w;
        b.height = h;
        b.channels = 4;
    }
    return b;
}

}  // namespace

extern "C" {

Q_CUDA_EXPORT uint32_t Q_plugin_abi_version(void) { return 3u; }

Q_CUDA_EXPORT Q_plugin_info Q_plugin_get_info(void) {
    Q_plugin_info info;
    info.name = k_name;
    info.version.major = 1;
    info.version.minor = 0;
    info.version.patch = 0;
    info.description = k_description;
    info.author = k_author;
    return info;
}

Q_CUDA_EXPORT Q_plugin_handle* Q_plugin_create(Q_plugin_context* ctx) {
    if (!ctx || !ctx->gpu) return nullptr;
    if (ctx->gpu->backend != Q_GPU_BACKEND_CUDA) {
        log_ctx(ctx, "CUDA backend requires a CUDA GPU context");
        return nullptr;
    }
    auto* st = new (std::nothrow) PluginState{};
    if (!st) return nullptr;
    st->ctx = ctx;
    st->device = ctx->gpu->device ? *static_cast<int*>(ctx->gpu->device) : 0;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || st->device < 0 || st->device >= count) {
        log_ctx(ctx, "CUDA backend: no usable CUDA device");
        delete st;
        return nullptr;
    }
    st->renderer = new (std::nothrow)
        quasi::Renderer(st->device, static_cast<cudaStream_t>(ctx->gpu->queue), false);
    if (!st->renderer || st->renderer->init() != QUASI_OK) {
        log_ctx(ctx, st->renderer ? st->renderer->last_error().c_str() : "out of memory");
        delete st->renderer;
        delete st;
        return nullptr;
    }
    Q_cuda_options opt{};
    opt.spp_per_frame = env_u32("QUASI_SPP", 1);
    opt.max_depth = env_u32("QUASI_DEPTH", 0);
    opt.seed = env_u32("QUASI_SEED", 0);
    const char* integ = std::getenv("QUASI_INTEGRATOR");
    opt.integrator = (integ && std::strcmp(integ, "reference") == 0) ? QUASI_INTEGRATOR_REFERENCE
                                                                      : QUASI_INTEGRATOR_NEE;
    opt.rebuild_each_frame = env_u32("QUASI_REBUILD", 1);
    if (opt.max_depth == 0) opt.max_depth = opt.integrator == QUASI_INTEGRATOR_REFERENCE ? 5 : 4;
    const char* spec = std::getenv("QUASI_SCENE");
    Q_cuda_scene scene{};
    int rc = Q_cuda_make_scene(spec && *spec ? spec : "refcornell", &scene);
    if (rc == QUASI_OK) rc = st->renderer->set_options(opt);
    if (rc == QUASI_OK) rc = st->renderer->set_scene(scene);
    Q_cuda_free_scene(&scene);
    if (rc != QUASI_OK) {
        log_ctx(ctx, ("CUDA backend: scene setup failed: " + st->renderer->last_error()).c_str());
        delete st->renderer;
        delete st;
        return nullptr;
    }
    log_msg(st, "CUDA path tracer initialized");
    return reinterpret_cast<Q_plugin_handle*>(st);
}

Q_CUDA_EXPORT void Q_plugin_destroy(Q_plugin_handle* handle) {
    if (!handle) return;
    PluginState* st = state_of(handle);
    log_msg(st, "CUDA path tracer destroyed");
    delete st->renderer;  // synchronises its stream and frees every device allocation
    delete st;
}

Q_CUDA_EXPORT void Q_plugin_update(Q_plugin_handle* handle, float delta_time) {
    (void)handle;
    (void)delta_time;
}

Q_CUDA_EXPORT void Q_plugin_render(Q_plugin_handle* handle, Q_render_frame* frame) {
    if (!handle || !frame) return;
    PluginState* st = state_of(handle);
    const int rc = st->renderer->render(*frame);
    if (rc != QUASI_OK && !st->reported_error) {
        log_msg(st, "CUDA render failed: " + st->renderer->last_error());
        st->reported_error = true;
    }
}

Q_CUDA_EXPORT Q_readback_result Q_plugin_readback(Q_plugin_handle* handle) {
    Q_readback_result r{};
    if (!handle) return r;
    PluginState* st = state_of(handle);
    const uint32_t w = st->renderer->width(), h = st->renderer->height();
    if (w == 0 || h == 0) return r;
    Q_aov_buffer b = alloc_buffer(w, h);
    if (!b.data) return r;
    if (st->renderer->resolve_host(b.data, nullptr, nullptr, nullptr) != QUASI_OK) {
        std::free(b.data);
        log_msg(st, "HDR readback failed: " + st->renderer->last_error());
        return r;
    }
    r.data = b.data;
    r.width = w;
    r.height = h;
    r.channels = 4;
    log_msg(st, "HDR readback complete");
    return r;
}

Q_CUDA_EXPORT void Q_plugin_readback_free(Q_readback_result* result) {
    if (result && result->data) {
        std::free(result->data);
        result->data = nullptr;
    }
}

Q_CUDA_EXPORT Q_readback_aov_result Q_plugin_readback_aov(Q_plugin_handle* handle) {
    Q_readback_aov_result r{};
    if (!handle) return r;
    PluginState* st = state_of(handle);
    const uint32_t w = st->renderer->width(), h = st->renderer->height();
    if (w == 0 || h == 0) return r;
    for (uint32_t i = 0; i < Q_AOV_COUNT; ++i) r.buffers[i] = alloc_buffer(w, h);
    const bool ok = r.buffers[0].data && r.buffers[1].data && r.buffers[2].data && r.buffers[3].data &&
                    st->renderer->resolve_host(r.buffers[0].data, r.buffers[1].data, r.buffers[2].data,
                                               r.buffers[3].data) == QUASI_OK;
    if (!ok) {
        Q_plugin_readback_aov_free(&r);
        log_msg(st, "AOV readback failed: " + st->renderer->last_error());
        return Q_readback_aov_result{};
    }
    log_msg(st, "AOV readback complete");
    return r;
}

Q_CUDA_EXPORT void Q_plugin_readback_aov_free(Q_readback_aov_result* result) {
    if (!result) return;
    for (uint32_t i = 0; i < Q_AOV_COUNT; ++i) {
        if (result->buffers[i].data) {
            std::free(result->buffers[i].data);
            result->buffers[i].data = nullptr;
        }
    }
}

#define Q_STATE_OR_FAIL(h)                             \
    if (!(h)) return QUASI_ERR_INVALID;                \
    quasi::Renderer* r = state_of(h)->renderer

Q_CUDA_EXPORT int Q_cuda_set_scene(Q_plugin_handle* handle, const Q_cuda_scene* scene) {
    Q_STATE_OR_FAIL(handle);
    if (!scene) return QUASI_ERR_INVALID;
    return r->set_scene(*scene);
}

Q_CUDA_EXPORT int Q_cuda_update_vertices(Q_plugin_handle* handle, const float* vertices, uint32_t tri_count) {
    Q_STATE_OR_FAIL(handle);
    return r->update_vertices(vertices, tri_count);
}

Q_CUDA_EXPORT int Q_cuda_set_materials(Q_plugin_handle* handle, const float* albedo, const float* emission,
                                       uint32_t tri_count) {
    Q_STATE_OR_FAIL(handle);
    return r->set_materials(albedo, emission, tri_count);
}

Q_CUDA_EXPORT int Q_cuda_set_options(Q_plugin_handle* handle, const Q_cuda_options* options) {
    Q_STATE_OR_FAIL(handle);
    if (!options) return QUASI_ERR_INVALID;
    return r->set_options(*options);
}

Q_CUDA_EXPORT int Q_cuda_get_options(Q_plugin_handle* handle, Q_cuda_options* options) {
    Q_STATE_OR_FAIL(handle);
    if (!options) return QUASI_ERR_INVALID;
    *options = r->options();
    return QUASI_OK;
}

Q_CUDA_EXPORT int Q_cuda_reset(Q_plugin_handle* handle) {
    Q_STATE_OR_FAIL(handle);
    return r->reset();
}

Q_CUDA_EXPORT int Q_cuda_synchronize(Q_plugin_handle* handle) {
    Q_STATE_OR_FAIL(handle);
    return r->synchronize();
}

Q_CUDA_EXPORT int Q_cuda_get_stats(Q_plugin_handle* handle, Q_cuda_stats* stats) {
    Q_STATE_OR_FAIL(handle);
    if (!stats) return QUASI_ERR_INVALID;
    return r->stats(stats);
}

Q_CUDA_EXPORT int Q_cuda_kernel_times(Q_plugin_handle* handle, Q_cuda_kernel_time* out, uint32_t capacity,
                                      uint32_t* count) {
    Q_STATE_OR_FAIL(handle);
    return r->kernel_times(out, capacity, count);
}

Q_CUDA_EXPORT const char* Q_cuda_last_error(Q_plugin_handle* handle) {
    if (!handle) return "null handle";
    return state_of(handle)->renderer->last_error().c_str();
}

Q_CUDA_EXPORT int Q_cuda_read_bvh(Q_plugin_handle* handle, uint32_t* morton, uint32_t* order, int32_t* children,
                                  float* boxes, float* bounds) {
    Q_STATE_OR_FAIL(handle);
    return r->read_bvh(morton, order, children, boxes, bounds);
}

Q_CUDA_EXPORT int Q_cuda_read_wide_bvh(Q_plugin_handle* handle, uint32_t* words) {
    Q_STATE_OR_FAIL(handle);
    if (!words) return QUASI_ERR_INVALID;
    return r->read_wide_bvh(words);
}

Q_CUDA_EXPORT int Q_cuda_read_samples(Q_plugin_handle* handle, float* radiance, uint32_t* signatures) {
    Q_STATE_OR_FAIL(handle);
    return r->read_samples(radiance, signatures);
}

Q_CUDA_EXPORT int Q_cuda_resolve_device(Q_plugin_handle* handle, float* device_rgba) {
    Q_STATE_OR_FAIL(handle);
    if (!device_rgba) return QUASI_ERR_INVALID;
    return r->resolve_device(device_rgba);
}

Q_CUDA_EXPORT int Q_cuda_set_materials_device(Q_plugin_handle* handle, const float* device_albedo,
                                              const float* device_emission, uint32_t tri_count) {
    Q_STATE_OR_FAIL(handle);
    return r->set_materials_device(device_albedo, device_emission, tri_count);
}

Q_CUDA_EXPORT int Q_cuda_backward(Q_plugin_handle* handle, const float* device_grad_image, uint32_t spp,
                                  uint32_t sample_base, float* device_grad_albedo, float* device_grad_emission,
                                  void* stream) {
    Q_STATE_OR_FAIL(handle);
    return r->backward(device_grad_image, spp, sample_base, device_grad_albedo, device_grad_emission,
                       static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_autotune(Q_plugin_handle* handle, double budget_ms) {
    Q_STATE_OR_FAIL(handle);
    return r->autotune(budget_ms);
}

// ------------------------------------------------------------------ scene batches

Q_CUDA_EXPORT int Q_cuda_batch_create(Q_plugin_handle* handle, const Q_cuda_batch_scene* scenes, uint32_t count,
                                      const Q_cuda_batch_options* options, Q_cuda_batch** out) {
    Q_STATE_OR_FAIL(handle);
    if (!out) return QUASI_ERR_INVALID;
    *out = nullptr;
    quasi::BatchRenderer* b = new (std::nothrow) quasi::BatchRenderer(*r);
    if (!b) return QUASI_ERR_OOM;
    const int rc = b->create(scenes, count, options);
    if (rc) {
        r->fail(rc, "batch: " + b->last_error());
        delete b;
        return rc;
    }
    *out = reinterpret_cast<Q_cuda_batch*>(b);
    return QUASI_OK;
}

#define Q_BATCH_OR_FAIL(batch)              \
    if (!(batch)) return QUASI_ERR_INVALID; \
    quasi::BatchRenderer* b = reinterpret_cast<quasi::BatchRenderer*>(batch)

Q_CUDA_EXPORT void Q_cuda_batch_destroy(Q_cuda_batch* batch) { delete reinterpret_cast<quasi::BatchRenderer*>(batch); }

Q_CUDA_EXPORT int Q_cuda_batch_set_options(Q_cuda_batch* batch, const Q_cuda_batch_options* options) {
    Q_BATCH_OR_FAIL(batch);
    if (!options) return QUASI_ERR_INVALID;
    return b->set_options(*options);
}

Q_CUDA_EXPORT int Q_cuda_batch_get_options(Q_cuda_batch* batch, Q_cuda_batch_options* options) {
    Q_BATCH_OR_FAIL(batch);
    if (!options) return QUASI_ERR_INVALID;
    *options = b->options();
    return QUASI_OK;
}

Q_CUDA_EXPORT int Q_cuda_batch_render(Q_cuda_batch* batch, void* stream) {
    Q_BATCH_OR_FAIL(batch);
    return b->render(static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_batch_reset(Q_cuda_batch* batch) {
    Q_BATCH_OR_FAIL(batch);
    return b->reset();
}

Q_CUDA_EXPORT int Q_cuda_batch_set_seed(Q_cuda_batch* batch, uint32_t seed, void* stream) {
    Q_BATCH_OR_FAIL(batch);
    return b->set_seed(seed, static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_batch_synchronize(Q_cuda_batch* batch) {
    Q_BATCH_OR_FAIL(batch);
    return b->synchronize();
}

Q_CUDA_EXPORT int Q_cuda_batch_get_stats(Q_cuda_batch* batch, Q_cuda_batch_stats* stats) {
    Q_BATCH_OR_FAIL(batch);
    return b->stats(stats);
}

Q_CUDA_EXPORT int Q_cuda_batch_readback(Q_cuda_batch* batch, uint32_t index, float* host_rgba) {
    Q_BATCH_OR_FAIL(batch);
    return b->readback(index, host_rgba);
}

Q_CUDA_EXPORT int Q_cuda_batch_resolve_device(Q_cuda_batch* batch, float* device_rgb, void* stream) {
    Q_BATCH_OR_FAIL(batch);
    return b->resolve_device(device_rgb, static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_batch_offsets(Q_cuda_batch* batch, uint32_t index, uint64_t* tri_offset,
                                       uint64_t* px_offset) {
    Q_BATCH_OR_FAIL(batch);
    return b->offsets(index, tri_offset, px_offset);
}

Q_CUDA_EXPORT int Q_cuda_batch_set_materials_device(Q_cuda_batch* batch, const float* device_albedo,
                                                    const float* device_emission, void* stream) {
    Q_BATCH_OR_FAIL(batch);
    return b->set_materials_device(device_albedo, device_emission, static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_batch_backward(Q_cuda_batch* batch, const float* device_grad_image,
                                        float* device_grad_albedo, float* device_grad_emission, void* stream) {
    Q_BATCH_OR_FAIL(batch);
    return b->backward(device_grad_image, device_grad_albedo, device_grad_emission,
                       static_cast<cudaStream_t>(stream));
}

Q_CUDA_EXPORT int Q_cuda_batch_autotune(Q_cuda_batch* batch, double budget_ms, Q_cuda_batch_options* chosen) {
    Q_BATCH_OR_FAIL(batch);
    return b->autotune(budget_ms, chosen);
}

Q_CUDA_EXPORT const char* Q_cuda_batch_last_error(Q_cuda_batch* batch) {
    if (!batch) return "null batch";
    return reinterpret_cast<quasi::BatchRenderer*>(batch)->last_error().c_str();
}

}  // extern "C"
