// wavefront.cu - host side of the NEE path tracer: the Renderer (scene upload, per-frame
// LBVH, the wavefront launch sequence, accumulation, readback, statistics). The device
// kernels are in wavefront_kernels.cuh.
#include "renderer.hpp"
#include "wavefront_kernels.cuh"
#include "megakernel.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

namespace quasi {

// ---------------------------------------------------------------------------- host

namespace {

inline uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace

CameraFF make_camera_basis(const Q_camera& c, uint32_t w, uint32_t h) {
    // plugin.mm:649-674 (host direction) and plugin.mm:134-147 (shader basis), in double.
    double dir[3] = {double(c.target[0]) - c.position[0], double(c.target[1]) - c.position[1],
                     double(c.target[2]) - c.position[2]};
    double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (len > 0) for (double& v : dir) v /= len;
    double wv[3] = {-dir[0], -dir[1], -dir[2]};
    len = std::sqrt(wv[0] * wv[0] + wv[1] * wv[1] + wv[2] * wv[2]);
    if (len > 0) for (double& v : wv) v /= len;
    const double up[3] = {c.up[0], c.up[1], c.up[2]};
    double r[3] = {up[1] * wv[2] - up[2] * wv[1], up[2] * wv[0] - up[0] * wv[2], up[0] * wv[1] - up[1] * wv[0]};
    len = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (len > 0) for (double& v : r) v /= len;
    const double u2[3] = {wv[1] * r[2] - wv[2] * r[1], wv[2] * r[0] - wv[0] * r[2], wv[0] * r[1] - wv[1] * r[0]};
    const double theta = double(c.fov) * 3.14159265358979323846 / 180.0;
    const double vh = 2.0 * std::tan(theta / 2.0);
    const double vw = (double(w) / double(h)) * vh;
    CameraFF b;
    b.origin = make_float3(c.position[0], c.position[1], c.position[2]);
    // ll + u h + v vv - o with u = px / w, v = 1 - py / h is
    // (ll + vv - o) + (h / w) px - (vv / h) py
    double base[3], sx[3], sy[3];
    for (int k = 0; k < 3; ++k) {
        const double H = vw * r[k], V = vh * u2[k];
        const double LL = double(c.position[k]) - H * 0.5 - V * 0.5 - wv[k];
        base[k] = LL + V - double(c.position[k]);
        sx[k] = H / double(w);
        sy[k] = V / double(h);
    }
    // Each double splits into hi = nearest float and lo = nearest float of the remainder.
    auto split = [](const double* d, float3& hi, float3& lo) {
        hi = make_float3(float(d[0]), float(d[1]), float(d[2]));
        lo = make_float3(float(d[0] - double(hi.x)), float(d[1] - double(hi.y)), float(d[2] - double(hi.z)));
    };
    split(base, b.base_hi, b.base_lo);
    split(sx, b.sx_hi, b.sx_lo);
    split(sy, b.sy_hi, b.sy_lo);
    return b;
}

// Reference-integrator entry point (refmode.cu).
cudaError_t launch_reference_frame(const float4* quads, uint32_t n_quads, const Q_camera& cam, uint32_t width,
                                   uint32_t height, uint32_t sample_base, uint32_t spp, float4* accum, float4* comp,
                                   float4* aov_a, float4* aov_n, cudaStream_t s, KernelProfiler& prof);

Renderer::Renderer(int device, cudaStream_t stream, bool own_stream)
    : device_(device), stream_(stream), own_stream_(own_stream) {
    opt_.spp_per_frame = 1;
    opt_.max_depth = 4;
    opt_.rebuild_each_frame = 1;
    opt_.ray_eps = 1e-4f;
}

Renderer::~Renderer() {
    if (stream_) cudaStreamSynchronize(stream_);
    bvh_.release();
    for (DeviceBuffer* b : {&raw_vertices_, &tri_in_, &albedo_, &emission_, &emitters_, &quads_, &accum_, &comp_,
                            &aov_albedo_, &aov_normal_, &record_rad_, &record_sig_, &resolve_, &queue_[0], &queue_[1],
                            &hits_,
                            &shadow_, &beta_, &lpath_, &aov_a_, &aov_n_, &sig_, &ray_ff_, &defer_,
                            &counters_, &stats_dev_, &err_dev_})
        b->release();
    if (counters_host_) cudaFreeHost(counters_host_);
    if (stats_host_) cudaFreeHost(stats_host_);
    if (err_host_) cudaFreeHost(err_host_);
    for (cudaEvent_t e : {ev_frame0_, ev_frame1_, ev_bvh0_, ev_bvh1_})
        if (e) cudaEventDestroy(e);
    if (owned_stream_) {
        cudaStreamSynchronize(owned_stream_);
        cudaStreamDestroy(owned_stream_);
    }
}

int Renderer::cuda_fail(cudaError_t e, const char* where) {
    error_ = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QUASI_ERR_OOM : QUASI_ERR_CUDA;
}

#define R_TRY(expr, where)                                  \
    do {                                                    \
        cudaError_t r_err_ = (expr);                        \
        if (r_err_ != cudaSuccess) return cuda_fail(r_err_, where); \
    } while (0)

int Renderer::init() {
    R_TRY(cudaSetDevice(device_), "cudaSetDevice");
    R_TRY(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, device_), "sm count");
    if (!stream_) {
        R_TRY(cudaStreamCreateWithFlags(&owned_stream_, cudaStreamNonBlocking), "stream");
        stream_ = owned_stream_;
    }
    R_TRY(cudaEventCreate(&ev_frame0_), "event");
    R_TRY(cudaEventCreate(&ev_frame1_), "event");
    R_TRY(cudaEventCreate(&ev_bvh0_), "event");
    R_TRY(cudaEventCreate(&ev_bvh1_), "event");
    R_TRY(stats_dev_.reserve(sizeof(unsigned long long) * 8), "stats");
    R_TRY(err_dev_.reserve(sizeof(uint32_t)), "err");
    R_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, stats_dev_.bytes, stream_), "memset");
    R_TRY(cudaMemsetAsync(err_dev_.ptr, 0, err_dev_.bytes, stream_), "memset");
    R_TRY(cudaMallocHost(&stats_host_, sizeof(unsigned long long) * 8), "pinned");
    R_TRY(cudaMallocHost(&err_host_, sizeof(uint32_t)), "pinned");
    std::memset(stats_host_, 0, sizeof(unsigned long long) * 8);
    *err_host_ = 0;
    return QUASI_OK;
}

int Renderer::upload_materials_host(const float* albedo, const float* emission, uint32_t n) {
    std::vector<float4> a(n), e(n);
    std::vector<int> emit;
    for (uint32_t i = 0; i < n; ++i) {
        a[i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.f);
        e[i] = make_float4(emission[3 * i], emission[3 * i + 1], emission[3 * i + 2], 0.f);
        if (e[i].x > 0.f || e[i].y > 0.f || e[i].z > 0.f) emit.push_back(static_cast<int>(i));
    }
    R_TRY(albedo_.reserve(sizeof(float4) * n), "albedo");
    R_TRY(emission_.reserve(sizeof(float4) * n), "emission");
    R_TRY(emitters_.reserve(sizeof(int) * std::max<size_t>(emit.size(), 1)), "emitters");
    if (n) {
        R_TRY(cudaMemcpyAsync(albedo_.ptr, a.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream_), "h2d");
        R_TRY(cudaMemcpyAsync(emission_.ptr, e.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, stream_), "h2d");
    }
    if (!emit.empty())
        R_TRY(cudaMemcpyAsync(emitters_.ptr, emit.data(), sizeof(int) * emit.size(), cudaMemcpyHostToDevice, stream_),
              "h2d");
    n_emit_ = static_cast<uint32_t>(emit.size());
    // The staging vectors die at return: wait for the copies.
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    return QUASI_OK;
}

int Renderer::set_scene(const Q_cuda_scene& sc) {
    if (sc.tri_count > 0 && (!sc.vertices || !sc.albedo || !sc.emission))
        return fail(QUASI_ERR_INVALID, "scene arrays missing");
    if (sc.quad_count > 0 && (!sc.quads || !sc.quad_albedo || !sc.quad_emission))
        return fail(QUASI_ERR_INVALID, "quad arrays missing");
    if (sc.tri_count > (1u << 28)) return fail(QUASI_ERR_INVALID, "too many triangles");
    n_tris_ = sc.tri_count;
    R_TRY(raw_vertices_.reserve(sizeof(float) * 9ull * n_tris_), "vertices");
    R_TRY(tri_in_.reserve(sizeof(float4) * 3ull * n_tris_), "tri_in");
    int rc = update_vertices(sc.vertices, sc.tri_count);
    if (rc) return rc;
    rc = upload_materials_host(sc.albedo, sc.emission, n_tris_);
    if (rc) return rc;
    n_quads_ = sc.quad_count;
    if (n_quads_) {
        std::vector<float4> q(5ull * n_quads_);
        for (uint32_t i = 0; i < n_quads_; ++i) {
            const float* g = sc.quads + 9ull * i;
            q[5 * i + 0] = make_float4(g[0], g[1], g[2], 0.f);
            q[5 * i + 1] = make_float4(g[3], g[4], g[5], 0.f);
            q[5 * i + 2] = make_float4(g[6], g[7], g[8], 0.f);
            q[5 * i + 3] = make_float4(sc.quad_albedo[3 * i], sc.quad_albedo[3 * i + 1], sc.quad_albedo[3 * i + 2], 0.f);
            q[5 * i + 4] = make_float4(sc.quad_emission[3 * i], sc.quad_emission[3 * i + 1], sc.quad_emission[3 * i + 2], 0.f);
        }
        R_TRY(quads_.reserve(sizeof(float4) * q.size()), "quads");
        R_TRY(cudaMemcpy(quads_.ptr, q.data(), sizeof(float4) * q.size(), cudaMemcpyHostToDevice), "h2d");
    }
    scene_camera_ = sc.camera;
    has_scene_ = true;
    bvh_dirty_ = true;
    return reset();
}

int Renderer::update_vertices(const float* vertices, uint32_t tri_count) {
    if (tri_count != n_tris_) return fail(QUASI_ERR_INVALID, "vertex count differs from the scene");
    if (tri_count == 0) return QUASI_OK;
    if (!vertices) return fail(QUASI_ERR_INVALID, "null vertices");
    R_TRY(cudaMemcpyAsync(raw_vertices_.ptr, vertices, sizeof(float) * 9ull * tri_count, cudaMemcpyHostToDevice, stream_),
          "h2d vertices");
    R_TRY(QUASI_LAUNCH(prof_, "pack_tris", stream_,
                       (k_pack_tris<<<ceil_div(tri_count, 256), 256, 0, stream_>>>(raw_vertices_.as<float>(), tri_count,
                                                                                 tri_in_.as<float4>()))),
          "pack_tris");
    bvh_dirty_ = true;
    return QUASI_OK;
}

int Renderer::set_materials(const float* albedo, const float* emission, uint32_t tri_count) {
    if (tri_count != n_tris_) return fail(QUASI_ERR_INVALID, "material count differs from the scene");
    if (tri_count && (!albedo || !emission)) return fail(QUASI_ERR_INVALID, "null materials");
    int rc = upload_materials_host(albedo, emission, tri_count);
    if (rc) return rc;
    bvh_dirty_ = true;  // the emitters' light-sampling records are rebuilt with the hierarchy
    return reset();
}

int Renderer::set_options(const Q_cuda_options& o) {
    Q_cuda_options n = o;
    if (n.spp_per_frame == 0) n.spp_per_frame = 1;
    if (n.max_depth == 0) n.max_depth = 4;
    if (n.max_depth > 64) return fail(QUASI_ERR_INVALID, "max_depth above 64");
    if (n.integrator > QUASI_INTEGRATOR_REFERENCE) return fail(QUASI_ERR_INVALID, "unknown integrator");
    if (!(n.ray_eps > 0.f)) n.ray_eps = 1e-4f;
    if (n.trace_block != 0 && (n.trace_block % 32 != 0 || n.trace_block > 256))
        return fail(QUASI_ERR_INVALID, "trace_block must be a multiple of 32 up to 256");
    if (n.refill_lanes > 32) return fail(QUASI_ERR_INVALID, "refill_lanes must be at most 32");
    if (n.smem_levels > 9 && n.smem_levels != 32)
        return fail(QUASI_ERR_INVALID, "smem_levels must be 0 (default), 1..9, or 32 (none)");
    if (n.bvh_width != 0 && n.bvh_width != 2 && n.bvh_width != 8)
        return fail(QUASI_ERR_INVALID, "bvh_width must be 0 (default), 2 or 8");
    if (n.bvh_cluster > 32) return fail(QUASI_ERR_INVALID, "bvh_cluster must be at most 32");
    if (n.bvh_cluster == 0) n.bvh_cluster = 32;
    if (n.bvh_collapse > 1) return fail(QUASI_ERR_INVALID, "bvh_collapse must be 0 or 1");
    if (n.bvh_split > 100 && n.bvh_split != QUASI_BVH_SPLIT_NONE)
        return fail(QUASI_ERR_INVALID, "bvh_split must be 0 (default), 1..100 or QUASI_BVH_SPLIT_NONE");
    if (n.bvh_split == 0) n.bvh_split = QUASI_BVH_SPLIT_PERCENT == 0 ? QUASI_BVH_SPLIT_NONE : QUASI_BVH_SPLIT_PERCENT;
    if (n.bvh_split != opt_.bvh_split) {
        bvh_.set_split_percent(n.bvh_split == QUASI_BVH_SPLIT_NONE ? 0 : static_cast<int>(n.bvh_split));
        bvh_dirty_ = true;
    }
    if (n.bvh_collapse != opt_.bvh_collapse) {
        bvh_.set_dp_collapse(n.bvh_collapse == 0);
        bvh_dirty_ = true;
    }
    const bool changed = n.seed != opt_.seed || n.max_depth != opt_.max_depth || n.integrator != opt_.integrator ||
                         n.ray_eps != opt_.ray_eps;
    if (n.bvh_cluster != opt_.bvh_cluster) {
        bvh_.set_sah_cluster(static_cast<int>(n.bvh_cluster));
        bvh_dirty_ = true;
    }
    opt_ = n;
    prof_.set_enabled(opt_.profile != 0);
    if (changed) return reset();
    return QUASI_OK;
}

int Renderer::reset() {
    samples_ = 0;
    frame_index_ = 0;
    if (accum_.ptr) {
        R_TRY(cudaMemsetAsync(accum_.ptr, 0, accum_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(comp_.ptr, 0, comp_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(aov_albedo_.ptr, 0, aov_albedo_.bytes, stream_), "memset");
        R_TRY(cudaMemsetAsync(aov_normal_.ptr, 0, aov_normal_.bytes, stream_), "memset");
    }
    return QUASI_OK;
}

int Renderer::ensure_frame_buffers(uint32_t w, uint32_t h) {
    if (w == width_ && h == height_ && accum_.ptr) return QUASI_OK;
    const size_t px = static_cast<size_t>(w) * h;
    accum_.release(); comp_.release(); aov_albedo_.release(); aov_normal_.release();
    R_TRY(accum_.reserve(sizeof(float4) * px), "accum");
    R_TRY(comp_.reserve(sizeof(float4) * px), "accum");
    R_TRY(aov_albedo_.reserve(sizeof(float4) * px), "accum");
    R_TRY(aov_normal_.reserve(sizeof(float4) * px), "accum");
    width_ = w;
    height_ = h;
    return reset();
}

// Bytes of wave state per path slot: two ray queues (2 x 32), hit 16, shadow ray 64 (with the
// lo parts of its exact origin), beta, radiance and two AOVs (4 x 16), signature 4,
// double-float ray 48, fixup list entry 8.
constexpr size_t k_wave_bytes_per_path = 268;

int Renderer::ensure_wave_buffers(uint32_t paths) {
    if (paths <= wave_capacity_) return QUASI_OK;
    R_TRY(queue_[0].reserve(sizeof(float4) * 2ull * paths), "queue");
    R_TRY(queue_[1].reserve(sizeof(float4) * 2ull * paths), "queue");
    R_TRY(hits_.reserve(sizeof(float4) * paths), "hits");
    R_TRY(shadow_.reserve(sizeof(float4) * 4ull * paths), "shadow");
    R_TRY(beta_.reserve(sizeof(float4) * paths), "beta");
    R_TRY(lpath_.reserve(sizeof(float4) * paths), "lpath");
    R_TRY(aov_a_.reserve(sizeof(float4) * paths), "aov");
    R_TRY(aov_n_.reserve(sizeof(float4) * paths), "aov");
    R_TRY(sig_.reserve(sizeof(uint32_t) * paths), "sig");
    R_TRY(ray_ff_.reserve(sizeof(float4) * 3ull * paths), "ray_ff");
    R_TRY(defer_.reserve(sizeof(int2) * paths), "defer");
    wave_capacity_ = paths;
    return QUASI_OK;
}

uint32_t Renderer::effective_wave_spp(uint32_t spp) const {
    if (opt_.wave_spp > 0) return std::min(opt_.wave_spp, spp);
    const uint32_t tiles = ceil_div(width_, 8) * ceil_div(height_, 4);
    const uint32_t slots = tiles * 32;
    // up to 2^27 paths per wave (~36 GB of wave state, all 64 samples of a 1080p frame): the
    // later bounces of a wave shrink as paths end, larger waves keep those queues long enough
    // to fill the GPU, and every wave pays each kernel's fixed drain once (1080p, 64 spp on
    // the 1M soup, GB300: 16 spp per wave 1403.5, 32 spp 1441.8, 64 spp 1462.9 Mrays/s; the
    // fixup kernels, whose time is mostly a fixed tail per launch, halve with the waves)
    const uint64_t target = wave_paths_fitting(1u << 27, k_wave_bytes_per_path,
                                               size_t(wave_capacity_) * k_wave_bytes_per_path);
    return std::max<uint32_t>(1, static_cast<uint32_t>(std::min<uint64_t>(spp, target / std::max<uint32_t>(slots, 1))));
}

int Renderer::render(const Q_render_frame& fr) {
    NvtxRange frame_range("quasi.frame");
    error_.clear();
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (fr.width == 0 || fr.height == 0) return fail(QUASI_ERR_INVALID, "zero-sized frame");
    if (static_cast<uint64_t>(fr.width) * fr.height > (1ull << 26)) return fail(QUASI_ERR_INVALID, "frame too large");
    if (fr.command_buffer) stream_ = static_cast<cudaStream_t>(fr.command_buffer);
    cudaStream_t s = stream_;
    int rc = ensure_frame_buffers(fr.width, fr.height);
    if (rc) return rc;
    if (fr.camera_dirty) {
        rc = reset();
        if (rc) return rc;
    }
    camera_ = fr.camera;
    prof_.reset_launches();
    R_TRY(cudaEventRecord(ev_frame0_, s), "event");
    bvh_timed_ = false;
    if (opt_.integrator == QUASI_INTEGRATOR_NEE && (bvh_dirty_ || opt_.rebuild_each_frame)) {
        NvtxRange bvh_range("quasi.lbvh");
        R_TRY(cudaEventRecord(ev_bvh0_, s), "event");
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, emitters_.as<int>(), n_emit_, s, prof_,
                         err_dev_.as<uint32_t>()),
              "lbvh build");
        const int levels = opt_.smem_levels ? static_cast<int>(opt_.smem_levels) : k_default_smem_levels;
        R_TRY(bvh_.build_treelet(levels >= 31 ? 0 : (1 << levels) - 1, s, prof_), "treelet");
        R_TRY(cudaEventRecord(ev_bvh1_, s), "event");
        bvh_timed_ = true;
        bvh_dirty_ = false;
    }
    const uint32_t spp = opt_.spp_per_frame;
    if (opt_.record_samples) {
        const size_t n = static_cast<size_t>(width_) * height_ * spp;
        R_TRY(record_rad_.reserve(sizeof(float) * 3 * n), "record");
        R_TRY(record_sig_.reserve(sizeof(uint32_t) * n), "record");
        record_spp_ = spp;
    }
    if (opt_.integrator == QUASI_INTEGRATOR_REFERENCE) rc = render_reference(s, spp);
    else if (opt_.megakernel) rc = render_megakernel(s, spp);
    else rc = render_wavefront(s, spp);
    if (rc) return rc;
    samples_ += spp;
    total_samples_ += spp;
    ++frame_index_;
    R_TRY(cudaEventRecord(ev_frame1_, s), "event");
    frame_timed_ = true;
    if (fr.drawable) {
        const uint32_t px = width_ * height_;
        R_TRY(QUASI_LAUNCH(prof_, "tonemap", s,
                           (k_tonemap<<<ceil_div(px, 256), 256, 0, s>>>(accum_.as<float4>(), px, float(samples_),
                                                                       static_cast<uchar4*>(fr.drawable)))),
              "tonemap");
    }
    return QUASI_OK;
}

int Renderer::render_wavefront(cudaStream_t s, uint32_t spp) {
    const uint32_t D = opt_.max_depth;
    const uint32_t tiles_x = ceil_div(width_, 8), tiles_y = ceil_div(height_, 4);
    const uint32_t slots = tiles_x * tiles_y * 32;
    const uint32_t S = effective_wave_spp(spp);
    const uint32_t waves = ceil_div(spp, S);
    int rc = ensure_wave_buffers(slots * S);
    if (rc) return rc;
    const uint32_t per_wave = k_counters_per_bounce * D;
    const uint32_t need = per_wave * waves;
    if (need > counter_capacity_) {
        R_TRY(counters_.reserve(sizeof(int) * need), "counters");
        if (counters_host_) cudaFreeHost(counters_host_);
        R_TRY(cudaMallocHost(&counters_host_, sizeof(int) * need), "pinned");
        counter_capacity_ = need;
    }
    counters_used_ = need;
    R_TRY(cudaMemsetAsync(counters_.ptr, 0, sizeof(int) * need, s), "memset");
    if (opt_.collect_stats) R_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, sizeof(unsigned long long) * 4, s), "memset");

    const LbvhView bv = bvh_.view();
    const bool wide = opt_.bvh_width != 2;
    SceneDev sd{tri_in_.as<float4>(), albedo_.as<float4>(), emission_.as<float4>(),
                bv.nodes,
                bv.tris,
                n_tris_,
                n_emit_,
                opt_.refill_lanes ? static_cast<int>(opt_.refill_lanes) : (wide ? k_wide_refill_lanes : k_refill_lanes),
                opt_.trace_steps ? static_cast<int>(opt_.trace_steps) : k_trace_steps,
                wide ? nullptr : bv.tree,
                wide ? 0 : bv.tree_n,
                wide ? bv.wide : nullptr,
                bv.tri_plane,
                bv.emit_tab};
    const size_t tree_smem = sizeof(float4) * 4 * static_cast<size_t>(sd.tree_n);
    PathDev pd{beta_.as<float4>(),  lpath_.as<float4>(), aov_a_.as<float4>(),
               aov_n_.as<float4>(), ray_ff_.as<float4>(), opt_.record_samples ? sig_.as<uint32_t>() : nullptr};
    FrameParams f{};
    f.cam = make_camera_basis(camera_, width_, height_);
    f.width = width_;
    f.height = height_;
    f.tiles_x = tiles_x;
    f.slots = slots;
    f.seed = opt_.seed;
    f.max_depth = D;
    f.eps = opt_.ray_eps;
    f.frame_spp = spp;

    // default block: 256 threads over the 8-wide records (with the shared-memory stacks,
    // 0.3% faster than 128 on the 1M soup), 128 over the binary LBVH
    const int tb = opt_.trace_block ? static_cast<int>(opt_.trace_block) : (wide ? 256 : 128);
    using ClosestFn = void (*)(SceneDev, ClosestJob, const int*, int, int*, uint32_t*, unsigned long long*);
    using ShadowFn = void (*)(SceneDev, ShadowJob, const int*, int, int*, uint32_t*, unsigned long long*);
    const int mode = wide ? (sd.refill < 32 ? k_mode_wide_refill : k_mode_wide)
                          : sd.refill < 32 ? k_mode_refill : (sd.tree_n > 0 ? k_mode_batch_tree : k_mode_batch);
    static const ClosestFn closest_fns[2][5] = {
        {k_trace_closest<false, k_mode_batch>, k_trace_closest<false, k_mode_batch_tree>,
         k_trace_closest<false, k_mode_refill>, k_trace_closest<false, k_mode_wide>,
         k_trace_closest<false, k_mode_wide_refill>},
        {k_trace_closest<true, k_mode_batch>, k_trace_closest<true, k_mode_batch_tree>,
         k_trace_closest<true, k_mode_refill>, k_trace_closest<true, k_mode_wide>,
         k_trace_closest<true, k_mode_wide_refill>}};
    static const ShadowFn shadow_fns[2][5] = {
        {k_trace_shadow<false, k_mode_batch>, k_trace_shadow<false, k_mode_batch_tree>,
         k_trace_shadow<false, k_mode_refill>, k_trace_shadow<false, k_mode_wide>,
         k_trace_shadow<false, k_mode_wide_refill>},
        {k_trace_shadow<true, k_mode_batch>, k_trace_shadow<true, k_mode_batch_tree>,
         k_trace_shadow<true, k_mode_refill>, k_trace_shadow<true, k_mode_wide>,
         k_trace_shadow<true, k_mode_wide_refill>}};
    const ClosestFn kc = closest_fns[opt_.collect_stats ? 1 : 0][mode];
    const ShadowFn ks = shadow_fns[opt_.collect_stats ? 1 : 0][mode];
    // dynamic shared memory: the staged treelet (binary forms) or the stacks' shared part
    // (8-wide refill)
    const bool shared_stacks = mode == k_mode_wide_refill;
    const size_t smem_c = shared_stacks ? wide_stack_smem_bytes<false>(tb) : tree_smem;
    const size_t smem_s = shared_stacks ? wide_stack_smem_bytes<true>(tb) : tree_smem;
    const int grid_c = sm_count_ * resident_blocks(kc, tb, smem_c);
    const int grid_s = sm_count_ * resident_blocks(ks, tb, smem_s);
// Blocks per SM of the shading launch (grid-stride over the hits, 3 resident per SM): 3, 8,
// 16, 32 and 64 gave 34.8, 33.6, 32.8, 32.3 and 32.4 ms per 1080p frame.
#ifndef QUASI_SHADE_GRID_PER_SM
#define QUASI_SHADE_GRID_PER_SM 32
#endif
    const int grid_shade = sm_count_ * QUASI_SHADE_GRID_PER_SM;
    // The fixup kernels are latency-bound (dependent loads, then double-float arithmetic):
    // as many blocks as fit.
    const int grid_fixup = sm_count_ * resident_blocks(k_fixup<ClosestJob>, 128, 0);
    uint32_t* err = err_dev_.as<uint32_t>();
    unsigned long long* st = stats_dev_.as<unsigned long long>();
    const uint32_t px = width_ * height_;
    const int cap = static_cast<int>(slots * S);

    for (uint32_t w = 0; w < waves; ++w) {
        NvtxRange wave_range("quasi.wave");
        const uint32_t Sw = std::min(S, spp - w * S);
        f.wave_spp = Sw;
        f.sample_base = samples_ + w * S;
        f.wave_offset = w * S;
        int* cnt = counters_.as<int>() + w * per_wave;
        R_TRY(QUASI_LAUNCH(prof_, "camera", s,
                           (k_camera<<<ceil_div(Sw * slots, 256), 256, 0, s>>>(f, sd, pd, queue_[0].as<float4>(), cnt))),
              "camera");
        for (uint32_t k = 1; k <= D; ++k) {
            float4* qcur = queue_[(k - 1) & 1].as<float4>();
            float4* qnext = queue_[k & 1].as<float4>();
            int* c_cur = cnt + (k - 1);
            int* c_next = cnt + k;  // unused when k == D (index D is the first shadow counter, never appended)
            int* c_shadow = cnt + D + (k - 1);
            int* f_cur = cnt + 2 * D + (k - 1);
            int* f_shadow = cnt + 3 * D + (k - 1);
            const ClosestJob cjob{qcur, hits_.as<float4>(), ray_ff_.as<float4>(), lpath_.as<float4>(),
                                  DeferList{defer_.as<int2>(), cnt + 4 * D + (k - 1), cnt + 8 * D + (k - 1), cap},
                                  nullptr};
            const ShadowJob sjob{shadow_.as<float4>(), pd,
                                 DeferList{defer_.as<int2>(), cnt + 5 * D + (k - 1), cnt + 9 * D + (k - 1), cap}};
            R_TRY(QUASI_LAUNCH(prof_, "trace_closest", s,
                               (kc<<<grid_c, tb, smem_c, s>>>(sd, cjob, c_cur, cap, f_cur, err, st))),
                  "trace_closest");
            R_TRY(QUASI_LAUNCH(prof_, "fixup_closest", s,
                               (k_fixup<ClosestJob><<<grid_fixup, 128, 0, s>>>(sd, cjob, cnt + 6 * D + (k - 1), err))),
                  "fixup_closest");
            R_TRY(QUASI_LAUNCH(prof_, "shade", s,
                               (k_shade<<<grid_shade, 256, 0, s>>>(f, sd, pd, k, hits_.as<float4>(), c_cur, cap, qnext,
                                                                  k < D ? c_next : nullptr, shadow_.as<float4>(),
                                                                  c_shadow))),
                  "shade");
            R_TRY(QUASI_LAUNCH(prof_, "trace_shadow", s,
                               (ks<<<grid_s, tb, smem_s, s>>>(sd, sjob, c_shadow, cap, f_shadow, err, st))),
                  "trace_shadow");
            R_TRY(QUASI_LAUNCH(prof_, "fixup_shadow", s,
                               (k_fixup<ShadowJob><<<grid_fixup, 128, 0, s>>>(sd, sjob, cnt + 7 * D + (k - 1), err))),
                  "fixup_shadow");
        }
        R_TRY(QUASI_LAUNCH(prof_, "accumulate", s,
                           (k_accumulate<<<ceil_div(px, 256), 256, 0, s>>>(
                               f, pd, accum_.as<float4>(), comp_.as<float4>(), aov_albedo_.as<float4>(),
                               aov_normal_.as<float4>(), opt_.record_samples ? record_rad_.as<float>() : nullptr,
                               opt_.record_samples ? record_sig_.as<uint32_t>() : nullptr))),
              "accumulate");
    }
    R_TRY(QUASI_LAUNCH(prof_, "tally", s, (k_tally<<<1, 32, 0, s>>>(counters_.as<int>(), waves, D, st))), "tally");
    R_TRY(cudaMemcpyAsync(counters_host_, counters_.ptr, sizeof(int) * need, cudaMemcpyDeviceToHost, s), "d2h");
    R_TRY(cudaMemcpyAsync(stats_host_, stats_dev_.ptr, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost, s), "d2h");
    R_TRY(cudaMemcpyAsync(err_host_, err_dev_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "d2h");
    last_frame_megakernel_ = false;
    stats_pending_ = true;
    return QUASI_OK;
}

SceneDev Renderer_scene_dev(const LbvhView& bv, const DeviceBuffer& tri_in, const DeviceBuffer& albedo,
                            const DeviceBuffer& emission, uint32_t n_tris, uint32_t n_emit, uint32_t bvh_width) {
    return SceneDev{tri_in.as<float4>(), albedo.as<float4>(), emission.as<float4>(), bv.nodes, bv.tris, n_tris, n_emit,
                    k_refill_lanes, k_trace_steps, nullptr, 0, bvh_width == 2 ? nullptr : bv.wide, bv.tri_plane,
                    bv.emit_tab};
}

FrameParams Renderer::frame_params(uint32_t spp, uint32_t slots, uint32_t tiles_x) const {
    FrameParams f{};
    f.cam = make_camera_basis(camera_, width_, height_);
    f.width = width_;
    f.height = height_;
    f.tiles_x = tiles_x;
    f.slots = slots;
    f.seed = opt_.seed;
    f.max_depth = opt_.max_depth;
    f.eps = opt_.ray_eps;
    f.frame_spp = spp;
    return f;
}

// One-thread-per-path renderer: same waves, path ids and accumulation as the wavefront, so
// its per-sample radiance (and therefore the image) is bit-identical.
int Renderer::render_megakernel(cudaStream_t s, uint32_t spp) {
    const uint32_t tiles_x = ceil_div(width_, 8), tiles_y = ceil_div(height_, 4);
    const uint32_t slots = tiles_x * tiles_y * 32;
    const uint32_t S = effective_wave_spp(spp);
    const uint32_t waves = ceil_div(spp, S);
    int rc = ensure_wave_buffers(slots * S);
    if (rc) return rc;
    if (counter_capacity_ < waves + 2) {
        R_TRY(counters_.reserve(sizeof(int) * (waves + 2)), "counters");
        if (counters_host_) cudaFreeHost(counters_host_);
        R_TRY(cudaMallocHost(&counters_host_, sizeof(int) * (waves + 2)), "pinned");
        counter_capacity_ = waves + 2;
    }
    counters_used_ = 0;
    R_TRY(cudaMemsetAsync(counters_.ptr, 0, sizeof(int) * (waves + 2), s), "memset");
    R_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, sizeof(unsigned long long) * 4, s), "memset");
    R_TRY(cudaMemsetAsync(stats_dev_.as<unsigned long long>() + 5, 0, sizeof(unsigned long long) * 2, s), "memset");
    const SceneDev sd = Renderer_scene_dev(bvh_.view(), tri_in_, albedo_, emission_, n_tris_, n_emit_,
                                           opt_.bvh_width);
    PathDev pd{beta_.as<float4>(),  lpath_.as<float4>(), aov_a_.as<float4>(),
               aov_n_.as<float4>(), ray_ff_.as<float4>(), opt_.record_samples ? sig_.as<uint32_t>() : nullptr};
    FrameParams f = frame_params(spp, slots, tiles_x);
    auto kern = opt_.collect_stats ? k_megakernel<true> : k_megakernel<false>;
    const int grid = sm_count_ * resident_blocks(kern, 128, 0);
    unsigned long long* st = stats_dev_.as<unsigned long long>();
    const uint32_t px = width_ * height_;
    for (uint32_t w = 0; w < waves; ++w) {
        f.wave_spp = std::min(S, spp - w * S);
        f.sample_base = samples_ + w * S;
        f.wave_offset = w * S;
        R_TRY(QUASI_LAUNCH(prof_, "megakernel", s,
                           (kern<<<grid, 128, 0, s>>>(f, sd, pd, counters_.as<int>() + w, err_dev_.as<uint32_t>(), st))),
              "megakernel");
        R_TRY(QUASI_LAUNCH(prof_, "accumulate", s,
                           (k_accumulate<<<ceil_div(px, 256), 256, 0, s>>>(
                               f, pd, accum_.as<float4>(), comp_.as<float4>(), aov_albedo_.as<float4>(),
                               aov_normal_.as<float4>(), opt_.record_samples ? record_rad_.as<float>() : nullptr,
                               opt_.record_samples ? record_sig_.as<uint32_t>() : nullptr))),
              "accumulate");
    }
    R_TRY(cudaMemcpyAsync(stats_host_, stats_dev_.ptr, sizeof(unsigned long long) * 7, cudaMemcpyDeviceToHost, s), "d2h");
    R_TRY(cudaMemcpyAsync(err_host_, err_dev_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s), "d2h");
    mk_paths_ = static_cast<uint64_t>(px) * spp;
    last_frame_megakernel_ = true;
    stats_pending_ = true;
    return QUASI_OK;
}

int Renderer::set_materials_device(const float* albedo, const float* emission, uint32_t tri_count) {
    if (tri_count != n_tris_) return fail(QUASI_ERR_INVALID, "material count differs from the scene");
    if (tri_count == 0) return QUASI_OK;
    R_TRY(QUASI_LAUNCH(prof_, "pack_materials", stream_,
                       (k_pack_materials<<<ceil_div(tri_count, 256), 256, 0, stream_>>>(
                           albedo, emission, tri_count, albedo_.as<float4>(), emission_.as<float4>()))),
          "pack_materials");
    return reset();
}

int Renderer::backward(const float* grad_image, uint32_t spp, uint32_t sample_base, float* grad_albedo,
                       float* grad_emission, cudaStream_t stream) {
    if (stream) stream_ = stream;
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (opt_.integrator != QUASI_INTEGRATOR_NEE) return fail(QUASI_ERR_STATE, "backward needs the NEE integrator");
    if (!grad_image || !grad_albedo || !grad_emission || spp == 0) return fail(QUASI_ERR_INVALID, "backward arguments");
    if (opt_.max_depth > static_cast<uint32_t>(k_adjoint_max_depth))
        return fail(QUASI_ERR_INVALID, "backward supports max_depth up to 16");
    if (width_ == 0 || height_ == 0) return fail(QUASI_ERR_STATE, "render a frame before backward");
    cudaStream_t s = stream_;
    if (bvh_dirty_) {
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, emitters_.as<int>(), n_emit_, s, prof_,
                         err_dev_.as<uint32_t>()),
              "lbvh build");
        bvh_dirty_ = false;
    }
    R_TRY(cudaMemsetAsync(grad_albedo, 0, sizeof(float) * 3ull * n_tris_, s), "memset");
    R_TRY(cudaMemsetAsync(grad_emission, 0, sizeof(float) * 3ull * n_tris_, s), "memset");
    if (counter_capacity_ < 1) {
        R_TRY(counters_.reserve(sizeof(int) * 4), "counters");
        if (counters_host_) cudaFreeHost(counters_host_);
        R_TRY(cudaMallocHost(&counters_host_, sizeof(int) * 4), "pinned");
        counter_capacity_ = 4;
    }
    R_TRY(cudaMemsetAsync(counters_.ptr, 0, sizeof(int), s), "memset");
    const uint32_t tiles_x = ceil_div(width_, 8), tiles_y = ceil_div(height_, 4);
    const uint32_t slots = tiles_x * tiles_y * 32;
    FrameParams f = frame_params(spp, slots, tiles_x);
    f.wave_spp = spp;
    f.sample_base = sample_base;
    f.wave_offset = 0;
    const SceneDev sd = Renderer_scene_dev(bvh_.view(), tri_in_, albedo_, emission_, n_tris_, n_emit_,
                                           opt_.bvh_width);
    const int grid = sm_count_ * resident_blocks(k_adjoint, 128, 0);
    R_TRY(QUASI_LAUNCH(prof_, "adjoint", s,
                       (k_adjoint<<<grid, 128, 0, s>>>(f, sd, grad_image, 1.0f / static_cast<float>(spp), grad_albedo,
                                                      grad_emission, counters_.as<int>(), err_dev_.as<uint32_t>(),
                                                      stats_dev_.as<unsigned long long>()))),
          "adjoint");
    return QUASI_OK;
}

int Renderer::render_reference(cudaStream_t s, uint32_t spp) {
    if (n_quads_ == 0) return fail(QUASI_ERR_STATE, "reference integrator needs quads");
    R_TRY(launch_reference_frame(quads_.as<float4>(), n_quads_, camera_, width_, height_, samples_, spp,
                                 accum_.as<float4>(), comp_.as<float4>(), aov_albedo_.as<float4>(),
                                 aov_normal_.as<float4>(), s, prof_),
          "reference frame");
    counters_used_ = 0;
    stats_pending_ = false;
    return QUASI_OK;
}

int Renderer::synchronize() {
    R_TRY(cudaStreamSynchronize(stream_), "synchronize");
    return QUASI_OK;
}

int Renderer::resolve_device(float* device_rgba) {
    if (!accum_.ptr) return fail(QUASI_ERR_STATE, "nothing rendered");
    const uint32_t px = width_ * height_;
    R_TRY(QUASI_LAUNCH(prof_, "resolve", stream_,
                       (k_resolve<<<ceil_div(px, 256), 256, 0, stream_>>>(accum_.as<float4>(), aov_albedo_.as<float4>(),
                                                                         aov_normal_.as<float4>(), px, float(samples_), 0,
                                                                         reinterpret_cast<float4*>(device_rgba)))),
          "resolve");
    return QUASI_OK;
}

int Renderer::resolve_host(float* beauty, float* albedo, float* normal, float* depth) {
    if (!accum_.ptr) return fail(QUASI_ERR_STATE, "nothing rendered");
    const uint32_t px = width_ * height_;
    // kept between readbacks: a cudaFree per call would synchronise the device
    R_TRY(resolve_.reserve(sizeof(float4) * px), "resolve buffer");
    float* outs[4] = {beauty, albedo, normal, depth};
    for (int mode = 0; mode < 4; ++mode) {
        if (!outs[mode]) continue;
        cudaError_t e = QUASI_LAUNCH(prof_, "resolve", stream_,
                                     (k_resolve<<<ceil_div(px, 256), 256, 0, stream_>>>(
                                         accum_.as<float4>(), aov_albedo_.as<float4>(), aov_normal_.as<float4>(), px,
                                         float(samples_), mode, resolve_.as<float4>())));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(outs[mode], resolve_.ptr, sizeof(float4) * px, cudaMemcpyDeviceToHost, stream_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
        if (e != cudaSuccess) return cuda_fail(e, "resolve");
    }
    return QUASI_OK;
}

int Renderer::read_samples(float* radiance, uint32_t* signatures) {
    if (!opt_.record_samples || !record_rad_.ptr) return fail(QUASI_ERR_STATE, "record_samples was off");
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    const size_t n = static_cast<size_t>(width_) * height_ * record_spp_;
    if (radiance) R_TRY(cudaMemcpy(radiance, record_rad_.ptr, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost), "d2h");
    if (signatures) R_TRY(cudaMemcpy(signatures, record_sig_.ptr, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost), "d2h");
    return QUASI_OK;
}

int Renderer::read_bvh(uint32_t* morton, uint32_t* order, int32_t* children, float* boxes, float* bounds) {
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (bvh_dirty_) {
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, emitters_.as<int>(), n_emit_, stream_, prof_,
                         err_dev_.as<uint32_t>()),
              "lbvh build");
        bvh_dirty_ = false;
    }
    if (bvh_.split_active()) return fail(QUASI_ERR_STATE, "the hierarchy has split references (bvh_split)");
    R_TRY(bvh_.read(morton, order, children, boxes, bounds, stream_), "read bvh");
    return QUASI_OK;
}

int Renderer::read_wide_bvh(uint32_t* words) {
    if (!has_scene_) return fail(QUASI_ERR_STATE, "no scene");
    if (bvh_dirty_) {
        R_TRY(bvh_.build(tri_in_.as<float4>(), n_tris_, emitters_.as<int>(), n_emit_, stream_, prof_,
                         err_dev_.as<uint32_t>()),
              "lbvh build");
        bvh_dirty_ = false;
    }
    if (bvh_.split_active()) return fail(QUASI_ERR_STATE, "the hierarchy has split references (bvh_split)");
    R_TRY(bvh_.read_wide(words, stream_), "read wide bvh");
    return QUASI_OK;
}

int Renderer::stats(Q_cuda_stats* out) {
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    Q_cuda_stats st{};
    if (stats_pending_ && last_frame_megakernel_) {
        st.camera_rays = mk_paths_;
        st.extension_rays = stats_host_[5] - mk_paths_;
        st.shadow_rays = stats_host_[6];
        if (opt_.collect_stats) {
            st.node_visits = stats_host_[0];
            st.tri_tests = stats_host_[1];
        }
        last_stats_ = st;
    } else if (stats_pending_) {
        const uint32_t D = opt_.max_depth;
        const uint32_t per_wave = k_counters_per_bounce * D;
        const uint32_t waves = per_wave ? counters_used_ / per_wave : 0;
        for (uint32_t w = 0; w < waves; ++w) {
            const int* c = counters_host_ + w * per_wave;
            st.camera_rays += static_cast<uint64_t>(c[0]);
            for (uint32_t k = 1; k < D; ++k) st.extension_rays += static_cast<uint64_t>(c[k]);
            for (uint32_t k = 0; k < D; ++k) st.shadow_rays += static_cast<uint64_t>(c[D + k]);
            for (uint32_t k = 0; k < 2 * D; ++k)
                st.redecided_rays += static_cast<uint64_t>(c[4 * D + k]) + static_cast<uint64_t>(c[8 * D + k]);
        }
        if (opt_.collect_stats) {
            st.node_visits = stats_host_[0];
            st.tri_tests = stats_host_[1];
            st.shadow_node_visits = stats_host_[2];
            st.shadow_tri_tests = stats_host_[3];
        }
        last_stats_ = st;
    } else {
        st = last_stats_;
    }
    st.total_rays = stats_host_[4];
    unsigned long long adj = 0;
    R_TRY(cudaMemcpy(&adj, stats_dev_.as<unsigned long long>() + 7, sizeof(adj), cudaMemcpyDeviceToHost), "d2h");
    st.adjoint_rays = adj;
    st.samples_accumulated = samples_;
    st.kernel_launches = prof_.launches();
    st.error_flags = err_host_ ? *err_host_ : 0u;
    float ms = 0.f;
    if (frame_timed_ && cudaEventElapsedTime(&ms, ev_frame0_, ev_frame1_) == cudaSuccess) st.frame_ms = ms;
    if (bvh_timed_ && cudaEventElapsedTime(&ms, ev_bvh0_, ev_bvh1_) == cudaSuccess) st.bvh_ms = ms;
    prof_.collect();
    *out = st;
    return QUASI_OK;
}

int Renderer::kernel_times(Q_cuda_kernel_time* out, uint32_t capacity, uint32_t* count) {
    R_TRY(cudaStreamSynchronize(stream_), "sync");
    prof_.collect();
    const auto& t = prof_.totals();
    uint32_t i = 0;
    for (const auto& kv : t) {
        if (out && i < capacity) {
            std::memset(out[i].name, 0, sizeof(out[i].name));
            std::strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
            out[i].launches = kv.second.first;
            out[i].total_ms = kv.second.second;
        }
        ++i;
    }
    if (count) *count = i;
    if (!out && !count) prof_.reset_totals();  // (NULL, 0, NULL) clears the totals
    return QUASI_OK;
}

// Coordinate search over the renderer form, wave size, trace block size and the refill
// threshold (8-wide records) or treelet depth (binary LBVH), timing short progressive frames
// (at most 8 spp, LBVH kept) with the frame events.
int Renderer::autotune(double budget_ms) {
    if (!has_scene_ || width_ == 0 || height_ == 0) return fail(QUASI_ERR_STATE, "render a frame before autotune");
    if (opt_.integrator != QUASI_INTEGRATOR_NEE) return fail(QUASI_ERR_STATE, "autotune needs the NEE integrator");
    if (budget_ms <= 0.0) budget_ms = 2000.0;
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&]() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    const Q_cuda_options saved = opt_;
    Q_cuda_options base = opt_;
    base.spp_per_frame = std::min<uint32_t>(saved.spp_per_frame, 8);
    base.rebuild_each_frame = 0;
    base.record_samples = 0;
    base.collect_stats = 0;
    base.profile = 0;
    const uint32_t slots = ceil_div(width_, 8) * ceil_div(height_, 4) * 32;
    if (base.wave_spp == 0) base.wave_spp = effective_wave_spp(base.spp_per_frame);
    Q_render_frame fr{};
    fr.width = width_;
    fr.height = height_;
    fr.camera = camera_;
    auto measure = [&](const Q_cuda_options& o, float& ms) -> int {
        if (o.smem_levels != opt_.smem_levels) bvh_dirty_ = true;  // rebuild the treelet (untimed frame)
        opt_ = o;
        prof_.set_enabled(false);
        for (int rep = 0; rep < 2; ++rep) {
            const int rc = render(fr);
            if (rc) return rc;
        }
        R_TRY(cudaEventSynchronize(ev_frame1_), "sync");
        R_TRY(cudaEventElapsedTime(&ms, ev_frame0_, ev_frame1_), "event time");
        return QUASI_OK;
    };
    // the last dimension: refill threshold for the 8-wide records, treelet depth for the binary
    const bool wide = base.bvh_width != 2;
    Q_cuda_options best = base;
    float best_ms = 0.f;
    int rc = measure(best, best_ms);
    if (rc) {
        opt_ = saved;
        return rc;
    }
    for (int dim = 0; dim < 4 && elapsed() < budget_ms; ++dim) {
        std::vector<uint32_t> vals;
        if (dim == 0) vals = {0u, 1u};
        if (dim == 1)
            for (uint32_t target : {8u << 20, 16u << 20, 32u << 20, 64u << 20})
                vals.push_back(std::max<uint32_t>(1, std::min<uint32_t>(base.spp_per_frame, target / slots)));
        if (dim == 2) vals = {64u, 128u, 256u};
        if (dim == 3) vals = wide ? std::vector<uint32_t>{2u, 4u, 8u} : std::vector<uint32_t>{0u, 7u, 32u};
        for (uint32_t v : vals) {
            if (elapsed() >= budget_ms) break;
            Q_cuda_options o = best;
            uint32_t& field = dim == 0   ? o.megakernel
                              : dim == 1 ? o.wave_spp
                              : dim == 2 ? o.trace_block
                              : wide     ? o.refill_lanes
                                         : o.smem_levels;
            if (field == v || (dim == 2 && field == 0 && v == (wide ? 256u : 128u))) continue;
            if (dim == 3 && wide && field == 0 && v == static_cast<uint32_t>(k_wide_refill_lanes)) continue;
            if (dim == 2 && o.megakernel) continue;  // the megakernel runs 128-thread blocks
            if (dim == 3 && o.megakernel) continue;
            field = v;
            float ms = 0.f;
            rc = measure(o, ms);
            if (rc) {
                opt_ = saved;
                return rc;
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = o;
            }
        }
    }
    opt_ = saved;
    opt_.megakernel = best.megakernel;
    opt_.wave_spp = best.wave_spp;
    opt_.trace_block = best.trace_block;
    opt_.smem_levels = best.smem_levels;
    opt_.refill_lanes = best.refill_lanes;
    prof_.set_enabled(opt_.profile != 0);
    bvh_dirty_ = true;  // the treelet depth may have changed
    return reset();
}

}  // namespace quasi
