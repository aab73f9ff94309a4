// batch.cu - host side of the multi-scene batch renderer (Q_cuda_batch_*).
//
// create() uploads every scene into shared pools (triangles, materials, emitters, images)
// and builds one LBVH per scene. plan() cuts each scene's frame into items of whole sample
// planes and packs them into waves of at most wave_paths path slots; the item table is
// uploaded to the device, where it is the work queue every kernel of the frame reads. The
// frame's launch sequence (all waves of all scenes) is captured once into a CUDA graph and
// replayed by render(); the adjoint sequence likewise. autotune() times frames of
// candidate launch configurations (the batch's own, or capped at fewer samples per pixel
// when those would not fit its budget) and keeps the fastest.
#include "batch.hpp"
#include "batch_kernels.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace quasi {

CameraFF make_camera_basis(const Q_camera& c, uint32_t w, uint32_t h);  // wavefront.cu

namespace {

inline uint32_t ceil_div(uint32_t a, uint32_t b) { return (a + b - 1) / b; }
constexpr uint32_t k_default_wave_paths = 1u << 27;  // as the single-scene renderer's waves
constexpr uint32_t k_max_wave_paths = 1u << 27;

}  // namespace

#define B_TRY(expr, where)                                          \
    do {                                                            \
        cudaError_t b_err_ = (expr);                                \
        if (b_err_ != cudaSuccess) return cuda_fail(b_err_, where); \
    } while (0)

BatchRenderer::BatchRenderer(Renderer& owner) : owner_(owner), stream_(owner.stream()) {}

BatchRenderer::~BatchRenderer() {
    cudaStreamSynchronize(stream_);
    if (capture_) cudaStreamSynchronize(capture_);
    drop_graphs();
    for (auto& b : bvh_) b->release();
    for (DeviceBuffer* b : {&tri_in_, &albedo_, &emission_, &emitters_, &accum_, &comp_, &aov_a_, &aov_n_, &table_,
                            &items_, &queue_[0], &queue_[1], &hits_, &shadow_, &beta_, &lpath_, &pa_, &pn_, &ray_ff_, &defer_,
                            &meta_, &counters_, &adj_counters_, &stats_dev_, &err_dev_, &grad_image_, &grad_albedo_,
                            &grad_emission_})
        b->release();
    if (stats_host_) cudaFreeHost(stats_host_);
    if (err_host_) cudaFreeHost(err_host_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (capture_) cudaStreamDestroy(capture_);
}

int BatchRenderer::cuda_fail(cudaError_t e, const char* where) {
    error_ = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? QUASI_ERR_OOM : QUASI_ERR_CUDA;
}

int BatchRenderer::validate(Q_cuda_batch_options& o) const {
    if (o.max_depth == 0) o.max_depth = 6;
    if (o.max_depth > 64) return QUASI_ERR_INVALID;
    if (o.form > QUASI_BATCH_MEGAKERNEL) return QUASI_ERR_INVALID;
    if (o.trace_block == 0) o.trace_block = 128;
    if (o.trace_block % 32 != 0 || o.trace_block > 256) return QUASI_ERR_INVALID;
    if (o.fetch_rays == 0) o.fetch_rays = 32;
    if (o.fetch_rays % 32 != 0 || o.fetch_rays > 1024) return QUASI_ERR_INVALID;
    if (o.use_graph == 0) o.use_graph = 1;
    if (o.use_graph > 2) return QUASI_ERR_INVALID;
    if (o.wave_paths > k_max_wave_paths) return QUASI_ERR_INVALID;
    if (!(o.ray_eps > 0.f)) o.ray_eps = 1e-4f;
    if (o.bvh_width == 0) o.bvh_width = 8;
    if (o.bvh_width != 2 && o.bvh_width != 8) return QUASI_ERR_INVALID;
    if (o.refill_lanes == 0) o.refill_lanes = k_wide_refill_lanes;
    if (o.refill_lanes > 32) return QUASI_ERR_INVALID;
    return QUASI_OK;
}

int BatchRenderer::create(const Q_cuda_batch_scene* scenes, uint32_t count, const Q_cuda_batch_options* options) {
    if (!scenes || count == 0) return fail(QUASI_ERR_INVALID, "no scenes");
    Q_cuda_batch_options o = options ? *options : Q_cuda_batch_options{};
    if (validate(o)) return fail(QUASI_ERR_INVALID, "invalid batch options");
    opt_ = o;
    B_TRY(cudaSetDevice(owner_.device()), "cudaSetDevice");
    stream_ = owner_.stream();
    scenes_.resize(count);
    uint64_t tri = 0, px = 0, emit = 0;
    std::vector<std::vector<int>> emitters(count);
    for (uint32_t i = 0; i < count; ++i) {
        const Q_cuda_batch_scene& b = scenes[i];
        if (!b.scene) return fail(QUASI_ERR_INVALID, "null scene");
        const Q_cuda_scene& sc = *b.scene;
        if (sc.tri_count > 0 && (!sc.vertices || !sc.albedo || !sc.emission))
            return fail(QUASI_ERR_INVALID, "scene arrays missing");
        if (b.width == 0 || b.height == 0 || b.spp == 0) return fail(QUASI_ERR_INVALID, "zero width, height or spp");
        if (static_cast<uint64_t>(b.width) * b.height > (1ull << 26)) return fail(QUASI_ERR_INVALID, "scene too large");
        if (static_cast<uint64_t>(ceil_div(b.width, 8)) * ceil_div(b.height, 4) * 32ull > k_max_wave_paths)
            return fail(QUASI_ERR_INVALID, "scene too large");
        for (uint32_t t = 0; t < sc.tri_count; ++t)
            if (sc.emission[3 * t] > 0.f || sc.emission[3 * t + 1] > 0.f || sc.emission[3 * t + 2] > 0.f)
                emitters[i].push_back(static_cast<int>(t));
        scenes_[i] = HostScene{static_cast<uint32_t>(tri), sc.tri_count, b.width, b.height, b.spp,
                               static_cast<uint32_t>(px), static_cast<uint32_t>(emit),
                               static_cast<uint32_t>(emitters[i].size()), sc.camera};
        tri += sc.tri_count;
        px += static_cast<uint64_t>(b.width) * b.height;
        emit += emitters[i].size();
        if (tri >= (1ull << 30) || px >= (1ull << 31)) return fail(QUASI_ERR_INVALID, "batch too large");
    }
    tri_total_ = tri;
    px_total_ = px;
    camera_rays_ = 0;
    max_slots_ = 0;
    for (const HostScene& h : scenes_) {
        camera_rays_ += static_cast<uint64_t>(h.width) * h.height * h.spp;
        max_slots_ = std::max(max_slots_, ceil_div(h.width, 8) * ceil_div(h.height, 4) * 32);
    }
    cudaStream_t s = stream_;
    // geometry and material pools
    {
        std::vector<float4> t4(3 * tri), a4(tri), e4(tri);
        std::vector<int> em;
        em.reserve(emit);
        for (uint32_t i = 0; i < count; ++i) {
            const Q_cuda_scene& sc = *scenes[i].scene;
            const size_t off = scenes_[i].tri_offset;
            for (uint32_t t = 0; t < sc.tri_count; ++t) {
                const float* v = sc.vertices + 9ull * t;
                t4[3 * (off + t) + 0] = make_float4(v[0], v[1], v[2], 0.f);
                t4[3 * (off + t) + 1] = make_float4(v[3], v[4], v[5], 0.f);
                t4[3 * (off + t) + 2] = make_float4(v[6], v[7], v[8], 0.f);
                a4[off + t] = make_float4(sc.albedo[3 * t], sc.albedo[3 * t + 1], sc.albedo[3 * t + 2], 0.f);
                e4[off + t] = make_float4(sc.emission[3 * t], sc.emission[3 * t + 1], sc.emission[3 * t + 2], 0.f);
            }
            em.insert(em.end(), emitters[i].begin(), emitters[i].end());
        }
        B_TRY(tri_in_.reserve(sizeof(float4) * std::max<size_t>(t4.size(), 1)), "triangles");
        B_TRY(albedo_.reserve(sizeof(float4) * std::max<size_t>(a4.size(), 1)), "albedo");
        B_TRY(emission_.reserve(sizeof(float4) * std::max<size_t>(e4.size(), 1)), "emission");
        B_TRY(emitters_.reserve(sizeof(int) * std::max<size_t>(em.size(), 1)), "emitters");
        if (tri) {
            B_TRY(cudaMemcpy(tri_in_.ptr, t4.data(), sizeof(float4) * t4.size(), cudaMemcpyHostToDevice), "h2d");
            B_TRY(cudaMemcpy(albedo_.ptr, a4.data(), sizeof(float4) * a4.size(), cudaMemcpyHostToDevice), "h2d");
            B_TRY(cudaMemcpy(emission_.ptr, e4.data(), sizeof(float4) * e4.size(), cudaMemcpyHostToDevice), "h2d");
        }
        if (!em.empty())
            B_TRY(cudaMemcpy(emitters_.ptr, em.data(), sizeof(int) * em.size(), cudaMemcpyHostToDevice), "h2d");
    }
    for (DeviceBuffer* b : {&accum_, &comp_, &aov_a_, &aov_n_}) B_TRY(b->reserve(sizeof(float4) * px), "image pool");
    B_TRY(stats_dev_.reserve(sizeof(unsigned long long) * 9), "stats");
    B_TRY(err_dev_.reserve(sizeof(uint32_t)), "err");
    B_TRY(cudaMemsetAsync(err_dev_.ptr, 0, sizeof(uint32_t), s), "memset");
    B_TRY(cudaMallocHost(&stats_host_, sizeof(unsigned long long) * 9), "pinned");
    B_TRY(cudaMallocHost(&err_host_, sizeof(uint32_t)), "pinned");
    std::memset(stats_host_, 0, sizeof(unsigned long long) * 9);
    *err_host_ = 0;
    B_TRY(cudaEventCreate(&ev0_), "event");
    B_TRY(cudaEventCreate(&ev1_), "event");
    B_TRY(cudaStreamCreateWithFlags(&capture_, cudaStreamNonBlocking), "stream");
    // one LBVH per scene, over the triangles themselves: on the 64-scene soup mix, split leaf
    // references (the single-scene default for scenes of 2^17 triangles and more) rendered
    // the batch at 1437.7 against 1464.4 Mrays/s (its autotuner then chose smaller waves)
    KernelProfiler build_prof;
    bvh_.clear();
    for (uint32_t i = 0; i < count; ++i) {
        bvh_.emplace_back(new LbvhBuilder());
        bvh_[i]->set_split_percent(0);
        const HostScene& h = scenes_[i];
        B_TRY(bvh_[i]->build(tri_in_.as<float4>() + 3ull * h.tri_offset, h.n_tris, emitters_.as<int>() + h.emit_offset,
                             h.n_emit, s, build_prof, err_dev_.as<uint32_t>()),
              "lbvh build");
    }
    int rc = upload_table();
    if (rc) return rc;
    rc = plan(0xffffffffu);
    if (rc) return rc;
    B_TRY(cudaStreamSynchronize(s), "sync");
    return reset();
}

// Uploads the per-scene table (sample bases back to 0).
int BatchRenderer::upload_table() {
    std::vector<BatchSceneDev> t(scenes_.size());
    for (size_t i = 0; i < scenes_.size(); ++i) {
        const HostScene& h = scenes_[i];
        BatchSceneDev& d = t[i];
        std::memset(&d, 0, sizeof(d));
        FrameParams& f = d.f;
        f.cam = make_camera_basis(h.camera, h.width, h.height);
        f.width = h.width;
        f.height = h.height;
        f.tiles_x = ceil_div(h.width, 8);
        f.slots = f.tiles_x * ceil_div(h.height, 4) * 32;
        f.sample_base = 0;
        f.seed = opt_.seed;
        f.max_depth = opt_.max_depth;
        f.eps = opt_.ray_eps;
        f.frame_spp = h.spp;
        const LbvhView bv = bvh_[i]->view();
        d.s = SceneDev{tri_in_.as<float4>() + 3ull * h.tri_offset,
                       albedo_.as<float4>() + h.tri_offset,
                       emission_.as<float4>() + h.tri_offset,
                       bv.nodes,
                       bv.tris,
                       h.n_tris,
                       h.n_emit,
                       k_refill_lanes,
                       k_trace_steps,
                       nullptr,
                       0,
                       opt_.bvh_width == 2 ? nullptr : bv.wide,
                       bv.tri_plane,
                       bv.emit_tab};
        d.px_offset = h.px_offset;
        d.tri_offset = h.tri_offset;
        d.spp = h.spp;
    }
    B_TRY(table_.reserve(sizeof(BatchSceneDev) * t.size()), "scene table");
    B_TRY(cudaStreamSynchronize(stream_), "sync");
    B_TRY(cudaMemcpy(table_.ptr, t.data(), sizeof(BatchSceneDev) * t.size(), cudaMemcpyHostToDevice), "h2d");
    frames_since_reset_ = 0;
    return QUASI_OK;
}

// Cuts every scene's frame (min(spp, spp_cap) samples) into items of whole sample planes and
// packs them into waves of at most W path slots, scene after scene.
int BatchRenderer::plan(uint32_t spp_cap) {
    // per path slot: two ray queues (2 x 32), hit 16, shadow ray 64, beta, radiance and two
    // AOVs (4 x 16), double-float ray 48, (scene, local path) 8, fixup list entry 8
    constexpr size_t bytes_per_path = 272;
    uint32_t W = opt_.wave_paths ? opt_.wave_paths
                                 : static_cast<uint32_t>(wave_paths_fitting(k_default_wave_paths, bytes_per_path,
                                                                            size_t(wave_capacity_) * bytes_per_path));
    W = std::max(W, max_slots_);
    items_host_.clear();
    waves_.clear();
    Wave cur{0, 0, 0, 0};
    auto close = [&]() {
        if (cur.n_items) waves_.push_back(cur);
        cur = Wave{static_cast<uint32_t>(items_host_.size()), 0, 0, 0};
    };
    for (uint32_t s = 0; s < scenes_.size(); ++s) {
        const HostScene& h = scenes_[s];
        const uint32_t slots = ceil_div(h.width, 8) * ceil_div(h.height, 4) * 32;
        const uint32_t spp = std::min(h.spp, spp_cap);
        uint32_t j = 0;
        while (j < spp) {
            if (W - cur.paths < slots) close();
            const uint32_t nj = std::min(spp - j, (W - cur.paths) / slots);
            items_host_.push_back(Item{s, j, nj, slots, cur.paths, cur.acc_threads});
            cur.paths += nj * slots;
            cur.acc_threads += slots;
            ++cur.n_items;
            j += nj;
        }
    }
    close();
    plan_cap_ = spp_cap;
    plan_wave_paths_ = W;
    std::vector<BatchItem> dev(items_host_.size());
    for (size_t i = 0; i < dev.size(); ++i) {
        const Item& it = items_host_[i];
        dev[i] = BatchItem{it.scene, it.j0, it.nj, it.slots, it.pid_base, it.acc_base};
    }
    B_TRY(items_.reserve(sizeof(BatchItem) * std::max<size_t>(dev.size(), 1)), "items");
    if (!dev.empty())
        B_TRY(cudaMemcpy(items_.ptr, dev.data(), sizeof(BatchItem) * dev.size(), cudaMemcpyHostToDevice), "h2d");
    graphs_dirty_ = true;
    return ensure_buffers();
}

int BatchRenderer::ensure_buffers() {
    uint32_t paths = 0;
    for (const Wave& w : waves_) paths = std::max(paths, w.paths);
    if (paths > wave_capacity_) {
        B_TRY(queue_[0].reserve(sizeof(float4) * 2ull * paths), "queue");
        B_TRY(queue_[1].reserve(sizeof(float4) * 2ull * paths), "queue");
        B_TRY(hits_.reserve(sizeof(float4) * paths), "hits");
        B_TRY(shadow_.reserve(sizeof(float4) * 4ull * paths), "shadow");
        B_TRY(beta_.reserve(sizeof(float4) * paths), "beta");
        B_TRY(lpath_.reserve(sizeof(float4) * paths), "lpath");
        B_TRY(pa_.reserve(sizeof(float4) * paths), "aov");
        B_TRY(pn_.reserve(sizeof(float4) * paths), "aov");
        B_TRY(ray_ff_.reserve(sizeof(float4) * 3ull * paths), "ray_ff");
        B_TRY(defer_.reserve(sizeof(int2) * paths), "defer");
        B_TRY(meta_.reserve(sizeof(uint2) * paths), "meta");
        wave_capacity_ = paths;
        graphs_dirty_ = true;
    }
    const size_t nw = std::max<size_t>(waves_.size(), 1);
    const size_t need = sizeof(int) * k_batch_counters_per_bounce * opt_.max_depth * nw;
    if (need > counters_.bytes || sizeof(int) * nw > adj_counters_.bytes) graphs_dirty_ = true;
    B_TRY(counters_.reserve(need), "counters");
    B_TRY(adj_counters_.reserve(sizeof(int) * nw), "counters");
    return QUASI_OK;
}

// Grid sizes of the persistent kernels for the current block sizes: SMs x resident blocks.
void BatchRenderer::compute_grids() {
    const bool stats = opt_.collect_stats != 0;
    const bool wide = opt_.bvh_width != 2;
    auto kc = stats ? (wide ? k_batch_trace_closest<true, true> : k_batch_trace_closest<true, false>)
                    : (wide ? k_batch_trace_closest<false, true> : k_batch_trace_closest<false, false>);
    auto ks = stats ? (wide ? k_batch_trace_shadow<true, true> : k_batch_trace_shadow<true, false>)
                    : (wide ? k_batch_trace_shadow<false, true> : k_batch_trace_shadow<false, false>);
    auto km = stats ? k_batch_megakernel<true> : k_batch_megakernel<false>;
    const int tb = static_cast<int>(opt_.trace_block), mb = std::min(tb, 128);
    smem_c_ = wide ? wide_stack_smem_bytes<false>(tb) : 0;
    smem_s_ = wide ? wide_stack_smem_bytes<true>(tb) : 0;
    const int sm = owner_.sm_count();
    grid_c_ = sm * resident_blocks(kc, tb, smem_c_);
    grid_s_ = sm * resident_blocks(ks, tb, smem_s_);
    grid_m_ = sm * resident_blocks(km, mb, 0);
    grid_adj_ = sm * resident_blocks(k_batch_adjoint, 128, 0);
}

// Enqueues one frame (every wave of the plan) on s; `launches` receives the kernel count.
int BatchRenderer::record_frame(cudaStream_t s, uint32_t& launches) {
    prof_.reset_launches();
    const uint32_t D = opt_.max_depth;
    const int n_scenes = static_cast<int>(scenes_.size());
    const BatchSceneDev* table = table_.as<BatchSceneDev>();
    const BatchItem* items = items_.as<BatchItem>();
    PathDev pd{beta_.as<float4>(), lpath_.as<float4>(), pa_.as<float4>(), pn_.as<float4>(), ray_ff_.as<float4>(),
               nullptr};
    uint2* meta = meta_.as<uint2>();
    uint32_t* err = err_dev_.as<uint32_t>();
    unsigned long long* st = stats_dev_.as<unsigned long long>();
    const int sm = owner_.sm_count();
    const int tb = static_cast<int>(opt_.trace_block);
    const int mb = std::min(tb, 128);
    const int chunk = static_cast<int>(opt_.fetch_rays);
    const int refill = static_cast<int>(opt_.refill_lanes);
    const size_t per_wave = size_t(k_batch_counters_per_bounce) * D;
    B_TRY(cudaMemsetAsync(counters_.ptr, 0, sizeof(int) * per_wave * std::max<size_t>(waves_.size(), 1), s), "memset");
    const bool stats = opt_.collect_stats != 0;
    const bool wide = opt_.bvh_width != 2;
    auto kc = stats ? (wide ? k_batch_trace_closest<true, true> : k_batch_trace_closest<true, false>)
                    : (wide ? k_batch_trace_closest<false, true> : k_batch_trace_closest<false, false>);
    auto ks = stats ? (wide ? k_batch_trace_shadow<true, true> : k_batch_trace_shadow<true, false>)
                    : (wide ? k_batch_trace_shadow<false, true> : k_batch_trace_shadow<false, false>);
    auto km = stats ? k_batch_megakernel<true> : k_batch_megakernel<false>;
    const int grid_c = grid_c_, grid_s = grid_s_, grid_m = grid_m_;
    const int grid_shade = sm * 32;  // as the single-scene renderer's shading launch
    const int grid_fixup = sm * resident_blocks(k_batch_fixup<ClosestJob>, 128, 0);
    const int cap = static_cast<int>(wave_capacity_);
    for (size_t w = 0; w < waves_.size(); ++w) {
        const Wave& wv = waves_[w];
        const BatchItem* wi = items + wv.item0;
        const int ni = static_cast<int>(wv.n_items);
        int* cnt = counters_.as<int>() + w * per_wave;
        if (opt_.form == QUASI_BATCH_MEGAKERNEL) {
            B_TRY(QUASI_LAUNCH(prof_, "batch_megakernel", s,
                               (km<<<grid_m, mb, 0, s>>>(table, wi, ni, wv.paths, pd, chunk, cnt, err, st))),
                  "batch_megakernel");
        } else {
            B_TRY(QUASI_LAUNCH(prof_, "batch_camera", s,
                               (k_batch_camera<<<ceil_div(wv.paths, 256), 256, 0, s>>>(table, wi, ni, wv.paths, pd, meta,
                                                                                       queue_[0].as<float4>(), cnt))),
                  "batch_camera");
            for (uint32_t k = 1; k <= D; ++k) {
                float4* qcur = queue_[(k - 1) & 1].as<float4>();
                float4* qnext = queue_[k & 1].as<float4>();
                int* c_cur = cnt + (k - 1);
                int* c_next = cnt + k;
                int* c_shadow = cnt + D + (k - 1);
                int* f_cur = cnt + 2 * D + (k - 1);
                int* f_shadow = cnt + 3 * D + (k - 1);
                const ClosestJob cjob{qcur, hits_.as<float4>(), ray_ff_.as<float4>(), lpath_.as<float4>(),
                                      DeferList{defer_.as<int2>(), cnt + 4 * D + (k - 1), cnt + 8 * D + (k - 1), cap},
                                      nullptr};
                const ShadowJob sjob{shadow_.as<float4>(), pd,
                                     DeferList{defer_.as<int2>(), cnt + 5 * D + (k - 1), cnt + 9 * D + (k - 1), cap}};
                B_TRY(QUASI_LAUNCH(prof_, "batch_trace_closest", s,
                                   (kc<<<grid_c, tb, smem_c_, s>>>(table, meta, cjob, c_cur, cap, chunk, refill, f_cur, err,
                                                                   st))),
                      "batch_trace_closest");
                B_TRY(QUASI_LAUNCH(prof_, "batch_fixup_closest", s,
                                   (k_batch_fixup<ClosestJob><<<grid_fixup, 128, 0, s>>>(table, meta, cjob,
                                                                                        cnt + 6 * D + (k - 1), err))),
                      "batch_fixup_closest");
                B_TRY(QUASI_LAUNCH(prof_, "batch_shade", s,
                                   (k_batch_shade<<<grid_shade, 256, 0, s>>>(table, meta, pd, k, hits_.as<float4>(),
                                                                             c_cur, cap, qnext, k < D ? c_next : nullptr,
                                                                             shadow_.as<float4>(), c_shadow))),
                      "batch_shade");
                B_TRY(QUASI_LAUNCH(prof_, "batch_trace_shadow", s,
                                   (ks<<<grid_s, tb, smem_s_, s>>>(table, meta, sjob, c_shadow, cap, chunk, refill, f_shadow,
                                                                   err, st))),
                      "batch_trace_shadow");
                B_TRY(QUASI_LAUNCH(prof_, "batch_fixup_shadow", s,
                                   (k_batch_fixup<ShadowJob><<<grid_fixup, 128, 0, s>>>(table, meta, sjob,
                                                                                       cnt + 7 * D + (k - 1), err))),
                      "batch_fixup_shadow");
            }
        }
        B_TRY(QUASI_LAUNCH(prof_, "batch_accumulate", s,
                           (k_batch_accumulate<<<ceil_div(wv.acc_threads, 256), 256, 0, s>>>(
                               table, wi, ni, wv.acc_threads, pd, accum_.as<float4>(), comp_.as<float4>(),
                               aov_a_.as<float4>(), aov_n_.as<float4>()))),
              "batch_accumulate");
    }
    if (opt_.form != QUASI_BATCH_MEGAKERNEL)
        B_TRY(QUASI_LAUNCH(prof_, "batch_tally", s,
                           (k_batch_tally<<<1, 32, 0, s>>>(counters_.as<int>(), static_cast<uint32_t>(waves_.size()), D,
                                                           st))),
              "batch_tally");
    B_TRY(QUASI_LAUNCH(prof_, "batch_advance", s,
                       (k_batch_advance<<<1, 256, 0, s>>>(table_.as<BatchSceneDev>(), n_scenes, st))),
          "batch_advance");
    launches = prof_.launches();
    return QUASI_OK;
}

// Enqueues the adjoint of the last frame: grad_image_ -> grad_albedo_, grad_emission_.
int BatchRenderer::record_adjoint(cudaStream_t s) {
    B_TRY(cudaMemsetAsync(grad_albedo_.ptr, 0, sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1), s), "memset");
    B_TRY(cudaMemsetAsync(grad_emission_.ptr, 0, sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1), s),
          "memset");
    B_TRY(cudaMemsetAsync(adj_counters_.ptr, 0, sizeof(int) * std::max<size_t>(waves_.size(), 1), s), "memset");
    const int grid = grid_adj_;
    for (size_t w = 0; w < waves_.size(); ++w) {
        const Wave& wv = waves_[w];
        B_TRY(QUASI_LAUNCH(prof_, "batch_adjoint", s,
                           (k_batch_adjoint<<<grid, 128, 0, s>>>(
                               table_.as<BatchSceneDev>(), items_.as<BatchItem>() + wv.item0,
                               static_cast<int>(wv.n_items), wv.paths, grad_image_.as<float>(), grad_albedo_.as<float>(),
                               grad_emission_.as<float>(), static_cast<int>(opt_.fetch_rays),
                               adj_counters_.as<int>() + w, err_dev_.as<uint32_t>(),
                               stats_dev_.as<unsigned long long>()))),
              "batch_adjoint");
    }
    return QUASI_OK;
}

void BatchRenderer::drop_graphs() {
    if (frame_exec_) cudaGraphExecDestroy(frame_exec_);
    if (adjoint_exec_) cudaGraphExecDestroy(adjoint_exec_);
    frame_exec_ = adjoint_exec_ = nullptr;
}

// Captures the frame (and, for max_depth <= 16, the adjoint) launch sequences.
int BatchRenderer::ensure_graphs() {
    if (!graphs_dirty_) return QUASI_OK;
    drop_graphs();
    compute_grids();
    uint32_t launches = 0;
    if (opt_.use_graph == 1) {
        for (int which = 0; which < 2; ++which) {
            if (which == 1 && opt_.max_depth > static_cast<uint32_t>(k_adjoint_max_depth)) break;
            if (which == 1) {
                B_TRY(grad_image_.reserve(sizeof(float) * 3ull * px_total_), "grad image");
                B_TRY(grad_albedo_.reserve(sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1)), "grads");
                B_TRY(grad_emission_.reserve(sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1)), "grads");
            }
            B_TRY(cudaStreamBeginCapture(capture_, cudaStreamCaptureModeThreadLocal), "begin capture");
            uint32_t n = 0;
            const int rc = which == 0 ? record_frame(capture_, n) : record_adjoint(capture_);
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(capture_, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            B_TRY(ec, "end capture");
            cudaGraphExec_t exec = nullptr;
            const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            B_TRY(ei, "graph instantiate");
            if (which == 0) {
                frame_exec_ = exec;
                launches = n;
            } else {
                adjoint_exec_ = exec;
            }
        }
    } else {
        // Plain launches: count the kernels of one frame without enqueueing them.
        const uint32_t D = opt_.max_depth;
        const uint32_t nw = static_cast<uint32_t>(waves_.size());
        launches = opt_.form == QUASI_BATCH_MEGAKERNEL ? 2 * nw + 1 : nw * (2 + 5 * D) + 2;
    }
    kernels_per_frame_ = launches;
    graphs_dirty_ = false;
    return QUASI_OK;
}

int BatchRenderer::render(cudaStream_t stream) {
    error_.clear();
    cudaStream_t s = pick(stream);
    if (plan_cap_ != 0xffffffffu) {
        int rc = plan(0xffffffffu);
        if (rc) return rc;
    }
    int rc = ensure_graphs();
    if (rc) return rc;
    B_TRY(cudaEventRecord(ev0_, s), "event");
    if (frame_exec_) {
        B_TRY(cudaGraphLaunch(frame_exec_, s), "graph launch");
    } else {
        uint32_t n = 0;
        compute_grids();
        rc = record_frame(s, n);
        if (rc) return rc;
    }
    B_TRY(cudaEventRecord(ev1_, s), "event");
    timed_ = true;
    ++frames_since_reset_;
    return QUASI_OK;
}

int BatchRenderer::reset() {
    cudaStream_t s = stream_;
    for (DeviceBuffer* b : {&accum_, &comp_, &aov_a_, &aov_n_})
        if (b->ptr) B_TRY(cudaMemsetAsync(b->ptr, 0, b->bytes, s), "memset");
    B_TRY(cudaMemsetAsync(stats_dev_.ptr, 0, sizeof(unsigned long long) * 9, s), "memset");
    B_TRY(QUASI_LAUNCH(prof_, "batch_rewind", s,
                       (k_batch_rewind<<<1, 256, 0, s>>>(table_.as<BatchSceneDev>(),
                                                         static_cast<uint32_t>(scenes_.size())))),
          "batch_rewind");
    timed_ = false;
    frames_since_reset_ = 0;
    return QUASI_OK;
}

int BatchRenderer::set_seed(uint32_t seed, cudaStream_t stream) {
    cudaStream_t s = pick(stream);
    opt_.seed = seed;
    for (DeviceBuffer* b : {&accum_, &comp_, &aov_a_, &aov_n_}) B_TRY(cudaMemsetAsync(b->ptr, 0, b->bytes, s), "memset");
    B_TRY(QUASI_LAUNCH(prof_, "batch_reseed", s,
                       (k_batch_reseed<<<1, 256, 0, s>>>(table_.as<BatchSceneDev>(),
                                                         static_cast<uint32_t>(scenes_.size()), seed))),
          "batch_reseed");
    frames_since_reset_ = 0;
    return QUASI_OK;
}

int BatchRenderer::set_options(const Q_cuda_batch_options& o) {
    Q_cuda_batch_options n = o;
    if (validate(n)) return fail(QUASI_ERR_INVALID, "invalid batch options");
    B_TRY(cudaStreamSynchronize(stream_), "sync");
    opt_ = n;
    int rc = upload_table();
    if (rc) return rc;
    rc = plan(0xffffffffu);
    if (rc) return rc;
    return reset();
}

int BatchRenderer::synchronize() {
    B_TRY(cudaStreamSynchronize(stream_), "synchronize");
    B_TRY(cudaMemcpy(err_host_, err_dev_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost), "d2h");
    if (*err_host_ & QUASI_DEVERR_STACK) return fail(QUASI_ERR_STACK, "BVH traversal stack overflow");
    if (*err_host_ & (QUASI_DEVERR_TIMEOUT | QUASI_DEVERR_TRAVERSAL))
        return fail(QUASI_ERR_TIMEOUT, "a bounded device loop gave up");
    return QUASI_OK;
}

int BatchRenderer::stats(Q_cuda_batch_stats* out) {
    if (!out) return fail(QUASI_ERR_INVALID, "null stats");
    B_TRY(cudaStreamSynchronize(stream_), "synchronize");
    B_TRY(cudaMemcpy(stats_host_, stats_dev_.ptr, sizeof(unsigned long long) * 9, cudaMemcpyDeviceToHost), "d2h");
    B_TRY(cudaMemcpy(err_host_, err_dev_.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost), "d2h");
    Q_cuda_batch_stats r{};
    r.frames = stats_host_[4];
    r.camera_rays = camera_rays_;
    r.closest_rays = stats_host_[5];
    r.shadow_rays = stats_host_[6];
    r.node_visits = stats_host_[0] + stats_host_[2];
    r.tri_tests = stats_host_[1] + stats_host_[3];
    r.adjoint_rays = stats_host_[7];
    r.redecided_rays = stats_host_[8];
    r.scenes = static_cast<uint32_t>(scenes_.size());
    r.waves = static_cast<uint32_t>(waves_.size());
    r.kernels_per_frame = kernels_per_frame_;
    r.error_flags = *err_host_;
    r.tri_total = tri_total_;
    r.px_total = px_total_;
    float ms = 0.f;
    if (timed_ && cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) r.frame_ms = ms;
    *out = r;
    return QUASI_OK;
}

int BatchRenderer::readback(uint32_t index, float* host_rgba) {
    if (index >= scenes_.size() || !host_rgba) return fail(QUASI_ERR_INVALID, "bad scene index or buffer");
    const HostScene& h = scenes_[index];
    const uint32_t n = h.width * h.height;
    DeviceBuffer tmp;
    B_TRY(tmp.reserve(sizeof(float4) * n), "resolve buffer");
    cudaStream_t s = stream_;
    B_TRY(QUASI_LAUNCH(prof_, "batch_resolve", s,
                       (k_batch_resolve<<<ceil_div(n, 256), 256, 0, s>>>(
                           table_.as<BatchSceneDev>(), static_cast<int>(scenes_.size()), accum_.as<float4>(),
                           h.px_offset, n, false, tmp.as<float>()))),
          "batch_resolve");
    B_TRY(cudaMemcpyAsync(host_rgba, tmp.ptr, sizeof(float4) * n, cudaMemcpyDeviceToHost, s), "d2h");
    B_TRY(cudaStreamSynchronize(s), "sync");
    tmp.release();
    return QUASI_OK;
}

int BatchRenderer::resolve_device(float* device_rgb, cudaStream_t stream) {
    if (!device_rgb) return fail(QUASI_ERR_INVALID, "null output");
    cudaStream_t s = pick(stream);
    const uint32_t n = static_cast<uint32_t>(px_total_);
    B_TRY(QUASI_LAUNCH(prof_, "batch_resolve", s,
                       (k_batch_resolve<<<ceil_div(n, 256), 256, 0, s>>>(table_.as<BatchSceneDev>(),
                                                                          static_cast<int>(scenes_.size()),
                                                                          accum_.as<float4>(), 0u, n, true, device_rgb))),
          "batch_resolve");
    return QUASI_OK;
}

int BatchRenderer::offsets(uint32_t index, uint64_t* tri_offset, uint64_t* px_offset) const {
    if (index >= scenes_.size()) return QUASI_ERR_INVALID;
    if (tri_offset) *tri_offset = scenes_[index].tri_offset;
    if (px_offset) *px_offset = scenes_[index].px_offset;
    return QUASI_OK;
}

int BatchRenderer::set_materials_device(const float* albedo, const float* emission, cudaStream_t stream) {
    cudaStream_t s = pick(stream);
    if (tri_total_) {
        const uint32_t n = static_cast<uint32_t>(tri_total_);
        B_TRY(QUASI_LAUNCH(prof_, "batch_pack_materials", s,
                           (k_batch_pack_materials<<<ceil_div(n, 256), 256, 0, s>>>(
                               albedo, emission, n, albedo_.as<float4>(), emission_.as<float4>()))),
              "batch_pack_materials");
    }
    for (DeviceBuffer* b : {&accum_, &comp_, &aov_a_, &aov_n_}) B_TRY(cudaMemsetAsync(b->ptr, 0, b->bytes, s), "memset");
    B_TRY(QUASI_LAUNCH(prof_, "batch_rewind", s,
                       (k_batch_rewind<<<1, 256, 0, s>>>(table_.as<BatchSceneDev>(),
                                                         static_cast<uint32_t>(scenes_.size())))),
          "batch_rewind");
    frames_since_reset_ = 0;
    return QUASI_OK;
}

int BatchRenderer::backward(const float* grad_image, float* grad_albedo, float* grad_emission, cudaStream_t stream) {
    if (!grad_image) return fail(QUASI_ERR_INVALID, "null gradient image");
    if (opt_.max_depth > static_cast<uint32_t>(k_adjoint_max_depth))
        return fail(QUASI_ERR_INVALID, "backward supports max_depth up to 16");
    if (plan_cap_ != 0xffffffffu || frames_since_reset_ == 0)
        return fail(QUASI_ERR_STATE, "render a frame before backward");
    cudaStream_t s = pick(stream);
    int rc = ensure_graphs();
    if (rc) return rc;
    B_TRY(grad_image_.reserve(sizeof(float) * 3ull * px_total_), "grad image");
    B_TRY(grad_albedo_.reserve(sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1)), "grads");
    B_TRY(grad_emission_.reserve(sizeof(float) * 3ull * std::max<uint64_t>(tri_total_, 1)), "grads");
    B_TRY(cudaMemcpyAsync(grad_image_.ptr, grad_image, sizeof(float) * 3ull * px_total_, cudaMemcpyDeviceToDevice, s),
          "d2d");
    if (adjoint_exec_) {
        B_TRY(cudaGraphLaunch(adjoint_exec_, s), "graph launch");
    } else {
        rc = record_adjoint(s);
        if (rc) return rc;
    }
    if (grad_albedo && tri_total_)
        B_TRY(cudaMemcpyAsync(grad_albedo, grad_albedo_.ptr, sizeof(float) * 3ull * tri_total_,
                              cudaMemcpyDeviceToDevice, s),
              "d2d");
    if (grad_emission && tri_total_)
        B_TRY(cudaMemcpyAsync(grad_emission, grad_emission_.ptr, sizeof(float) * 3ull * tri_total_,
                              cudaMemcpyDeviceToDevice, s),
              "d2d");
    return QUASI_OK;
}

// Device time of one frame of the current plan and options (after one untimed frame).
int BatchRenderer::time_frame(float& ms) {
    cudaStream_t s = stream_;
    int rc = ensure_graphs();
    if (rc) return rc;
    for (int rep = 0; rep < 2; ++rep) {
        B_TRY(cudaEventRecord(ev0_, s), "event");
        if (frame_exec_) {
            B_TRY(cudaGraphLaunch(frame_exec_, s), "graph launch");
        } else {
            uint32_t n = 0;
            rc = record_frame(s, n);
            if (rc) return rc;
        }
        B_TRY(cudaEventRecord(ev1_, s), "event");
        B_TRY(cudaEventSynchronize(ev1_), "sync");
    }
    B_TRY(cudaEventElapsedTime(&ms, ev0_, ev1_), "event time");
    return QUASI_OK;
}

// Coordinate search over form, wave size, block size and fetch size (warp chunks over the
// binary LBVH) or refill threshold (8-wide records). Candidates are timed on the batch's own
// frame when the whole search over it fits half the budget, else on frames capped at fewer
// samples per pixel (at least 1) so that it does. The cap matters: a 1-spp frame of 64 small
// scenes weighs the wavefront form's fixed launch work 4x more than their 4-spp frame, where
// the wavefront form is the faster one (3.1 vs 4.6 ms per frame on GB300), and a search on
// 1-spp frames chose the megakernel.
int BatchRenderer::autotune(double budget_ms, Q_cuda_batch_options* chosen) {
    if (budget_ms <= 0.0) budget_ms = 5000.0;
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&]() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    uint32_t tune_spp = 1;
    auto measure = [&](const Q_cuda_batch_options& o, float& ms) -> int {
        opt_ = o;
        int rc = plan(tune_spp);
        if (rc) return rc;
        return time_frame(ms);
    };
    Q_cuda_batch_options best = opt_;
    float best_ms = 0.f;
    int rc = measure(best, best_ms);
    if (rc) return rc;
    // A frame capped at c samples per pixel costs at most c times the 1-spp frame, and each
    // of the ~12 candidates times two frames.
    constexpr double k_candidates = 12.0;
    uint32_t max_spp = 1;
    for (const HostScene& h : scenes_) max_spp = std::max(max_spp, h.spp);
    const double cap = 0.5 * budget_ms / k_candidates / (2.0 * std::max(static_cast<double>(best_ms), 1e-3));
    tune_spp = cap >= max_spp ? 0xffffffffu : std::max<uint32_t>(1, static_cast<uint32_t>(cap));
    if (tune_spp != 1) {
        rc = measure(best, best_ms);
        if (rc) return rc;
    }
    const uint32_t forms[] = {QUASI_BATCH_WAVEFRONT, QUASI_BATCH_MEGAKERNEL};
    const uint32_t waves[] = {16u << 20, 32u << 20, 64u << 20, 128u << 20};
    const uint32_t blocks[] = {64, 128, 256};
    const uint32_t fetches[] = {32, 64, 128};
    const uint32_t refills[] = {4, 8, 16};
    const bool wide = opt_.bvh_width != 2;
    for (int dim = 0; dim < 4 && elapsed() < budget_ms; ++dim) {
        const uint32_t* vals = dim == 0 ? forms : dim == 1 ? waves : dim == 2 ? blocks : wide ? refills : fetches;
        const int nv = dim == 0 ? 2 : dim == 1 ? 4 : 3;
        for (int v = 0; v < nv && elapsed() < budget_ms; ++v) {
            Q_cuda_batch_options o = best;
            uint32_t& field = dim == 0   ? o.form
                              : dim == 1 ? o.wave_paths
                              : dim == 2 ? o.trace_block
                              : wide     ? o.refill_lanes
                                         : o.fetch_rays;
            const uint32_t cur = dim == 1 && field == 0 ? k_default_wave_paths : field;
            if (vals[v] == cur) continue;
            if (dim == 1 && vals[v] < max_slots_) continue;
            if (dim == 2 && o.form == QUASI_BATCH_MEGAKERNEL && vals[v] > 128) continue;
            field = vals[v];
            float ms = 0.f;
            rc = measure(o, ms);
            if (rc) return rc;
            if (ms < best_ms) {
                best_ms = ms;
                best = o;
            }
        }
    }
    opt_ = best;
    rc = plan(0xffffffffu);
    if (rc) return rc;
    if (chosen) *chosen = best;
    return reset();
}

}  // namespace quasi
