/* quasi_cuda.h - C ABI of libquasi_cuda.so, the GB300 (sm_103a) rendering backend.
 *
 * Part 1 declares the host<->plugin boundary that the unchanged Quasi host binds.
 * It mirrors, with the same member order, types and sizes:
 *   src/quasi/gpu/types.hpp:14-19   Q_gpu_backend (a uint32_t enum; CUDA is added as value 4)
 *   src/quasi/gpu/types.hpp:37-42   Q_gpu_context
 *   src/quasi/gpu/types.hpp:45-50   Q_camera
 *   src/quasi/gpu/types.hpp:63-70   Q_render_frame
 *   src/quasi/plugin/plugin_interface.hpp:27-92   handle, version, info, context, readback structs
 *   src/quasi/plugin/plugin_interface.hpp:107-148 the ten Q_plugin_* entry points
 * The host resolves these by name with dlsym (src/quasi/plugin/loader.hpp:72-128), so a
 * plugin built against this header is a drop-in for backends/metal/libquasi_metal.
 *
 * Part 2 declares CUDA-only extensions (Q_cuda_*). The reference host never looks them
 * up; tests, the benchmark and the autograd binding resolve them with dlsym/ctypes.
 * Every Q_cuda_* call returns an int status: QUASI_OK (0) or a negative QUASI_ERR_*.
 */
#ifndef QUASI_CUDA_H
#define QUASI_CUDA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define Q_CUDA_EXPORT __attribute__((visibility("default")))
#else
#define Q_CUDA_EXPORT
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ Part 1: plugin ABI */

/* Backend identifier. The reference declares `enum Q_gpu_backend : uint32_t` with values
 * 0..3 (src/quasi/gpu/types.hpp:14-19); the field stays 4 bytes, CUDA is value 4. */
typedef uint32_t Q_gpu_backend;
#define Q_GPU_BACKEND_NONE   0u
#define Q_GPU_BACKEND_METAL  1u
#define Q_GPU_BACKEND_VULKAN 2u
#define Q_GPU_BACKEND_WEBGPU 3u
#define Q_GPU_BACKEND_CUDA   4u

/* src/quasi/gpu/types.hpp:37-42. For CUDA: device = int* (device ordinal, NULL = 0),
 * queue = cudaStream_t (NULL = the plugin creates its own stream), layer = NULL. */
typedef struct Q_gpu_context {
    Q_gpu_backend backend;
    void* device;
    void* queue;
    void* layer;
} Q_gpu_context;

/* src/quasi/gpu/types.hpp:45-50 */
typedef struct Q_camera {
    float position[3];
    float target[3];
    float up[3];
    float fov; /* vertical field of view, degrees */
} Q_camera;

/* src/quasi/gpu/types.hpp:63-70. For CUDA: command_buffer = cudaStream_t to render on
 * (NULL = the plugin's stream); drawable = optional device buffer of width*height RGBA8
 * pixels that receives the tonemapped image (NULL = no display output, headless). */
typedef struct Q_render_frame {
    void* drawable;
    void* command_buffer;
    uint32_t width;
    uint32_t height;
    Q_camera camera;
    uint32_t camera_dirty;
} Q_render_frame;

/* src/quasi/plugin/plugin_interface.hpp:27 */
typedef struct Q_plugin_handle Q_plugin_handle;

/* src/quasi/plugin/plugin_interface.hpp:30-34 */
typedef struct Q_plugin_version {
    uint32_t major;
    uint32_t minor;
    uint32_t patch;
} Q_plugin_version;

/* src/quasi/plugin/plugin_interface.hpp:37-42 */
typedef struct Q_plugin_info {
    const char* name;
    Q_plugin_version version;
    const char* description;
    const char* author;
} Q_plugin_info;

/* src/quasi/plugin/plugin_interface.hpp:48-59 */
typedef struct Q_plugin_context {
    uint32_t viewport_width;
    uint32_t viewport_height;
    void* host_data;
    Q_gpu_context* gpu;
    void (*log)(void* host_data, const char* message);
    void (*request_shutdown)(void* host_data);
} Q_plugin_context;

/* src/quasi/plugin/plugin_interface.hpp:65-70. RGBA float, row-major, top row first. */
typedef struct Q_readback_result {
    float* data;
    uint32_t width;
    uint32_t height;
    uint32_t channels;
} Q_readback_result;

/* src/quasi/plugin/plugin_interface.hpp:73-79 (a uint32_t enum in the reference) */
typedef uint32_t Q_aov_type;
#define Q_AOV_BEAUTY 0u
#define Q_AOV_ALBEDO 1u
#define Q_AOV_NORMAL 2u
#define Q_AOV_DEPTH  3u
#define Q_AOV_COUNT  4u

/* src/quasi/plugin/plugin_interface.hpp:82-87 */
typedef struct Q_aov_buffer {
    float* data;
    uint32_t width;
    uint32_t height;
    uint32_t channels;
} Q_aov_buffer;

/* src/quasi/plugin/plugin_interface.hpp:90-92 */
typedef struct Q_readback_aov_result {
    Q_aov_buffer buffers[Q_AOV_COUNT];
} Q_readback_aov_result;

/* Replaces plugin_interface.hpp:108 / plugin.mm:543-545. Returns 3. */
Q_CUDA_EXPORT uint32_t Q_plugin_abi_version(void);
/* Replaces plugin_interface.hpp:111 / plugin.mm:547-554. Static strings. */
Q_CUDA_EXPORT Q_plugin_info Q_plugin_get_info(void);
/* Replaces plugin_interface.hpp:116 / plugin.mm:556-592. Returns NULL on failure after
 * logging through ctx->log; requires ctx->gpu->backend == Q_GPU_BACKEND_CUDA. */
Q_CUDA_EXPORT Q_plugin_handle* Q_plugin_create(Q_plugin_context* ctx);
/* Replaces plugin_interface.hpp:120 / plugin.mm:594-617. Synchronises and frees all. */
Q_CUDA_EXPORT void Q_plugin_destroy(Q_plugin_handle* handle);
/* Replaces plugin_interface.hpp:125 / plugin.mm:619-622 (no-op). */
Q_CUDA_EXPORT void Q_plugin_update(Q_plugin_handle* handle, float delta_time);
/* Replaces plugin_interface.hpp:130 / plugin.mm:624-792: one progressive frame. */
Q_CUDA_EXPORT void Q_plugin_render(Q_plugin_handle* handle, Q_render_frame* frame);
/* Replaces plugin_interface.hpp:135 / plugin.mm:846-863: malloc'd mean HDR image. */
Q_CUDA_EXPORT Q_readback_result Q_plugin_readback(Q_plugin_handle* handle);
/* Replaces plugin_interface.hpp:139 / plugin.mm:865-870. */
Q_CUDA_EXPORT void Q_plugin_readback_free(Q_readback_result* result);
/* Replaces plugin_interface.hpp:144 / plugin.mm:872-892: beauty, albedo, normal, depth. */
Q_CUDA_EXPORT Q_readback_aov_result Q_plugin_readback_aov(Q_plugin_handle* handle);
/* Replaces plugin_interface.hpp:148 / plugin.mm:894-902. */
Q_CUDA_EXPORT void Q_plugin_readback_aov_free(Q_readback_aov_result* result);

/* ------------------------------------------------------------ Part 2: CUDA extensions */

#define QUASI_OK              0
#define QUASI_ERR_INVALID    -1 /* bad argument or unsupported size */
#define QUASI_ERR_CUDA       -2 /* a CUDA runtime call failed */
#define QUASI_ERR_OOM        -3 /* device or host allocation failed */
#define QUASI_ERR_TIMEOUT    -4 /* a bounded device-side wait gave up */
#define QUASI_ERR_STACK      -5 /* BVH traversal stack would have overflowed */
#define QUASI_ERR_STATE      -6 /* call made in the wrong state (e.g. no scene) */

/* Integrators. NEE is the triangle/LBVH/next-event path tracer; REFERENCE reproduces the
 * Metal path_trace loop (plugin.mm:223-276) over quads, brute force, with its seeding. */
#define QUASI_INTEGRATOR_NEE       0u
#define QUASI_INTEGRATOR_REFERENCE 1u

/* A scene in host memory, triangles in original order. Arrays are owned by whoever
 * filled the struct (Q_cuda_make_scene allocates; Q_cuda_free_scene releases). */
typedef struct Q_cuda_scene {
    uint32_t tri_count;
    float* vertices;   /* tri_count * 9: v0.xyz v1.xyz v2.xyz */
    float* albedo;     /* tri_count * 3 */
    float* emission;   /* tri_count * 3 */
    uint32_t quad_count; /* reference-integrator primitives (may be 0) */
    float* quads;        /* quad_count * 9: origin.xyz u.xyz v.xyz (plugin.mm:57-64) */
    float* quad_albedo;  /* quad_count * 3 */
    float* quad_emission;/* quad_count * 3 */
    Q_camera camera;     /* the scene's own camera */
} Q_cuda_scene;

/* Render options; zero-initialise and set what you need. A zero field means default. */
typedef struct Q_cuda_options {
    uint32_t spp_per_frame;      /* samples per pixel per Q_plugin_render call (1) */
    uint32_t max_depth;          /* path vertices after the camera (4) */
    uint32_t seed;               /* RNG seed (0) */
    uint32_t integrator;         /* QUASI_INTEGRATOR_* */
    uint32_t rebuild_each_frame; /* rebuild the LBVH in every frame (1 = yes) */
    uint32_t wave_spp;           /* samples per pixel per wavefront (0 = as many as fit 2^27
                                    path slots, fewer if free device memory is short) */
    uint32_t trace_block;        /* threads per block of the trace kernels (0 = 256 over the 8-wide records, 128 binary) */
    uint32_t record_samples;     /* keep per-sample radiance and path signatures */
    uint32_t collect_stats;      /* count BVH node visits and triangle tests */
    uint32_t profile;            /* time every kernel launch with CUDA events */
    uint32_t megakernel;         /* 1 = one-kernel path tracer instead of the wavefront */
    uint32_t smem_levels;        /* binary LBVH only: top levels staged in shared memory per
                                    block (0 = default 5, 1..9, 32 = none) */
    float ray_eps;               /* ray origin offset along the normal (1e-4) */
    uint32_t refill_lanes;       /* trace kernels refill a warp once this many lanes idle
                                    (1..32; 32 = refill only whole warps; 0 = default:
                                    4 for the 8-wide records, 32 for the binary LBVH) */
    uint32_t trace_steps;        /* binary LBVH with refill only: node visits per lane
                                    between refill checks (0 = default) */
    uint32_t bvh_width;          /* traversal structure: 8 = 8-wide records collapsed from the
                                    LBVH (default, 0), 2 = the binary LBVH nodes */
    uint32_t bvh_cluster;        /* the LBVH's largest subtrees of at most this many leaves are
                                    rebuilt with the least surface-area split (0 = default 32;
                                    3..32; 1 or 2 = none: the plain Morton hierarchy) */
    uint32_t bvh_collapse;       /* children of the 8-wide records: 0 = the spread of least
                                    surface-area cost (default), 1 = the largest child opened
                                    greedily */
    uint32_t bvh_split;          /* percentage of the triangles whose boxes are split in two
                                    leaf references before the LBVH is built, the ones whose
                                    boxes leave the most surface area empty, in scenes of at
                                    least 131072 triangles (0 = default 30;
                                    1..100; QUASI_BVH_SPLIT_NONE = none: leaf i is the
                                    triangle at Morton position i, as the oracle builds it) */
} Q_cuda_options;

#define QUASI_BVH_SPLIT_NONE 0xFFFFFFFFu

/* Counters of the last frame (rays actually traced) and of the whole accumulation. */
typedef struct Q_cuda_stats {
    uint64_t camera_rays;
    uint64_t extension_rays;  /* closest-hit rays after the camera ray */
    uint64_t shadow_rays;
    uint64_t node_visits;     /* only with collect_stats: closest-hit traversal */
    uint64_t tri_tests;       /* only with collect_stats: closest-hit traversal */
    uint64_t shadow_node_visits; /* only with collect_stats: any-hit traversal */
    uint64_t shadow_tri_tests;   /* only with collect_stats: any-hit traversal */
    uint64_t total_rays;      /* all rays traced since the plugin was created */
    uint64_t samples_accumulated;
    uint32_t kernel_launches; /* kernels this library launched in the last frame */
    uint32_t error_flags;     /* device-side error bits (QUASI_DEVERR_*) */
    double frame_ms;          /* device time of the last frame (events on the stream) */
    double bvh_ms;            /* device time of the last LBVH build */
    uint64_t adjoint_rays;    /* rays replayed by Q_cuda_backward since the plugin was created */
    uint64_t redecided_rays;  /* rays of the last frame that met a triangle test the FP32 error
                                 bound could not decide: the fixup kernels re-decided their one
                                 undecided candidate in double-float, or re-traced the ray with
                                 exact decisions when it met several (wavefront form; 0
                                 otherwise) */
} Q_cuda_stats;

#define QUASI_DEVERR_STACK     1u
#define QUASI_DEVERR_TIMEOUT   2u
#define QUASI_DEVERR_TRAVERSAL 4u /* a traversal or tree climb exceeded its bound */

/* Per-kernel timing from the profile option (one entry per kernel name). */
typedef struct Q_cuda_kernel_time {
    char name[48];
    uint32_t launches;
    double total_ms;
} Q_cuda_kernel_time;

/* Builds one of the built-in scenes on the host (no GPU needed). spec is one of
 *   "cornell36"                 Cornell box of 36 triangles (unit box, camera looking +z)
 *   "refcornell"                src/quasi/scene/cornell_box.hpp:95-134 as 32 triangles + 16 quads
 *   "soup:n=<N>,seed=<S>"       seeded random triangle soup, 1% emitters
 * Returns QUASI_OK and fills *out; free with Q_cuda_free_scene. */
Q_CUDA_EXPORT int Q_cuda_make_scene(const char* spec, Q_cuda_scene* out);
Q_CUDA_EXPORT void Q_cuda_free_scene(Q_cuda_scene* scene);

/* Replaces the plugin's scene (copied to the device; the host arrays may be freed). */
Q_CUDA_EXPORT int Q_cuda_set_scene(Q_plugin_handle* handle, const Q_cuda_scene* scene);
/* Updates triangle vertices in place (same count); the next frame rebuilds the LBVH. */
Q_CUDA_EXPORT int Q_cuda_update_vertices(Q_plugin_handle* handle, const float* vertices,
                                         uint32_t tri_count);
/* Replaces per-triangle materials (host arrays, tri_count*3 each); resets accumulation. */
Q_CUDA_EXPORT int Q_cuda_set_materials(Q_plugin_handle* handle, const float* albedo,
                                       const float* emission, uint32_t tri_count);
Q_CUDA_EXPORT int Q_cuda_set_options(Q_plugin_handle* handle, const Q_cuda_options* options);
Q_CUDA_EXPORT int Q_cuda_get_options(Q_plugin_handle* handle, Q_cuda_options* options);
/* Clears the accumulation (next frame starts at sample 0). */
Q_CUDA_EXPORT int Q_cuda_reset(Q_plugin_handle* handle);
/* Waits for the plugin's stream; returns the first pending error, if any. */
Q_CUDA_EXPORT int Q_cuda_synchronize(Q_plugin_handle* handle);
Q_CUDA_EXPORT int Q_cuda_get_stats(Q_plugin_handle* handle, Q_cuda_stats* stats);
/* Copies up to capacity per-kernel timing entries; *count receives how many exist. */
Q_CUDA_EXPORT int Q_cuda_kernel_times(Q_plugin_handle* handle, Q_cuda_kernel_time* out,
                                      uint32_t capacity, uint32_t* count);
Q_CUDA_EXPORT const char* Q_cuda_last_error(Q_plugin_handle* handle);

/* Copies the current LBVH to host arrays (any pointer may be NULL). n = tri_count. Only
 * without split references (bvh_split = QUASI_BVH_SPLIT_NONE; QUASI_ERR_STATE otherwise), so
 * that its leaves are the triangles.
 *   morton    [n]        30-bit Morton code per triangle, original order
 *   order     [n]        original triangle index of each sorted position
 *   children  [2*(n-1)]  per internal node: child >= 0 internal node, child < 0 leaf ~pos
 *   boxes     [12*(n-1)] per internal node: child0 lo.xyz hi.xyz, child1 lo.xyz hi.xyz
 *   bounds    [6]        centroid bounds lo.xyz hi.xyz used for quantisation */
Q_CUDA_EXPORT int Q_cuda_read_bvh(Q_plugin_handle* handle, uint32_t* morton, uint32_t* order,
                                  int32_t* children, float* boxes, float* bounds);
/* Copies the 8-wide traversal records collapsed from the LBVH: 24 words (96 bytes) per
 * internal node (max(n - 1, 1) records; layout in csrc/wide.cuh); like Q_cuda_read_bvh, only
 * without split references. Record 0 is the root; only
 * records reachable from it through internal child references are used. No reference
 * counterpart: the reference traces by brute force (plugin.mm:199-212). */
Q_CUDA_EXPORT int Q_cuda_read_wide_bvh(Q_plugin_handle* handle, uint32_t* words);

/* With record_samples: copies the last frame's per-sample radiance (width*height*spp*3,
 * ordered pixel-major then sample) and path signatures (width*height*spp). */
Q_CUDA_EXPORT int Q_cuda_read_samples(Q_plugin_handle* handle, float* radiance,
                                      uint32_t* signatures);

/* Writes the mean HDR image (RGBA float) into a caller-provided device pointer. */
Q_CUDA_EXPORT int Q_cuda_resolve_device(Q_plugin_handle* handle, float* device_rgba);

/* Sorts n (key, value) pairs in place on the device with the library's LSD radix sort
 * (stable; keys compared as unsigned 32-bit over bits [0, key_bits)). Device pointers. */
Q_CUDA_EXPORT int Q_cuda_radix_sort_pairs(uint32_t* device_keys, uint32_t* device_values,
                                          uint32_t n, uint32_t key_bits, void* stream);

/* The same sort for callers that cannot let the library allocate device memory: a real-time
 * frame loop where cudaMalloc/cudaFree could synchronise the device mid-frame, or a host that
 * owns all device memory through its own pool. It has no counterpart in the reference.
 * Scratch comes from one fixed array in device memory that every GPU loading the library
 * holds until exit (QUASI_NOALLOC_SORT_SCRATCH_BYTES); the caller still owns keys and values.
 * Limits and behaviour:
 *  - n above QUASI_NOALLOC_SORT_MAX_KEYS returns QUASI_ERR_TOO_LARGE and touches nothing;
 *  - the first call on a device looks up the array's device address (cudaGetSymbolAddress,
 *    with that device current) and keeps it for the life of the process; make that first
 *    call before any stream capture, and do not reset the device's primary context
 *    (cudaDeviceReset) after it: the module would be reloaded and the kept address stale;
 *  - all calls share the one array and it keeps the last call's contents, so calls that
 *    overlap on the GPU (other streams, other threads) race; serialise them on one stream;
 *  - the sort is enqueued on `stream` and the function returns without waiting for it. */
#define QUASI_ERR_TOO_LARGE -7 /* input larger than a fixed-capacity entry point accepts */
#define QUASI_NOALLOC_SORT_MAX_KEYS 1048576u
#define QUASI_NOALLOC_SORT_SCRATCH_BYTES 8912896u /* 2 x 4 MiB key/value buffers + 512 KiB histograms */
Q_CUDA_EXPORT int Q_cuda_radix_sort_pairs_noalloc(uint32_t* device_keys, uint32_t* device_values,
                                                  uint32_t n, uint32_t key_bits, void* stream);

/* Replaces per-triangle materials from DEVICE arrays (tri_count*3 floats each; either may be
 * NULL to keep it) and resets accumulation. The set of emitters (triangles whose emission
 * was > 0 when the scene or host materials were last set) is kept. Used by optimisation
 * loops that update materials on the GPU every step. */
Q_CUDA_EXPORT int Q_cuda_set_materials_device(Q_plugin_handle* handle, const float* device_albedo,
                                              const float* device_emission, uint32_t tri_count);

/* Path-replay adjoint (no reference counterpart): for the current scene, camera, frame size
 * and options (NEE integrator, max_depth <= 16), replays samples [sample_base,
 * sample_base + spp) of every pixel from their RNG keys and writes
 *   device_grad_albedo[3*i+c]   = dLoss/d albedo_i,c
 *   device_grad_emission[3*i+c] = dLoss/d emission_i,c
 * where Loss depends on the image I = mean of those samples through
 * device_grad_image[3*(y*width+x)+c] = dLoss/dI(x,y,c) (top row first). All pointers are
 * device pointers; the call is asynchronous on `stream` (a cudaStream_t; NULL = the plugin's
 * stream; pass cudaStreamLegacy, (void*)1, for the legacy default stream). */
Q_CUDA_EXPORT int Q_cuda_backward(Q_plugin_handle* handle, const float* device_grad_image, uint32_t spp,
                                  uint32_t sample_base, float* device_grad_albedo,
                                  float* device_grad_emission, void* stream);

/* Runs the autotuner on the current scene, frame size and options: times short frames
 * (at most 8 spp) of each candidate form (wavefront or megakernel), wave size, trace block
 * size and refill threshold (8-wide records) or shared-memory treelet depth (binary LBVH),
 * keeps the fastest in the options (megakernel, wave_spp, trace_block, refill_lanes or
 * smem_levels) and resets the accumulation. Needs a previous render
 * (for the frame size). budget_ms bounds the time spent (0 = 2000 ms). */
Q_CUDA_EXPORT int Q_cuda_autotune(Q_plugin_handle* handle, double budget_ms);

/* ------------------------------------------------------------- Part 3: scene batches
 *
 * Many scenes of uneven size rendered together (no reference counterpart): every frame
 * renders spp samples of every pixel of every scene as one launch sequence over all of
 * them, fed from a device table of work items (runs of whole sample planes, packed into
 * waves of wave_paths path slots), captured once as a CUDA graph and replayed. Each
 * scene's image is bit-identical to rendering that scene alone through the plugin with the
 * same seed, depth and ray_eps. A batch belongs to the plugin handle it was created from
 * (same device, stream by default) and must be destroyed before that handle. */
typedef struct Q_cuda_batch Q_cuda_batch;

typedef struct Q_cuda_batch_scene {
    const Q_cuda_scene* scene; /* triangles, materials and camera (quads are ignored) */
    uint32_t width;
    uint32_t height;
    uint32_t spp;              /* samples per pixel per Q_cuda_batch_render */
} Q_cuda_batch_scene;

#define QUASI_BATCH_WAVEFRONT  0u
#define QUASI_BATCH_MEGAKERNEL 1u

/* Zero-initialise and set what you need; a zero field means default. */
typedef struct Q_cuda_batch_options {
    uint32_t max_depth;     /* path vertices after the camera (6) */
    uint32_t seed;          /* RNG seed, shared by all scenes (0) */
    uint32_t form;          /* QUASI_BATCH_WAVEFRONT (default) or QUASI_BATCH_MEGAKERNEL */
    uint32_t wave_paths;    /* path slots per wave (0 = 2^27, fewer if device memory is short; at most 2^27;
                               raised to the largest sample plane) */
    uint32_t trace_block;   /* threads per block of the persistent kernels (0 = 128) */
    uint32_t fetch_rays;    /* rays or paths a warp takes per atomic, multiple of 32 (0 = 32) */
    uint32_t use_graph;     /* 0 = default (graph), 1 = graph, 2 = plain launches */
    uint32_t collect_stats; /* count BVH node visits and triangle tests */
    float ray_eps;          /* ray origin offset along the normal (1e-4) */
    uint32_t bvh_width;     /* 8 = 8-wide traversal records (default, 0), 2 = binary LBVH */
    uint32_t refill_lanes;  /* 8-wide trace kernels refill a warp once this many lanes are
                               idle (1..32; 0 = default) */
} Q_cuda_batch_options;

typedef struct Q_cuda_batch_stats {
    uint64_t frames;            /* frames rendered since the last reset */
    uint64_t camera_rays;       /* per frame (fixed by the batch) */
    uint64_t closest_rays;      /* closest-hit rays (camera rays included), since the last reset */
    uint64_t shadow_rays;       /* since the last reset */
    uint64_t node_visits;       /* with collect_stats, since the last reset */
    uint64_t tri_tests;         /* with collect_stats, since the last reset */
    uint32_t scenes;
    uint32_t waves;             /* waves per frame */
    uint32_t kernels_per_frame; /* kernel launches (graph kernel nodes) per frame */
    uint32_t error_flags;       /* QUASI_DEVERR_* bits */
    uint64_t tri_total;         /* triangles of all scenes */
    uint64_t px_total;          /* pixels of all scenes (the batch image pool) */
    double frame_ms;            /* device time of the last frame */
    uint64_t adjoint_rays;      /* rays replayed by Q_cuda_batch_backward since the last reset */
    uint64_t redecided_rays;    /* rays with an undecided triangle test, re-decided by the
                                   fixup kernels as in Q_cuda_stats (wavefront form), since
                                   the last reset */
} Q_cuda_batch_stats;

/* Uploads the scenes and builds their LBVHs. *out receives the batch; on failure returns
 * an error (details in Q_cuda_last_error(handle)). */
Q_CUDA_EXPORT int Q_cuda_batch_create(Q_plugin_handle* handle, const Q_cuda_batch_scene* scenes, uint32_t count,
                                      const Q_cuda_batch_options* options, Q_cuda_batch** out);
Q_CUDA_EXPORT void Q_cuda_batch_destroy(Q_cuda_batch* batch);
/* Changes options (the next frame re-plans and re-captures); resets the accumulation. */
Q_CUDA_EXPORT int Q_cuda_batch_set_options(Q_cuda_batch* batch, const Q_cuda_batch_options* options);
Q_CUDA_EXPORT int Q_cuda_batch_get_options(Q_cuda_batch* batch, Q_cuda_batch_options* options);
/* Renders one frame of every scene on `stream` (NULL = the plugin's stream; (void*)1 =
 * cudaStreamLegacy); asynchronous. */
Q_CUDA_EXPORT int Q_cuda_batch_render(Q_cuda_batch* batch, void* stream);
/* Clears the accumulation of every scene (the next frame starts at sample 0). */
Q_CUDA_EXPORT int Q_cuda_batch_reset(Q_cuda_batch* batch);
/* Changes the RNG seed of every scene and clears the accumulation, on `stream` (NULL = the
 * plugin's stream): a device-side update of the scene table, so the captured frame and
 * adjoint graphs stay valid. An optimisation loop calls it once per step to draw new paths
 * (the target and the rendered image of a step then share the seed). */
Q_CUDA_EXPORT int Q_cuda_batch_set_seed(Q_cuda_batch* batch, uint32_t seed, void* stream);
/* Waits for the batch's work; returns QUASI_ERR_STACK / QUASI_ERR_TIMEOUT for device errors. */
Q_CUDA_EXPORT int Q_cuda_batch_synchronize(Q_cuda_batch* batch);
Q_CUDA_EXPORT int Q_cuda_batch_get_stats(Q_cuda_batch* batch, Q_cuda_batch_stats* stats);
/* Mean HDR image of scene `index` as host RGBA float (width*height*4, top row first). */
Q_CUDA_EXPORT int Q_cuda_batch_readback(Q_cuda_batch* batch, uint32_t index, float* host_rgba);
/* Mean HDR images of all scenes as device RGB float: scene after scene, 3 floats per pixel,
 * px_total pixels (the layout of the gradient image of Q_cuda_batch_backward). */
Q_CUDA_EXPORT int Q_cuda_batch_resolve_device(Q_cuda_batch* batch, float* device_rgb, void* stream);
/* Triangle and pixel offsets of scene `index` in the batch pools (either may be NULL). */
Q_CUDA_EXPORT int Q_cuda_batch_offsets(Q_cuda_batch* batch, uint32_t index, uint64_t* tri_offset,
                                       uint64_t* px_offset);
/* Replaces the materials of all scenes from DEVICE arrays (tri_total*3 floats each, scenes
 * back to back; either may be NULL to keep it) and resets the accumulation. */
Q_CUDA_EXPORT int Q_cuda_batch_set_materials_device(Q_cuda_batch* batch, const float* device_albedo,
                                                    const float* device_emission, void* stream);
/* Path-replay adjoint of the last frame of every scene: device_grad_image holds
 * dLoss/dI for every pixel of the batch image pool (layout of Q_cuda_batch_resolve_device);
 * gradients are written (not accumulated) to tri_total*3 floats each. Captured as a CUDA
 * graph like the frame. */
Q_CUDA_EXPORT int Q_cuda_batch_backward(Q_cuda_batch* batch, const float* device_grad_image,
                                        float* device_grad_albedo, float* device_grad_emission, void* stream);
/* Times frames of each candidate form, wave size, block size and fetch size (binary LBVH)
 * or refill threshold (8-wide records), keeps the fastest in the options, writes them to
 * *chosen (may be NULL) and resets the accumulation. The frames are the batch's own when
 * the search over them fits half of budget_ms, else capped at fewer samples per pixel (at
 * least 1). budget_ms bounds the time spent (0 = 5000 ms). */
Q_CUDA_EXPORT int Q_cuda_batch_autotune(Q_cuda_batch* batch, double budget_ms, Q_cuda_batch_options* chosen);
/* Message of the batch's last failed call (owned by the batch). */
Q_CUDA_EXPORT const char* Q_cuda_batch_last_error(Q_cuda_batch* batch);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* QUASI_CUDA_H */
