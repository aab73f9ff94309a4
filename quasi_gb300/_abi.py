"""ctypes mirrors of include/quasi_cuda.h (the plugin ABI and the Q_cuda_* extensions).

Layouts follow src/quasi/gpu/types.hpp:37-70 and src/quasi/plugin/plugin_interface.hpp:30-92
member for member; a test checks the sizes against the C compiler's view.
"""
from __future__ import annotations

import ctypes as C

Q_GPU_BACKEND_NONE = 0
Q_GPU_BACKEND_METAL = 1
Q_GPU_BACKEND_VULKAN = 2
Q_GPU_BACKEND_WEBGPU = 3
Q_GPU_BACKEND_CUDA = 4

Q_AOV_BEAUTY, Q_AOV_ALBEDO, Q_AOV_NORMAL, Q_AOV_DEPTH, Q_AOV_COUNT = 0, 1, 2, 3, 4

QUASI_OK = 0
QUASI_ERR_INVALID = -1
QUASI_ERR_CUDA = -2
QUASI_ERR_OOM = -3
QUASI_ERR_TIMEOUT = -4
QUASI_ERR_STACK = -5
QUASI_ERR_STATE = -6
QUASI_ERR_TOO_LARGE = -7

QUASI_INTEGRATOR_NEE = 0
QUASI_INTEGRATOR_REFERENCE = 1

QUASI_BVH_SPLIT_NONE = 0xFFFFFFFF

QUASI_DEVERR_STACK = 1
QUASI_DEVERR_TIMEOUT = 2
QUASI_DEVERR_TRAVERSAL = 4

QUASI_BATCH_WAVEFRONT = 0
QUASI_BATCH_MEGAKERNEL = 1


class Q_gpu_context(C.Structure):
    _fields_ = [("backend", C.c_uint32), ("device", C.c_void_p), ("queue", C.c_void_p), ("layer", C.c_void_p)]


class Q_camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float)]


class Q_render_frame(C.Structure):
    _fields_ = [("drawable", C.c_void_p), ("command_buffer", C.c_void_p), ("width", C.c_uint32),
                ("height", C.c_uint32), ("camera", Q_camera), ("camera_dirty", C.c_uint32)]


class Q_plugin_version(C.Structure):
    _fields_ = [("major", C.c_uint32), ("minor", C.c_uint32), ("patch", C.c_uint32)]


class Q_plugin_info(C.Structure):
    _fields_ = [("name", C.c_char_p), ("version", Q_plugin_version), ("description", C.c_char_p),
                ("author", C.c_char_p)]


LOG_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p)
SHUTDOWN_FN = C.CFUNCTYPE(None, C.c_void_p)


class Q_plugin_context(C.Structure):
    _fields_ = [("viewport_width", C.c_uint32), ("viewport_height", C.c_uint32), ("host_data", C.c_void_p),
                ("gpu", C.POINTER(Q_gpu_context)), ("log", LOG_FN), ("request_shutdown", SHUTDOWN_FN)]


class Q_readback_result(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_float)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("channels", C.c_uint32)]


class Q_aov_buffer(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_float)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("channels", C.c_uint32)]


class Q_readback_aov_result(C.Structure):
    _fields_ = [("buffers", Q_aov_buffer * Q_AOV_COUNT)]


class Q_cuda_scene(C.Structure):
    _fields_ = [("tri_count", C.c_uint32), ("vertices", C.POINTER(C.c_float)), ("albedo", C.POINTER(C.c_float)),
                ("emission", C.POINTER(C.c_float)), ("quad_count", C.c_uint32), ("quads", C.POINTER(C.c_float)),
                ("quad_albedo", C.POINTER(C.c_float)), ("quad_emission", C.POINTER(C.c_float)),
                ("camera", Q_camera)]


class Q_cuda_options(C.Structure):
    _fields_ = [("spp_per_frame", C.c_uint32), ("max_depth", C.c_uint32), ("seed", C.c_uint32),
                ("integrator", C.c_uint32), ("rebuild_each_frame", C.c_uint32), ("wave_spp", C.c_uint32),
                ("trace_block", C.c_uint32), ("record_samples", C.c_uint32), ("collect_stats", C.c_uint32),
                ("profile", C.c_uint32), ("megakernel", C.c_uint32), ("smem_levels", C.c_uint32),
                ("ray_eps", C.c_float), ("refill_lanes", C.c_uint32), ("trace_steps", C.c_uint32),
                ("bvh_width", C.c_uint32), ("bvh_cluster", C.c_uint32), ("bvh_collapse", C.c_uint32),
                ("bvh_split", C.c_uint32)]


class Q_cuda_stats(C.Structure):
    _fields_ = [("camera_rays", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64), ("shadow_node_visits", C.c_uint64),
                ("shadow_tri_tests", C.c_uint64), ("total_rays", C.c_uint64), ("samples_accumulated", C.c_uint64),
                ("kernel_launches", C.c_uint32), ("error_flags", C.c_uint32), ("frame_ms", C.c_double),
                ("bvh_ms", C.c_double), ("adjoint_rays", C.c_uint64), ("redecided_rays", C.c_uint64)]

    @property
    def rays(self) -> int:
        return self.camera_rays + self.extension_rays + self.shadow_rays


class Q_cuda_kernel_time(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("total_ms", C.c_double)]


class Q_cuda_batch_scene(C.Structure):
    _fields_ = [("scene", C.POINTER(Q_cuda_scene)), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp", C.c_uint32)]


class Q_cuda_batch_options(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("seed", C.c_uint32), ("form", C.c_uint32), ("wave_paths", C.c_uint32),
                ("trace_block", C.c_uint32), ("fetch_rays", C.c_uint32), ("use_graph", C.c_uint32),
                ("collect_stats", C.c_uint32), ("ray_eps", C.c_float), ("bvh_width", C.c_uint32),
                ("refill_lanes", C.c_uint32)]


class Q_cuda_batch_stats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("camera_rays", C.c_uint64), ("closest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64),
                ("scenes", C.c_uint32), ("waves", C.c_uint32), ("kernels_per_frame", C.c_uint32),
                ("error_flags", C.c_uint32), ("tri_total", C.c_uint64), ("px_total", C.c_uint64),
                ("frame_ms", C.c_double), ("adjoint_rays", C.c_uint64), ("redecided_rays", C.c_uint64)]

    @property
    def rays(self) -> int:
        """Rays traced since the last reset (closest-hit, camera included, plus shadow)."""
        return self.closest_rays + self.shadow_rays


# Symbol table: name -> (restype, argtypes). Required/optional split follows
# src/quasi/plugin/loader.hpp:72-128.
REQUIRED_SYMBOLS = {
    "Q_plugin_abi_version": (C.c_uint32, []),
    "Q_plugin_get_info": (Q_plugin_info, []),
    "Q_plugin_create": (C.c_void_p, [C.POINTER(Q_plugin_context)]),
    "Q_plugin_destroy": (None, [C.c_void_p]),
    "Q_plugin_update": (None, [C.c_void_p, C.c_float]),
    "Q_plugin_render": (None, [C.c_void_p, C.POINTER(Q_render_frame)]),
}
OPTIONAL_SYMBOLS = {
    "Q_plugin_readback": (Q_readback_result, [C.c_void_p]),
    "Q_plugin_readback_free": (None, [C.POINTER(Q_readback_result)]),
    "Q_plugin_readback_aov": (Q_readback_aov_result, [C.c_void_p]),
    "Q_plugin_readback_aov_free": (None, [C.POINTER(Q_readback_aov_result)]),
}
CUDA_SYMBOLS = {
    "Q_cuda_make_scene": (C.c_int, [C.c_char_p, C.POINTER(Q_cuda_scene)]),
    "Q_cuda_free_scene": (None, [C.POINTER(Q_cuda_scene)]),
    "Q_cuda_set_scene": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_scene)]),
    "Q_cuda_update_vertices": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "Q_cuda_set_materials": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]),
    "Q_cuda_set_options": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_options)]),
    "Q_cuda_get_options": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_options)]),
    "Q_cuda_reset": (C.c_int, [C.c_void_p]),
    "Q_cuda_synchronize": (C.c_int, [C.c_void_p]),
    "Q_cuda_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_stats)]),
    "Q_cuda_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_kernel_time), C.c_uint32,
                                      C.POINTER(C.c_uint32)]),
    "Q_cuda_last_error": (C.c_char_p, [C.c_void_p]),
    "Q_cuda_read_bvh": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "Q_cuda_read_wide_bvh": (C.c_int, [C.c_void_p, C.c_void_p]),
    "Q_cuda_read_samples": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "Q_cuda_resolve_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "Q_cuda_radix_sort_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    "Q_cuda_radix_sort_pairs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    "Q_cuda_autotune": (C.c_int, [C.c_void_p, C.c_double]),
    "Q_cuda_set_materials_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]),
    "Q_cuda_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "Q_cuda_batch_create": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_batch_scene), C.c_uint32,
                                      C.POINTER(Q_cuda_batch_options), C.POINTER(C.c_void_p)]),
    "Q_cuda_batch_destroy": (None, [C.c_void_p]),
    "Q_cuda_batch_set_options": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_batch_options)]),
    "Q_cuda_batch_get_options": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_batch_options)]),
    "Q_cuda_batch_render": (C.c_int, [C.c_void_p, C.c_void_p]),
    "Q_cuda_batch_reset": (C.c_int, [C.c_void_p]),
    "Q_cuda_batch_set_seed": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "Q_cuda_batch_synchronize": (C.c_int, [C.c_void_p]),
    "Q_cuda_batch_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Q_cuda_batch_stats)]),
    "Q_cuda_batch_readback": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "Q_cuda_batch_resolve_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "Q_cuda_batch_offsets": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "Q_cuda_batch_set_materials_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "Q_cuda_batch_backward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "Q_cuda_batch_autotune": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(Q_cuda_batch_options)]),
    "Q_cuda_batch_last_error": (C.c_char_p, [C.c_void_p]),
}
