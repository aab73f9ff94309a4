"""Python host for libquasi_cuda.so, mirroring the reference's plugin loader.

`PluginHost` follows src/quasi/plugin/loader.hpp:65-137: it resolves the six required
Q_plugin_* symbols (symbol_not_found otherwise), checks the ABI version is in 1..3
(abi_mismatch), resolves the optional readback symbols, then calls Q_plugin_create
(create_failed on NULL). The CUDA-only Q_cuda_* calls are exposed as methods. There is no
CPU fallback: if the library is missing or a call fails, an exception says so.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from contextlib import contextmanager
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi as A

_PKG = Path(__file__).resolve().parent
DEFAULT_LIBRARY = _PKG / "_build" / "libquasi_cuda.so"


class LoaderError(RuntimeError):
    """Raised by PluginHost; `kind` is one of the reference loader's error codes."""

    def __init__(self, kind: str, message: str = ""):
        super().__init__(f"{kind}: {message}" if message else kind)
        self.kind = kind


class QuasiError(RuntimeError):
    def __init__(self, call: str, code: int, detail: str = ""):
        super().__init__(f"{call} failed with status {code}" + (f": {detail}" if detail else ""))
        self.code = code


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """dlopen()s the plugin library (RTLD_NOW | RTLD_LOCAL as dynamic_library.hpp:107)."""
    p = Path(path) if path else DEFAULT_LIBRARY
    if not p.exists():
        raise LoaderError("file_not_found", f"{p} is not built (run __graft_entry__.build())")
    try:
        lib = C.CDLL(str(p), mode=os.RTLD_NOW | os.RTLD_LOCAL)
    except OSError as e:
        raise LoaderError("load_failed", str(e)) from e
    for table in (A.REQUIRED_SYMBOLS, A.OPTIONAL_SYMBOLS, A.CUDA_SYMBOLS):
        for name, (res, args) in table.items():
            fn = getattr(lib, name, None)
            if fn is not None:
                fn.restype = res
                fn.argtypes = args
    return lib


@dataclass
class Scene:
    """A scene in host memory (original triangle order)."""

    vertices: np.ndarray            # (n, 9) float32
    albedo: np.ndarray              # (n, 3) float32
    emission: np.ndarray            # (n, 3) float32
    camera: dict = field(default_factory=dict)
    quads: np.ndarray | None = None         # (q, 9)
    quad_albedo: np.ndarray | None = None   # (q, 3)
    quad_emission: np.ndarray | None = None # (q, 3)

    @property
    def tri_count(self) -> int:
        return int(self.vertices.shape[0])

    def to_c(self) -> tuple[A.Q_cuda_scene, list]:
        keep = []

        def ptr(a):
            if a is None or a.size == 0:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_float))

        s = A.Q_cuda_scene()
        s.tri_count = self.tri_count
        s.vertices, s.albedo, s.emission = ptr(self.vertices), ptr(self.albedo), ptr(self.emission)
        q = 0 if self.quads is None else int(self.quads.shape[0])
        s.quad_count = q
        s.quads, s.quad_albedo, s.quad_emission = ptr(self.quads), ptr(self.quad_albedo), ptr(self.quad_emission)
        s.camera = make_camera(**self.camera) if self.camera else A.Q_camera()
        return s, keep


def make_camera(position, target, up=(0.0, 1.0, 0.0), fov=40.0) -> A.Q_camera:
    c = A.Q_camera()
    c.position[:] = [float(x) for x in position]
    c.target[:] = [float(x) for x in target]
    c.up[:] = [float(x) for x in up]
    c.fov = float(fov)
    return c


def camera_dict(c: A.Q_camera) -> dict:
    return {"position": tuple(c.position), "target": tuple(c.target), "up": tuple(c.up), "fov": float(c.fov)}


def make_scene(spec: str, lib: C.CDLL | None = None) -> Scene:
    """Builds a built-in scene on the host via Q_cuda_make_scene (no GPU needed)."""
    lib = lib or load_library()
    s = A.Q_cuda_scene()
    rc = lib.Q_cuda_make_scene(spec.encode(), C.byref(s))
    if rc != A.QUASI_OK:
        raise QuasiError("Q_cuda_make_scene", rc, spec)
    try:
        n, q = s.tri_count, s.quad_count

        def arr(p, count, width):
            if count == 0 or not p:
                return np.zeros((0, width), np.float32)
            return np.ctypeslib.as_array(p, shape=(count * width,)).reshape(count, width).copy()

        return Scene(arr(s.vertices, n, 9), arr(s.albedo, n, 3), arr(s.emission, n, 3), camera_dict(s.camera),
                     arr(s.quads, q, 9) if q else None, arr(s.quad_albedo, q, 3) if q else None,
                     arr(s.quad_emission, q, 3) if q else None)
    finally:
        lib.Q_cuda_free_scene(C.byref(s))


@contextmanager
def _env(overrides: dict | None):
    old = {}
    try:
        for k, v in (overrides or {}).items():
            old[k] = os.environ.get(k)
            os.environ[k] = str(v)
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


class PluginHost:
    """Loads the plugin like the reference host and drives it headless on one GPU."""

    def __init__(self, path=None, *, device: int = 0, stream: int | None = None, width: int = 256,
                 height: int = 256, backend: int = A.Q_GPU_BACKEND_CUDA, env: dict | None = None):
        self.lib = load_library(path)
        for name in A.REQUIRED_SYMBOLS:
            if getattr(self.lib, name, None) is None:
                raise LoaderError("symbol_not_found", name)
        abi = int(self.lib.Q_plugin_abi_version())
        if abi < 1 or abi > 3:
            raise LoaderError("abi_mismatch", str(abi))
        self.abi = abi
        self.logs: list[str] = []
        self._device = C.c_int(device)
        self._gpu = A.Q_gpu_context(backend, C.cast(C.pointer(self._device), C.c_void_p), stream, None)
        self._log_cb = A.LOG_FN(lambda _h, msg: self.logs.append(msg.decode(errors="replace")))
        self._shutdown_cb = A.SHUTDOWN_FN(lambda _h: None)
        self._ctx = A.Q_plugin_context(width, height, None, C.pointer(self._gpu), self._log_cb, self._shutdown_cb)
        with _env(env):
            h = self.lib.Q_plugin_create(C.byref(self._ctx))
        if not h:
            raise LoaderError("create_failed", "; ".join(self.logs))
        self.handle = C.c_void_p(h)
        self.width, self.height = width, height
        self.camera = None

    # -- lifecycle ---------------------------------------------------------------------
    def destroy(self) -> None:
        if getattr(self, "handle", None):
            self.lib.Q_plugin_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def info(self) -> dict:
        i = self.lib.Q_plugin_get_info()
        return {"name": i.name.decode(), "version": (i.version.major, i.version.minor, i.version.patch),
                "description": i.description.decode(), "author": i.author.decode()}

    def _check(self, call: str, rc: int) -> None:
        if rc != A.QUASI_OK:
            detail = self.lib.Q_cuda_last_error(self.handle)
            raise QuasiError(call, rc, detail.decode(errors="replace") if detail else "")

    # -- plugin ABI ----------------------------------------------------------------------
    def render(self, width: int | None = None, height: int | None = None, camera=None, dirty: bool = False,
               stream: int | None = None, drawable: int | None = None) -> None:
        f = A.Q_render_frame()
        f.drawable = drawable
        f.command_buffer = stream
        f.width = width or self.width
        f.height = height or self.height
        if camera is not None:
            self.camera = camera if isinstance(camera, A.Q_camera) else make_camera(**camera)
        if self.camera is None:
            raise ValueError("no camera: pass camera= or call set_scene() first")
        f.camera = self.camera
        f.camera_dirty = 1 if dirty else 0
        self.width, self.height = f.width, f.height
        self.lib.Q_plugin_render(self.handle, C.byref(f))
        err = self.lib.Q_cuda_last_error(self.handle)
        if err:
            msg = err.decode(errors="replace")
            if msg:
                raise QuasiError("Q_plugin_render", A.QUASI_ERR_CUDA, msg)

    def readback(self) -> np.ndarray:
        """The mean beauty image as an (H, W, 4) float32 array over the plugin's own buffer
        (no copy): Q_plugin_readback_free runs when the array is garbage-collected."""
        r = self.lib.Q_plugin_readback(self.handle)
        if not r.data:
            raise QuasiError("Q_plugin_readback", A.QUASI_ERR_STATE, "no data")
        try:
            arr = np.ctypeslib.as_array(r.data, shape=(r.height, r.width, r.channels))
        except BaseException:
            self.lib.Q_plugin_readback_free(C.byref(r))
            raise
        weakref.finalize(arr, self.lib.Q_plugin_readback_free, C.byref(r))
        return arr

    def readback_aov(self) -> dict[str, np.ndarray]:
        r = self.lib.Q_plugin_readback_aov(self.handle)
        try:
            out = {}
            for i, name in enumerate(("beauty", "albedo", "normal", "depth")):
                b = r.buffers[i]
                if not b.data:
                    raise QuasiError("Q_plugin_readback_aov", A.QUASI_ERR_STATE, f"no {name}")
                out[name] = np.ctypeslib.as_array(b.data, shape=(b.height, b.width, b.channels)).copy()
            return out
        finally:
            self.lib.Q_plugin_readback_aov_free(C.byref(r))

    # -- CUDA extensions -----------------------------------------------------------------
    def set_scene(self, scene: Scene, use_camera: bool = True) -> None:
        s, keep = scene.to_c()
        self._check("Q_cuda_set_scene", self.lib.Q_cuda_set_scene(self.handle, C.byref(s)))
        del keep
        if use_camera and scene.camera:
            self.camera = make_camera(**scene.camera)

    def update_vertices(self, vertices_ptr: int, tri_count: int) -> None:
        self._check("Q_cuda_update_vertices", self.lib.Q_cuda_update_vertices(self.handle, vertices_ptr, tri_count))

    def set_materials(self, albedo: np.ndarray, emission: np.ndarray) -> None:
        a = np.ascontiguousarray(albedo, np.float32)
        e = np.ascontiguousarray(emission, np.float32)
        self._check("Q_cuda_set_materials",
                    self.lib.Q_cuda_set_materials(self.handle, a.ctypes.data, e.ctypes.data, a.shape[0]))

    def options(self) -> A.Q_cuda_options:
        o = A.Q_cuda_options()
        self._check("Q_cuda_get_options", self.lib.Q_cuda_get_options(self.handle, C.byref(o)))
        return o

    def set_options(self, **kw) -> None:
        o = self.options()
        for k, v in kw.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        self._check("Q_cuda_set_options", self.lib.Q_cuda_set_options(self.handle, C.byref(o)))

    def reset(self) -> None:
        self._check("Q_cuda_reset", self.lib.Q_cuda_reset(self.handle))

    def synchronize(self) -> None:
        self._check("Q_cuda_synchronize", self.lib.Q_cuda_synchronize(self.handle))

    def stats(self) -> A.Q_cuda_stats:
        s = A.Q_cuda_stats()
        self._check("Q_cuda_get_stats", self.lib.Q_cuda_get_stats(self.handle, C.byref(s)))
        return s

    def kernel_times(self, reset: bool = False) -> dict[str, tuple[int, float]]:
        n = C.c_uint32(0)
        self._check("Q_cuda_kernel_times", self.lib.Q_cuda_kernel_times(self.handle, None, 0, C.byref(n)))
        buf = (A.Q_cuda_kernel_time * max(n.value, 1))()
        self._check("Q_cuda_kernel_times", self.lib.Q_cuda_kernel_times(self.handle, buf, n.value, C.byref(n)))
        out = {buf[i].name.decode(): (int(buf[i].launches), float(buf[i].total_ms)) for i in range(n.value)}
        if reset:
            self._check("Q_cuda_kernel_times", self.lib.Q_cuda_kernel_times(self.handle, None, 0, None))
        return out

    def read_bvh(self, n: int) -> dict[str, np.ndarray]:
        nodes = max(n - 1, 1)
        morton = np.zeros(n, np.uint32)
        order = np.zeros(n, np.uint32)
        children = np.zeros(2 * nodes, np.int32)
        boxes = np.zeros(12 * nodes, np.float32)
        bounds = np.zeros(6, np.float32)
        self._check("Q_cuda_read_bvh", self.lib.Q_cuda_read_bvh(self.handle, morton.ctypes.data, order.ctypes.data,
                                                                children.ctypes.data, boxes.ctypes.data,
                                                                bounds.ctypes.data))
        return {"morton": morton, "order": order, "children": children, "boxes": boxes, "bounds": bounds}

    def read_wide_bvh(self, n: int) -> np.ndarray:
        """The 8-wide traversal records, (max(n - 1, 1), 24) uint32."""
        words = np.zeros((max(n - 1, 1), 24), np.uint32)
        self._check("Q_cuda_read_wide_bvh", self.lib.Q_cuda_read_wide_bvh(self.handle, words.ctypes.data))
        return words

    def read_samples(self, spp: int) -> tuple[np.ndarray, np.ndarray]:
        n = self.width * self.height * spp
        rad = np.zeros(3 * n, np.float32)
        sig = np.zeros(n, np.uint32)
        self._check("Q_cuda_read_samples", self.lib.Q_cuda_read_samples(self.handle, rad.ctypes.data, sig.ctypes.data))
        return rad.reshape(self.height, self.width, spp, 3), sig.reshape(self.height, self.width, spp)

    def resolve_device(self, device_ptr: int) -> None:
        self._check("Q_cuda_resolve_device", self.lib.Q_cuda_resolve_device(self.handle, device_ptr))

    def autotune(self, budget_ms: float = 2000.0) -> None:
        self._check("Q_cuda_autotune", self.lib.Q_cuda_autotune(self.handle, budget_ms))


class Batch:
    """A set of scenes rendered together (Q_cuda_batch_*), owned by a PluginHost.

    scenes: list of (Scene, width, height, spp). Each frame renders spp samples of every
    pixel of every scene; images are bit-identical to rendering each scene alone with the
    same seed, depth and ray_eps.
    """

    def __init__(self, host: PluginHost, scenes, **options):
        self.host = host
        self.lib = host.lib
        self.sizes = [(int(w), int(h), int(spp)) for _, w, h, spp in scenes]
        self._keep = []
        cs = []
        for sc, w, h, spp in scenes:
            c, keep = sc.to_c()
            self._keep.append((c, keep))
            cs.append(c)
        arr = (A.Q_cuda_batch_scene * len(cs))()
        for i, (c, (w, h, spp)) in enumerate(zip(cs, self.sizes)):
            arr[i].scene = C.pointer(c)
            arr[i].width, arr[i].height, arr[i].spp = w, h, spp
        o = A.Q_cuda_batch_options()
        for k, v in options.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        out = C.c_void_p()
        rc = self.lib.Q_cuda_batch_create(host.handle, arr, len(cs), C.byref(o), C.byref(out))
        host._check("Q_cuda_batch_create", rc)
        self._keep = None  # the batch copied the scenes
        self.handle = out
        self.tri_counts = [sc.tri_count for sc, *_ in scenes]

    def destroy(self) -> None:
        if getattr(self, "handle", None):
            self.lib.Q_cuda_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def _check(self, call: str, rc: int) -> None:
        if rc != A.QUASI_OK:
            detail = self.lib.Q_cuda_batch_last_error(self.handle)
            raise QuasiError(call, rc, detail.decode(errors="replace") if detail else "")

    def options(self) -> A.Q_cuda_batch_options:
        o = A.Q_cuda_batch_options()
        self._check("Q_cuda_batch_get_options", self.lib.Q_cuda_batch_get_options(self.handle, C.byref(o)))
        return o

    def set_options(self, **kw) -> None:
        o = self.options()
        for k, v in kw.items():
            if not hasattr(o, k):
                raise AttributeError(k)
            setattr(o, k, v)
        self._check("Q_cuda_batch_set_options", self.lib.Q_cuda_batch_set_options(self.handle, C.byref(o)))

    def render(self, stream: int | None = None) -> None:
        self._check("Q_cuda_batch_render", self.lib.Q_cuda_batch_render(self.handle, stream))

    def reset(self) -> None:
        self._check("Q_cuda_batch_reset", self.lib.Q_cuda_batch_reset(self.handle))

    def set_seed(self, seed: int, stream: int | None = None) -> None:
        """New RNG seed for every scene (device-side; the captured graphs stay valid)."""
        self._check("Q_cuda_batch_set_seed", self.lib.Q_cuda_batch_set_seed(self.handle, seed, stream))

    def synchronize(self) -> None:
        self._check("Q_cuda_batch_synchronize", self.lib.Q_cuda_batch_synchronize(self.handle))

    def stats(self) -> A.Q_cuda_batch_stats:
        s = A.Q_cuda_batch_stats()
        self._check("Q_cuda_batch_get_stats", self.lib.Q_cuda_batch_get_stats(self.handle, C.byref(s)))
        return s

    def readback(self, index: int) -> np.ndarray:
        w, h, _ = self.sizes[index]
        out = np.zeros((h, w, 4), np.float32)
        self._check("Q_cuda_batch_readback", self.lib.Q_cuda_batch_readback(self.handle, index, out.ctypes.data))
        return out

    def offsets(self, index: int) -> tuple[int, int]:
        t, p = C.c_uint64(), C.c_uint64()
        self._check("Q_cuda_batch_offsets", self.lib.Q_cuda_batch_offsets(self.handle, index, C.byref(t), C.byref(p)))
        return int(t.value), int(p.value)

    def resolve_device(self, device_rgb: int, stream: int | None = None) -> None:
        self._check("Q_cuda_batch_resolve_device", self.lib.Q_cuda_batch_resolve_device(self.handle, device_rgb, stream))

    def set_materials_device(self, albedo_ptr: int | None, emission_ptr: int | None, stream: int | None = None) -> None:
        self._check("Q_cuda_batch_set_materials_device",
                    self.lib.Q_cuda_batch_set_materials_device(self.handle, albedo_ptr, emission_ptr, stream))

    def backward(self, grad_image_ptr: int, grad_albedo_ptr: int | None, grad_emission_ptr: int | None,
                 stream: int | None = None) -> None:
        self._check("Q_cuda_batch_backward", self.lib.Q_cuda_batch_backward(self.handle, grad_image_ptr,
                                                                            grad_albedo_ptr, grad_emission_ptr,
                                                                            stream))

    def autotune(self, budget_ms: float = 5000.0) -> A.Q_cuda_batch_options:
        o = A.Q_cuda_batch_options()
        self._check("Q_cuda_batch_autotune", self.lib.Q_cuda_batch_autotune(self.handle, budget_ms, C.byref(o)))
        return o
