"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so). TEST INFRASTRUCTURE ONLY.

Imported by the tests, by __graft_entry__.smoke() and by bench.py's CPU baseline / reference
leg, always as the checker or the timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_lib = None


class OracleConfig(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32), ("sample_base", C.c_uint32),
                ("max_depth", C.c_uint32), ("seed", C.c_uint32), ("cam_pos", C.c_float * 3),
                ("cam_target", C.c_float * 3), ("cam_up", C.c_float * 3), ("cam_fov", C.c_float),
                ("ray_eps", C.c_float), ("precision", C.c_uint32), ("threads", C.c_uint32)]


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "oracle.cpp").stat().st_mtime:
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.oracle_pcg_hash.restype = C.c_uint32
        L.oracle_pcg_hash.argtypes = [C.c_uint32]
        L.oracle_random_float.restype = C.c_float
        L.oracle_random_float.argtypes = [C.POINTER(C.c_uint32)]
        L.oracle_path_key.restype = C.c_uint32
        L.oracle_path_key.argtypes = [C.c_uint32] * 4
        L.oracle_cosine_sample.argtypes = [P, C.c_float, C.c_float, P]
        L.oracle_camera_dir.argtypes = [P, P, P, C.c_float, C.c_uint32, C.c_uint32, C.c_double, C.c_double, P]
        L.oracle_ref_camera_ray.argtypes = [P, P, P, C.c_float, C.c_float, C.c_double, C.c_double,
                                            C.POINTER(C.c_uint32), P, P]
        L.oracle_intersect_quad.restype = C.c_int
        L.oracle_intersect_quad.argtypes = [P, P, P, C.c_double, C.c_double, P, P, P]
        L.oracle_lbvh.restype = C.c_int
        L.oracle_lbvh.argtypes = [C.c_uint32, P, P, P, P, P, P]
        L.oracle_collapse8.restype = C.c_int
        L.oracle_collapse8.argtypes = [C.c_uint32, P, P]
        L.oracle_render_nee.restype = C.c_int
        L.oracle_render_nee.argtypes = [C.c_uint32, P, P, P, C.POINTER(OracleConfig), P, C.c_uint32, P, P, P, P, P]
        L.oracle_render_reference.restype = C.c_int
        L.oracle_render_reference.argtypes = [C.c_uint32, P, P, P, C.POINTER(OracleConfig), P, P]
        L.oracle_hardware_threads.restype = C.c_uint32
        L.oracle_backward.restype = C.c_int
        L.oracle_backward.argtypes = [C.c_uint32, P, P, P, C.POINTER(OracleConfig), P, P, P]
        L.oracle_make_scene.restype = C.c_int
        L.oracle_make_scene.argtypes = [C.c_char_p, C.POINTER(C.c_uint32), C.POINTER(C.POINTER(C.c_float)),
                                        C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.POINTER(C.c_float)), P]
        L.oracle_free.argtypes = [P]
        L.oracle_soup_centres.restype = C.c_int
        L.oracle_soup_centres.argtypes = [C.c_uint32, C.c_uint64, P]
        _lib = L
    return _lib


class OracleScene:
    """A scene built by the oracle's own generators: vertices (n, 9), albedo and emission
    (n, 3) float32 and the camera (position, target, up, fov), the fields the oracle's render
    functions read."""

    def __init__(self, vertices, albedo, emission, camera):
        self.vertices, self.albedo, self.emission, self.camera = vertices, albedo, emission, camera

    @property
    def tri_count(self) -> int:
        return int(self.vertices.shape[0])


def make_scene(spec: str) -> OracleScene:
    """The benchmark scenes "cornell36" and "soup:n=N,seed=S" from the oracle's restatement of
    the library's generators (bit-identical to Q_cuda_make_scene), without the product."""
    n = C.c_uint32(0)
    pv, pa, pe = C.POINTER(C.c_float)(), C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
    cam = np.zeros(10, np.float32)
    rc = lib().oracle_make_scene(spec.encode(), C.byref(n), C.byref(pv), C.byref(pa), C.byref(pe), cam.ctypes.data)
    if rc:
        raise ValueError(f"oracle_make_scene: unknown spec {spec!r}")
    try:
        k = int(n.value)

        def arr(p, width):
            return np.ctypeslib.as_array(p, shape=(k * width,)).reshape(k, width).copy()

        v, a, e = arr(pv, 9), arr(pa, 3), arr(pe, 3)
    finally:
        for ptr in (pv, pa, pe):
            lib().oracle_free(C.cast(ptr, C.c_void_p))
    camera = {"position": tuple(float(x) for x in cam[0:3]), "target": tuple(float(x) for x in cam[3:6]),
              "up": tuple(float(x) for x in cam[6:9]), "fov": float(cam[9])}
    return OracleScene(v, a, e, camera)


def soup_centres(n: int, seed: int) -> np.ndarray:
    """The (n, 3) centres the soup generator draws for "soup:n=N,seed=S"."""
    out = np.zeros((n, 3), np.float64)
    if lib().oracle_soup_centres(n, seed, out.ctypes.data):
        raise ValueError("oracle_soup_centres")
    return out


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def hardware_threads() -> int:
    return int(lib().oracle_hardware_threads())


def pcg_hash(x: int) -> int:
    return int(lib().oracle_pcg_hash(x & 0xFFFFFFFF))


def random_floats(seed: int, count: int) -> tuple[list[float], int]:
    st = C.c_uint32(seed)
    vals = [float(lib().oracle_random_float(C.byref(st))) for _ in range(count)]
    return vals, int(st.value)


def path_key(seed: int, pixel: int, sample: int, bounce: int) -> int:
    return int(lib().oracle_path_key(seed, pixel, sample, bounce))


def cosine_sample(normal, r1: float, r2: float) -> np.ndarray:
    n = np.ascontiguousarray(normal, np.float64)
    out = np.zeros(3, np.float64)
    lib().oracle_cosine_sample(n.ctypes.data, r1, r2, out.ctypes.data)
    return out


def camera_dir(pos, target, up, fov, width, height, u, v) -> np.ndarray:
    p, t, w = _f32(pos), _f32(target), _f32(up)
    out = np.zeros(3, np.float64)
    lib().oracle_camera_dir(p.ctypes.data, t.ctypes.data, w.ctypes.data, fov, width, height, u, v, out.ctypes.data)
    return out


def ref_camera_ray(pos, direction, up, fov, aspect, ux, uy, state: int):
    p, d, u = _f32(pos), _f32(direction), _f32(up)
    st = C.c_uint32(state)
    o = np.zeros(3, np.float64)
    dd = np.zeros(3, np.float64)
    lib().oracle_ref_camera_ray(p.ctypes.data, d.ctypes.data, u.ctypes.data, fov, aspect, ux, uy, C.byref(st),
                                o.ctypes.data, dd.ctypes.data)
    return o, dd, int(st.value)


def intersect_quad(ro, rd, quad, tmin=0.001, tmax=1e30):
    ro = np.ascontiguousarray(ro, np.float64)
    rd = np.ascontiguousarray(rd, np.float64)
    q = _f32(quad)
    t = np.zeros(1, np.float64)
    p = np.zeros(3, np.float64)
    n = np.zeros(3, np.float64)
    hit = lib().oracle_intersect_quad(ro.ctypes.data, rd.ctypes.data, q.ctypes.data, tmin, tmax, t.ctypes.data,
                                      p.ctypes.data, n.ctypes.data)
    return (float(t[0]), p, n) if hit else None


def lbvh(vertices: np.ndarray) -> dict[str, np.ndarray]:
    v = _f32(vertices).reshape(-1, 9)
    n = v.shape[0]
    nodes = max(n - 1, 1)
    out = {"morton": np.zeros(n, np.uint32), "order": np.zeros(n, np.uint32),
           "children": np.zeros(2 * nodes, np.int32), "boxes": np.zeros(12 * nodes, np.float32),
           "bounds": np.zeros(6, np.float32)}
    rc = lib().oracle_lbvh(n, v.ctypes.data, *(out[k].ctypes.data for k in ("morton", "order", "children", "boxes",
                                                                          "bounds")))
    if rc:
        raise RuntimeError(f"oracle_lbvh failed: {rc}")
    return out


def collapse8(vertices: np.ndarray) -> np.ndarray:
    """8-wide traversal records of the LBVH, (max(n - 1, 1), 24) uint32 (n = 0: empty)."""
    v = _f32(vertices).reshape(-1, 9)
    n = v.shape[0]
    out = np.zeros((max(n - 1, 1) if n else 0, 24), np.uint32)
    rc = lib().oracle_collapse8(n, v.ctypes.data, out.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_collapse8 failed: {rc}")
    return out


def wide_reachable(words: np.ndarray) -> list[int]:
    """Indices of the 8-wide records reachable from record 0 through internal references."""
    if words.shape[0] == 0:
        return []
    refs = words[:, 16:24].view(np.int32)
    imask = words[:, 3] >> 24
    seen, todo = [], [0]
    while todo:
        i = todo.pop()
        seen.append(i)
        for s in range(8):
            if (int(imask[i]) >> s) & 1:
                todo.append(int(refs[i, s]))
    return sorted(seen)


def _config(width, height, spp, depth, seed, camera, precision, threads, sample_base, eps) -> OracleConfig:
    c = OracleConfig()
    c.width, c.height, c.spp, c.sample_base, c.max_depth, c.seed = width, height, spp, sample_base, depth, seed
    c.cam_pos[:] = list(camera["position"])
    c.cam_target[:] = list(camera["target"])
    c.cam_up[:] = list(camera.get("up", (0.0, 1.0, 0.0)))
    c.cam_fov = float(camera.get("fov", 40.0))
    c.ray_eps = float(eps)
    c.precision = int(precision)
    c.threads = int(threads or hardware_threads())
    return c


def render_nee(scene, width: int, height: int, spp: int, depth: int, seed: int = 0, camera: dict | None = None,
               precision: int = 64, threads: int | None = None, pixels=None, sample_base: int = 0,
               eps: float = 1e-4, want_samples: bool = False) -> dict:
    """Renders the NEE integrator for all pixels or the listed pixel indices (y*width+x)."""
    v, a, e = _f32(scene.vertices), _f32(scene.albedo), _f32(scene.emission)
    cam = camera or scene.camera
    cfg = _config(width, height, spp, depth, seed, cam, precision, threads, sample_base, eps)
    pix = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
    npix = width * height if pix is None else pix.size
    mean = np.zeros((npix, 3), np.float64)
    aov = np.zeros((npix, 7), np.float64)
    samples = np.zeros((npix, spp, 3), np.float64) if want_samples else None
    sig = np.zeros((npix, spp), np.uint32) if want_samples else None
    rays = np.zeros(3, np.uint64)
    rc = lib().oracle_render_nee(v.shape[0], v.ctypes.data, a.ctypes.data, e.ctypes.data, C.byref(cfg),
                                 None if pix is None else pix.ctypes.data, npix, mean.ctypes.data,
                                 None if samples is None else samples.ctypes.data,
                                 None if sig is None else sig.ctypes.data, aov.ctypes.data, rays.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_render_nee failed: {rc}")
    return {"mean": mean, "aov": aov, "samples": samples, "sig": sig,
            "rays": {"camera": int(rays[0]), "extension": int(rays[1]), "shadow": int(rays[2])}}


def backward(scene, width: int, height: int, spp: int, depth: int, grad_image, seed: int = 0,
             camera: dict | None = None, threads: int | None = None, sample_base: int = 0, eps: float = 1e-4):
    """FP64 analytic dLoss/dalbedo and dLoss/demission (each (n, 3)) for dLoss/dI = grad_image."""
    v, a, e = _f32(scene.vertices), _f32(scene.albedo), _f32(scene.emission)
    cfg = _config(width, height, spp, depth, seed, camera or scene.camera, 64, threads, sample_base, eps)
    g = np.ascontiguousarray(grad_image, np.float64).reshape(-1)
    assert g.size == width * height * 3
    n = v.shape[0]
    ga = np.zeros((n, 3), np.float64)
    ge = np.zeros((n, 3), np.float64)
    rc = lib().oracle_backward(n, v.ctypes.data, a.ctypes.data, e.ctypes.data, C.byref(cfg), g.ctypes.data,
                               ga.ctypes.data, ge.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_backward failed: {rc}")
    return ga, ge


def render_reference(quads, quad_albedo, quad_emission, width: int, height: int, frames: int, camera: dict,
                     precision: int = 64, threads: int | None = None, sample_base: int = 0) -> dict:
    """The reference integrator (plugin.mm:223-309) over quads; camera uses position/target."""
    q, qa, qe = _f32(quads), _f32(quad_albedo), _f32(quad_emission)
    cfg = _config(width, height, frames, 5, 0, camera, precision, threads, sample_base, 1e-3)
    mean = np.zeros((width * height, 3), np.float64)
    aov = np.zeros((width * height, 7), np.float64)
    rc = lib().oracle_render_reference(q.shape[0], q.ctypes.data, qa.ctypes.data, qe.ctypes.data, C.byref(cfg),
                                       mean.ctypes.data, aov.ctypes.data)
    if rc:
        raise RuntimeError(f"oracle_render_reference failed: {rc}")
    return {"mean": mean.reshape(height, width, 3), "aov": aov.reshape(height, width, 7)}
