"""GPU path tracer parity against the FP64 oracle at matched seeds.

Tolerance: per-pixel relative error |gpu - oracle| / max(|oracle|, 1e-3) <= 1e-4 for every
pixel and every sample, and every path signature (the sequence of triangles hit and
shadow-ray outcomes) equal to the oracle's: hit decisions are exact (FP32 tests with an error
bound, undecided candidates re-decided in double-float), so no path may take another branch
than FP64 takes.
"""
from __future__ import annotations

import ctypes
import json

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import _abi as A
from tests.parity_stats import error_stats

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4
FLOOR = 1e-3


@pytest.fixture(scope="module")
def host(cuda_ok):
    h = q.PluginHost(width=64, height=64)
    yield h
    h.destroy()


def _render(host, scene, w, h, spp, depth, seed=0, frames=1, **opts):
    host.set_scene(scene)
    host.set_options(spp_per_frame=spp, max_depth=depth, seed=seed, record_samples=1, **opts)
    for f in range(frames):
        host.render(w, h, dirty=(f == 0))
    img = host.readback()
    rad, sig = host.read_samples(spp)
    st = host.stats()
    assert st.error_flags == 0, st.error_flags
    return img, rad, sig, st


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), FLOOR)


def _report(name, g_img, g_rad, g_sig, ref, spp):
    """Prints the error statistics of one workload (shown with pytest -s)."""
    st = error_stats(g_img, g_rad, g_sig, ref["mean"], ref["samples"], ref["sig"], spp)
    print(json.dumps({"workload": name, **st}))
    return st


def _check_parity(img, rad, sig, ref, w, h, spp, name=""):
    _report(name, img[..., :3], rad, sig, ref, spp)
    osig = ref["sig"].reshape(h, w, spp)
    osamp = ref["samples"].reshape(h, w, spp, 3)
    match = sig == osig
    # every path takes the oracle's branches
    assert match.all(), np.argwhere(~match)[:8]
    # every sample and every pixel within the bound
    s_err = _rel(rad.astype(np.float64), osamp).max(-1)
    assert s_err.max() <= REL_TOL, s_err.max()
    p_err = _rel(img[..., :3].astype(np.float64), ref["mean"].reshape(h, w, 3)).max(-1)
    assert p_err.max() <= REL_TOL, p_err.max()
    return p_err


def test_cornell36_parity(host, orc):
    """Cornell box of 36 triangles, 256x256, 16 spp, depth 4, seed 0."""
    w = h = 256
    spp, depth = 16, 4
    scene = q.make_scene("cornell36", host.lib)
    img, rad, sig, st = _render(host, scene, w, h, spp, depth)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=0, want_samples=True)
    _check_parity(img, rad, sig, ref, w, h, spp, name="cornell36 256x256 16spp depth4")
    assert st.camera_rays == w * h * spp
    # every path takes the oracle's branches, so the ray counts are the oracle's exactly
    for k, v in (("camera", st.camera_rays), ("extension", st.extension_rays), ("shadow", st.shadow_rays)):
        assert int(v) == ref["rays"][k], (k, v, ref["rays"][k])


def test_refcornell_triangles_parity(host, orc):
    """The reference's own Cornell scene (cornell_box.hpp) as 32 triangles, NEE integrator."""
    w, h = 96, 72
    spp, depth = 8, 5
    scene = q.make_scene("refcornell", host.lib)
    img, rad, sig, _ = _render(host, scene, w, h, spp, depth, seed=7)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=7, want_samples=True)
    _check_parity(img, rad, sig, ref, w, h, spp, name="refcornell 96x72 8spp depth5")


def test_soup_parity_subset(host, orc):
    """A 100k-triangle soup (1% emitters), 8 bounces: full GPU frame, oracle on 1500 pixels."""
    w, h = 320, 180
    spp, depth = 4, 8
    scene = q.make_scene("soup:n=100000,seed=1", host.lib)
    img, rad, sig, _ = _render(host, scene, w, h, spp, depth, seed=3)
    rng = np.random.default_rng(0)
    pix = rng.choice(w * h, size=1500, replace=False).astype(np.uint32)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=3, pixels=pix, want_samples=True)
    ys, xs = pix // w, pix % w
    g_sig = sig[ys, xs]
    g_rad = rad[ys, xs].astype(np.float64)
    _report("soup-100k 320x180 4spp depth8 (1500 random pixels)", img[ys, xs, :3], g_rad, g_sig, ref, spp)
    match = g_sig == ref["sig"]
    assert match.all(), np.argwhere(~match)[:8]
    assert _rel(g_rad, ref["samples"]).max() <= REL_TOL
    p_err = _rel(img[ys, xs, :3].astype(np.float64), ref["mean"]).max(-1)
    assert p_err.max() <= REL_TOL


def test_full_size_soup_parity_sampled_pixels(host, orc):
    """The benchmark configuration (1M triangles, 1920x1080, depth 8) at 2 spp: the GPU frame
    against the oracle on 20,000 random pixels, plus size-independent properties."""
    w, h = 1920, 1080
    spp, depth = 2, 8
    scene = q.make_scene("soup:n=1000000,seed=0", host.lib)
    img, rad, sig, st = _render(host, scene, w, h, spp, depth, seed=0)
    assert np.isfinite(img).all() and (img[..., :3] >= 0).all()
    assert np.all(img[..., 3] == 1.0)
    rng = np.random.default_rng(1)
    pix = rng.choice(w * h, size=20_000, replace=False).astype(np.uint32)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=0, pixels=pix, want_samples=True)
    ys, xs = pix // w, pix % w
    _report("soup-1M 1920x1080 2spp depth8 (20,000 random pixels)", img[ys, xs, :3], rad[ys, xs], sig[ys, xs], ref, spp)
    match = sig[ys, xs] == ref["sig"]
    assert match.all(), np.argwhere(~match)[:8]
    assert _rel(rad[ys, xs].astype(np.float64), ref["samples"]).max() <= REL_TOL
    # every path starts with exactly one camera ray; shadow rays never exceed vertices
    assert st.camera_rays == w * h * spp
    assert st.shadow_rays <= st.camera_rays + st.extension_rays


def test_progressive_frames_equal_one_frame(host):
    """Kahan accumulation over frames is order-preserving: 2 frames of 8 spp give the same
    bits as one frame of 16 spp, and the wavefront size does not change results."""
    scene = q.make_scene("cornell36", host.lib)
    w = h = 64
    host.set_scene(scene)
    outs = []
    for spp, frames, wave in ((16, 1, 0), (8, 2, 0), (16, 1, 1), (4, 4, 3)):
        host.set_options(spp_per_frame=spp, max_depth=4, seed=5, wave_spp=wave, record_samples=0)
        for f in range(frames):
            host.render(w, h, dirty=(f == 0))
        outs.append(host.readback())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_deterministic_and_seed_sensitive(host):
    scene = q.make_scene("soup:n=20000,seed=4", host.lib)
    host.set_scene(scene)
    host.set_options(spp_per_frame=4, max_depth=6, seed=1, record_samples=0, wave_spp=0)
    host.render(160, 90, dirty=True)
    a = host.readback()
    host.render(160, 90, dirty=True)
    b = host.readback()
    assert np.array_equal(a, b)
    host.set_options(spp_per_frame=4, max_depth=6, seed=2)
    host.render(160, 90, dirty=True)
    c = host.readback()
    assert not np.array_equal(a, c)


def test_aovs_match_oracle(host, orc):
    w = h = 64
    spp, depth = 4, 4
    scene = q.make_scene("cornell36", host.lib)
    host.set_scene(scene)
    host.set_options(spp_per_frame=spp, max_depth=depth, seed=0, record_samples=1)
    host.render(w, h, dirty=True)
    aov = host.readback_aov()
    _, sig = host.read_samples(spp)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=0, want_samples=True)
    first_hit_ok = np.ones((h, w), bool)  # AOVs depend only on the camera ray's first hit
    o = ref["aov"].reshape(h, w, 7)
    assert np.abs(aov["albedo"][..., :3] - o[..., 0:3]).max() < 1e-5
    assert np.abs(aov["depth"][..., 0] - o[..., 3]).max() < 1e-4
    assert np.abs(aov["normal"][..., :3] - o[..., 4:7]).max() < 1e-4
    assert np.all(aov["depth"][..., 3] == 1.0) and first_hit_ok.all()


def test_white_furnace_closed_box(host):
    """A closed box whose every triangle has albedo rho and emission Le: with emission on
    camera hits plus NEE at each of D vertices, every pixel converges to Le * sum_{i<=D} rho^i."""
    rho, le, depth = 0.5, 1.0, 4
    s = q.make_scene("cornell36", host.lib)
    box = np.array([[0, 0, 0, 1, 0, 0, 1, 0, 1], [0, 0, 0, 1, 0, 1, 0, 0, 1],   # floor
                    [0, 1, 0, 1, 1, 1, 1, 1, 0], [0, 1, 0, 0, 1, 1, 1, 1, 1],   # ceiling
                    [0, 0, 1, 1, 0, 1, 1, 1, 1], [0, 0, 1, 1, 1, 1, 0, 1, 1],   # back
                    [0, 0, 0, 0, 1, 0, 1, 1, 0], [0, 0, 0, 1, 1, 0, 1, 0, 0],   # front
                    [0, 0, 0, 0, 0, 1, 0, 1, 1], [0, 0, 0, 0, 1, 1, 0, 1, 0],   # x = 0
                    [1, 0, 0, 1, 1, 0, 1, 1, 1], [1, 0, 0, 1, 1, 1, 1, 0, 1]],  # x = 1
                   np.float32)
    n = box.shape[0]
    scene = q.Scene(box, np.full((n, 3), rho, np.float32), np.full((n, 3), le, np.float32),
                    {"position": (0.5, 0.5, 0.5), "target": (0.5, 0.5, 1.0), "fov": 60.0})
    del s
    host.set_scene(scene)
    host.set_options(spp_per_frame=64, max_depth=depth, seed=0, record_samples=0)
    host.render(64, 64, dirty=True)
    img = host.readback()[..., :3]
    expect = le * sum(rho ** i for i in range(depth + 1))
    assert abs(img.mean() / expect - 1.0) < 5e-3, (img.mean(), expect)


def test_reference_integrator_matches_reference_shader(host, golden):
    """The CUDA restatement of plugin.mm's path_trace (quads, brute force, the reference's
    seeding and Russian roulette) against the shader run on the CPU, 24x24, 16 frames."""
    r = golden["render"]
    w, h, frames = r["width"], r["height"], r["frames"]
    scene = q.make_scene("refcornell", host.lib)
    host.set_scene(scene)
    host.set_options(integrator=1, spp_per_frame=1, max_depth=5, record_samples=0)
    for f in range(frames):
        host.render(w, h, camera=r["camera"], dirty=(f == 0))
    aov = host.readback_aov()
    ref = np.array(r["beauty"], np.float64).reshape(h, w, 4)[..., :3]
    err = _rel(aov["beauty"][..., :3].astype(np.float64), ref).max(-1)
    print(f"reference integrator vs shader: {int((err > REL_TOL).sum())} of {err.size} pixels over {REL_TOL}, "
          f"largest errors {np.sort(err.ravel())[-8:]}")
    assert err.max() <= REL_TOL, (np.sort(err.ravel())[-8:])
    assert np.abs(aov["albedo"][..., :3] - np.array(r["albedo"]).reshape(h, w, 4)[..., :3]).max() < 1e-4
    host.set_options(integrator=0, spp_per_frame=1, max_depth=4)


def test_tonemap_into_device_buffer(host):
    import torch

    w = h = 32
    host.set_scene(q.make_scene("cornell36", host.lib))
    host.set_options(spp_per_frame=4, max_depth=4, seed=0, record_samples=0)
    buf = torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    host.render(w, h, dirty=True, drawable=buf.data_ptr())
    hdr = host.readback()[..., :3]
    host.synchronize()
    ldr = buf.cpu().numpy().reshape(h, w, 4)
    expect = np.clip(np.power(hdr / (hdr + 1.0), 1.0 / 2.2) * 255.0 + 0.5, 0, 255).astype(np.uint8)
    assert np.abs(ldr[..., :3].astype(int) - expect.astype(int)).max() <= 1
    assert np.all(ldr[..., 3] == 255)


def test_autotune_keeps_images(cuda_ok):
    """Q_cuda_autotune picks among bit-identical forms and launch shapes: the first frame after
    it (accumulation reset) equals the first frame before it."""
    sc = q.make_scene("soup:n=50000,seed=3")
    h = q.PluginHost(width=160, height=96)
    h.set_scene(sc)
    h.set_options(spp_per_frame=16, max_depth=6, seed=0)
    h.render(160, 96, dirty=True)
    ref = h.readback()
    h.autotune(1500)
    o = h.options()
    assert o.megakernel in (0, 1) and o.trace_block in (0, 64, 128, 256) and o.smem_levels in (0, 7, 32)
    assert o.refill_lanes in (0, 2, 4, 8)
    assert o.spp_per_frame == 16 and o.max_depth == 6 and o.wave_spp in (1, 2, 4, 8, 16)
    h.render(160, 96)
    assert np.array_equal(h.readback(), ref)
    assert h.stats().error_flags == 0
    h.destroy()


@pytest.mark.parametrize("spec,w,h,spp,depth", [("cornell36", 128, 128, 8, 4), ("soup:n=200000,seed=5", 320, 180, 4, 8)])
def test_wide_and_binary_traversal_agree(host, spec, w, h, spp, depth):
    """The 8-wide records and the binary LBVH return the same closest hits (smallest t, ties
    to the lower triangle index) and the same shadow-ray outcomes: both forms give the same
    path signatures and the same radiance bits, in the wavefront and the megakernel."""
    scene = q.make_scene(spec, host.lib)
    # (bvh_width, megakernel, refill_lanes, smem_levels): binary with a shared-memory treelet,
    # binary with per-lane refill, binary without treelet, 8-wide with refill (default),
    # 8-wide whole-warp batches, megakernel
    forms = ((2, 0, 0, 0), (2, 0, 8, 0), (2, 0, 0, 32), (8, 0, 0, 0), (8, 0, 32, 0), (8, 1, 0, 0))
    out = {}
    for width, mega, refill, levels in forms:
        img, rad, sig, st = _render(host, scene, w, h, spp, depth, seed=11, bvh_width=width, megakernel=mega,
                                    refill_lanes=refill, smem_levels=levels)
        out[(width, mega, refill, levels)] = (img, rad, sig, st)
    img2, rad2, sig2, st2 = out[forms[0]]
    for key in forms[1:]:
        img8, rad8, sig8, st8 = out[key]
        same = sig8 == sig2
        assert same.mean() >= 1.0 - 1e-5, (key, same.mean())
        assert np.array_equal(rad8[same], rad2[same]), key
        assert st8.camera_rays == st2.camera_rays
        if same.all():
            assert np.array_equal(img8, img2), key
    host.set_options(bvh_width=0, megakernel=0, refill_lanes=0, smem_levels=0)


def _edge_scene(kind: str) -> q.Scene:
    rng = np.random.default_rng(21)
    cam = {"position": (0.5, 0.5, -1.0), "target": (0.5, 0.5, 0.5), "fov": 40.0}
    if kind == "empty":
        v = np.zeros((0, 9), np.float32)
    elif kind == "one_emitter":
        v = np.array([[0.1, 0.1, 0.5, 0.9, 0.1, 0.5, 0.5, 0.9, 0.5]], np.float32)
    elif kind == "two":
        v = np.array([[0.1, 0.1, 0.5, 0.9, 0.1, 0.5, 0.5, 0.9, 0.5],
                      [0.0, 0.0, 0.2, 1.0, 0.0, 0.2, 0.5, 0.0, 1.0]], np.float32)
    elif kind == "no_emitters":
        v = (rng.random((400, 9)) * 0.8 + 0.1).astype(np.float32)
    else:  # "degenerate": a soup with zero-area triangles (a vertex repeated), some emitting
        v = (rng.random((500, 9)) * 0.8 + 0.1).astype(np.float32)
        v[::7, 3:6] = v[::7, 0:3]
        v[1::11, 6:9] = v[1::11, 3:6]
    n = v.shape[0]
    albedo = np.full((n, 3), 0.6, np.float32)
    emission = np.zeros((n, 3), np.float32)
    if kind in ("one_emitter", "two"):
        emission[0] = (5.0, 4.0, 3.0)
    if kind == "degenerate":
        emission[::9] = (3.0, 3.0, 3.0)
    return q.Scene(v, albedo, emission, cam)


@pytest.mark.parametrize("kind,w,h,spp,depth", [("empty", 16, 8, 2, 4), ("one_emitter", 37, 23, 4, 1),
                                                 ("two", 37, 23, 4, 3), ("no_emitters", 24, 20, 2, 4),
                                                 ("degenerate", 40, 28, 4, 5)])
def test_edge_scenes_parity(host, orc, kind, w, h, spp, depth):
    """Empty and tiny scenes, a scene without emitters, zero-area triangles, image sizes that
    are not multiples of the 8x4 pixel tile, and depth 1: parity with the FP64 oracle."""
    scene = _edge_scene(kind)
    img, rad, sig, st = _render(host, scene, w, h, spp, depth, seed=4)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=4, camera=scene.camera, want_samples=True)
    _check_parity(img, rad, sig, ref, w, h, spp)
    assert st.camera_rays == w * h * spp
    if kind in ("empty", "no_emitters"):
        assert np.all(img[..., :3] == 0.0) and st.shadow_rays == 0


def _needle_scene(n=20000, seed=4, width=0.01) -> q.Scene:
    """Long thin triangles across the unit cube: their boxes are large and overlap along
    every ray while the triangles themselves are rarely hit, so a ray stacks many subtrees
    before a hit culls them. In a CPU model of the same 8-wide records (same camera) most
    rays stack more than 20 entries at some point (up to ~37): past the shared-memory part
    of the stacks (16 entries closest-hit, 20 any-hit) into the thread-local part."""
    rng = np.random.default_rng(seed)
    a = rng.random((n, 3)) * 0.9 + 0.05
    b = rng.random((n, 3)) * 0.9 + 0.05
    d = rng.normal(0.0, 1.0, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    v = np.concatenate([a, b, a + d * width], axis=1).astype(np.float32)
    albedo = np.full((n, 3), 0.7, np.float32)
    emission = np.zeros((n, 3), np.float32)
    emission[::31] = (4.0, 3.5, 3.0)
    cam = {"position": (0.5, 0.5, -1.0), "target": (0.5, 0.5, 0.5), "fov": 40.0}
    return q.Scene(v, albedo, emission, cam)


def test_deep_stacks_forms_agree_and_match_oracle(host, orc):
    """Rays whose traversal stacks overflow the shared-memory part: the 8-wide refill kernels
    (256- and 64-thread blocks, so two shared-memory layouts) return the same hits and shadow
    outcomes as the binary LBVH, and the image matches the FP64 oracle."""
    scene = _needle_scene()
    w, h, spp, depth = 64, 48, 4, 4
    out = {}
    for width, tb in ((2, 0), (8, 0), (8, 64)):
        out[(width, tb)] = _render(host, scene, w, h, spp, depth, seed=9, bvh_width=width, trace_block=tb)
    _, rad2, sig2, st2 = out[(2, 0)]
    for key in ((8, 0), (8, 64)):
        _, rad8, sig8, st8 = out[key]
        same = sig8 == sig2
        assert same.mean() >= 1.0 - 1e-4, (key, same.mean())
        assert np.array_equal(rad8[same], rad2[same]), key
        assert st8.camera_rays == st2.camera_rays and st8.error_flags == 0
    img, rad, sig, st = out[(8, 0)]
    assert st.shadow_rays > 0
    ref = orc.render_nee(scene, w, h, spp, depth, seed=9, camera=scene.camera, want_samples=True)
    _check_parity(img, rad, sig, ref, w, h, spp)
    host.set_options(bvh_width=0, trace_block=0)


def test_options_and_frames_are_validated(host):
    host.set_scene(q.make_scene("cornell36", host.lib))
    for bad in (dict(bvh_width=4), dict(refill_lanes=33), dict(trace_block=48), dict(max_depth=65)):
        with pytest.raises(q.QuasiError):
            host.set_options(**bad)
    host.set_options(bvh_width=0, refill_lanes=0, trace_block=0, max_depth=4)
    # frames: more than 2^26 pixels and a zero extent are refused with a message, and the
    # next valid frame renders (the error is per call, not sticky)
    with pytest.raises(q.QuasiError, match="too large"):
        host.render(8193, 8193, dirty=True)
    f = A.Q_render_frame()
    f.width, f.height, f.camera = 0, 16, host.camera
    host.lib.Q_plugin_render(host.handle, ctypes.byref(f))
    assert b"zero-sized" in host.lib.Q_cuda_last_error(host.handle)
    host.render(16, 16, dirty=True)
    assert host.readback().shape == (16, 16, 4)
    assert host.stats().error_flags == 0


def test_benchmark_frame_parity_sampled_pixels(orc):
    """The benchmark configuration itself: 1M-triangle soup, 1920x1080, 64 spp, depth 8, LBVH
    built on the GPU. Every sample of 20,000 random pixels (1.28 M paths, about 1 % of the
    frame) against the FP64 oracle: the same path signatures and per-sample and per-pixel
    relative error <= 1e-4."""
    w, h, spp, depth = 1920, 1080, 64, 8
    host = q.PluginHost(width=w, height=h)
    scene = q.make_scene("soup:n=1000000,seed=0", host.lib)
    host.set_scene(scene)
    host.set_options(spp_per_frame=spp, max_depth=depth, seed=17, record_samples=1)
    host.render(w, h, dirty=True)
    img = host.readback()
    rad, sig = host.read_samples(spp)
    st = host.stats()
    host.destroy()
    assert st.error_flags == 0
    rng = np.random.default_rng(3)
    pix = rng.choice(w * h, size=20_000, replace=False).astype(np.uint32)
    ref = orc.render_nee(scene, w, h, spp, depth, seed=17, pixels=pix, want_samples=True)
    ys, xs = pix // w, pix % w
    _report("soup-1M 1920x1080 64spp depth8 (20,000 random pixels)", img[ys, xs, :3], rad[ys, xs], sig[ys, xs], ref, spp)
    match = sig[ys, xs] == ref["sig"]
    assert match.all(), np.argwhere(~match)[:8]
    assert _rel(rad[ys, xs].astype(np.float64), ref["samples"]).max() <= REL_TOL
    p_err = _rel(img[ys, xs, :3].astype(np.float64), ref["mean"]).max(-1)
    assert p_err.max() <= REL_TOL, p_err.max()
