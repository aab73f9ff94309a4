"""Pins the oracle against golden vectors produced by the reference's own code.

tests/golden/reference_golden.json was written by tests/golden/make_golden.py, which compiles
the reference's C++ scene headers and the shader source of backends/metal/plugin.mm as
plain C++ (oracle/ref_golden.cpp) and runs them on the CPU.
"""
from __future__ import annotations

import numpy as np
import pytest


def _pcg_np(x: np.ndarray) -> np.ndarray:
    """plugin.mm:98-102 vectorised over uint32 arrays (for searching inputs)."""
    x = x.astype(np.uint64)
    state = (x * np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
    word = (((state >> ((state >> np.uint64(28)) + np.uint64(4))) ^ state) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
    return ((word >> np.uint64(22)) ^ word).astype(np.uint32)


def test_pcg_hash_matches_reference(golden, orc):
    ins, outs = golden["pcg_hash"]["in"], golden["pcg_hash"]["out"]
    assert len(ins) == 64
    for i, o in zip(ins, outs):
        assert orc.pcg_hash(i) == o
    assert np.array_equal(_pcg_np(np.array(ins, np.uint32)), np.array(outs, np.uint32))


def test_random_float_chain_matches_reference(golden, orc):
    for rec in golden["random_float"]:
        vals, final = orc.random_floats(rec["seed"], 16)
        assert np.array_equal(np.float32(vals), np.float32(rec["values"]))
        assert final == rec["final_state"]


def test_random_float_can_return_one(orc):
    # float(state) / float(0xFFFFFFFF) rounds to exactly 1.0 for the top 128 hash values.
    hits = np.zeros(0, np.uint32)
    for start in range(0, 1 << 28, 1 << 22):
        xs = np.arange(start, start + (1 << 22), dtype=np.uint32)
        hits = xs[_pcg_np(xs) >= np.uint32(0xFFFFFF80)]
        if hits.size:
            break
    assert hits.size > 0
    vals, _ = orc.random_floats(int(hits[0]), 1)
    assert vals[0] == 1.0


def test_path_key_is_a_hash_chain(orc):
    assert orc.path_key(0, 5, 7, 2) == orc.pcg_hash(orc.pcg_hash(orc.pcg_hash(0 ^ 5) + 7) + 2)
    assert orc.path_key(3, 5, 7, 2) != orc.path_key(3, 5, 7, 3)


def test_cosine_sample_matches_reference(golden, orc):
    for rec in golden["cosine_sample"]:
        (r1, r2), _ = orc.random_floats(rec["state"], 2)
        d = orc.cosine_sample(rec["normal"], r1, r2)
        ref = np.array(rec["dir"], np.float64)
        assert np.abs(d - ref).max() < 2e-6, rec
        n = np.array(rec["normal"], np.float64)
        assert abs(np.linalg.norm(d) - 1.0) < 1e-12
        assert np.dot(d, n / np.linalg.norm(n)) >= -1e-7


def test_camera_matches_reference_get_ray(golden, orc):
    cam = golden["cornell"]["camera"]  # position, direction, up, fov, aspect
    pos = cam[0:3]
    target = [cam[0] + cam[3], cam[1] + cam[4], cam[2] + cam[5]]
    for u, v, ox, oy, oz, dx, dy, dz in golden["camera_get_ray"]:
        d = orc.camera_dir(pos, target, cam[6:9], cam[9], 100, 100, u, v)
        assert np.abs(d - np.array([dx, dy, dz])).max() < 2e-6
        assert (ox, oy, oz) == tuple(np.float32(pos))


def test_shader_camera_ray_matches_reference(golden, orc):
    pos, target, up = [0.0, 1.0, 3.5], [0.0, 1.0, 0.0], [0.0, 1.0, 0.0]
    direction = np.float32(target) - np.float32(pos)
    direction = direction / np.float32(np.sqrt(np.float32(direction @ direction)))
    for rec in golden["msl_camera_ray"]:
        ux, uy, ox, oy, oz, dx, dy, dz = rec["ray"]
        o, d, _ = orc.ref_camera_ray(pos, direction, up, 40.0, 1.0, ux, uy, rec["state"])
        assert np.abs(d - np.array([dx, dy, dz])).max() < 2e-6
        assert np.allclose(o, [ox, oy, oz])


def test_quad_intersection_matches_shader(golden, orc):
    quads = golden["cornell"]["quads"]
    n_hits = 0
    for rec in golden["quad_hits"]:
        r = rec["ray"]
        hit = orc.intersect_quad(r[0:3], r[3:6], quads[rec["quad"]][0:9])
        assert (hit is not None) == rec["msl_hit"], rec
        if hit is not None:
            n_hits += 1
            t, p, n = hit
            m = rec["msl"]
            assert abs(t - m[0]) <= 1e-5 * max(1.0, abs(m[0]))
            assert np.abs(p - np.array(m[1:4])).max() < 1e-5
            assert np.abs(n - np.array(m[4:7])).max() < 1e-6
    assert n_hits > 20


def test_reference_cpu_quad_twin_differs_from_shader(golden):
    """src/quasi/scene/quad.hpp:83-84 computes alpha/beta with the opposite sign of the
    shader (plugin.mm:183-184), so the reference's CPU twin and its GPU path disagree on
    some rays. The shader is the render path; the oracle and the CUDA kernels follow it."""
    disagree = [h for h in golden["quad_hits"] if h["cpp_hit"] != h["msl_hit"]]
    assert len(disagree) > 0
    q = np.array(golden["cornell"]["quads"][0][0:9], np.float64)  # floor
    o, u, v = q[0:3], q[3:6], q[6:9]
    n = np.cross(u, v)
    w = n / (n @ n)
    planar = (o + 0.25 * u + 0.5 * v) - o
    alpha_shader = w @ np.cross(planar, v)
    alpha_cpp = np.cross(w, v) @ planar
    assert alpha_shader == pytest.approx(0.25) and alpha_cpp == pytest.approx(-0.25)


def test_reference_scene_matches_product_generator(golden, qlib):
    from quasi_gb300 import make_scene

    sc = make_scene("refcornell", qlib)
    ref = np.array(golden["cornell"]["quads"], np.float32)
    assert sc.quads.shape == (16, 9)
    assert np.array_equal(sc.quads, ref[:, 0:9]), np.abs(sc.quads - ref[:, 0:9]).max()
    assert np.array_equal(sc.quad_albedo, ref[:, 9:12])
    assert np.array_equal(sc.quad_emission, ref[:, 12:15])
    assert golden["cornell"]["light_index"] == 5 and sc.quad_emission[5].max() == 15.0
    assert sc.tri_count == 32
    assert tuple(np.float32(sc.camera["position"])) == (0.0, 1.0, 3.5)


def _golden_render(golden):
    r = golden["render"]
    w, h = r["width"], r["height"]
    return {k: np.array(r[k], np.float64).reshape(h, w, 4) for k in ("beauty", "albedo", "normal", "depth")}, r


def test_oracle_reference_integrator_fp32_matches_shader(golden, orc):
    """The FP32 instance of the oracle's reference integrator against the shader run on the
    CPU: same seeds, same operation order; only the running-mix vs mean accumulation differs."""
    g, r = _golden_render(golden)
    q = np.array(golden["cornell"]["quads"], np.float32)
    out = orc.render_reference(q[:, 0:9], q[:, 9:12], q[:, 12:15], r["width"], r["height"], r["frames"],
                               r["camera"], precision=32)
    ref = g["beauty"][..., :3]
    err = np.abs(out["mean"] - ref) / np.maximum(np.abs(ref), 1e-3)
    assert err.max() < 1e-6, err.max()
    assert np.abs(out["aov"][..., 0:3] - g["albedo"][..., :3]).max() < 1e-5
    assert np.abs(out["aov"][..., 4:7] - g["normal"][..., :3]).max() < 1e-5
    assert np.abs(out["aov"][..., 3] - g["depth"][..., 0]).max() < 1e-5


def test_oracle_reference_integrator_fp64_close_to_shader(golden, orc):
    """FP64 oracle vs the FP32 shader: paths whose branch decisions agree match to ~1e-5;
    a few pixels may differ by a whole path (a Russian-roulette or hit decision flips)."""
    g, r = _golden_render(golden)
    q = np.array(golden["cornell"]["quads"], np.float32)
    out = orc.render_reference(q[:, 0:9], q[:, 9:12], q[:, 12:15], r["width"], r["height"], r["frames"],
                               r["camera"], precision=64)
    ref = g["beauty"][..., :3]
    err = (np.abs(out["mean"] - ref) / np.maximum(np.abs(ref), 1e-3)).max(axis=-1)
    close = err < 1e-4
    assert close.mean() >= 0.99, (close.mean(), np.sort(err.ravel())[-10:])
