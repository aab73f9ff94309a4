"""The benchmark scene generators (CPU).

* The oracle's restatement of the library's generators gives the same bits as
  Q_cuda_make_scene (vertices, albedo, emission, camera) for "cornell36" and for soups of
  several sizes and seeds, so the CPU baseline builds its scene without the product library.
* Both match the configurations they implement: the 36-triangle Cornell box (unit box, walls,
  0.25 x 0.25 light with emission (17, 12, 4), boxes 0.3^3 and 0.3 x 0.6 x 0.3 rotated by
  -18 and +18 degrees, the stated wall colours) and the soup (centres in [0,1)^3, lognormal
  edge lengths of median 0.005 and sigma 0.5, albedo in [0.2, 0.8), round(n/100) emitters
  with emission in [1, 10)).
"""
from __future__ import annotations

import math

import numpy as np
import pytest


@pytest.mark.parametrize("spec", ["cornell36", "soup:n=1000,seed=0", "soup:n=1000,seed=1", "soup:n=1000,seed=7",
                                  "soup:n=20011,seed=3", "soup:n=100000,seed=42"])
def test_oracle_generator_is_bit_identical_to_the_library(qlib, orc, spec):
    import quasi_gb300 as q

    a = q.make_scene(spec, qlib)
    b = orc.make_scene(spec)
    assert a.tri_count == b.tri_count
    for x, y in ((a.vertices, b.vertices), (a.albedo, b.albedo), (a.emission, b.emission)):
        assert x.dtype == y.dtype == np.float32
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    for key in ("position", "target", "up", "fov"):
        assert np.array_equal(np.float32(a.camera[key]), np.float32(b.camera[key])), key


def test_cornell36_matches_its_configuration(orc):
    s = orc.make_scene("cornell36")
    assert s.tri_count == 36
    v = s.vertices.reshape(-1, 3, 3).astype(np.float64)
    alb, em = s.albedo, s.emission
    # unit box: every vertex inside [0, 1]^3
    assert v.min() >= -1e-6 and v.max() <= 1 + 1e-6
    # one emitting quad (2 triangles), emission (17, 12, 4), 0.25 x 0.25 just below the ceiling
    lit = np.flatnonzero(em.max(1) > 0)
    assert lit.size == 2 and np.allclose(em[lit], (17, 12, 4))
    lv = v[lit].reshape(-1, 3)
    assert np.allclose(lv.max(0)[[0, 2]] - lv.min(0)[[0, 2]], 0.25) and np.allclose(lv[:, 1], 0.999)
    # wall colours: floor, ceiling and back white, x = 1 red, x = 0 green (2 triangles each)
    for first, colour in ((0, (0.73, 0.73, 0.73)), (2, (0.73, 0.73, 0.73)), (4, (0.73, 0.73, 0.73)),
                          (6, (0.63, 0.065, 0.05)), (8, (0.14, 0.45, 0.09))):
        assert np.array_equal(alb[first:first + 2], np.float32([colour, colour])), first
    assert np.array_equal(alb[12:], np.full((24, 3), 0.73, np.float32))
    # the two boxes: 12 triangles each after the 10 wall and 2 light triangles; box sizes and
    # rotations from their corner sets
    for first, (sx, sy, sz), deg in ((12, (0.3, 0.3, 0.3), -18.0), (24, (0.3, 0.6, 0.3), 18.0)):
        pts = np.unique(np.round(v[first:first + 12].reshape(-1, 3), 9), axis=0)
        assert len(pts) == 8
        assert np.isclose(pts[:, 1].max() - pts[:, 1].min(), sy)
        base = pts[pts[:, 1] == pts[:, 1].min()]
        centre = base.mean(0)
        edges = [np.linalg.norm(p - q) for i, p in enumerate(base) for q in base[i + 1:]]
        assert np.isclose(sorted(edges)[0], min(sx, sz)) and np.isclose(sorted(edges)[3], max(sx, sz))
        # rotation about y: angle of a base edge against the x axis
        angles = {round(math.degrees(math.atan2(q[2] - p[2], q[0] - p[0])) % 90.0, 6)
                  for i, p in enumerate(base) for q in base[i + 1:]
                  if np.isclose(np.linalg.norm(p - q), sx)}
        assert any(np.isclose(a, abs(deg) % 90.0) or np.isclose(a, 90.0 - abs(deg) % 90.0) for a in angles), angles
        assert 0.0 < centre[0] < 1.0 and 0.0 < centre[2] < 1.0


def test_soup_matches_its_configuration(orc):
    n, seed = 100_000, 5
    s = orc.make_scene(f"soup:n={n},seed={seed}")
    c = orc.soup_centres(n, seed)
    assert c.min() >= 0.0 and c.max() < 1.0
    assert np.allclose(c.mean(0), 0.5, atol=0.005)
    # every vertex is its centre plus a direction times a lognormal length (median 0.005,
    # sigma 0.5); the float32 vertices carry the length to ~1e-7 of the coordinate
    v = s.vertices.reshape(n, 3, 3).astype(np.float64)
    off = v - c[:, None, :]
    lens = np.linalg.norm(off, axis=2).ravel()
    logs = np.log(lens)
    assert abs(logs.mean() - math.log(0.005)) < 0.01, logs.mean()
    assert abs(logs.std() - 0.5) < 0.01, logs.std()
    # directions uniform on the sphere: mean direction ~0, each axis' second moment ~1/3
    dirs = (off / np.linalg.norm(off, axis=2, keepdims=True)).reshape(-1, 3)
    assert np.abs(dirs.mean(0)).max() < 0.01 and np.allclose((dirs ** 2).mean(0), 1 / 3, atol=0.01)
    alb = s.albedo.astype(np.float64)
    assert alb.min() >= 0.2 and alb.max() < 0.8
    assert abs(alb.mean() - 0.5) < 0.005
    lit = np.flatnonzero(s.emission.max(1) > 0)
    assert lit.size == round(n / 100)
    em = s.emission[lit].astype(np.float64)
    assert em.min() >= 1.0 and em.max() < 10.0 and abs(em.mean() - 5.5) < 0.1
    assert np.all(s.emission[np.setdiff1d(np.arange(n), lit)] == 0.0)
