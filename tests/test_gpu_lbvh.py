"""GPU LBVH and radix sort, bit-exact against the oracle and numpy (integer work), and the
8-wide traversal records collapsed from the LBVH, bit-exact against the oracle's collapse."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import _abi as A

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host(cuda_ok):
    h = q.PluginHost(width=32, height=32)
    # the plain Morton hierarchy over the triangles themselves (no split references, no
    # surface-area refinement), records by greedy opening
    h.set_options(bvh_cluster=1, bvh_collapse=1, bvh_split=A.QUASI_BVH_SPLIT_NONE)
    yield h
    h.destroy()


def _scene_from_vertices(v: np.ndarray) -> q.Scene:
    n = v.shape[0]
    return q.Scene(v.astype(np.float32), np.full((n, 3), 0.5, np.float32), np.zeros((n, 3), np.float32),
                   {"position": (0.5, 0.5, -1.0), "target": (0.5, 0.5, 0.5)})


def _compare(host, orc, scene: q.Scene) -> None:
    host.set_scene(scene)
    g = host.read_bvh(scene.tri_count)
    o = orc.lbvh(scene.vertices)
    assert np.array_equal(g["bounds"], o["bounds"]), (g["bounds"], o["bounds"])
    assert np.array_equal(g["morton"], o["morton"]), "Morton codes differ"
    assert np.array_equal(g["order"], o["order"]), "sort order differs"
    assert np.array_equal(g["children"], o["children"]), "topology differs"
    assert np.array_equal(g["boxes"].view(np.uint32), o["boxes"].view(np.uint32)), "child boxes differ"
    gw = host.read_wide_bvh(scene.tri_count)
    ow = orc.collapse8(scene.vertices)
    reach = orc.wide_reachable(ow)
    assert orc.wide_reachable(gw) == reach
    assert np.array_equal(gw[reach], ow[reach]), "8-wide records differ"
    assert host.stats().error_flags == 0


@pytest.mark.parametrize("spec", ["cornell36", "refcornell", "soup:n=1000,seed=3", "soup:n=65537,seed=11",
                                  "soup:n=250000,seed=2"])
def test_lbvh_bit_exact(host, orc, spec):
    _compare(host, orc, q.make_scene(spec, host.lib))


def test_lbvh_bit_exact_full_size(host, orc):
    """1,000,000 triangles: the Morton codes, sort order, topology and boxes of the
    benchmark scene match the oracle bit for bit."""
    _compare(host, orc, q.make_scene("soup:n=1000000,seed=0", host.lib))


def test_lbvh_edge_cases(host, orc):
    rng = np.random.default_rng(5)
    one = rng.random((1, 9), np.float32)
    _compare(host, orc, _scene_from_vertices(one))
    two = rng.random((2, 9), np.float32)
    _compare(host, orc, _scene_from_vertices(two))
    same = np.tile(rng.random((1, 9), np.float32), (300, 1))  # every Morton code equal
    _compare(host, orc, _scene_from_vertices(same))
    clustered = (rng.random((5000, 9), np.float32) * 1e-4).astype(np.float32)
    clustered[::97] += 1.0  # a few outliers stretch the bounds: most codes collide
    _compare(host, orc, _scene_from_vertices(clustered))
    flat = rng.random((777, 9), np.float32)
    flat[:, 1::3] = 0.25  # zero extent on y
    _compare(host, orc, _scene_from_vertices(flat))


def _sort_on_gpu(host, keys: np.ndarray, vals: np.ndarray, bits: int) -> tuple[np.ndarray, np.ndarray]:
    import torch

    n = keys.size
    kt = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    vt = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    torch.cuda.synchronize()
    rc = host.lib.Q_cuda_radix_sort_pairs(C.c_void_p(kt.data_ptr() if n else 0), C.c_void_p(vt.data_ptr() if n else 0),
                                          n, bits, None)
    assert rc == 0
    return kt.cpu().numpy().view(np.uint32), vt.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("n", [0, 1, 2, 31, 2047, 2048, 2049, 100_003, 1_000_000])
@pytest.mark.parametrize("bits", [8, 30, 32])
def test_radix_sort_stable(host, n, bits):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
    if n > 10:
        keys[: n // 3] = keys[0]  # heavy duplicates exercise stability
        rng.shuffle(keys)
    vals = np.arange(n, dtype=np.uint32)
    k, v = _sort_on_gpu(host, keys, vals, bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order])
    assert np.array_equal(v, vals[order])


def test_radix_sort_rejects_bad_arguments(host):
    assert host.lib.Q_cuda_radix_sort_pairs(None, None, 10, 32, None) == -1
    assert host.lib.Q_cuda_radix_sort_pairs(None, None, 0, 32, None) == 0
