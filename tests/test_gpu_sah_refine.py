"""Surface-area refinement of the LBVH (bvh_cluster: the largest subtrees of at most 32
leaves rebuilt with the least-cost split) and the surface-area-optimal spread of the binary
nodes over the 8-wide records (bvh_collapse). Checked as a hierarchy (every leaf once, every
child box the exact union of its triangles' boxes, the 8-wide records covering and
containing what they hold), as an improvement (lower surface-area sum, fewer records, fewer
record visits), and by their effect on images: none, since every hit decision is exact, so
frames rendered over the refined and the plain hierarchy are identical bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import _abi as A
from test_wide_oracle import _decode

pytestmark = pytest.mark.gpu


def _tri_boxes(vertices: np.ndarray, order: np.ndarray):
    v = vertices.reshape(-1, 3, 3)[order]
    return v.min(axis=1), v.max(axis=1)


def _leaf_sets(children: np.ndarray, n: int) -> list[np.ndarray]:
    """Leaf positions under each internal node (children: 2 per node, ~pos for a leaf)."""
    sets: list[np.ndarray | None] = [None] * max(n - 1, 1)
    order, todo = [], [0]
    while todo:  # pre-order, then children before parents when reversed
        c = todo.pop()
        order.append(c)
        for k in (0, 1):
            ch = int(children[2 * c + k])
            if ch >= 0:
                todo.append(ch)
    for c in reversed(order):
        parts = []
        for k in (0, 1):
            ch = int(children[2 * c + k])
            parts.append(np.array([~ch]) if ch < 0 else sets[ch])
        sets[c] = np.concatenate(parts)
    return sets


def _area_sum(boxes: np.ndarray) -> float:
    b = boxes.reshape(-1, 2, 2, 3).astype(np.float64)  # node, child, lo/hi, axis
    d = b[:, :, 1] - b[:, :, 0]
    return float((d[..., 0] * d[..., 1] + d[..., 1] * d[..., 2] + d[..., 2] * d[..., 0]).sum())


@pytest.mark.parametrize("spec", ["cornell36", "soup:n=1000,seed=3", "soup:n=65537,seed=11"])
def test_refined_hierarchy_is_valid_and_better(cuda_ok, orc, spec):
    host = q.PluginHost(width=32, height=32)
    try:
        scene = q.make_scene(spec, host.lib)
        n = scene.tri_count
        host.set_scene(scene)
        host.set_options(bvh_split=A.QUASI_BVH_SPLIT_NONE)  # leaves = triangles, to compare them
        g = host.read_bvh(n)
        words = host.read_wide_bvh(n)
        assert host.stats().error_flags == 0
        host.set_options(bvh_collapse=1)
        greedy_words = host.read_wide_bvh(n)
        host.set_options(bvh_cluster=1, bvh_collapse=1)
        plain = host.read_bvh(n)
    finally:
        host.destroy()
    o = orc.lbvh(scene.vertices)
    assert np.array_equal(g["morton"], o["morton"]) and np.array_equal(g["order"], o["order"])
    assert np.array_equal(plain["children"], o["children"])
    ch = g["children"]
    # every leaf once, every internal node but the root once
    leaves = np.sort(~ch[ch < 0])
    assert np.array_equal(leaves, np.arange(n))
    inner = np.sort(ch[ch >= 0])
    assert np.array_equal(inner, np.arange(1, n - 1))
    # child boxes: exact unions of their triangles' boxes
    tlo, thi = _tri_boxes(scene.vertices, g["order"])
    sets = _leaf_sets(ch, n)
    boxes = g["boxes"].reshape(-1, 2, 2, 3)
    for c in range(n - 1):
        for k in (0, 1):
            x = int(ch[2 * c + k])
            s = np.array([~x]) if x < 0 else sets[x]
            assert np.array_equal(boxes[c, k, 0], tlo[s].min(axis=0)), (c, k)
            assert np.array_equal(boxes[c, k, 1], thi[s].max(axis=0)), (c, k)
    # the 8-wide records over the refined tree: every triangle in one reachable leaf, every
    # decoded child box contains the boxes of what it holds
    cover = np.zeros(n, np.int64)
    for i in orc.wide_reachable(words):
        for lo, hi, ref, internal in _decode(words, i):
            if internal:
                s = sets[ref]
                assert s.size > 1
            else:
                xr = (~ref) & 0xFFFFFFFF
                cnt = ((xr & 3) + 1) & 3
                if cnt == 0:
                    continue
                s = np.arange(xr >> 2, (xr >> 2) + cnt)
                cover[s] += 1
            assert (lo <= tlo[s].min(axis=0)).all() and (hi >= thi[s].max(axis=0)).all()
    assert (cover == 1).all()
    if n > 100:
        assert _area_sum(g["boxes"]) < _area_sum(plain["boxes"])
    # the spread over the records minimises the summed surface area of the records' boxes:
    # no more than greedy opening of the same binary tree
    node_lo, node_hi = boxes[:, :, 0].min(axis=1).astype(np.float64), boxes[:, :, 1].max(axis=1).astype(np.float64)
    d = node_hi - node_lo
    half = d[:, 0] * d[:, 1] + d[:, 1] * d[:, 2] + d[:, 2] * d[:, 0]
    dp_cost = half[orc.wide_reachable(words)].sum()
    greedy_cost = half[orc.wide_reachable(greedy_words)].sum()
    assert dp_cost <= greedy_cost * (1 + 1e-6), (dp_cost, greedy_cost)


def _render(spec: str, cluster: int, collapse: int, w: int, h: int, spp: int, depth: int,
            split: int = A.QUASI_BVH_SPLIT_NONE):
    host = q.PluginHost(width=w, height=h)
    try:
        host.set_scene(q.make_scene(spec, host.lib))
        host.set_options(spp_per_frame=spp, max_depth=depth, seed=11, record_samples=1, collect_stats=1,
                         bvh_cluster=cluster, bvh_collapse=collapse, bvh_split=split)
        host.render(w, h, dirty=True)
        img = np.array(host.readback())
        aov = host.readback_aov()
        rad, sig = host.read_samples(spp)
        st = host.stats()
        assert st.error_flags == 0
        return img, aov, sig, st
    finally:
        host.destroy()


@pytest.mark.parametrize("spec,w,h,spp,depth", [("cornell36", 64, 48, 8, 4), ("soup:n=100000,seed=5", 160, 90, 8, 6)])
def test_refinement_leaves_images_identical(cuda_ok, spec, w, h, spp, depth):
    runs = [_render(spec, cl, co, w, h, spp, depth) for cl, co in ((0, 0), (1, 0), (1, 1))]
    a_img, a_aov, a_sig, a_st = runs[0]
    for b_img, b_aov, b_sig, b_st in runs[1:]:
        assert np.array_equal(a_img, b_img)
        for k in a_aov:
            assert np.array_equal(a_aov[k], b_aov[k]), k
        assert np.array_equal(a_sig, b_sig)
        assert (a_st.camera_rays, a_st.extension_rays, a_st.shadow_rays) == (b_st.camera_rays, b_st.extension_rays,
                                                                             b_st.shadow_rays)
    if spec.startswith("soup"):
        # each step is cheaper to traverse: refined + optimal spread, plain + optimal spread,
        # plain + greedy opening
        visits = [r[3].node_visits for r in runs]
        assert visits[0] < visits[1] < visits[2], visits


@pytest.mark.parametrize("spec,w,h,spp,depth", [("cornell36", 64, 48, 8, 4), ("soup:n=200000,seed=5", 160, 90, 8, 6)])
def test_split_references_leave_images_identical(cuda_ok, spec, w, h, spp, depth):
    """Early split clipping (bvh_split): in scenes of at least 2^17 triangles, the triangles
    whose boxes leave the most area empty become two leaf references with the boxes of their
    halves. Every hit decision is exact, so the frames over the split hierarchy (the default
    share, and half of the triangles) equal those over the unsplit one bit for bit; on the
    200k soup the tighter leaf boxes mean fewer triangle tests per ray (the Cornell box is
    below the size and stays unsplit)."""
    runs = [_render(spec, 0, 0, w, h, spp, depth, split) for split in (A.QUASI_BVH_SPLIT_NONE, 0, 50)]
    a_img, a_aov, a_sig, a_st = runs[0]
    for b_img, b_aov, b_sig, b_st in runs[1:]:
        assert np.array_equal(a_img, b_img)
        for k in a_aov:
            assert np.array_equal(a_aov[k], b_aov[k]), k
        assert np.array_equal(a_sig, b_sig)
        assert (a_st.camera_rays, a_st.extension_rays, a_st.shadow_rays) == (b_st.camera_rays, b_st.extension_rays,
                                                                             b_st.shadow_rays)
    if spec.startswith("soup"):
        tests = [r[3].tri_tests for r in runs]
        assert tests[0] > tests[1] > tests[2], tests


def test_split_hierarchy_is_not_read_back(cuda_ok):
    """Q_cuda_read_bvh and Q_cuda_read_wide_bvh describe leaves that are triangles; over split
    references they refuse with QUASI_ERR_STATE instead of returning arrays of another size."""
    host = q.PluginHost(width=16, height=16)
    try:
        scene = q.make_scene("soup:n=140000,seed=1", host.lib)
        host.set_scene(scene)
        host.set_options(bvh_split=20)
        with pytest.raises(q.QuasiError) as e1:
            host.read_bvh(scene.tri_count)
        with pytest.raises(q.QuasiError) as e2:
            host.read_wide_bvh(scene.tri_count)
        assert e1.value.code == A.QUASI_ERR_STATE and e2.value.code == A.QUASI_ERR_STATE
        host.set_options(bvh_split=A.QUASI_BVH_SPLIT_NONE)
        assert host.read_bvh(scene.tri_count)["order"].size == scene.tri_count
    finally:
        host.destroy()
