"""The oracle's 8-wide collapse of the LBVH (the restatement the GPU records are checked
against bit for bit): every triangle sits in exactly one reachable leaf, every decoded child
box contains the exact box of what it holds, and the records are deterministic."""
from __future__ import annotations

import numpy as np
import pytest

import quasi_gb300 as q


def _decode(words: np.ndarray, i: int):
    """Per slot: (lo[3], hi[3]) decoded exactly in float64, ref, internal flag."""
    w = words[i]
    p = w[0:3].view(np.float32).astype(np.float64)
    ex = [(int(w[3]) >> (8 * a)) & 0xFF for a in range(3)]
    imask = int(w[3]) >> 24
    out = []
    for s in range(8):
        lo, hi = np.zeros(3), np.zeros(3)
        for a in range(3):
            words_a = w[4 + 4 * a: 8 + 4 * a]
            qlo = (int(words_a[s >> 2]) >> (8 * (s & 3))) & 0xFF
            qhi = (int(words_a[2 + (s >> 2)]) >> (8 * (s & 3))) & 0xFF
            scale = 2.0 ** (ex[a] - 127)
            lo[a] = p[a] + qlo * scale
            hi[a] = p[a] + qhi * scale
        out.append((lo, hi, int(w[16:24].view(np.int32)[s]), bool((imask >> s) & 1)))
    return out


def _tri_boxes(vertices: np.ndarray, order: np.ndarray):
    v = vertices.reshape(-1, 3, 3)[order].astype(np.float64)
    return v.min(axis=1), v.max(axis=1)


def _subtree_range(children: np.ndarray, node: int) -> tuple[int, int]:
    lo, hi, todo = None, None, [node]
    while todo:
        c = todo.pop()
        for k in (0, 1):
            ch = int(children[2 * c + k])
            if ch < 0:
                lo = ~ch if lo is None else min(lo, ~ch)
                hi = ~ch if hi is None else max(hi, ~ch)
            else:
                todo.append(ch)
    return lo, hi


@pytest.mark.parametrize("spec", ["cornell36", "refcornell", "soup:n=1,seed=1", "soup:n=2,seed=1",
                                  "soup:n=5000,seed=9"])
def test_collapse8_covers_and_contains(orc, spec):
    sc = q.make_scene(spec)
    n = sc.tri_count
    words = orc.collapse8(sc.vertices)
    lb = orc.lbvh(sc.vertices)
    tlo, thi = _tri_boxes(sc.vertices, lb["order"])
    cover = np.zeros(n, np.int64)
    for i in orc.wide_reachable(words):
        for lo, hi, ref, internal in _decode(words, i):
            if internal:
                a, b = _subtree_range(lb["children"], ref)
                assert b - a + 1 > 1  # every leaf holds one triangle
            else:
                x = (~ref) & 0xFFFFFFFF
                cnt = ((x & 3) + 1) & 3
                if cnt == 0:
                    # empty slot: inverted box (on a zero-extent axis of the node the grid
                    # step is 2^-100 and both planes decode to the origin); no triangles
                    assert (lo > hi).any() or (lo == hi).all()
                    continue
                a, b = x >> 2, (x >> 2) + cnt - 1
                cover[a:b + 1] += 1
            assert (lo <= tlo[a:b + 1].min(axis=0)).all() and (hi >= thi[a:b + 1].max(axis=0)).all()
    if n == 1:
        assert cover[0] == 2  # the one-triangle tree lists its triangle under both children
    else:
        assert (cover == 1).all()


def test_collapse8_is_deterministic(orc):
    sc = q.make_scene("soup:n=20000,seed=4")
    assert np.array_equal(orc.collapse8(sc.vertices), orc.collapse8(sc.vertices))


def test_collapse8_degenerate_axes(orc):
    """Flat and coincident triangles: zero-extent axes get the smallest grid and still
    contain their children."""
    rng = np.random.default_rng(3)
    flat = rng.random((500, 9), np.float32)
    flat[:, 1::3] = 0.25
    same = np.tile(rng.random((1, 9), np.float32), (40, 1))
    for v in (flat, same):
        words = orc.collapse8(v)
        lb = orc.lbvh(v)
        tlo, thi = _tri_boxes(v, lb["order"])
        for i in orc.wide_reachable(words):
            for lo, hi, ref, internal in _decode(words, i):
                if internal:
                    a, b = _subtree_range(lb["children"], ref)
                else:
                    x = (~ref) & 0xFFFFFFFF
                    cnt = ((x & 3) + 1) & 3
                    if cnt == 0:
                        continue
                    a, b = x >> 2, (x >> 2) + cnt - 1
                assert (lo <= tlo[a:b + 1].min(axis=0)).all() and (hi >= thi[a:b + 1].max(axis=0)).all()
