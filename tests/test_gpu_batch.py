"""Scene batches (Q_cuda_batch_*): every scene of a batch renders bit-identically to the same
scene rendered alone through the plugin, whatever the batch form (wavefront or megakernel),
wave size, block size, fetch size and launch mode (CUDA graph or plain launches); the batch
adjoint equals the single-scene adjoint per scene."""
from __future__ import annotations

import numpy as np
import pytest

import quasi_gb300 as q

pytestmark = pytest.mark.gpu

DEPTH = 6
# (spec, width, height, spp): uneven triangle counts, sizes that are not multiples of the
# 8x4 pixel tile, and spp that splits across waves. "needles" is a scene of long thin
# triangles whose rays stack past the shared-memory part of the traversal stacks.
SCENES = [
    ("soup:n=1000,seed=1", 64, 64, 4),
    ("soup:n=20000,seed=2", 96, 54, 16),
    ("soup:n=3000,seed=3", 128, 128, 3),
    ("soup:n=150000,seed=4", 200, 120, 5),
    ("cornell36", 64, 64, 8),
    ("needles", 48, 40, 4),
]


def _needles(n=20000, seed=4, width=0.01) -> q.Scene:
    """Long thin triangles across the unit cube: large overlapping boxes, rare hits."""
    rng = np.random.default_rng(seed)
    a = rng.random((n, 3)) * 0.9 + 0.05
    b = rng.random((n, 3)) * 0.9 + 0.05
    d = rng.normal(0.0, 1.0, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    v = np.concatenate([a, b, a + d * width], axis=1).astype(np.float32)
    emission = np.zeros((n, 3), np.float32)
    emission[::31] = (4.0, 3.5, 3.0)
    cam = {"position": (0.5, 0.5, -1.0), "target": (0.5, 0.5, 0.5), "fov": 40.0}
    return q.Scene(v, np.full((n, 3), 0.7, np.float32), emission, cam)


@pytest.fixture(scope="module")
def scenes(cuda_ok):
    return [(_needles() if spec == "needles" else q.make_scene(spec), w, h, spp) for spec, w, h, spp in SCENES]


@pytest.fixture(scope="module")
def single(scenes):
    """Two progressive frames of every scene rendered alone: images after frame 1 and 2, and
    the rays each frame traced."""
    out = []
    for sc, w, h, spp in scenes:
        host = q.PluginHost(width=w, height=h)
        host.set_scene(sc)
        host.set_options(spp_per_frame=spp, max_depth=DEPTH, seed=0)
        host.render(w, h, dirty=True)
        img1 = host.readback()
        st = host.stats()
        host.render(w, h)
        img2 = host.readback()
        out.append((img1, img2, st.camera_rays + st.extension_rays, st.shadow_rays))
        host.destroy()
    return out


def _check_batch(host, scenes, single, **opts):
    with q.Batch(host, scenes, max_depth=DEPTH, **opts) as b:
        b.render()
        b.synchronize()
        first = [b.readback(i) for i in range(len(scenes))]
        st = b.stats()
        b.render()
        b.synchronize()
        second = [b.readback(i) for i in range(len(scenes))]
        for i, (ref1, ref2, _, _) in enumerate(single):
            assert np.array_equal(first[i], ref1), (opts, SCENES[i], np.abs(first[i] - ref1).max())
            assert np.array_equal(second[i], ref2), (opts, SCENES[i])
        assert st.error_flags == 0
        assert st.frames == 1
        assert st.closest_rays == sum(s[2] for s in single)
        assert st.shadow_rays == sum(s[3] for s in single)
        assert st.camera_rays == sum(w * h * spp for _, w, h, spp in scenes)
        return st


def test_batch_equals_single_scene_renders(scenes, single):
    host = q.PluginHost()
    st = _check_batch(host, scenes, single)
    assert st.scenes == len(scenes) and st.waves == 1 and st.kernels_per_frame == 2 + 5 * DEPTH + 2
    host.destroy()


def test_batch_waves_split_samples_and_scenes(scenes, single):
    """Waves of 32768 path slots: scenes split across waves and several scenes share a wave."""
    host = q.PluginHost()
    st = _check_batch(host, scenes, single, wave_paths=32768)
    assert st.waves > len(scenes)
    host.destroy()


@pytest.mark.parametrize("opts", [
    dict(form=1),
    dict(form=1, wave_paths=40000, fetch_rays=64, trace_block=64),
    dict(use_graph=2),
    dict(use_graph=2, form=1),
    dict(trace_block=256, fetch_rays=128, wave_paths=50000),
    dict(collect_stats=1),
    dict(refill_lanes=1),
    dict(refill_lanes=32, trace_block=64),
    dict(bvh_width=2),
    dict(bvh_width=2, fetch_rays=64, collect_stats=1),
])
def test_batch_forms_and_launch_modes(scenes, single, opts):
    host = q.PluginHost()
    st = _check_batch(host, scenes, single, **opts)
    if opts.get("collect_stats"):
        assert st.node_visits > st.closest_rays and st.tri_tests > 0
    host.destroy()


def test_batch_autotune_keeps_images(scenes, single):
    host = q.PluginHost()
    with q.Batch(host, scenes, max_depth=DEPTH, wave_paths=32768) as b:
        chosen = b.autotune(budget_ms=3000)
        assert chosen.form in (0, 1)
        assert chosen.trace_block in (64, 128, 256) and chosen.fetch_rays in (32, 64, 128)
        assert chosen.bvh_width == 8 and chosen.refill_lanes in (4, 8, 16)
        o = b.options()
        assert (o.form, o.trace_block, o.fetch_rays, o.wave_paths, o.refill_lanes) == (
            chosen.form, chosen.trace_block, chosen.fetch_rays, chosen.wave_paths, chosen.refill_lanes)
        b.render()
        b.synchronize()
        for i, (ref1, _, _, _) in enumerate(single):
            assert np.array_equal(b.readback(i), ref1)
    host.destroy()


def test_batch_backward_matches_single_scene_adjoint(scenes):
    torch = pytest.importorskip("torch")
    from quasi_gb300 import autograd as qa

    picked = [scenes[0], scenes[1], scenes[4]]
    rng = np.random.default_rng(5)
    host = q.PluginHost(stream=qa.torch_stream_handle())
    stream = qa.torch_stream_handle()
    with q.Batch(host, picked, max_depth=4) as b:
        st = b.stats()
        b.render(stream)
        img = torch.empty((st.px_total, 3), dtype=torch.float32, device="cuda")
        b.resolve_device(img.data_ptr(), stream)
        g = torch.tensor(rng.normal(size=(st.px_total, 3)).astype(np.float32), device="cuda")
        ga = torch.empty((st.tri_total, 3), dtype=torch.float32, device="cuda")
        ge = torch.empty_like(ga)
        b.backward(g.data_ptr(), ga.data_ptr(), ge.data_ptr(), stream)
        torch.cuda.synchronize()
        for i, (sc, w, h, spp) in enumerate(picked):
            t0, p0 = b.offsets(i)
            n = sc.tri_count
            single = qa.make_host(sc, w, h, max_depth=4, seed=0)
            alb = torch.tensor(sc.albedo, device="cuda")
            emi = torch.tensor(sc.emission, device="cuda")
            ref_img = qa.render(alb, emi, single, w, h, spp)
            assert torch.equal(ref_img.reshape(-1, 3), img[p0:p0 + w * h]), picked[i][1:]
            gs = g[p0:p0 + w * h].reshape(h, w, 3).contiguous()
            ra = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            re = torch.empty_like(ra)
            rc = single.lib.Q_cuda_backward(single.handle, gs.data_ptr(), spp, 0, ra.data_ptr(), re.data_ptr(), stream)
            assert rc == 0
            torch.cuda.synchronize()
            # float atomics add in a different order: equal to rounding of sums whose terms
            # cancel (random-signed image gradient), so the absolute tolerance scales with the
            # largest gradient entry of the scene
            torch.testing.assert_close(ga[t0:t0 + n], ra, rtol=1e-4, atol=1e-4 * float(ra.abs().max()) + 1e-9)
            torch.testing.assert_close(ge[t0:t0 + n], re, rtol=1e-4, atol=1e-4 * float(re.abs().max()) + 1e-9)
            single.destroy()
    host.destroy()


def test_batch_rejects_bad_input(scenes):
    host = q.PluginHost()
    sc = scenes[0][0]
    with pytest.raises(q.QuasiError):
        q.Batch(host, [(sc, 64, 64, 0)])
    with pytest.raises(q.QuasiError):
        q.Batch(host, [(sc, 64, 64, 1)], trace_block=48)
    with pytest.raises(q.QuasiError):
        q.Batch(host, [(sc, 64, 64, 1)], fetch_rays=40)
    with pytest.raises(q.QuasiError):
        q.Batch(host, [(sc, 64, 64, 1)], bvh_width=4)
    with pytest.raises(q.QuasiError):
        q.Batch(host, [(sc, 64, 64, 1)], refill_lanes=33)
    with q.Batch(host, [(sc, 64, 64, 1)], max_depth=4) as b:
        with pytest.raises(q.QuasiError) as e:
            b.backward(1, None, None)  # nothing rendered since the reset
        assert e.value.code == -6
    host.destroy()


def test_batch_fit_recovers_albedo(scenes):
    """Batched differentiation: Adam on the albedo of 3 scenes. Every step re-seeds the batch
    and renders its target from the true albedo with that seed, so the fit sees new paths each
    step (with one fixed set of paths the image constrains products of the albedos along them,
    not each albedo). The loss falls and the albedo error of the triangles seen falls."""
    torch = pytest.importorskip("torch")
    from quasi_gb300 import autograd as qa

    picked = [scenes[0], scenes[1], scenes[2]]
    host, batch = qa.make_batch(picked, max_depth=4)
    gt = torch.tensor(np.concatenate([sc.albedo for sc, *_ in picked]), device="cuda")
    em = torch.tensor(np.concatenate([sc.emission for sc, *_ in picked]), device="cuda")
    rng = np.random.default_rng(11)
    init = torch.tensor(np.clip(gt.cpu().numpy() + rng.normal(0, 0.1, gt.shape), 0.05, 0.95).astype(np.float32),
                        device="cuda")
    with torch.no_grad():
        target = qa.render_batch(gt, em, batch).clone()
    a0 = init.clone().requires_grad_(True)
    ((qa.render_batch(a0, em, batch) - target) ** 2).mean().backward()
    seen = a0.grad.abs().sum(dim=1) > 0
    assert int(seen.sum()) > 50
    fitted, losses = qa.fit_albedo(batch, None, init, em, steps=40, lr=0.01, target_albedo=gt, seed0=1)
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])

    def rmse(a, m):
        return float(((a - gt)[m] ** 2).mean().sqrt())

    print(f"albedo RMSE over seen triangles {rmse(init, seen):.4f} -> {rmse(fitted, seen):.4f}")
    assert rmse(fitted, seen) < 0.7 * rmse(init, seen), (rmse(init, seen), rmse(fitted, seen))
    st = batch.stats()
    assert st.error_flags == 0 and st.adjoint_rays > 0
    batch.destroy()
    host.destroy()
