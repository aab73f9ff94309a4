"""The differentiation, batch and batched-differentiation configurations against the FP64
oracle (not against the product's own single-scene renderer):

* adjoint: the 10,000-triangle soup (seed 7) at 512x512, 16 spp, depth 4, L2 loss against a
  target rendered with Gaussian-perturbed albedo: every albedo and emission gradient entry
  above 1e-3 of the largest against the oracle's analytic FP64 gradient, and 64 seeded
  emission entries against central finite differences (eps 1e-3);
* batch: the 64-scene batch (seeds 1..64, 1e3..5e5 triangles, 64^2..1024^2 pixels, 4/16/64
  spp, depth 6) rendered as one batch; the 3 largest scenes (the largest of these seeds has
  380,382 triangles) and every 1024^2 scene checked on 2,000 random pixels each against the
  oracle;
* batched differentiation: the 32-scene batch (seeds 101..132, 2e3..1e5 triangles,
  128^2..512^2 pixels, 8 spp, depth 4); the batch adjoint of the smallest and the largest
  scene against the oracle's gradient.

Tolerances: per-pixel relative error |gpu - oracle| / max(|oracle|, 1e-3) <= 1e-4; gradient
entries within 1e-3 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import workloads

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4
GRAD_TOL = 1e-3


@pytest.fixture(scope="module")
def torch_mod(cuda_ok):
    import torch

    return torch


def _grad_errors(got: np.ndarray, ref: np.ndarray, floor_frac: float = 1e-3):
    big = np.abs(ref) > floor_frac * np.abs(ref).max()
    rel = np.abs(got[big] - ref[big]) / np.abs(ref[big])
    return int(big.sum()), rel


def test_adjoint_config_matches_fp64_oracle_gradient(torch_mod, orc):
    torch = torch_mod
    from quasi_gb300 import autograd as qa

    w = h = 512
    spp, depth = 16, 4
    scene = q.make_scene("soup:n=10000,seed=7")
    host = qa.make_host(scene, w, h, max_depth=depth, seed=0)
    rng = np.random.default_rng(7)
    tgt_alb = np.clip(scene.albedo + rng.normal(0.0, 0.1, scene.albedo.shape), 0.05, 0.95).astype(np.float32)
    albedo = torch.tensor(scene.albedo, device="cuda", requires_grad=True)
    emission = torch.tensor(scene.emission, device="cuda", requires_grad=True)
    with torch.no_grad():
        target = qa.render(torch.tensor(tgt_alb, device="cuda"), emission.detach(), host, w, h, spp).clone()
    img = qa.render(albedo, emission, host, w, h, spp)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    ga = albedo.grad.cpu().numpy().astype(np.float64)
    ge = emission.grad.cpu().numpy().astype(np.float64)
    grad_image = (2.0 * (img - target)).detach().cpu().numpy().astype(np.float64)
    oa, oe = orc.backward(scene, w, h, spp, depth, grad_image, seed=0)
    for got, ref, name in ((ga, oa, "albedo"), (ge, oe, "emission")):
        n, rel = _grad_errors(got, ref)
        print(f"{name}: {n} entries above 1e-3 of the largest, max rel err {rel.max():.2e}, "
              f"median {np.median(rel):.2e}")
        assert n > 100, name
        assert rel.max() <= GRAD_TOL, (name, np.sort(rel)[-5:])
    host.destroy()


def test_adjoint_emission_matches_central_finite_differences(torch_mod):
    """64 seeded emission entries against central differences (eps 1e-3). The image is
    linear in emission, so the differences are exact up to the FP32 image's rounding, which
    hides gradients below ~1e-2 of the largest; the entries are drawn from those above it."""
    torch = torch_mod
    from quasi_gb300 import autograd as qa

    w = h = 512
    spp, depth = 16, 4
    scene = q.make_scene("soup:n=10000,seed=7")
    host = qa.make_host(scene, w, h, max_depth=depth, seed=0)
    rng = np.random.default_rng(7)
    tgt_alb = np.clip(scene.albedo + rng.normal(0.0, 0.1, scene.albedo.shape), 0.05, 0.95).astype(np.float32)
    albedo = torch.tensor(scene.albedo, device="cuda")
    emission = torch.tensor(scene.emission, device="cuda", requires_grad=True)
    with torch.no_grad():
        target = qa.render(torch.tensor(tgt_alb, device="cuda"), emission.detach(), host, w, h, spp).clone()
    img = qa.render(albedo, emission, host, w, h, spp)
    ((img - target) ** 2).sum().backward()
    ge = emission.grad.cpu().numpy().astype(np.float64)
    tgt = target.double()

    def loss_at(em: torch.Tensor) -> float:
        with torch.no_grad():
            im = qa.render(albedo, em, host, w, h, spp).double()
            return float(((im - tgt) ** 2).sum())

    cand = np.argwhere(np.abs(ge) > 1e-2 * np.abs(ge).max())
    picks = cand[np.random.default_rng(64).choice(len(cand), size=64, replace=False)]
    errs = []
    for tri, ch in picks:
        base = emission.detach().clone()
        plus, minus = base.clone(), base.clone()
        plus[tri, ch] += 1e-3
        minus[tri, ch] -= 1e-3
        denom = float(plus[tri, ch]) - float(minus[tri, ch])
        fd = (loss_at(plus) - loss_at(minus)) / denom
        errs.append(abs(ge[tri, ch] - fd) / max(abs(fd), 1e-30))
    errs = np.array(errs)
    print(f"emission vs central differences: max rel err {errs.max():.2e} over {len(errs)} entries "
          f"({len(cand)} candidates)")
    assert errs.max() <= GRAD_TOL, np.sort(errs)[-5:]
    host.destroy()


def test_batch_config_matches_oracle(cuda_ok, orc):
    scenes = workloads.BATCH_64.scenes()
    host = q.PluginHost()
    with q.Batch(host, scenes, max_depth=workloads.BATCH_64.depth) as b:
        b.render()
        b.synchronize()
        st = b.stats()
        assert st.error_flags == 0 and st.scenes == 64
        largest = sorted(range(len(scenes)), key=lambda i: scenes[i][0].tri_count)[-3:]
        big_images = [i for i, (_, w, h, _) in enumerate(scenes) if w * h == 1024 * 1024]
        assert big_images
        for i in sorted(set(largest) | set(big_images)):
            sc, w, h, spp = scenes[i]
            img = b.readback(i)[..., :3].astype(np.float64)
            pix = np.random.default_rng(i).choice(w * h, size=min(2000, w * h), replace=False).astype(np.uint32)
            ref = orc.render_nee(sc, w, h, spp, workloads.BATCH_64.depth, seed=0, pixels=pix)
            ys, xs = pix // w, pix % w
            err = (np.abs(img[ys, xs] - ref["mean"]) / np.maximum(np.abs(ref["mean"]), 1e-3)).max(-1)
            print(f"scene {i}: {sc.tri_count} triangles, {w}x{h}, {spp} spp: max rel err {err.max():.2e}")
            assert err.max() <= REL_TOL, (i, np.sort(err)[-5:])
    host.destroy()


def test_batched_adjoint_config_matches_oracle(torch_mod, orc):
    torch = torch_mod
    from quasi_gb300 import autograd as qa

    wl = workloads.BATCH_DIFF_32
    scenes = wl.scenes()
    host, batch = qa.make_batch(scenes, max_depth=wl.depth)
    stream = qa.torch_stream_handle()
    batch.render(stream)
    st = batch.stats()
    g = torch.tensor(np.random.default_rng(32).normal(size=(st.px_total, 3)).astype(np.float32), device="cuda")
    ga = torch.empty((st.tri_total, 3), dtype=torch.float32, device="cuda")
    ge = torch.empty_like(ga)
    batch.backward(g.data_ptr(), ga.data_ptr(), ge.data_ptr(), stream)
    torch.cuda.synchronize()
    assert batch.stats().error_flags == 0
    order = sorted(range(len(scenes)), key=lambda i: scenes[i][0].tri_count)
    for i in (order[0], order[-1]):
        sc, w, h, spp = scenes[i]
        t0, p0 = batch.offsets(i)
        n = sc.tri_count
        gi = g[p0:p0 + w * h].cpu().numpy().astype(np.float64).reshape(h, w, 3)
        oa, oe = orc.backward(sc, w, h, spp, wl.depth, gi, seed=0)
        for got, ref, name in ((ga[t0:t0 + n], oa, "albedo"), (ge[t0:t0 + n], oe, "emission")):
            cnt, rel = _grad_errors(got.cpu().numpy().astype(np.float64), ref)
            print(f"scene {i} ({n} triangles, {w}x{h}) {name}: {cnt} entries, max rel err {rel.max():.2e}")
            assert cnt > 20, (i, name)
            assert rel.max() <= GRAD_TOL, (i, name, np.sort(rel)[-5:])
    batch.destroy()
    host.destroy()
