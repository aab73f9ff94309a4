"""Path-replay adjoint: gradients of an L2 image loss with respect to per-triangle albedo
against central finite differences (eps 1e-3) of the GPU forward renderer; plus
megakernel/wavefront identity. The FP64 oracle gradient and the emission differences are
checked at the differentiation configuration in test_gpu_configs.py.

Tolerance: relative error <= 1e-3 on every checked gradient entry.
"""
from __future__ import annotations

import numpy as np
import pytest

import quasi_gb300 as q

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-3


def _perturbed_target_albedo(albedo: np.ndarray, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.clip(albedo + rng.normal(0.0, 0.1, albedo.shape), 0.05, 0.95).astype(np.float32)


@pytest.fixture(scope="module")
def torch_mod(cuda_ok):
    import torch

    return torch


def _setup(torch, spec, w, h, spp, depth):
    from quasi_gb300 import autograd as qa

    scene = q.make_scene(spec)
    host = qa.make_host(scene, w, h, max_depth=depth, seed=0)
    albedo = torch.tensor(scene.albedo, device="cuda", requires_grad=True)
    emission = torch.tensor(scene.emission, device="cuda", requires_grad=True)
    target_alb = torch.tensor(_perturbed_target_albedo(scene.albedo, 7), device="cuda")
    with torch.no_grad():
        target = qa.render(target_alb, emission.detach(), host, w, h, spp).clone()
    return qa, scene, host, albedo, emission, target


def test_adjoint_matches_central_finite_differences(torch_mod):
    """The differentiation configuration: 10,000-triangle soup (seed 7), 512x512, 16 spp,
    depth 4, L2 loss against a target rendered with Gaussian-perturbed albedo; 64 random
    gradient entries checked against central differences with eps 1e-3."""
    torch = torch_mod
    w = h = 512
    spp, depth = 16, 4
    qa, scene, host, albedo, emission, target = _setup(torch, "soup:n=10000,seed=7", w, h, spp, depth)
    img = qa.render(albedo, emission, host, w, h, spp)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    ga = albedo.grad.cpu().numpy().astype(np.float64)
    tgt = target.double()

    def loss_at(alb: torch.Tensor) -> float:
        with torch.no_grad():
            im = qa.render(alb, emission.detach(), host, w, h, spp).double()
            return float(((im - tgt) ** 2).sum())

    rng = np.random.default_rng(3)
    # Central differences of an FP32 image resolve a gradient only above the image's rounding
    # noise (an entry at 1e-3 of the largest gradient already shows 2e-3 relative noise), so
    # the 64 entries are drawn from those above 1e-2 of the largest.
    cand = np.argwhere(np.abs(ga) > 1e-2 * np.abs(ga).max())
    picks = cand[rng.choice(len(cand), size=min(64, len(cand)), replace=False)]
    assert len(picks) == 64
    errs = []
    for tri, ch in picks:
        base = albedo.detach().clone()
        plus, minus = base.clone(), base.clone()
        plus[tri, ch] += 1e-3
        minus[tri, ch] -= 1e-3
        denom = float(plus[tri, ch]) - float(minus[tri, ch])
        fd = (loss_at(plus) - loss_at(minus)) / denom
        errs.append(abs(ga[tri, ch] - fd) / max(abs(fd), 1e-30))
    errs = np.array(errs)
    assert errs.max() <= GRAD_TOL, np.sort(errs)[-5:]
    host.destroy()


def test_megakernel_equals_wavefront(cuda_ok):
    """Both forms share the per-vertex code: per-sample radiance and signatures are identical."""
    for spec, w, h, spp, depth in (("cornell36", 64, 64, 8, 4), ("soup:n=50000,seed=2", 96, 54, 4, 8)):
        host = q.PluginHost(width=w, height=h)
        host.set_scene(q.make_scene(spec, host.lib))
        outs = []
        for mk in (0, 1):
            host.set_options(spp_per_frame=spp, max_depth=depth, seed=3, record_samples=1, megakernel=mk)
            host.render(w, h, dirty=True)
            img = host.readback()
            rad, sig = host.read_samples(spp)
            st = host.stats()
            assert st.error_flags == 0
            outs.append((img, rad, sig, st.camera_rays, st.extension_rays, st.shadow_rays))
        assert np.array_equal(outs[0][0], outs[1][0])
        assert np.array_equal(outs[0][1], outs[1][1])
        assert np.array_equal(outs[0][2], outs[1][2])
        assert outs[0][3:] == outs[1][3:]
        host.destroy()
