"""torch.autograd binding of the renderer: image = render(albedo, emission).

Forward sets the per-triangle materials from device tensors (Q_cuda_set_materials_device),
renders `spp` samples per pixel through the plugin and resolves the mean HDR image into a
torch tensor. Backward calls the path-replay adjoint (Q_cuda_backward), which regenerates
the same paths from their RNG keys and returns dLoss/dalbedo and dLoss/demission.

render_batch does the same for a scene batch (Q_cuda_batch_*): one captured graph renders
every scene, one captured graph runs the adjoint of every scene; materials and images are
the batch pools (scenes back to back). fit_albedo drives Adam with it.

Every plugin call is issued on torch's current CUDA stream, so the tensors it reads and
writes are ordered with the surrounding torch work without extra synchronisation. torch's
default stream has the handle 0, which the plugin ABI reads as "use your own stream"; it is
passed as cudaStreamLegacy (1) instead.
"""
from __future__ import annotations

import ctypes as C

import torch

from .host import Batch, PluginHost, QuasiError

CUDA_STREAM_LEGACY = 1


def torch_stream_handle() -> int:
    """cudaStream_t of torch's current stream, usable by the plugin (never 0)."""
    return torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY


def _check(host: PluginHost, call: str, rc: int) -> None:
    if rc != 0:
        raise QuasiError(call, rc, host.lib.Q_cuda_last_error(host.handle).decode(errors="replace"))


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo: torch.Tensor, emission: torch.Tensor, host: PluginHost, width: int, height: int,
                spp: int, sample_base: int):
        if not (albedo.is_cuda and emission.is_cuda):
            raise ValueError("albedo and emission must be CUDA tensors")
        a = albedo.detach().float().contiguous()
        e = emission.detach().float().contiguous()
        n = a.shape[0]
        lib = host.lib
        _check(host, "Q_cuda_set_materials_device",
               lib.Q_cuda_set_materials_device(host.handle, C.c_void_p(a.data_ptr()), C.c_void_p(e.data_ptr()), n))
        host.set_options(spp_per_frame=spp)
        host.render(width, height, dirty=True, stream=torch_stream_handle())
        out = torch.empty((height, width, 4), dtype=torch.float32, device=albedo.device)
        _check(host, "Q_cuda_resolve_device", lib.Q_cuda_resolve_device(host.handle, C.c_void_p(out.data_ptr())))
        ctx.host, ctx.spp, ctx.sample_base, ctx.n = host, spp, sample_base, n
        ctx.keep = (a, e)
        return out[..., :3]

    @staticmethod
    def backward(ctx, grad_image: torch.Tensor):
        host = ctx.host
        g = grad_image.detach().float().contiguous()
        ga = torch.empty((ctx.n, 3), dtype=torch.float32, device=g.device)
        ge = torch.empty((ctx.n, 3), dtype=torch.float32, device=g.device)
        _check(host, "Q_cuda_backward",
               host.lib.Q_cuda_backward(host.handle, C.c_void_p(g.data_ptr()), ctx.spp, ctx.sample_base,
                                        C.c_void_p(ga.data_ptr()), C.c_void_p(ge.data_ptr()),
                                        C.c_void_p(torch_stream_handle())))
        return ga, ge, None, None, None, None, None


def make_host(scene, width: int, height: int, max_depth: int = 4, seed: int = 0, **options) -> PluginHost:
    """A plugin instance on torch's current stream with `scene` loaded (NEE integrator)."""
    host = PluginHost(stream=torch_stream_handle(), width=width, height=height)
    host.set_scene(scene)
    host.set_options(max_depth=max_depth, seed=seed, **options)
    return host


def render(albedo: torch.Tensor, emission: torch.Tensor, host: PluginHost, width: int, height: int, spp: int,
           sample_base: int = 0) -> torch.Tensor:
    """Differentiable render: returns the (height, width, 3) mean image of `spp` samples."""
    return RenderFunction.apply(albedo, emission, host, width, height, spp, sample_base)


class BatchRenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo: torch.Tensor, emission: torch.Tensor, batch: Batch, px_total: int):
        if not (albedo.is_cuda and emission.is_cuda):
            raise ValueError("albedo and emission must be CUDA tensors")
        a = albedo.detach().float().contiguous()
        e = emission.detach().float().contiguous()
        stream = torch_stream_handle()
        batch.set_materials_device(a.data_ptr(), e.data_ptr(), stream)
        batch.render(stream)
        out = torch.empty((px_total, 3), dtype=torch.float32, device=albedo.device)
        batch.resolve_device(out.data_ptr(), stream)
        ctx.batch, ctx.n = batch, a.shape[0]
        ctx.keep = (a, e)
        return out

    @staticmethod
    def backward(ctx, grad_image: torch.Tensor):
        g = grad_image.detach().float().contiguous()
        ga = torch.empty((ctx.n, 3), dtype=torch.float32, device=g.device)
        ge = torch.empty((ctx.n, 3), dtype=torch.float32, device=g.device)
        ctx.batch.backward(g.data_ptr(), ga.data_ptr(), ge.data_ptr(), torch_stream_handle())
        return ga, ge, None, None


def make_batch(scenes, max_depth: int = 4, seed: int = 0, **options) -> tuple[PluginHost, Batch]:
    """A plugin instance on torch's current stream and a batch of `scenes`
    [(Scene, width, height, spp), ...]."""
    host = PluginHost(stream=torch_stream_handle())
    batch = Batch(host, scenes, max_depth=max_depth, seed=seed, **options)
    return host, batch


def render_batch(albedo: torch.Tensor, emission: torch.Tensor, batch: Batch) -> torch.Tensor:
    """Differentiable render of every scene: returns the (px_total, 3) pool of mean images
    (scene after scene, rows top first); albedo/emission are (tri_total, 3)."""
    return BatchRenderFunction.apply(albedo, emission, batch, int(batch.stats().px_total))


def fit_albedo(batch: Batch, target: torch.Tensor | None, albedo0: torch.Tensor, emission: torch.Tensor,
               steps: int = 100, lr: float = 0.01, target_albedo: torch.Tensor | None = None,
               seed0: int = 0) -> tuple[torch.Tensor, list[float]]:
    """Adam on the per-triangle albedo of every scene of the batch against target images
    (L2 loss, mean over pixels and channels); albedo is kept in [0, 1] after each step.
    Adam's eps is 1e-15: the gradients of these mostly dark images are ~1e-10, far below the
    usual 1e-8, which would otherwise shrink every step by that ratio.
    With target_albedo, every step k draws new paths: the batch is re-seeded with seed0 + k
    and the target is rendered from target_albedo with that seed before the fitted image, so
    both see the same paths (target is then unused). Otherwise every step renders the same
    samples against the fixed target.
    Returns the fitted albedo and the loss of every step."""
    albedo = albedo0.detach().clone().requires_grad_(True)
    opt = torch.optim.Adam([albedo], lr=lr, eps=1e-15)
    px = int(batch.stats().px_total)
    stream = torch_stream_handle()
    losses = []
    for k in range(steps):
        opt.zero_grad(set_to_none=True)
        if target_albedo is not None:
            batch.set_seed(seed0 + k, stream)
            with torch.no_grad():
                target = BatchRenderFunction.apply(target_albedo, emission, batch, px).clone()
        img = BatchRenderFunction.apply(albedo, emission, batch, px)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        opt.step()
        with torch.no_grad():
            albedo.clamp_(0.0, 1.0)
        losses.append(loss.detach())
    return albedo.detach(), [float(v) for v in losses]
