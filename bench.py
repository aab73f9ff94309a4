"""Benchmark: Mrays/s of the plain renderer on the 1M-triangle soup at 1080p, 64 spp, depth 8.

One step = one Q_plugin_render frame of 64 samples per pixel with the LBVH rebuilt on the GPU
(30-bit Morton codes, 32-bit key radix sort, Karras hierarchy) followed by the wavefront
path tracer. Each step uses its own seed; nothing is cached between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` is device-timed (CUDA events on the plugin's stream,
inputs resident in HBM); `e2e` times the same frames through the plugin C ABI with the scene
uploaded from pinned host memory and the HDR image read back into host memory every step.
The reference arm (--impl reference) times the CPU oracle on the host cores: the reference's
own renderer is Metal shader code that cannot run on this machine.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s at 1080p 64spp 1M tris; batched & backward Mrays/s at rel err≤1e-4"
SCENE = "soup:n=1000000,seed=0"
WIDTH, HEIGHT, SPP, DEPTH = 1920, 1080, 64, 8
WORKLOAD = "soup-1M 1920x1080 64spp depth8 NEE, LBVH rebuilt every frame"
# a shadow ray reads 48 of its 64 queue bytes (the origin lo parts only when re-decided)
TRI_BYTES, RAY_BYTES, HIT_BYTES, SHADOW_BYTES = 48, 32, 16, 48
NODE_BYTES = {2: 64, 8: 96}  # binary LBVH node / 8-wide record


def workload_config() -> dict:
    """The workload both arms time (the same dict in both JSON lines)."""
    return {"workload": WORKLOAD, "scene": SCENE, "tri_count": 1000000, "width": WIDTH, "height": HEIGHT, "spp": SPP,
            "max_depth": DEPTH, "lbvh": "built in every step, inside the timed region",
            "l2": "GPU arm: 256 MiB write before every step, inside the timed region; CPU arm: not applicable"}


def _peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"quasi_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in self.path.read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def replica_totals(total_ms: float, rays: int, device) -> tuple[float, int]:
    """Replicas: every rank renders its own frames (own seeds), nothing is exchanged on the
    data path. The job's time is the slowest rank's and its rays are every rank's."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return total_ms, rays
    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    r = torch.tensor([float(rays)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(r)
    return float(t.item()), int(r.item())


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample(scene, precision: int = 32, target_s: float = 12.0, seed: int = 0, threads: int | None = None):
    """Times the CPU oracle on a bounded sample of the benchmark frame: one oracle call that
    builds its LBVH (Morton codes, sort, hierarchy, as the GPU arm does every frame) and
    renders random pixels with all 64 samples each; the build is inside the timed call.
    Returns (Mrays/s, cores, description)."""
    import numpy as np

    from oracle import oracle as orc

    threads = threads or orc.hardware_threads()
    rng = np.random.default_rng(seed)
    # calibration: the build alone (a 1-pixel, 1-sample call), then 4096 pixels at full spp
    calib = rng.choice(WIDTH * HEIGHT, size=4096, replace=False).astype(np.uint32)
    t0 = time.perf_counter()
    orc.render_nee(scene, WIDTH, HEIGHT, 1, 1, seed=seed, precision=precision, threads=threads, pixels=calib[:1])
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    orc.render_nee(scene, WIDTH, HEIGHT, SPP, DEPTH, seed=seed, precision=precision, threads=threads, pixels=calib)
    per_pixel = max(time.perf_counter() - t0 - build_s, 1e-3) / calib.size
    npix = int(min(WIDTH * HEIGHT, max(1024, (target_s - build_s) / per_pixel)))
    pix = rng.choice(WIDTH * HEIGHT, size=npix, replace=False).astype(np.uint32)
    t0 = time.perf_counter()
    out = orc.render_nee(scene, WIDTH, HEIGHT, SPP, DEPTH, seed=seed, precision=precision, threads=threads,
                         pixels=pix)
    dt = time.perf_counter() - t0
    rays = sum(out["rays"].values())
    desc = (f"{npix} random pixels of the 1920x1080 frame x 64 spp, depth 8 (soup-1M built by the oracle's own "
            f"generator), FP{precision} oracle on {threads} threads; {rays} rays in {dt:.2f} s, LBVH build "
            f"(~{build_s:.2f} s) included")
    return rays / dt / 1e6, threads, desc


def bench_batch(host, stream, flush, steps: int, warmup: int, budget_ms: float, small: bool = False) -> dict:
    """Batching workload: 64 soup scenes (seeds 1..64, 1e3..5e5 triangles, 64^2..1024^2 pixels,
    4/16/64 spp, depth 6) rendered as one batch (one graph launch per frame, autotuned),
    against the same frames as 64 plain plugin renders, one scene after the other.
    small: 64 scenes that each leave the GPU mostly idle when rendered alone (seeds 1..64,
    1e3..5e4 triangles, 64^2 or 128^2 pixels, 4 spp, depth 6)."""
    import torch

    import quasi_gb300 as q
    from quasi_gb300 import workloads

    if small:
        scenes = workloads.BATCH_64_SMALL.scenes(host.lib)
        label = "64 soup scenes, seeds 1..64, log-uniform 1e3..5e4 triangles, 64^2..128^2 pixels, 4 spp, depth 6"
    else:
        scenes = workloads.BATCH_64.scenes(host.lib)
        label = "64 soup scenes, seeds 1..64, log-uniform 1e3..5e5 triangles, 64^2..1024^2 pixels, spp 4/16/64, depth 6"
    depth = 6
    res = {"workload": label + ", BVHs built once",
           "tri_total": sum(s.tri_count for s, *_ in scenes),
           "px_total": sum(w * h for _, w, h, _ in scenes),
           "samples_per_frame": sum(w * h * spp for _, w, h, spp in scenes)}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h = stream.cuda_stream
    with q.Batch(host, scenes, max_depth=depth) as b:
        t0 = time.perf_counter()
        chosen = b.autotune(budget_ms)
        res["autotune_s"] = time.perf_counter() - t0
        res["autotuned"] = {"form": ["wavefront", "megakernel"][chosen.form], "wave_paths": chosen.wave_paths,
                            "trace_block": chosen.trace_block, "fetch_rays": chosen.fetch_rays,
                            "refill_lanes": chosen.refill_lanes, "bvh_width": chosen.bvh_width}
        for _ in range(warmup):
            b.render(h)
        b.synchronize()
        st0 = b.stats()
        ev0.record(stream)
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            b.render(h)
        ev1.record(stream)
        torch.cuda.synchronize()
        st1 = b.stats()
        ms = ev0.elapsed_time(ev1) / steps
        rays = (st1.rays - st0.rays) / steps
        res.update(value=rays / ms / 1e3, unit="Mrays/s", ms_per_frame=ms, rays_per_frame=rays, waves=st1.waves,
                   kernels_per_frame=st1.kernels_per_frame, error_flags=st1.error_flags)
    # the same frames as 64 plain renders (LBVH built once per scene, as in the batch)
    hosts = []
    try:
        for sc, w, hh, spp in scenes:
            ph = q.PluginHost(device=torch.cuda.current_device(), stream=h, width=w, height=hh)
            ph.set_scene(sc)
            ph.set_options(spp_per_frame=spp, max_depth=depth, seed=0, rebuild_each_frame=0)
            hosts.append(ph)
        for _ in range(warmup):
            for ph in hosts:
                ph.render(dirty=False, stream=h)
        torch.cuda.synchronize()
        r0 = sum(ph.stats().total_rays for ph in hosts)
        ev0.record(stream)
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            for ph in hosts:
                ph.render(dirty=False, stream=h)
        ev1.record(stream)
        torch.cuda.synchronize()
        r1 = sum(ph.stats().total_rays for ph in hosts)
        pms = ev0.elapsed_time(ev1) / steps
        prays = (r1 - r0) / steps
        res.update(plain_value=prays / pms / 1e3, plain_ms_per_frame=pms, plain_rays_per_frame=prays,
                   speedup=(rays / ms) / (prays / pms) if prays else None)
    finally:
        for ph in hosts:
            ph.destroy()
    return res


def bench_diff(stream, steps: int, fit_steps: int) -> dict:
    """Differentiation workloads: (a) forward vs adjoint cost on the 10,000-triangle soup
    (seed 7), 512x512, 16 spp, depth 4; (b) 32 soup scenes (seeds 101..132, 2e3..1e5
    triangles, 128^2..512^2 pixels, 8 spp, depth 4) fitted by Adam (lr 0.01) from albedo
    perturbed by N(0, 0.1) clamped to [0.05, 0.95], one forward and one adjoint graph launch
    per step."""
    import numpy as np
    import torch

    import quasi_gb300 as q
    from quasi_gb300 import autograd as qa
    from quasi_gb300 import workloads

    out = {}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with torch.cuda.stream(stream):
        # (a) adjoint cost
        scene = q.make_scene("soup:n=10000,seed=7")
        w = hh = 512
        spp = 16
        host = qa.make_host(scene, w, hh, max_depth=4, seed=0)
        alb = torch.tensor(scene.albedo, device="cuda", requires_grad=True)
        emi = torch.tensor(scene.emission, device="cuda", requires_grad=True)
        rng = np.random.default_rng(7)
        tgt_alb = np.clip(scene.albedo + rng.normal(0.0, 0.1, scene.albedo.shape), 0.05, 0.95).astype(np.float32)
        with torch.no_grad():
            target = qa.render(torch.tensor(tgt_alb, device="cuda"), emi.detach(), host, w, hh, spp).clone()
        fwd_ms, bwd_ms = [], []
        r_f = r_b = 0
        for i in range(2 + steps):
            s0 = host.stats()
            ev[0].record()
            img = qa.render(alb, emi, host, w, hh, spp)
            loss = ((img - target) ** 2).sum()
            ev[1].record()
            loss.backward()
            ev[2].record()
            torch.cuda.synchronize()
            s1 = host.stats()
            alb.grad = None
            emi.grad = None
            if i >= 2:
                fwd_ms.append(ev[0].elapsed_time(ev[1]))
                bwd_ms.append(ev[1].elapsed_time(ev[2]))
                r_f += s1.total_rays - s0.total_rays
                r_b += s1.adjoint_rays - s0.adjoint_rays
        host.destroy()
        f, bk = sum(fwd_ms), sum(bwd_ms)
        out["adjoint"] = {"workload": "soup-10k seed 7, 512x512, 16 spp, depth 4, L2 loss",
                          "forward_ms": f / steps, "adjoint_ms": bk / steps, "adjoint_over_forward": bk / f,
                          "forward_mrays_s": r_f / f / 1e3, "adjoint_mrays_s": r_b / bk / 1e3,
                          "rays_forward": r_f / steps, "rays_adjoint": r_b / steps}
        # (b) batched differentiation
        lib = q.load_library()
        scenes = workloads.BATCH_DIFF_32.scenes(lib)
        bhost, batch = qa.make_batch(scenes, max_depth=4, seed=0)
        gt = torch.tensor(np.concatenate([sc.albedo for sc, *_ in scenes]), device="cuda")
        em = torch.tensor(np.concatenate([sc.emission for sc, *_ in scenes]), device="cuda")
        rng = np.random.default_rng(2024)
        init = torch.tensor(np.clip(gt.cpu().numpy() + rng.normal(0.0, 0.1, gt.shape), 0.05, 0.95).astype(np.float32),
                            device="cuda")
        with torch.no_grad():
            target = qa.render_batch(gt, em, batch).clone()
        # triangles the images depend on: nonzero albedo gradient at the start
        a0 = init.clone().requires_grad_(True)
        ((qa.render_batch(a0, em, batch) - target) ** 2).mean().backward()
        seen = (a0.grad.abs().sum(dim=1) > 0)
        st0 = batch.stats()
        ev[0].record()
        fitted, losses = qa.fit_albedo(batch, None, init, em, steps=fit_steps, lr=0.01, target_albedo=gt, seed0=1)
        ev[1].record()
        torch.cuda.synchronize()
        st1 = batch.stats()
        ms = ev[0].elapsed_time(ev[1])
        rays = (st1.rays - st0.rays) + (st1.adjoint_rays - st0.adjoint_rays)

        def rmse(a, m=None):
            d = (a - gt) if m is None else (a - gt)[m]
            return float(torch.sqrt((d ** 2).mean()))

        out["batched_fit"] = {
            "workload": "32 soup scenes, seeds 101..132, log-uniform 2e3..1e5 triangles, 128^2..512^2 pixels, "
                        "8 spp, depth 4, Adam lr 0.01; every step re-seeded, its target rendered from the true "
                        "albedo with the step's seed (rays of both forwards and the adjoint counted)",
            "steps": fit_steps, "tri_total": int(gt.shape[0]), "px_total": int(st1.px_total),
            "mrays_s_forward_plus_adjoint": rays / ms / 1e3, "ms_per_step": ms / fit_steps,
            "rmse_init_all": rmse(init), "rmse_final_all": rmse(fitted),
            "triangles_seen": int(seen.sum()), "rmse_init_seen": rmse(init, seen), "rmse_final_seen": rmse(fitted, seen),
            "loss_first": losses[0], "loss_last": losses[-1], "graph_launches_per_step": 3}
        batch.destroy()
        bhost.destroy()
    return out


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import oracle as orc

    scene = orc.make_scene(SCENE)  # the oracle's own generator: nothing of the product is loaded
    threads = orc.hardware_threads()
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, desc = cpu_sample(scene, precision=32, target_s=args.ref_seconds, seed=i, threads=threads)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference renderer is a Metal shader (macOS graphics API) and cannot run here; "
                    "this arm times the CPU oracle port of the same algorithm"}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch

    import quasi_gb300 as q

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    host = q.PluginHost(device=local, stream=stream.cuda_stream, width=WIDTH, height=HEIGHT)
    scene = q.make_scene(SCENE, host.lib)
    host.set_scene(scene)
    opts = dict(spp_per_frame=SPP, max_depth=DEPTH, rebuild_each_frame=1, record_samples=0, wave_spp=args.wave_spp,
                trace_block=args.trace_block, bvh_width=args.bvh_width, refill_lanes=args.refill_lanes)
    node_bytes = NODE_BYTES[2 if args.bvh_width == 2 else 8]
    host.set_options(seed=0, **opts)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step(i: int) -> None:
        host.set_options(seed=1000 * rank + i, **opts)
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush: 256 MiB write (L2 is 126 MiB)
        host.render(WIDTH, HEIGHT, dirty=True, stream=stream.cuda_stream)

    # algorithmic bytes: one untimed frame with traversal counters on
    host.set_options(seed=999_999, collect_stats=1, **opts)
    host.render(WIDTH, HEIGHT, dirty=True, stream=stream.cuda_stream)
    cs = host.stats()
    host.set_options(seed=0, collect_stats=0, **opts)
    closest_rays = cs.camera_rays + cs.extension_rays
    alg_closest = closest_rays * (RAY_BYTES + HIT_BYTES) + cs.node_visits * node_bytes + cs.tri_tests * TRI_BYTES
    alg_shadow = cs.shadow_rays * SHADOW_BYTES + cs.shadow_node_visits * node_bytes + cs.shadow_tri_tests * TRI_BYTES

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    host.kernel_times(reset=True)
    host.set_options(seed=0, profile=1, **opts)
    opts["profile"] = 1
    rays0 = host.stats().total_rays
    with ClockSampler(local) as clocks:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for i in range(args.steps):
            step(args.warmup + i)
        ev1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
    st = host.stats()
    launches = st.kernel_launches * args.steps
    total_ms = ev0.elapsed_time(ev1)
    rays = st.total_rays - rays0
    times = host.kernel_times(reset=True)
    opts["profile"] = 0
    host.set_options(seed=0, **opts)
    total_ms, rays = replica_totals(total_ms, rays, "cuda")
    value = rays / (total_ms / 1e3) / 1e6

    # end to end through the plugin ABI: pinned host scene upload + render + host readback
    e2e = None
    if not args.no_e2e:
        vert_pinned = torch.from_numpy(np.ascontiguousarray(scene.vertices)).pin_memory()
        e2e_steps = max(2, min(args.steps, 3))
        torch.cuda.synchronize()
        r0 = host.stats().total_rays
        t0 = time.perf_counter()
        for i in range(e2e_steps):
            host.set_options(seed=50_000 + i, **opts)
            host.update_vertices(vert_pinned.data_ptr(), scene.tri_count)
            host.render(WIDTH, HEIGHT, dirty=True, stream=stream.cuda_stream)
            img = host.readback()
        e2e_s = time.perf_counter() - t0
        e2e_rays = host.stats().total_rays - r0
        e2e = {"value": e2e_rays / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": int(scene.vertices.nbytes),
               "d2h_bytes_per_step": int(img.nbytes), "steps": e2e_steps,
               "path": "Q_cuda_update_vertices(pinned host) + Q_plugin_render + Q_plugin_readback"}

    # roofline of the dominant kernel
    peak, peak_kind = _peaks()
    top = max(times.items(), key=lambda kv: kv[1][1]) if times else ("trace_closest", (1, 1.0))
    name, (n_launch, kms) = top
    frames = args.steps
    alg = {"trace_closest": alg_closest, "trace_shadow": alg_shadow}.get(name)
    achieved = (alg * frames / (kms / 1e3) / 1e9) if alg is not None and kms > 0 else None
    # DRAM traffic per launch: bytes per ray from a committed ncu capture (a smaller image of
    # the same scene) times the rays of an average launch here
    traffic = traffic_note = None
    tf = ROOT / "profiles" / "trace_traffic.json"
    rays_of = {"trace_closest": closest_rays, "trace_shadow": cs.shadow_rays}
    if tf.exists() and name in rays_of:
        try:
            entry = json.loads(tf.read_text()).get(name)
            if entry:
                traffic = entry["dram_bytes_per_ray"] * rays_of[name] * frames / n_launch
                traffic_note = entry["source"] + "; " + entry["scaling"]
        except Exception:
            traffic = None
    frame_ms = total_ms / args.steps
    share = {k: round(v[1] / max(sum(x[1] for x in times.values()), 1e-9), 4) for k, v in times.items()}
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "traffic_source": traffic_note,
                "alg_bytes_per_launch": (alg * frames / n_launch) if alg else None,
                "avg_launch_ms": kms / n_launch, "launches": n_launch, "kernel_share": share,
                "bytes_model": f"closest: rays*(32+16) + node_visits*{node_bytes} + tri_tests*48; shadow: rays*48 + "
                               f"node_visits*{node_bytes} + tri_tests*48 (counted in an untimed frame)",
                "per_ray": {"closest_node_visits": cs.node_visits / max(closest_rays, 1),
                            "closest_tri_tests": cs.tri_tests / max(closest_rays, 1),
                            "shadow_node_visits": cs.shadow_node_visits / max(cs.shadow_rays, 1),
                            "shadow_tri_tests": cs.shadow_tri_tests / max(cs.shadow_rays, 1)}}

    batch = diff = None
    if rank == 0 and not args.no_batch:
        batch = bench_batch(host, stream, flush, steps=2, warmup=1, budget_ms=args.tune_ms)
        batch["small_scenes"] = bench_batch(host, stream, flush, steps=3, warmup=1, budget_ms=min(args.tune_ms, 2000.0),
                                            small=True)
    if rank == 0 and not args.no_diff:
        diff = bench_diff(stream, steps=3, fit_steps=args.fit_steps)

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc

        v, cores, desc = cpu_sample(orc.make_scene(SCENE), precision=32, target_s=args.ref_seconds)
        cpu = {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": frame_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(),
                "details": {"rays_per_step": rays / args.steps / world, "bvh_ms": st.bvh_ms,
                            "redecided_rays_per_step": st.redecided_rays, "parallelism": f"replicas x{world}",
                            "wave_spp": args.wave_spp, "trace_block": args.trace_block,
                            "refill_lanes": args.refill_lanes,
                            "bvh": ("binary LBVH" if args.bvh_width == 2 else "8-wide records collapsed from the LBVH")
                                   + " (30% of the triangles split into two leaf references; subtrees of <= 32 "
                                     "leaves rebuilt with the SAH split; records from the SAH-optimal spread)"},
                "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
                "clocks": clocks.summary(), "batch": batch, "diff": diff}
        print(json.dumps(line), flush=True)
    host.destroy()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--wave-spp", type=int, default=0)
    ap.add_argument("--trace-block", type=int, default=0)
    ap.add_argument("--refill-lanes", type=int, default=0,
                    help="trace kernels refill a warp once this many lanes are idle (0 = library default)")
    ap.add_argument("--bvh-width", type=int, default=0, choices=[0, 2, 8],
                    help="traversal structure: 8-wide records (0, 8) or the binary LBVH (2)")
    ap.add_argument("--ref-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batching workload")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation workloads")
    ap.add_argument("--tune-ms", type=float, default=5000.0, help="batch autotuner budget")
    ap.add_argument("--fit-steps", type=int, default=100, help="Adam steps of the batched fit")
    # Size overrides, for profiling captures on a small case only (not benchmark numbers).
    ap.add_argument("--width", type=int, default=WIDTH)
    ap.add_argument("--height", type=int, default=HEIGHT)
    ap.add_argument("--spp", type=int, default=SPP)
    args = ap.parse_args()
    globals().update(WIDTH=args.width, HEIGHT=args.height, SPP=args.spp)
    if (args.width, args.height, args.spp) != (1920, 1080, 64):
        globals()["WORKLOAD"] = f"soup-1M {args.width}x{args.height} {args.spp}spp depth8 (profiling case)"
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
