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
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES, SHADOW_BYTES = 64, 48, 32, 16, 48


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


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample(scene, precision: int = 32, target_s: float = 12.0, seed: int = 0, threads: int | None = None):
    """Times the CPU oracle on a bounded sample of the benchmark frame (random pixels, all
    64 samples each). Returns (Mrays/s, cores, description)."""
    import numpy as np

    from oracle import oracle as orc

    threads = threads or orc.hardware_threads()
    rng = np.random.default_rng(seed)
    calib = rng.choice(WIDTH * HEIGHT, size=64, replace=False).astype(np.uint32)
    t0 = time.perf_counter()
    orc.render_nee(scene, WIDTH, HEIGHT, 4, DEPTH, seed=seed, precision=precision, threads=threads, pixels=calib)
    build_and_calib = time.perf_counter() - t0
    # one oracle call rebuilds its LBVH; time it separately on a 1-pixel render
    t0 = time.perf_counter()
    orc.render_nee(scene, WIDTH, HEIGHT, 1, 1, seed=seed, precision=precision, threads=threads, pixels=calib[:1])
    build_s = time.perf_counter() - t0
    per_pixel_4spp = max(build_and_calib - build_s, 1e-3) / calib.size
    npix = int(min(WIDTH * HEIGHT, max(64, target_s / (per_pixel_4spp * SPP / 4))))
    pix = rng.choice(WIDTH * HEIGHT, size=npix, replace=False).astype(np.uint32)
    t0 = time.perf_counter()
    out = orc.render_nee(scene, WIDTH, HEIGHT, SPP, DEPTH, seed=seed, precision=precision, threads=threads,
                         pixels=pix)
    dt = time.perf_counter() - t0 - build_s
    rays = sum(out["rays"].values())
    desc = (f"{npix} random pixels of the 1920x1080 frame x 64 spp, depth 8 (soup-1M), FP{precision} oracle on "
            f"{threads} threads; {rays} rays in {dt:.2f} s (LBVH build {build_s:.2f} s excluded)")
    return rays / dt / 1e6, threads, desc


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    import quasi_gb300 as q
    from oracle import oracle as orc

    scene = q.make_scene(SCENE)
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
            "config": {"workload": WORKLOAD, "tri_count": 1000000, "width": WIDTH, "height": HEIGHT, "spp": SPP,
                       "max_depth": DEPTH, "sample": "bounded pixel sample per step"},
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
                trace_block=args.trace_block)
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
    alg_closest = closest_rays * (RAY_BYTES + HIT_BYTES) + cs.node_visits * NODE_BYTES + cs.tri_tests * TRI_BYTES
    alg_shadow = cs.shadow_rays * SHADOW_BYTES + cs.shadow_node_visits * NODE_BYTES + cs.shadow_tri_tests * TRI_BYTES

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
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], device="cuda")
        r = torch.tensor([float(rays)], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(r)
        total_ms, rays = float(t.item()), int(r.item())
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
    traffic = None
    tf = ROOT / "profiles" / "trace_traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(name)
        except Exception:
            traffic = None
    frame_ms = total_ms / args.steps
    share = {k: round(v[1] / max(sum(x[1] for x in times.values()), 1e-9), 4) for k, v in times.items()}
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "alg_bytes_per_launch": (alg * frames / n_launch) if alg else None,
                "avg_launch_ms": kms / n_launch, "launches": n_launch, "kernel_share": share,
                "bytes_model": "closest: rays*(32+16) + node_visits*64 + tri_tests*48; shadow: rays*48 + node_visits*64 + tri_tests*48 (counted in an untimed frame)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, desc = cpu_sample(scene, precision=32, target_s=args.ref_seconds)
        cpu = {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": desc}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": frame_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "tri_count": scene.tri_count, "width": WIDTH, "height": HEIGHT,
                           "spp": SPP, "max_depth": DEPTH, "rays_per_step": rays / args.steps / world,
                           "bvh_ms": st.bvh_ms, "l2": "flushed before every step (256 MiB write, inside the "
                           "timed region)", "parallelism": f"replicas x{world}", "wave_spp": args.wave_spp,
                           "trace_block": args.trace_block},
                "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
                "clocks": clocks.summary()}
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
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
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
