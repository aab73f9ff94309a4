"""Error statistics of the GPU renderer against the FP64 oracle at matched seeds, per
workload: the per-pixel relative error |gpu - oracle| / max(|oracle|, 1e-3) (worst channel),
its maximum and 99.99th percentile over pixels whose path signatures all agree with the
oracle's, the pixels above 1e-4 split into path-divergent and non-divergent ones, and the
divergent samples. Needs a CUDA GPU; prints one JSON object per workload.

    python tests/parity_report.py

The parity tests (test_gpu_render.py) assert the same bounds; this script reports them.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import quasi_gb300 as q  # noqa: E402
from oracle import oracle as orc  # noqa: E402

FLOOR = 1e-3
TOL = 1e-4

# (name, scene spec, width, height, spp, depth, seed, sampled pixels or None for all)
WORKLOADS = [
    ("cornell36 256x256 16spp depth4", "cornell36", 256, 256, 16, 4, 0, None),
    ("refcornell 96x72 8spp depth5", "refcornell", 96, 72, 8, 5, 7, None),
    ("soup-100k 320x180 4spp depth8 (1500 random pixels)", "soup:n=100000,seed=1", 320, 180, 4, 8, 3, 1500),
    ("soup-1M 1920x1080 64spp depth8 (300 random pixels)", "soup:n=1000000,seed=0", 1920, 1080, 64, 8, 17, 300),
]


def error_stats(g_img, g_rad, g_sig, o_mean, o_samp, o_sig, spp: int) -> dict:
    """Statistics over n pixels: g_img (n, 3) GPU pixel means, g_rad (n, spp, 3) GPU samples,
    g_sig (n, spp) GPU path signatures, and the oracle's o_mean, o_samp, o_sig alike."""
    g_img = np.asarray(g_img, np.float64).reshape(-1, 3)
    g_rad = np.asarray(g_rad, np.float64).reshape(-1, spp, 3)
    o_mean = np.asarray(o_mean, np.float64).reshape(-1, 3)
    o_samp = np.asarray(o_samp, np.float64).reshape(-1, spp, 3)
    match = np.asarray(g_sig).reshape(-1, spp) == np.asarray(o_sig).reshape(-1, spp)
    px_ok = match.all(-1)
    p_err = (np.abs(g_img - o_mean) / np.maximum(np.abs(o_mean), FLOOR)).max(-1)
    s_err = (np.abs(g_rad - o_samp) / np.maximum(np.abs(o_samp), FLOOR)).max(-1)
    ok = p_err[px_ok]
    return {
        "pixels": int(px_ok.size),
        "samples": int(match.size),
        "max_rel_err": float(ok.max()) if ok.size else 0.0,
        "p99.99_rel_err": float(np.quantile(ok, 0.9999)) if ok.size else 0.0,
        "max_sample_rel_err": float(s_err[match].max()) if match.any() else 0.0,
        "pixels_over_1e-4_non_divergent": int((ok > TOL).sum()),
        "pixels_over_1e-4_divergent": int((p_err[~px_ok] > TOL).sum()),
        "divergent_pixels": int((~px_ok).sum()),
        "divergent_samples": int((~match).sum()),
    }


def report(name, spec, w, h, spp, depth, seed, n_pix) -> dict:
    host = q.PluginHost(width=w, height=h)
    scene = q.make_scene(spec, host.lib)
    host.set_scene(scene)
    host.set_options(spp_per_frame=spp, max_depth=depth, seed=seed, record_samples=1)
    host.render(w, h, dirty=True)
    img = host.readback()
    rad, sig = host.read_samples(spp)
    st = host.stats()
    host.destroy()
    if n_pix is None:
        pix = np.arange(w * h, dtype=np.uint32)
        ref = orc.render_nee(scene, w, h, spp, depth, seed=seed, want_samples=True)
    else:
        pix = np.random.default_rng(5).choice(w * h, size=n_pix, replace=False).astype(np.uint32)
        ref = orc.render_nee(scene, w, h, spp, depth, seed=seed, pixels=pix, want_samples=True)
    ys, xs = pix // w, pix % w
    out = {"workload": name}
    out.update(error_stats(img[ys, xs, :3], rad[ys, xs], sig[ys, xs], ref["mean"], ref["samples"], ref["sig"], spp))
    out["error_flags"] = int(st.error_flags)
    return out


def main() -> None:
    orc.build()
    for wl in WORKLOADS:
        print(json.dumps(report(*wl)), flush=True)


if __name__ == "__main__":
    main()
