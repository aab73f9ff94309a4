"""Error statistics of a GPU render against the FP64 oracle at matched seeds (a test helper).

Per pixel, the relative error |gpu - oracle| / max(|oracle|, 1e-3) (worst channel): its
maximum and 99.99th percentile over pixels whose path signatures all agree with the oracle's,
the pixels above 1e-4 split into path-divergent and non-divergent ones, and the divergent
samples. The GPU parity tests print these statistics for each workload
(python -m pytest tests/test_gpu_render.py -m gpu -s -k parity).
"""
from __future__ import annotations

import numpy as np

FLOOR = 1e-3
TOL = 1e-4

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
