"""The parity statistics helper (tests/parity_stats.py) on planted data (CPU): divergent
pixels are kept out of the max and percentile, and counted apart."""
from __future__ import annotations

import numpy as np
import pytest

pr = pytest.importorskip("tests.parity_stats", reason="needs the tests package importable")


def test_error_stats_split_divergent_pixels():
    rng = np.random.default_rng(0)
    n, spp = 50, 4
    o_samp = rng.uniform(0.1, 1.0, (n, spp, 3))
    o_mean = o_samp.mean(1)
    o_sig = rng.integers(0, 1 << 30, (n, spp))
    g_samp = o_samp * (1.0 + 1e-6)
    g_mean = g_samp.mean(1)
    g_sig = o_sig.copy()
    # pixel 3: one sample took another path and its mean is far off
    g_sig[3, 1] ^= 1
    g_samp[3, 1] *= 2.0
    g_mean[3] = g_samp[3].mean(0)
    # pixel 7: agreeing paths but a 1e-3 error
    g_mean[7] *= 1.0 + 1e-3
    st = pr.error_stats(g_mean, g_samp, g_sig, o_mean, o_samp, o_sig, spp)
    assert st["pixels"] == n and st["samples"] == n * spp
    assert st["divergent_pixels"] == 1 and st["divergent_samples"] == 1
    assert st["pixels_over_1e-4_divergent"] == 1
    assert st["pixels_over_1e-4_non_divergent"] == 1
    assert st["max_rel_err"] == pytest.approx((1 + 1e-6) * (1 + 1e-3) - 1, rel=1e-6)
    assert st["max_sample_rel_err"] < 2e-6
