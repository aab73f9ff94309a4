"""The headless C++ host (quasi_gb300/host): CUDA GPU context, plugin loading through the C ABI,
update + render frames, readback and AOV readback written as OpenEXR, and a hot reload
(destroy, dlclose, copy, dlopen, create) that must reproduce the image bit for bit."""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest
from exr_format import parse_exr

import quasi_gb300 as q
from quasi_gb300 import build as qbuild

pytestmark = pytest.mark.gpu


def _run(*args):
    exe = qbuild.HEADLESS
    assert exe.exists(), "quasi_headless is built by __graft_entry__.build()"
    p = subprocess.run([str(exe), "--lib", str(q.DEFAULT_LIBRARY), *args], capture_output=True, text=True,
                       timeout=300)
    return p.returncode, json.loads(p.stdout.strip().splitlines()[-1])


def test_headless_renders_writes_exr_and_hot_reloads(cuda_ok, tmp_path):
    w, h, spp, frames = 96, 64, 4, 2
    rc, out = _run("--scene", "cornell36", "--width", str(w), "--height", str(h), "--spp", str(spp), "--depth", "4",
                   "--frames", str(frames), "--exr", str(tmp_path / "beauty.exr"), "--aov-exr",
                   str(tmp_path / "aov.exr"), "--reload")
    assert rc == 0, out
    assert out["ok"] and out["abi"] == 3 and out["name"] == "CUDA Path Tracer"
    assert out["reload"] == {"loaded": True, "identical": True, "checksum": out["checksum"]}
    # the same frames through the Python host
    host = q.PluginHost(width=w, height=h)
    host.set_scene(q.make_scene("cornell36", host.lib))
    host.set_options(spp_per_frame=spp, max_depth=4, seed=0)
    for f in range(frames):
        host.render(w, h, dirty=(f == 0))
    ref = host.readback()
    aov = host.readback_aov()
    host.destroy()
    # the host sums the mean in double
    assert np.allclose(np.array(out["mean"]), ref[..., :3].reshape(-1, 3).astype(np.float64).mean(0), rtol=1e-6)
    half = lambda a: a.astype(np.float16).astype(np.float32)  # noqa: E731
    _, ch = parse_exr(tmp_path / "beauty.exr")
    for k, c in enumerate("RGBA"):
        assert np.array_equal(ch[c], half(ref[..., k]))
    _, ch = parse_exr(tmp_path / "aov.exr")
    for k, c in enumerate("RGB"):
        assert np.array_equal(ch[c], half(aov["beauty"][..., k]))
        assert np.array_equal(ch[f"albedo.{c}"], half(aov["albedo"][..., k]))
    for k, c in enumerate("XYZ"):
        assert np.array_equal(ch[f"normal.{c}"], half(aov["normal"][..., k]))
    assert np.array_equal(ch["depth.Z"], aov["depth"][..., 0])


def test_headless_reports_load_errors(cuda_ok, tmp_path):
    p = subprocess.run([str(qbuild.HEADLESS), "--lib", str(tmp_path / "missing.so")], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 2
    assert json.loads(p.stdout.strip())["load_error"] == "file_not_found"
