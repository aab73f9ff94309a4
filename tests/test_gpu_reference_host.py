"""The drop-in claim on the GPU: libquasi_cuda.so driven by the reference host's own, unchanged
plugin code (src/quasi/plugin/loader.hpp and manager.hpp, the async scheduler of
src/quasi/async), as the host drives backends/metal.

tests/reference_host_probe.cpp is compiled against those headers, which the oracle's build
recipe copies from the reference checkout into the git-ignored oracle/_ref/include (the GPU
machine has no checkout; the test is skipped only when they were not staged).

* loader: create with a CUDA context, three progressive frames, readback and readback_aov
  and their *_free: the beauty and every AOV equal the Python host's render bit for bit.
* manager: load_sync, frames into a device RGBA8 drawable, a newer library file, the
  manager's watch loop ticked on the reference scheduler until it has reloaded (destroy,
  dlclose, copy to a temporary file, dlopen, create; the pre_unload hook synchronises the
  host's stream), the same frames again: identical tonemapped images, one successful reload.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import quasi_gb300 as q
from quasi_gb300 import build as qbuild

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
STAGED = ROOT / "oracle" / "_ref" / "include"
W, H, FRAMES = 96, 64, 3
ENV = {"QUASI_SCENE": "cornell36", "QUASI_SPP": "4", "QUASI_DEPTH": "4", "QUASI_SEED": "3"}


@pytest.fixture(scope="module")
def probe(tmp_path_factory, cuda_ok):
    if not (STAGED / "quasi" / "plugin" / "manager.hpp").exists():
        pytest.skip("the reference host headers were not staged into oracle/_ref/include")
    qbuild.build()
    d = tmp_path_factory.mktemp("refhost")
    exe = d / "probe"
    cuda = qbuild.CUDA_HOME
    libdir = qbuild._cuda_lib_dir()
    subprocess.run(["g++", "-std=c++23", "-O1", "-I", str(STAGED), "-I", str(cuda / "include"),
                    str(ROOT / "tests" / "reference_host_probe.cpp"), "-o", str(exe), "-L", str(libdir),
                    f"-Wl,-rpath,{libdir}", "-lcudart", "-ldl", "-pthread"], check=True)
    return exe


def _run(probe, mode: str, lib: Path, out: Path) -> str:
    env = dict(os.environ, **ENV)
    p = subprocess.run([str(probe), mode, str(lib), str(FRAMES), str(W), str(H), str(out)], capture_output=True,
                       text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    return p.stdout


def test_reference_loader_renders_and_reads_back(probe, tmp_path):
    out = tmp_path / "loader.bin"
    log = _run(probe, "loader", q.DEFAULT_LIBRARY, out)
    assert "loaded abi=3 readback=1 aov=1" in log, log
    got = np.fromfile(out, dtype=np.float32).reshape(4, H, W, 4)
    host = q.PluginHost(width=W, height=H)
    host.set_scene(q.make_scene("cornell36", host.lib))
    host.set_options(spp_per_frame=4, max_depth=4, seed=3)
    for f in range(FRAMES):
        host.render(W, H, dirty=(f == 0))
    beauty = host.readback()
    aov = host.readback_aov()
    host.destroy()
    assert np.array_equal(got[0], beauty)
    for k, name in enumerate(("albedo", "normal", "depth"), start=1):
        assert np.array_equal(got[k], aov[name]), name
    assert beauty[..., :3].max() > 0.0


def test_reference_manager_hot_reloads_the_plugin(probe, tmp_path):
    lib = tmp_path / "libquasi_cuda.so"
    shutil.copy2(q.DEFAULT_LIBRARY, lib)
    out = tmp_path / "manager.bin"
    log = _run(probe, "manager", lib, out)
    assert "reloads=1 success=1 failure=0 pre_unload=1 loaded=1" in log, log
    imgs = np.fromfile(out, dtype=np.uint8).reshape(2, H, W, 4)
    assert imgs[0].any()
    assert np.array_equal(imgs[0], imgs[1])
