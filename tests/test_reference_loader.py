"""The reference host's own plugin loader binds libquasi_cuda.so (no GPU needed).

A probe is compiled against the reference checkout's src/quasi/plugin/loader.hpp and
dynamic_library.hpp (unchanged, read where they lie; skipped when the checkout is absent)
and loads our library the way the host loads libquasi_metal. Without a GPU the plugin's
create fails after symbol resolution and the ABI check, so the loader must report
create_failed (not symbol_not_found or abi_mismatch) and the plugin must have logged why
through the host's log callback.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

import quasi_gb300 as q

REF = Path(os.environ.get("REF", "/root/reference"))

PROBE = r"""
#include <quasi/plugin/loader.hpp>
#include <cstdio>
#include <cstdlib>

static void log_fn(void*, const char* m) { std::printf("log: %s\n", m); }

int main(int argc, char** argv) {
    auto lib = Q::plugin::dynamic_library::open(argv[1]);
    if (!lib) { std::printf("open_failed\n"); return 1; }
    int ordinal = 0;
    Q_gpu_context gpu{};
    gpu.backend = static_cast<Q_gpu_backend>(std::atoi(argv[2]));
    gpu.device = &ordinal;
    Q::plugin::plugin_context ctx{};
    ctx.viewport_width = 64;
    ctx.viewport_height = 64;
    ctx.gpu = &gpu;
    ctx.log = log_fn;
    auto p = Q::plugin::loader::load(*lib, &ctx);
    if (p) {
        std::printf("loaded abi=%u readback=%d aov=%d\n", p->abi_version(), int(p->supports_readback()),
                    int(p->supports_readback_aov()));
        return 0;
    }
    switch (p.error()) {
        case Q::plugin::loader::error::abi_mismatch: std::printf("abi_mismatch\n"); break;
        case Q::plugin::loader::error::symbol_not_found: std::printf("symbol_not_found\n"); break;
        case Q::plugin::loader::error::create_failed: std::printf("create_failed\n"); break;
    }
    return 2;
}
"""


@pytest.fixture(scope="module")
def probe(tmp_path_factory, qlib):
    if not (REF / "src" / "quasi" / "plugin" / "loader.hpp").exists():
        pytest.skip("reference checkout not present")
    d = tmp_path_factory.mktemp("refloader")
    src = d / "probe.cpp"
    src.write_text(PROBE)
    exe = d / "probe"
    subprocess.run(["g++", "-std=c++23", "-O1", "-I", str(REF / "src"), str(src), "-o", str(exe), "-ldl"],
                   check=True)
    return exe


def test_reference_loader_resolves_symbols_and_accepts_abi(probe):
    out = subprocess.run([str(probe), str(q.DEFAULT_LIBRARY), "4"], capture_output=True, text=True).stdout
    lines = out.splitlines()
    # no GPU here: create fails after resolution + ABI check, and says why through ctx.log
    assert lines[-1] == "create_failed", out
    assert any(line.startswith("log: ") and "CUDA" in line for line in lines), out


def test_reference_loader_sees_backend_check(probe):
    out = subprocess.run([str(probe), str(q.DEFAULT_LIBRARY), "1"], capture_output=True, text=True).stdout
    lines = out.splitlines()
    assert lines[-1] == "create_failed", out
    assert any("backend" in line for line in lines if line.startswith("log: ")), out
