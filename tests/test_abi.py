"""The C ABI boundary, checked without a GPU: exports, struct layouts, loader behaviour."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import quasi_gb300 as q
from quasi_gb300 import _abi as A

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "quasi_cuda.h"


def _declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"Q_CUDA_EXPORT\s+[^;(]*?\b(Q_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(qlib):
    names = _declared_functions()
    assert "Q_plugin_render" in names and "Q_cuda_make_scene" in names
    out = subprocess.run(["nm", "-D", "--defined-only", str(q.DEFAULT_LIBRARY)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert getattr(qlib, n) is not None


def test_only_plugin_and_extension_symbols_are_exported(qlib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(q.DEFAULT_LIBRARY)], capture_output=True, text=True,
                         check=True).stdout
    exported = [line.split()[-1] for line in out.splitlines() if " T " in line]
    stray = [s for s in exported if not s.startswith(("Q_plugin_", "Q_cuda_")) and not s.startswith("_")]
    assert not stray, stray


def test_struct_layouts_match_c_compiler(tmp_path):
    """The ctypes mirrors and the C header agree on every size and offset."""
    probe = tmp_path / "probe.c"
    structs = {"Q_gpu_context": A.Q_gpu_context, "Q_camera": A.Q_camera, "Q_render_frame": A.Q_render_frame,
               "Q_plugin_info": A.Q_plugin_info, "Q_plugin_context": A.Q_plugin_context,
               "Q_readback_result": A.Q_readback_result, "Q_aov_buffer": A.Q_aov_buffer,
               "Q_readback_aov_result": A.Q_readback_aov_result, "Q_cuda_scene": A.Q_cuda_scene,
               "Q_cuda_options": A.Q_cuda_options, "Q_cuda_stats": A.Q_cuda_stats,
               "Q_cuda_kernel_time": A.Q_cuda_kernel_time, "Q_cuda_batch_scene": A.Q_cuda_batch_scene,
               "Q_cuda_batch_options": A.Q_cuda_batch_options, "Q_cuda_batch_stats": A.Q_cuda_batch_stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines.append("return 0; }")
    probe.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-Wall", str(probe), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for fname, _ in cls._fields_:
            assert int(got[f"{name}.{fname}"]) == getattr(cls, fname).offset, (name, fname)


def test_plugin_metadata(qlib):
    assert qlib.Q_plugin_abi_version() == 3
    info = qlib.Q_plugin_get_info()
    assert info.name == b"CUDA Path Tracer" and info.version.major == 1 and info.author == b"Quasi"


def test_create_rejects_non_cuda_backend(qlib):
    """Like plugin.mm:561-566 for Metal: a non-CUDA context logs and returns NULL."""
    for backend in (A.Q_GPU_BACKEND_NONE, A.Q_GPU_BACKEND_METAL, A.Q_GPU_BACKEND_VULKAN):
        with pytest.raises(q.LoaderError) as e:
            q.PluginHost(backend=backend)
        assert e.value.kind == "create_failed"
        assert "CUDA backend requires a CUDA GPU context" in str(e.value)
    assert qlib.Q_plugin_create(None) is None


def test_null_handles_are_ignored(qlib):
    qlib.Q_plugin_destroy(None)
    qlib.Q_plugin_update(None, 0.0)
    qlib.Q_plugin_render(None, None)
    r = qlib.Q_plugin_readback(None)
    assert not r.data
    qlib.Q_plugin_readback_free(None)
    r2 = qlib.Q_plugin_readback_aov(None)
    assert not any(r2.buffers[i].data for i in range(4))
    qlib.Q_plugin_readback_aov_free(None)
    assert qlib.Q_cuda_set_options(None, None) == A.QUASI_ERR_INVALID
    assert qlib.Q_cuda_last_error(None) == b"null handle"


def _stub_library(tmp_path: Path, body: str) -> Path:
    src = tmp_path / "stub.c"
    src.write_text("#include <stdint.h>\n" + body)
    so = tmp_path / "libstub.so"
    subprocess.run(["gcc", "-shared", "-fPIC", str(src), "-o", str(so)], check=True)
    return so


def test_loader_mirror_error_kinds(tmp_path):
    """PluginHost reports the reference loader's error codes (loader.hpp:38-42, 72-134)."""
    with pytest.raises(q.LoaderError) as e:
        q.PluginHost(tmp_path / "missing.so")
    assert e.value.kind == "file_not_found"
    partial = _stub_library(tmp_path, "uint32_t Q_plugin_abi_version(void){return 3;}\n")
    with pytest.raises(q.LoaderError) as e:
        q.PluginHost(partial)
    assert e.value.kind == "symbol_not_found"
    full = """
    typedef struct { const char* n; uint32_t a,b,c; const char* d; const char* e; } info;
    uint32_t Q_plugin_abi_version(void){return ABI;}
    info Q_plugin_get_info(void){info i={0}; return i;}
    void* Q_plugin_create(void* c){(void)c; return 0;}
    void Q_plugin_destroy(void* h){(void)h;}
    void Q_plugin_update(void* h, float d){(void)h;(void)d;}
    void Q_plugin_render(void* h, void* f){(void)h;(void)f;}
    """
    (tmp_path / "abi4").mkdir()
    with pytest.raises(q.LoaderError) as e:
        q.PluginHost(_stub_library(tmp_path / "abi4", "#define ABI 4\n" + full))
    assert e.value.kind == "abi_mismatch"
    (tmp_path / "abi3").mkdir()
    with pytest.raises(q.LoaderError) as e:
        q.PluginHost(_stub_library(tmp_path / "abi3", "#define ABI 3\n" + full))
    assert e.value.kind == "create_failed"


def test_loader_missing_library_is_loud(monkeypatch, tmp_path):
    with pytest.raises(q.LoaderError):
        q.load_library(tmp_path / "nope.so")
