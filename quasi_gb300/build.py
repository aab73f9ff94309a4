"""Builds libquasi_cuda.so (and the headless host) in-tree with nvcc and g++.

Sources are compiled in parallel into quasi_gb300/_build/ and linked with the shared CUDA
runtime, so the library can be dlclose'd and reloaded (hot reload) without leaving a static
runtime behind. Device code targets sm_103a only.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
LIB = BUILD / "libquasi_cuda.so"
HEADLESS = BUILD / "quasi_headless"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall", "-Wextra"]
# Extra nvcc flags (e.g. -D tuning constants); objects are not rebuilt when only these change.
EXTRA_NVCC = os.environ.get("QUASI_NVCC_FLAGS", "").split()


def _cuda_lib_dir() -> Path:
    for cand in (CUDA_HOME / "lib64", CUDA_HOME / "lib"):
        if (cand / "libcudart.so").exists():
            return cand
    return CUDA_HOME / "lib64"


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    if proc.stdout.strip():
        sys.stderr.write(proc.stdout)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + sorted((ROOT / "include").glob("*.h"))


def compile_objects(verbose_ptxas: bool = False) -> list[Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = _headers()
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", ",".join(HOST_FLAGS),
               "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), *EXTRA_NVCC, "-c", str(src), "-o", str(obj)]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, [src, *headers], cmd))
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".cpp.o")
        cmd = ["g++", "-std=c++20", *HOST_FLAGS, "-I", str(ROOT / "include"), "-I", str(CUDA_HOME / "include"),
               "-c", str(src), "-o", str(obj)]
        jobs.append((obj, [src, *headers], cmd))
    todo = [(o, c) for o, d, c in jobs if verbose_ptxas or not _newer(o, d)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda oc: _run(oc[1]), todo))
    return [o for o, _, _ in jobs]


def link(objs: list[Path]) -> Path:
    if _newer(LIB, objs):
        return LIB
    libdir = _cuda_lib_dir()
    tmp = LIB.with_suffix(".so.tmp")
    _run([NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
          "-Xlinker", f"-rpath,{libdir}", "-L", str(libdir)])
    os.replace(tmp, LIB)
    return LIB


def build_headless() -> Path | None:
    src = HOST / "quasi_headless.cpp"
    if not src.exists():
        return None
    deps = [src, *sorted(HOST.glob("*.hpp")), *sorted(HOST.glob("*.cpp")), ROOT / "include" / "quasi_cuda.h"]
    if _newer(HEADLESS, deps):
        return HEADLESS
    libdir = _cuda_lib_dir()
    srcs = [str(p) for p in sorted(HOST.glob("*.cpp"))]
    _run(["g++", "-std=c++23", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), "-I", str(CUDA_HOME / "include"),
          *srcs, "-o", str(HEADLESS), "-ldl", "-L", str(libdir), "-lcudart", f"-Wl,-rpath,{libdir}"])
    return HEADLESS


def build(verbose_ptxas: bool = False) -> Path:
    if not Path(NVCC).exists() and shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    lib = link(compile_objects(verbose_ptxas))
    build_headless()
    return lib


if __name__ == "__main__":
    print(build(verbose_ptxas="--ptxas" in sys.argv))
