"""Double-float arithmetic used for path geometry (quasi_gb300/csrc/ffmath.cuh), checked on the
host: its device intrinsics are IEEE round-to-nearest float operations, so a host build with
-ffp-contract=off computes the same values. Every operation must carry ~46 bits."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_double_float_operations_are_accurate(tmp_path):
    exe = tmp_path / "ffcheck"
    subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-I", "/usr/local/cuda/include",
                    str(ROOT / "tests" / "ffmath_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    errs = {k: float(v) for k, v in (line.split() for line in out.splitlines())}
    assert set(errs) == {"add", "mul", "div", "sqrt", "sin", "cos"}
    for k, v in errs.items():
        assert v < 5e-14, (k, v)
