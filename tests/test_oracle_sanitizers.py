"""The CPU oracle under AddressSanitizer and UndefinedBehaviorSanitizer (oracle/sanitize_check.cpp):
LBVH, 8-wide collapse, NEE integrator (FP64, FP32), adjoint and reference integrator on seeded
scenes with the edge cases (0/1/2 triangles, coincident, flat)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ORACLE = Path(__file__).resolve().parent.parent / "oracle"


def test_oracle_clean_under_asan_and_ubsan():
    b = subprocess.run(["make", "-s", "-C", str(ORACLE), "sanitize"], capture_output=True, text=True, timeout=600)
    if b.returncode != 0:
        if "sanitize" in b.stderr and ("cannot find" in b.stderr or "unrecognized" in b.stderr):
            pytest.skip("this compiler has no ASan/UBSan runtime")
        pytest.fail(b.stderr)
    r = subprocess.run([str(ORACLE / "_build" / "sanitize_check")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all ok" in r.stdout
