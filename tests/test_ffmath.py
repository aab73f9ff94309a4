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
    assert set(errs) == {"add", "addf", "mul", "div", "sqrt", "sin", "cos", "dotsub"}
    for k, v in errs.items():
        assert v < 5e-14, (k, v)


def _decimal_pi():
    from decimal import Decimal

    def arctan_inv(x: int) -> Decimal:  # arctan(1/x) by its series
        x = Decimal(x)
        s, t, n, sign = Decimal(0), 1 / x, 1, 1
        while t / n > Decimal(10) ** -58:
            s += sign * t / n
            t /= x * x
            n += 2
            sign = -sign
        return s

    return 16 * arctan_inv(5) - 4 * arctan_inv(239)  # Machin's formula


def test_sincospi_table_holds_the_rounded_exact_values():
    """k_sincospi_tab in ffmath.cuh: sin and cos of j pi / 128 (j = 0..32) as (hi, lo) float
    pairs, recomputed here from their Taylor series in 60-digit decimal arithmetic."""
    import re
    import struct
    from decimal import Decimal, getcontext

    getcontext().prec = 60
    pi = _decimal_pi()

    def f32(v) -> float:
        return struct.unpack("f", struct.pack("f", float(v)))[0]

    def split(v: Decimal) -> tuple[float, float]:
        hi = f32(v)
        return hi, f32(v - Decimal(hi))

    def sincos(a: Decimal) -> tuple[Decimal, Decimal]:
        s = c = Decimal(0)
        term = Decimal(1)
        for k in range(60):
            if k % 4 == 0:
                c += term
            elif k % 4 == 1:
                s += term
            elif k % 4 == 2:
                c -= term
            else:
                s -= term
            term = term * a / (k + 1)
        return s, c

    src = (ROOT / "quasi_gb300" / "csrc" / "ffmath.cuh").read_text()
    body = src[src.index("k_sincospi_tab[33][4] = {"):]
    body = body[: body.index("};")]
    rows = re.findall(r"\{([^{}]+)\}", body)
    assert len(rows) == 33
    for j, row in enumerate(rows):
        got = [f32(v.strip().rstrip("f")) for v in row.split(",")]
        s, c = sincos(pi * j / 128)
        assert got == [*split(s), *split(c)], j
