"""OpenEXR output of the headless host (quasi_gb300/host/exr_writer.cpp), checked on the CPU:
the files are parsed back here from the OpenEXR file layout (magic, version, header
attributes, line offset table, uncompressed scanlines) and compared with the input; half
conversion is compared with numpy's IEEE binary16 rounding; the error codes follow the
reference writer (src/quasi/io/exr_writer.hpp: invalid_data, write_failed, directory_error)."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np
import pytest
from exr_format import parse_exr

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = tmp_path_factory.mktemp("exr") / "exr_check"
    subprocess.run(["g++", "-std=c++23", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), "-I",
                    str(ROOT / "quasi_gb300" / "host"), str(ROOT / "tests" / "exr_check.cpp"),
                    str(ROOT / "quasi_gb300" / "host" / "exr_writer.cpp"), "-o", str(out)], check=True)
    return out


def test_half_conversion_rounds_like_ieee(exe, tmp_path):
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.normal(0, 1, 20000), rng.normal(0, 1e4, 5000), rng.uniform(-7e-5, 7e-5, 5000),  # subnormal halves
        np.array([0.0, -0.0, 1.0, 65504.0, 65519.9, 65520.0, 1e9, -1e9, 2.0 ** -24, 2.0 ** -25, 2.0 ** -25 * 1.01,
                  np.inf, -np.inf, 5.9604645e-8, 6.1035156e-5, 6.1031e-5]),
        # exact ties between neighbouring halves
        (np.arange(1, 2000) + 0.5) * 2.0 ** -10,
    ]).astype(np.float32)
    src, dst = tmp_path / "in.f32", tmp_path / "out.u16"
    vals.tofile(src)
    subprocess.run([str(exe), "half", str(src), str(dst)], check=True)
    got = np.fromfile(dst, np.uint16)
    with np.errstate(over="ignore"):
        want = vals.astype(np.float16).view(np.uint16)
    assert np.array_equal(got, want)
    nan = np.array([np.nan], np.float32)
    nan.tofile(src)
    subprocess.run([str(exe), "half", str(src), str(dst)], check=True)
    assert np.isnan(np.fromfile(dst, np.uint16).view(np.float16)[0])


def test_rgba_file_round_trips(exe, tmp_path):
    rng = np.random.default_rng(1)
    w, h = 37, 23
    img = rng.uniform(0, 20, (h, w, 4)).astype(np.float32)
    img.tofile(tmp_path / "img.f32")
    out = tmp_path / "sub" / "beauty.exr"  # the writer creates missing directories
    subprocess.run([str(exe), "rgba", str(w), str(h), str(tmp_path / "img.f32"), str(out)], check=True)
    _, ch = parse_exr(out)
    assert sorted(ch) == ["A", "B", "G", "R"]
    for k, c in enumerate("RGBA"):
        assert np.array_equal(ch[c], img[..., k].astype(np.float16).astype(np.float32))


def test_aov_file_has_layers(exe, tmp_path):
    rng = np.random.default_rng(2)
    w, h = 16, 9
    bufs = [rng.uniform(0, 5, (h, w, 4)).astype(np.float32) for _ in range(4)]
    names = []
    for k, b in enumerate(bufs):
        p = tmp_path / f"b{k}.f32"
        b.tofile(p)
        names.append(str(p))
    out = tmp_path / "aov.exr"
    subprocess.run([str(exe), "aov", str(w), str(h), *names, str(out)], check=True)
    attrs, ch = parse_exr(out)
    assert sorted(ch) == ["A", "B", "G", "R", "albedo.B", "albedo.G", "albedo.R", "depth.Z", "normal.X",
                          "normal.Y", "normal.Z"]
    half = lambda a: a.astype(np.float16).astype(np.float32)  # noqa: E731
    for k, c in enumerate("RGBA"):
        assert np.array_equal(ch[c], half(bufs[0][..., k]))
    for k, c in enumerate("RGB"):
        assert np.array_equal(ch[f"albedo.{c}"], half(bufs[1][..., k]))
    for k, c in enumerate("XYZ"):
        assert np.array_equal(ch[f"normal.{c}"], half(bufs[2][..., k]))
    assert np.array_equal(ch["depth.Z"], bufs[3][..., 0])  # full float
    # absent layers are left out
    out2 = tmp_path / "beauty_only.exr"
    subprocess.run([str(exe), "aov", str(w), str(h), names[0], "-", "-", "-", str(out2)], check=True)
    assert sorted(parse_exr(out2)[1]) == ["A", "B", "G", "R"]


def test_invalid_inputs_return_the_reference_error_codes(exe, tmp_path):
    out = subprocess.run([str(exe), "invalid", str(tmp_path / "x.exr")], capture_output=True, text=True,
                         check=True).stdout.splitlines()
    assert out[:4] == ["Invalid readback data"] * 4
    assert out[4] == "Could not create output directory"
    assert re.fullmatch(r"dir/quasi_\d{8}_\d{6}\.exr", out[5])
