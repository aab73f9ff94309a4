"""Regenerates the golden fixtures in this directory from the reference's own code.

Needs the reference checkout (default /root/reference, or REF=<path>): it builds
oracle/_ref/ref_golden, which compiles the reference's C++ scene headers and the shader
source of backends/metal/plugin.mm as plain C++, and stores what it prints as
reference_golden.json. The fixtures are committed; tests only read them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent


def main() -> int:
    ref = os.environ.get("REF", "/root/reference")
    if not Path(ref, "backends", "metal", "plugin.mm").exists():
        print(f"reference checkout not found at {ref}", file=sys.stderr)
        return 1
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref", f"REF={ref}"], check=True)
    out = subprocess.run([str(ROOT / "oracle" / "_ref" / "ref_golden")], check=True, capture_output=True, text=True)
    data = json.loads(out.stdout)
    data["_generated_by"] = "tests/golden/make_golden.py (oracle/ref_golden.cpp over the reference sources)"
    (HERE / "reference_golden.json").write_text(json.dumps(data, separators=(",", ":")) + "\n")
    print("wrote", HERE / "reference_golden.json")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
