"""The integer-arithmetic FP32 <-> FP64 conversions of the mixed-precision
kernels (strm::widen, strm::narrow) equal the IEEE conversions bit for bit
outside the flushed range; checked on the host with the header the kernels
include."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_conversions_match_ieee(tmp_path):
    exe = tmp_path / "conversion_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "stroemung_gb300" / "csrc"), "-I", "/usr/local/cuda/include",
                    str(ROOT / "tests" / "conversion_check.cpp"), "-o", str(exe), "-lm"],
                   check=True)
    r = subprocess.run([str(exe), "500000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout
