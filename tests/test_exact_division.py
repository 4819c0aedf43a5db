"""The correctly rounded division the FP64 kernels use (xdiv: reciprocal of a
known divisor plus two remainder corrections) equals IEEE division bit for
bit; checked on the host with the same header the kernels include."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_xdiv_matches_ieee_division(tmp_path):
    exe = tmp_path / "xdiv_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "stroemung_gb300" / "csrc"), "-I", "/usr/local/cuda/include",
                    str(ROOT / "tests" / "xdiv_check.cpp"), "-o", str(exe), "-lm"], check=True)
    r = subprocess.run([str(exe), "400000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout
