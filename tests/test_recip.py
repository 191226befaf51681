"""The block solve's integer-pipe reciprocal (csrc/khs_device_math.cuh
dm::recip_rn, compiled for the host) equals the IEEE division 1.0 / x bit
for bit (tests/native/test_recip.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_reciprocal_is_correctly_rounded(tmp_path):
    exe = tmp_path / "recip"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{REPO / 'kami-hair-solver_gb300' / 'csrc'}",
                    str(REPO / "tests" / "native" / "test_recip.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(1 << 22)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0 and "PASS" in out.stdout, out.stdout + out.stderr
