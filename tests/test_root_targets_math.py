"""The product's root-target math (csrc/khs_device_math.cuh, compiled for the
host) against the oracle's restatement of the reference's root frames
(src/solver.cpp:416-447, src/math.hpp:26-58) on random curves, bit for bit
(tests/native/test_root_targets.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_root_target_math_matches_oracle_bitwise(tmp_path):
    exe = tmp_path / "root_targets"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{REPO / 'kami-hair-solver_gb300' / 'csrc'}",
                    f"-I{REPO / 'oracle'}", f"-I{REPO / 'include'}", str(REPO / "tests" / "native" / "test_root_targets.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0 and "PASS" in out.stdout, out.stdout + out.stderr
