"""The product's closed-form element strain Jacobian and Gauss-Newton
Hessian (csrc/khs_device_math.cuh, compiled for the host) against the
oracle's forward-mode dual numbers on random element states
(tests/native/test_element_math.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_closed_form_element_derivatives_match_duals(tmp_path):
    exe = tmp_path / "element_math"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{REPO / 'kami-hair-solver_gb300' / 'csrc'}",
                    f"-I{REPO / 'oracle'}", f"-I{REPO / 'include'}", str(REPO / "tests" / "native" / "test_element_math.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0 and "PASS" in out.stdout, out.stdout + out.stderr
