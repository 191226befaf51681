"""Shared pytest fixtures.

* ``oracle_lib`` -- the CPU FP64 oracle (oracle/_build/libkhs_oracle.so),
  built on first use with ``make -C oracle``.
* ``gpu_lib``    -- the GB300 product library; only available on a machine
  with a CUDA device.  Tests that need it are marked ``@pytest.mark.gpu``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
PACKAGE = REPO / "kami-hair-solver_gb300"
if str(PACKAGE) not in sys.path:
    sys.path.insert(0, str(PACKAGE))
if str(REPO / "tests") not in sys.path:
    sys.path.insert(0, str(REPO / "tests"))
# oracle/refgpu.py: the binding of the reference's own CUDA backend.
if str(REPO / "oracle") not in sys.path:
    sys.path.append(str(REPO / "oracle"))

ORACLE_SO = REPO / "oracle" / "_build" / "libkhs_oracle.so"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built product library")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle")], check=True)
    return ORACLE_SO


@pytest.fixture(scope="session")
def oracle_path() -> Path:
    return build_oracle()


@pytest.fixture(scope="session")
def oracle_lib(oracle_path):
    import khs_native
    return khs_native.Library(oracle_path)


@pytest.fixture(scope="session")
def gpu_lib():
    import khs_build
    import khs_native
    path = khs_build.build()
    return khs_native.Library(path)
