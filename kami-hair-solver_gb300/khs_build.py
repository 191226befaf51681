"""Builds the GB300 solver library ``_build/libkami_hair_solver.so``.

nvcc compiles the CUDA translation unit for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); the host C++ units are
compiled with the system g++ (``-ffp-contract=off`` so the host builder
rounds the same on x86_64 and aarch64).  Translation units build in
parallel; an up-to-date library is reused.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
REPO = PACKAGE.parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = BUILD / "libkami_hair_solver.so"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["khs_engine.cu", "khs_peaks.cu"]
HOST_UNITS = ["khs_model.cpp", "khs_api.cpp"]
HEADERS = ["khs_engine.hpp", "khs_model.hpp", "khs_device_math.cuh"]


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    candidate = Path(cuda_home) / "bin" / "nvcc"
    return str(candidate) if candidate.exists() else (shutil.which("nvcc") or "nvcc")


def _sources() -> list[Path]:
    return [CSRC / u for u in CUDA_UNITS + HOST_UNITS + HEADERS] + [INCLUDE / "kami_hair_solver.h"]


def _stale() -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    return any(p.stat().st_mtime > built for p in _sources()) or Path(__file__).stat().st_mtime > built


def _run(cmd: list[str], log: Path) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    log.write_text(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({log}):\n{proc.stdout}{proc.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the library if any source changed; returns its path."""
    if not force and not _stale():
        return LIBRARY
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    common_inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    for unit in CUDA_UNITS:
        obj = BUILD / (unit + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xptxas", "-v", "-Xcompiler", "-fPIC,-fvisibility=hidden",
               *common_inc, "-c", str(CSRC / unit), "-o", str(obj)]
        jobs.append((cmd, BUILD / (unit + ".log"), obj))
    for unit in HOST_UNITS:
        obj = BUILD / (unit + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall", "-Wextra", "-Wno-unknown-pragmas",
               *common_inc, f"-I{os.environ.get('CUDA_HOME', '/usr/local/cuda')}/include", "-c", str(CSRC / unit),
               "-o", str(obj)]
        jobs.append((cmd, BUILD / (unit + ".log"), obj))
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as pool:
        for f in [pool.submit(_run, cmd, log) for cmd, log, _ in jobs]:
            f.result()
    tmp = BUILD / (LIBRARY.name + ".tmp")
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *[str(o) for _, _, o in jobs],
            "-Xlinker", "-Bsymbolic"]
    _run(link, BUILD / "link.log")
    os.replace(tmp, LIBRARY)
    if verbose:
        print((BUILD / "khs_engine.cu.log").read_text())
    return LIBRARY


def register_report() -> str:
    """ptxas resource usage lines of the last build (registers, spills, smem)."""
    log = BUILD / "khs_engine.cu.log"
    return log.read_text() if log.exists() else ""


if __name__ == "__main__":
    print(build(force=True, verbose=True))
