"""The drop-in boundary on CPU: this repository's header declares the
reference ABI v5 unchanged (structs field for field, enum values, function
signatures; tests/golden/reference_abi.json is generated from the reference
header by tests/golden/make_reference_abi.py), the struct layouts gcc
computes from the header equal an independent ctypes mirror of the
reference fields, and both libraries load and export what the header
declares.  No compute call is made, so no GPU is needed.
"""
import ctypes
import json
import shutil
import subprocess
from pathlib import Path

import pytest

from abi_parse import parse_header

REPO = Path(__file__).resolve().parents[1]
HEADER = REPO / "include" / "kami_hair_solver.h"
GOLDEN = json.loads((REPO / "tests" / "golden" / "reference_abi.json").read_text())
OURS = parse_header(HEADER.read_text(encoding="utf-8"))

CTYPES = {"uint32_t": ctypes.c_uint32, "uint64_t": ctypes.c_uint64, "int32_t": ctypes.c_int32, "double": ctypes.c_double,
          "float": ctypes.c_float, "char": ctypes.c_char, "int": ctypes.c_int}


def test_structs_identical_to_reference():
    for name, fields in GOLDEN["structs"].items():
        assert OURS["structs"].get(name) == fields, name


def test_enum_values_identical_to_reference():
    for name, members in GOLDEN["enums"].items():
        ours = OURS["enums"].get(name)
        assert ours is not None, name
        for member, value in members.items():
            assert ours.get(member) == value, (name, member)


def test_function_signatures_identical_to_reference():
    for name, sig in GOLDEN["functions"].items():
        assert OURS["functions"].get(name) == sig, name


def _mirror(name, cache={}):
    """ctypes structure built from the reference field list alone."""
    if name in cache:
        return cache[name]
    fields = []
    for ftype, fname, arr in GOLDEN["structs"][name]:
        # C enums are int-sized on every ABI this library targets.
        t = CTYPES.get(ftype) or (ctypes.c_int if ftype in GOLDEN["enums"] else _mirror(ftype))
        fields.append((fname, t * arr if arr else t))
    cls = type(name, (ctypes.Structure,), {"_fields_": fields})
    cache[name] = cls
    return cls


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layouts_match_reference_mirror(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "kami_hair_solver.h"', "int main(void) {"]
    for name, fields in GOLDEN["structs"].items():
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for _, fname, _ in fields:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", f"-I{REPO / 'include'}", str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                               text=True).stdout.splitlines())
    for name, fields in GOLDEN["structs"].items():
        cls = _mirror(name)
        assert int(got[f"{name} size"]) == ctypes.sizeof(cls), name
        for _, fname, _ in fields:
            assert int(got[f"{name}.{fname}"]) == getattr(cls, fname).offset, (name, fname)


def test_oracle_exports_declared_functions(oracle_path):
    import khs_native as kn

    lib = ctypes.CDLL(str(oracle_path))
    for name in OURS["functions"]:
        if name in kn.DEVICE_ONLY:
            continue
        assert hasattr(lib, name), name


def test_product_library_loads_and_exports_declared_functions():
    """The GB300 library loads without a GPU (the CUDA runtime is linked
    statically and initialises on the first CUDA call) and exports every
    function the header declares."""
    import khs_build

    if not khs_build.LIBRARY.exists():
        if shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists():
            pytest.skip("no nvcc to build the product library")
        khs_build.build()
    lib = ctypes.CDLL(str(khs_build.LIBRARY))
    lib.khsGetAbiVersion.restype = ctypes.c_uint32
    assert lib.khsGetAbiVersion() == 5
    for name in OURS["functions"]:
        assert hasattr(lib, name), name
    assert set(GOLDEN["functions"]) <= set(OURS["functions"])
