"""Generates tests/golden/reference_abi.json from the reference project's
public header (include/kami_hair_solver.h, ABI v5): every typedef'd struct
with its field types, names and array lengths, every enum with its member
values, and every exported function with its normalised signature.

    python tests/golden/make_reference_abi.py <reference checkout>/include/kami_hair_solver.h
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from abi_parse import parse_header  # noqa: E402


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_abi.py <path of the reference's include/kami_hair_solver.h>")
    src = Path(sys.argv[1])
    abi = parse_header(src.read_text(encoding="utf-8"))
    abi["source"] = "reference include/kami_hair_solver.h (ABI version 5)"
    (HERE / "reference_abi.json").write_text(json.dumps(abi, indent=1, sort_keys=True) + "\n")
    print(f"{len(abi['structs'])} structs, {len(abi['enums'])} enums, {len(abi['functions'])} functions")


if __name__ == "__main__":
    main()
