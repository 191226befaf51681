"""Minimal parser of the solver's C header: typedef'd structs (field type,
name, array length), enums (member values) and exported function
declarations (normalised signature).  Used by the golden-fixture generator
for the reference header and by the ABI tests for this repository's header.
"""
from __future__ import annotations

import re

_COMMENT = re.compile(r"/\*.*?\*/|//[^\n]*", re.S)


def _clean(text: str) -> str:
    text = _COMMENT.sub(" ", text)
    return "\n".join(line for line in text.splitlines() if not line.lstrip().startswith("#"))


def _norm(s: str) -> str:
    s = re.sub(r"\s+", " ", s.strip())
    s = re.sub(r"\s*\*\s*", " *", s)
    return s.replace(" *", "*").replace("*", " *").strip()


def parse_header(text: str) -> dict:
    src = _clean(text)
    structs, enums, functions = {}, {}, {}
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", src, re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            fm = re.match(r"(.+?)\s*(\w+)\s*(?:\[(\w+)\])?$", decl, re.S)
            ftype, fname, arr = fm.group(1), fm.group(2), fm.group(3)
            fields.append([_norm(ftype), fname, int(arr) if arr else 0])
        structs[m.group(3)] = fields
    for m in re.finditer(r"typedef\s+enum\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", src, re.S):
        members, value = {}, -1
        for item in m.group(2).split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, val = (x.strip() for x in item.split("=", 1))
                value = int(val, 0)
            else:
                name, value = item, value + 1
            members[name] = value
        enums[m.group(3)] = members
    for m in re.finditer(r"KHS_API\s+([^;{]*?)\b(khs\w+)\s*\(([^)]*)\)\s*;", src, re.S):
        ret = _norm(m.group(1))
        params = []
        for p in m.group(3).split(","):
            p = _norm(p)
            if p in ("", "void"):
                continue
            pm = re.match(r"(.+?)\s*(\w+)$", p)
            params.append(_norm(pm.group(1)) if pm and pm.group(1).strip() not in ("", "const") else p)
        functions[m.group(2)] = [ret, params]
    return {"structs": structs, "enums": enums, "functions": functions}
