"""The Julia binding's mirrors of the C structs have the C layout.

There is no Julia here, so the check is made from both sources: every
`struct Crg...` in the binding is parsed (field names and types, in order), its
layout computed by the C rules Julia applies to isbits structs (each field at
the next multiple of its alignment, the size rounded up to the largest
alignment), and compared with `offsetof` / `sizeof` of the matching struct in
include/crg.h, compiled by the host C compiler.  A field added, removed,
retyped or reordered on either side fails the test.  The binding returns the
reference's `Regridder` (src/regridder/regridder.jl:25-36) around these
handles, so a mismatch would corrupt every call.
"""
from __future__ import annotations

import re
import shutil
import subprocess

import pytest

from conftest import ROOT

JL = ROOT / "conservativeregridding.jl_gb300" / "julia" / "ConservativeRegriddingGB300" / "src" / "ConservativeRegriddingGB300.jl"
C_NAMES = {"CrgGridDesc": "crg_grid_desc", "CrgBuildOpts": "crg_build_opts", "CrgInfo": "crg_info",
           "CrgApplyItem": "crg_apply_item", "CrgSeSpace": "crg_se_space", "CrgSeOpts": "crg_se_opts"}
PRIM = {"Int32": 4, "Int64": 8, "Float64": 8, "Cint": 4, "Int8": 1, "UInt32": 4, "UInt64": 8, "Float32": 4}


def parse_structs(text):
    out = {}
    for m in re.finditer(r"^struct (Crg\w+)\n(.*?)^end", text, re.S | re.M):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#")[0]
            for part in line.split(";"):
                part = part.strip()
                if part:
                    name, typ = part.split("::")
                    fields.append((name.strip(), typ.strip()))
        out[m.group(1)] = fields
    return out


def size_align(typ, structs):
    if typ in PRIM:
        return PRIM[typ], PRIM[typ]
    if typ.startswith("Ptr{"):
        return 8, 8
    m = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", typ)
    if m:
        s, a = size_align(m.group(2), structs)
        return int(m.group(1)) * s, a
    if typ in structs:
        lay = layout(structs[typ], structs)
        return lay["__size__"], lay["__align__"]
    raise ValueError(f"unknown Julia field type {typ}")


def layout(fields, structs):
    off, amax, res = 0, 1, {}
    for name, typ in fields:
        s, a = size_align(typ, structs)
        off = (off + a - 1) // a * a
        res[name] = off
        off += s
        amax = max(amax, a)
    res["__size__"] = (off + amax - 1) // amax * amax
    res["__align__"] = amax
    return res


def test_julia_structs_match_c_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = parse_structs(JL.read_text())
    assert set(C_NAMES) <= set(structs), f"binding lacks {set(C_NAMES) - set(structs)}"
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "crg.h"', "int main(void) {"]
    for jl, c in C_NAMES.items():
        lines.append(f'printf("{jl} __size__ %zu\\n", sizeof({c}));')
        for name, _ in structs[jl]:
            lines.append(f'printf("{jl} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr  # a field name the C struct lacks fails here
    c_off = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        jl, name, v = line.split()
        c_off[(jl, name)] = int(v)
    for jl in C_NAMES:
        lay = layout(structs[jl], structs)
        for name, _ in structs[jl]:
            assert lay[name] == c_off[(jl, name)], f"{jl}.{name}: Julia offset {lay[name]}, C {c_off[(jl, name)]}"
        assert lay["__size__"] == c_off[(jl, "__size__")], f"{jl}: Julia size {lay['__size__']}, C {c_off[(jl, '__size__')]}"


def test_layout_rules_catch_a_drift():
    """The comparison sees a reordered field (a planted drift, on the Julia side)."""
    structs = parse_structs(JL.read_text())
    good = layout(structs["CrgBuildOpts"], structs)
    bad = layout([structs["CrgBuildOpts"][2], *structs["CrgBuildOpts"][:2]], structs)
    assert good["stream"] != bad["stream"]
