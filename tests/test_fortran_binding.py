"""The ISO_C_BINDING module (fortran/pfgpu.f90) against the C header it
binds (include/pfgpu.h).  No Fortran compiler is available here, so the
module is read as text: every bind(C) derived type must list the C struct's
members in the same order with interoperable types, every bound procedure
must name a function the header declares and the library exports, with the
same number of arguments, and every named constant must equal the header's
#define."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
F90 = ROOT / "phase-field-microstructure-evolution_gb300" / "fortran" / "pfgpu.f90"
HDR = ROOT / "include" / "pfgpu.h"

F2C = {"integer(c_int)": "int", "real(c_double)": "double"}


def _strip_f90(text):
    lines = []
    for ln in text.splitlines():
        ln = ln.split("!", 1)[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + ln.strip()
        else:
            lines.append(ln)
    return lines


def _f90_types(lines):
    types, cur = {}, None
    for ln in lines:
        m = re.match(r"\s*type,\s*bind\(C\)\s*::\s*(\w+)", ln, re.I)
        if m:
            cur = m.group(1).lower()
            types[cur] = []
            continue
        if cur and re.match(r"\s*end\s+type", ln, re.I):
            cur = None
            continue
        if cur:
            m = re.match(r"\s*(integer\(c_int\)|real\(c_double\))\s*::\s*(.+)", ln, re.I)
            assert m, ln
            for item in m.group(2).split(","):
                item = item.strip()
                mm = re.match(r"(\w+)(?:\((\d+)\))?$", item)
                types[cur].append((F2C[m.group(1).lower()], mm.group(1).lower(), int(mm.group(2) or 1)))
    return types


def _c_structs(text, names=("pf_config", "pf_diag")):
    structs = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", text, re.S):
        if m.group(1) not in names:
            continue
        fields = []
        body = re.sub(r"/\*.*?\*/", "", m.group(2), flags=re.S)
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            ctype, items = decl.split(None, 1)
            for item in items.split(","):
                item = item.strip()
                mm = re.match(r"(\w+)(?:\[(\d+)\])?$", item)
                fields.append((ctype, mm.group(1).lower(), int(mm.group(2) or 1)))
        structs[m.group(1)] = fields
    return structs


def _f90_functions(lines):
    funcs = {}
    for ln in lines:
        m = re.match(r".*function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", ln, re.I)
        if m:
            args = [a.strip() for a in m.group(2).split(",") if a.strip()]
            funcs[m.group(3)] = len(args)
    return funcs


def _c_function_arity(text, name):
    m = re.search(r"\b" + name + r"\s*\(([^)]*)\)\s*;", text)
    assert m, name
    args = m.group(1).strip()
    return 0 if args in ("", "void") else len(args.split(","))


@pytest.fixture(scope="module")
def f90():
    return _strip_f90(F90.read_text())


def test_derived_types_match_the_c_structs(f90):
    types = _f90_types(f90)
    structs = _c_structs(HDR.read_text())
    assert set(types) == {"pf_config", "pf_diag"}
    for name, members in types.items():
        assert members == structs[name], (name, members, structs[name])


def test_bound_functions_are_declared_and_exported(f90, lib):
    hdr = HDR.read_text()
    funcs = _f90_functions(f90)
    assert {"pf_create", "pf_set_fields", "pf_step", "pf_get_fields", "pf_destroy", "pf_last_error"} <= set(funcs)
    for name, nargs in funcs.items():
        assert _c_function_arity(hdr, name) == nargs, name
        assert hasattr(lib, name), name


def test_named_constants_equal_the_header(f90):
    hdr = HDR.read_text()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define (PF_\w+) \(?(-?\d+)\)?", hdr)}
    consts = {}
    for ln in f90:
        m = re.match(r"\s*integer\(c_int\),\s*parameter\s*::\s*(.+)", ln, re.I)
        if m:
            for item in m.group(1).split(","):
                k, v = item.split("=")
                consts[k.strip()] = int(v.strip())
    assert consts and all(defines[k] == v for k, v in consts.items()), consts


def test_struct_sizes_match_ctypes(pkg):
    """The Python binding's structures (the same layout again) have the C
    sizes the Fortran types imply: 4-byte ints, 8-byte doubles, natural
    alignment."""
    sizes = {"int": 4, "double": 8}
    structs = _c_structs(HDR.read_text())
    for cname, pyname in (("pf_config", "Config"), ("pf_diag", "Diag")):
        off = 0
        for ctype, _, n in structs[cname]:
            sz = sizes[ctype]
            off = (off + sz - 1) // sz * sz + sz * n
        off = (off + 7) // 8 * 8
        assert C.sizeof(getattr(pkg, pyname)) == off, (cname, C.sizeof(getattr(pkg, pyname)), off)
