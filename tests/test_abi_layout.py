"""The C ABI's struct layouts, three ways: include/swgb300.h as gcc lays it
out (sizeof / offsetof from a probe compiled here), the ctypes mirror in
seismicwaves.jl_gb300/_lib.py, and the Julia structs of the Julia binding
(julia/SeismicWavesGB300/src/abi.jl: field names and order).  A field added
to the header but not to a binding shifts every later field or the array
stride.  Also: every library function the Julia binding calls is declared in
the header."""
import json
import re
import shutil
import subprocess
from pathlib import Path

import pytest

import __graft_entry__

ROOT = Path(__file__).resolve().parents[1]
BUILD = Path(__file__).resolve().parent / "_build"
sw = __graft_entry__.load_package()
L = sw._lib

JULIA = ROOT / "julia" / "SeismicWavesGB300"
STRUCTS = {  # C typedef -> (ctypes class, Julia struct of the Julia binding)
    "sw_acoustic_params": (L.SwAcousticParams, "SwAcousticParams"),
    "sw_acoustic_shot": (L.SwAcousticShot, "SwAcousticShot"),
    "sw_grad_params": (L.SwGradParams, "SwGradParams"),
    "sw_elastic_params": (L.SwElasticParams, "SwElasticParams"),
    "sw_point_table": (L.SwPointTable, "SwPointTable"),
    "sw_elastic_shot": (L.SwElasticShot, "SwElasticShot"),
}


@pytest.fixture(scope="module")
def c_layout():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    BUILD.mkdir(exist_ok=True)
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "swgb300.h"', "int main(void) {",
             '  printf("{");']
    first = True
    for cname, (cls, _) in STRUCTS.items():
        sep = "" if first else ","
        first = False
        lines.append(f'  printf("{sep}\\"{cname}\\": {{\\"size\\": %zu", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf(", \\"{fname}\\": %zu", offsetof({cname}, {fname}));')
        lines.append('  printf("}");')
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    src = BUILD / "layout_probe.c"
    exe = BUILD / "layout_probe"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    return json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_layout_matches_header(c_layout, cname):
    cls, _ = STRUCTS[cname]
    lay = c_layout[cname]
    assert ctypes_sizeof(cls) == lay["size"], cname
    for fname, _ in cls._fields_:
        assert getattr(cls, fname).offset == lay[fname], f"{cname}.{fname}"


def ctypes_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


def _julia_fields(text, name):
    m = re.search(rf"struct {name}\b(.*?)\bend\b", text, re.S)
    assert m, name
    body = re.sub(r"#[^\n]*", "", m.group(1))
    return re.findall(r"([A-Za-z_]\w*)::", body)


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_julia_binding_structs_match_header(cname):
    cls, jname = STRUCTS[cname]
    text = (JULIA / "src" / "abi.jl").read_text()
    assert _julia_fields(text, jname) == [f for f, _ in cls._fields_], jname


def test_julia_binding_calls_only_declared_functions():
    called = set()
    for f in sorted(JULIA.rglob("*.jl")):
        called |= set(re.findall(r"ccall\(\(:(sw_\w+),", f.read_text()))
    assert called, "no ccall found in the Julia binding"
    missing = sorted(called - set(_prototypes()))
    assert not missing, missing


def _prototypes():
    """name -> [parameter C types] for every function the header declares."""
    text = (ROOT / "include" / "swgb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|void|const char\s*\*|void\s*\*|int32_t)\s*\**\s*(sw_\w+)\s*\(([^;{]*?)\)\s*;",
                         text, re.S):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(1)] = params
    return protos


def _kind_c(p):
    if "*" in p:
        return "ptr"
    if p.startswith("double"):
        return "f64"
    if p.startswith("int64_t"):
        return "i64"
    return "i32"  # int, int32_t


def _kind_ctypes(t):
    import ctypes
    if t in (ctypes.c_double,):
        return "f64"
    if t in (ctypes.c_int64, ctypes.c_longlong):
        return "i64"
    if t in (ctypes.c_int32, ctypes.c_int):
        return "i32"
    return "ptr"  # c_void_p, POINTER(...), c_char_p


def test_ctypes_signatures_match_header():
    """Every exported function's ctypes argtypes agree with its prototype in
    count and kind (32-bit integer, double, pointer)."""
    protos = _prototypes()
    lib = L.load()
    assert set(L.EXPORTS) <= set(protos), sorted(set(L.EXPORTS) - set(protos))
    checked = 0
    for name in L.EXPORTS:
        argtypes = getattr(lib, name).argtypes
        if argtypes is None:
            continue
        assert [_kind_ctypes(t) for t in argtypes] == [_kind_c(p) for p in protos[name]], name
        checked += 1
    assert checked >= 20
