"""The ctypes view of the C-ABI (glemur_gb300/_abi.py) against include/glemur.h.

- Structs: the size of every struct and the offset of every field, as the C
  compiler lays them out (a small C program prints sizeof and offsetof for
  each field the mirrors name).
- Functions: every declared entry point has a ctypes signature and the other
  way round, and each parameter and return value has the same ABI class
  (pointer, 32- or 64-bit integer, float, double).

A mismatch would pass wrong arguments or read wrong results without any
error, which is why it is checked here."""
import ctypes as C
import re
import shutil
import subprocess

import pytest

from glemur_gb300 import _abi

MIRRORS = [("gm_params", _abi.GmParams), ("gm_step_result", _abi.GmStepResult), ("gm_state", _abi.GmState),
           ("gm_reduction", _abi.GmReduction), ("gm_batch_case", _abi.GmBatchCase)]


def _include_dir():
    from pathlib import Path
    return Path(__file__).resolve().parents[1] / "include"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "glemur.h"', "int main(void) {"]
    for cname, py in MIRRORS:
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(_include_dir()), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = {}
    for line in out:
        if line:
            s, f, v = line.split()
            c[(s, f)] = int(v)
    for cname, py in MIRRORS:
        assert c[(cname, "sizeof")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert c[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def _declarations():
    """name -> (return type, [parameter types]) of every gm_* declaration."""
    src = (_include_dir() / "glemur.h").read_text()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = re.sub(r"#[^\n]*", " ", src)
    out = {}
    for ret, name, args in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(gm_\w+)\s*\(([^;{}]*?)\)\s*;", src):
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        # drop the parameter name: the type is everything before the last identifier
        types = [re.sub(r"\b\w+$", "", a).strip() if not a.endswith("*") else a for a in params]
        out[name] = (" ".join(ret.split()), types)
    return out


def _c_class(t):
    t = " ".join(t.replace("const", " ").split())
    if "*" in t:
        return "ptr"
    return {"int": "i32", "int32_t": "i32", "int64_t": "i64", "long long": "i64", "long": "i64", "size_t": "i64",
            "double": "f64", "float": "f32"}[t]


def _ctypes_class(t):
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    if t in (C.c_float,):
        return "f32"
    if t in (C.c_double,):
        return "f64"
    return {4: "i32", 8: "i64"}[C.sizeof(t)]


def test_every_entry_point_has_a_matching_ctypes_signature():
    decl = _declarations()
    assert len(decl) >= 50
    assert set(decl) == set(_abi.SIGNATURES), (set(decl) ^ set(_abi.SIGNATURES))
    for name, (ret, params) in decl.items():
        rt, at = _abi.SIGNATURES[name]
        assert _c_class(ret) == _ctypes_class(rt), (name, ret)
        assert [_c_class(t) for t in params] == [_ctypes_class(t) for t in at], name
