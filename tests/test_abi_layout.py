"""The ctypes mirrors of the C-ABI structs (glemur_gb300/_abi.py) against the
C compiler's layout of include/glemur.h: the size of every struct and the
offset of every field.  A mismatch would pass wrong parameters or read
wrong results without any error, so it is checked by compiling a small C
program that prints sizeof and offsetof for each field the mirrors name."""
import ctypes as C
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
