"""Build the native parts in-tree.

* ``glemur_gb300/_lib/libglemur.so`` -- the CUDA library behind the C-ABI of
  ``include/glemur.h`` (csrc/*.cu with nvcc for sm_103a, csrc/*.cpp with g++),
  statically linked against the CUDA runtime.
* ``glemur_gb300/_lib/glemur`` -- the drop-in executable (csrc/driver/).

The checker (the CPU oracle and the reference-kernel harness) has its own
recipe, oracle/build.py.

Every step runs in parallel and is skipped when its outputs are newer than
its inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "glemur_gb300"
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_lib" / "obj"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.environ.get("NVCC", str(Path(CUDA_HOME) / "bin" / "nvcc"))
if not Path(NVCC).exists():
    NVCC = shutil.which("nvcc") or NVCC

NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-O3", "-I" + str(INCLUDE), "-I" + str(CSRC),
    "-diag-suppress", "177",
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off",
             "-I" + str(INCLUDE), "-I" + str(CSRC), "-I" + str(Path(CUDA_HOME) / "include")]


def _newer(out: Path, inputs) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(i).stat().st_mtime <= t for i in inputs)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _headers(d: Path):
    return sorted(list(d.glob("*.h")) + list(d.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def _compile_obj(src: Path, verbose_ptx: bool = False) -> Path:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    obj = OBJ_DIR / (src.stem + (".cu.o" if src.suffix == ".cu" else ".cpp.o"))
    deps = [src] + _headers(CSRC)
    if _newer(obj, deps):
        return obj
    if src.suffix == ".cu":
        cmd = [NVCC] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptx else []) + ["-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)]
    out = _run(cmd)
    if verbose_ptx and out:
        (OBJ_DIR / (src.stem + ".ptxas.txt")).write_text(out)
    return obj


def build_library(jobs: int = 8, verbose_ptx: bool = False) -> Path:
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile_obj(s, verbose_ptx), srcs))
    lib = LIB_DIR / "libglemur.so"
    if not _newer(lib, objs):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", str(lib)] + [str(o) for o in objs]
             + ["-lpthread", "-ldl", "-lrt"])
    return lib


def build_driver() -> Path | None:
    ddir = CSRC / "driver"
    srcs = sorted(ddir.glob("*.cpp")) if ddir.exists() else []
    if not srcs:
        return None
    exe = LIB_DIR / "glemur"
    lib = LIB_DIR / "libglemur.so"
    if _newer(exe, srcs + [lib] + _headers(ddir)):
        return exe
    _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + str(INCLUDE), "-I" + str(ddir)] + [str(s) for s in srcs]
         + ["-o", str(exe), "-L" + str(LIB_DIR), "-lglemur", "-Wl,-rpath,$ORIGIN"])
    return exe


def build_all(verbose: bool = False) -> None:
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    lib = build_library()
    exe = build_driver()
    if verbose:
        for p in [lib, exe]:
            if p:
                print("built", p)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
