"""ORACLE build recipe (test infrastructure): the CPU restatement and the
reference-kernel harness, built in-tree.

* ``oracle/_build/liboracle{32,64}.so`` -- the CPU restatement
  (glemur_oracle.c), built with -ffp-contract=off so x86 and Arm agree.
* ``oracle/_ref/glemur_ref{64,32}{,_nofma}.cubin`` -- the reference's own
  kernels (src/maths.cu, boundaries.cu, current.cu, gradP.cu, rungeKutta.cu),
  compiled unchanged from where they lie in the reference tree, for sm_103a:
  a stock build (nvcc's default --fmad=true) and one without FMA contraction,
  two builds of the same reference that differ only in rounding.  Only where
  the reference tree exists; the cubins are device code and travel with the
  repository to the GPU machine.
* ``oracle/_ref/libref_launcher.so`` -- the driver-API launcher that replays
  src/main.cu's launch sequence on those cubins (everywhere).

The reference sources are read from GLEMUR_REFERENCE_SRC, else from the
reference checkout this recipe was written against (/root/reference/src);
this recipe is the one place that names that location.  Outputs go only to
oracle/_build/ and oracle/_ref/.  Every step runs in parallel and is skipped
when its outputs are newer than its inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
INCLUDE = ROOT / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.environ.get("NVCC", str(Path(CUDA_HOME) / "bin" / "nvcc"))
if not Path(NVCC).exists():
    NVCC = shutil.which("nvcc") or NVCC
REF_SRC = Path(os.environ.get("GLEMUR_REFERENCE_SRC", "/root/reference/src"))

# (precision, file suffix, extra nvcc flags) of the reference builds
REF_BUILDS = ((64, "", []), (32, "", []), (64, "_nofma", ["--fmad=false"]), (32, "_nofma", ["--fmad=false"]))


def _newer(out: Path, inputs) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(i).stat().st_mtime <= t for i in inputs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_oracle() -> list[Path]:
    out_dir = HERE / "_build"
    out_dir.mkdir(parents=True, exist_ok=True)
    src = HERE / "glemur_oracle.c"
    outs, cmds = [], []
    for bits in (64, 32):
        so = out_dir / f"liboracle{bits}.so"
        outs.append(so)
        if not _newer(so, [src, INCLUDE / "glemur.h"]):
            cmds.append(["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                         "-shared", f"-DORC_BITS={bits}", str(src), "-o", str(so), "-lm"])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, cmds))
    return outs


def build_reference_harness() -> list[Path]:
    ref_dir = HERE / "_ref"
    ref_dir.mkdir(parents=True, exist_ok=True)
    outs = []
    wrapper = HERE / "ref" / "ref_kernels.cu"
    if (REF_SRC / "rungeKutta.cu").exists():
        deps = [wrapper] + sorted(REF_SRC.glob("*.cu")) + sorted(REF_SRC.glob("*.h"))
        cmds = []
        for prec, variant, extra in REF_BUILDS:
            cub = ref_dir / f"glemur_ref{prec}{variant}.cubin"
            outs.append(cub)
            if not _newer(cub, deps):
                cmds.append([NVCC, "-cubin"] + ARCH + ["-O3", f"-DPRECISION={prec}", "-I" + str(REF_SRC), "-w"]
                            + extra + [str(wrapper), "-o", str(cub)])
        with cf.ThreadPoolExecutor(max_workers=4) as ex:
            list(ex.map(_run, cmds))
    launcher_src = HERE / "ref" / "ref_launcher.cpp"
    so = ref_dir / "libref_launcher.so"
    if not _newer(so, [launcher_src, INCLUDE / "glemur.h"]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + str(Path(CUDA_HOME) / "include"),
              str(launcher_src), "-o", str(so), "-ldl"])
    outs.append(so)
    return outs


def build_all(verbose: bool = False) -> list[Path]:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference_harness)
        outs = f_orc.result() + f_ref.result()
    if verbose:
        for p in outs:
            print("built", p)
    return outs


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
