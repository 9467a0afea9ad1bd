"""Generate tests/golden/folded_currents.npz: the currents of the reference's
own kernels on a folded grid, where the quintilateral and triangular
currents take their corner triangles.

The grid is the 17x12x17 FP64 braid with every face line-tied, each inner
point moved by a uniform random offset of up to 0.45 spacings per component
(numpy default_rng(3)); some cells fold.  For each jMethod (Stokes,
Stokes4th, StokesQuint, StokesTri, Classic) the reference's kernels
(oracle/_ref/glemur_ref64.cubin through the launcher) compute B, detJac and J
at that grid, as after an accepted step (src/main.cu:343-353).  Stored:

  params      raw bytes of gm_params (jMethod "Stokes")
  B0, x       the initial field and the folded grid (ghosted AoS)
  B           B at the grid (inner points; the same for every method)
  J_<method>  J of each method (inner points); StokesTri is NaN where a
              plane takes a triangle

Needs a GPU; run it on a GB300 after the build:
  python tests/golden/make_folded.py [OUT_DIR]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from glemur_gb300 import configs  # noqa: E402
from oracle.pyoracle import RefLauncher  # noqa: E402

METHODS = ("Stokes", "Stokes4th", "StokesQuint", "StokesTri", "Classic")


def folded_case(method="Stokes"):
    """Parameters, B0 and the folded grid (the same for every method)."""
    p = configs.braid2(17, 12, 17, precision=64)
    p.xPeri = p.yPeri = p.zPeri = 0
    p.errMode = 0
    p.set_str("jMethod", method)
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    rng = np.random.default_rng(3)
    x = xb.copy()
    sp = np.array([p.dx, p.dy, p.dz])
    x[1:-1, 1:-1, 1:-1] += rng.uniform(-0.45, 0.45, size=x[1:-1, 1:-1, 1:-1].shape) * sp
    return p, B0, x


def main():
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE
    out.mkdir(parents=True, exist_ok=True)
    data = {}
    for m in METHODS:
        p, B0, x = folded_case(m)
        r = RefLauncher(p, B0, x)
        try:
            r.refresh()
            f = r.get()
        finally:
            r.close()
        data[f"J_{m}"] = f["J"]
        if m == "Stokes":
            data["params"] = np.frombuffer(bytes(p), dtype=np.uint8).copy()
            data["B0"], data["x"] = B0, x
            data["B"] = np.ascontiguousarray(f["B"][1:-1, 1:-1, 1:-1])
    path = out / "folded_currents.npz"
    np.savez_compressed(path, **data)
    print("wrote", path, path.stat().st_size)


if __name__ == "__main__":
    main()
