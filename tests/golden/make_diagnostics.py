"""Generate tests/golden/diagnostics_f{64,32}.npz: the grid-quality fields,
eps* and the analytic-error norms from the reference's own kernels.

Cases (each stored under its prefix):
  folded   the folded 17x12x17 grid of make_folded.py (every face line-tied,
           inner points moved by up to 0.45 spacings), B and J refreshed at
           that grid;
  braid    braid_f64 / braid_f32 of cases.py after 10 accepted steps of the
           reference's kernels;
  analytic analytic_f64 after 10 accepted steps (FP64 file only).
For each: params (raw gm_params bytes), B0, x (the grid, ghosted AoS), and
from the reference's kernels dirCellVol, gridConvexity, gridWedgeMin
(src/maths.cu:443-643, with prepareDump's launch shapes), eps* (JB_B2 +
epsilonStar + findDevMax, src/diagnostics.cu:32-47), errB_1ez and
errXb_XbAn (src/diagnostics.cu:51-71).

Needs a GPU; run it on a GB300 after the build:
  python tests/golden/make_diagnostics.py [OUT_DIR]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import cases  # noqa: E402
import make_folded  # noqa: E402
from glemur_gb300 import configs  # noqa: E402
from oracle.pyoracle import RefLauncher  # noqa: E402


def case_inputs(kind: str, precision: int):
    """(params, B0, x) before the reference's steps, and the accepted steps."""
    if kind == "folded":
        p, B0, x = make_folded.folded_case("Stokes")
        if precision == 32:
            p = configs.braid2(17, 12, 17, precision=32)
            p.xPeri = p.yPeri = p.zPeri = 0
            p.errMode = 0
            p = configs.derive(p)
            B0 = B0.astype(np.float32)
            x = x.astype(np.float32)
        return p, B0, x, 0
    if kind == "braid":
        p = cases.make("braid_f64" if precision == 64 else "braid_f32")
    else:
        p = cases.make("analytic_f64")
    B0, x = configs.init_state(p)
    return p, B0, x, cases.N_ACCEPTED


def reference_diagnostics(p, B0, x, steps):
    r = RefLauncher(p, B0, x)
    try:
        if steps:
            r.run(steps, max_attempts=10 * steps)
        r.refresh()
        f = r.get()
        g = r.grid_fields()
        eps = r.eps_star()
        e1, e2 = r.errors()
    finally:
        r.close()
    return f["xb"], g, eps, e1, e2


def main():
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE
    out.mkdir(parents=True, exist_ok=True)
    for precision in (64, 32):
        data = {}
        kinds = ("folded", "braid", "analytic") if precision == 64 else ("folded", "braid")
        for kind in kinds:
            p, B0, x0, steps = case_inputs(kind, precision)
            x, g, eps, e1, e2 = reference_diagnostics(p, B0, x0, steps)
            data[f"{kind}_params"] = np.frombuffer(bytes(p), dtype=np.uint8).copy()
            data[f"{kind}_B0"] = B0
            data[f"{kind}_x"] = x
            for k, v in g.items():
                data[f"{kind}_{k}"] = v
            data[f"{kind}_scalars"] = np.array([eps, e1, e2])
            print(precision, kind, "eps*", eps, "errB_1ez", e1, "errXb_XbAn", e2,
                  "convex min", float(g["convexity"].min()), flush=True)
        path = out / f"diagnostics_f{precision}.npz"
        np.savez_compressed(path, **data)
        print("wrote", path, path.stat().st_size)


if __name__ == "__main__":
    main()
