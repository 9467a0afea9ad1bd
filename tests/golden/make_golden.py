"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference's own CUDA kernels (oracle/_ref/glemur_ref{32,64}.cubin,
compiled unchanged from the reference sources) through the launcher that
replays src/main.cu's launch sequence, on the cases of cases.py, and stores
their outputs as tests/golden/<case>.npz:

  params   raw bytes of gm_params
  B0       initial field (ghosted AoS) the reference consumed
  k0, x1   stage 0: increment k_0 and stage position x_1 (inner points)
  maxDelta1, xnew1  error norm and x_new of the first attempted step
  B1, J1, D1        B, J, detJac after the first step's refresh (inner points)
  log      (maxDelta, dt, accepted) per attempt until N_ACCEPTED accepted steps
  xN, BN, JN, DN    state after N_ACCEPTED accepted steps (inner points)
  u1, unew1, uN     with inertia: the velocity after stage 0, u_new of the
                    first step and the velocity after N_ACCEPTED steps

Needs a GPU; run it on a GB300 after the build:
  python tests/golden/make_golden.py [OUT_DIR [CASE ...]]
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
from glemur_gb300 import configs  # noqa: E402
from oracle.pyoracle import RefLauncher  # noqa: E402


def inner(a):
    return np.ascontiguousarray(a[1:-1, 1:-1, 1:-1])


def generate(name: str, out_dir: Path) -> Path:
    p = cases.make(name)
    B0, xb = configs.init_state(p)
    rec = {"params": np.frombuffer(bytes(p), dtype=np.uint8), "B0": B0}
    r = RefLauncher(p, B0, xb)
    r.stage(0)
    rec["k0"] = r.k(0)
    rec["x1"] = inner(r.get()["xb"])
    if p.inertia:
        rec["u1"] = r.u()
    r.close()
    r = RefLauncher(p, B0, xb)
    r.step()
    s = r.scalars()
    rec["maxDelta1"] = np.array(s["maxDelta"])
    rec["xnew1"] = inner(r.xnew())
    if p.inertia:
        rec["unew1"] = r.u(new=True)
    f = r.get()
    rec["B1"], rec["J1"], rec["D1"] = inner(f["B"]), f["J"], inner(f["detJac"])
    n, lg = r.run(cases.N_ACCEPTED, max_attempts=500)
    rec["log"] = np.concatenate([[[s["maxDelta"], s["dt"], 1.0 if s["timeIndex"] == 1 else 0.0]], lg])
    f = r.get()
    rec["xN"], rec["BN"], rec["JN"], rec["DN"] = inner(f["xb"]), inner(f["B"]), f["J"], inner(f["detJac"])
    if p.inertia:
        rec["uN"] = r.u()
    rec["scalarsN"] = np.array([r.scalars()[k] for k in ("t", "dt", "maxDelta", "timeIndex", "nAttempted")])
    r.close()
    path = out_dir / f"{name}.npz"
    np.savez_compressed(path, **rec)
    return path


def main(argv):
    out = Path(argv[1]) if len(argv) > 1 else HERE
    out.mkdir(parents=True, exist_ok=True)
    for name in (argv[2:] or cases.NAMES):
        path = generate(name, out)
        print("wrote", path, path.stat().st_size)


if __name__ == "__main__":
    main(sys.argv)
