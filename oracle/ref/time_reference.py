"""Wall time of the reference's own CUDA kernels on the bench workload.

Measurement tooling of the oracle directory, not part of the product: it
drives the cubin built from the reference sources (oracle/_ref, made by
oracle/build.py) with the launch sequence and host synchronisations of
src/main.cu:259-384, through ref_launcher.cpp's ref_time_steps, on the
128x128x256 FP32 six-blob braid that bench.py times.  One JSON line:

    python oracle/ref/time_reference.py [--steps 20] [--warmup 3]
"""
import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args()
    from glemur_gb300 import configs
    from oracle.pyoracle import RefLauncher
    p = configs.braid6(128, 128, 256, precision=32)
    B0, xb = configs.init_state(p)
    r = RefLauncher(p, B0, xb)
    try:
        r.time_steps(args.warmup)
        sec, done = r.time_steps(args.steps)
    finally:
        r.close()
    n = p.nx * p.ny * p.nz
    print(json.dumps({
        "impl": "reference CUDA kernels (cubin from the reference sources, sm_103a)",
        "workload": f"braid6 {p.nx}x{p.ny}x{p.nz} FP32", "attempted_steps": done,
        "ms_per_step": 1e3 * sec / max(done, 1),
        "value": n * 6 * done / sec, "unit": "cell-RK-stages/s"}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
