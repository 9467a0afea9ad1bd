"""Benchmark of the relaxation hot path (one JSON line on stdout).

Workload: the six-blob braid on 128x128x256 inner points (periodic x, y;
line-tied z), FP32 storage with the cancellation-free error norm (errMode 1)
and the FP64 controller.  A step
is one attempted adaptive Runge-Kutta step (6 stages + accept/reject) over
the whole grid; the metric is cell-RK-stages/s = N x 6 x steps / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  python bench.py --workload batch64 [--batch-residual R] [--batch-cycles C]

--workload large times the 256x256x512 braid with k = +-1.2 and the
pressure term with the p0(r) profile (the plain path of the large case);
--large-shape nx,ny,nz runs the same braid on another grid (a smaller case
for a profiler capture).

--workload batch64 runs the batched configuration instead: 64 seeded random
braids of uneven sizes (seeds 1000..1063, drawn as configs.random_braid) in
one persistent launch per RK stage, each case until its weighted force-free
residual reaches R, its dt falls to dtMin, or C accepted steps; it reports
the aggregate cell-RK-stages/s and the p50/p99 time per case, and the same
cases run one after another through the single-case path for comparison.

--impl reference times the reference's relaxation arithmetic on the host
cores: the reference is CUDA-only, so its CPU form is the C restatement in
oracle/ (OpenMP over all cores) on the same workload, with parameters and
initial state from the oracle (the product library is not loaded).

Besides the timed region, the braid6 line carries baselines and comparisons,
each run after the timed region: cpu_baseline (the oracle on the host cores,
a bounded sample), ref_cuda (the reference's own kernels, compiled from its
sources, on the same GPU and workload), warm_start (plain against
warm-started time to residual on three held-out braids) and batched (the
64-case batched configuration).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-RK-stages/s (time to mean|JxB|/(|J||B|)<=1e-2 workload, plain path)"
UNIT = "cell-RK-stages/s"
BYTES_PER_CELL_STAGE = {32: 82, 64: 164}   # algorithmic: 20.5 REALs per cell and stage
SHAPE = (128, 128, 256)


WORKLOAD = "braid6"
LARGE_SHAPE = (256, 256, 512)


def workload_params(precision=32):
    from glemur_gb300 import configs
    if WORKLOAD == "large":
        return configs.braid6_large(*LARGE_SHAPE, precision=precision)
    p = configs.braid6(*SHAPE, precision=precision)
    return p


def workload_config(p, extra=None):
    name = (f"braid6 {p.nx}x{p.ny}x{p.nz}: six alternating twisted blobs, periodic x,y, line-tied z"
            if WORKLOAD != "large" else
            f"large {p.nx}x{p.ny}x{p.nz}: six-blob braid with k = +-1.2, pressure p0 = 0.1 (1 + 0.5 exp(-r^2/4))")
    c = {
        "workload": name,
        "grid": [p.nx, p.ny, p.nz],
        "storage": "fp32" if p.precision == 32 else "fp64",
        "error_norm": ("errMode 1 (the FP32 default): |sum (c - c*) k| per point in the run precision, "
                       "its maximum, t, dt and the controller in fp64" if p.errMode == 1 else
                       "errMode 0: |x_new - x*| in the run precision, as the reference"),
        "step": "one attempted adaptive Cash-Karp RK step (6 stages + accept/reject)",
        "l2": f"working set ~{p.nx * p.ny * p.nz * 117 * (p.precision // 8) / 1e9:.1f} GB > 129 MB L2 "
              "(inputs larger than L2, no flush)",
        "parallelism": "replicas" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else "single",
    }
    if extra:
        c.update(extra)
    return c


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_init():
    """(dist, rank, world_size): NCCL under torchrun; replicas, no exchange."""
    from glemur_gb300 import replicas
    return replicas.init("nccl")


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        # the raw samples: GLEMUR_CLOCKS_CSV keeps them at a chosen path,
        # otherwise a temporary file is used and removed after the summary
        keep = os.environ.get("GLEMUR_CLOCKS_CSV")
        if keep:
            self.path, self.temp = Path(keep), False
        else:
            import tempfile
            fd, name = tempfile.mkstemp(prefix="glemur_clocks_", suffix=".csv")
            os.close(fd)
            self.path, self.temp = Path(name), True

    def __enter__(self):
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()
        self.text = self.path.read_text() if self.path.exists() else ""
        if self.temp:
            self.path.unlink(missing_ok=True)

    def summary(self):
        text = getattr(self, "text", "")
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in text.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (read-only queries)
    about every millisecond in a thread during the timed region, so that a
    timed region of a few milliseconds still has samples.  Falls back to
    nvidia-smi (Clocks) when NVML cannot be loaded."""

    # clock-event reason bits of nvml.h
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu_index=0, period_s=0.001):
        import ctypes as C
        self.C = C
        self.idx, self.period = gpu_index, period_s
        self.samples = []
        self.lib = None
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return
            h = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(gpu_index), C.byref(h)) != 0:
                return
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
            mx = C.c_uint()
            self.max_mhz = float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 else None
            self.lib, self.h = lib, h
        except Exception:
            self.lib = None

    def _run(self):
        C = self.C
        mhz, rs = C.c_uint(), C.c_ulonglong()
        while not self.stop:
            ok1 = self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0     # NVML_CLOCK_SM
            ok2 = self.reasons_fn(self.h, C.byref(rs)) == 0
            if ok1 and ok2:
                self.samples.append((float(mhz.value), int(rs.value)))
            time.sleep(self.period)

    def __enter__(self):
        import threading
        self.stop = False
        self.thread = None
        if self.lib is not None:
            self.thread = threading.Thread(target=self._run, daemon=True)
            self.thread.start()
        return self

    def __exit__(self, *a):
        if self.thread is not None:
            self.stop = True
            self.thread.join(timeout=2)
        if self.lib is not None:
            try:
                self.lib.nvmlShutdown()
            except Exception:
                pass
            self.lib = None

    def summary(self):
        if not self.samples:
            return None
        reasons = sorted({n for _, r in self.samples for bit, n in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(m for m, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples), "sampler": "nvml, ~1 ms"}


def traffic_per_launch(p):
    """DRAM bytes per stage launch from the committed ncu summary, if any."""
    f = ROOT / "profiles" / "stage_kernel_traffic.json"
    if not f.exists():
        return None, None
    d = json.loads(f.read_text())
    key = f"{p.nx}x{p.ny}x{p.nz}_fp{p.precision}" + ("_pressure" if p.pressure else "")
    e = d.get(key)
    if e:
        return float(e["bytes_per_launch"]), e.get("source")
    # a per-point figure measured on a smaller grid of the same kernel scales
    # with the inner points (the traffic is streaming: each plane once)
    e = d.get(f"per_point_fp{p.precision}" + ("_pressure" if p.pressure else ""))
    if not e:
        return None, None
    n = p.nx * p.ny * p.nz
    return float(e["bytes_per_point"]) * n, f"{e.get('source')}, scaled to {n} inner points"


def oracle_workload_params(precision=32):
    """The workload's parameters from the checker's own builder (oracle/params.py),
    byte-identical to workload_params() but without loading the library."""
    from oracle import params as op
    if WORKLOAD == "large":
        return op.braid6_large(*LARGE_SHAPE, precision=precision)
    return op.braid6(*SHAPE, precision=precision)


def cpu_baseline(seconds=20.0):
    """The oracle (C restatement of the reference arithmetic, all host cores)
    on a bounded sample of the workload: whole attempted steps on the full grid.
    Parameters and initial state come from the oracle itself."""
    from oracle.pyoracle import Oracle
    p = oracle_workload_params()
    cores = os.cpu_count() or 1
    B0, xb = Oracle.init_state(p)
    o = Oracle(p, B0, xb)
    o.step()                      # warm-up (first-touch of the arrays)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.step()
        n += 1
        if time.perf_counter() - t0 > seconds or n >= 50:
            break
    dt = time.perf_counter() - t0
    o.close()
    N = p.nx * p.ny * p.nz
    return {"value": N * 6 * n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} attempted steps of the {p.nx}x{p.ny}x{p.nz} workload (OpenMP, {cores} threads)"}


# held-out seeds of the warm-start comparison: offsets 0, 2, 5 from the
# held-out range, the cases tests/test_warmstart_gain.py replays
WARM_SEEDS = (0, 2, 5)
WARM_RESIDUAL = 0.1
WARM_MAX_ATTEMPTS = 12000


def warm_start_comparison():
    """Plain against warm-started relaxation on held-out random braids
    (64x64x128, FP32): wall time from the initial state to the |J||B|-weighted
    force-free residual sum|JxB| / sum|J||B| <= 0.1, the warm start's own cost
    (inference, grid build, validity check) included, with min Delta of each
    run.  Runs after the timed region."""
    from glemur_gb300 import train_warmstart as tw
    from glemur_gb300.warmstart import UNet, WEIGHTS, load_weights, n_params, weights_width
    if not WEIGHTS.exists():
        return None
    w = load_weights()
    net = UNet(tw.SHAPE, seed=0, wb=weights_width(w))
    net.load_state_dict(w)
    seeds = [tw.EVAL_SEED0 + s for s in WARM_SEEDS]
    rows = tw.evaluate(net, seeds, WARM_RESIDUAL, WARM_MAX_ATTEMPTS, log=lambda m: None)
    net.check_status()
    per = [{"seed": r["seed"], "plain_s": r["plain_s"], "warm_s": r["warm_s"], "plain_attempts": r["plain_attempts"],
            "warm_attempts": r["warm_attempts"], "plain_reached": r["plain_reached"],
            "warm_reached": r["warm_reached"], "accepted": r["accepted"], "warm_grid_min_delta": r["warm_minDet"],
            "plain_min_delta": r["plain_minDet"], "residual_after_warm_start": r["warm_res0"],
            "residual_at_identity_grid": r["plain_res0"], "warm_start_cost_s": r["net_s"]} for r in rows]
    tp = sum(r["plain_s"] for r in rows)
    tws = sum(r["warm_s"] for r in rows)
    return {"residual": f"|J||B|-weighted sum|JxB| / sum|J||B| <= {WARM_RESIDUAL} (the unweighted point mean "
                        "levels off near 0.19 on these braids, and 1e-2 is not reached before the grid folds, "
                        "in the reference's kernels too)",
            "grid": list(tw.SHAPE), "seeds": seeds, "network_parameters": n_params(weights_width(w)),
            "weights": str(WEIGHTS.relative_to(ROOT)), "plain_s": tp, "warm_s": tws,
            "speedup_total": tp / tws if tws > 0 else None,
            "accepted": sum(r["accepted"] for r in rows), "cases": per}


def batched_comparison(residual=0.2, max_accepted=3000):
    """The batched configuration on this GPU, after the timed region: 64
    seeded random braids of uneven sizes (seeds 1000..1063, drawn as
    configs.random_braid) in one persistent launch per RK stage, each case
    until its weighted force-free residual reaches `residual`, its dt falls
    to dtMin, or `max_accepted` accepted steps.  Aggregate cell-RK-stages/s
    and the p50 / p99 wall time per case (`--workload batch64` runs the same
    with the single-case comparison)."""
    import torch
    from glemur_gb300 import BatchRelaxation, configs
    ps = [configs.random_braid(1000 + i, precision=32) for i in range(64)]
    inits = [configs.init_state(p) for p in ps]
    b = BatchRelaxation(ps)
    for c, (B0, xb) in enumerate(inits):
        b.upload(c, xb, B0)
    tune = b.autotune(2)
    b.steps_async(3)
    b.state(0)
    for c, (B0, xb) in enumerate(inits):
        b.upload(c, xb, B0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = b.run(max_accepted, residual, pointwise=False, check_every=10)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    b.close()
    work = sum(p.nx * p.ny * p.nz * 6 * o["attempted"] for p, o in zip(ps, out))
    secs = sorted(o["seconds"] for o in out)
    return {"value": work / wall, "unit": UNIT, "wall_s": wall, "cases": 64,
            "p50_case_s": secs[len(secs) // 2], "p99_case_s": secs[min(len(secs) - 1, int(0.99 * len(secs)))],
            "converged": int(sum(o["converged"] for o in out)),
            "folded_dtmin": int(sum(1 for o in out if not o["converged"] and o["status"] & 4)),
            "residual_target": f"|J||B|-weighted residual <= {residual}", "max_accepted": max_accepted,
            "tile_z": tune["tzb"], "what": "64 random braids (seeds 1000..1063) of 32^3, 48x48x96, 64x64x128 and "
                                          "96x96x192 cells, one persistent launch per RK stage under a CUDA graph, "
                                          "run after the timed region"}


def reference_cuda_baseline(steps, warmup):
    """The reference's own CUDA kernels (the cubin nvcc built from the
    reference sources for sm_103a, oracle/_ref) on this GPU and workload,
    driven with src/main.cu's launch sequence and host synchronisations
    (oracle/ref/ref_launcher.cpp).  Parameters and initial state from the
    oracle.  Host wall time of whole attempted steps; None when the cubin is
    absent (it is built only where the reference sources are)."""
    from oracle.pyoracle import REF, RefLauncher, Oracle
    p = oracle_workload_params()
    if not (REF / "libref_launcher.so").exists() or not (REF / f"glemur_ref{p.precision}.cubin").exists():
        return None
    B0, xb = Oracle.init_state(p)
    r = RefLauncher(p, B0, xb)
    try:
        r.time_steps(warmup)
        sec, done = r.time_steps(steps)
    finally:
        r.close()
    N = p.nx * p.ny * p.nz
    return {"value": N * 6 * done / sec, "unit": UNIT, "ms_per_step": 1e3 * sec / max(done, 1), "steps": done,
            "warmup": warmup, "timing": "host wall clock around the reference's launch loop (it synchronises "
                                        "after every kernel)",
            "what": "the reference's own kernels compiled unchanged from its sources for sm_103a, same GPU and "
                    "workload, run outside this line's timed region"}


def run_reference(args):
    """--impl reference: the reference arithmetic on the host cores.  Nothing
    of the product library is loaded: parameters, initial state and the
    relaxation all come from the oracle.  Under torchrun rank 0 alone runs."""
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    from oracle.pyoracle import Oracle
    p = oracle_workload_params()
    B0, xb = Oracle.init_state(p)
    o = Oracle(p, B0, xb)
    for _ in range(args.warmup):
        o.step()
    budget = 150.0
    t0 = time.perf_counter()
    n = 0
    for _ in range(args.steps):
        o.step()
        n += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    N = p.nx * p.ny * p.nz
    value = N * 6 * n / dt
    cores = os.cpu_count() or 1
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": n,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(p),
        "impl_note": "reference relaxation arithmetic on host cores (C restatement in oracle/; the reference "
                     "itself is CUDA-only); parameters and initial state from the oracle, no product library loaded",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} attempted steps of the full grid (bounded at {budget:.0f} s)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    from glemur_gb300 import Relaxation, configs
    dist, rank, ws = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    p = workload_params()
    N = p.nx * p.ny * p.nz
    B0, xb = configs.init_state(p)
    stream = torch.cuda.Stream()
    g = Relaxation(p)
    g.set_stream(stream.cuda_stream)
    g.upload(xb, B0)
    # tile depth chosen by timing (stages 0..4 on the uploaded state, untimed here)
    if args.tile_z:
        g.set_tile_z(args.tile_z)
        tune = {"tz": args.tile_z}
    else:
        tune = g.autotune(3) if not args.no_autotune else None
    # warm-up (also captures the step graph)
    g.steps_async(max(args.warmup, 3))
    g.state()

    # --- device-timed whole-job throughput: K graph replays --------------------
    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
            torch.cuda.synchronize()

    l0 = g.launches
    a0 = g.state()["nAttempted"]
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as ck, NvmlClocks(local) as nk:
        with torch.cuda.stream(stream):
            e0.record(stream)
        g.steps_async(args.steps)
        with torch.cuda.stream(stream):
            e1.record(stream)
        stream.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = g.launches - l0
    st = g.state()
    from glemur_gb300 import replicas
    ms = replicas.max_over_ranks(dist, ms)        # the slowest replica's time
    # the attempted steps counted on the device: a run that stopped early (its
    # status done) skips the remaining replays' work, and they do not count
    ran = st["nAttempted"] - a0
    if ran != args.steps:
        print(f"warning: {ran} of {args.steps} timed steps ran (status {st['status']})", file=sys.stderr)
    value = N * 6 * replicas.sum_over_ranks(dist, ran) / (ms / 1e3)

    # --- roofline of the stage kernel: per-launch time with events -----------
    reps = 3
    stage_ms = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
        for n in range(6):
            g.stage(n)
        with torch.cuda.stream(stream):
            b.record(stream)
        g.control()
        stream.synchronize()
        stage_ms.append(a.elapsed_time(b) / 6)
    launch_ms = statistics.median(stage_ms)
    alg_bytes = BYTES_PER_CELL_STAGE[p.precision] * N
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic, traffic_src = traffic_per_launch(p)

    # --- end to end through the C-ABI with host buffers ------------------------
    xb_h = torch.from_numpy(xb).pin_memory()
    B0_h = torch.from_numpy(B0).pin_memory()
    out_h = torch.empty_like(xb_h).pin_memory()
    g2 = Relaxation(p)
    g2.set_stream(stream.cuda_stream)
    g2.upload_ptr(xb_h.data_ptr(), B0_h.data_ptr())
    if args.tile_z:
        g2.set_tile_z(args.tile_z)
    elif not args.no_autotune:
        g2.autotune(3)
    g2.steps_async(3)
    g2.state()
    barrier()
    t0 = time.perf_counter()
    g2.upload_ptr(xb_h.data_ptr(), B0_h.data_ptr())
    for _ in range(args.steps):
        g2.steps_async(1)
        g2.state()                      # the step's result (t, dt, maxDelta, accepted count) to the host
    import ctypes as C
    from glemur_gb300 import _abi
    _abi.check(g2.lib.gm_download(g2.h, C.c_void_p(out_h.data_ptr()), None, None, None), "gm_download")
    t1 = time.perf_counter()
    barrier()
    e2e_s = t1 - t0
    e2e_s = replicas.max_over_ranks(dist, e2e_s)
    e2e_value = N * 6 * args.steps * ws / e2e_s
    h2d = (xb.nbytes + B0.nbytes) / args.steps
    d2h = (xb.nbytes + 40) / args.steps + 40
    g2.close()

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(seconds=args.cpu_seconds)
    ref_cuda = None
    if rank == 0 and not args.no_ref_cuda:
        ref_cuda = reference_cuda_baseline(args.steps, args.warmup)
    warm = None
    if rank == 0 and not args.no_warm_start and WORKLOAD == "braid6":
        warm = warm_start_comparison()
    batched = None
    if rank == 0 and not args.no_batched and WORKLOAD == "braid6":
        batched = batched_comparison(args.batch_residual, args.batch_cycles)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / max(ran, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(p),
            "run": {"attempted": st["nAttempted"], "accepted": st["timeIndex"], "timed_steps_ran": ran,
                    "tile_z": tune["tz"] if tune else None},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "kernel": "k_stage (one RK stage)",
                         "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": launch_ms,
                         "traffic_source": traffic_src},
            "cpu_baseline": cb,
            "ref_cuda": ref_cuda,
            "warm_start": warm,
            "batched": batched,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "one relaxation job through the C-ABI from pinned host buffers: the grid and B0 "
                            "uploaded once, the step state (t, dt, maxDelta, counts) read back after every "
                            "step, the final grid downloaded once; per-step bytes are those copies divided "
                            "by the steps (the grid stays on the device between steps)"},
            "gpu_launches": launches,
            "clocks": nk.summary() or ck.summary(),
        }
        print(json.dumps(line))
    g.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_batch(args):
    """--workload batch64: the batched configuration (see the module docstring)."""
    import torch
    from glemur_gb300 import BatchRelaxation, Relaxation, configs, replicas
    dist, rank, ws = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    # the 64 cases, split over the ranks (case i on rank i mod N)
    mine = replicas.shard(64, rank, ws)
    ps = [configs.random_braid(1000 + i, precision=32) for i in mine]
    inits = [configs.init_state(p) for p in ps]
    Ns = [p.nx * p.ny * p.nz for p in ps]
    b = BatchRelaxation(ps)
    for c, (B0, xb) in enumerate(inits):
        b.upload(c, xb, B0)
    tune = b.autotune(2) if not args.no_autotune else None   # work-item depth, untimed
    b.steps_async(max(args.warmup, 3))       # warm-up, captures the step graph
    b.state(0)
    for c, (B0, xb) in enumerate(inits):     # start every case afresh
        b.upload(c, xb, B0)
    l0 = b.launches()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as ck:
        t0 = time.perf_counter()
        out = b.run(args.batch_cycles, args.batch_residual, pointwise=False, check_every=10)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = b.launches() - l0
    att = [o["attempted"] for o in out]
    my_work = sum(N * 6 * a for N, a in zip(Ns, att))
    # the job: work summed over the ranks, time of the slowest rank
    work = replicas.sum_over_ranks(dist, my_work)
    wall = replicas.max_over_ranks(dist, wall)
    value = work / wall
    secs = sorted(replicas.gather_lists(dist, [o["seconds"] for o in out]))
    conv = int(replicas.sum_over_ranks(dist, sum(o["converged"] for o in out)))
    folded = int(replicas.sum_over_ranks(dist, sum(1 for o in out if not o["converged"] and o["status"] & 4)))
    total_att = int(replicas.sum_over_ranks(dist, sum(att)))
    launches = int(replicas.sum_over_ranks(dist, launches))
    b.close()
    # the same cases, one after another, same attempted steps, single-case path
    seq_t = 0.0
    for p, (B0, xb), a in zip(ps, inits, att):
        g = Relaxation(p)
        g.upload(xb, B0)
        g.steps_async(3)
        g.state()
        g.upload(xb, B0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g.steps_async(a)
        g.state()
        seq_t += time.perf_counter() - t1
        g.close()
    seq_t = replicas.max_over_ranks(dist, seq_t)
    if rank == 0:
        shapes = {}
        for i in range(64):
            p = configs.random_braid(1000 + i, precision=32)
            k = f"{p.nx}x{p.ny}x{p.nz}"
            shapes[k] = shapes.get(k, 0) + 1
        line = {
            "metric": "cell-RK-stages/s (64 batched random braids, each to weighted residual <= R)",
            "value": value, "unit": UNIT, "n_gpus": ws, "steps": total_att, "warmup": args.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch64: random braids, seeds 1000..1063, 2-8 blobs, sizes drawn from "
                                   "32^3, 48x48x96, 64x64x128, 96x96x192", "shapes": shapes,
                       "residual_target": args.batch_residual, "max_accepted": args.batch_cycles,
                       "check_every": 10, "tile_z": tune["tzb"] if tune else 32,
                       "parallelism": "single" if ws == 1 else f"replicas: case i on rank i mod {ws}"},
            "wall_s": wall, "p50_case_s": secs[len(secs) // 2], "p99_case_s": secs[min(len(secs) - 1, int(0.99 * len(secs)))],
            "converged": conv, "folded_dtmin": folded, "budget_reached": 64 - conv - folded,
            "sequential_single_case": {"value": work / seq_t, "unit": UNIT, "seconds": seq_t},
            "gpu_launches": launches, "clocks": ck.summary(),
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference's own kernels")
    ap.add_argument("--no-warm-start", action="store_true", help="skip the warm-start comparison")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-case batched run")
    ap.add_argument("--no-autotune", action="store_true", help="keep the cost model's tile depth")
    ap.add_argument("--tile-z", type=int, default=0, help="set the stage kernel's z-chunk depth (no autotuning)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--workload", default="braid6", choices=["braid6", "batch64", "large"])
    ap.add_argument("--large-shape", default="256,256,512", help="grid of --workload large")
    ap.add_argument("--batch-residual", type=float, default=0.2)
    ap.add_argument("--batch-cycles", type=int, default=3000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global WORKLOAD, LARGE_SHAPE
    WORKLOAD = args.workload
    LARGE_SHAPE = tuple(int(v) for v in args.large_shape.split(","))
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch64":
        return run_batch(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
