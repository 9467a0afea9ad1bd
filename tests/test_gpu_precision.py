"""What FP32 storage costs the relaxation at production size: the six-blob
braid on 128x128x256 inner points (the bench workload), run with FP32 storage
and the cancellation-free error norm (errMode 1, the FP32 default) and in
FP64 with the reference's arithmetic (errMode 0), compared at matched
physical time.

The two runs take different dt sequences, so they are compared at the FP32
run's time t32 after N accepted steps: the FP64 grid is interpolated linearly
in t between its two steps around t32, and B and J of the FP64 run are
recomputed at that interpolated grid (a fresh FP64 handle, gm_refresh).  The
errors are max |a - b| / max |b| for B and J, the position difference against
the largest displacement, and the relative difference of the |J||B|-weighted
force-free residual; the test prints them.  Measured on a GB300:

  100 FP32 steps (t = 0.427): x 7.6e-3, B 6.5e-4, J 6.4e-3, residual 5.7e-4
  500 FP32 steps (t = 2.253): x 1.3e-2, B 9.6e-4, J 1.1e-2, residual 1.1e-3

The two runs' controllers take different dt sequences, each step's error
bounded by maxError = 1e-5 in position, so the difference holds both runs'
truncation errors as well as the FP32 rounding; the bounds are about twice
the measured values."""
import numpy as np
import pytest

from conftest import inner, relerr
from glemur_gb300 import Relaxation, configs

pytestmark = pytest.mark.gpu

SHAPE = (128, 128, 256)


def _fp64_at_time(p64, B0, xb, t_target):
    """FP64 run until t >= t_target; the grid interpolated linearly to
    t_target between the two accepted steps around it."""
    g = Relaxation(p64)
    g.upload(xb, B0)
    prev_t, prev_x = 0.0, xb.astype(np.float64)
    s = g.state()
    while s["t"] < t_target:
        if s["t"] + 2.5 * s["dt"] >= t_target:
            prev_t, prev_x = s["t"], g.grid()
        s = g.run(1)
        assert s["status"] & 0x17 == 0, s
    t1, x1 = s["t"], g.grid()
    g.close()
    w = (t_target - prev_t) / (t1 - prev_t)
    return (1 - w) * prev_x + w * x1


def _fields_at(p, B0, xb):
    g = Relaxation(p)
    g.upload(xb, B0)
    red = g.refresh()
    f = g.download()
    g.close()
    return f, red


def test_fp32_storage_error_against_fp64_at_production_size():
    p32 = configs.braid6(*SHAPE, precision=32)
    p64 = configs.braid6(*SHAPE, precision=64)
    p64.errMode = 0
    p64 = configs.derive(p64)
    B064, xb64 = configs.init_state(p64)
    B032, xb32 = configs.init_state(p32)
    g32 = Relaxation(p32)
    g32.upload(xb32, B032)
    done = 0
    rows = []
    for n in (100, 500):
        s32 = g32.run(n - done)
        done = n
        t32 = s32["t"]
        red32 = g32.refresh()
        f32 = g32.download()
        x64 = _fp64_at_time(p64, B064, xb64, t32)
        f64, red64 = _fields_at(p64, B064, x64)
        disp = np.abs(inner(x64) - inner(xb64)).max()
        ex = np.abs(inner(f32["xb"]).astype(np.float64) - inner(x64)).max() / disp
        eB = relerr(inner(f32["B"]), inner(f64["B"]))
        eJ = relerr(f32["J"], f64["J"])
        er = abs(red32["residual"] - red64["residual"]) / red64["residual"]
        print(f"FP32 vs FP64 at {n} accepted FP32 steps (t = {t32:.4f}): max|dx|/max disp {ex:.2e}, "
              f"B {eB:.2e}, J {eJ:.2e}, weighted residual {er:.2e} (FP64 {red64['residual']:.4e}), "
              f"max displacement {disp:.3e}")
        rows.append((n, ex, eB, eJ, er, disp))
    g32.close()
    for n, ex, eB, eJ, er, disp in rows:
        assert disp > 0.01                       # the grid has moved
        assert ex < 2.5e-2 and eB < 2e-3 and eJ < 2.2e-2 and er < 2.5e-3, (n, ex, eB, eJ, er)
