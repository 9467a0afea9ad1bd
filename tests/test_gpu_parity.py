"""GPU parity: the CUDA path through the C-ABI against the oracle and against
the reference's own kernels, stage by stage and over whole runs.

Tolerances (max |a-b| / max |b| per field): FP64 1e-12 after one stage and
1e-10 after N steps; FP32 storage 1e-5 (J: x100, since J is a difference
quotient of B and so loses the leading digits)."""
import numpy as np
import pytest

from conftest import inner, relerr
from glemur_gb300 import Relaxation, configs
from oracle.pyoracle import Oracle, RefLauncher

pytestmark = pytest.mark.gpu

import cases  # noqa: E402


def tolerances(p):
    return (1e-12, 1e-10) if p.precision == 64 else (1e-5, 1e-5)


def stage_by_stage(p, ref):
    """Run the six stages with the library and `ref` (oracle or reference
    kernels) and compare k_n and x_{n+1} after each."""
    tol, _ = tolerances(p)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    r = ref(p, B0, xb)
    for n in range(6):
        g.stage(n)
        r.stage(n)
        if n < 5:
            assert relerr(g.k(n), r.k(n)) < tol, f"k_{n}"
            assert relerr(inner(g.x(n)), inner(r.get()["xb"])) < tol, f"x_{n + 1}"
    md = r.combine()
    assert relerr(inner(g.x(6)), inner(r.xnew())) < tol, "x_new"
    assert relerr(inner(g.x(5)), inner(r.get()["xb"])) < tol, "x_6"
    g.control()
    s = g.state()
    assert abs(s["maxDelta"] - md) <= max(tol * 100 * md, 1e-300)
    g.close()
    r.close()


@pytest.mark.parametrize("name", cases.NAMES)
def test_stages_match_oracle(name):
    stage_by_stage(cases.make(name), Oracle)


@pytest.mark.parametrize("name", ["braid_f64", "braid_f32", "tied_f64", "press_f64"])
def test_stages_match_reference_kernels(name):
    stage_by_stage(cases.make(name), RefLauncher)


@pytest.mark.parametrize("name", cases.NAMES)
def test_run_matches_oracle(name):
    p = cases.make(name)
    _, tol = tolerances(p)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    o = Oracle(p, B0, xb)
    nacc = 25
    sg = g.run(nacc)
    n, lg = o.run(nacc, log=True)
    so = o.scalars()
    assert sg["timeIndex"] == so["timeIndex"] == nacc
    assert sg["nAttempted"] == so["nAttempted"], "accept/reject sequences differ"
    assert abs(sg["t"] - so["t"]) <= tol * abs(so["t"]) * 10
    red = g.refresh()
    o.refresh()
    f = g.download()
    fo = o.get()
    assert relerr(inner(f["xb"]), inner(fo["xb"])) < tol
    assert relerr(inner(f["B"]), inner(fo["B"])) < tol * 10
    assert relerr(f["J"], fo["J"]) < tol * 100
    assert relerr(inner(f["detJac"]), inner(fo["detJac"])) < tol * 10
    ro = o.reduce()
    for k in ("B2", "JMax", "JxB_B2Max", "residual", "residualPw", "minDetJac", "wedgeMin"):
        assert abs(red[k] - ro[k]) <= 1e-6 * max(abs(ro[k]), 1e-30) + (1e-4 if p.precision == 32 else 1e-9) * abs(ro[k]), k
    assert red["convex"] == ro["convex"]


def test_braid2_fp64_2000_steps_vs_reference_kernels():
    """The 32x32x64 two-blob braid in FP64 for 2000 accepted steps: x, B and
    J against the reference's own kernels to 1e-10."""
    p = configs.braid2(precision=64)
    p.errMode = 0
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    sg = g.run(2000)
    g.refresh()
    f = g.download()
    r = RefLauncher(p, B0, xb)
    n, lg = r.run(2000, max_attempts=100000)
    fr = r.get()
    sr = r.scalars()
    r.close()
    assert sg["timeIndex"] == sr["timeIndex"] == 2000
    assert sg["nAttempted"] == sr["nAttempted"]
    assert relerr(inner(f["xb"]), inner(fr["xb"])) < 1e-10
    assert relerr(inner(f["B"]), inner(fr["B"])) < 1e-10
    assert relerr(f["J"], fr["J"]) < 1e-10


def test_fp32_storage_vs_fp64_step():
    """FP32 storage against FP64 over one attempted step from the same state
    and dt (the only difference is rounding)."""
    p64 = configs.braid2(24, 24, 48, precision=64)
    p32 = configs.braid2(24, 24, 48, precision=32)
    B0, xb = configs.init_state(p64)
    g64 = Relaxation(p64)
    g64.upload(xb, B0)
    g32 = Relaxation(p32)
    g32.upload(xb.astype(np.float32), B0.astype(np.float32))
    for n in range(6):
        g64.stage(n)
        g32.stage(n)
    for m in range(5):
        assert relerr(g32.k(m), g64.k(m)) < 1e-5
    assert relerr(g32.x(6), g64.x(6)) < 1e-6
    g64.control()
    g32.control()
    g64.refresh()
    g32.refresh()
    f64, f32 = g64.download(), g32.download()
    assert relerr(inner(f32["B"]), inner(f64["B"])) < 1e-5
    assert relerr(f32["J"], f64["J"]) < 1e-3


def test_graph_replay_equals_single_steps():
    p = cases.make("braid_f64")
    B0, xb = configs.init_state(p)
    a = Relaxation(p)
    a.upload(xb, B0)
    b = Relaxation(p)
    b.upload(xb, B0)
    for _ in range(12):
        a.step()
    b.steps_async(12)
    sa, sb = a.state(), b.state()
    assert sa["nAttempted"] == sb["nAttempted"] == 12
    assert np.array_equal(a.grid(), b.grid())


def test_run_stops_at_dtmin():
    p = cases.make("braid_f64")
    p.dtMin = 1.0            # above dt0: the reference loop never starts
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    s = g.run(10)
    assert s["nAttempted"] == 0
    assert s["status"] & 4


def test_nan_in_b0_is_reported():
    p = cases.make("braid_f64")
    B0, xb = configs.init_state(p)
    B0[5, 5, 5, 0] = np.nan
    g = Relaxation(p)
    g.upload(xb, B0)
    with pytest.raises(Exception):
        g.run(5)
    assert g.state()["status"] & 1
