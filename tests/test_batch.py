"""Batched relaxation: many cases of uneven sizes in one persistent launch per
stage.  Every case must evolve exactly as it does alone (the arithmetic per
point does not depend on the tiling, and each case has its own controller),
stopped cases must stay frozen, and gm_batch_run must stop each case at its
residual, its step budget or its own stop rule."""
import ctypes as C

import numpy as np
import pytest

from glemur_gb300 import BatchRelaxation, Relaxation, _abi, configs


def cases(precision):
    ps = [configs.braid2(16, 16, 32, precision=precision),
          configs.random_braid(3, shape=(32, 32, 32), precision=precision),
          configs.random_braid(5, shape=(48, 24, 40), precision=precision),
          configs.random_braid(8, shape=(20, 12, 70), precision=precision)]
    ps[2].zPeri = 1     # a periodic-z case in the same launch
    ps[3].xPeri = 0     # and a line-tied x face
    return [configs.derive(p) for p in ps]


def test_mixed_precision_refused():
    a = configs.braid2(8, 8, 8, precision=64)
    b = configs.braid2(8, 8, 8, precision=32)
    arr = (_abi.GmParams * 2)(a, b)
    h = C.c_void_p()
    assert _abi.load().gm_batch_create(arr, 2, C.byref(h)) == _abi.GM_EPARAM


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_batch_equals_single_case_runs(precision):
    ps = cases(precision)
    b = BatchRelaxation(ps)
    singles = []
    for c, p in enumerate(ps):
        B0, xb = configs.init_state(p)
        b.upload(c, xb, B0)
        g = Relaxation(p)
        g.upload(xb, B0)
        singles.append(g)
    nsteps = 40
    b.steps_async(nsteps)
    for c, g in enumerate(singles):
        g.steps_async(nsteps)
        s1, s2 = b.state(c), g.state()
        for k in ("t", "dt", "maxDelta", "timeIndex", "nAttempted", "nRejected"):
            assert s1[k] == s2[k], (c, k, s1[k], s2[k])
        r1, r2 = b.refresh(c), g.refresh()
        assert r1 == r2
        f1, f2 = b.download(c), g.download()
        for k in ("xb", "B", "J", "detJac"):
            np.testing.assert_array_equal(f1[k], f2[k], err_msg=f"case {c} {k}")
        g.close()
    assert b.launches() == 7 * nsteps
    b.close()


@pytest.mark.gpu
def test_stopped_case_stays_frozen():
    ps = cases(32)
    b = BatchRelaxation(ps)
    for c, p in enumerate(ps):
        B0, xb = configs.init_state(p)
        b.upload(c, xb, B0)
    b.steps_async(5)
    b.stop(1)
    before = b.download(1)["xb"].copy()
    s_before = b.state(1)
    b.steps_async(10)
    assert b.state(1)["nAttempted"] == s_before["nAttempted"]
    np.testing.assert_array_equal(b.download(1)["xb"], before)
    assert b.state(0)["nAttempted"] == 15
    b.close()


@pytest.mark.gpu
def test_batch_run_stops_each_case():
    ps = cases(32)
    b = BatchRelaxation(ps)
    for c, p in enumerate(ps):
        B0, xb = configs.init_state(p)
        b.upload(c, xb, B0)
    start = [b.refresh(c)["residual"] for c in range(len(ps))]
    # a target between the start residuals: some cases converge, the rest hit the step budget
    target = float(np.median(start)) * 0.8
    out = b.run(nCycle=300, residual=target, check_every=5)
    for c, o in enumerate(out):
        s = b.state(c)
        if o["converged"]:
            assert o["residual"] <= target
            assert s["timeIndex"] <= 300
        else:
            assert s["timeIndex"] == 300 or s["status"] & _abi.GM_ST_DTMIN
        assert o["seconds"] > 0 and o["attempted"] == s["nAttempted"]
    assert any(o["converged"] for o in out)
    b.close()


@pytest.mark.gpu
def test_autotuners_keep_results_identical():
    """gm_autotune / gm_batch_autotune time tile depths on the uploaded state
    (stages 0..4 only) and keep the fastest: the run that follows must equal
    an untuned run bit for bit, since no arithmetic depends on the tiling."""
    p = configs.random_braid(11, shape=(64, 48, 96), precision=32)
    B0, xb = configs.init_state(p)
    runs = []
    for tune in (False, True):
        g = Relaxation(p)
        g.upload(xb, B0)
        if tune:
            r = g.autotune(2)
            assert r["tz"] >= 4 and r["ms_stages_0_4"] > 0
        g.steps_async(30)
        runs.append((g.state(), g.download()))
        g.close()
    (s0, f0), (s1, f1) = runs
    for k in ("t", "dt", "timeIndex", "nAttempted"):
        assert s0[k] == s1[k], k
    np.testing.assert_array_equal(f0["xb"], f1["xb"])
    ps = cases(32)
    outs = []
    for tune in (False, True):
        b = BatchRelaxation(ps)
        for c, q in enumerate(ps):
            B0, xb = configs.init_state(q)
            b.upload(c, xb, B0)
        if tune:
            r = b.autotune(2)
            assert r["tzb"] in (16, 32, 64) and r["ms_stages_0_4"] > 0
        b.steps_async(20)
        outs.append([(b.state(c)["nAttempted"], b.download(c)["xb"]) for c in range(len(ps))])
        b.close()
    for (n0, x0), (n1, x1) in zip(*outs):
        assert n0 == n1
        np.testing.assert_array_equal(x0, x1)
