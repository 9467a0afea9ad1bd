"""Failure detection on the GPU without a fault: bounded device waits that
are made to run out, through the test hooks of the C-ABI.

* The stage kernel (gm_debug_stall): its copy producer withholds the copies
  of each tile's first position planes, so the bounded mbarrier waits for
  them give up.  The CTA records GM_ST_TIMEOUT, waits (bounded) for the
  copies it did issue and returns; the later stages of the step return at
  once, the controller neither accepts the step nor adapts dt, the run stops
  and gm_run returns GM_ETIMEOUT.  A new handle in the same process then
  relaxes clean and matches the oracle stage by stage.
* The tensor-core convolutions (gm_nn_debug_stall): each CTA first waits on
  an mbarrier that nothing arrives on; the wait runs out before any MMA is
  issued, the CTA frees its tensor memory and sets the status word.  With the
  hook off again the network's forward pass matches its CPU oracle.

Nothing is left in flight and no wait is unbounded, so neither test faults
or hangs the GPU."""
import numpy as np
import pytest

from conftest import inner, relerr
from glemur_gb300 import GlemurError, Relaxation, _abi, configs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

import cases  # noqa: E402


def _one_step_matches_oracle(p, B0, xb):
    g = Relaxation(p)
    g.upload(xb, B0)
    o = Oracle(p, B0, xb)
    for n in range(6):
        g.stage(n)
        o.stage(n)
        if n < 5:
            assert relerr(g.k(n), o.k(n)) < 1e-5, n
    o.combine()
    assert relerr(inner(g.x(6)), inner(o.xnew())) < 1e-5
    g.control()
    assert g.state()["status"] & (_abi.GM_ST_TIMEOUT | _abi.GM_ST_NAN | _abi.GM_ST_ALIGN) == 0
    g.close()
    o.close()


def test_stage_kernel_wait_runs_out_and_stops_the_run():
    p = cases.make("braid_f32")          # runs on the TMA stage kernel
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    lib = _abi.load()
    _abi.check(lib.gm_debug_stall(g.h, 1), "gm_debug_stall")
    with pytest.raises(GlemurError, match="GM_ETIMEOUT"):
        g.run(3)
    s = g.state()
    assert s["status"] & _abi.GM_ST_TIMEOUT
    assert s["timeIndex"] == 0 and s["nAttempted"] == 1 and s["t"] == 0.0
    assert s["dt"] == pytest.approx(p.dt0)
    g.close()
    # the context stays usable: a new handle relaxes and matches the oracle
    _one_step_matches_oracle(p, B0, xb)
    g = Relaxation(p)
    g.upload(xb, B0)
    s = g.run(3)
    assert s["timeIndex"] == 3 and s["status"] & _abi.GM_ST_TIMEOUT == 0
    g.close()


def test_stage_kernel_hook_off_again_runs_clean():
    """The hook is per handle and can be switched off: the same handle then
    runs normally after a fresh upload."""
    p = cases.make("braid_f32")
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    lib = _abi.load()
    _abi.check(lib.gm_debug_stall(g.h, 1), "gm_debug_stall")
    with pytest.raises(GlemurError, match="GM_ETIMEOUT"):
        g.run(1)
    _abi.check(lib.gm_debug_stall(g.h, 0), "gm_debug_stall")
    g.upload(xb, B0)
    s = g.run(3)
    assert s["timeIndex"] == 3 and s["status"] & _abi.GM_ST_TIMEOUT == 0
    g.close()


def test_convolution_wait_runs_out_and_is_reported():
    import torch
    from glemur_gb300.warmstart import UNet
    from oracle import unet_oracle as uo

    nx, ny, nz = 8, 8, 16
    net = UNet((nx, ny, nz), seed=3)
    rng = np.random.default_rng(7)
    x = rng.normal(size=(nz, ny, nx, 3))
    X0 = np.zeros((nx * ny * nz, 8), np.float32)
    X0[:, :3] = x.reshape(-1, 3)
    net.A["X0"].copy_(torch.from_numpy(X0).to(torch.bfloat16))
    lib = _abi.load()
    try:
        _abi.check(lib.gm_nn_debug_stall(1), "gm_nn_debug_stall")
        net.forward()
        torch.cuda.synchronize()
    finally:
        _abi.check(lib.gm_nn_debug_stall(0), "gm_nn_debug_stall")
    with pytest.raises(GlemurError):
        net.check_status()
    # the device is still usable: the forward pass runs and matches the oracle
    net.status.zero_()
    y = net.forward()
    torch.cuda.synchronize()
    net.check_status()

    def bf16(a):
        u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
        return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32).astype(np.float64)

    P = {n: (bf16(W), b) for n, (W, b) in net.params_numpy().items()}
    a = uo.forward(P, bf16(x))
    yg = y[:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3)
    assert np.linalg.norm(yg - a["y"]) / np.linalg.norm(a["y"]) < 1.5e-2
