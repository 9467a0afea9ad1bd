"""The learned warm start pays: with the shipped weights
(glemur_gb300/weights/unet_64x64x128.npz), held-out random braids on the
64x64x128 grid reach the force-free residual 0.1 sooner from the network's
grid than from the identity grid, counting the warm start's own cost
(inference, the grid build on the device, the min Delta > 0 acceptance
check) in its time.  The held-out seeds lie outside the training range; every predicted
grid must be accepted (no folded cell).  The predicted grid starts at a
higher residual than the identity grid (its small grid-scale errors show up
as current), but its displacement is close to the relaxed one, so it needs
far fewer attempts: on these seeds 1150 / 2050 / 950 against 3900 / 5050 /
2650, and 2.1x less total wall time over 256 held-out seeds."""
import pytest

pytestmark = pytest.mark.gpu

SEEDS = (0, 2, 5)          # offsets from the held-out seed range
RESIDUAL = 0.1
MAX_ATTEMPTS = 12000


def test_warm_start_reaches_residual_sooner():
    from glemur_gb300 import train_warmstart as tw
    from glemur_gb300.warmstart import UNet, WEIGHTS, load_weights, weights_width
    assert WEIGHTS.exists(), f"missing trained weights {WEIGHTS}"
    w = load_weights()
    net = UNet(tw.SHAPE, seed=0, wb=weights_width(w))
    net.load_state_dict(w)
    rows = tw.evaluate(net, [tw.EVAL_SEED0 + s for s in SEEDS], RESIDUAL, MAX_ATTEMPTS, log=lambda m: None)
    net.check_status()
    for r in rows:
        assert r["accepted"], r
        assert r["warm_minDet"] > 0, r
        assert r["plain_reached"] and r["warm_reached"], r
        # the relaxation from the network's grid is much shorter
        assert r["warm_attempts"] < 0.75 * r["plain_attempts"], r
    wins = sum(r["warm_s"] < r["plain_s"] for r in rows)
    assert wins >= 2, [(r["plain_s"], r["warm_s"]) for r in rows]
    assert sum(r["warm_s"] for r in rows) < sum(r["plain_s"] for r in rows)
