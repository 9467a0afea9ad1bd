"""The seeded random braids of the batched and warm-start workloads
(glemur_gb300/configs.py: random_braid) against their specification:
2-8 blobs; per blob twist k ~ +-U[0.5, 1.2] with a uniform sign, scale
a ~ U[1, 2], length l ~ U[1.5, 3], centre (x, y) ~ U[-2, 2]^2 and heights
evenly spread, z_b = Oz + (b + 1/2) Lz / nBlobs; grids drawn from 32^3,
48x48x96, 64x64x128 and 96x96x192.  The parameter mapping is the
reference's blob field (src/init.cu:109-124): blobTwist = k a / 2,
blobScale = a, blobZl = l."""
import numpy as np

from glemur_gb300 import configs

SHAPES = {(32, 32, 32), (48, 48, 96), (64, 64, 128), (96, 96, 192)}


def _blobs(p):
    n = p.nBlobs
    return [dict(x=p.blobXc[b], y=p.blobYc[b], z=p.blobZc[b], a=p.blobScale[b], l=p.blobZl[b],
                 k=2 * p.blobTwist[b] / p.blobScale[b]) for b in range(n)]


def test_random_braids_follow_their_distribution():
    counts, shapes, signs = set(), set(), set()
    ks, As, ls, xs = [], [], [], []
    for seed in range(400):
        p = configs.random_braid(seed, precision=64)
        shapes.add((p.nx, p.ny, p.nz))
        counts.add(p.nBlobs)
        assert 2 <= p.nBlobs <= 8
        for b, d in enumerate(_blobs(p)):
            assert 0.5 <= abs(d["k"]) <= 1.2 + 1e-12
            assert 1.0 <= d["a"] <= 2.0 and 1.5 <= d["l"] <= 3.0
            assert -2.0 <= d["x"] <= 2.0 and -2.0 <= d["y"] <= 2.0
            assert abs(d["z"] - (p.Oz + (b + 0.5) * p.Lz / p.nBlobs)) < 1e-12
            signs.add(np.sign(d["k"]))
            ks.append(abs(d["k"])); As.append(d["a"]); ls.append(d["l"]); xs.append(d["x"])
    assert shapes == SHAPES and counts == set(range(2, 9)) and signs == {-1.0, 1.0}
    # uniform draws: means near the interval centres
    assert abs(np.mean(ks) - 0.85) < 0.03 and abs(np.mean(As) - 1.5) < 0.03
    assert abs(np.mean(ls) - 2.25) < 0.05 and abs(np.mean(xs)) < 0.1


def test_random_braids_are_reproducible_and_distinct():
    a, b = configs.random_braid(17), configs.random_braid(17)
    assert bytes(a) == bytes(b)
    assert bytes(configs.random_braid(18)) != bytes(a)
    p = configs.random_braid(5, shape=(40, 24, 56))
    assert (p.nx, p.ny, p.nz) == (40, 24, 56)


def test_warm_start_seed_ranges_are_disjoint():
    """Training pairs use seeds TRAIN_SEED0 + i (up to the 4096 braids the
    configuration names), held-out evaluation EVAL_SEED0 + i (256), and the
    batched bench 1000..1063: no seed is shared."""
    from glemur_gb300 import train_warmstart as tw
    train = set(range(tw.TRAIN_SEED0, tw.TRAIN_SEED0 + 4096))
    held = set(range(tw.EVAL_SEED0, tw.EVAL_SEED0 + 256))
    bench = set(range(1000, 1064))
    assert not train & held and not train & bench and not held & bench
