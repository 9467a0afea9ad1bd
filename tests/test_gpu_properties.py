"""Parity at the edges of the input space: small and odd grids (partial
tiles, fewer planes than a z-chunk, three-point directions) against the
oracle; grids below three points, which the library refuses; and the largest
configured grid (256x256x512 with the pressure term and its p0(r) profile)
stage by stage against the oracle.  (A uniform field is no test of rest: its
error estimate is at rounding level, so the step-size rule grows dt far past
the explicit scheme's stability limit until the amplified rounding currents
become visible -- in the oracle as here.)"""
import numpy as np
import pytest

from conftest import inner, relerr
from glemur_gb300 import Relaxation, configs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def braid(shape, xper=1, yper=1, zper=0):
    p = configs.braid_box(*shape, precision=64)
    configs.set_blobs(p, [(0.5, 0.0, -4.0, 1.0, 2.0, 3.0), (-0.5, 0.2, 6.0, -0.8, 1.5, 2.5)])
    p.xPeri, p.yPeri, p.zPeri = xper, yper, zper
    p.errMode = 0
    return configs.derive(p)


@pytest.mark.parametrize("shape,per", [((4, 3, 5), (1, 1, 0)), ((33, 9, 7), (0, 0, 0)), ((5, 17, 40), (1, 0, 1)),
                                       ((3, 6, 4), (1, 1, 1)), ((40, 3, 9), (0, 1, 0))])
def test_small_and_odd_grids_match_oracle(shape, per):
    p = braid(shape, *per)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    o = Oracle(p, B0, xb)
    for _ in range(3):
        g.step()
        o.step()
    g.refresh()
    o.refresh()
    f, fo = g.download(), o.get()
    assert relerr(inner(f["xb"]), inner(fo["xb"])) < 1e-10
    assert relerr(inner(f["B"]), inner(fo["B"])) < 1e-9
    assert relerr(f["J"], fo["J"]) < 1e-8
    g.close()
    o.close()


def test_grids_below_three_points_are_refused():
    from glemur_gb300 import _abi
    p = braid((2, 6, 4), 1, 1, 1)
    with pytest.raises(_abi.GlemurError, match="GM_EPARAM"):
        Relaxation(p)


@pytest.mark.parametrize("precision,tol", [(64, 1e-10), (32, 1e-3)])
def test_large_pressure_case_stages_match_oracle(precision, tol):
    """The largest configured case, 256x256x512 with the pressure term and the
    p0(r) profile: every stage increment of the first step and x_new against
    the oracle.  FP64 checks the full-size path (indexing, tiling, copies) to
    rounding.  In FP32 the pressure term's second differences of positions
    carry rounding noise ulp(|x|) / d^2 (1.9e-6 / 0.0088 near z = 24 at this
    resolution) times beta dt, about 2e-4 of |k| here, and the GPU's fused
    multiply-adds round differently from the oracle's plain operations: hence
    the FP32 tolerance, five times that noise."""
    p = configs.braid6_large(256, 256, 512, precision=precision)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    o = Oracle(p, B0, xb)
    for n in range(6):
        g.stage(n)
        o.stage(n)
        if n < 5:
            assert relerr(g.k(n), o.k(n)) < tol, f"k_{n}"
    o.combine()
    assert relerr(inner(g.x(6)), inner(o.xnew())) < tol, "x_new"
    g.close()
    o.close()


def test_pressure_profile_stages_match_oracle_fp64():
    """The p0(r) pressure profile (this library's extension of the uniform
    reference pressure) stage by stage against the oracle in FP64."""
    p = configs.braid6(20, 16, 24, precision=64, k=1.2)
    p.pressure = 1
    p.beta = 0.1
    p.p0Amp = 0.5
    p.p0Width = 2.0
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    o = Oracle(p, B0, xb)
    for n in range(6):
        g.stage(n)
        o.stage(n)
        if n < 5:
            assert relerr(g.k(n), o.k(n)) < 1e-12, f"k_{n}"
            assert relerr(inner(g.x(n)), inner(o.get()["xb"])) < 1e-12, f"x_{n + 1}"
    o.combine()
    assert relerr(inner(g.x(6)), inner(o.xnew())) < 1e-12
    g.close()
    o.close()


@pytest.mark.parametrize("sym", [1, 4])
def test_mirror_and_swap_equivariance_at_production_size(sym):
    """A size-independent property at the bench size (the six-blob braid on
    128x128x256, FP64): the first stage's increments k_0 from the field moved
    by the x mirror (sym 1) or the x <-> y swap (sym 4) are the moved
    increments, to rounding.  Whole runs are not compared: the oracle shows
    the same symmetry over runs on small grids
    (test_mirror_and_swap_are_symmetries_of_the_relaxation), but at this
    resolution a few ill-conditioned points amplify rounding about 15x per
    stage, so two mirrored runs part at the 1e-5 level within a few steps, in
    the oracle as here."""
    from test_oracle_cpu import _sym_field
    p = configs.braid6(128, 128, 256, precision=64)
    B0, xb = configs.init_state(p)
    ks = []
    for field in (B0, _sym_field(B0, sym)):
        g = Relaxation(p)
        g.upload(xb, field)
        g.stage(0)
        ks.append(g.k(0))
        g.close()
    pad = np.zeros(B0.shape)
    pad[1:-1, 1:-1, 1:-1] = ks[0]
    want = _sym_field(pad, sym)[1:-1, 1:-1, 1:-1]
    assert relerr(ks[1], want) < 1e-11
