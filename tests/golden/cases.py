"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a small relaxation chosen to exercise one part of the
reference's boundary handling:

* braid_f64 / braid_f32 -- periodic x, y; line-tied z; 17 points across so the
  line-tied ghost planes cross an edge of the reference's 16-wide launch
  blocks (src/boundaries.cu:72-109).
* tied_f64   -- every face line-tied (the x and y ghost-face formulas).
* zperi_f64  -- periodic y and z, line-tied x.
* press_f64  -- the pressure term (src/gradP.cu) with uniform p0 = beta.
* analytic_f64 -- the reference's analytic field (src/init.cu:71-78).
* classic_tied_f64 / classic_tied_f32 -- the finite-difference current
  (jMethod = "Classic", src/current.cu:10-218) with every face line-tied.
  (With a periodic face the reference's ghost detJac there is not defined on
  every row -- updateBbound's periodic branch, boundaries.cu:278,406 -- and
  the Classic current reads it, so periodic Classic runs are checked against
  the oracle only.)
* inertia_f64 / inertia_f32 -- the velocity equation (inertia = T,
  src/rungeKutta.cu:195-212, 311-322) with damping nu = 1.
* inertia_press_f64, classic_press_tied_f64, classic_inertia_tied_f64 -- the
  options together: the pressure force in the velocity equation, the
  pressure gradient beside the Classic current (both read Delta), and the
  Classic current driving the velocity equation.
* jxbaver_f64 -- the neighbour-averaged Lorentz force (jxbAver = T,
  src/rungeKutta.cu:172-178, 357-443), weight 0.3.
* oct_f64 / oct_tied_f64 / oct_f32 -- the octilateral Stokes current
  (jMethod = "Stokes4th", src/current.cu:413-736), periodic x, y and every
  face line-tied: it reads B at the in-plane edge neighbours, ghost edges
  included.
* quint_f64 / quint_tied_f64 -- the quintilateral Stokes current
  (jMethod = "StokesQuint", src/current.cu:737-1199).
* tri_tied_f64 -- the triangular Stokes current (jMethod = "StokesTri",
  src/current.cu:1202-1681), every face line-tied.
* shear_f64 / shear_f32 -- an initially sheared grid (initDist =
  "initShearX", src/init.cu:401-407): the line-tied z ghost planes carry the
  addDist correction (src/boundaries.cu:11-35, 63-107).
* centershift_tied_f64 (checked live against the reference's kernels, no
  fixture) -- initDist = "centerShift" on a small all-line-tied box.
"""
from __future__ import annotations

import math

from glemur_gb300 import configs


def _braid(shape, precision, peri=(1, 1, 0)):
    p = configs.braid2(*shape, precision=precision)
    p.xPeri, p.yPeri, p.zPeri = peri
    p.errMode = 0
    return configs.derive(p)


def make(name: str):
    if name == "braid_f64":
        return _braid((17, 17, 18), 64)
    if name == "braid_f32":
        return _braid((17, 17, 18), 32)
    if name == "tied_f64":
        return _braid((17, 12, 17), 64, peri=(0, 0, 0))
    if name == "zperi_f64":
        return _braid((12, 10, 16), 64, peri=(0, 1, 1))
    if name == "press_f64":
        p = _braid((12, 12, 14), 64)
        p.pressure = 1
        p.beta = 0.05
        return configs.derive(p)
    if name in ("classic_tied_f64", "classic_tied_f32"):
        p = _braid((17, 12, 17), 64 if name.endswith("64") else 32, peri=(0, 0, 0))
        p.set_str("jMethod", "Classic")
        return configs.derive(p)
    if name in ("inertia_f64", "inertia_f32"):
        p = _braid((17, 17, 18), 64 if name.endswith("64") else 32)
        p.inertia = 1
        p.nu = 1.0
        return configs.derive(p)
    if name == "inertia_press_f64":
        p = _braid((17, 17, 18), 64)
        p.inertia = 1
        p.nu = 1.0
        p.pressure = 1
        p.beta = 0.05
        return configs.derive(p)
    if name in ("classic_press_tied_f64", "classic_inertia_tied_f64"):
        # nz = 18 with inertia: the reference's inertia blocks are 4 deep, and
        # JClassic leaves the edge halo of a block one layer deep unloaded
        p = _braid((17, 12, 17 if name == "classic_press_tied_f64" else 18), 64, peri=(0, 0, 0))
        p.set_str("jMethod", "Classic")
        if name == "classic_press_tied_f64":
            p.pressure = 1
            p.beta = 0.05
        else:
            p.inertia = 1
            p.nu = 1.0
        return configs.derive(p)
    if name == "jxbaver_f64":
        p = _braid((17, 17, 18), 64)
        p.jxbAver = 1
        p.jxbAverWeight = 0.3
        return configs.derive(p)
    if name in ("oct_f64", "oct_tied_f64", "oct_f32"):
        if name == "oct_tied_f64":
            p = _braid((17, 12, 17), 64, peri=(0, 0, 0))
        else:
            p = _braid((17, 17, 18), 32 if name.endswith("32") else 64)
        p.set_str("jMethod", "Stokes4th")
        return configs.derive(p)
    if name == "tri_tied_f64":
        p = _braid((17, 12, 17), 64, peri=(0, 0, 0))
        p.set_str("jMethod", "StokesTri")
        return configs.derive(p)
    if name in ("quint_f64", "quint_tied_f64"):
        p = _braid((17, 12, 17), 64, peri=(0, 0, 0)) if name == "quint_tied_f64" else _braid((17, 17, 18), 64)
        p.set_str("jMethod", "StokesQuint")
        return configs.derive(p)
    if name in ("shear_f64", "shear_f32"):
        p = _braid((17, 17, 18), 64 if name.endswith("64") else 32)
        p.set_str("initDist", "initShearX")
        p.initDistCode = 0
        p.initShearA, p.initShearB, p.initShearK = p.rnd(0.05), p.rnd(0.03), 1.0
        return configs.derive(p)
    if name == "centershift_tied_f64":
        p = configs.braid2(17, 17, 12, precision=64)
        p.xPeri = p.yPeri = p.zPeri = 0
        p.Lx, p.Ly, p.Lz = 2.0, 2.0, 4.0
        p.Ox, p.Oy, p.Oz = -1.0, -1.0, 0.0
        configs.set_blobs(p, [(0.3, 0.0, 1.5, 1.0, 0.5, 0.8), (-0.3, 0.0, 2.5, -1.0, 0.5, 0.8)])
        p.errMode = 0
        p.set_str("initDist", "centerShift")
        p.initDistCode = 1
        p.initShearA, p.initShearB, p.initShearK = 0.02, 0.0, 1.0
        return configs.derive(p)
    if name == "analytic_f64":
        p = configs.defaults(64)
        p.nx, p.ny, p.nz = 16, 16, 16
        p.Lx, p.Ly, p.Lz = 8.0, 8.0, 20.0
        p.Ox, p.Oy, p.Oz = -4.0, -4.0, -10.0
        p.set_str("bInit", "analytic")
        p.ampl = 1.0
        p.phi1 = math.pi / 2
        p.phi2 = -math.pi / 2
        p.dt0 = 3e-4
        p.dtMin = 1e-8
        p.maxError = 5e-6
        p.errMode = 0
        return configs.derive(p)
    raise KeyError(name)


NAMES = ["braid_f64", "braid_f32", "tied_f64", "zperi_f64", "press_f64", "analytic_f64", "classic_tied_f64",
         "classic_tied_f32", "inertia_f64", "inertia_f32", "inertia_press_f64", "classic_press_tied_f64",
         "classic_inertia_tied_f64", "jxbaver_f64", "oct_f64", "oct_tied_f64", "oct_f32", "quint_f64",
         "quint_tied_f64", "tri_tied_f64", "shear_f64", "shear_f32"]
N_ACCEPTED = 10
