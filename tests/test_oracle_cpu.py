"""CPU checks of the oracle: known answers the reference's own diagnostics
imply (src/init.cu:13-26, 71-106; src/maths.cu:294-377) and the golden
fixtures produced by the reference's own kernels."""
from pathlib import Path

import numpy as np
import pytest

from conftest import inner, relerr
from glemur_gb300 import configs
from oracle.pyoracle import Oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def small(precision=64, shape=(12, 10, 14)):
    p = configs.braid2(*shape, precision=precision)
    p.errMode = 0
    return configs.derive(p)


def test_identity_grid_gives_b0_and_unit_jacobian():
    p = small()
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    f = o.get()
    assert np.allclose(inner(f["detJac"]), 1.0, atol=1e-13)
    assert relerr(inner(f["B"]), inner(B0)) < 1e-13


def test_homz_is_a_fixed_point():
    # B0 = ampl e_z gives J = 0, so k = 0 and the grid stays bit-identical
    p = small()
    p.set_str("bInit", "homZ")
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    n = o.run(5)
    assert n == 5
    assert np.array_equal(inner(o.get()["xb"]), inner(xb))
    assert o.scalars()["maxDelta"] == 0.0


def test_stokes_current_exact_for_linear_field_on_affine_grid():
    # On an affine grid x = A X and B linear in x, the circulation around the
    # planar quads is exact, so J equals the analytic curl.
    p = small(shape=(8, 8, 8))
    p.xPeri = p.yPeri = p.zPeri = 0
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    A = np.array([[1.1, 0.2, 0.0], [0.1, 0.9, 0.15], [0.0, 0.05, 1.2]])
    X = xb.reshape(-1, 3)
    x = (X @ A.T).reshape(xb.shape)
    # B0 chosen so that B = A B0 / det A equals a field with constant curl
    M = np.array([[0.0, 0.3, -0.2], [-0.1, 0.0, 0.4], [0.25, -0.05, 0.0]])   # B(x) = M x + e_z
    Bx = (x.reshape(-1, 3) @ M.T + np.array([0, 0, 1.0])).reshape(xb.shape)
    detA = np.linalg.det(A)
    B0n = (np.linalg.solve(A, Bx.reshape(-1, 3).T).T * detA).reshape(xb.shape)
    o = Oracle(p, B0n, x)
    o.refresh()
    f = o.get()
    curl = np.array([M[2, 1] - M[1, 2], M[0, 2] - M[2, 0], M[1, 0] - M[0, 1]])
    J = f["J"].reshape(-1, 3)
    # interior points only (the line-tied ghost formula extrapolates)
    Jin = f["J"][1:-1, 1:-1, 1:-1].reshape(-1, 3)
    assert np.allclose(Jin, curl[None, :], atol=1e-11), np.abs(Jin - curl).max()
    assert J.shape[0] == 8 * 8 * 8


def test_analytic_field_relaxes_towards_known_state():
    # bInit = "analytic" has a known relaxed grid (src/maths.cu:332-377)
    p = configs.defaults(64)
    p.nx, p.ny, p.nz = 12, 12, 12
    p.Lx, p.Ly, p.Lz = 8.0, 8.0, 20.0
    p.Ox, p.Oy, p.Oz = -4.0, -4.0, -10.0
    p.set_str("bInit", "analytic")
    p.phi1 = np.pi / 2
    p.maxError = 1e-5
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    e0 = o.reduce()
    o.run(150)
    o.refresh()
    e1 = o.reduce()
    assert e1["errB_1ez"] < 0.5 * e0["errB_1ez"]
    assert e1["errXb_XbAn"] < e0["errXb_XbAn"]
    assert e1["residual"] < e0["residual"]


def test_energy_decreases_and_cells_stay_valid():
    p = small()
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    r0 = o.reduce()
    o.run(40)
    o.refresh()
    r1 = o.reduce()
    assert r1["B2"] < r0["B2"]
    assert r1["minDetJac"] > 0 and r1["wedgeMin"] > 0


def test_fp32_tracks_fp64():
    # one attempted step from the same state and dt: only rounding differs
    p64 = small(64)
    p32 = small(32)
    B0, xb = configs.init_state(p64)
    o64 = Oracle(p64, B0, xb)
    o32 = Oracle(p32, B0.astype(np.float32), xb.astype(np.float32))
    for n in range(6):
        o64.stage(n)
        o32.stage(n)
    o64.combine()
    o32.combine()
    assert relerr(o32.k(0), o64.k(0)) < 1e-5
    assert relerr(o32.xnew(), o64.xnew()) < 1e-6


# ---- pinning against the reference's own kernels ---------------------------

def _golden_cases():
    import cases
    return [n for n in cases.NAMES if (GOLDEN / f"{n}.npz").exists()]


def _load(name):
    from glemur_gb300._abi import GmParams
    z = np.load(GOLDEN / f"{name}.npz")
    p = GmParams.from_buffer_copy(z["params"].tobytes())
    return p, z


# Run-level tolerances.  With dt0 = 3e-4 the error norm of the first steps is
# rounding noise (|x_new - x*| ~ 1e-15 against a true value ~ 1e-18), so the
# first dt updates differ at ~1e-7 between any two builds that round
# differently (FMA or not); after 10 accepted steps that leaves x within
# ~1e-11, B ~ 1e-10, J ~ 1e-9 (measured by perturbing dt0 by 1e-7).
RUN_TOL = {64: dict(dt=1e-6, x=1e-10, B=1e-9, J=1e-8), 32: dict(dt=1e-2, x=1e-4, B=1e-3, J=1e-2)}


@pytest.mark.parametrize("name", _golden_cases())
def test_oracle_matches_reference_kernels(name):
    p, z = _load(name)
    tol_stage = 1e-12 if p.precision == 64 else 2e-6
    rt = RUN_TOL[p.precision]
    B0 = z["B0"]
    _, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.stage(0)
    assert relerr(o.k(0), z["k0"]) < tol_stage
    assert relerr(inner(o.get()["xb"]), z["x1"]) < tol_stage
    if p.inertia:
        assert relerr(o.u(), z["u1"]) < tol_stage
    o.close()
    if p.inertia and p.precision == 32:
        # From rest the position increments k_x = dt u are O(dt^2), so in FP32
        # |x_new - x*| (formed in float, errMode 0) is rounding of x for the
        # first steps (multiples of ulp(4) = 4.8e-7, or ~1e-15 near x = 0): the
        # error norm, and the dt sequence it drives, are rounding noise that
        # differs between any two builds.  This case pins the stage arithmetic
        # (k_0, x_1, u_1 above) and the step's fields below, not the run.
        o = Oracle(p, B0, xb)
        o.step()
        assert relerr(inner(o.xnew()), z["xnew1"]) < tol_stage
        assert relerr(o.u(new=True), z["unew1"]) < tol_stage
        o.close()
        return
    o = Oracle(p, B0, xb)
    o.step()
    s = o.scalars()
    assert abs(s["maxDelta"] - float(z["maxDelta1"])) <= tol_stage * 10 * max(abs(float(z["maxDelta1"])), 1e-300) + 1e-300
    assert relerr(inner(o.xnew()), z["xnew1"]) < tol_stage
    if p.inertia:
        assert relerr(o.u(new=True), z["unew1"]) < tol_stage
    f = o.get()
    assert relerr(inner(f["B"]), z["B1"]) < tol_stage
    assert relerr(f["J"], z["J1"]) < tol_stage * 100
    assert relerr(inner(f["detJac"]), z["D1"]) < tol_stage
    import cases
    n, lg = o.run(cases.N_ACCEPTED, max_attempts=500, log=True)
    ref_log = z["log"][1:]
    assert len(lg) == len(ref_log)
    assert np.array_equal(lg[:, 2], ref_log[:, 2]), "accept/reject sequence differs"
    assert relerr(lg[:, 1], ref_log[:, 1]) < rt["dt"]
    f = o.get()
    assert relerr(inner(f["xb"]), z["xN"]) < rt["x"]
    assert relerr(inner(f["B"]), z["BN"]) < rt["B"]
    assert relerr(f["J"], z["JN"]) < rt["J"]
    if p.inertia:
        assert relerr(o.u(), z["uN"]) < rt["B"]


# ---- the Classic current (jMethod = "Classic", src/current.cu:10-218) ------

def _classic(p):
    p.set_str("jMethod", "Classic")
    return configs.derive(p)


def test_classic_current_on_identity_grid_is_central_curl_of_b0():
    """On the identity grid jac = I, Delta = 1 and the second derivatives of
    x vanish, so the Classic current is the central-difference curl of B0."""
    p = _classic(configs.braid2(12, 10, 14, precision=64))
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    J = o.get()["J"]
    o.close()
    b = B0.astype(np.float64)

    def d(comp, axis):
        # central difference of B0[comp] along array axis (0 = z, 1 = y, 2 = x) at the inner points
        sl_p = [slice(1, -1)] * 3
        sl_m = [slice(1, -1)] * 3
        sl_p[axis] = slice(2, None)
        sl_m[axis] = slice(0, -2)
        h = (p.dz, p.dy, p.dx)[axis]
        return (b[tuple(sl_p) + (comp,)] - b[tuple(sl_m) + (comp,)]) / (2 * h)

    curl = np.stack([d(2, 1) - d(1, 0), d(0, 0) - d(2, 2), d(1, 2) - d(0, 1)], axis=-1)
    assert relerr(J, curl) < 1e-12


def test_classic_and_stokes_currents_agree_to_truncation_error():
    """Both currents approximate curl B on a distorted grid (here a smooth
    prescribed displacement, every face line-tied); away from the boundary
    layer their difference is second order in the spacing, so it drops about
    fourfold when the grid is refined by two (measured 3.5e-3 -> 7.7e-4)."""
    def current(n, method):
        p = configs.braid2(n, n, 2 * n, precision=64)
        p.xPeri = p.yPeri = 0
        p = _classic(p) if method == "Classic" else configs.derive(p)
        B0, xb = configs.init_state(p)
        X, Y, Z = xb[..., 0].copy(), xb[..., 1].copy(), xb[..., 2].copy()
        x = xb.astype(np.float64).copy()
        x[..., 0] += 0.15 * np.sin(0.7 * Y) * np.cos(0.1 * Z)
        x[..., 1] += 0.15 * np.sin(0.6 * X + 0.05 * Z)
        x[..., 2] += 0.15 * np.cos(0.5 * X) * np.sin(0.4 * Y)
        o = Oracle(p, B0, x)
        o.refresh()
        J = o.get()["J"]
        o.close()
        return J

    errs = []
    for n in (16, 32):
        Js, Jc = current(n, "Stokes"), current(n, "Classic")
        errs.append(float(np.abs(Jc - Js)[1:-1, 1:-1, 1:-1].max() / np.abs(Js).max()))
    assert errs[0] < 1e-2
    assert errs[1] < errs[0] / 3.5, errs


def test_corner_triangle_currents_on_a_folded_grid():
    """On a grid with random displacements of up to 0.45 spacings (every face
    line-tied), the quintilateral and triangular currents leave the diamond
    only where a plane's orientation tests pick a corner triangle: elsewhere
    both equal the Stokes current to rounding.  Where a triangle is taken, the
    quintilateral current is finite, and the triangular one is NaN in all three
    components, as the reference's kernel returns there (current.cu:1420-1424
    add to an area vector that nothing set)."""
    def current(method):
        p = configs.braid2(17, 12, 17, precision=64)
        p.xPeri = p.yPeri = p.zPeri = 0
        p.set_str("jMethod", method)
        p = configs.derive(p)
        B0, xb = configs.init_state(p)
        rng = np.random.default_rng(3)
        x = xb.copy()
        sp = np.array([p.dx, p.dy, p.dz])
        x[1:-1, 1:-1, 1:-1] += rng.uniform(-0.45, 0.45, size=x[1:-1, 1:-1, 1:-1].shape) * sp
        o = Oracle(p, B0, x)
        o.refresh()
        J = o.get()["J"]
        o.close()
        return J

    Js, Jq, Jt = current("Stokes"), current("StokesQuint"), current("StokesTri")
    scale = np.abs(Js).max()
    tri = np.isnan(Jt).any(-1)
    assert np.isnan(Jt[tri]).all() and tri.sum() == 618
    assert np.isfinite(Jq).all()
    moved = np.abs(Jq - Js).max(-1) > 1e-12 * scale
    assert np.array_equal(moved, tri)
    assert np.abs(Jt[~tri] - Js[~tri]).max() < 1e-12 * scale


def test_currents_on_the_folded_grid_match_reference_kernels():
    """Every current on the folded grid of tests/golden/folded_currents.npz
    (made by make_folded.py from the reference's own kernels): the oracle's
    J to 1e-10 for each jMethod, with the triangular current NaN at exactly
    the reference's 618 points.  This pins the corner-triangle branches of
    the quintilateral and triangular currents (current.cu:737-1681), which
    smooth grids never take, without a GPU."""
    import make_folded
    z = np.load(GOLDEN / "folded_currents.npz")
    for m in make_folded.METHODS:
        p, B0, x = make_folded.folded_case(m)
        assert np.array_equal(x, z["x"]) and np.array_equal(B0, z["B0"])
        o = Oracle(p, z["B0"], z["x"])
        o.refresh()
        f = o.get()
        o.close()
        Jr, Jo = z[f"J_{m}"], f["J"]
        nr, no = np.isnan(Jr), np.isnan(Jo)
        assert np.array_equal(nr, no), (m, int(nr.sum()), int(no.sum()))
        assert relerr(np.where(no, 0, Jo), np.where(nr, 0, Jr)) < 1e-10, m
        assert relerr(inner(f["B"]), z["B"]) < 1e-12, m
        if m == "StokesTri":
            assert nr.any(-1).sum() == 618
        else:
            assert not nr.any(), m


def test_sheared_initial_grid_ghost_planes_follow_the_shear():
    """initDist = "initShearX" (src/init.cu:401-407) with the ghost-plane
    correction addDist (src/boundaries.cu:11-35, 63-107).  The shear is smooth
    and linear in z, so the line-tied ghost planes' B and Delta equal central
    differences of the analytically sheared grid: the second ghost plane and
    the in-plane neighbours at the 16-wide block edges are extrapolated by
    addDist.  Without the correction the z-derivative would miss the shear
    (about 0.3 here).  (For "centerShift" the reference's addDist uses the
    constant 0.15366 where initDistortion uses 5.0805, so its block-edge
    neighbours leave the grid; the oracle keeps that as written.)"""
    p = configs.braid6(20, 16, 24, precision=64)
    p.set_str("initDist", "initShearX")
    p.initShearA, p.initShearB, p.initShearK = 0.3, 0.2, 1.0
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    f = o.get()
    o.close()
    A, Bs, K = p.initShearA, p.initShearB, p.initShearK

    def sheared(x, y, z):
        yy = y - A * np.sin(K * 2 * np.pi * (x + p.Ox - p.dx / 2) / (p.Lx + p.dx)) * z
        xx = x - Bs * np.sin(K * 2 * np.pi * (yy + p.Oy - p.dy / 2) / (p.Ly + p.dy)) * z
        return np.stack([xx, yy, z + 0 * x], -1)

    I, Jg = np.meshgrid(np.arange(p.nx), np.arange(p.ny), indexing="xy")
    x, y = p.dx * I + p.Ox, p.dy * Jg + p.Oy
    for k in (0, p.nz + 1):
        zg = p.dz * (k - 1) + p.Oz
        jac = np.stack([(sheared(x + p.dx, y, zg) - sheared(x - p.dx, y, zg)) / (2 * p.dx),
                        (sheared(x, y + p.dy, zg) - sheared(x, y - p.dy, zg)) / (2 * p.dy),
                        (sheared(x, y, zg + p.dz) - sheared(x, y, zg - p.dz)) / (2 * p.dz)], -1)
        det = np.linalg.det(jac)
        b0 = B0[k, 1:-1, 1:-1]
        Bn = np.einsum("...la,...a->...l", jac, b0) / det[..., None]
        Bn[..., 2] = b0[..., 2]                       # B.n = B0.n on the face
        assert relerr(f["B"][k, 1:-1, 1:-1], Bn) < 1e-12
        assert np.abs(f["detJac"][k, 1:-1, 1:-1] - det).max() < 1e-12
        assert np.abs(det - 1).max() > 0.05            # the shear is felt


def test_fp32_storage_error_against_fp64():
    """What FP32 storage costs the relaxation: the six-blob braid at
    32x32x64 run 500 accepted steps with FP32 storage (the cancellation-free
    error norm, errMode = 1) and, to the same physical time, in FP64 (positions
    interpolated linearly in t between the two FP64 steps around it).  The
    positions then differ by about 3.4e-3 of the largest displacement and the
    force-free residual by about 0.2 %.  (The GPU's FP32 path matches the
    oracle's FP32 build per stage to 1e-5, so this is the figure for it.)"""
    inner_ = lambda a: a[1:-1, 1:-1, 1:-1].astype(np.float64)  # noqa: E731
    shape = (32, 32, 64)
    p32 = configs.braid6(*shape, precision=32)
    p32.errMode = 1
    p64 = configs.braid6(*shape, precision=64)
    o32 = Oracle(p32, *configs.init_state(p32))
    B064, xb64 = configs.init_state(p64)
    o64 = Oracle(p64, B064, xb64)
    o32.run(500)
    t32 = o32.scalars()["t"]
    x32 = inner_(o32.get()["xb"])
    prev_t, prev_x = 0.0, inner_(xb64)
    while o64.scalars()["t"] < t32:
        prev_t, prev_x = o64.scalars()["t"], inner_(o64.get()["xb"])
        assert o64.step(1 << 30) >= 0
    t64, x64 = o64.scalars()["t"], inner_(o64.get()["xb"])
    w = (t32 - prev_t) / (t64 - prev_t)
    x64t = (1 - w) * prev_x + w * x64
    disp = np.abs(x64 - inner_(xb64)).max()
    o32.refresh()
    o64.refresh()
    r32, r64 = o32.reduce()["residual"], o64.reduce()["residual"]
    o32.close()
    o64.close()
    assert disp > 0.5                                   # the grid has moved
    assert np.abs(x32 - x64t).max() < 6e-3 * disp       # measured 3.4e-3
    assert abs(r32 - r64) < 5e-3 * r64                  # measured 1.9e-3


# ---- the velocity equation (inertia = T, src/rungeKutta.cu:195-212) -------

def test_inertia_first_stage_from_rest():
    """From u = 0 the first stage moves no point (k_x = dt u = 0, x_1 = x_0
    exactly) and accelerates by k_u = dt Delta (J x B); u_1 = b_10 k_u."""
    import cases
    p = cases.make("inertia_f64")
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    o.refresh()
    f = o.get()
    JxB = np.cross(f["J"], inner(f["B"]))
    o.close()
    o = Oracle(p, B0, xb)
    o.stage(0)
    k = o.k(0)
    assert not k[..., :3].any()
    assert np.array_equal(inner(o.get()["xb"]), inner(xb))
    dt = p.dt0
    expect = JxB * (dt * inner(f["detJac"]))[..., None]
    assert relerr(k[..., 3:], expect) < 1e-13
    assert relerr(o.u(), 0.2 * k[..., 3:]) < 1e-15
    o.close()


def test_inertia_damping_removes_velocity_without_force():
    """With B0 uniform (J = 0) a velocity decays as exp(-nu t) and moves the
    grid by u0 (1 - exp(-nu t)) / nu: one Cash-Karp step of dt = 0.01 gives
    u to 1e-11.  (The step-size control measures the position error only,
    rungeKutta.cu:325-339, so over longer runs dt grows past the velocity
    equation's accuracy: after 5 steps u is off by 22 %, in the reference's
    method as here.)  The displacement is checked to 1e-10: it is a difference
    of positions of size 4."""
    p = configs.braid2(8, 8, 10, precision=64)
    p.set_str("bInit", "homZ")
    p.inertia = 1
    p.nu = 2.0
    p.xPeri = p.yPeri = 1
    p.zPeri = 1
    p.dt0 = 0.01
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    o = Oracle(p, B0, xb)
    u0 = np.zeros((p.nz, p.ny, p.nx, 3))
    u0[..., 0] = 0.01
    o.set_u(u0)
    o.run(1)
    t = o.scalars()["t"]
    assert t == 0.01
    u = o.u()
    assert np.allclose(u[..., 0], 0.01 * np.exp(-2.0 * t), rtol=1e-11, atol=0)
    assert np.abs(u[..., 1:]).max() < 1e-16
    # the displacement (1e-4) is a difference of positions up to 4: rounding 1e-15 / 1e-4
    dx = inner(o.get()["xb"])[..., 0] - inner(xb)[..., 0]
    assert np.allclose(dx, 0.01 * (1 - np.exp(-2.0 * t)) / 2.0, rtol=1e-10, atol=0)
    o.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_diagnostics_match_reference_kernels(precision):
    """The oracle's per-point grid fields (dirCellVol, gridConvexity,
    gridWedgeMin), eps* and the analytic-error norms against
    tests/golden/diagnostics_f{64,32}.npz, made by make_diagnostics.py from
    the reference's own kernels on a folded grid, a relaxed braid and (FP64)
    the relaxed analytic field."""
    from glemur_gb300._abi import GmParams
    z = np.load(GOLDEN / f"diagnostics_f{precision}.npz")
    tol = 1e-12 if precision == 64 else 1e-5
    kinds = ("folded", "braid", "analytic") if precision == 64 else ("folded", "braid")
    for kind in kinds:
        p = GmParams.from_buffer_copy(z[f"{kind}_params"].tobytes())
        o = Oracle(p, z[f"{kind}_B0"], z[f"{kind}_x"])
        o.refresh()
        g = o.grid_fields()
        for key in ("cellVol", "wedgeMin"):
            assert relerr(g[key], z[f"{kind}_{key}"]) < tol, (kind, key)
        assert np.array_equal(g["convexity"], z[f"{kind}_convexity"]), kind
        eps, e1, e2 = z[f"{kind}_scalars"]
        assert abs(o.eps_star() - eps) <= tol * eps, (kind, o.eps_star(), eps)
        r = o.reduce()
        assert abs(r["errB_1ez"] - e1) <= tol * e1, (kind, r["errB_1ez"], e1)
        if kind == "analytic":
            assert abs(r["errXb_XbAn"] - e2) <= tol * e2, (kind, r["errXb_XbAn"], e2)
        if kind == "folded":
            assert (g["convexity"] < 0).any()
        o.close()


def test_grid_fields_known_answers():
    """On the identity grid every cell volume is dx dy dz, every cell is
    convex and every corner wedge is dx dy dz in gridWedgeMin's sign
    convention; under a uniform shear x += s y the volumes stay dx dy dz."""
    p = configs.braid2(10, 9, 12, precision=64)
    p.xPeri = p.yPeri = p.zPeri = 0
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    v = p.dx * p.dy * p.dz
    o = Oracle(p, B0, xb)
    g = o.grid_fields()
    assert np.allclose(g["cellVol"], v, rtol=1e-12) and np.all(g["convexity"] == 1)
    assert np.allclose(g["wedgeMin"], v, rtol=1e-12)
    o.close()
    xs = xb.copy()
    xs[..., 0] += 0.3 * xs[..., 1]
    o = Oracle(p, B0, xs)
    assert np.allclose(o.grid_fields()["cellVol"], v, rtol=1e-10)
    o.close()


def _sym_field(a, sym):
    """Ghosted array [nz + 2][ny + 2][nx + 2][3] moved by the mirror / swap
    symmetry `sym` (the bits of gm_nn_input, no translation): cell (I, J)
    reads (U, V) with 4: U <-> V, 2: V -> ny + 1 - V, 1: U -> nx + 1 - U, and
    the x, y components follow as polar vectors."""
    nzg, nyg, nxg = a.shape[:3]
    I = np.arange(nxg)[None, :].repeat(nyg, 0)
    J = np.arange(nyg)[:, None].repeat(nxg, 1)
    U, V = (J, I) if sym & 4 else (I, J)
    if sym & 2:
        V = nyg - 1 - V
    if sym & 1:
        U = nxg - 1 - U
    out = a[:, V, U].copy()
    if sym & 1:
        out[..., 0] *= -1
    if sym & 2:
        out[..., 1] *= -1
    if sym & 4:
        out[..., [0, 1]] = out[..., [1, 0]]
    return out


@pytest.mark.parametrize("sym", [1, 2, 4, 7])
def test_mirror_and_swap_are_symmetries_of_the_relaxation(sym):
    """The warm-start network's training pairs are augmented with the mirrors
    and the x <-> y swap of the periodic cross-section (gm_nn_input,
    gm_nn_mse), the field and the displacement moved as polar vectors.  That
    is exact for the relaxation: the oracle run from the moved field gives the
    moved displacement (FP64, a random braid, 6 accepted steps) with the same
    steps, up to rounding (the x mirror evaluates the same sums in another
    order: 3e-12 in t and in the displacement)."""
    from glemur_gb300 import configs
    p = configs.random_braid(4242, shape=(12, 12, 16), precision=64)
    B0, xb = Oracle.init_state(p)
    o = Oracle(p, B0, xb)
    o.run(6)
    s = o.scalars()
    d = o.get()["xb"] - xb
    o.close()
    o2 = Oracle(p, _sym_field(B0, sym), xb)
    o2.run(6)
    s2 = o2.scalars()
    d2 = o2.get()["xb"] - xb
    o2.close()
    assert s2["nAttempted"] == s["nAttempted"] and s2["t"] == pytest.approx(s["t"], rel=1e-10)
    want = _sym_field(d, sym)[1:-1, 1:-1, 1:-1]
    assert np.abs(d2[1:-1, 1:-1, 1:-1] - want).max() <= 1e-10 * np.abs(want).max()
