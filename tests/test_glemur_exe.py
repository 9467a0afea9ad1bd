"""The `glemur` run-directory executable (src/main.cu's process contract):
params.in in, cuda.info, data/B0.vtk, data/time_series.dat, data/dump<n>.vtk
and data/save.vtk out, restart from data/save.vtk.  Its fields must equal
the library's own run of the same parameters bit for bit, its time-series
rows the step-by-step controller values, and a restarted run must continue
exactly where the saved one stopped."""
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

from glemur_gb300 import Relaxation, configs
from vtk_legacy import LegacyVtk

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
EXE = ROOT / "glemur_gb300" / "_lib" / "glemur"


def params_text(nCycle, restart=False, nTs=5, dtDump=0.05, dtSave=0.1, n=(16, 16, 32), pressure=False,
                inertia=False):
    a = math.sqrt(2.0)
    return f"""&comp
 nx = {n[0]}; ny = {n[1]}; nz = {n[2]}
/
&start
 Lx = 8; Ly = 8; Lz = 48
 Ox = -4; Oy = -4; Oz = -24
 bInit = "blobs"
 ampl = 1.
 nBlobs = 2
 blobXc = 1., -1.
 blobYc = 0., 0.
 blobZc = -4., 4.
 blobTwist = {a / 2!r}, {-a / 2!r}
 blobScale = {a!r}, {a!r}
 blobZl = 2., 2.
 fRestart = {'T' if restart else 'F'}
/
&run
 nCycle = {nCycle}
 dt0 = 3e-4
 dtMin = 1e-8
 maxError = 1e-5
 xPeri = T; yPeri = T; zPeri = F
 pressure = {'T' if pressure else 'F'}
 inertia = {'T' if inertia else 'F'}
 nu = 1.
 beta = 0.05
 jMethod = "Stokes"
/
&io
 nTs = {nTs}
 dtDump = {dtDump}
 dtSave = {dtSave}
 dumpJ = T; dumpDetJac = T; dumpCellVol = T; dumpConvexity = T; dumpWedgeMin = T
 redJxB_B2Max = T; redEpsilonStar = T; redB2 = T; redB2f = T; redConvex = T; redWedgeMin = T; redJMax = T
 redU2 = T; redUMax = T
/
"""


def make_run(d: Path, nCycle, **kw):
    (d / "data").mkdir(parents=True, exist_ok=True)
    (d / "params.in").write_text(params_text(nCycle, **kw))


def run_exe(d: Path, precision=64):
    r = subprocess.run([str(EXE), "-p", str(precision)], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.rstrip().endswith("glemur terminated successfully"), r.stdout[-2000:]
    return r.stdout


def read_params(d: Path, precision):
    from glemur_gb300 import _abi
    import ctypes as C
    lib = _abi.load()
    p = _abi.GmParams()
    _abi.check(lib.gm_params_read(C.byref(p), str(d / "params.in").encode(), precision), "params")
    return p


def read_ts(d: Path):
    """As readTs (python/glemur/ts.py:30-44): loadtxt, keys from the header."""
    path = d / "data" / "time_series.dat"
    data = np.loadtxt(path, ndmin=2)
    keys = open(path).readline().split()[1:]
    return {k: data[:, i] for i, k in enumerate(keys)}


@pytest.mark.parametrize("precision", [64, 32])
def test_run_directory_matches_library(tmp_path, precision):
    d = tmp_path / "run"
    nCycle = 30
    make_run(d, nCycle)
    out = run_exe(d, precision)
    assert "jMethod = Stokes" in out
    assert (d / "cuda.info").read_text().startswith("number of CUDA devices:")
    p = read_params(d, precision)
    B0, xb = configs.init_state(p)
    b0 = LegacyVtk(d / "data" / "B0.vtk")
    np.testing.assert_array_equal(b0.point_data["bfield"], B0.reshape(-1, 3))

    # the library, step by step: accepted steps' t, dt used, maxDelta, reductions
    g = Relaxation(p)
    g.upload(xb, B0)
    rows = []
    dt_used = g.state()["dt"]
    while g.state()["timeIndex"] < nCycle:
        r = g.step()
        if r["accepted"]:
            it = r["timeIndex"] - 1
            if it % p.nTs == 0:
                rows.append((it, r["t"], dt_used, r["maxDelta"], g.refresh()))
        dt_used = r["dt"]
    s = g.state()
    red = g.refresh()
    f = g.download()
    g.close()

    ts = read_ts(d)
    assert list(ts) == ["it", "t", "dt", "maxDelta", "JMax", "JxB_B2Max", "epsilonStar", "B2", "B2f", "convex",
                        "wedgeMin"]
    assert list(ts["it"]) == [r[0] for r in rows]
    for i, (it, t, dtu, md, rd) in enumerate(rows):
        for key, v in (("t", t), ("dt", dtu), ("maxDelta", md), ("JMax", rd["JMax"]),
                       ("JxB_B2Max", rd["JxB_B2Max"]), ("B2", rd["B2"]), ("epsilonStar", rd["epsilonStar"]),
                       ("convex", rd["convex"]), ("wedgeMin", rd["wedgeMin"])):
            assert ts[key][i] == pytest.approx(v, rel=6e-6, abs=1e-300), (key, it)
    B2res = float(np.float32(8 * 8 * 48)) if precision == 32 else 8.0 * 8 * 48
    # B2f = B2 - B2res, each printed with 6 significant digits
    assert np.allclose(ts["B2f"], ts["B2"] - B2res, rtol=0, atol=1e-5 * ts["B2"].max())

    # data/save.vtk = the state after the last step, bit for bit
    sv = LegacyVtk(d / "data" / "save.vtk")
    assert sv.field["t"][0] == p.rnd(s["t"]) and sv.field["dt"][0] == p.rnd(s["dt"])
    np.testing.assert_array_equal(sv.points, f["xb"].reshape(-1, 3))
    np.testing.assert_array_equal(sv.point_data["bfield"], f["B"].reshape(-1, 3))
    np.testing.assert_array_equal(sv.point_data["jfield"].reshape(f["B"].shape)[1:-1, 1:-1, 1:-1], f["J"])
    np.testing.assert_array_equal(sv.point_data["detJac"], f["detJac"].reshape(-1))
    wm = sv.point_data["wedgeMin"].reshape(f["detJac"].shape)[1:-1, 1:-1, 1:-1]
    assert wm.min() == pytest.approx(red["wedgeMin"], rel=1e-6)
    cx = sv.point_data["convexity"].reshape(f["detJac"].shape)[1:-1, 1:-1, 1:-1]
    assert set(np.unique(cx)) <= {-1.0, 1.0} and cx.min() == red["convex"]
    cv = sv.point_data["cellVol"].reshape(f["detJac"].shape)[1:-1, 1:-1, 1:-1]
    assert abs(cv.mean() - p.dx * p.dy * p.dz) < 0.5 * p.dx * p.dy * p.dz

    # dump<n>.vtk: n = ceil((t - dt) / dtDump) with the file's own t and adapted dt
    R = np.float32 if precision == 32 else np.float64
    dumps = sorted(d.glob("data/dump*.vtk"))
    assert len(dumps) >= 2
    for fp in dumps:
        v = LegacyVtk(fp)
        t, dt = R(v.field["t"][0]), R(v.field["dt"][0])
        assert int(fp.stem[4:]) == math.ceil(R(t - dt) / R(p.dtDump))


def test_restart_continues_exactly(tmp_path):
    a, c = tmp_path / "a", tmp_path / "c"
    make_run(a, 15)
    run_exe(a)
    rows_a = read_ts(a)["it"]
    (a / "params.in").write_text(params_text(15, restart=True))
    out = run_exe(a)
    assert "initial B: blobs" in out
    make_run(c, 30)
    run_exe(c)
    sa, sc = LegacyVtk(a / "data" / "save.vtk"), LegacyVtk(c / "data" / "save.vtk")
    assert sa.field["t"][0] == sc.field["t"][0] and sa.field["dt"][0] == sc.field["dt"][0]
    np.testing.assert_array_equal(sa.points, sc.points)
    np.testing.assert_array_equal(sa.point_data["bfield"], sc.point_data["bfield"])
    np.testing.assert_array_equal(sa.point_data["jfield"], sc.point_data["jfield"])
    # the restarted run appends rows (its loop index starts again at 0)
    ts = read_ts(a)
    assert len(ts["it"]) == 2 * len(rows_a)
    assert (a / "data" / "time_series.dat").read_text().count("#") == 1


def test_invalid_method(tmp_path):
    d = tmp_path / "bad"
    make_run(d, 5)
    txt = (d / "params.in").read_text()
    (d / "params.in").write_text(txt.replace('jMethod = "Stokes"', 'jMethod = "Nonsense"'))
    r = subprocess.run([str(EXE)], cwd=d, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "invalid method for computing J" in r.stdout


def test_inertia_run_directory_and_restart(tmp_path):
    """inertia = T: the velocity is written as VECTORS ufield (zero ghosts)
    after bfield in dumps and save.vtk, the time series gains U2 and UMax,
    and a restart from save.vtk continues exactly, velocity included."""
    a, c = tmp_path / "a", tmp_path / "c"
    make_run(a, 10, inertia=True)
    out = run_exe(a)
    assert "initial U: nil" in out
    ts = read_ts(a)
    assert list(ts)[-2:] == ["U2", "UMax"] and ts["UMax"][-1] > 0
    sv = LegacyVtk(a / "data" / "save.vtk")
    assert list(sv.point_data)[:3] == ["bfield", "ufield", "jfield"]
    p = read_params(a, 64)
    uf = sv.point_data["ufield"].reshape(p.nz + 2, p.ny + 2, p.nx + 2, 3)
    assert np.abs(uf[1:-1, 1:-1, 1:-1]).max() > 0 and not uf[0].any() and not uf[:, :, 0].any()
    # the same run through the library: the velocity of the last state
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    g.run(10)
    np.testing.assert_array_equal(uf[1:-1, 1:-1, 1:-1], g.u())
    g.close()
    (a / "params.in").write_text(params_text(10, restart=True, inertia=True))
    run_exe(a)
    make_run(c, 20, inertia=True)
    run_exe(c)
    sa, sc = LegacyVtk(a / "data" / "save.vtk"), LegacyVtk(c / "data" / "save.vtk")
    assert sa.field["t"][0] == sc.field["t"][0]
    np.testing.assert_array_equal(sa.points, sc.points)
    np.testing.assert_array_equal(sa.point_data["ufield"], sc.point_data["ufield"])
    np.testing.assert_array_equal(sa.point_data["bfield"], sc.point_data["bfield"])
