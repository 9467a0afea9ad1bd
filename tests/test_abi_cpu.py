"""CPU checks of the C-ABI library: it loads, exports every entry point the
header declares, and its host-side logic (namelist defaults and reader,
initial state) follows src/readNamelist.f90 and src/init.cu."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from glemur_gb300 import _abi, configs
from oracle.pyoracle import Oracle

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "glemur.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+\*?(gm_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_entry_point():
    lib = _abi.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if getattr(lib, n, None) is None]
    assert not missing, missing
    assert set(names) == set(_abi.SIGNATURES), set(names) ^ set(_abi.SIGNATURES)


def test_defaults_use_single_precision_literals():
    p = configs.defaults(64)
    assert p.dt0 == float(np.float32(3e-4)) and p.dt0 != 3e-4
    assert p.maxError == float(np.float32(5e-5))
    assert p.ar == float(np.float32(1.414213562373095))
    assert p.get_str("jMethod") == "Stokes" and bytes(p.jMethod)[:7] == b"Stokes "
    assert p.nx == 16 and p.Lz == 20.0 and p.epsilonProf == 1 and p.zUpdate == 1
    assert p.dx == 8.0 / 15 and p.dx1 == 1.0 / (8.0 / 15)
    q = configs.defaults(32)
    assert q.dx == float(np.float32(8.0) / np.float32(15))


def test_namelist_reader(tmp_path):
    text = """
&comp
    nx = 20;  ny = 18;  nz = 40   ! inner mesh points
/
&start
    Lx = 8;     Ly = 8;     Lz = 48
    Ox = -4;    Oy = -4;    Oz = -24
    bInit = "blobs"      ! comment with a / slash
    nBlobs = 2
    blobXc = 1.0, -1.0
    blobYc = 2*0.0
    blobZc(1) = -4.d0, blobZc(2) = 4
    blobZl = 2, 2
    blobTwist = 0.7071067811865476, -0.7071067811865476
    blobScale = 1.4142135623730951 1.4142135623730951
    fRestart = f
/
&run
    nCycle = 2000
    dt0 = 3e-4
    dtMin = 1e-8
    maxError = 1e-5
    xPeri = True;  yPeri = .true.; zPeri = False
    jMethod = 'Stokes'
/
&io
    nTs = 5
    dtDump = 1; dtSave = .2
    redB2 = T
/
"""
    f = tmp_path / "params.in"
    f.write_text(text)
    p = _abi.GmParams()
    _abi.check(_abi.load().gm_params_read(p, str(f).encode(), 64), "read")
    assert (p.nx, p.ny, p.nz) == (20, 18, 40)
    assert p.Lz == 48.0 and p.Oz == -24.0
    assert p.get_str("bInit") == "blobs"
    assert list(p.blobXc[:2]) == [1.0, -1.0] and list(p.blobYc[:2]) == [0.0, 0.0]
    assert list(p.blobZc[:2]) == [-4.0, 4.0]
    assert p.blobTwist[1] == -0.7071067811865476
    assert p.xPeri == 1 and p.yPeri == 1 and p.zPeri == 0 and p.fRestart == 0
    assert p.dt0 == 3e-4 and p.maxError == 1e-5 and p.nCycle == 2000
    assert p.nTs == 5 and p.dtSave == 0.2 and p.redB2 == 1
    assert p.dx == 8.0 / 19
    p32 = _abi.GmParams()
    _abi.check(_abi.load().gm_params_read(p32, str(f).encode(), 32), "read32")
    assert p32.dt0 == float(np.float32(3e-4))


@pytest.mark.parametrize("dist,code", [("none", 0), ("initShearX", 0), ("centerShift", 1)])
def test_namelist_reader_initial_distortion(tmp_path, dist, code):
    """initDist and the initShear parameters (namelist start) and the code the
    Fortran reader derives from initDist (src/readNamelist.f90:256-262)."""
    f = tmp_path / "params.in"
    f.write_text(f'&comp nx = 8; ny = 8; nz = 8 /\n&start initDist = "{dist}"; initShearA = 0.25; '
                 f'initShearB = 0.5; initShearK = 2 /\n&run /\n&io /\n')
    p = _abi.GmParams()
    _abi.check(_abi.load().gm_params_read(p, str(f).encode(), 64), "read")
    assert p.get_str("initDist") == dist and p.initDistCode == code
    assert (p.initShearA, p.initShearB, p.initShearK) == (0.25, 0.5, 2.0)
    # the parameter check accepts initially distorted grids (the ghost planes
    # carry addDist); without a GPU gm_create stops later, at the device
    h = C.c_void_p()
    rc = _abi.load().gm_create(p, C.byref(h))
    assert rc != -1 and b"initShear" not in _abi.load().gm_last_error()
    if rc == 0:
        _abi.load().gm_destroy(h)


@pytest.mark.parametrize("line,ok", [
    ("blobYc = 10*0.5", True),                    # a repeat count that fills the array
    ("blobYc = 2147483647*0.0", False),           # refused before it is expanded
    ("blobYc = 1,2,3,4,5,6,7,8,9,10,11, 2000000000*0", False),
    ("blobYc = 0*1.0", False),                    # repeat counts are >= 1
    ("blobXc(11) = 1", False), ("blobXc(0) = 1", False), ("blobXc(99999999999) = 1", False),
    ("blobXc( 2 ) = 1", True),
    ("nBlobs = 2147483647", True), ("nBlobs = 2147483648", False), ("nBlobs = 99999999999999999999", False),
    ("Lx = 1e400", False), ("Lx = 8.d0", True), ("Lx = 1e-400", True),
])
def test_namelist_reader_values_at_the_limits(tmp_path, line, ok):
    """Repeat counts, indices and numbers at and past their limits: an
    out-of-range integer or index, an overflowing real and a repeat count that
    runs past the array are errors (as in the Fortran reader), returned at
    once instead of being truncated or expanded."""
    f = tmp_path / "params.in"
    f.write_text(f"&comp nx = 8; ny = 8; nz = 8 /\n&start nBlobs = 2\n    {line}\n/\n&run /\n&io /\n")
    p = _abi.GmParams()
    rc = _abi.load().gm_params_read(p, str(f).encode(), 64)
    assert (rc == 0) == ok, (line, rc, _abi.load().gm_last_error())
    if line.startswith("blobYc = 10*"):
        assert list(p.blobYc[:10]) == [0.5] * 10
    if line.startswith("nBlobs = 2147483647"):
        assert p.nBlobs == 2147483647


def test_namelist_reader_rejects_unknown_names(tmp_path):
    f = tmp_path / "params.in"
    f.write_text("&comp nx = 4 /\n&start bogus = 1 /\n&run /\n&io /\n")
    p = _abi.GmParams()
    rc = _abi.load().gm_params_read(p, str(f).encode(), 64)
    assert rc == -9
    assert b"bogus" in _abi.load().gm_last_error()


def test_namelist_reader_missing_group(tmp_path):
    f = tmp_path / "params.in"
    f.write_text("&comp nx = 4 /\n&start /\n")
    p = _abi.GmParams()
    assert _abi.load().gm_params_read(p, str(f).encode(), 64) == -9


@pytest.mark.parametrize("prec", [32, 64])
def test_init_state_matches_oracle(prec):
    p = configs.braid6(20, 16, 24, precision=prec)
    B0, xb = configs.init_state(p)
    B0o, xbo = Oracle.init_state(p)
    assert np.array_equal(B0, B0o) and np.array_equal(xb, xbo)
    # periodic ghost copies of B0 (setPeriHost order z, y, x)
    assert np.array_equal(B0[:, :, 0], B0[:, :, -2]) and np.array_equal(B0[:, :, -1], B0[:, :, 1])
    assert np.array_equal(B0[:, 0, :], B0[:, -2, :]) and np.array_equal(B0[:, -1, :], B0[:, 1, :])


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("dist", ["initShearX", "centerShift"])
def test_initial_distortion_matches_oracle_and_formula(prec, dist):
    """initDistortion (src/init.cu:386-420) on the grid, ghosts included: the
    library and the oracle agree bit for bit, and the displacement follows
    the formula (restated in numpy, double arithmetic as the reference's
    double PI makes it; FP32 stores round once).  B0 is unchanged."""
    p = configs.braid6(20, 16, 24, precision=prec)
    p.set_str("initDist", dist)
    p.initShearA, p.initShearB, p.initShearK = 0.3, 0.2, 1.0
    B0, xb = configs.init_state(p)
    B0o, xbo = Oracle.init_state(p)
    assert np.array_equal(B0, B0o) and np.array_equal(xb, xbo)
    p0 = configs.braid6(20, 16, 24, precision=prec)
    B00, xb0 = configs.init_state(p0)
    assert np.array_equal(B0, B00)
    dt = np.float32 if prec == 32 else np.float64
    f = lambda v: dt(v)  # noqa: E731  run-precision parameters
    X, Y, Z = (xb0[..., c] for c in range(3))    # run precision, as REAL x[i], y[j], z[k]
    if dist == "initShearX":
        # sums in the run precision, then double from K * 2 * PI on
        two_k_pi = np.float64(f(p.initShearK) * dt(2)) * np.pi
        ey = (Y - np.float64(f(p.initShearA)) * np.sin(two_k_pi * (X + f(p.Ox) - f(p.dx) / dt(2)) /
                                                       np.float64(f(p.Lx) + f(p.dx))) * Z).astype(dt)
        ex = (X - np.float64(f(p.initShearB)) * np.sin(two_k_pi * (ey + f(p.Oy) - f(p.dy) / dt(2)) /
                                                       np.float64(f(p.Ly) + f(p.dy))) * Z).astype(dt)
        ulp = np.spacing(np.abs(xb).max().astype(dt))
        assert np.abs(xb[..., 1] - ey).max() <= ulp and np.abs(xb[..., 0] - ex).max() <= ulp
        assert np.array_equal(xb[..., 2], xb0[..., 2])
    else:
        X, Y, Z = (a.astype(np.float64) for a in (X, Y, Z))
        ey = Y + f(p.initShearA) * np.exp(-f(p.initShearK) * X * X) * (1 - Y * Y) * (np.exp(-Z + 1) - 5.0804508111226507)
        tol = 1e-4 if prec == 32 else 1e-12
        assert np.abs(xb[..., 1] - ey).max() / np.abs(ey).max() < tol
        assert np.array_equal(xb[..., 0], xb0[..., 0]) and np.array_equal(xb[..., 2], xb0[..., 2])
    assert np.abs(xb - xb0).max() > 0.01


def test_create_rejects_unsupported_options():
    lib = _abi.load()
    h = C.c_void_p()
    p = configs.braid2(8, 8, 8)
    p.set_str("jMethod", "Stokes2nd")
    assert lib.gm_create(p, C.byref(h)) == -1


def test_configs_blob_mapping():
    p = configs.braid6()
    assert p.nBlobs == 6 and (p.nx, p.ny, p.nz) == (128, 128, 256)
    assert [p.blobZc[b] for b in range(6)] == [-20.0, -12.0, -4.0, 4.0, 12.0, 20.0]
    assert p.blobXc[0] == 1.0 and p.blobXc[1] == -1.0
    assert p.blobTwist[0] == float(np.float32(np.sqrt(2) / 2)) and p.blobTwist[1] < 0
    q = configs.braid2()
    assert q.precision == 64 and q.nCycle == 2000 and q.maxError == 1e-5


def test_executable_without_a_gpu_stops_before_any_output(tmp_path):
    """No CPU fallback: on a machine without a CUDA device the glemur
    executable stops with the reference's message (src/main.cu:49-56) and a
    non-zero status, before reading params.in or writing anything."""
    import subprocess
    n = C.c_int(0)
    if _abi.load().gm_device_count(C.byref(n)) == 0 and n.value > 0:
        pytest.skip("a CUDA device is present")
    exe = Path(__file__).resolve().parents[1] / "glemur_gb300" / "_lib" / "glemur"
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert "could not locate CUDA devices" in r.stdout or "no CUDA compatible devices" in r.stdout
    assert list(tmp_path.iterdir()) == []
