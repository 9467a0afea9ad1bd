"""Run-directory files (src/io.cu) written by the library's host code: byte
layout of data/B0.vtk and data/dump<n>.vtk, the restart reader, and the
time-series lines.  CPU only (no device call)."""
import ctypes as C

import numpy as np
import pytest

from glemur_gb300 import _abi, configs
from vtk_legacy import LegacyVtk


@pytest.fixture(scope="module")
def lib():
    return _abi.load()


def small(precision):
    p = configs.braid_box(6, 5, 7, precision)
    p.dumpJ = p.dumpDetJac = p.dumpCellVol = p.dumpConvexity = p.dumpWedgeMin = 1
    return configs.derive(p)


def fields(p, seed=0):
    rng = np.random.default_rng(seed)
    dt = p.real_dtype()
    G = (p.nz + 2, p.ny + 2, p.nx + 2)
    I = (p.nz, p.ny, p.nx)
    f = dict(xb=rng.normal(size=G + (3,)), B=rng.normal(size=G + (3,)), J=rng.normal(size=I + (3,)),
             D=rng.normal(size=G), cv=rng.normal(size=I), cx=np.sign(rng.normal(size=I)), wm=rng.normal(size=I))
    return {k: np.ascontiguousarray(v.astype(dt)) for k, v in f.items()}


@pytest.mark.parametrize("precision", [64, 32])
def test_b0_file_layout(lib, tmp_path, precision):
    p = small(precision)
    B0 = fields(p)["B"]
    path = tmp_path / "B0.vtk"
    _abi.check(lib.gm_io_write_b0(C.byref(p), str(path).encode(), _abi.ptr(B0)), "write B0")
    v = LegacyVtk(path)
    rs = "float" if precision == 32 else "double"
    R = np.float32 if precision == 32 else np.float64
    # header lines of writeB0 (io.cu:183-191), REAL arithmetic for origin and spacing
    org = [float(R(p.Ox) - R(p.dx)), float(R(p.Oy) - R(p.dy)), float(R(p.Oz) - R(p.dz))]
    spc = [float(R(p.Lx) / R(p.nx - 1)), float(R(p.Ly) / R(p.ny - 1)), float(R(p.Lz) / R(p.nz - 1))]
    assert v.lines == ["# vtk DataFile Version 2.0", "GLEMuR B0 dump", "BINARY", "DATASET STRUCTURED_POINTS",
                       "DIMENSIONS %9i %9i %9i" % (p.nx + 2, p.ny + 2, p.nz + 2),
                       "ORIGIN %8.12f %8.12f %8.12f" % tuple(org),
                       "SPACING %8.12f %8.12f %8.12f" % tuple(spc),
                       "POINT_DATA %9i" % ((p.nx + 2) * (p.ny + 2) * (p.nz + 2)),
                       "VECTORS bfield %s" % rs]
    np.testing.assert_array_equal(v.point_data["bfield"], B0.reshape(-1, 3))
    assert v.pos == len(v.raw)


@pytest.mark.parametrize("precision", [64, 32])
def test_dump_file_layout_and_restart(lib, tmp_path, precision):
    p = small(precision)
    f = fields(p, 1)
    t, dt = p.rnd(1.2345678), p.rnd(3.25e-3)
    path = tmp_path / "save.vtk"
    _abi.check(lib.gm_io_write_dump(C.byref(p), str(path).encode(), t, dt, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                                    _abi.ptr(f["J"]), _abi.ptr(f["D"]), _abi.ptr(f["cv"]), _abi.ptr(f["cx"]),
                                    _abi.ptr(f["wm"]), None), "write dump")
    v = LegacyVtk(path)
    rs = "float" if precision == 32 else "double"
    G = (p.nx + 2) * (p.ny + 2) * (p.nz + 2)
    assert v.lines[:6] == ["# vtk DataFile Version 2.0", "GLEMuR data dump", "BINARY", "DATASET STRUCTURED_GRID",
                           "DIMENSIONS %9i %9i %9i" % (p.nx + 2, p.ny + 2, p.nz + 2), "FIELD parameters 9"]
    names = [ln.split()[0] for ln in v.lines[6:15]]
    assert names == ["t", "dt", "nx_ny_nz", "Lx_Ly_Lz", "Ox_Oy_Oz", "dx_dy_dz", "ampl", "phi1_phi2", "maxError"]
    assert v.lines[8] == "nx_ny_nz 1 3 int" and v.lines[6] == f"t 1 1 {rs}"
    fd = v.field
    assert fd["t"][0] == t and fd["dt"][0] == dt
    assert list(fd["nx_ny_nz"]) == [p.nx, p.ny, p.nz]
    assert list(fd["Lx_Ly_Lz"]) == [p.Lx, p.Ly, p.Lz] and list(fd["dx_dy_dz"]) == [p.dx, p.dy, p.dz]
    assert fd["maxError"][0] == p.maxError
    assert v.lines[15] == "POINTS %9i %s" % (G, rs)
    np.testing.assert_array_equal(v.points, f["xb"].reshape(-1, 3))
    np.testing.assert_array_equal(v.point_data["bfield"], f["B"].reshape(-1, 3))
    # J, cellVol, convexity, wedgeMin: zero on the ghost layer, inner values inside
    jf = v.point_data["jfield"].reshape(p.nz + 2, p.ny + 2, p.nx + 2, 3)
    np.testing.assert_array_equal(jf[1:-1, 1:-1, 1:-1], f["J"])
    gh = np.ones((p.nz + 2, p.ny + 2, p.nx + 2), bool)
    gh[1:-1, 1:-1, 1:-1] = False
    assert not jf[gh].any()
    np.testing.assert_array_equal(v.point_data["detJac"], f["D"].reshape(-1))
    for key, name in (("cv", "cellVol"), ("cx", "convexity"), ("wm", "wedgeMin")):
        a = v.point_data[name].reshape(p.nz + 2, p.ny + 2, p.nx + 2)
        np.testing.assert_array_equal(a[1:-1, 1:-1, 1:-1], f[key])
        assert not a[gh].any()
    assert list(v.point_data) == ["bfield", "jfield", "detJac", "cellVol", "convexity", "wedgeMin"]
    assert v.pos == len(v.raw)

    # restart: t, dt and xb from the save file, B0 from the B0 file
    b0 = tmp_path / "B0.vtk"
    _abi.check(lib.gm_io_write_b0(C.byref(p), str(b0).encode(), _abi.ptr(f["B"])), "write B0")
    xb = np.zeros_like(f["xb"])
    B0 = np.zeros_like(f["B"])
    tt, dd = C.c_double(), C.c_double()
    _abi.check(lib.gm_io_read_state(C.byref(p), str(path).encode(), str(b0).encode(), _abi.ptr(xb), _abi.ptr(B0),
                                    C.byref(tt), C.byref(dd), None), "read state")
    assert tt.value == t and dd.value == dt
    np.testing.assert_array_equal(xb, f["xb"])
    np.testing.assert_array_equal(B0, f["B"])


def test_dump_without_optional_fields(lib, tmp_path):
    p = configs.braid_box(4, 4, 5, 64)
    p = configs.derive(p)
    f = fields(p, 2)
    path = tmp_path / "dump3.vtk"
    _abi.check(lib.gm_io_write_dump(C.byref(p), str(path).encode(), 1.0, 0.1, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                                    None, None, None, None, None, None), "write dump")
    v = LegacyVtk(path)
    assert list(v.point_data) == ["bfield"]
    # a selected field passed as NULL is refused
    p.dumpJ = 1
    rc = lib.gm_io_write_dump(C.byref(p), str(path).encode(), 1.0, 0.1, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                              None, None, None, None, None, None)
    assert rc == _abi.GM_EPARAM


def test_restart_reader_errors(lib, tmp_path):
    p = small(64)
    xb = np.zeros(((p.nz + 2) * (p.ny + 2) * (p.nx + 2) * 3,))
    tt, dd = C.c_double(), C.c_double()
    rc = lib.gm_io_read_state(C.byref(p), str(tmp_path / "missing.vtk").encode(), b"x", _abi.ptr(xb), _abi.ptr(xb),
                              C.byref(tt), C.byref(dd), None)
    assert rc == _abi.GM_EIO
    (tmp_path / "short.vtk").write_bytes(b"# vtk DataFile Version 2.0\nGLEMuR data dump\n")
    rc = lib.gm_io_read_state(C.byref(p), str(tmp_path / "short.vtk").encode(), b"x", _abi.ptr(xb), _abi.ptr(xb),
                              C.byref(tt), C.byref(dd), None)
    assert rc == _abi.GM_EIO


def test_restart_reader_refuses_truncated_files(lib, tmp_path):
    """A save or B0 file cut inside the data the restart reads (the header,
    the positions, the field) is an error, not a partial state."""
    p = small(64)
    f = fields(p, 1)
    save, b0 = tmp_path / "save.vtk", tmp_path / "B0.vtk"
    _abi.check(lib.gm_io_write_dump(C.byref(p), str(save).encode(), 1.0, 0.1, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                                    _abi.ptr(f["J"]), _abi.ptr(f["D"]), _abi.ptr(f["cv"]), _abi.ptr(f["cx"]),
                                    _abi.ptr(f["wm"]), None), "write dump")
    _abi.check(lib.gm_io_write_b0(C.byref(p), str(b0).encode(), _abi.ptr(f["B"])), "write B0")
    good_s, good_b = save.read_bytes(), b0.read_bytes()
    xb = np.zeros_like(f["xb"])
    B0 = np.zeros_like(f["B"])
    tt, dd = C.c_double(), C.c_double()

    def read():
        return lib.gm_io_read_state(C.byref(p), str(save).encode(), str(b0).encode(), _abi.ptr(xb), _abi.ptr(B0),
                                    C.byref(tt), C.byref(dd), None)

    assert read() == 0
    np.testing.assert_array_equal(xb, f["xb"])
    npos = good_s.index(b"POINTS")
    for cut in (0, 200, npos + 40, npos + 40 + f["xb"].nbytes // 2):
        save.write_bytes(good_s[:cut])
        assert read() == _abi.GM_EIO, cut
    save.write_bytes(good_s)
    for cut in (0, 100, len(good_b) // 2, len(good_b) - 1):
        b0.write_bytes(good_b[:cut])
        assert read() == _abi.GM_EIO, cut


@pytest.mark.parametrize("precision", [64, 32])
def test_time_series_lines(lib, precision):
    p = small(precision)
    p.redJxB_B2Max = p.redEpsilonStar = p.redB2 = p.redB2f = p.redConvex = p.redWedgeMin = 1
    buf = C.create_string_buffer(2048)
    n = lib.gm_io_ts_line(C.byref(p), None, 0.0, 0.0, 0.0, 0, 0.0, 1, 1, buf, 2048)
    hdr = buf.value.decode()
    assert n == len(hdr)
    expect = "#%7s" % "it" + "".join("%13s" % k for k in ["t", "dt", "maxDelta", "JxB_B2Max", "epsilonStar", "B2",
                                                           "B2f", "convex", "wedgeMin"]) + "\n"
    assert hdr == expect
    lib.gm_io_ts_line(C.byref(p), None, 0.0, 0.0, 0.0, 0, 0.0, 1, 0, buf, 2048)
    assert buf.value.decode() == expect.replace("maxDelta", "maxError")
    r = _abi.GmReduction()
    r.JxB_B2Max, r.epsilonStar, r.B2, r.convex, r.wedgeMin = 0.5, 1.25e-3, 3088.5191, 1.0, 2.5e-4
    B2res = 3072.0
    lib.gm_io_ts_line(C.byref(p), C.byref(r), B2res, 13.8125, 0.0140625, 40, 7.5e-6, 0, 1, buf, 2048)
    R = np.float32 if precision == 32 else np.float64
    vals = [13.8125, 0.0140625, 7.5e-6, 0.5, 1.25e-3, 3088.5191, R(3088.5191) - R(B2res), 1.0, 2.5e-4]
    row = "%8i " % 40 + "".join("%12.5e " % float(R(v)) for v in vals) + "\n"
    assert buf.value.decode() == row
    # the row reads back as readTs (ts.py:30-44) reads the file: loadtxt under the header keys
    data = np.loadtxt([hdr, row])
    keys = hdr.split()[1:]
    assert dict(zip(keys, data))["epsilonStar"] == pytest.approx(1.25e-3, rel=1e-4)
    assert lib.gm_io_ts_line(C.byref(p), C.byref(r), 0.0, 0.0, 0.0, 0, 0.0, 0, 1, buf, 8) == _abi.GM_EPARAM


@pytest.mark.parametrize("precision", [64, 32])
def test_inertia_dump_and_restart(lib, tmp_path, precision):
    """With inertia the dump carries VECTORS ufield after bfield, zero on the
    ghost layer (io.cu:269-291), and the restart reads it back into the
    inner-point velocity (io.cu:466-481)."""
    p = small(precision)
    p.inertia = 1
    f = fields(p, 3)
    u = np.ascontiguousarray(np.random.default_rng(4).normal(size=(p.nz, p.ny, p.nx, 3)).astype(p.real_dtype()))
    path = tmp_path / "save.vtk"
    rc = lib.gm_io_write_dump(C.byref(p), str(path).encode(), 0.5, 0.01, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                              _abi.ptr(f["J"]), _abi.ptr(f["D"]), _abi.ptr(f["cv"]), _abi.ptr(f["cx"]),
                              _abi.ptr(f["wm"]), None)
    assert rc == _abi.GM_EPARAM      # the velocity is required with inertia
    _abi.check(lib.gm_io_write_dump(C.byref(p), str(path).encode(), 0.5, 0.01, _abi.ptr(f["xb"]), _abi.ptr(f["B"]),
                                    _abi.ptr(f["J"]), _abi.ptr(f["D"]), _abi.ptr(f["cv"]), _abi.ptr(f["cx"]),
                                    _abi.ptr(f["wm"]), _abi.ptr(u)), "write dump")
    v = LegacyVtk(path)
    assert list(v.point_data)[:3] == ["bfield", "ufield", "jfield"]
    uf = v.point_data["ufield"].reshape(p.nz + 2, p.ny + 2, p.nx + 2, 3)
    np.testing.assert_array_equal(uf[1:-1, 1:-1, 1:-1], u)
    gh = np.ones((p.nz + 2, p.ny + 2, p.nx + 2), bool)
    gh[1:-1, 1:-1, 1:-1] = False
    assert not uf[gh].any()
    b0 = tmp_path / "B0.vtk"
    _abi.check(lib.gm_io_write_b0(C.byref(p), str(b0).encode(), _abi.ptr(f["B"])), "write B0")
    xb = np.zeros_like(f["xb"])
    B0 = np.zeros_like(f["B"])
    ur = np.zeros_like(u)
    tt, dd = C.c_double(), C.c_double()
    _abi.check(lib.gm_io_read_state(C.byref(p), str(path).encode(), str(b0).encode(), _abi.ptr(xb), _abi.ptr(B0),
                                    C.byref(tt), C.byref(dd), _abi.ptr(ur)), "read state")
    np.testing.assert_array_equal(ur, u)
    np.testing.assert_array_equal(xb, f["xb"])


def test_time_series_velocity_columns(lib):
    p = small(64)
    p.inertia = 1
    p.redU2 = p.redUMax = 1
    buf = C.create_string_buffer(2048)
    lib.gm_io_ts_line(C.byref(p), None, 0.0, 0.0, 0.0, 0, 0.0, 1, 1, buf, 2048)
    assert buf.value.decode().split()[-2:] == ["U2", "UMax"]
    r = _abi.GmReduction()
    r.U2, r.UMax = 0.125, 2.5e-3
    lib.gm_io_ts_line(C.byref(p), C.byref(r), 0.0, 1.0, 0.1, 3, 1e-6, 0, 1, buf, 2048)
    assert buf.value.decode().split()[-2:] == ["1.25000e-01", "2.50000e-03"]
