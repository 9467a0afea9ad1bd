"""ORACLE (test infrastructure): run parameters without the library.

A ctypes mirror of gm_params (include/glemur.h, itself the reference's
struct Parameters, src/global.h:44-108), the namelist defaults of
src/readNamelist.f90:91-150, the derived spacing of :185-186, and the
parameters of the benchmark workloads.  Used where the checker must not load
the product library: the reference arm and the CPU-baseline leg of bench.py.
tests/test_oracle_params.py checks that every field matches the library's own
builder (glemur_gb300.configs) byte for byte.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

STR = 30


class Params(C.Structure):
    """gm_params, field by field (REAL widened to double)."""
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("Ox", C.c_double), ("Oy", C.c_double), ("Oz", C.c_double),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("dx1", C.c_double), ("dy1", C.c_double), ("dz1", C.c_double),
        ("bInit", C.c_char * STR), ("uInit", C.c_char * STR),
        ("ampl", C.c_double), ("phi1", C.c_double), ("phi2", C.c_double),
        ("L1", C.c_double), ("L2", C.c_double), ("ar", C.c_double), ("az", C.c_double),
        ("nBlobs", C.c_int32),
        ("width", C.c_double), ("minor", C.c_double), ("major", C.c_double),
        ("stretch", C.c_double), ("bGround", C.c_double),
        ("blobXc", C.c_double * 10), ("blobYc", C.c_double * 10), ("blobZc", C.c_double * 10),
        ("blobZl", C.c_double * 10), ("blobTwist", C.c_double * 10), ("blobScale", C.c_double * 10),
        ("initDist", C.c_char * STR), ("initDistCode", C.c_int32),
        ("initShearA", C.c_double), ("initShearB", C.c_double), ("initShearK", C.c_double),
        ("pert", C.c_double), ("twist", C.c_double),
        ("fRestart", C.c_int32), ("nCycle", C.c_int32),
        ("dt0", C.c_double), ("dtMin", C.c_double), ("maxError", C.c_double),
        ("zUpdate", C.c_int32), ("inertia", C.c_int32), ("pressure", C.c_int32),
        ("nu", C.c_double), ("beta", C.c_double),
        ("jxbAver", C.c_int32), ("jxbAverWeight", C.c_double),
        ("xPeri", C.c_int32), ("yPeri", C.c_int32), ("zPeri", C.c_int32),
        ("epsilonProf", C.c_int32),
        ("jMethod", C.c_char * STR), ("pMethod", C.c_char * STR),
        ("nTs", C.c_int32), ("dtDump", C.c_double), ("dtSave", C.c_double),
        ("dumpJ", C.c_int32), ("dumpDetJac", C.c_int32), ("dumpCellVol", C.c_int32),
        ("dumpConvexity", C.c_int32), ("dumpWedgeMin", C.c_int32),
        ("redB2", C.c_int32), ("redB2f", C.c_int32), ("redBMax", C.c_int32), ("redJMax", C.c_int32),
        ("redJxB_B2Max", C.c_int32), ("redEpsilonStar", C.c_int32), ("redErrB_1ez", C.c_int32),
        ("redErrXb_XbAn", C.c_int32), ("redConvex", C.c_int32), ("redWedgeMin", C.c_int32),
        ("redU2", C.c_int32), ("redUMax", C.c_int32),
        ("precision", C.c_int32), ("errMode", C.c_int32),
        ("p0Amp", C.c_double), ("p0Width", C.c_double),
        ("stageKernel", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]

    def set_str(self, name: str, value: str) -> None:
        """Blank padded to 29 characters plus NUL, as copyString leaves a
        Fortran string (src/readNamelist.f90:267-283)."""
        setattr(self, name, value.encode()[: STR - 1].ljust(STR - 1, b" "))

    def rnd(self, v: float) -> float:
        """A real read into REAL."""
        return float(np.float32(v)) if self.precision == 32 else float(v)


def _flit(v: float) -> float:
    # a Fortran default initialiser such as `dt0 = 3e-4` is a default-kind
    # (single precision) literal converted to the variable's kind
    return float(np.float32(v))


def defaults(precision: int) -> Params:
    """The namelist variables' initial values, src/readNamelist.f90:91-150,
    plus this library's extensions (errMode: the cancellation-free error
    norm |sum (c - c*) k| of FP32 runs; p0Amp, p0Width: the pressure
    profile, off)."""
    p = Params()
    p.precision = precision
    p.nx = p.ny = p.nz = 16
    p.Lx, p.Ly, p.Lz = 8.0, 8.0, 20.0
    p.Ox = p.Oy = p.Oz = 0.0
    p.set_str("bInit", "Pontin09")
    p.set_str("uInit", "nil")
    p.ampl = 1.0
    p.phi1, p.phi2 = 2.0, -2.0
    p.L1, p.L2 = -4.0, 4.0
    p.ar, p.az = _flit(math.sqrt(2.0)), 2.0
    p.width = _flit(0.6)
    p.minor, p.major = 1.0, 2.5
    p.stretch = 1.0
    p.set_str("initDist", "none")
    p.initShearK = 1.0
    p.pert = p.twist = 1.0
    p.nCycle = 10
    p.dt0, p.dtMin, p.maxError = _flit(3e-4), _flit(1e-9), _flit(5e-5)
    p.zUpdate = 1
    p.nu = p.beta = 1.0
    p.epsilonProf = 1
    p.set_str("jMethod", "Stokes")
    p.set_str("pMethod", "Classic")
    p.nTs = 10
    p.dtDump, p.dtSave = 10.0, 1.0
    p.errMode = 1 if precision == 32 else 0
    p.p0Width = 2.0
    return derive(p)


def derive(p: Params) -> Params:
    """dx = L/(n-1) and its inverse in REAL (src/readNamelist.f90:185-186)."""
    if p.precision == 32:
        f = np.float32
        d = [f(p.Lx) / f(p.nx - 1), f(p.Ly) / f(p.ny - 1), f(p.Lz) / f(p.nz - 1)]
        p.dx, p.dy, p.dz = (float(v) for v in d)
        p.dx1, p.dy1, p.dz1 = (float(f(1.0) / v) for v in d)
    else:
        p.dx, p.dy, p.dz = p.Lx / (p.nx - 1), p.Ly / (p.ny - 1), p.Lz / (p.nz - 1)
        p.dx1, p.dy1, p.dz1 = 1.0 / p.dx, 1.0 / p.dy, 1.0 / p.dz
    return p


def braid6(nx=128, ny=128, nz=256, precision=32, k=1.0, nCycle=100000) -> Params:
    """The six-blob braid over [-4,4]x[-4,4]x[-24,24], periodic in x and y,
    line-tied in z: blobs at z = -20,-12,-4,4,12,20, x = +1,-1,..., k = +1,-1,
    ..., a = sqrt(2), l = 2, entering the "blobs" field (src/init.cu:109-124)
    as blobTwist = k a / 2, blobScale = a, blobZl = l; maxError 1e-5,
    dt0 3e-4, dtMin 1e-8."""
    p = defaults(precision)
    p.nx, p.ny, p.nz = nx, ny, nz
    p.Lx, p.Ly, p.Lz = (p.rnd(v) for v in (8.0, 8.0, 48.0))
    p.Ox, p.Oy, p.Oz = (p.rnd(v) for v in (-4.0, -4.0, -24.0))
    p.xPeri, p.yPeri, p.zPeri = 1, 1, 0
    p.ampl = 1.0
    p.dt0, p.dtMin, p.maxError = p.rnd(3e-4), p.rnd(1e-8), p.rnd(1e-5)
    p.nTs = 10
    a = math.sqrt(2.0)
    p.set_str("bInit", "blobs")
    p.nBlobs = 6
    for b, z in enumerate((-20.0, -12.0, -4.0, 4.0, 12.0, 20.0)):
        s = 1.0 if b % 2 == 0 else -1.0
        p.blobXc[b] = p.rnd(s)
        p.blobYc[b] = 0.0
        p.blobZc[b] = p.rnd(z)
        p.blobTwist[b] = p.rnd(s * k * a / 2.0)
        p.blobScale[b] = p.rnd(a)
        p.blobZl[b] = p.rnd(2.0)
    p.nCycle = nCycle
    return derive(p)


def braid6_large(nx=256, ny=256, nz=512, precision=32) -> Params:
    """The six-blob braid with k = +-1.2 and the pressure term with
    p0 = 0.1 (1 + 0.5 exp(-r^2/4))."""
    p = braid6(nx, ny, nz, precision, k=1.2)
    p.pressure = 1
    p.beta = p.rnd(0.1)
    p.p0Amp = p.rnd(0.5)
    p.p0Width = p.rnd(2.0)
    return derive(p)
