"""ORACLE (test infrastructure): Python handles on the CPU restatement
(oracle/glemur_oracle.c) and on the reference-kernel launcher
(oracle/ref/ref_launcher.cpp).  Imported only by the tests, the smoke check
and the CPU-baseline leg of bench.py.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"

_libs: dict[int, C.CDLL] = {}


def _lib(bits: int) -> C.CDLL:
    if bits in _libs:
        return _libs[bits]
    p = BUILD / f"liboracle{bits}.so"
    if not p.exists():
        raise RuntimeError(f"{p} missing: run the build (oracle/build.py)")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [vp, vp, vp, C.c_double, C.c_double]
    lib.orc_destroy.argtypes = [vp]
    lib.orc_init_state.argtypes = [vp, vp, vp]
    lib.orc_init_state.restype = C.c_int
    lib.orc_get.argtypes = [vp, vp, vp, vp, vp]
    lib.orc_get_k.argtypes = [vp, C.c_int, vp]
    lib.orc_get_u.argtypes = [vp, C.c_int, vp]
    lib.orc_set_u.argtypes = [vp, vp]
    lib.orc_get_xnew.argtypes = [vp, vp]
    lib.orc_get_scalars.argtypes = [vp, vp]
    lib.orc_set_time.argtypes = [vp, C.c_double, C.c_double, C.c_int]
    lib.orc_refresh_fields.argtypes = [vp]
    lib.orc_stage.argtypes = [vp, C.c_int]
    lib.orc_combine.argtypes = [vp]
    lib.orc_step.argtypes = [vp, C.c_int]
    lib.orc_step.restype = C.c_int
    lib.orc_run.argtypes = [vp, C.c_int, C.c_int, vp]
    lib.orc_run.restype = C.c_int
    lib.orc_reduce.argtypes = [vp, vp]
    lib.orc_grid_fields.argtypes = [vp, vp, vp, vp]
    lib.orc_eps_star.argtypes = [vp]
    lib.orc_eps_star.restype = C.c_double
    lib.orc_real_bits.restype = C.c_int
    assert lib.orc_real_bits() == bits
    _libs[bits] = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def set_threads(n: int | None) -> None:
    """OpenMP threads of the oracle (must be set before its first parallel region)."""
    if n:
        os.environ["OMP_NUM_THREADS"] = str(n)


class Oracle:
    """CPU restatement of the relaxation, one run."""

    def __init__(self, params, B0: np.ndarray, xb: np.ndarray, t: float = 0.0, dt: float | None = None):
        self.p = params
        self.bits = params.precision
        self.dtype = np.float32 if self.bits == 32 else np.float64
        self.lib = _lib(self.bits)
        B0 = np.ascontiguousarray(B0, dtype=self.dtype)
        xb = np.ascontiguousarray(xb, dtype=self.dtype)
        self.h = self.lib.orc_create(C.byref(params), _p(B0), _p(xb), t, params.dt0 if dt is None else dt)
        if not self.h:
            raise MemoryError("orc_create failed")
        nx, ny, nz = params.nx, params.ny, params.nz
        self.G = (nz + 2, ny + 2, nx + 2)
        self.I = (nz, ny, nx)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    __del__ = close

    @staticmethod
    def init_state(params):
        dt = np.float32 if params.precision == 32 else np.float64
        G = (params.nz + 2, params.ny + 2, params.nx + 2, 3)
        B0 = np.zeros(G, dt)
        xb = np.zeros(G, dt)
        rc = _lib(params.precision).orc_init_state(C.byref(params), _p(B0), _p(xb))
        if rc != 0:
            raise ValueError(f"orc_init_state: {rc}")
        return B0, xb

    def stage(self, n):
        self.lib.orc_stage(self.h, n)

    def combine(self):
        self.lib.orc_combine(self.h)
        return self.scalars()["maxDelta"]

    def refresh(self):
        self.lib.orc_refresh_fields(self.h)

    def step(self, nCycle=1 << 30):
        return self.lib.orc_step(self.h, nCycle)

    def run(self, nCycle, max_attempts=1 << 30, log=False):
        lg = np.zeros((max_attempts if log else 1, 3)) if log else None
        n = self.lib.orc_run(self.h, nCycle, max_attempts, _p(lg))
        return (n, lg[:n]) if log else n

    def set_time(self, t, dt, timeIndex=0):
        self.lib.orc_set_time(self.h, t, dt, timeIndex)

    def scalars(self):
        out = np.zeros(5)
        self.lib.orc_get_scalars(self.h, _p(out))
        return dict(t=out[0], dt=out[1], maxDelta=out[2], timeIndex=int(out[3]), nAttempted=int(out[4]))

    def get(self):
        xb = np.zeros(self.G + (3,), self.dtype)
        B = np.zeros(self.G + (3,), self.dtype)
        J = np.zeros(self.I + (3,), self.dtype)
        dj = np.zeros(self.G, self.dtype)
        self.lib.orc_get(self.h, _p(xb), _p(B), _p(J), _p(dj))
        return dict(xb=xb, B=B, J=J, detJac=dj)

    def k(self, m):
        k = np.zeros(self.I + (6 if self.p.inertia else 3,), self.dtype)
        self.lib.orc_get_k(self.h, m, _p(k))
        return k

    def xnew(self):
        x = np.zeros(self.G + (3,), self.dtype)
        self.lib.orc_get_xnew(self.h, _p(x))
        return x

    def u(self, new=False):
        """Velocity (inertia) at the inner points: the current one, or u_new of the last combine."""
        u = np.zeros(self.I + (3,), self.dtype)
        self.lib.orc_get_u(self.h, 1 if new else 0, _p(u))
        return u

    def set_u(self, u):
        u = np.ascontiguousarray(u, dtype=self.dtype)
        self.lib.orc_set_u(self.h, _p(u))

    def grid_fields(self):
        """Per inner point: signed cell volume, convexity flag, minimum wedge
        product (inner layout (nz, ny, nx))."""
        out = [np.zeros(self.I, self.dtype) for _ in range(3)]
        self.lib.orc_grid_fields(self.h, *(_p(a) for a in out))
        return dict(cellVol=out[0], convexity=out[1], wedgeMin=out[2])

    def eps_star(self):
        return self.lib.orc_eps_star(self.h)

    def reduce(self):
        from glemur_gb300._abi import GmReduction
        r = GmReduction()
        self.lib.orc_reduce(self.h, C.byref(r))
        return r.as_dict()


class RefLauncher:
    """The reference's own CUDA kernels (cubin built from the reference
    sources) driven with the launch sequence of src/main.cu.  GPU only."""

    def __init__(self, params, B0, xb, t=0.0, dt=None, variant=""):
        so = REF / "libref_launcher.so"
        cub = REF / f"glemur_ref{params.precision}{variant}.cubin"
        if not so.exists() or not cub.exists():
            raise RuntimeError(f"reference harness missing ({so}, {cub})")
        lib = C.CDLL(str(so))
        vp = C.c_void_p
        lib.ref_open.argtypes = [C.c_char_p, vp, vp, vp, C.c_double, C.c_double]
        lib.ref_stage.argtypes = [C.c_int]
        lib.ref_combine.argtypes = [vp]
        lib.ref_step.argtypes = [C.c_int, vp]
        lib.ref_run.argtypes = [C.c_int, C.c_int, vp, vp]
        lib.ref_time_steps.argtypes = [C.c_int, vp, vp]
        lib.ref_get.argtypes = [vp, vp, vp, vp]
        lib.ref_get_k.argtypes = [C.c_int, vp]
        lib.ref_get_u.argtypes = [C.c_int, vp]
        lib.ref_get_xnew.argtypes = [vp]
        lib.ref_scalars.argtypes = [vp]
        lib.ref_grid_fields.argtypes = [vp, vp, vp]
        lib.ref_eps_star.argtypes = [vp]
        lib.ref_errors.argtypes = [vp, vp]
        lib.ref_last_error.restype = C.c_char_p
        self.lib = lib
        self.p = params
        self.dtype = np.float32 if params.precision == 32 else np.float64
        B0 = np.ascontiguousarray(B0, dtype=self.dtype)
        xb = np.ascontiguousarray(xb, dtype=self.dtype)
        self._chk(lib.ref_open(str(cub).encode(), C.byref(params), _p(B0), _p(xb), t,
                               params.dt0 if dt is None else dt), "ref_open")
        nx, ny, nz = params.nx, params.ny, params.nz
        self.G = (nz + 2, ny + 2, nx + 2)
        self.I = (nz, ny, nx)

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {rc}: {self.lib.ref_last_error().decode()}")

    def close(self):
        self.lib.ref_close()

    def stage(self, n):
        self._chk(self.lib.ref_stage(n), "ref_stage")

    def combine(self):
        md = C.c_double()
        self._chk(self.lib.ref_combine(C.byref(md)), "ref_combine")
        return md.value

    def refresh(self):
        self._chk(self.lib.ref_refresh(), "ref_refresh")

    def step(self, nCycle=1 << 30):
        acc = C.c_int()
        self._chk(self.lib.ref_step(nCycle, C.byref(acc)), "ref_step")
        return acc.value

    def run(self, nCycle, max_attempts=1 << 30):
        lg = np.zeros((max_attempts, 3))
        n = C.c_int()
        self._chk(self.lib.ref_run(nCycle, max_attempts, _p(lg), C.byref(n)), "ref_run")
        return n.value, lg[: n.value]

    def time_steps(self, n):
        s = C.c_double()
        done = C.c_int()
        self._chk(self.lib.ref_time_steps(n, C.byref(s), C.byref(done)), "ref_time_steps")
        return s.value, done.value

    def scalars(self):
        out = np.zeros(5)
        self.lib.ref_scalars(_p(out))
        return dict(t=out[0], dt=out[1], maxDelta=out[2], timeIndex=int(out[3]), nAttempted=int(out[4]))

    def get(self):
        xb = np.zeros(self.G + (3,), self.dtype)
        B = np.zeros(self.G + (3,), self.dtype)
        J = np.zeros(self.I + (3,), self.dtype)
        dj = np.zeros(self.G, self.dtype)
        self._chk(self.lib.ref_get(_p(xb), _p(B), _p(J), _p(dj)), "ref_get")
        return dict(xb=xb, B=B, J=J, detJac=dj)

    def k(self, m):
        k = np.zeros(self.I + (6 if self.p.inertia else 3,), self.dtype)
        self._chk(self.lib.ref_get_k(m, _p(k)), "ref_get_k")
        return k

    def u(self, new=False):
        u = np.zeros(self.I + (3,), self.dtype)
        self._chk(self.lib.ref_get_u(1 if new else 0, _p(u)), "ref_get_u")
        return u

    def xnew(self):
        x = np.zeros(self.G + (3,), self.dtype)
        self._chk(self.lib.ref_get_xnew(_p(x)), "ref_get_xnew")
        return x

    def grid_fields(self):
        """dirCellVol, gridConvexity, gridWedgeMin on the current grid
        (inner layout (nz, ny, nx))."""
        out = [np.zeros(self.I, self.dtype) for _ in range(3)]
        self._chk(self.lib.ref_grid_fields(*(_p(a) for a in out)), "ref_grid_fields")
        return dict(cellVol=out[0], convexity=out[1], wedgeMin=out[2])

    def eps_star(self):
        v = C.c_double()
        self._chk(self.lib.ref_eps_star(C.byref(v)), "ref_eps_star")
        return v.value

    def errors(self):
        """(errB_1ez, errXb_XbAn) from the reference's kernels."""
        a, b = C.c_double(), C.c_double()
        self._chk(self.lib.ref_errors(C.byref(a), C.byref(b)), "ref_errors")
        return a.value, b.value
