"""ctypes view of the C-ABI declared in include/glemur.h."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libglemur.so"

GM_OK = 0
ERRORS = {
    -1: "GM_EPARAM", -2: "GM_EALLOC", -3: "GM_ECUDA", -4: "GM_ENAN", -5: "GM_EDETJAC",
    -6: "GM_EDTMIN", -7: "GM_ETIMEOUT", -8: "GM_ENOTREADY", -9: "GM_EIO",
}
GM_ST_NAN, GM_ST_DETJAC, GM_ST_DTMIN, GM_ST_DONE = 1, 2, 4, 8
GM_ST_TIMEOUT, GM_ST_ALIGN, GM_ST_EVENT = 16, 32, 64
GM_EV_TS, GM_EV_DUMP, GM_EV_SAVE, GM_EV_LAST = 1, 2, 4, 8
GM_EPARAM, GM_EALLOC, GM_ECUDA, GM_ENAN, GM_EDETJAC, GM_EDTMIN, GM_ETIMEOUT, GM_ENOTREADY, GM_EIO = range(-1, -10, -1)
STR = 30


class GmParams(C.Structure):
    """Mirror of gm_params (include/glemur.h), itself a mirror of the
    reference's struct Parameters (src/global.h:44-108)."""
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

    def real_dtype(self):
        return np.float32 if self.precision == 32 else np.float64

    def set_str(self, name: str, value: str) -> None:
        """Blank-pad to 29 characters plus NUL as the Fortran reader leaves strings."""
        v = value.encode()[: STR - 1].ljust(STR - 1, b" ")
        setattr(self, name, v)

    def get_str(self, name: str) -> str:
        return bytes(getattr(self, name)).split(b"\0")[0].decode().rstrip()

    def rnd(self, v: float) -> float:
        """Round a real to the run precision."""
        return float(np.float32(v)) if self.precision == 32 else float(v)

    def copy(self) -> "GmParams":
        c = GmParams()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(GmParams))
        return c

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)


class GmStepResult(C.Structure):
    _fields_ = [("maxDelta", C.c_double), ("t", C.c_double), ("dt", C.c_double),
                ("accepted", C.c_int32), ("timeIndex", C.c_int32), ("status", C.c_uint32), ("pad", C.c_int32)]


class GmState(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("maxDelta", C.c_double),
                ("timeIndex", C.c_int32), ("nAttempted", C.c_int32), ("nRejected", C.c_int32),
                ("status", C.c_uint32), ("dtUsed", C.c_double), ("event", C.c_int32), ("pad", C.c_int32)]


class GmReduction(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("B2", "BMax", "JMax", "JxB_B2Max", "residual", "residualPw", "minDetJac",
                                           "wedgeMin", "convex", "errB_1ez", "errXb_XbAn", "epsilonStar", "U2",
                                           "UMax")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class GmBatchCase(C.Structure):
    _fields_ = [("seconds", C.c_double), ("residual", C.c_double), ("t", C.c_double), ("dt", C.c_double),
                ("attempted", C.c_int32), ("accepted", C.c_int32), ("status", C.c_uint32), ("converged", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


# name -> (restype, argtypes) of every entry point declared in include/glemur.h
P = C.POINTER
VP = C.c_void_p
SIGNATURES = {
    "gm_params_default": (C.c_int, [P(GmParams), C.c_int]),
    "gm_params_derive": (C.c_int, [P(GmParams)]),
    "gm_params_read": (C.c_int, [P(GmParams), C.c_char_p, C.c_int]),
    "gm_init_state": (C.c_int, [P(GmParams), VP, VP]),
    "gm_create": (C.c_int, [P(GmParams), P(VP)]),
    "gm_destroy": (C.c_int, [VP]),
    "gm_set_stream": (C.c_int, [VP, VP]),
    "gm_upload": (C.c_int, [VP, VP, VP, C.c_double, C.c_double]),
    "gm_stage": (C.c_int, [VP, C.c_int]),
    "gm_control": (C.c_int, [VP]),
    "gm_step": (C.c_int, [VP, P(GmStepResult)]),
    "gm_steps_async": (C.c_int, [VP, C.c_int]),
    "gm_run": (C.c_int, [VP, C.c_int, P(GmState)]),
    "gm_run_events": (C.c_int, [VP, C.c_int, P(GmState)]),
    "gm_grid_fields": (C.c_int, [VP, VP, VP, VP]),
    "gm_get_state": (C.c_int, [VP, P(GmState)]),
    "gm_set_dt": (C.c_int, [VP, C.c_double, C.c_double, C.c_int]),
    "gm_refresh": (C.c_int, [VP, P(GmReduction)]),
    "gm_download": (C.c_int, [VP, VP, VP, VP, VP]),
    "gm_autotune": (C.c_int, [VP, C.c_int, P(C.c_int), P(C.c_double)]),
    "gm_set_tile_z": (C.c_int, [VP, C.c_int]),
    "gm_debug_stall": (C.c_int, [VP, C.c_int]),
    "gm_download_k": (C.c_int, [VP, C.c_int, VP]),
    "gm_download_x": (C.c_int, [VP, C.c_int, VP]),
    "gm_upload_u": (C.c_int, [VP, VP]),
    "gm_download_u": (C.c_int, [VP, C.c_int, VP]),
    "gm_reduce_noalloc": (C.c_int, [P(GmParams), VP, VP, VP, VP, VP]),
    "gm_batch_create": (C.c_int, [P(GmParams), C.c_int, P(VP)]),
    "gm_batch_autotune": (C.c_int, [VP, C.c_int, P(C.c_int), P(C.c_double)]),
    "gm_batch_destroy": (C.c_int, [VP]),
    "gm_batch_upload": (C.c_int, [VP, C.c_int, VP, VP, C.c_double, C.c_double]),
    "gm_batch_steps_async": (C.c_int, [VP, C.c_int]),
    "gm_batch_get_state": (C.c_int, [VP, C.c_int, P(GmState)]),
    "gm_batch_refresh": (C.c_int, [VP, C.c_int, P(GmReduction)]),
    "gm_batch_download": (C.c_int, [VP, C.c_int, VP, VP, VP, VP]),
    "gm_batch_stop": (C.c_int, [VP, C.c_int]),
    "gm_batch_run": (C.c_int, [VP, C.c_int, C.c_double, C.c_int, C.c_int, P(GmBatchCase)]),
    "gm_batch_launch_count": (C.c_int64, [VP]),
    "gm_nn_tc_gemm_check": (C.c_int, [VP, VP, VP, C.c_int, C.c_int, VP]),
    "gm_nn_conv": (C.c_int, [VP, C.c_int, C.c_int, VP, C.c_int, C.c_int, VP, P(C.c_float), VP, C.c_int, C.c_int,
                             VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                             VP, VP]),
    "gm_nn_conv_wgrad": (C.c_int, [VP, C.c_int, C.c_int, VP, C.c_int, C.c_int, VP, C.c_int, C.c_int, P(C.c_float),
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, VP, VP]),
    "gm_nn_bias_grad": (C.c_int, [VP, C.c_int, C.c_int, C.c_longlong, P(C.c_float), VP]),
    "gm_nn_pool": (C.c_int, [VP, C.c_int, VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, VP]),
    "gm_nn_upsample": (C.c_int, [VP, C.c_int, VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, VP]),
    "gm_nn_relu_bwd": (C.c_int, [VP, C.c_int, VP, C.c_int, C.c_int, C.c_longlong, VP]),
    "gm_nn_mse": (C.c_int, [VP, C.c_int, P(C.c_float), VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                            P(C.c_float), C.c_int, C.c_int, C.c_int, VP]),
    "gm_nn_adam": (C.c_int, [P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float), P(C.c_float),
                             P(C.c_float), P(C.c_float), C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                             C.c_float, VP, C.c_int, C.c_int, VP, C.c_int, C.c_int, P(C.c_float), VP]),
    "gm_nn_input": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, VP, C.c_int, C.c_int, C.c_int, C.c_int, VP]),
    "gm_nn_disp_accumulate": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                         C.c_int, VP, VP]),
    "gm_nn_warm_grid": (C.c_int, [VP, P(GmParams), C.c_int, VP, VP, VP, VP]),
    "gm_nn_zero": (C.c_int, [VP, C.c_size_t, VP]),
    "gm_nn_debug_stall": (C.c_int, [C.c_int]),
    "gm_device_count": (C.c_int, [P(C.c_int)]),
    "gm_set_device": (C.c_int, [C.c_int]),
    "gm_io_write_cuda_info": (C.c_int, [C.c_char_p, C.c_int, C.c_long]),
    "gm_io_write_b0": (C.c_int, [P(GmParams), C.c_char_p, VP]),
    "gm_io_write_dump": (C.c_int, [P(GmParams), C.c_char_p, C.c_double, C.c_double, VP, VP, VP, VP, VP, VP, VP,
                                   VP]),
    "gm_io_read_state": (C.c_int, [P(GmParams), C.c_char_p, C.c_char_p, VP, VP, P(C.c_double), P(C.c_double),
                                   VP]),
    "gm_io_ts_line": (C.c_int, [P(GmParams), P(GmReduction), C.c_double, C.c_double, C.c_double, C.c_int,
                                C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_int]),
    "gm_launch_count": (C.c_int64, [VP]),
    "gm_last_error": (C.c_char_p, []),
    "gm_version": (C.c_char_p, []),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libglemur.so (built in-tree by glemur_gb300._build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:  # reported by missing_symbols(); calls fail loudly
            continue
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def missing_symbols(lib: C.CDLL | None = None) -> list[str]:
    """Entry points of include/glemur.h that the loaded library lacks."""
    lib = lib or load()
    return [n for n in SIGNATURES if getattr(lib, n, None) is None]


class GlemurError(RuntimeError):
    pass


def check(rc: int, what: str = "") -> None:
    if rc != GM_OK:
        msg = load().gm_last_error().decode(errors="replace")
        raise GlemurError(f"{what}: {ERRORS.get(rc, rc)}: {msg}")


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)
