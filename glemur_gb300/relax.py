"""Python handle over the C-ABI (include/glemur.h).

``Relaxation`` owns one gm_handle: device buffers, a stream, the device-side
controller and the step graph.  Arrays cross in the reference layout
(ghosted AoS, numpy shape (nz+2, ny+2, nx+2, 3)).  There is no CPU fallback:
every call goes to libglemur.so and raises if it is missing or fails.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import GmParams, GmReduction, GmState, GmStepResult, check, ptr


class Relaxation:
    def __init__(self, params: GmParams):
        self.lib = _abi.load()
        self.p = params.copy()
        self.dtype = params.real_dtype()
        self.h = C.c_void_p()
        check(self.lib.gm_create(self.p, C.byref(self.h)), "gm_create")
        nx, ny, nz = params.nx, params.ny, params.nz
        self.G = (nz + 2, ny + 2, nx + 2)
        self.I = (nz, ny, nx)

    # -- lifecycle -----------------------------------------------------------
    def close(self):
        if self.h:
            self.lib.gm_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr: int | None):
        check(self.lib.gm_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None), "gm_set_stream")

    # -- state ----------------------------------------------------------------
    def upload(self, xb: np.ndarray, B0: np.ndarray, t: float = 0.0, dt: float | None = None):
        xb = np.ascontiguousarray(xb, dtype=self.dtype)
        B0 = np.ascontiguousarray(B0, dtype=self.dtype)
        if xb.shape != self.G + (3,) or B0.shape != self.G + (3,):
            raise ValueError(f"expected arrays of shape {self.G + (3,)}")
        check(self.lib.gm_upload(self.h, ptr(xb), ptr(B0), t, self.p.dt0 if dt is None else dt), "gm_upload")

    def upload_ptr(self, xb_ptr: int, B0_ptr: int, t: float = 0.0, dt: float | None = None):
        """Upload from host pointers (pinned buffers in the reference layout)."""
        check(self.lib.gm_upload(self.h, C.c_void_p(xb_ptr), C.c_void_p(B0_ptr), t,
                                 self.p.dt0 if dt is None else dt), "gm_upload")

    def state(self) -> dict:
        s = GmState()
        check(self.lib.gm_get_state(self.h, C.byref(s)), "gm_get_state")
        return dict(t=s.t, dt=s.dt, maxDelta=s.maxDelta, timeIndex=s.timeIndex, nAttempted=s.nAttempted,
                    nRejected=s.nRejected, status=s.status)

    def set_time(self, t: float, dt: float, timeIndex: int = 0):
        check(self.lib.gm_set_dt(self.h, t, dt, timeIndex), "gm_set_dt")

    # -- hot path -------------------------------------------------------------
    def stage(self, n: int):
        check(self.lib.gm_stage(self.h, n), "gm_stage")

    def control(self):
        check(self.lib.gm_control(self.h), "gm_control")

    def step(self) -> dict:
        r = GmStepResult()
        check(self.lib.gm_step(self.h, C.byref(r)), "gm_step")
        return dict(maxDelta=r.maxDelta, t=r.t, dt=r.dt, accepted=r.accepted, timeIndex=r.timeIndex, status=r.status)

    def steps_async(self, n: int):
        check(self.lib.gm_steps_async(self.h, n), "gm_steps_async")

    def run(self, nCycle: int) -> dict:
        s = GmState()
        check(self.lib.gm_run(self.h, nCycle, C.byref(s)), "gm_run")
        return dict(t=s.t, dt=s.dt, maxDelta=s.maxDelta, timeIndex=s.timeIndex, nAttempted=s.nAttempted,
                    nRejected=s.nRejected, status=s.status)

    def run_events(self, nCycle: int) -> dict:
        """gm_run_events: run until nCycle accepted steps, stopping after each
        step whose output is due; 'event' holds the GM_EV_* bits."""
        s = GmState()
        check(self.lib.gm_run_events(self.h, nCycle, C.byref(s)), "gm_run_events")
        return dict(t=s.t, dt=s.dt, maxDelta=s.maxDelta, timeIndex=s.timeIndex, nAttempted=s.nAttempted,
                    nRejected=s.nRejected, status=s.status, dtUsed=s.dtUsed, event=s.event)

    def grid_fields(self) -> dict:
        """Cell volume, convexity and minimum wedge product per inner point."""
        out = {k: np.empty(self.I, self.dtype) for k in ("cellVol", "convexity", "wedgeMin")}
        check(self.lib.gm_grid_fields(self.h, ptr(out["cellVol"]), ptr(out["convexity"]), ptr(out["wedgeMin"])),
              "gm_grid_fields")
        return out

    def refresh(self) -> dict:
        r = GmReduction()
        check(self.lib.gm_refresh(self.h, C.byref(r)), "gm_refresh")
        return r.as_dict()

    # -- transfers ------------------------------------------------------------
    def download(self) -> dict:
        xb = np.empty(self.G + (3,), self.dtype)
        B = np.empty(self.G + (3,), self.dtype)
        J = np.empty(self.I + (3,), self.dtype)
        D = np.empty(self.G, self.dtype)
        check(self.lib.gm_download(self.h, ptr(xb), ptr(B), ptr(J), ptr(D)), "gm_download")
        return dict(xb=xb, B=B, J=J, detJac=D)

    def grid(self) -> np.ndarray:
        xb = np.empty(self.G + (3,), self.dtype)
        check(self.lib.gm_download(self.h, ptr(xb), None, None, None), "gm_download")
        return xb

    def k(self, m: int) -> np.ndarray:
        """k_m, [nz, ny, nx, 3] (or 6 with inertia: position then velocity increment)."""
        k = np.empty(self.I + (6 if self.p.inertia else 3,), self.dtype)
        check(self.lib.gm_download_k(self.h, m, ptr(k)), "gm_download_k")
        return k

    def x(self, which: int) -> np.ndarray:
        x = np.empty(self.G + (3,), self.dtype)
        check(self.lib.gm_download_x(self.h, which, ptr(x)), "gm_download_x")
        return x

    def autotune(self, trials: int = 3) -> dict:
        """gm_autotune: time the stage kernel's z-chunk depths, keep the fastest."""
        tz, ms = C.c_int(), C.c_double()
        check(self.lib.gm_autotune(self.h, trials, C.byref(tz), C.byref(ms)), "gm_autotune")
        return dict(tz=tz.value, ms_stages_0_4=ms.value)

    def set_tile_z(self, tz: int):
        check(self.lib.gm_set_tile_z(self.h, tz), "gm_set_tile_z")

    def upload_u(self, u: np.ndarray):
        """Velocity of an inertia run at the inner points, [nz, ny, nx, 3]."""
        u = np.ascontiguousarray(u, dtype=self.dtype)
        assert u.shape == self.I + (3,)
        check(self.lib.gm_upload_u(self.h, ptr(u)), "gm_upload_u")

    def u(self, which: int = 5) -> np.ndarray:
        """Velocity: which = 0..4 stage velocity u_{which+1}; 5 the current one; 6 u_new."""
        u = np.empty(self.I + (3,), self.dtype)
        check(self.lib.gm_download_u(self.h, which, ptr(u)), "gm_download_u")
        return u

    @property
    def launches(self) -> int:
        return int(self.lib.gm_launch_count(self.h))
