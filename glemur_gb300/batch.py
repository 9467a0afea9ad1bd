"""Python handle over the batched entry points of include/glemur.h.

``BatchRelaxation`` owns one gm_batch: many independent cases of uneven grid
sizes whose Runge-Kutta stages run as one persistent launch each, with one
controller launch per step and the step captured as one CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import GmBatchCase, GmParams, GmReduction, GmState, check, ptr


class BatchRelaxation:
    def __init__(self, cases: list[GmParams]):
        self.lib = _abi.load()
        self.ps = [p.copy() for p in cases]
        arr = (GmParams * len(cases))(*self.ps)
        self.h = C.c_void_p()
        check(self.lib.gm_batch_create(arr, len(cases), C.byref(self.h)), "gm_batch_create")
        self.n = len(cases)

    def close(self):
        if self.h:
            self.lib.gm_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shapes(self, c):
        p = self.ps[c]
        return (p.nz + 2, p.ny + 2, p.nx + 2), (p.nz, p.ny, p.nx), p.real_dtype()

    def upload(self, c: int, xb: np.ndarray, B0: np.ndarray, t: float = 0.0, dt: float | None = None):
        G, _, dt_ = self._shapes(c)
        xb = np.ascontiguousarray(xb, dtype=dt_)
        B0 = np.ascontiguousarray(B0, dtype=dt_)
        if xb.shape != G + (3,) or B0.shape != G + (3,):
            raise ValueError(f"case {c}: expected arrays of shape {G + (3,)}")
        check(self.lib.gm_batch_upload(self.h, c, ptr(xb), ptr(B0), t, self.ps[c].dt0 if dt is None else dt),
              "gm_batch_upload")

    def steps_async(self, n: int):
        check(self.lib.gm_batch_steps_async(self.h, n), "gm_batch_steps_async")

    def state(self, c: int) -> dict:
        s = GmState()
        check(self.lib.gm_batch_get_state(self.h, c, C.byref(s)), "gm_batch_get_state")
        return dict(t=s.t, dt=s.dt, maxDelta=s.maxDelta, timeIndex=s.timeIndex, nAttempted=s.nAttempted,
                    nRejected=s.nRejected, status=s.status)

    def refresh(self, c: int) -> dict:
        r = GmReduction()
        check(self.lib.gm_batch_refresh(self.h, c, C.byref(r)), "gm_batch_refresh")
        return r.as_dict()

    def download(self, c: int) -> dict:
        G, I, dt_ = self._shapes(c)
        out = dict(xb=np.empty(G + (3,), dt_), B=np.empty(G + (3,), dt_), J=np.empty(I + (3,), dt_),
                   detJac=np.empty(G, dt_))
        check(self.lib.gm_batch_download(self.h, c, ptr(out["xb"]), ptr(out["B"]), ptr(out["J"]),
                                         ptr(out["detJac"])), "gm_batch_download")
        return out

    def autotune(self, trials: int = 3) -> dict:
        """gm_batch_autotune: time work-item depths 16, 32, 64; keep the fastest."""
        tzb, ms = C.c_int(), C.c_double()
        check(self.lib.gm_batch_autotune(self.h, trials, C.byref(tzb), C.byref(ms)), "gm_batch_autotune")
        return dict(tzb=tzb.value, ms_stages_0_4=ms.value)

    def stop(self, c: int):
        check(self.lib.gm_batch_stop(self.h, c), "gm_batch_stop")

    def run(self, nCycle: int, residual: float, pointwise: bool = False, check_every: int = 10) -> list[dict]:
        out = (GmBatchCase * self.n)()
        check(self.lib.gm_batch_run(self.h, nCycle, residual, 1 if pointwise else 0, check_every, out),
              "gm_batch_run")
        return [o.as_dict() for o in out]

    def launches(self) -> int:
        return int(self.lib.gm_batch_launch_count(self.h))
