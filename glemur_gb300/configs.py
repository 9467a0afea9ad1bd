"""Run parameters of the relaxation workloads.

Each builder starts from the namelist defaults (gm_params_default, which
restates src/readNamelist.f90:92-150) and sets what a params.in for the
workload would set.  Real values are rounded to the run precision, as the
namelist reader reads them into REAL.

Workloads (synthetic initial fields; no dataset is involved):

* ``braid2``   -- 32x32x64 inner points over [-4,4]x[-4,4]x[-24,24], periodic in
  x and y, line-tied in z, B0 = e_z plus two twisted Gaussian blobs
  (x,y,z) = (1,0,-4) k=+1 and (-1,0,4) k=-1, a = sqrt(2), l = 2, FP64,
  maxError 1e-5, dt0 3e-4, 2000 accepted steps.
* ``braid6``   -- 128x128x256 inner points, same domain and boundaries, six
  alternating blobs at z = -20,-12,-4,4,12,20 (x = +1,-1,..., k = +1,-1,...),
  FP32 storage, run to mean |JxB|/(|J||B|) <= 1e-2.
* ``braid6_large`` -- 256x256x512, the six-blob braid with k = +-1.2 and the
  pressure term with p0 = 0.1 (1 + 0.5 exp(-r^2/4)).
* ``random_braid`` -- seeded braids of 2..8 blobs used for the batched mode.

A blob of strength k and width a enters the reference's "blobs" field
(src/init.cu:109-124) as blobTwist = k a / 2, blobScale = a, blobZl = l.
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi
from ._abi import GmParams


def defaults(precision: int) -> GmParams:
    p = GmParams()
    _abi.check(_abi.load().gm_params_default(p, precision), "gm_params_default")
    return p


def derive(p: GmParams) -> GmParams:
    _abi.check(_abi.load().gm_params_derive(p), "gm_params_derive")
    return p


def set_blobs(p: GmParams, blobs) -> None:
    """blobs: iterable of (x, y, z, k, a, l)."""
    blobs = list(blobs)
    if len(blobs) > 10:
        raise ValueError("at most 10 blobs (src/global.h:62)")
    p.set_str("bInit", "blobs")
    p.nBlobs = len(blobs)
    for b, (x, y, z, k, a, l) in enumerate(blobs):
        p.blobXc[b] = p.rnd(x)
        p.blobYc[b] = p.rnd(y)
        p.blobZc[b] = p.rnd(z)
        p.blobTwist[b] = p.rnd(k * a / 2.0)
        p.blobScale[b] = p.rnd(a)
        p.blobZl[b] = p.rnd(l)


def braid_box(nx: int, ny: int, nz: int, precision: int, L=(8.0, 8.0, 48.0), O=(-4.0, -4.0, -24.0)) -> GmParams:
    """Periodic x and y, line-tied z, the relaxation's usual box."""
    p = defaults(precision)
    p.nx, p.ny, p.nz = nx, ny, nz
    p.Lx, p.Ly, p.Lz = (p.rnd(v) for v in L)
    p.Ox, p.Oy, p.Oz = (p.rnd(v) for v in O)
    p.xPeri, p.yPeri, p.zPeri = 1, 1, 0
    p.ampl = 1.0
    p.dt0 = p.rnd(3e-4)
    p.dtMin = p.rnd(1e-8)
    p.maxError = p.rnd(1e-5)
    p.nTs = 10
    return derive(p)


def braid2(nx=32, ny=32, nz=64, precision=64, nCycle=2000) -> GmParams:
    p = braid_box(nx, ny, nz, precision)
    a = math.sqrt(2.0)
    set_blobs(p, [(1.0, 0.0, -4.0, 1.0, a, 2.0), (-1.0, 0.0, 4.0, -1.0, a, 2.0)])
    p.nCycle = nCycle
    return derive(p)


def braid6(nx=128, ny=128, nz=256, precision=32, k=1.0, nCycle=100000) -> GmParams:
    p = braid_box(nx, ny, nz, precision)
    a = math.sqrt(2.0)
    zs = [-20.0, -12.0, -4.0, 4.0, 12.0, 20.0]
    set_blobs(p, [((1.0 if i % 2 == 0 else -1.0), 0.0, z, (k if i % 2 == 0 else -k), a, 2.0)
                  for i, z in enumerate(zs)])
    p.nCycle = nCycle
    return derive(p)


def braid6_large(nx=256, ny=256, nz=512, precision=32) -> GmParams:
    p = braid6(nx, ny, nz, precision, k=1.2)
    p.pressure = 1
    p.beta = p.rnd(0.1)
    p.p0Amp = p.rnd(0.5)
    p.p0Width = p.rnd(2.0)
    return derive(p)


def random_braid(seed: int, shape=None, precision=32) -> GmParams:
    """Seeded braid: 2-8 blobs, k ~ +-U[0.5,1.2], a ~ U[1,2], l ~ U[1.5,3],
    (x,y) ~ U[-2,2]^2, z evenly spread (z_b = Oz + (b+1/2) Lz/nBlobs)."""
    rng = np.random.default_rng(seed)
    if shape is None:
        shapes = [(32, 32, 32), (48, 48, 96), (64, 64, 128), (96, 96, 192)]
        shape = shapes[int(rng.integers(len(shapes)))]
    p = braid_box(*shape, precision=precision)
    nb = int(rng.integers(2, 9))
    blobs = []
    for b in range(nb):
        k = float(rng.uniform(0.5, 1.2)) * (1.0 if rng.random() < 0.5 else -1.0)
        a = float(rng.uniform(1.0, 2.0))
        l = float(rng.uniform(1.5, 3.0))
        x, y = (float(v) for v in rng.uniform(-2.0, 2.0, size=2))
        z = -24.0 + (b + 0.5) * 48.0 / nb
        blobs.append((x, y, z, k, a, l))
    set_blobs(p, blobs)
    return derive(p)


def init_state(p: GmParams):
    """Initial B0 and grid in the reference layout (gm_init_state)."""
    dt = p.real_dtype()
    G = (p.nz + 2, p.ny + 2, p.nx + 2, 3)
    B0 = np.zeros(G, dtype=dt)
    xb = np.zeros(G, dtype=dt)
    _abi.check(_abi.load().gm_init_state(p, _abi.ptr(B0), _abi.ptr(xb)), "gm_init_state")
    return B0, xb
