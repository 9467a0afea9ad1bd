"""Training and evaluation of the learned warm start (glemur_gb300/warmstart.py).

    python -m glemur_gb300.train_warmstart --train 256 --eval 32 --residual 0.15 \\
        --minutes 6 --out weights.npz --report report.json

1. Data: seeded random braids (configs.random_braid: 2-8 blobs, k ~ +-U[0.5,
   1.2], a ~ U[1, 2], l ~ U[1.5, 3]) on a fixed 64x64x128 grid are relaxed by
   the batched plain path (FP32) until the weighted force-free residual reaches
   `--residual`; each converged case gives a pair (B0, (x - X) / spacing).
   Cases whose grid folds first (dt <= dtMin) are left out.
2. Training: the U-Net on those pairs with Adam (cosine learning-rate decay)
   for a wall-clock budget, every step in this library's kernels.
3. Evaluation on held-out seeds: for each case, the wall time from the
   initial state to the residual target for the plain relaxation, and for the
   warm start (network inference + grid build + validity check + relaxation),
   the residual right after the warm start, whether it was accepted
   (min Delta > 0) and min Delta over the run.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import BatchRelaxation, Relaxation, configs
from .warmstart import WB, UNet, load_weights, n_params, save_weights, weights_width

SHAPE = (64, 64, 128)
TRAIN_SEED0 = 100000      # training seeds TRAIN_SEED0 + i
EVAL_SEED0 = 900000       # held-out seeds EVAL_SEED0 + i


def case(seed, shape=None):
    return configs.random_braid(seed, shape=shape or SHAPE, precision=32)


def displacement(p, xb, xb0):
    """(x - X) / spacing at the inner points, float32 [V][3] in voxel order."""
    sp = np.array([p.dx, p.dy, p.dz], dtype=np.float64)
    d = (xb[1:-1, 1:-1, 1:-1].astype(np.float64) - xb0[1:-1, 1:-1, 1:-1].astype(np.float64)) / sp
    return d.reshape(-1, 3).astype(np.float32)


def relax_to_residual_batched(ps, residual, max_cycles, check_every=10):
    """Relax cases together; returns (final grids, per-case outcomes)."""
    b = BatchRelaxation(ps)
    for c, p in enumerate(ps):
        B0, xb = configs.init_state(p)
        b.upload(c, xb, B0)
    out = b.run(max_cycles, residual, pointwise=False, check_every=check_every)
    grids = [b.download(c)["xb"] for c in range(len(ps))]
    b.close()
    return grids, out


def make_data(seeds, residual, max_cycles, log=print):
    """Training pairs from relaxed random braids (converged cases only)."""
    import torch
    data = []
    t0 = time.perf_counter()
    for i0 in range(0, len(seeds), 64):
        ps = [case(s) for s in seeds[i0:i0 + 64]]
        grids, out = relax_to_residual_batched(ps, residual, max_cycles)
        for p, xb, o in zip(ps, grids, out):
            if not o["converged"]:
                continue
            B0, xb0 = configs.init_state(p)
            data.append((torch.from_numpy(B0).cuda(), torch.from_numpy(displacement(p, xb, xb0)).cuda()))
        log(f"data: {len(data)} pairs from {i0 + len(ps)} braids, {time.perf_counter() - t0:.1f} s")
    return data


def train(net, data, minutes, lr=1e-3, batch=4, log=print, symmetries=True):
    """Adam with cosine decay over a wall-clock budget; returns the loss
    history.  Each sample is moved by a random whole-cell translation along
    the periodic axes and, with `symmetries`, a random mirror / x <-> y swap
    of the cross-section (gm_nn_input): exact copies of the problem, so a
    pair stands for 8 nx ny pairs."""
    import torch
    nx, ny, nz = net.shape
    scale = 1.0 / (batch * nx * ny * nz * 3)
    rng = np.random.default_rng(0)
    hist = []
    t0 = time.perf_counter()
    budget = 60.0 * minutes
    step = 0
    while True:
        order = rng.permutation(len(data))
        for q in range(0, len(order) - batch + 1, batch):
            el = time.perf_counter() - t0
            if el > budget:
                return hist
            frac = el / budget
            lr_t = 0.1 * lr + 0.9 * lr * 0.5 * (1 + np.cos(np.pi * frac))
            net.zero_grad()
            for k in order[q:q + batch]:
                B0, tgt = data[k]
                # whole-cell translations along the periodic axes and the
                # mirrors / swap of the cross-section: exact copies of the problem
                sh = (int(rng.integers(nx)), int(rng.integers(ny)))
                sym = int(rng.integers(8 if nx == ny else 4)) if symmetries else 0
                net.set_input_b0(B0, 32, sh, sym)
                net.forward()
                net.backward(tgt, scale, sh, sym)
            net.refresh_weights(lr=lr_t, step=True)
            step += 1
            if step % 25 == 0:
                hist.append((step, time.perf_counter() - t0, float(net.loss_acc.item())))
                log(f"train: step {step} {hist[-1][1]:.0f} s loss {hist[-1][2]:.4e} lr {lr_t:.2e}")
                net.check_status()


def smooth_displacement(d, passes, xper=True, yper=True):
    """`passes` 3x3x3 box-filter passes over a displacement [nz, ny, nx, 3]
    (periodic in x / y, zero beyond the z range): removes the network's
    grid-scale noise, which would otherwise show up as current."""
    for _ in range(passes):
        acc = np.zeros_like(d)
        for dk in (-1, 0, 1):
            if dk == 0:
                dz = d
            else:
                dz = np.zeros_like(d)
                if dk > 0:
                    dz[:-dk] = d[dk:]
                else:
                    dz[-dk:] = d[:dk]
            for dj in (-1, 0, 1):
                for di in (-1, 0, 1):
                    acc += np.roll(dz, (-dj, -di), axis=(1, 2))
        d = acc / 27.0
    return d


def warm_grid(net, p, B0, smooth=2):
    """The predicted grid in the reference layout (ghosted AoS): the identity
    grid plus the network's displacement at the inner points (optionally
    smoothed; zero on the first and last z-planes), periodic ghosts as shifted
    images."""
    import torch
    nx, ny, nz = p.nx, p.ny, p.nz
    net.set_input_b0(torch.from_numpy(B0).cuda(), 32)
    y = net.forward()[:, :3].float().cpu().numpy().reshape(nz, ny, nx, 3)
    if smooth:
        y = smooth_displacement(y.astype(np.float64), smooth, bool(p.xPeri), bool(p.yPeri))
    _, xb = configs.init_state(p)
    xb = xb.astype(np.float64)
    sp = np.array([p.dx, p.dy, p.dz])
    d = y * sp
    d[0] = 0.0
    d[-1] = 0.0
    xb[1:-1, 1:-1, 1:-1] += d
    if p.xPeri:
        xb[:, :, 0] = xb[:, :, nx]
        xb[:, :, 0, 0] -= p.Lx + p.dx
        xb[:, :, nx + 1] = xb[:, :, 1]
        xb[:, :, nx + 1, 0] += p.Lx + p.dx
    if p.yPeri:
        xb[:, 0] = xb[:, ny]
        xb[:, 0, :, 1] -= p.Ly + p.dy
        xb[:, ny + 1] = xb[:, 1]
        xb[:, ny + 1, :, 1] += p.Ly + p.dy
    return xb.astype(np.float32)


# input translations for test-time averaging: not multiples of 4 (the two 2x
# poolings make the network equivariant to those, so they would repeat the
# same prediction)
TTA_SHIFTS = ((0, 0), (2, 2), (1, 3), (3, 1), (2, 0), (0, 2), (1, 1), (3, 3))


class DeviceWarmGrid:
    """The warm grid built on the device: the network's displacement
    (optionally averaged over input translations, gm_nn_disp_accumulate),
    smoothed and added to the identity grid with periodic ghosts set
    (gm_nn_warm_grid), without a host round trip; with one translation and
    the same smoothing it is the grid warm_grid builds on the host, up to the
    float rounding of the smoothing."""

    def __init__(self, p, xid):
        import torch
        from . import _abi
        self.p = p
        self.lib = _abi.load()
        self.xid = torch.from_numpy(np.ascontiguousarray(xid)).cuda()
        self.xb = torch.empty_like(self.xid)
        V = p.nx * p.ny * p.nz
        self.d = torch.empty(3 * V, dtype=torch.float32, device="cuda")
        self.scratch = torch.empty(6 * V, dtype=torch.float32, device="cuda")

    def build(self, net, B0_dev, smooth=2, tta=1):
        import torch
        from . import _abi
        p = self.p
        stream = _abi.VP(torch.cuda.current_stream().cuda_stream)
        shifts = TTA_SHIFTS[:max(1, tta)]
        for q, sh in enumerate(shifts):
            net.set_input_b0(B0_dev, p.precision, sh)
            y = net.forward()
            _abi.check(self.lib.gm_nn_disp_accumulate(_abi.VP(y.data_ptr()), y.stride(0), p.nx, p.ny, p.nz, sh[0], sh[1],
                                                      1.0 / len(shifts), 1 if q == 0 else 0,
                                                      _abi.VP(self.d.data_ptr()), stream), "gm_nn_disp_accumulate")
        _abi.check(self.lib.gm_nn_warm_grid(_abi.VP(self.d.data_ptr()), p, smooth, _abi.VP(self.xid.data_ptr()),
                                            _abi.VP(self.scratch.data_ptr()), _abi.VP(self.xb.data_ptr()), stream),
                   "gm_nn_warm_grid")
        return self.xb


def time_to_residual(g, p, xb, B0, residual, max_attempts, check_every=50):
    """Upload, then relax until the weighted residual is at most `residual`.
    Returns (seconds, attempts, residual at start, min Delta seen, reached)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.upload(xb, B0)
    r = g.refresh()
    r0, mind = r["residual"], r["minDetJac"]
    att = 0
    reached = r0 <= residual
    while not reached and att < max_attempts:
        g.steps_async(check_every)
        s = g.state()
        r = g.refresh()
        att = s["nAttempted"]
        mind = min(mind, r["minDetJac"])
        if r["residual"] <= residual:
            reached = True
        elif s["status"] & 0x17:
            break
    return time.perf_counter() - t0, att, r0, mind, reached


def evaluate(net, seeds, residual, max_attempts, log=print, smooth=2, tta=1):
    import torch
    rows = []
    for s in seeds:
        p = case(s)
        B0, xb0 = configs.init_state(p)
        g = Relaxation(p)
        g.upload(xb0, B0)
        g.steps_async(2)       # capture the step graph outside the timed runs
        g.state()
        tp, ap, rp0, mdp, okp = time_to_residual(g, p, xb0, B0, residual, max_attempts)
        d_true = displacement(p, g.download()["xb"], xb0)
        # the warm start's own cost: B0 to the device, inference, grid build
        # (on the device), upload, validity check
        wg = DeviceWarmGrid(p, xb0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        B0_dev = torch.from_numpy(B0).cuda()
        xw_dev = wg.build(net, B0_dev, smooth, tta)
        torch.cuda.synchronize()
        g.upload_ptr(xw_dev.data_ptr(), B0_dev.data_ptr())
        accepted = g.refresh()["minDetJac"] > 0
        t_net = time.perf_counter() - t0
        xw = xw_dev.cpu().numpy() if accepted else xb0
        d_pred = displacement(p, xw, xb0)
        rms_true = float(np.sqrt((d_true.astype(np.float64) ** 2).mean()))
        rms_err = float(np.sqrt(((d_pred.astype(np.float64) - d_true) ** 2).mean()))
        tw, aw, rw0, mdw, okw = time_to_residual(g, p, xw, B0, residual, max_attempts)
        tw += t_net
        g.close()
        rows.append(dict(seed=s, plain_s=tp, plain_attempts=ap, plain_reached=okp, plain_res0=rp0, plain_minDet=mdp,
                         warm_s=tw, warm_attempts=aw, warm_reached=okw, warm_res0=rw0, warm_minDet=mdw,
                         accepted=bool(accepted), net_s=t_net, rms_disp=rms_true, rms_err=rms_err))
        log(f"eval seed {s}: plain {tp:.2f} s ({ap} att, reached {okp}), warm {tw:.2f} s ({aw} att, res0 "
            f"{rw0:.3f}, accepted {accepted}, reached {okw}), displacement rms {rms_true:.3f} err {rms_err:.3f}")
    return rows


def coarse_b0(p, B0, f):
    """B0 averaged over f x f x f blocks of inner points, in a ghosted array
    of the coarse grid (ghost values unused by the network input)."""
    nx, ny, nz = p.nx // f, p.ny // f, p.nz // f
    inner = B0[1:-1, 1:-1, 1:-1].astype(np.float64).reshape(nz, f, ny, f, nx, f, 3).mean(axis=(1, 3, 5))
    out = np.zeros((nz + 2, ny + 2, nx + 2, 3), np.float32)
    out[1:-1, 1:-1, 1:-1] = inner
    return out


def upsample_displacement(d, f, fine, per=(True, True)):
    """Trilinear interpolation of a coarse displacement field [cz, cy, cx, 3]
    (coarse voxel I centred on fine index f I + (f - 1) / 2) to the fine inner
    points; periodic in x and y, clamped in z."""
    nx, ny, nz = fine
    out = d
    for axis, n, periodic in ((2, nx, per[0]), (1, ny, per[1]), (0, nz, False)):
        c = out.shape[axis]
        pos = (np.arange(n) - (f - 1) / 2.0) / f
        i0 = np.floor(pos).astype(int)
        w = pos - i0
        if periodic:
            a, b = i0 % c, (i0 + 1) % c
        else:
            a, b = np.clip(i0, 0, c - 1), np.clip(i0 + 1, 0, c - 1)
        shape = [1, 1, 1, 1]
        shape[axis] = n
        w = w.reshape(shape)
        out = np.take(out, a, axis=axis) * (1 - w) + np.take(out, b, axis=axis) * w
    return out


LARGE_LEVELS = (0.4, 0.3, 0.25, 0.2, 0.15, 0.1)


def residual_history(g, xb, B0, max_attempts, stop_at, check_every=200):
    """Upload, then relax for at most `max_attempts` attempts or until the
    weighted residual is at most `stop_at`, reading the residual every
    `check_every` attempts.  Returns [(seconds, attempts, residual, min
    Delta)], the first entry at the start, and the final status word (a
    fold stops the run: GM_ST_DETJAC, GM_ST_DTMIN or GM_ST_NAN)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.upload(xb, B0)
    r = g.refresh()
    hist = [(time.perf_counter() - t0, 0, r["residual"], r["minDetJac"])]
    status = 0
    while hist[-1][1] < max_attempts and hist[-1][2] > stop_at:
        g.steps_async(check_every)
        s = g.state()
        r = g.refresh()
        hist.append((time.perf_counter() - t0, s["nAttempted"], r["residual"], r["minDetJac"]))
        status = s["status"]
        if status & 0x17:
            break
    return hist, status


def first_reach(hist, level, offset=0.0):
    """(seconds + offset, attempts) of the first entry at or below `level`."""
    for t, att, res, _ in hist:
        if res <= level:
            return t + offset, att
    return None, None


def level_times(plain, warm, t_net, folded, levels=LARGE_LEVELS):
    """Per residual level: the plain run's and the warm-started run's time and
    attempts to reach it (residual_history entries), the warm start's own
    cost t_net included.  A warm grid that folded during its run is replaced
    by the identity grid: its levels are then the plain run's, plus the time
    and attempts the folded run took."""
    out = {}
    spent, spent_att = warm[-1][0] + t_net, warm[-1][1]
    for lv in levels:
        tp, ap = first_reach(plain, lv)
        if folded:
            tw, aw = first_reach(plain, lv, spent)
            aw = aw + spent_att if aw is not None else None
        else:
            tw, aw = first_reach(warm, lv, t_net)
        out[str(lv)] = dict(plain_s=tp, plain_attempts=ap, warm_s=tw, warm_attempts=aw,
                            speedup=(tp / tw) if (tp and tw) else None)
    return out


def evaluate_large(weights, residual, max_attempts, factors=(2, 4), log=print):
    """The large case (256x256x512, k = +-1.2, pressure with the p0 profile):
    the network runs on B0 averaged over f x f x f blocks and its displacement
    is trilinearly upsampled to the fine grid.  The plain run and one warm run
    per factor record the residual every 200 attempts, up to `max_attempts`
    or `residual`; the report gives, per residual level, the time each run
    took to reach it (the warm start's own cost included).  A warm grid that
    folds during the run (the controller stops on Delta <= 0, dt below dtMin
    or a NaN) is replaced by the identity grid: the levels are then the plain
    run's, plus the time the warm start and its run took."""
    import torch
    p = configs.braid6_large(256, 256, 512, precision=32)
    B0, xb0 = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb0, B0)
    g.steps_async(2)
    g.state()
    plain, _ = residual_history(g, xb0, B0, max_attempts, residual)
    out = dict(shape=(p.nx, p.ny, p.nz), max_attempts=max_attempts,
               plain=dict(res0=plain[0][2], res_end=plain[-1][2], attempts=plain[-1][1], s=plain[-1][0],
                          minDet=min(h[3] for h in plain), history=[(round(h[0], 3), h[1], h[2]) for h in plain[::5]]),
               warm={})
    log(f"large plain: {out['plain']}")
    for f in factors:
        cshape = (p.nx // f, p.ny // f, p.nz // f)
        net = UNet(cshape, seed=0, wb=weights_width(weights))
        net.load_state_dict(weights)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Bc = coarse_b0(p, B0, f)
        net.set_input_b0(torch.from_numpy(Bc).cuda(), 32)
        y = net.forward()[:, :3].float().cpu().numpy().reshape(cshape[2], cshape[1], cshape[0], 3)
        y = smooth_displacement(y.astype(np.float64), 2)
        # coarse grid units -> physical -> fine inner points
        sp_c = np.array([p.dx, p.dy, p.dz]) * f
        d = upsample_displacement(y * sp_c, f, (p.nx, p.ny, p.nz))
        d[0] = 0.0
        d[-1] = 0.0
        xw = xb0.astype(np.float64)
        xw[1:-1, 1:-1, 1:-1] += d
        nx, ny = p.nx, p.ny
        xw[:, :, 0] = xw[:, :, nx]; xw[:, :, 0, 0] -= p.Lx + p.dx
        xw[:, :, nx + 1] = xw[:, :, 1]; xw[:, :, nx + 1, 0] += p.Lx + p.dx
        xw[:, 0] = xw[:, ny]; xw[:, 0, :, 1] -= p.Ly + p.dy
        xw[:, ny + 1] = xw[:, 1]; xw[:, ny + 1, :, 1] += p.Ly + p.dy
        xw = xw.astype(np.float32)
        g.upload(xw, B0)
        accepted = g.refresh()["minDetJac"] > 0
        if not accepted:
            xw = xb0
        t_net = time.perf_counter() - t0
        del net
        warm, wstat = residual_history(g, xw, B0, max_attempts, residual)
        folded = bool(wstat & 0x7) and warm[-1][2] > residual
        levels = level_times(plain, warm, t_net, folded)
        out["warm"][str(f)] = dict(coarse_shape=cshape, accepted=bool(accepted), net_s=t_net, res0=warm[0][2],
                                   res_end=warm[-1][2], attempts=warm[-1][1], s=warm[-1][0] + t_net, status=wstat,
                                   folded_in_run=folded, minDet=min(h[3] for h in warm), levels=levels,
                                   history=[(round(h[0], 3), h[1], h[2]) for h in warm[::5]])
        log(f"large warm, factor {f}: {out['warm'][str(f)]}")
    g.close()
    return out


def evaluate_batched(net, seeds, residual, max_cycles, smooth=2, chunk=64, log=print):
    """Held-out seeds in batches of `chunk` cases: every case of a batch is
    relaxed together by the batched plain path (one persistent launch per
    stage), first from the identity grid, then from the network's grid (built
    on the device; a grid with min Delta <= 0 is replaced by the identity
    grid).  Per case: attempts to the residual target, the residual at the
    start, min Delta of the warm grid; per batch: the wall time of the plain
    run and of the warm run, the latter including inference, grid builds,
    uploads and validity checks."""
    import torch
    from . import _abi
    lib = _abi.load()
    rows, batches = [], []
    for i0 in range(0, len(seeds), chunk):
        ss = seeds[i0:i0 + chunk]
        ps = [case(s) for s in ss]
        inits = [configs.init_state(p) for p in ps]
        b = BatchRelaxation(ps)
        for c, (B0, xb) in enumerate(inits):
            b.upload(c, xb, B0)
        b.steps_async(2)            # capture the step graph outside the timed runs
        b.state(0)
        for c, (B0, xb) in enumerate(inits):
            b.upload(c, xb, B0)
        res0p = [b.refresh(c)["residual"] for c in range(len(ps))]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        outp = b.run(max_cycles, residual, pointwise=False, check_every=10)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        # warm start: inference and grid build on the device, then the same run
        t0 = time.perf_counter()
        acc, mind, res0w = [], [], []
        for c, (p, (B0, xb0)) in enumerate(zip(ps, inits)):
            B0d = torch.from_numpy(B0).cuda()
            xw = DeviceWarmGrid(p, xb0).build(net, B0d, smooth)
            torch.cuda.synchronize()
            _abi.check(lib.gm_batch_upload(b.h, c, _abi.VP(xw.data_ptr()), _abi.VP(B0d.data_ptr()), 0.0, p.dt0),
                       "gm_batch_upload")
            r = b.refresh(c)
            ok = r["minDetJac"] > 0
            if not ok:
                b.upload(c, xb0, B0)
                r = b.refresh(c)
            acc.append(ok)
            mind.append(r["minDetJac"])
            res0w.append(r["residual"])
        torch.cuda.synchronize()
        t_net = time.perf_counter() - t0
        t0 = time.perf_counter()
        outw = b.run(max_cycles, residual, pointwise=False, check_every=10)
        torch.cuda.synchronize()
        tw = time.perf_counter() - t0 + t_net
        b.close()
        for q, s in enumerate(ss):
            rows.append(dict(seed=s, plain_attempts=outp[q]["attempted"], plain_reached=bool(outp[q]["converged"]),
                             plain_res0=res0p[q], warm_attempts=outw[q]["attempted"],
                             warm_reached=bool(outw[q]["converged"]), warm_res0=res0w[q], accepted=acc[q],
                             warm_minDet=mind[q]))
        batches.append(dict(cases=len(ss), plain_s=tp, warm_s=tw, warm_start_s=t_net))
        log(f"eval batch {i0 // chunk}: {len(ss)} cases, plain {tp:.1f} s, warm {tw:.1f} s "
            f"(warm start {t_net:.1f} s), accepted {sum(acc)}")
    both = [r for r in rows if r["plain_reached"] and r["warm_reached"]]
    att = [r["plain_attempts"] / max(r["warm_attempts"], 1) for r in both]
    tp = sum(x["plain_s"] for x in batches)
    tw = sum(x["warm_s"] for x in batches)
    summary = dict(cases=len(rows), accepted=sum(r["accepted"] for r in rows),
                   plain_reached=sum(r["plain_reached"] for r in rows),
                   warm_reached=sum(r["warm_reached"] for r in rows), both_reached=len(both),
                   plain_s=tp, warm_s=tw, speedup_total=tp / tw if tw > 0 else None,
                   attempts_ratio_median=float(np.median(att)) if att else None,
                   plain_res0_median=float(np.median([r["plain_res0"] for r in rows])),
                   warm_res0_median=float(np.median([r["warm_res0"] for r in rows])),
                   min_delta_warm=float(min(r["warm_minDet"] for r in rows)))
    return dict(summary=summary, batches=batches, rows=rows)


def summarize(rows):
    both = [r for r in rows if r["plain_reached"] and r["warm_reached"]]
    sp = [r["plain_s"] / r["warm_s"] for r in both]
    return dict(cases=len(rows), both_reached=len(both), accepted=sum(r["accepted"] for r in rows),
                speedup_median=float(np.median(sp)) if sp else None,
                speedup_total=float(sum(r["plain_s"] for r in both) / sum(r["warm_s"] for r in both)) if both else None,
                plain_res0_median=float(np.median([r["plain_res0"] for r in rows])),
                warm_res0_median=float(np.median([r["warm_res0"] for r in rows])),
                min_delta_warm=float(min(r["warm_minDet"] for r in rows)),
                rms_disp_median=float(np.median([r["rms_disp"] for r in rows])),
                rms_err_median=float(np.median([r["rms_err"] for r in rows])))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=256)
    ap.add_argument("--eval", type=int, default=32)
    ap.add_argument("--residual", type=float, default=0.15)
    ap.add_argument("--max-cycles", type=int, default=8000)
    ap.add_argument("--minutes", type=float, default=6.0)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="")
    ap.add_argument("--report", default="")
    ap.add_argument("--weights", default="", help="evaluate these weights instead of training")
    ap.add_argument("--init", default="", help="start training from these weights (fine-tuning)")
    ap.add_argument("--train-offset", type=int, default=0,
                    help="first training seed: TRAIN_SEED0 + this (braids beyond those of an --init network)")
    ap.add_argument("--no-symmetries", action="store_true",
                    help="augment with translations only (no mirrors / x <-> y swap)")
    ap.add_argument("--shape", default="64,64,128", help="grid (nx,ny,nz), each divisible by 4")
    ap.add_argument("--large", action="store_true", help="also evaluate the 256x256x512 pressure case")
    ap.add_argument("--large-residual", type=float, default=0.0,
                    help="residual target of the large case (default: --residual)")
    ap.add_argument("--large-attempts", type=int, default=24000, help="attempts per run of the large case at most")
    ap.add_argument("--smooth", default="2", help="comma-separated box-filter passes to evaluate")
    ap.add_argument("--tta", default="1", help="comma-separated numbers of input translations to average")
    ap.add_argument("--wb", type=int, default=WB, help="bottleneck channels of a network trained here")
    ap.add_argument("--eval-batched", type=int, default=0,
                    help="also evaluate this many held-out seeds with the batched path")
    a = ap.parse_args(argv)
    global SHAPE
    SHAPE = tuple(int(v) for v in a.shape.split(","))
    log = lambda m: print(m, flush=True)
    w = load_weights(a.weights) if a.weights else None
    w0 = load_weights(a.init) if a.init else None
    wb = weights_width(w) if w is not None else (weights_width(w0) if w0 is not None else a.wb)
    net = UNet(SHAPE, seed=7, wb=wb)
    log(f"U-Net: {n_params(wb)} parameters")
    report = dict(shape=SHAPE, residual=a.residual, params=n_params(wb), wb=wb)
    if w is not None:
        net.load_state_dict(w)
    else:
        if w0 is not None:
            net.load_state_dict(w0)
            report.update(init=a.init)
        t0 = time.perf_counter()
        seeds = [TRAIN_SEED0 + a.train_offset + i for i in range(a.train)]
        data = make_data(seeds, a.residual, a.max_cycles, log)
        report.update(train_seeds=[seeds[0], seeds[-1]], train_pairs=len(data), data_s=time.perf_counter() - t0,
                      symmetries=not a.no_symmetries,
                      target_rms=float(np.sqrt(np.mean([float((t.double() ** 2).mean()) for _, t in data]))))
        log(f"target rms {report['target_rms']:.3f} grid spacings")
        hist = train(net, data, a.minutes, lr=a.lr, log=log, symmetries=not a.no_symmetries)
        report.update(train_steps=hist[-1][0] if hist else 0, loss_first=hist[0][2] if hist else None,
                      loss_last=hist[-1][2] if hist else None)
        if a.out:
            save_weights(net.state_dict(), a.out)
    variants = [(int(s), int(q)) for s in a.smooth.split(",") for q in a.tta.split(",")] if a.eval > 0 else []
    key = lambda v: f"smooth{v[0]}" + (f"_tta{v[1]}" if v[1] > 1 else "")
    for sm, tt in variants:
        rows = evaluate(net, [EVAL_SEED0 + i for i in range(a.eval)], a.residual, a.max_cycles, log, smooth=sm,
                        tta=tt)
        report[key((sm, tt))] = dict(summary=summarize(rows), rows=rows)
        log(f"{key((sm, tt))}: " + json.dumps(report[key((sm, tt))]["summary"]))
    best = min(variants, key=lambda v: -(report[key(v)]["summary"]["speedup_total"] or 0)) if variants else (2, 1)
    if variants:
        report.update(best_variant=key(best), summary=report[key(best)]["summary"])
    if a.eval_batched:
        report["batched"] = evaluate_batched(net, [EVAL_SEED0 + a.eval + i for i in range(a.eval_batched)],
                                             a.residual, a.max_cycles, smooth=best[0], log=log)
        log("batched: " + json.dumps(report["batched"]["summary"]))
    if a.large:
        report["large"] = evaluate_large(net.state_dict(), a.large_residual or a.residual, a.large_attempts, log=log)
    log(json.dumps(report.get("summary")))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(report, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
