"""Learned warm start: a 3-D U-Net that maps the initial field B0 to a grid
displacement near the relaxed state, so the plain relaxation starts closer to
its end.  Every arithmetic step runs in this library's own kernels
(glemur_gb300/csrc/nn_kernels.cu): the 3x3x3 convolutions, their input and
weight gradients on the 5th-generation tensor cores (BF16 operands, FP32
accumulation in tensor memory), pooling, upsampling, the loss and Adam.
torch only allocates the buffers.

Network (3 levels, base width 24): two convolutions per level on the way
down (24, 48 and wb channels, 2x2x2 mean pooling between levels), nearest
upsampling and concatenation with the skip on the way up (48, 24 channels),
and a 3x3x3 head to 3 channels: the displacement in grid spacings.  The
bottleneck width wb is 192 for networks trained here (1.79 M parameters; 96
gives 0.80 M parameters); a weights file records it in the shapes of its
arrays.  Padding is periodic in x, y and zero in z.  The displacement of the
first and last z-planes is imposed to be zero, and a predicted grid whose
cells are not all positive (min Delta <= 0) is rejected in favour of the
identity grid.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from pathlib import Path

from . import _abi
from ._abi import check

WEIGHTS = Path(__file__).resolve().parent / "weights" / "unet_64x64x128.npz"

WB = 192   # bottleneck channels of a network trained here


def layers(wb=WB):
    """(name, input channels of the weights, output channels, ReLU) per layer."""
    return [("e0a", 3, 24, True), ("e0b", 24, 24, True), ("e1a", 24, 48, True), ("e1b", 48, 48, True),
            ("ba", 48, wb, True), ("bb", wb, wb, True), ("d1a", wb + 48, 48, True), ("d1b", 48, 48, True),
            ("d0a", 72, 24, True), ("d0b", 24, 24, True), ("head", 24, 3, False)]


LAYERS = layers()


def view_in(wb=WB):
    """Channels of the buffer view each layer reads (the input is stored with 8 channels)."""
    return {"e0a": 8, "d1a": wb + 48, "d0a": 72}


def r16(n):
    return (n + 15) // 16 * 16


def r8(n):
    return (n + 7) // 8 * 8


def n_params(wb=WB):
    return sum(27 * ci * co + co for _, ci, co, _ in layers(wb))


def weights_width(d):
    """Bottleneck width of a weights dictionary (load_weights)."""
    return int(d["bb.W"].shape[1])


def bf16_bits(a):
    """float32 -> BF16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def save_weights(state, path):
    """Weights as BF16 bit patterns, the precision the network computes with."""
    np.savez(path, **{k: bf16_bits(v) for k, v in state.items()})


def load_weights(path=None):
    """Weights saved by save_weights (BF16 bits, widened to float32) or as float32."""
    d = np.load(path or WEIGHTS)
    return {k: (d[k].astype(np.uint32) << 16).view(np.float32) if d[k].dtype == np.uint16 else d[k].astype(np.float32)
            for k in d.files}


class _Layer:
    def __init__(self, name, ci, co, relu, rng, torch, dev, view):
        self.name, self.ci, self.co, self.relu = name, ci, co, relu
        self.view = view
        self.kin, self.npo = r16(self.view), r16(co)          # forward conv: K, padded outputs
        self.kco, self.npi = r16(co), r16(self.view)          # input-gradient conv
        f32 = dict(dtype=torch.float32, device=dev)
        std = math.sqrt(2.0 / (27 * ci)) if relu else math.sqrt(1.0 / (27 * ci))
        self.W = torch.from_numpy(rng.normal(0.0, std, (27, co, ci)).astype(np.float32)).to(dev)
        self.b = torch.zeros(co, **f32)
        self.mW, self.vW, self.gW = (torch.zeros_like(self.W) for _ in range(3))
        self.mb, self.vb, self.gb = (torch.zeros_like(self.b) for _ in range(3))
        self.Wf = torch.zeros((27, self.npo, self.kin), dtype=torch.bfloat16, device=dev)
        self.Wb = torch.zeros((27, self.npi, self.kco), dtype=torch.bfloat16, device=dev)
        self.bpad = torch.zeros(self.npo, **f32)


class UNet:
    """The network on one grid shape (nx, ny, nz divisible by 4)."""

    def __init__(self, shape, seed=0, xper=True, yper=True, device="cuda", wb=WB):
        import torch
        self.torch = torch
        self.lib = _abi.load()
        nx, ny, nz = shape
        if nx % 4 or ny % 4 or nz % 4:
            raise ValueError("grid sizes must be divisible by 4")
        self.shape = (nx, ny, nz)
        self.xper, self.yper = int(xper), int(yper)
        self.dev = device
        rng = np.random.default_rng(seed)
        self.wb = wb
        vin = view_in(wb)
        self.layers = {n: _Layer(n, ci, co, r, rng, torch, device, vin.get(n, ci)) for n, ci, co, r in layers(wb)}
        self.V = [nx * ny * nz, nx * ny * nz // 8, nx * ny * nz // 64]
        self.dims = [(nx, ny, nz), (nx // 2, ny // 2, nz // 2), (nx // 4, ny // 4, nz // 4)]
        bf = dict(dtype=torch.bfloat16, device=device)
        A = {}
        for name, lvl, ch in [("X0", 0, 8), ("E0a", 0, 24), ("CAT0", 0, 72), ("P1", 1, 24), ("E1a", 1, 48),
                              ("CAT1", 1, wb + 48), ("P2", 2, 48), ("Ba", 2, wb), ("Bb", 2, wb), ("D1a", 1, 48),
                              ("D1b", 1, 48), ("D0a", 0, 24), ("D0b", 0, 24), ("Y", 0, 8),
                              ("dY", 0, 8), ("dD0b", 0, 24), ("dD0a", 0, 24), ("dCAT0", 0, 72), ("dD1b", 1, 48),
                              ("dD1a", 1, 48), ("dCAT1", 1, wb + 48), ("dBb", 2, wb), ("dBa", 2, wb), ("dP2", 2, 48),
                              ("dE1a", 1, 48), ("dP1", 1, 24), ("dE0a", 0, 24)]:
            A[name] = torch.zeros((self.V[lvl], ch), **bf)
        self.A = A
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.loss_acc = torch.zeros(1, dtype=torch.float32, device=device)
        self.stream = torch.cuda.current_stream().cuda_stream
        self.t = 0
        self.refresh_weights()

    # -- views: (pointer, channel stride) of a buffer from channel offset c0 ----
    def v(self, name, c0=0):
        t = self.A[name]
        return C.c_void_p(t.data_ptr() + 2 * c0), t.shape[1]

    def _conv(self, L, src, out, co, lvl, relu, mask=None, backward=False, src_c=None):
        (p1, l1) = src
        nx, ny, nz = self.dims[lvl]
        W = L.Wb if backward else L.Wf
        Kc = L.kco if backward else L.kin
        Np = L.npi if backward else L.npo
        c1 = src_c if src_c is not None else (r8(L.co) if backward else L.view)
        mp, ml = (mask if mask is not None else (None, 0))
        check(self.lib.gm_nn_conv(p1, l1, c1, None, 0, 0, C.c_void_p(W.data_ptr()),
                                  None if backward else C.cast(L.bpad.data_ptr(), C.POINTER(C.c_float)),
                                  out[0], out[1], co, mp, ml, 1 if relu else 0, nx, ny, nz, self.xper, self.yper,
                                  Kc, Np, C.c_void_p(self.status.data_ptr()), C.c_void_p(self.stream)), "gm_nn_conv")

    def _wgrad(self, L, dout, src, lvl):
        nx, ny, nz = self.dims[lvl]
        check(self.lib.gm_nn_conv_wgrad(dout[0], dout[1], L.co, src[0], src[1], L.view, None, 0, 0,
                                        C.cast(L.gW.data_ptr(), C.POINTER(C.c_float)), L.ci, nx, ny, nz, self.xper,
                                        self.yper, 0, C.c_void_p(self.status.data_ptr()), C.c_void_p(self.stream)),
              "gm_nn_conv_wgrad")
        check(self.lib.gm_nn_bias_grad(dout[0], dout[1], L.co, self.V[lvl],
                                       C.cast(L.gb.data_ptr(), C.POINTER(C.c_float)), C.c_void_p(self.stream)),
              "gm_nn_bias_grad")

    def _pool(self, src, dst, c, lvl, backward=False, accumulate=False):
        nx, ny, nz = self.dims[lvl]          # the fine grid
        check(self.lib.gm_nn_pool(src[0], src[1], dst[0], dst[1], c, nx, ny, nz, int(backward), int(accumulate),
                                  C.c_void_p(self.stream)), "gm_nn_pool")

    def _up(self, src, dst, c, lvl, backward=False):
        nx, ny, nz = self.dims[lvl]          # the fine grid
        check(self.lib.gm_nn_upsample(src[0], src[1], dst[0], dst[1], c, nx, ny, nz, int(backward),
                                      C.c_void_p(self.stream)), "gm_nn_upsample")

    def _relu_bwd(self, d, y, c, lvl):
        check(self.lib.gm_nn_relu_bwd(d[0], d[1], y[0], y[1], c, self.V[lvl], C.c_void_p(self.stream)),
              "gm_nn_relu_bwd")

    # -- the network ----------------------------------------------------------
    def set_input_b0(self, B0_dev, precision, shift=(0, 0), sym=0):
        """B0: device array of the reference layout (ghosted AoS, REAL), read
        translated by `shift` whole cells in x and y (periodic) and moved by
        the mirror / swap symmetry `sym` (bits of gm_nn_input)."""
        nx, ny, nz = self.shape
        check(self.lib.gm_nn_input(C.c_void_p(B0_dev.data_ptr()), precision, nx, ny, nz,
                                   self.v("X0")[0], 8, shift[0], shift[1], sym, C.c_void_p(self.stream)),
              "gm_nn_input")

    def forward(self):
        Ls, v = self.layers, self.v
        self._conv(Ls["e0a"], v("X0"), v("E0a"), 24, 0, True)
        self._conv(Ls["e0b"], v("E0a"), v("CAT0", 48), 24, 0, True)
        self._pool(v("CAT0", 48), v("P1"), 24, 0)
        self._conv(Ls["e1a"], v("P1"), v("E1a"), 48, 1, True)
        wb = self.wb
        self._conv(Ls["e1b"], v("E1a"), v("CAT1", wb), 48, 1, True)
        self._pool(v("CAT1", wb), v("P2"), 48, 1)
        self._conv(Ls["ba"], v("P2"), v("Ba"), wb, 2, True)
        self._conv(Ls["bb"], v("Ba"), v("Bb"), wb, 2, True)
        self._up(v("Bb"), v("CAT1"), wb, 1)
        self._conv(Ls["d1a"], v("CAT1"), v("D1a"), 48, 1, True)
        self._conv(Ls["d1b"], v("D1a"), v("D1b"), 48, 1, True)
        self._up(v("D1b"), v("CAT0"), 48, 0)
        self._conv(Ls["d0a"], v("CAT0"), v("D0a"), 24, 0, True)
        self._conv(Ls["d0b"], v("D0a"), v("D0b"), 24, 0, True)
        self._conv(Ls["head"], v("D0b"), v("Y"), 3, 0, False)
        return self.A["Y"]

    def zero_grad(self):
        for L in self.layers.values():
            for t in (L.gW, L.gb):
                check(self.lib.gm_nn_zero(C.c_void_p(t.data_ptr()), t.numel() * 4, C.c_void_p(self.stream)), "zero")
        check(self.lib.gm_nn_zero(C.c_void_p(self.loss_acc.data_ptr()), 4, C.c_void_p(self.stream)), "zero")

    def backward(self, target, scale, shift=(0, 0), sym=0):
        """Loss scale * sum (y - target)^2 (planes 1..nz-2, 3 channels) and the
        accumulation of every weight gradient; target: float32 [V][3] on the
        device, moved by `shift` and `sym` as the input was."""
        Ls, v = self.layers, self.v
        nx, ny, nz = self.shape
        check(self.lib.gm_nn_mse(v("Y")[0], 8, C.cast(target.data_ptr(), C.POINTER(C.c_float)), v("dY")[0], 8,
                                 nx, ny, nz, C.c_float(scale), C.cast(self.loss_acc.data_ptr(), C.POINTER(C.c_float)),
                                 shift[0], shift[1], sym, C.c_void_p(self.stream)), "gm_nn_mse")
        L = Ls["head"]
        self._wgrad(L, v("dY"), v("D0b"), 0)
        self._conv(L, v("dY"), v("dD0b"), 24, 0, False, mask=v("D0b"), backward=True, src_c=8)
        L = Ls["d0b"]
        self._wgrad(L, v("dD0b"), v("D0a"), 0)
        self._conv(L, v("dD0b"), v("dD0a"), 24, 0, False, mask=v("D0a"), backward=True)
        L = Ls["d0a"]
        self._wgrad(L, v("dD0a"), v("CAT0"), 0)
        self._conv(L, v("dD0a"), v("dCAT0"), 72, 0, False, backward=True)
        self._up(v("dCAT0"), v("dD1b"), 48, 0, backward=True)
        self._relu_bwd(v("dD1b"), v("D1b"), 48, 1)
        L = Ls["d1b"]
        self._wgrad(L, v("dD1b"), v("D1a"), 1)
        self._conv(L, v("dD1b"), v("dD1a"), 48, 1, False, mask=v("D1a"), backward=True)
        L = Ls["d1a"]
        self._wgrad(L, v("dD1a"), v("CAT1"), 1)
        wb = self.wb
        self._conv(L, v("dD1a"), v("dCAT1"), wb + 48, 1, False, backward=True)
        self._up(v("dCAT1"), v("dBb"), wb, 1, backward=True)
        self._relu_bwd(v("dBb"), v("Bb"), wb, 2)
        L = Ls["bb"]
        self._wgrad(L, v("dBb"), v("Ba"), 2)
        self._conv(L, v("dBb"), v("dBa"), wb, 2, False, mask=v("Ba"), backward=True)
        L = Ls["ba"]
        self._wgrad(L, v("dBa"), v("P2"), 2)
        self._conv(L, v("dBa"), v("dP2"), 48, 2, False, backward=True)
        self._pool(v("dP2"), v("dCAT1", wb), 48, 1, backward=True, accumulate=True)
        self._relu_bwd(v("dCAT1", wb), v("CAT1", wb), 48, 1)
        L = Ls["e1b"]
        self._wgrad(L, v("dCAT1", wb), v("E1a"), 1)
        self._conv(L, v("dCAT1", wb), v("dE1a"), 48, 1, False, mask=v("E1a"), backward=True)
        L = Ls["e1a"]
        self._wgrad(L, v("dE1a"), v("P1"), 1)
        self._conv(L, v("dE1a"), v("dP1"), 24, 1, False, backward=True)
        self._pool(v("dP1"), v("dCAT0", 48), 24, 0, backward=True, accumulate=True)
        self._relu_bwd(v("dCAT0", 48), v("CAT0", 48), 24, 0)
        L = Ls["e0b"]
        self._wgrad(L, v("dCAT0", 48), v("E0a"), 0)
        self._conv(L, v("dCAT0", 48), v("dE0a"), 24, 0, False, mask=v("E0a"), backward=True)
        L = Ls["e0a"]
        self._wgrad(L, v("dE0a"), v("X0"), 0)

    def refresh_weights(self, lr=0.0, b1=0.9, b2=0.999, eps=1e-8, step=False):
        """Adam step (step=True) and the BF16 operand layouts of every layer."""
        if step:
            self.t += 1
        for L in self.layers.values():
            P = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_float))
            check(self.lib.gm_nn_adam(P(L.W), P(L.mW), P(L.vW), P(L.gW), P(L.b), P(L.mb), P(L.vb), P(L.gb), L.co,
                                      L.ci, C.c_float(lr), C.c_float(b1), C.c_float(b2), self.t if step else 0,
                                      C.c_float(eps), C.c_void_p(L.Wf.data_ptr()), L.npo, L.kin,
                                      C.c_void_p(L.Wb.data_ptr()), L.npi, L.kco, P(L.bpad),
                                      C.c_void_p(self.stream)), "gm_nn_adam")

    def params_numpy(self):
        return {n: (L.W.cpu().numpy().astype(np.float64), L.b.cpu().numpy().astype(np.float64))
                for n, L in self.layers.items()}

    def grads_numpy(self):
        return {n: (L.gW.cpu().numpy().astype(np.float64), L.gb.cpu().numpy().astype(np.float64))
                for n, L in self.layers.items()}

    def state_dict(self):
        return {f"{n}.{k}": getattr(L, k).cpu().numpy() for n, L in self.layers.items() for k in ("W", "b")}

    def load_state_dict(self, d):
        for n, L in self.layers.items():
            L.W.copy_(self.torch.from_numpy(d[f"{n}.W"]))
            L.b.copy_(self.torch.from_numpy(d[f"{n}.b"]))
        self.refresh_weights()

    def check_status(self):
        if int(self.status.item()) != 0:
            raise _abi.GlemurError("a tensor-core completion wait gave up (status set)")


def time_passes(shape=(64, 64, 128), wb=WB, reps=10, seed=1):
    """Mean wall time (CUDA events) of a forward pass and of a forward +
    backward pass of the network on random inputs, after three warm-up
    passes; then one more forward + backward inside cudaProfilerStart/Stop,
    so that a profiler started with profiling off captures exactly that pass."""
    import torch
    nx, ny, nz = shape
    net = UNet(shape, seed=seed, wb=wb)
    rng = np.random.default_rng(seed)
    X0 = np.zeros((nx * ny * nz, 8), np.float32)
    X0[:, :3] = rng.normal(size=(nx * ny * nz, 3))
    net.A["X0"].copy_(torch.from_numpy(X0).to(torch.bfloat16))
    tgt = torch.from_numpy(rng.normal(size=(nx * ny * nz, 3)).astype(np.float32)).cuda()
    scale = 1.0 / (nx * ny * nz * 3)

    def fb():
        net.zero_grad()
        net.forward()
        net.backward(tgt, scale)

    for _ in range(3):
        fb()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, fn in (("forward_backward_ms", fb), ("forward_ms", net.forward)):
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
    net.check_status()
    torch.cuda.profiler.start()
    fb()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time the warm-start network's passes on random inputs")
    ap.add_argument("--shape", default="64,64,128")
    ap.add_argument("--wb", type=int, default=WB)
    a = ap.parse_args()
    print(json.dumps(time_passes(tuple(int(v) for v in a.shape.split(",")), a.wb)))
