"""The tensor-core (tcgen05) MMA core of the warm-start network's kernels:
D = A . B^T with BF16 operands and FP32 accumulation in tensor memory, against
numpy on the same BF16-rounded inputs."""
import ctypes as C

import numpy as np
import pytest

from glemur_gb300 import _abi

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round float32 to bfloat16 (nearest even) and return the 16-bit patterns."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("N,K", [(16, 16), (32, 64), (48, 32), (96, 128), (128, 256)])
def test_tc_gemm(N, K):
    import torch
    rng = np.random.default_rng(N * 1000 + K)
    A = bf16_bits(rng.normal(size=(128, K)))
    B = bf16_bits(rng.normal(size=(N, K)))
    ref = bf16_value(A).astype(np.float64) @ bf16_value(B).astype(np.float64).T
    dA = torch.from_numpy(A.view(np.int16)).cuda()
    dB = torch.from_numpy(B.view(np.int16)).cuda()
    dD = torch.zeros((128, N), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = _abi.load()
    _abi.check(lib.gm_nn_tc_gemm_check(C.c_void_p(dA.data_ptr()), C.c_void_p(dB.data_ptr()),
                                       C.c_void_p(dD.data_ptr()), N, K, C.c_void_p(st.data_ptr())), "tc gemm")
    assert int(st.item()) == 0
    D = dD.cpu().numpy().astype(np.float64)
    err = np.abs(D - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def _shifted(x, di, dj, dk, xper, yper):
    """x[k][j][i] -> x at (i + di, j + dj, k + dk): periodic in x / y when asked,
    zero outside the grid otherwise (and always in z)."""
    nz, ny, nx = x.shape[:3]
    out = np.zeros_like(x)
    for k in range(nz):
        kk = k + dk
        if not 0 <= kk < nz:
            continue
        for j in range(ny):
            jj = j + dj
            if yper:
                jj %= ny
            elif not 0 <= jj < ny:
                continue
            ii = np.arange(nx) + di
            ok = np.ones(nx, bool) if xper else (ii >= 0) & (ii < nx)
            out[k, j, ok] = x[kk, jj, ii[ok] % nx]
    return out


# (nx, ny, nz, xper, yper, c1, c2 (second view), ci, co, vchunk): a partial last
# chunk, nx not a multiple of 8, one- and two-view inputs, the widest channels
WGRAD_CASES = [
    (8, 8, 16, 1, 1, 24, 0, 24, 24, 0),
    (8, 8, 16, 1, 1, 24, 0, 24, 24, 128),
    (12, 10, 6, 0, 1, 8, 0, 3, 3, 64),
    (8, 8, 8, 1, 0, 16, 40, 50, 48, 0),
    (16, 16, 8, 1, 1, 192, 48, 240, 48, 0),
    (16, 16, 8, 1, 1, 192, 0, 192, 192, 256),
    (8, 4, 8, 0, 0, 32, 0, 32, 256, 0),
]


@pytest.mark.parametrize("case", WGRAD_CASES)
def test_conv_wgrad(case):
    """dW[t][o][i] = sum_v dout[v][o] in[v + off(t)][i] against numpy (FP64 on
    the same BF16 values), added onto a non-zero dW."""
    import torch
    nx, ny, nz, xper, yper, c1, c2, ci, co, vchunk = case
    rng = np.random.default_rng(sum(case))
    V = nx * ny * nz
    ld1, ld2, ldd = c1 + 8, c2 + 16, (co + 7) // 8 * 8 + 8
    in1 = bf16_bits(rng.normal(size=(V, ld1)))
    in2 = bf16_bits(rng.normal(size=(V, max(ld2, 8))))
    dout = bf16_bits(rng.normal(size=(V, ldd)))
    dW0 = rng.normal(size=(27, co, ci)).astype(np.float32)
    x = np.concatenate([bf16_value(in1)[:, :c1], bf16_value(in2)[:, :c2]], 1)[:, :ci].astype(np.float64)
    x = x.reshape(nz, ny, nx, ci)
    g = bf16_value(dout)[:, :co].astype(np.float64)
    ref = dW0.astype(np.float64).copy()
    for t in range(27):
        xs = _shifted(x, t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1, xper, yper).reshape(V, ci)
        ref[t] += g.T @ xs
    d1 = torch.from_numpy(in1.view(np.int16)).cuda()
    d2 = torch.from_numpy(in2.view(np.int16)).cuda()
    dd = torch.from_numpy(dout.view(np.int16)).cuda()
    dW = torch.from_numpy(dW0).cuda()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = _abi.load()
    _abi.check(lib.gm_nn_conv_wgrad(C.c_void_p(dd.data_ptr()), ldd, co, C.c_void_p(d1.data_ptr()), ld1, c1,
                                    C.c_void_p(d2.data_ptr()) if c2 else None, ld2, c2,
                                    C.cast(dW.data_ptr(), C.POINTER(C.c_float)), ci, nx, ny, nz, xper, yper, vchunk,
                                    C.c_void_p(st.data_ptr()), None), "gm_nn_conv_wgrad")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    got = dW.cpu().numpy().astype(np.float64)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-5, (case, err)


def test_conv_wgrad_rejects_bad_arguments():
    """Argument checks that need no launch: channel counts, chunk, alignment."""
    import torch
    lib = _abi.load()
    buf = torch.zeros((64, 64), dtype=torch.int16, device="cuda")
    dW = torch.zeros(27 * 64 * 64, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    p, w = C.c_void_p(buf.data_ptr()), C.cast(dW.data_ptr(), C.POINTER(C.c_float))
    args = dict(ldd=64, co=16, ld1=64, c1=16, ci=16, vchunk=0)

    def call(**kw):
        a = {**args, **kw}
        return lib.gm_nn_conv_wgrad(p, a["ldd"], a["co"], p, a["ld1"], a["c1"], None, 0, 0, w, a["ci"], 4, 4, 4, 1, 1,
                                    a["vchunk"], C.c_void_p(st.data_ptr()), None)

    assert call(co=257) == _abi.GM_EPARAM
    assert call(ci=17) == _abi.GM_EPARAM          # more than the views hold
    assert call(vchunk=100) == _abi.GM_EPARAM     # not a multiple of 64
    assert call(ld1=60) == _abi.GM_EPARAM         # channel stride not a multiple of 8
    assert call(ldd=12) == _abi.GM_EPARAM
