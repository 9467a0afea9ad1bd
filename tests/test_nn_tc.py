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
