"""The allocation-free reduction entry point, gm_reduce_noalloc.

Callers that cannot allocate device memory where they want diagnostics
(applications whose device memory belongs to their own pool allocator,
stream pipelines that must not stall on cudaMalloc/cudaFree, services that
allocate nothing after start-up) pass fields they already hold; the entry
point keeps its partial sums in a fixed device array.  Checked through the C-ABI
against gm_refresh on the same state, on two calls in a row."""
import ctypes as C

import numpy as np
import pytest

from glemur_gb300 import Relaxation, _abi, configs
from glemur_gb300._abi import GmReduction

pytestmark = pytest.mark.gpu

FIELDS = ("B2", "BMax", "JMax", "JxB_B2Max", "residual", "residualPw", "minDetJac", "errB_1ez")


@pytest.mark.parametrize("precision,peri", [(64, (1, 1, 0)), (32, (1, 1, 0)), (64, (0, 0, 0))])
def test_reduce_noalloc_matches_refresh(precision, peri):
    import torch
    p = configs.braid2(17, 13, 19, precision=precision)
    p.xPeri, p.yPeri, p.zPeri = peri
    p = configs.derive(p)
    B0, xb = configs.init_state(p)
    g = Relaxation(p)
    g.upload(xb, B0)
    g.run(8)
    ref = g.refresh()
    f = g.download()
    dev = torch.device("cuda")
    Bd = torch.from_numpy(f["B"]).to(dev)
    Jd = torch.from_numpy(f["J"]).to(dev)
    Dd = torch.from_numpy(f["detJac"]).to(dev)
    out = torch.zeros(C.sizeof(GmReduction) // 8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    lib = _abi.load()
    results = []
    for _ in range(2):
        out.fill_(-1.0)
        _abi.check(lib.gm_reduce_noalloc(p, C.c_void_p(Bd.data_ptr()), C.c_void_p(Jd.data_ptr()),
                                         C.c_void_p(Dd.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(stream)),
                   "gm_reduce_noalloc")
        torch.cuda.synchronize()
        r = GmReduction.from_buffer_copy(out.cpu().numpy().tobytes()).as_dict()
        results.append(r)
    tol = 1e-12 if precision == 64 else 1e-5
    for r in results:
        for k in FIELDS:
            assert abs(r[k] - ref[k]) <= tol * max(abs(ref[k]), 1e-300), (k, r[k], ref[k])
        assert np.isnan(r["wedgeMin"]) and np.isnan(r["convex"])
    assert results[0] == {k: v for k, v in results[1].items()} or all(
        (np.isnan(results[0][k]) and np.isnan(results[1][k])) or results[0][k] == results[1][k] for k in results[0])
    g.close()


def test_reduce_noalloc_rejects_too_many_planes():
    p = configs.braid2(4, 4, 8, precision=64)
    p.nz = 4097
    lib = _abi.load()
    rc = lib.gm_reduce_noalloc(p, C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), None)
    assert rc == -1
    assert b"exceeds the scratch limit" in lib.gm_last_error()
