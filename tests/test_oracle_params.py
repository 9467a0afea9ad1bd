"""The checker's own parameter builder (oracle/params.py) against the
library's (glemur_gb300.configs): the same bytes for every workload the
bench's reference arm runs, and the same struct layout."""
import ctypes as C

import pytest

from glemur_gb300 import configs
from glemur_gb300._abi import GmParams
from oracle import params as op


def test_layout_matches_library_mirror():
    assert C.sizeof(op.Params) == C.sizeof(GmParams)
    a = [(n, getattr(GmParams, n).offset, getattr(GmParams, n).size) for n, _ in GmParams._fields_]
    b = [(n, getattr(op.Params, n).offset, getattr(op.Params, n).size) for n, _ in op.Params._fields_]
    assert a == b


@pytest.mark.parametrize("precision", [32, 64])
def test_defaults_match_library(precision):
    assert bytes(op.defaults(precision)) == bytes(configs.defaults(precision))


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("which", ["braid6", "braid6_large"])
def test_workloads_match_library(which, precision):
    shape = (24, 20, 40)
    assert bytes(getattr(op, which)(*shape, precision=precision)) == \
        bytes(getattr(configs, which)(*shape, precision=precision))


def test_oracle_initial_state_from_checker_params():
    """orc_init_state on the checker's parameters equals gm_init_state on the
    library's."""
    import numpy as np
    from oracle.pyoracle import Oracle
    p = op.braid6(12, 10, 16, precision=32)
    B0, xb = Oracle.init_state(p)
    B0l, xbl = configs.init_state(configs.braid6(12, 10, 16, precision=32))
    assert np.array_equal(B0, B0l) and np.array_equal(xb, xbl)
