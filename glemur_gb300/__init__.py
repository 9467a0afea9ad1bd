"""glemur_gb300 -- GB300-native magneto-frictional relaxation (the GLEMuR hot
path) behind the C-ABI of include/glemur.h.

    from glemur_gb300 import configs, Relaxation
    p = configs.braid2()                    # run parameters (params.in semantics)
    B0, xb = configs.init_state(p)          # initial field and grid
    r = Relaxation(p); r.upload(xb, B0)
    r.run(p.nCycle); red = r.refresh()      # relax, then B, J and reductions
"""
from ._abi import GlemurError, GmParams, load  # noqa: F401
from .relax import Relaxation  # noqa: F401
from .batch import BatchRelaxation  # noqa: F401
from . import configs  # noqa: F401

__all__ = ["Relaxation", "BatchRelaxation", "GmParams", "GlemurError", "configs", "load"]
