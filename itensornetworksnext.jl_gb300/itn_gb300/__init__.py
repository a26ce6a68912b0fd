"""itn_gb300 -- GB300-native belief propagation and network contraction for
ITensorNetworksNext.jl's hot path.

Layers:
* ``_lib``       ctypes binding of libitn_gpu.so (C ABI, include/itn_gpu.h)
* ``engine``     array-level engine (CSR network, packed tensors/messages on the GPU)
* ``graphs``     CSR network description + seeded synthetic generators
* ``generators`` known-answer single-layer networks (Ising, spin ice, deltas)
"""
from . import graphs, generators, contract  # noqa: F401
from .contract import contract_network, contraction_order  # noqa: F401
from ._lib import ItnError, ItnArgumentError, load as load_library  # noqa: F401
from .engine import BPEngine, RunResult  # noqa: F401
from . import network  # noqa: F401

__all__ = ["graphs", "generators", "contract", "contract_network", "contraction_order", "BPEngine", "RunResult", "ItnError", "ItnArgumentError",
           "load_library", "network"]
