"""GB300-native (sm_103a) flow-step hot path of SophT.

Drop-in counterparts of the reference's flow simulators, immersed-body
interactions and Eulerian/immersed-boundary operators, backed by the
hand-written CUDA kernels of ``libsopht_gb300.so`` (C ABI in
``include/sopht_gb300.h``).  Fields are CUDA tensors; there is no CPU
fallback: operators raise if the library is missing.
"""

import logging

from . import numeric, simulator, utils

logging.getLogger(__name__).addHandler(logging.NullHandler())

__all__ = ["numeric", "simulator", "utils"]
__version__ = "0.1.0"
