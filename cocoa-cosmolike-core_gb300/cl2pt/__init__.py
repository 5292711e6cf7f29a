"""cl2pt -- GB300-native 2-point theory (Limber C_l, bin-averaged Legendre
sums, non-Limber FFTLog clustering, FAST-PT convolutions) behind a C ABI.

The compute path is libcl2pt.so (CUDA, sm_103a); this package is its host
side: ctypes bindings, synthetic workload generators and the build step.
"""
from . import abi, synthetic  # noqa: F401
from .lib import (DEVICE, HOST, PREC_FP64, PREC_MIXED, CL2PTError, Plan,  # noqa: F401
                  load)
