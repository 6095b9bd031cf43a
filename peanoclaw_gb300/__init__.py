"""GB300-native SWE patch-update path behind PeanoClaw's Numerics interface.

libpcg.so (CUDA, sm_103a) holds the kernels and the C ABI declared in
include/pcg.h; `pcg` binds it with ctypes, `numerics` mirrors
peanoclaw::Numerics / SWEKernel, `scenarios` builds the synthetic workloads.
"""
from . import pcg  # noqa: F401
