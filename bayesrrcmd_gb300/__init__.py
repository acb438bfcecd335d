"""GB300-native (sm_103a) BayesR Gibbs-sweep path of BayesRRcmd.

The compute runs in libbrr_gpu.so (hand-written CUDA behind the C ABI of
include/brr_gpu.h); this package holds its build recipe, a ctypes binding and
PLINK helpers.
"""
from . import plink  # noqa: F401

__all__ = ["plink", "gpu", "build"]
