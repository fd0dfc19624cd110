"""GB300 implementation of MGLET-base's Runge-Kutta stage (host side).

The compute path is the CUDA library libmglet_gpu.so (sm_103a) behind the
C ABI of include/mglet_gpu.h; this package holds its ctypes binding, the
case generator and the build recipe.
"""
from . import abi, cases  # noqa: F401
