"""GB300-native (sm_103a) DQMC sweep hot path for carstenbauer/dqmc's O(3) model.

The product is the CUDA shared library `libdqmc_gpu.so` with the C ABI of
`include/dqmc_gpu.h`; `dqmc_gb300.api` is its Python (ctypes) host binding.
"""
from .api import DQMC, DQMCError, ModelParams, load_library  # noqa: F401
