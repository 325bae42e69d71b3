"""GB300-native engine for monofonIC's initial-condition hot path.

The compute path is libmfx.so (hand-written sm_103a CUDA kernels + cuFFT
behind the C ABI of include/mfx.h); ``monofonic_gb300.mfx`` is its ctypes
binding.
"""
from . import build  # noqa: F401
