"""GB300-native picFoam particle hot path.

The compute path is libpicgpu.so (hand-written CUDA for sm_103a behind the C
ABI in include/picgpu.h); this package holds the host-side mirror of the
picFoam cloud interface (Simulation), the case builders and the build recipe.
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
