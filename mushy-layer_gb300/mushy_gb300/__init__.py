"""GB300-native (sm_103a) elliptic/closure hot path of mushy-layer.

`abi` is the ctypes mirror of include/mlgpu.h, `ops` the reference-shaped
operator and solver classes over it, `build` compiles libmlgpu.so.
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
