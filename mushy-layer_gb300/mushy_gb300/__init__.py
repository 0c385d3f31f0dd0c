"""GB300-native (sm_103a) elliptic/closure hot path of mushy-layer.

`abi` is the ctypes mirror of include/mlgpu.h, `ops` the reference-shaped
operator and solver classes over it, `build` compiles libmlgpu.so,
`adjoint` the torch.autograd bindings of the discrete adjoint (with segment
and binomial checkpointing), `darcy_model` the differentiable solidification
model the adjoint is measured on, `chombo_hdf5` the plotfile and checkpoint reader,
`inputs` the reader of the reference's inputs files (parameters, walls, solver
settings).
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
