"""voxelproj_gb300 — exact-trapezoid parallel-beam projector pair (A, A^T)
for NVIDIA GB300 (sm_103a), a drop-in for the ``voxelproj`` package:

    import voxelproj_gb300 as voxelproj
    y = voxelproj.forward(x, angles, None)              # A x
    x = voxelproj.backward(y, angles, None)             # A^T y

The compute runs in hand-written CUDA kernels behind the C ABI declared in
``include/voxelproj_gb300.h``; ``voxelproj_gb300._CU`` exposes the
reference's extension functions on top of it.
"""

import torch  # noqa: F401  (loads the CUDA runtime used for tensors and streams)

from . import _CU
from ._CU import get_trig_mode, set_trig_mode
from .wrappers import backward, forward

__all__ = ["forward", "backward", "set_trig_mode", "get_trig_mode", "_CU"]
__version__ = "0.1.0"
