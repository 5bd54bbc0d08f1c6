"""ctypes binding of the CUDA C-ABI library ``lib/libvoxelproj_gb300.so``.

The signatures mirror ``include/voxelproj_gb300.h``.  There is no fallback:
if the library is missing, importing the package fails with instructions to
build it.
"""

from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libvoxelproj_gb300.so"

VP_OK = 0
VP_ERR_NULL_POINTER = 1
VP_ERR_BAD_SHAPE = 2
VP_ERR_ANGLES = 3
VP_ERR_CUDA = 4
VP_ERR_BAD_FLAGS = 5
VP_ERR_BAD_Z_ORDER = 6
VP_ERR_WORKSPACE = 7
VP_ERR_SCRATCH_LIMIT = 8
VP_ERR_BATCH = 9
VP_OP_FORWARD = 0
VP_OP_BACKWARD = 1


class BatchProblem(ctypes.Structure):
    """Mirror of vp_batch_problem (include/voxelproj_gb300.h)."""

    _fields_ = [
        ("op", ctypes.c_int),
        ("flags", ctypes.c_int),
        ("variant", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("in_", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("angles", ctypes.c_void_p),
        ("n_angles", ctypes.c_int64),
        ("in_dims", ctypes.c_int64 * 3),
        ("out_dims", ctypes.c_int64 * 3),
    ]
VP_NOALLOC_SCRATCH_BYTES = 64 << 20

VP_FLAG_TRIG_PRECISE = 1
VP_FLAG_OVERWRITE = 2

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I = ctypes.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    "vp_version": (_I, []),
    "vp_error_string": (ctypes.c_char_p, [_I]),
    "vp_last_cuda_error": (_I, []),
    "vp_launch_count": (ctypes.c_uint64, []),
    "vp_wait_timeouts": (ctypes.c_uint64, []),
    "vp_set_wait_limits": (_I, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]),
    "vp_set_kernel_variant": (_I, [_I, _I]),
    "vp_get_kernel_variant": (_I, [_I]),
    "vp_forward_z0": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_backward_z0": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_forward_z2": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_backward_z2": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_z2_workspace_bytes": (ctypes.c_size_t, [_I64, _I64, _I64, _I64, _I64, _I64]),
    "vp_forward_z2_ws": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P,
                              ctypes.c_size_t, _P]),
    "vp_backward_z2_ws": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P,
                               ctypes.c_size_t, _P]),
    "vp_forward_z2_noalloc": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I,
                                   _P]),
    "vp_batch_create": (_I, [_P, _I, _P]),
    "vp_batch_update": (_I, [_P, _P, _I, _P]),
    "vp_batch_run": (_I, [_P, _P]),
    "vp_batch_work_items": (_I64, [_P]),
    "vp_batch_error": (_I, [_P, _P]),
    "vp_batch_destroy": (_I, [_P]),
    "vp_forward_z0_host": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_backward_z0_host": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_forward_z2_host": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_backward_z2_host": (_I, [_P, _I64, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I, _P]),
    "vp_forward": (_I, [_P, _P, _P, _P, _P, _I64, _I, _I, _P]),
    "vp_backward": (_I, [_P, _P, _P, _P, _P, _I64, _I, _I, _P]),
}


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"voxelproj_gb300: native library {LIB_PATH} is missing; build it with "
            "`python voxelproj_gb300/build.py` (needs nvcc)")
    L = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


LIB = _load()


def error_text(status: int) -> str:
    msg = LIB.vp_error_string(status).decode()
    if status == VP_ERR_CUDA:
        msg += f" (cudaError {LIB.vp_last_cuda_error()})"
    return msg


def check(status: int, what: str) -> None:
    if status != VP_OK:
        raise RuntimeError(f"voxelproj_gb300.{what}: {error_text(status)}")
