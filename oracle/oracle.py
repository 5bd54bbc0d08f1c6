"""TEST INFRASTRUCTURE ONLY — the oracle.

ctypes binding of ``vp_oracle.c``, the CPU restatement of the reference
voxelproj projector pair (FP64 accuracy reference + FP32/OpenMP CPU baseline).
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module; the ``voxelproj_gb300`` package never does.

Array conventions follow the reference (voxelproj/wrappers.py:36-39):
    z_order 0: x (SY, SX, H), y (n_ang, PX, H)
    z_order 2: x (H, SY, SX), y (H, n_ang, PX)
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "vp_oracle.c"
LIB = HERE / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compiles vp_oracle.c with gcc + OpenMP into liboracle.so (in place)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-fvisibility=hidden",
           str(SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.vpo_forward_f64.argtypes = [P, I, I, I, I, P, I, I, P, I, P]
        L.vpo_backward_f64.argtypes = [P, I, I, I, I, P, I, I, P, I, P]
        L.vpo_forward_f32.argtypes = [P, P, I, I, I, I, I, I, P, I, I]
        L.vpo_backward_f32.argtypes = [P, P, I, I, I, I, I, I, P, I, I]
        L.vpo_angle_params_f64.argtypes = [ctypes.c_float, P]
        L.vpo_weights_f64.argtypes = [ctypes.c_float, ctypes.c_double, P]
        L.vpo_weights_f64.restype = I
        L.vpo_max_threads.restype = I
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _hlist(h_list, H):
    if h_list is None:
        return None, H
    hl = np.ascontiguousarray(np.asarray(h_list, dtype=np.int32))
    if hl.size and (hl.min() < 0 or hl.max() >= H):
        raise ValueError("height index out of range")
    return hl, int(hl.size)


def max_threads() -> int:
    return int(lib().vpo_max_threads())


def angle_params(phi: float) -> dict:
    out = np.zeros(5, np.float64)
    lib().vpo_angle_params_f64(ctypes.c_float(phi), _ptr(out))
    return dict(c=out[0], s=out[1], a=out[2], b=out[3], ymax=out[4])


def weights(phi: float, xp: float):
    w = np.zeros(3, np.float64)
    r = lib().vpo_weights_f64(ctypes.c_float(phi), ctypes.c_double(xp), _ptr(w))
    return int(r), w


def forward_f64(x, angles, PX: int, z_order: int = 0, h_list=None) -> np.ndarray:
    """A x in FP64 for the listed heights; returns (n_h, n_ang, PX) float64."""
    x = _f32(x)
    ang = _f32(angles).ravel()
    if z_order == 0:
        SY, SX, H = x.shape
    elif z_order == 2:
        H, SY, SX = x.shape
    else:
        raise KeyError(z_order)
    hl, n_h = _hlist(h_list, H)
    out = np.zeros((n_h, ang.size, PX), np.float64)
    lib().vpo_forward_f64(_ptr(x), z_order, SY, SX, H, _ptr(ang), ang.size, PX,
                          None if hl is None else _ptr(hl), n_h, _ptr(out))
    return out


def backward_f64(y, angles, SY: int, SX: int, z_order: int = 0, h_list=None) -> np.ndarray:
    """A^T y in FP64 for the listed heights; returns (n_h, SY, SX) float64."""
    y = _f32(y)
    ang = _f32(angles).ravel()
    if z_order == 0:
        n_ang, PX, H = y.shape
    elif z_order == 2:
        H, n_ang, PX = y.shape
    else:
        raise KeyError(z_order)
    if ang.size < n_ang:
        raise ValueError("fewer angles than the sinogram's angle extent")
    hl, n_h = _hlist(h_list, H)
    out = np.zeros((n_h, SY, SX), np.float64)
    lib().vpo_backward_f64(_ptr(y), z_order, n_ang, PX, H, _ptr(ang), SY, SX,
                           None if hl is None else _ptr(hl), n_h, _ptr(out))
    return out


def y_to_layout(compact: np.ndarray, z_order: int) -> np.ndarray:
    """(n_h, n_ang, PX) -> the z_order layout of y."""
    return np.ascontiguousarray(compact.transpose(1, 2, 0)) if z_order == 0 else compact


def x_to_layout(compact: np.ndarray, z_order: int) -> np.ndarray:
    """(n_h, SY, SX) -> the z_order layout of x."""
    return np.ascontiguousarray(compact.transpose(1, 2, 0)) if z_order == 0 else compact


def forward(x, angles, PX: int, z_order: int = 0) -> np.ndarray:
    """A x in FP64, laid out like y for this z_order."""
    return y_to_layout(forward_f64(x, angles, PX, z_order), z_order)


def backward(y, angles, SY: int, SX: int, z_order: int = 0) -> np.ndarray:
    """A^T y in FP64, laid out like x for this z_order."""
    return x_to_layout(backward_f64(y, angles, SY, SX, z_order), z_order)


def forward_f32_(x: np.ndarray, y: np.ndarray, angles, z_order: int = 0, a_lo: int = 0,
                 a_hi: int | None = None) -> None:
    """y += A x in float, in place (CPU baseline); angles [a_lo, a_hi) only."""
    ang = _f32(angles).ravel()
    assert x.dtype == np.float32 and y.dtype == np.float32
    assert x.flags.c_contiguous and y.flags.c_contiguous
    if z_order == 0:
        SY, SX, H = x.shape
        n_ang, PX, Hy = y.shape
    else:
        H, SY, SX = x.shape
        Hy, n_ang, PX = y.shape
    assert H == Hy and ang.size >= n_ang
    a_hi = n_ang if a_hi is None else a_hi
    lib().vpo_forward_f32(_ptr(x), _ptr(y), z_order, SY, SX, n_ang, PX, H, _ptr(ang), a_lo, a_hi)


def backward_f32_(y: np.ndarray, x: np.ndarray, angles, z_order: int = 0, a_lo: int = 0,
                  a_hi: int | None = None) -> None:
    """x += A^T y in float, in place (CPU baseline); angles [a_lo, a_hi) only."""
    ang = _f32(angles).ravel()
    assert x.dtype == np.float32 and y.dtype == np.float32
    assert x.flags.c_contiguous and y.flags.c_contiguous
    if z_order == 0:
        SY, SX, H = x.shape
        n_ang, PX, Hy = y.shape
    else:
        H, SY, SX = x.shape
        Hy, n_ang, PX = y.shape
    assert H == Hy and ang.size >= n_ang
    a_hi = n_ang if a_hi is None else a_hi
    lib().vpo_backward_f32(_ptr(y), _ptr(x), z_order, SY, SX, n_ang, PX, H, _ptr(ang), a_lo, a_hi)
