"""Drop-in Python API: ``forward`` (A) and ``backward`` (A^T).

Mirrors voxelproj/wrappers.py:10-122 of the reference:

* ``x``/``y`` may be numpy arrays, CPU tensors or CUDA tensors of any dtype;
  they are moved to CUDA as float32.
* The output argument may be ``None`` (default shape), a shape tuple, or a
  container.  A container is ACCUMULATED into (``out += result``) and is the
  object returned (same ``id``); numpy containers are filled with
  ``np.copyto``, tensors with ``copy_`` unless the CUDA float32 tensor itself
  was computed into.
* Without a container the result comes back in the input's kind: numpy in,
  numpy out; tensor in, tensor on the input's device.
* Default output shapes (wrappers.py:40-43, :88-91):
  forward z0 (n_ang, max(SY,SX), H), z2 (H, n_ang, max(SY,SX));
  backward z0 (PX, PX, H), z2 (H, PX, PX).
* ``z_order`` other than 0 or 2 raises ``KeyError`` (dict dispatch, :44-47).
* ``block_size`` is accepted for compatibility and ignored.

Beyond the reference: ``angles`` may also be a list or tuple (the reference
accepted only arrays/tensors), non-contiguous inputs and outputs are handled
instead of rejected or mis-written, and there is no 512-angle limit.  Host
angle arrays are copied to the device once per distinct content and reused
(``cached_angles``); the reference copies them on every call
(wrappers.py:50).

Host arrays (numpy or CPU tensors, with a host container or none) go
through the library's host-buffer entry points (``vp_forward_z0_host`` /
``vp_backward_z0_host``, ``vp_forward_z2_host`` / ``vp_backward_z2_host``),
which overlap the copies to and from the GPU with the projection; the
reference copies, projects and copies back one after another.  Page-locked CPU tensors
(``tensor.pin_memory()``) give the most overlap.
"""

from __future__ import annotations

import threading
from collections import OrderedDict

import numpy as np
import torch

from . import _CU, _lib
from ._CU import backward_z0, backward_z2, forward_z0, forward_z2


def gpu_array_with_default_shape(x=None, shape=None):
    """None or a shape tuple -> zeros on CUDA; array/tensor -> float32 CUDA
    tensor (no copy when it already is one).  As wrappers.py:10-25."""
    if x is None:
        return torch.zeros(shape, dtype=torch.float32, device="cuda")
    if isinstance(x, tuple):
        return torch.zeros(x, dtype=torch.float32, device="cuda")
    if isinstance(x, np.ndarray):
        return torch.tensor(x, dtype=torch.float32, device="cuda")
    if isinstance(x, torch.Tensor):
        return x.to(dtype=torch.float32, device="cuda")
    raise TypeError("x must be None, a shape tuple, or an array/tensor")


# Device copies of host angle arrays, keyed on their exact float32 bytes and
# the device: a caller that passes the same angles every call (the usual
# iterative reconstruction) pays the host-to-device copy once.  An array
# changed in place has other bytes, so it gets its own entry.
_ANGLE_CACHE: "OrderedDict[tuple, torch.Tensor]" = OrderedDict()
_ANGLE_CACHE_SIZE = 32
_ANGLE_CACHE_LOCK = threading.Lock()


def cached_angles(angles, device) -> torch.Tensor:
    """``angles`` on ``device`` as a contiguous float32 vector.  A tensor
    already there is used as it is; host angles (numpy, list, tuple, CPU
    tensor) come from the cache."""
    device = torch.device(device)
    if isinstance(angles, torch.Tensor) and angles.device == device:
        return angles.to(torch.float32).reshape(-1).contiguous()
    if isinstance(angles, torch.Tensor):
        angles = angles.detach().cpu().numpy()
    arr = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).reshape(-1))
    key = (str(device), arr.tobytes())
    with _ANGLE_CACHE_LOCK:
        t = _ANGLE_CACHE.get(key)
        if t is not None:
            _ANGLE_CACHE.move_to_end(key)
            return t
    t = torch.from_numpy(arr.copy()).to(device)
    with _ANGLE_CACHE_LOCK:
        _ANGLE_CACHE[key] = t
        while len(_ANGLE_CACHE) > _ANGLE_CACHE_SIZE:
            _ANGLE_CACHE.popitem(last=False)
    return t


def _angles_gpu(angles, device) -> torch.Tensor:
    return cached_angles(angles, device)


def _input_gpu(v) -> torch.Tensor:
    return gpu_array_with_default_shape(v).contiguous()


def _finish(out, out_gpu, work, src_kind, src_device):
    """Copies back into a caller's container or returns a new array in the
    input's kind (wrappers.py:57-73)."""
    if work is not out_gpu:
        out_gpu.copy_(work)
    if isinstance(out, np.ndarray):
        if out.dtype == np.float32 and out.flags.c_contiguous and out.flags.writeable:
            torch.from_numpy(out).copy_(out_gpu)  # one device-to-host copy
        else:
            np.copyto(out, out_gpu.cpu().numpy())
        return out
    if isinstance(out, torch.Tensor):
        if out.data_ptr() != out_gpu.data_ptr() or out.device != out_gpu.device:
            out.copy_(out_gpu)
        return out
    if src_kind == "numpy":
        return out_gpu.cpu().numpy()
    return out_gpu.to(src_device) if src_device is not None else out_gpu


def _kind(v):
    if isinstance(v, np.ndarray):
        return "numpy", None
    if isinstance(v, torch.Tensor) and not v.is_cuda:
        return "tensor", v.device
    return "cuda", None


def _host_out(out):
    return out is None or isinstance(out, (tuple, np.ndarray)) or (
        isinstance(out, torch.Tensor) and not out.is_cuda)


def _host_array(v):
    """Float32 C-contiguous host data of a numpy array or CPU tensor (no copy
    when it already is one): (holder, address)."""
    if isinstance(v, np.ndarray):
        a = np.ascontiguousarray(v, dtype=np.float32)
        return a, a.ctypes.data
    t = v.detach().to(torch.float32).contiguous()
    return t, t.data_ptr()


def _host_call(fn_name, inp, out, angles, default_shape, kind):
    """z_order 0 with host arrays through the host-buffer entry points."""
    src, src_ptr = _host_array(inp)
    if src.ndim != 3:
        raise RuntimeError("Tensor must be 3D")
    if isinstance(angles, torch.Tensor) and angles.is_cuda:
        ang = angles.detach().to(torch.float32).reshape(-1).contiguous()
        ang_ptr, n_ang = ang.data_ptr(), ang.numel()
    else:
        if isinstance(angles, torch.Tensor):
            angles = angles.detach().cpu().numpy()
        ang = np.ascontiguousarray(np.asarray(angles, dtype=np.float32).reshape(-1))
        ang_ptr, n_ang = ang.ctypes.data, ang.size
    flags = _CU._flags
    if out is None or isinstance(out, tuple):
        shape = default_shape if out is None else out
        work = (np.empty(shape, np.float32) if kind == "numpy"
                else torch.empty(shape, dtype=torch.float32))
        result, flags = work, flags | _lib.VP_FLAG_OVERWRITE
    else:
        result = out
        if isinstance(out, np.ndarray):
            direct = (out.dtype == np.float32 and out.flags.c_contiguous
                      and out.flags.writeable)
            work = out if direct else np.ascontiguousarray(out, dtype=np.float32).copy()
        else:
            direct = out.dtype == torch.float32 and out.is_contiguous()
            work = out if direct else out.to(torch.float32).contiguous()
    if work.ndim != 3:
        raise RuntimeError("out must be 3D")
    work_ptr = work.ctypes.data if isinstance(work, np.ndarray) else work.data_ptr()
    stream = torch.cuda.current_stream()
    status = getattr(_lib.LIB, fn_name)(src_ptr, *src.shape, work_ptr, *work.shape, ang_ptr,
                                        n_ang, flags, stream.cuda_stream)
    _lib.check(status, fn_name[3:])
    stream.synchronize()
    if work is not result:
        if isinstance(result, np.ndarray):
            np.copyto(result, work)
        else:
            result.copy_(work)
    return result


# block_size keeps the reference's list default (wrappers.py:28,76) so that
# the signatures match exactly; it is handed to the extension functions,
# which ignore it, and never mutated.
def forward(x, angles, y, z_order=0, block_size=[8, 8, 8]):
    """Forward projection: returns y + A x (see module docstring)."""
    kind, device = _kind(x)
    n_ang = len(angles)
    default_shape = {
        0: (n_ang, max(x.shape[0], x.shape[1]), x.shape[2]),
        2: (x.shape[0], n_ang, max(x.shape[1], x.shape[2])),
    }
    project = {0: forward_z0, 2: forward_z2}
    shape = default_shape[z_order]
    fn = project[z_order]
    if kind != "cuda" and _host_out(y):
        return _host_call("vp_forward_z%d_host" % z_order, x, y, angles, shape, kind)
    x_gpu = _input_gpu(x)
    a_gpu = _angles_gpu(angles, x_gpu.device)
    y_gpu = gpu_array_with_default_shape(y, shape=shape)
    work = y_gpu if y_gpu.is_contiguous() else y_gpu.contiguous()
    fn(x_gpu, work, a_gpu, block_size=block_size)
    return _finish(y, y_gpu, work, kind, device)


def backward(y, angles, x, z_order=0, block_size=[8, 8, 8]):
    """Backprojection: returns x + A^T y (see module docstring)."""
    kind, device = _kind(y)
    default_shape = {
        0: (y.shape[1], y.shape[1], y.shape[2]),
        2: (y.shape[0], y.shape[2], y.shape[2]),
    }
    project = {0: backward_z0, 2: backward_z2}
    shape = default_shape[z_order]
    fn = project[z_order]
    if kind != "cuda" and _host_out(x):
        return _host_call("vp_backward_z%d_host" % z_order, y, x, angles, shape, kind)
    y_gpu = _input_gpu(y)
    a_gpu = _angles_gpu(angles, y_gpu.device)
    x_gpu = gpu_array_with_default_shape(x, shape=shape)
    work = x_gpu if x_gpu.is_contiguous() else x_gpu.contiguous()
    fn(y_gpu, work, a_gpu, block_size=block_size)
    return _finish(x, x_gpu, work, kind, device)
