"""Extension surface of the reference, backed by the C-ABI library.

Same names, arguments and behaviour as the reference module ``voxelproj._CU``
(voxelproj/csrc/voxelproj.cpp:15-33; host code projectors.cu:34-299):

    forward_z0(in, out, angles, block_size=[8, 8, 8]) -> None    out += A in
    backward_z0(in, out, angles, block_size=[8, 8, 8]) -> None   out += A^T in
    forward_z2 / backward_z2                                     z_order 2 layouts

``in`` must be a contiguous 3-D float32 CUDA tensor; the reference's checks
(projectors.cu:36-40) raise ``RuntimeError`` with the same messages.  This
shim also validates ``out`` and ``angles`` (the reference did not, and would
fault or write out of bounds on a mismatch).  ``block_size`` is accepted and
ignored: launch shapes are chosen by the library.  Work is enqueued on the
current torch CUDA stream of ``in``'s device and is not synchronised.
"""

from __future__ import annotations

import os

import torch

from . import _lib

_TRIG_MODES = {"reference": 0, "precise": _lib.VP_FLAG_TRIG_PRECISE}
_flags = _TRIG_MODES.get(os.environ.get("VOXELPROJ_GB300_TRIG", "reference"), 0)


def set_trig_mode(mode: str) -> None:
    """Selects the per-angle trig: "reference" (default) uses the hardware
    approximations of the reference's fast-math build so results track its
    kernels; "precise" uses accurate sincosf and IEEE division."""
    global _flags
    if mode not in _TRIG_MODES:
        raise ValueError(f"trig mode must be one of {sorted(_TRIG_MODES)}")
    _flags = _TRIG_MODES[mode]


def get_trig_mode() -> str:
    return "precise" if _flags & _lib.VP_FLAG_TRIG_PRECISE else "reference"


def _check_in(t) -> None:
    # projectors.cu:36-40
    if not isinstance(t, torch.Tensor):
        raise TypeError("in must be a torch.Tensor")
    if not t.is_cuda:
        raise RuntimeError("Tensor must be on CUDA")
    if t.dtype != torch.float32:
        raise RuntimeError("Only float32 tensors supported")
    if not t.is_contiguous():
        raise RuntimeError("Tensor must be contiguous")
    if t.dim() != 3:
        raise RuntimeError("Tensor must be 3D")


def _check_other(t, name: str, device: torch.device, ndim: int | None) -> None:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda or t.device != device:
        raise RuntimeError(f"{name} must be on the same CUDA device as in")
    if t.dtype != torch.float32:
        raise RuntimeError(f"{name} must be float32")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if ndim is not None and t.dim() != ndim:
        raise RuntimeError(f"{name} must be {ndim}D")


def _call(fn_name: str, inp, out, angles) -> None:
    _check_in(inp)
    _check_other(out, "out", inp.device, 3)
    _check_other(angles, "angles", inp.device, None)
    if out.data_ptr() == inp.data_ptr() and inp.numel() > 0:
        raise RuntimeError("in and out must not alias")
    with torch.cuda.device(inp.device):
        stream = torch.cuda.current_stream(inp.device).cuda_stream
        if fn_name.endswith("z2"):
            # scratch for the transposed path, from torch's caching allocator
            x, y = (inp, out) if fn_name.startswith("vp_forward") else (out, inp)
            nbytes = _lib.LIB.vp_z2_workspace_bytes(*x.shape, *y.shape)
            ws = torch.empty((nbytes + 3) // 4, dtype=torch.float32, device=inp.device) \
                if nbytes else None
            fn = getattr(_lib.LIB, fn_name + "_ws")
            status = fn(inp.data_ptr(), *inp.shape, out.data_ptr(), *out.shape,
                        angles.data_ptr(), angles.numel(), _flags,
                        ws.data_ptr() if ws is not None else None, nbytes, stream)
        else:
            fn = getattr(_lib.LIB, fn_name)
            status = fn(inp.data_ptr(), *inp.shape, out.data_ptr(), *out.shape,
                        angles.data_ptr(), angles.numel(), _flags, stream)
    _lib.check(status, fn_name[3:])


def forward_z0(inp, out, angles, block_size=(8, 8, 8)) -> None:
    """out (n_ang, PX, H) += A inp (SY, SX, H).  Height as the fastest index."""
    _call("vp_forward_z0", inp, out, angles)


def backward_z0(inp, out, angles, block_size=(8, 8, 8)) -> None:
    """out (SY, SX, H) += A^T inp (n_ang, PX, H).  Height as the fastest index."""
    _call("vp_backward_z0", inp, out, angles)


def forward_z2(inp, out, angles, block_size=(8, 8, 8)) -> None:
    """out (H, n_ang, PX) += A inp (H, SY, SX).  Height as the slowest index."""
    _call("vp_forward_z2", inp, out, angles)


def backward_z2(inp, out, angles, block_size=(8, 8, 8)) -> None:
    """out (H, SY, SX) += A^T inp (H, n_ang, PX).  Height as the slowest index."""
    _call("vp_backward_z2", inp, out, angles)
