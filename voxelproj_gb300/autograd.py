"""Differentiable projector: A and A^T as torch.autograd functions.

``project(x, angles)`` computes y = A x and differentiates through the
hand-written adjoint kernel: dL/dx = A^T dL/dy.  ``backproject(y, angles)``
is A^T with A as its derivative.  Both run the CUDA kernels of this package
in float32; inputs of another floating dtype are cast to float32 for the
kernel and the result is cast back, so float64 inputs work (e.g. for
``torch.autograd.gradcheck``) while the arithmetic stays float32.

This layer has no counterpart in the reference, which exposes A and A^T as
plain functions (voxelproj/wrappers.py).

Geometry conventions are the reference's: z_order 0 x (SY, SX, H) and y
(n_ang, PX, H); z_order 2 x (H, SY, SX) and y (H, n_ang, PX).  The default
detector width is max(SY, SX) (wrappers.py:40-43).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _CU

_FWD = {0: _CU.forward_z0, 2: _CU.forward_z2}
_BWD = {0: _CU.backward_z0, 2: _CU.backward_z2}


def _angles_tensor(angles, device) -> torch.Tensor:
    if isinstance(angles, torch.Tensor):
        return angles.to(device=device, dtype=torch.float32).reshape(-1).contiguous()
    return torch.as_tensor(np.asarray(angles, dtype=np.float32), device=device).reshape(-1)


def _y_shape(vol_shape, n_ang, px, z_order):
    if z_order == 0:
        return (n_ang, px, vol_shape[2])
    return (vol_shape[0], n_ang, px)


def _x_shape(sino_shape, vol_yx, z_order):
    sy, sx = vol_yx
    if z_order == 0:
        return (sy, sx, sino_shape[2])
    return (sino_shape[0], sy, sx)


def _apply_forward(x32, a32, px, z_order):
    y = torch.zeros(_y_shape(x32.shape, a32.numel(), px, z_order), dtype=torch.float32,
                    device=x32.device)
    _FWD[z_order](x32, y, a32)
    return y


def _apply_backward(y32, a32, vol_yx, z_order):
    x = torch.zeros(_x_shape(y32.shape, vol_yx, z_order), dtype=torch.float32,
                    device=y32.device)
    _BWD[z_order](y32, x, a32)
    return x


def _vol_yx(x_shape, z_order):
    return (x_shape[0], x_shape[1]) if z_order == 0 else (x_shape[1], x_shape[2])


class ProjectFunction(torch.autograd.Function):
    """y = A x; backward: A^T (the adjoint kernel)."""

    @staticmethod
    def forward(ctx, x, angles, detector_width, z_order):
        if z_order not in _FWD:
            raise KeyError(z_order)
        a32 = _angles_tensor(angles, x.device)
        vol_yx = _vol_yx(x.shape, z_order)
        px = detector_width if detector_width is not None else max(vol_yx)
        ctx.save_for_backward(a32)
        ctx.meta = (vol_yx, z_order, x.dtype)
        y = _apply_forward(x.detach().to(torch.float32).contiguous(), a32, px, z_order)
        return y.to(x.dtype)

    @staticmethod
    def backward(ctx, gy):
        (a32,) = ctx.saved_tensors
        vol_yx, z_order, dtype = ctx.meta
        gx = _apply_backward(gy.detach().to(torch.float32).contiguous(), a32, vol_yx, z_order)
        return gx.to(dtype), None, None, None


class BackprojectFunction(torch.autograd.Function):
    """x = A^T y; backward: A (the forward kernel)."""

    @staticmethod
    def forward(ctx, y, angles, volume_yx, z_order):
        if z_order not in _BWD:
            raise KeyError(z_order)
        a32 = _angles_tensor(angles, y.device)
        px = y.shape[1] if z_order == 0 else y.shape[2]
        vol_yx = tuple(volume_yx) if volume_yx is not None else (px, px)
        ctx.save_for_backward(a32)
        ctx.meta = (px, z_order, y.dtype)
        x = _apply_backward(y.detach().to(torch.float32).contiguous(), a32, vol_yx, z_order)
        return x.to(y.dtype)

    @staticmethod
    def backward(ctx, gx):
        (a32,) = ctx.saved_tensors
        px, z_order, dtype = ctx.meta
        gy = _apply_forward(gx.detach().to(torch.float32).contiguous(), a32, px, z_order)
        return gy.to(dtype), None, None, None


def project(x: torch.Tensor, angles, detector_width: int | None = None,
            z_order: int = 0) -> torch.Tensor:
    """Differentiable A x for a CUDA tensor x."""
    return ProjectFunction.apply(x, angles, detector_width, z_order)


def backproject(y: torch.Tensor, angles, volume_yx=None, z_order: int = 0) -> torch.Tensor:
    """Differentiable A^T y for a CUDA tensor y; volume_yx = (SY, SX), default
    (PX, PX) as in the reference (wrappers.py:88-91)."""
    return BackprojectFunction.apply(y, angles, volume_yx, z_order)


class Projector(torch.nn.Module):
    """A fixed parallel-beam geometry as a module: ``P(x) = A x``,
    ``P.T(y) = A^T y``; both differentiable.  The angles live on the device,
    so repeated calls copy nothing from the host."""

    def __init__(self, angles, volume_yx, detector_width: int | None = None,
                 z_order: int = 0, device="cuda"):
        super().__init__()
        self.register_buffer("angles", _angles_tensor(angles, torch.device(device)))
        self.volume_yx = tuple(volume_yx)
        self.detector_width = detector_width if detector_width is not None else max(volume_yx)
        self.z_order = z_order

    def forward(self, x):
        return project(x, self.angles, self.detector_width, self.z_order)

    def T(self, y):
        return backproject(y, self.angles, self.volume_yx, self.z_order)
