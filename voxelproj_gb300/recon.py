"""Reconstruction on top of the projector pair: phantoms, Adam, SIRT, CGLS.

None of this exists in the reference, which provides only A and A^T
(voxelproj/wrappers.py).  All solvers keep the volume, the sinogram and their
iterates on the device and call the CUDA kernels directly (no host copies
inside the loops); inner products are accumulated in float64.

    python -m voxelproj_gb300.recon [--size 256] [--angles 360] [--steps 50]

runs the differentiable-reconstruction workload: a phantom of 20 random
ellipsoids, b = A phantom + N(0, (0.01 max)^2), and Adam steps on
0.5 ||A x - b||^2 through the autograd projector; it prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import _CU
from .autograd import Projector, _angles_tensor


def ellipsoid_phantom(n: int, count: int = 20, seed: int = 0, device="cuda") -> torch.Tensor:
    """n^3 float32 volume (z_order 0 layout: y, x, height) holding `count`
    additive axis-aligned ellipsoids in normalised [-1, 1]^3 coordinates:
    centres U[-0.7, 0.7], semi-axes U[0.05, 0.4], densities U[0, 1]."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-0.7, 0.7, (count, 3))
    axes = rng.uniform(0.05, 0.4, (count, 3))
    dens = rng.uniform(0.0, 1.0, count)
    t = torch.linspace(-1.0, 1.0, n, device=device, dtype=torch.float32)
    vol = torch.zeros((n, n, n), device=device, dtype=torch.float32)
    Y = t.view(n, 1, 1)
    X = t.view(1, n, 1)
    Z = t.view(1, 1, n)
    for c, a, d in zip(centres, axes, dens):
        q = ((Y - c[0]) / a[0]) ** 2 + ((X - c[1]) / a[1]) ** 2 + ((Z - c[2]) / a[2]) ** 2
        vol += (q <= 1.0).to(torch.float32) * float(d)
    return vol


def noisy_sinogram(P: Projector, phantom: torch.Tensor, noise: float = 0.01,
                   seed: int = 1) -> torch.Tensor:
    """b = A phantom + N(0, (noise * max|A phantom|)^2)."""
    with torch.no_grad():
        clean = P(phantom)
        g = torch.Generator(device=clean.device).manual_seed(seed)
        sigma = noise * float(clean.abs().max())
        return clean + sigma * torch.randn(clean.shape, device=clean.device, generator=g)


def adam_reconstruct(P: Projector, b: torch.Tensor, steps: int = 50, lr: float = 0.05,
                     x0: torch.Tensor | None = None):
    """Adam on 0.5 ||A x - b||^2 with gradients from the adjoint kernel.
    Returns (x, list of losses)."""
    vol_shape = (*P.volume_yx, b.shape[2]) if P.z_order == 0 else (b.shape[0], *P.volume_yx)
    x = (x0.clone() if x0 is not None else torch.zeros(vol_shape, device=b.device))
    x.requires_grad_(True)
    # one fused kernel per update on CUDA
    opt = torch.optim.Adam([x], lr=lr, fused=x.is_cuda)
    losses = []
    for _ in range(steps):
        opt.zero_grad(set_to_none=True)
        r = (P(x) - b).reshape(-1)
        # the gradient of 0.5 r.r with respect to r is r itself; the loss
        # value is a float32 dot product, kept on the device (no sync per step)
        loss = 0.5 * torch.dot(r, r)
        loss.backward()
        opt.step()
        losses.append(loss.detach())
    return x.detach(), [float(v) for v in torch.stack(losses).double().cpu()]


def _dot(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    return torch.sum(a.double() * b.double())


class Operator:
    """A and A^T of one geometry on device tensors, without autograd."""

    def __init__(self, angles, volume_shape, detector_width: int | None = None,
                 z_order: int = 0, device="cuda"):
        self.a = _angles_tensor(angles, torch.device(device))
        self.z = z_order
        self.vol_shape = tuple(volume_shape)
        vol_yx = self.vol_shape[:2] if z_order == 0 else self.vol_shape[1:]
        self.px = detector_width if detector_width is not None else max(vol_yx)
        n = self.a.numel()
        self.sino_shape = ((n, self.px, self.vol_shape[2]) if z_order == 0
                           else (self.vol_shape[0], n, self.px))
        self._fwd = _CU.forward_z0 if z_order == 0 else _CU.forward_z2
        self._bwd = _CU.backward_z0 if z_order == 0 else _CU.backward_z2

    def A(self, x, out=None):
        out = torch.zeros(self.sino_shape, device=x.device) if out is None else out.zero_()
        self._fwd(x, out, self.a)
        return out

    def AT(self, y, out=None):
        out = torch.zeros(self.vol_shape, device=y.device) if out is None else out.zero_()
        self._bwd(y, out, self.a)
        return out


def sirt(op: Operator, b: torch.Tensor, iters: int, x0: torch.Tensor | None = None):
    """SIRT: x <- x + C A^T (R (b - A x)), R = 1/(A 1), C = 1/(A^T 1), with
    zero where a row or column sum vanishes."""
    dev = b.device
    ones_x = torch.ones(op.vol_shape, device=dev)
    ones_y = torch.ones(op.sino_shape, device=dev)
    row = op.A(ones_x)
    col = op.AT(ones_y)
    R = torch.where(row > 0, 1.0 / row, torch.zeros_like(row))
    C = torch.where(col > 0, 1.0 / col, torch.zeros_like(col))
    x = x0.clone() if x0 is not None else torch.zeros(op.vol_shape, device=dev)
    ax = torch.empty(op.sino_shape, device=dev)
    g = torch.empty(op.vol_shape, device=dev)
    for _ in range(iters):
        op.A(x, ax)
        r = (b - ax).mul_(R)
        op.AT(r, g)
        x.addcmul_(C, g)
    return x


def cgls(op: Operator, b: torch.Tensor, iters: int, x0: torch.Tensor | None = None):
    """CGLS for min ||A x - b||^2 (textbook form), float64 inner products."""
    dev = b.device
    x = x0.clone() if x0 is not None else torch.zeros(op.vol_shape, device=dev)
    r = b - op.A(x)
    s = op.AT(r)
    p = s.clone()
    gamma = _dot(s, s)
    q = torch.empty(op.sino_shape, device=dev)
    for _ in range(iters):
        op.A(p, q)
        qq = _dot(q, q)
        if float(qq) == 0.0:
            break
        alpha = (gamma / qq).float()
        x.add_(alpha * p)
        r.sub_(alpha * q)
        op.AT(r, s)
        gamma_new = _dot(s, s)
        beta = (gamma_new / gamma).float() if float(gamma) > 0 else torch.zeros((), device=dev)
        p.mul_(beta).add_(s)
        gamma = gamma_new
    return x


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--angles", type=int, default=360)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--lr", type=float, default=0.05)
    args = ap.parse_args()
    n, na = args.size, args.angles
    angles = np.linspace(0, np.pi, na, endpoint=False).astype(np.float32)
    P = Projector(angles, (n, n))
    phantom = ellipsoid_phantom(n)
    b = noisy_sinogram(P, phantom)
    adam_reconstruct(P, b, steps=2, lr=args.lr)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x, losses = adam_reconstruct(P, b, steps=args.steps, lr=args.lr)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    rel = float((x - phantom).norm() / phantom.norm())
    vu = 2 * n**3 * na * args.steps  # one A and one A^T per step
    print(json.dumps({
        "workload": f"Adam reconstruction, {n}^3 ellipsoid phantom, {na} angles [0, pi)",
        "steps": args.steps, "s_total": round(dt, 4), "ms_per_step": round(dt / args.steps * 1e3, 3),
        "gvu_s": round(vu / dt / 1e9, 2), "loss_first": losses[0], "loss_last": losses[-1],
        "rel_error_vs_phantom": round(rel, 5),
    }))


if __name__ == "__main__":
    main()
