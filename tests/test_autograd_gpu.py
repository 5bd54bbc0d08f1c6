"""Differentiable projector and solvers.

* gradcheck in float64 at 16^3 with 8 angles (finite differences against the
  adjoint kernel's Jacobian; the operator is linear, so a large step costs no
  accuracy and keeps float32 rounding of the kernels small);
* the gradient is the adjoint kernel's output, matches the FP64 oracle and
  the reference's recorded backward;
* Adam, SIRT and CGLS reduce the data misfit.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

import voxelproj_gb300 as vp
from oracle import oracle
from tests import tolerances as tol
from tests.common import lin, rel_err, seeded
from voxelproj_gb300.autograd import Projector, backproject, project
from voxelproj_gb300.recon import (Operator, adam_reconstruct, cgls, ellipsoid_phantom,
                                   noisy_sinogram, sirt)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("z", [0, 2])
def test_gradcheck_float64(z):
    ang = torch.tensor(lin(8), device="cuda")
    x = torch.rand((16, 16, 16), dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda v: project(v, ang, 16, z), (x,), eps=1e-2,
                                    atol=1e-3, rtol=1e-3)
    y = torch.rand((8, 16, 16) if z == 0 else (16, 8, 16), dtype=torch.float64, device="cuda",
                   requires_grad=True)
    assert torch.autograd.gradcheck(lambda v: backproject(v, ang, (16, 16), z), (y,), eps=1e-2,
                                    atol=1e-3, rtol=1e-3)


def test_gradient_is_the_adjoint_kernel():
    ang = lin(45)
    x = torch.randn(24, 20, 8, device="cuda", requires_grad=True)
    w = torch.randn(45, 30, 8, device="cuda")
    (project(x, ang, 30) * w).sum().backward()
    ref = torch.zeros(24, 20, 8, device="cuda")
    vp._CU.backward_z0(w, ref, torch.tensor(ang, device="cuda"))
    assert torch.equal(x.grad, ref)
    oracle_grad = oracle.backward(w.cpu().numpy(), ang, 24, 20, 0)
    assert rel_err(x.grad.cpu().numpy(), oracle_grad) <= tol.REF_VS_FP64


def test_gradient_matches_reference_backward():
    """The gradient of <A x, y> is A^T y; the reference's kernels recorded it
    for these inputs (golden fixture)."""
    d = np.load(Path(__file__).resolve().parent / "golden" / "reference_outputs.npz")
    name = "rect_full_z0"
    ang = d[f"{name}/angles"]
    y = torch.tensor(d[f"{name}/y"], device="cuda")
    x = torch.zeros(d[f"{name}/x"].shape, device="cuda", requires_grad=True)
    (project(x, ang, y.shape[1]) * y).sum().backward()
    ref = d[f"{name}/bwd"] - d[f"{name}/x0"]
    assert rel_err(x.grad.cpu().numpy(), ref) <= tol.REF_VS_REFERENCE


def test_projector_module_roundtrip():
    ang = lin(30)
    P = Projector(ang, (20, 22), detector_width=32)
    x = torch.randn(20, 22, 4, device="cuda")
    y = P(x)
    assert y.shape == (30, 32, 4)
    xt = P.T(y)
    assert xt.shape == (20, 22, 4)
    # <Ax, Ax> = <x, A^T A x>
    lhs = float(torch.sum(y.double() ** 2))
    rhs = float(torch.sum(x.double() * xt.double()))
    assert abs(lhs - rhs) <= 1e-6 * lhs


def test_adam_reconstruction_reduces_misfit_and_error():
    n, na = 32, 60
    ang = np.linspace(0, np.pi, na, endpoint=False).astype(np.float32)
    P = Projector(ang, (n, n))
    ph = ellipsoid_phantom(n, seed=3)
    b = noisy_sinogram(P, ph)
    x, losses = adam_reconstruct(P, b, steps=40, lr=0.05)
    assert losses[-1] < 0.05 * losses[0]
    assert float((x - ph).norm() / ph.norm()) < 0.5


@pytest.mark.parametrize("z", [0, 2])
def test_sirt_and_cgls_reduce_residual(z):
    n, na = 24, 40
    ang = np.linspace(0, np.pi, na, endpoint=False).astype(np.float32)
    shape = (n, n, 4) if z == 0 else (4, n, n)
    op = Operator(ang, shape, z_order=z)
    xt = torch.rand(shape, device="cuda")
    b = op.A(xt)
    r0 = float(b.norm())
    for solver in (sirt, cgls):
        x = solver(op, b, 20)
        r = float((op.A(x) - b).norm())
        assert r < 0.2 * r0, solver.__name__
    # CGLS on a consistent system converges much further
    x = cgls(op, b, 60)
    assert float((op.A(x) - b).norm()) < 1e-2 * r0
