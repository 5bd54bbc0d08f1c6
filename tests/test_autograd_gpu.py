"""Differentiable projector and solvers.

* gradcheck in float64 at 16^3 with 8 angles (finite differences against the
  adjoint kernel's Jacobian; the operator is linear, so a large step costs no
  accuracy and keeps float32 rounding of the kernels small);
* the gradients against the Jacobian of the FP64 operator from FP64 finite
  differences, at the same size;
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


def fp64_jacobian(SY, SX, ang, PX, step=2.0 ** -4, seed=5):
    """The Jacobian (n*PX, SY*SX) of the FP64 operator on one height plane, by
    central finite differences in FP64 around a random float32 point.  Heights
    are independent, so one oracle call evaluates every basis direction: height
    j of the volume holds x0 + step * e_j (resp. - step).  x0 lies on a grid
    of 1/256 and the step is 1/16, so the oracle's float32 input holds the
    perturbed points exactly."""
    ncols = SY * SX
    # on a grid of 1/256, so that x0 +- step are float32 sums without rounding
    x0 = (np.random.default_rng(seed).integers(0, 256, (SY, SX)) / 256.0).astype(np.float32)
    E = np.eye(ncols, dtype=np.float32).reshape(ncols, SY, SX) * np.float32(step)
    plus = np.ascontiguousarray((x0[None] + E).transpose(1, 2, 0))  # (SY, SX, ncols)
    minus = np.ascontiguousarray((x0[None] - E).transpose(1, 2, 0))
    fp = oracle.forward_f64(plus, ang, PX, 0)   # (ncols, n, PX)
    fm = oracle.forward_f64(minus, ang, PX, 0)
    J = (fp - fm) / (2.0 * step)
    return J.reshape(ncols, -1).T  # (n*PX, ncols)


@pytest.mark.parametrize("trig", ["precise", "reference"])
@pytest.mark.parametrize("z", [0, 2])
def test_gradients_match_fp64_finite_differences(z, trig):
    """The spec check at the gradcheck size (16^3, 8 angles): the
    gradients autograd returns, computed by the hand-written float32 kernels
    (A^T for project, A for backproject), against the Jacobian of the FP64
    operator obtained by FP64 finite differences.  Bound: the float32 error
    of the chosen trig mode at this size (the Jacobian itself is exact up to
    FP64 rounding, the operator being linear)."""
    SY = SX = PX = 16
    n, H = 8, 8
    ang_np = lin(n)
    J = fp64_jacobian(SY, SX, ang_np, PX)
    rng = np.random.default_rng(17)
    xin = rng.standard_normal((SY, SX, H)).astype(np.float32)
    vin = rng.standard_normal((n, PX, H)).astype(np.float32)

    def to_layout(a):  # z_order 0 array -> the z_order's layout
        return np.ascontiguousarray(a if z == 0 else a.transpose(2, 0, 1))

    ang = torch.tensor(ang_np, device="cuda")
    vp.set_trig_mode(trig)
    try:
        # d<A x, v>/dx = A^T v
        x = torch.tensor(to_layout(xin), device="cuda", requires_grad=True)
        v = torch.tensor(to_layout(vin), device="cuda")
        (project(x, ang, PX, z) * v).sum().backward()
        gx = x.grad.cpu().numpy()
        # d<A^T y, w>/dy = A w
        y = torch.tensor(to_layout(vin), device="cuda", requires_grad=True)
        w = torch.tensor(to_layout(xin), device="cuda")
        (backproject(y, ang, (SY, SX), z) * w).sum().backward()
        gy = y.grad.cpu().numpy()
        torch.cuda.synchronize()
    finally:
        vp.set_trig_mode("reference")
    if z == 2:
        gx = gx.transpose(1, 2, 0)
        gy = gy.transpose(1, 2, 0)
    # FP64: per height, A^T v = J^T v_h and A w = J w_h
    want_gx = np.stack([(J.T @ vin[:, :, h].astype(np.float64).ravel()).reshape(SY, SX)
                        for h in range(H)], axis=-1)
    want_gy = np.stack([(J @ xin[:, :, h].astype(np.float64).ravel()).reshape(n, PX)
                        for h in range(H)], axis=-1)
    ex, ey = rel_err(gx, want_gx), rel_err(gy, want_gy)
    bound = tol.precise_vs_fp64(16) if trig == "precise" else tol.ref_vs_fp64(16)
    print(f"\n[fd64] z={z} {trig}: grad of project {ex:.3e}, grad of backproject {ey:.3e}")
    assert ex <= bound and ey <= bound


def test_fp64_finite_difference_jacobian_is_the_oracle_operator():
    """The finite-difference Jacobian reproduces the FP64 operator itself
    (a check of the check): J u equals the oracle's A u in FP64."""
    ang = lin(8)
    J = fp64_jacobian(16, 16, ang, 16)
    u = np.random.default_rng(3).standard_normal((16, 16, 1)).astype(np.float32)
    Au = oracle.forward_f64(u, ang, 16, 0)[0].ravel()
    assert np.abs(J @ u[:, :, 0].astype(np.float64).ravel() - Au).max() <= 1e-12 * np.abs(Au).max()


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
