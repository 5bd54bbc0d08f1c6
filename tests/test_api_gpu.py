"""The drop-in Python API on the GPU.

Mirrors the reference's own tests — test/test_identity.py:21-110 (output
identity and return kinds) and test/test_adjoitness.py:20-51 (adjoint
identity, full and interior detectors) — and adds what they leave out:
accumulation into a given output, height mismatch between input and output,
empty inputs, non-contiguous containers, dtype conversion, more than 512
angles, stream ordering and error behaviour of the extension functions.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import voxelproj_gb300 as voxelproj
from oracle import oracle
from tests import tolerances as tol
from tests.common import lin, rel_err, seeded, x_shape, y_shape

pytestmark = pytest.mark.gpu

SX, SY, H = 5, 6, 3
PX = SX + SY
N_ID = 7
ANG_ID = lin(N_ID)
YS = {0: (N_ID, PX, H), 2: (H, N_ID, PX)}
XS = {0: (SY, SX, H), 2: (H, SY, SX)}


# ---- test_identity.py ---------------------------------------------------

@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("kind", ["cuda", "cpu", "numpy"])
def test_forward_keeps_id(z, kind):
    if kind == "numpy":
        x = np.random.randn(*XS[z]).astype(np.float32)
        y = np.zeros(YS[z], np.float32)
    else:
        dev = "cuda" if kind == "cuda" else "cpu"
        x = torch.randn(XS[z], device=dev)
        y = torch.zeros(YS[z], device=dev)
    y_out = voxelproj.forward(x, ANG_ID, y, z_order=z)
    assert id(y_out) == id(y)


@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("kind", ["cuda", "cpu", "numpy"])
def test_backward_keeps_id(z, kind):
    if kind == "numpy":
        x = np.random.randn(*XS[z]).astype(np.float32)
        y = np.zeros(YS[z], np.float32)
    else:
        dev = "cuda" if kind == "cuda" else "cpu"
        x = torch.randn(XS[z], device=dev)
        y = torch.zeros(YS[z], device=dev)
    x_out = voxelproj.backward(y, ANG_ID, x, z_order=z)
    assert id(x_out) == id(x)


@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("kind", ["cuda", "cpu", "numpy"])
def test_forward_returns_new_when_none(z, kind):
    if kind == "numpy":
        x = np.random.randn(*XS[z]).astype(np.float32)
    else:
        x = torch.randn(XS[z], device="cuda" if kind == "cuda" else "cpu")
    y_out = voxelproj.forward(x, ANG_ID, None, z_order=z)
    if kind == "numpy":
        assert isinstance(y_out, np.ndarray)
    else:
        assert isinstance(y_out, torch.Tensor) and y_out.device == x.device
    # default detector width max(SY, SX) (wrappers.py:40-43)
    assert tuple(y_out.shape) == ((N_ID, max(SY, SX), H) if z == 0 else (H, N_ID, max(SY, SX)))


@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("kind", ["cuda", "cpu", "numpy"])
def test_backward_returns_new_when_none(z, kind):
    if kind == "numpy":
        y = np.random.randn(*YS[z]).astype(np.float32)
    else:
        y = torch.randn(YS[z], device="cuda" if kind == "cuda" else "cpu")
    x_out = voxelproj.backward(y, ANG_ID, None, z_order=z)
    if kind == "numpy":
        assert isinstance(x_out, np.ndarray)
    else:
        assert isinstance(x_out, torch.Tensor) and x_out.device == y.device
    # default volume (PX, PX) (wrappers.py:88-91)
    assert tuple(x_out.shape) == ((PX, PX, H) if z == 0 else (H, PX, PX))


# ---- test_adjoitness.py -------------------------------------------------

@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("px", [SX + SY, min(SY, SX) - 1], ids=["full", "interior"])
def test_adjointness(z, px):
    n = 31
    ang = lin(n)
    ys = y_shape(z, n, px, H)
    xs = x_shape(z, SY, SX, H)
    x = seeded(xs, 128437, "uniform")
    y = seeded(ys, 128438, "uniform")
    Ax = voxelproj.forward(x, ang, y=ys, z_order=z)
    ATy = voxelproj.backward(y, ang, x=xs, z_order=z)
    lhs = np.vdot(Ax.astype(np.float64), y.astype(np.float64))
    rhs = np.vdot(x.astype(np.float64), ATy.astype(np.float64))
    np.testing.assert_allclose(lhs, rhs, rtol=1e-3, atol=1e-4)  # the reference's bound
    den = np.linalg.norm(Ax) * np.linalg.norm(y)
    assert abs(lhs - rhs) / den <= tol.ADJOINT  # the parity target's bound


# ---- beyond the reference's tests ----------------------------------------

@pytest.mark.parametrize("z", [0, 2])
def test_accumulates_into_given_output(z):
    n, px = 20, 14
    ang = lin(n)
    x = seeded(x_shape(z, 10, 12, 4), 1)
    y0 = seeded(y_shape(z, n, px, 4), 2)
    y = torch.tensor(y0, device="cuda")
    voxelproj.forward(x, ang, y, z_order=z)
    voxelproj.forward(x, ang, y, z_order=z)
    ref = y0 + 2 * oracle.forward(x, ang, px, z)
    assert rel_err(y.cpu().numpy(), ref) < tol.REF_VS_FP64


@pytest.mark.parametrize("z", [0, 2])
def test_height_mismatch_leaves_extra_heights(z):
    """Reference semantics: heights past the input's extent read as zero
    (border-mode texture), so those output heights keep their content."""
    n, px = 16, 14
    ang = lin(n)
    x = seeded(x_shape(z, 10, 12, 6), 3)
    y0 = seeded(y_shape(z, n, px, 4), 4)  # fewer heights than x
    y = torch.tensor(y0, device="cuda")
    fwd = voxelproj._CU.forward_z0 if z == 0 else voxelproj._CU.forward_z2
    fwd(torch.tensor(x, device="cuda"), y, torch.tensor(ang, device="cuda"))
    x_in = x[:, :, :4] if z == 0 else x[:4]
    ref = y0 + oracle.forward(np.ascontiguousarray(x_in), ang, px, z)
    assert rel_err(y.cpu().numpy(), ref) < tol.REF_VS_FP64
    # backward into a volume with more heights than the sinogram
    yb = seeded(y_shape(z, n, px, 4), 5)
    x0 = seeded(x_shape(z, 10, 12, 6), 6)
    xo = torch.tensor(x0, device="cuda")
    fn = voxelproj._CU.backward_z0 if z == 0 else voxelproj._CU.backward_z2
    fn(torch.tensor(yb, device="cuda"), xo, torch.tensor(ang, device="cuda"))
    got = xo.cpu().numpy()
    ATy = oracle.backward(yb, ang, 10, 12, z)
    if z == 0:
        np.testing.assert_array_equal(got[:, :, 4:], x0[:, :, 4:])
        assert rel_err(got[:, :, :4], x0[:, :, :4] + ATy) < tol.REF_VS_FP64
    else:
        np.testing.assert_array_equal(got[4:], x0[4:])
        assert rel_err(got[:4], x0[:4] + ATy) < tol.REF_VS_FP64


@pytest.mark.parametrize("z", [0, 2])
def test_empty_inputs_are_noops(z):
    ang = lin(5)
    for SYs, SXs, Hs, n in [(0, 4, 2, 5), (4, 0, 2, 5), (4, 4, 0, 5), (4, 4, 2, 0)]:
        x = torch.zeros(x_shape(z, SYs, SXs, Hs), device="cuda")
        y = torch.full(y_shape(z, n, 6, Hs), 3.0, device="cuda")
        a = torch.tensor(ang[:n], device="cuda")
        f = voxelproj._CU.forward_z0 if z == 0 else voxelproj._CU.forward_z2
        b = voxelproj._CU.backward_z0 if z == 0 else voxelproj._CU.backward_z2
        f(x, y, a)
        b(y, x, a)
        torch.cuda.synchronize()
        assert (y == 3.0).all() and (x == 0).all()


@pytest.mark.parametrize("z", [0, 2])
def test_noncontiguous_container_and_dtype(z):
    n, px = 12, 16
    ang = lin(n)
    xs = x_shape(z, 10, 12, 4)
    x64 = seeded(xs, 7).astype(np.float64)
    big = torch.zeros(y_shape(z, n, px, 8), device="cuda")
    y = big[..., ::2] if z == 0 else big[::2]
    assert not y.is_contiguous()
    out = voxelproj.forward(torch.tensor(x64, device="cuda"), ang, y, z_order=z)
    assert out is y
    ref = oracle.forward(x64.astype(np.float32), ang, px, z)
    assert rel_err(y.cpu().numpy(), ref) < tol.REF_VS_FP64


def test_more_than_512_angles():
    """The reference adjoint keeps 512 angles in shared memory
    (sp_backward_z0.cuh:6); here any count works."""
    n = 1030
    ang = lin(n, 0, 2 * np.pi)
    y = seeded((n, 20, 3), 8)
    x = voxelproj.backward(y, ang, (16, 18, 3))
    ref = oracle.backward(y, ang, 16, 18, 0)
    assert rel_err(x, ref) < tol.REF_VS_FP64


def test_runs_on_current_stream():
    s = torch.cuda.Stream()
    ang = torch.tensor(lin(64), device="cuda")
    x = torch.randn(64, 64, 32, device="cuda")
    y = torch.zeros(64, 64, 32, device="cuda")
    with torch.cuda.stream(s):
        y_s = torch.zeros_like(y)
        voxelproj._CU.forward_z0(x, y_s, ang)
    s.synchronize()
    voxelproj._CU.forward_z0(x, y, ang)
    torch.cuda.synchronize()
    assert torch.equal(y, y_s)


@pytest.mark.parametrize("fn", ["forward_z0", "backward_z0", "forward_z2", "backward_z2"])
def test_extension_errors(fn):
    f = getattr(voxelproj._CU, fn)
    a = torch.zeros(4, device="cuda")
    ok = torch.zeros(4, 5, 6, device="cuda")
    with pytest.raises(RuntimeError, match="Only float32"):
        f(ok.double(), ok.clone(), a)
    with pytest.raises(RuntimeError, match="contiguous"):
        f(ok.transpose(0, 1), ok.clone(), a)
    with pytest.raises(RuntimeError, match="3D"):
        f(torch.zeros(4, 5, device="cuda"), ok.clone(), a)
    with pytest.raises(RuntimeError):
        f(ok, ok.clone(), torch.zeros(1, device="cuda"))  # too few angles
    with pytest.raises(RuntimeError):
        f(ok, ok.clone().double(), a)
    with pytest.raises(RuntimeError):
        f(ok, ok.clone(), a.cpu())
