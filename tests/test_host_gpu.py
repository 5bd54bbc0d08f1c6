"""Host-buffer entry points (vp_forward_z0_host / vp_backward_z0_host) and the
wrappers' host path: the same operator as the device entry points, with the
copies overlapped; several slabs, ragged row splits, both output modes."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import voxelproj_gb300 as vp
from oracle import oracle
from tests import tolerances as tol
from tests.common import lin, rel_err, seeded
from voxelproj_gb300 import _lib

pytestmark = pytest.mark.gpu

# (SY, SX, H, n_ang, PX): one slab; several forward slabs and adjoint row
# slabs with a ragged last one (SY not a multiple of the slab rows); heights
# of one float4 chunk and of two half-filled 256-height chunks
GEOMS = [(20, 24, 8, 30, 28), (300, 260, 260, 12, 300), (61, 47, 132, 25, 50)]


def _call(name, inp, out, ang, flags=0):
    stream = torch.cuda.current_stream()
    st = getattr(_lib.LIB, name)(inp.data_ptr(), *inp.shape, out.data_ptr(), *out.shape,
                                 ang.data_ptr(), ang.numel(), flags, stream.cuda_stream)
    _lib.check(st, name)
    stream.synchronize()


@pytest.mark.parametrize("geom", GEOMS, ids=lambda g: "x".join(map(str, g)))
@pytest.mark.parametrize("pinned", [True, False])
def test_host_entries_match_oracle_and_device_path(geom, pinned):
    SY, SX, H, n, PX = geom
    ang = lin(n, -0.3, 3.4)
    x = torch.tensor(seeded((SY, SX, H), 1))
    y = torch.tensor(seeded((n, PX, H), 2))
    y0 = torch.tensor(seeded((n, PX, H), 3))
    x0 = torch.tensor(seeded((SY, SX, H), 4))
    if pinned:
        x, y, y0, x0 = (t.pin_memory() for t in (x, y, y0, x0))
    a_host = torch.tensor(ang)

    yo = y0.clone()
    _call("vp_forward_z0_host", x, yo, a_host)
    xo = x0.clone()
    _call("vp_backward_z0_host", y, xo, a_host)

    n_ext = max(SY, SX, PX)
    assert rel_err(yo.numpy() - y0.numpy(), oracle.forward(x.numpy(), ang, PX, 0)) <= \
        tol.ref_vs_fp64(n_ext)
    assert rel_err(xo.numpy() - x0.numpy(), oracle.backward(y.numpy(), ang, SY, SX, 0)) <= \
        tol.ref_vs_fp64(n_ext)

    # the device entry points: same operator, summed in another order (the
    # host path's row and column pieces group the slab partial sums
    # differently from the device path's class slabs; a few ulp of the
    # largest output)
    yd = y0.cuda()
    vp._CU.forward_z0(x.cuda(), yd, a_host.cuda())
    xd = x0.cuda()
    vp._CU.backward_z0(y.cuda(), xd, a_host.cuda())
    torch.cuda.synchronize()
    assert rel_err(yo.numpy(), yd.cpu().numpy()) <= 4e-6
    assert rel_err(xo.numpy(), xd.cpu().numpy()) <= 4e-6


@pytest.mark.parametrize("geom", GEOMS[1:], ids=lambda g: "x".join(map(str, g)))
def test_overwrite_mode_and_device_angles(geom):
    """VP_FLAG_OVERWRITE: out = result, whatever the output held before;
    angles may live on the device."""
    SY, SX, H, n, PX = geom
    ang = lin(n)
    x = torch.tensor(seeded((SY, SX, H), 5)).pin_memory()
    y = torch.tensor(seeded((n, PX, H), 6)).pin_memory()
    a_dev = torch.tensor(ang, device="cuda")
    yo = torch.full((n, PX, H), 7.0).pin_memory()
    _call("vp_forward_z0_host", x, yo, a_dev, _lib.VP_FLAG_OVERWRITE)
    xo = torch.full((SY, SX, H), -3.0)
    _call("vp_backward_z0_host", y, xo, a_dev, _lib.VP_FLAG_OVERWRITE)
    assert rel_err(yo.numpy(), oracle.forward(x.numpy(), ang, PX, 0)) <= tol.ref_vs_fp64(PX)
    assert rel_err(xo.numpy(), oracle.backward(y.numpy(), ang, SY, SX, 0)) <= \
        tol.ref_vs_fp64(max(SY, SX))


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_host_entries_few_angles(n):
    """Angle counts below the forward's two angle halves and four output
    groups, and below the adjoint's first-angles split."""
    SY, SX, H, PX = 40, 36, 264, 44
    ang = lin(n, 0.1, 3.0)
    x = torch.tensor(seeded((SY, SX, H), 41)).pin_memory()
    y = torch.tensor(seeded((n, PX, H), 42)).pin_memory()
    y0 = torch.tensor(seeded((n, PX, H), 43)).pin_memory()
    x0 = torch.tensor(seeded((SY, SX, H), 44)).pin_memory()
    a = torch.tensor(ang)
    yo = y0.clone()
    _call("vp_forward_z0_host", x, yo, a)
    xo = x0.clone()
    _call("vp_backward_z0_host", y, xo, a)
    n_ext = max(SY, SX, PX)
    assert rel_err(yo.numpy() - y0.numpy(), oracle.forward(x.numpy(), ang, PX, 0)) <= \
        tol.ref_vs_fp64(n_ext)
    assert rel_err(xo.numpy() - x0.numpy(), oracle.backward(y.numpy(), ang, SY, SX, 0)) <= \
        tol.ref_vs_fp64(n_ext)


@pytest.mark.parametrize("trig", [0, 1])
def test_host_forward_angles_near_the_class_boundary(trig):
    """The host forward sends angles whose minor axis is x beyond doubt home
    before the column blocks run.  Angles at and around 45 and 135 degrees
    (inside and outside the margin), and large angles, must still come back
    complete."""
    offs = [0.0, 1e-6, -1e-6, 1e-4, -1e-4, 9e-4, -9e-4, 1.2e-3, -1.2e-3, 3e-3, -3e-3, 1e-2]
    base = [np.pi / 4, 3 * np.pi / 4, -np.pi / 4, 5 * np.pi / 4]
    ang = np.array([b + o for b in base for o in offs] + [15.0, -15.0, 15.7, 14.9, 0.0, 0.3],
                   dtype=np.float32)
    SY, SX, H, PX = 48, 40, 136, 60
    x = torch.tensor(seeded((SY, SX, H), 45)).pin_memory()
    y0 = torch.tensor(seeded((len(ang), PX, H), 46)).pin_memory()
    yo = y0.clone()
    flags = _lib.VP_FLAG_TRIG_PRECISE if trig else 0
    _call("vp_forward_z0_host", x, yo, torch.tensor(ang), flags)
    if trig:  # the fast sin/cos of the reference trig drift from FP64 at 15 rad
        ref = oracle.forward(x.numpy(), ang, PX, 0)
        assert rel_err(yo.numpy() - y0.numpy(), ref) <= tol.ref_vs_fp64(max(SY, SX, PX))
    # the device path: the same kernels and classes (an angle sent home
    # before its column blocks ran would differ by whole bins)
    xd, yd, ad = x.cuda(), y0.cuda(), torch.tensor(ang, device="cuda")
    _lib.check(_lib.LIB.vp_forward_z0(xd.data_ptr(), *xd.shape, yd.data_ptr(), *yd.shape,
                                      ad.data_ptr(), len(ang), flags,
                                      torch.cuda.current_stream().cuda_stream),
               "vp_forward_z0")
    torch.cuda.synchronize()
    assert rel_err(yo.numpy(), yd.cpu().numpy()) <= 4e-6


def test_height_extents_differ():
    """H = min(Hx, Hy): heights past the shorter array stay as they were
    (accumulate) or become zero (overwrite)."""
    SY, SX, n, PX = 18, 22, 14, 26
    ang = lin(n)
    x = torch.tensor(seeded((SY, SX, 12), 7))
    y0 = torch.tensor(seeded((n, PX, 20), 8))
    yo = y0.clone()
    _call("vp_forward_z0_host", x, yo, torch.tensor(ang))
    ref = oracle.forward(x.numpy(), ang, PX, 0)
    assert rel_err(yo.numpy()[:, :, :12] - y0.numpy()[:, :, :12], ref) <= tol.REF_VS_FP64
    np.testing.assert_array_equal(yo.numpy()[:, :, 12:], y0.numpy()[:, :, 12:])
    yw = y0.clone()
    _call("vp_forward_z0_host", x, yw, torch.tensor(ang), _lib.VP_FLAG_OVERWRITE)
    assert not yw[:, :, 12:].any()
    y = torch.tensor(seeded((n, PX, 8), 9))
    xw = torch.full((SY, SX, 12), 5.0)
    _call("vp_backward_z0_host", y, xw, torch.tensor(ang), _lib.VP_FLAG_OVERWRITE)
    assert not xw[:, :, 8:].any()
    assert rel_err(xw.numpy()[:, :, :8], oracle.backward(y.numpy(), ang, SY, SX, 0)) <= \
        tol.REF_VS_FP64


def test_wrappers_take_the_host_path_for_host_arrays():
    SY, SX, H, n = 40, 40, 16, 33
    ang = lin(n)
    x = seeded((SY, SX, H), 10)
    before = _lib.LIB.vp_launch_count()
    y = vp.forward(x, ang, None)  # numpy in, numpy out, overwrite
    assert isinstance(y, np.ndarray) and y.shape == (n, 40, H)
    assert rel_err(y, oracle.forward(x, ang, 40, 0)) <= tol.REF_VS_FP64
    # a float64 numpy container: accumulated into and returned
    c = np.ones((SY, SX, H))
    out = vp.backward(y, ang, c)
    assert out is c and out.dtype == np.float64
    assert rel_err(out - 1, oracle.backward(y, ang, SY, SX, 0)) <= tol.REF_VS_FP64
    # a CPU tensor in, a CPU tensor back
    t = vp.forward(torch.tensor(x), ang, (n, 40, H))
    assert isinstance(t, torch.Tensor) and not t.is_cuda
    assert rel_err(t.numpy(), y) <= 1e-6
    assert _lib.LIB.vp_launch_count() > before


def test_host_path_repeated_calls_reuse_pool():
    """Back-to-back calls (buffers freed and re-taken on the stream) give the
    same result every time."""
    SY, SX, H, n, PX = 64, 64, 136, 40, 64
    ang = torch.tensor(lin(n))
    x = torch.tensor(seeded((SY, SX, H), 11)).pin_memory()
    outs = []
    for _ in range(3):
        yo = torch.zeros(n, PX, H).pin_memory()
        _call("vp_forward_z0_host", x, yo, ang)
        outs.append(yo.clone())
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])


# z_order 2 (H, SY, SX): one chunk with the small-height kernels, two chunks
# through the transposed path, and chunks of 256 heights with a ragged last one
Z2_GEOMS = [(20, 24, 12, 30, 28), (33, 29, 100, 21, 40), (28, 26, 600, 17, 30)]


@pytest.mark.parametrize("geom", Z2_GEOMS, ids=lambda g: "x".join(map(str, g)))
def test_z2_host_entries(geom):
    SY, SX, H, n, PX = geom
    ang = lin(n, -0.2, 3.3)
    x = torch.tensor(seeded((H, SY, SX), 21)).pin_memory()
    y = torch.tensor(seeded((H, n, PX), 22)).pin_memory()
    y0 = torch.tensor(seeded((H, n, PX), 23)).pin_memory()
    x0 = torch.tensor(seeded((H, SY, SX), 24))
    a = torch.tensor(ang)
    yo = y0.clone()
    _call("vp_forward_z2_host", x, yo, a)
    xo = x0.clone()
    _call("vp_backward_z2_host", y, xo, a)
    n_ext = max(SY, SX, PX)
    assert rel_err(yo.numpy() - y0.numpy(), oracle.forward(x.numpy(), ang, PX, 2)) <= \
        tol.ref_vs_fp64(n_ext)
    assert rel_err(xo.numpy() - x0.numpy(), oracle.backward(y.numpy(), ang, SY, SX, 2)) <= \
        tol.ref_vs_fp64(n_ext)
    # the device z_order 2 path per chunk is the same arithmetic: equal
    yd = y0.cuda()
    vp._CU.forward_z2(x.cuda(), yd, a.cuda())
    xd = x0.cuda()
    vp._CU.backward_z2(y.cuda(), xd, a.cuda())
    torch.cuda.synchronize()
    assert rel_err(yo.numpy(), yd.cpu().numpy()) <= 4e-6
    assert rel_err(xo.numpy(), xd.cpu().numpy()) <= 4e-6
    # out = result, heights past the input's extent zeroed
    yw = torch.full((H + 8, n, PX), 3.0)
    _call("vp_forward_z2_host", x, yw, a, _lib.VP_FLAG_OVERWRITE)
    assert rel_err(yw.numpy()[:H], oracle.forward(x.numpy(), ang, PX, 2)) <= \
        tol.ref_vs_fp64(n_ext)
    assert not yw[H:].any()


@pytest.mark.parametrize("H", [100, 600])
def test_z2_host_overwrite_sinogram_larger_than_volume(H):
    """Out = result through the chunked pipeline, where a chunk of the
    sinogram (90 angles x 40 bins) is larger than a chunk of the volume
    (20 x 24), and back; two and three height chunks."""
    SY, SX, n, PX = 20, 24, 90, 40
    ang = lin(n, -0.4, 3.5)
    x = torch.tensor(seeded((H, SY, SX), 51)).pin_memory()
    y = torch.tensor(seeded((H, n, PX), 52)).pin_memory()
    a = torch.tensor(ang)
    yw = torch.full((H, n, PX), 9.0).pin_memory()
    _call("vp_forward_z2_host", x, yw, a, _lib.VP_FLAG_OVERWRITE)
    xw = torch.full((H, SY, SX), -2.0)
    _call("vp_backward_z2_host", y, xw, a, _lib.VP_FLAG_OVERWRITE)
    n_ext = max(SY, SX, PX)
    assert rel_err(yw.numpy(), oracle.forward(x.numpy(), ang, PX, 2)) <= tol.ref_vs_fp64(n_ext)
    assert rel_err(xw.numpy(), oracle.backward(y.numpy(), ang, SY, SX, 2)) <= \
        tol.ref_vs_fp64(n_ext)


def test_wrappers_take_the_host_path_for_z2():
    SY, SX, H, n = 30, 30, 40, 25
    ang = lin(n)
    x = seeded((H, SY, SX), 25)
    before = _lib.LIB.vp_launch_count()
    y = vp.forward(x, ang, None, z_order=2)
    assert isinstance(y, np.ndarray) and y.shape == (H, n, 30)
    assert rel_err(y, oracle.forward(x, ang, 30, 2)) <= tol.REF_VS_FP64
    xb = vp.backward(y, ang, None, z_order=2)
    assert rel_err(xb, oracle.backward(y, ang, 30, 30, 2)) <= tol.REF_VS_FP64
    assert _lib.LIB.vp_launch_count() > before
