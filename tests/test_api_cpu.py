"""API behaviour that needs no GPU: the reference's error paths."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import voxelproj_gb300 as vp


def test_public_surface():
    for name in ["forward", "backward"]:
        assert callable(getattr(vp, name))
    for name in ["forward_z0", "backward_z0", "forward_z2", "backward_z2"]:
        assert callable(getattr(vp._CU, name))


def test_signatures_match_reference():
    """forward(x, angles, y, z_order=0, block_size=[8, 8, 8]) and
    backward(y, angles, x, ...) as in wrappers.py:28,76: the output argument
    is positional with no default."""
    import inspect

    for fn, names in ((vp.forward, ["x", "angles", "y"]), (vp.backward, ["y", "angles", "x"])):
        params = list(inspect.signature(fn).parameters.values())
        assert [p.name for p in params] == names + ["z_order", "block_size"]
        assert all(p.default is inspect.Parameter.empty for p in params[:3])
        assert params[3].default == 0
        assert params[4].default == [8, 8, 8]
    with pytest.raises(TypeError):
        vp.forward(np.zeros((4, 4, 2), np.float32), np.zeros(3, np.float32))
    # the extension's functions: (in, out, angles, block_size=[8, 8, 8]); the
    # default is held as a tuple (block_size is accepted and ignored)
    for name in ["forward_z0", "backward_z0", "forward_z2", "backward_z2"]:
        params = list(inspect.signature(getattr(vp._CU, name)).parameters.values())
        assert len(params) == 4 and list(params[3].default) == [8, 8, 8]


@pytest.mark.parametrize("z", [1, 3, -1])
def test_bad_z_order_raises_key_error(z):
    # the reference dispatches through a dict (wrappers.py:44-47)
    x = np.zeros((4, 4, 2), np.float32)
    with pytest.raises(KeyError):
        vp.forward(x, np.zeros(3, np.float32), None, z_order=z)
    with pytest.raises(KeyError):
        vp.backward(x, np.zeros(4, np.float32), None, z_order=z)


@pytest.mark.parametrize("fn", ["forward_z0", "backward_z0", "forward_z2", "backward_z2"])
def test_extension_rejects_cpu_input(fn):
    # projectors.cu:36: TORCH_CHECK(in.is_cuda(), "Tensor must be on CUDA")
    with pytest.raises(RuntimeError, match="Tensor must be on CUDA"):
        getattr(vp._CU, fn)(torch.zeros(2, 2, 2), torch.zeros(2, 2, 2), torch.zeros(2))


def test_trig_mode_switch():
    assert vp.get_trig_mode() == "reference"
    vp.set_trig_mode("precise")
    assert vp.get_trig_mode() == "precise"
    vp.set_trig_mode("reference")
    with pytest.raises(ValueError):
        vp.set_trig_mode("fast")


def test_angle_cache_reuses_device_copies_by_content():
    """Host angles are copied to the device once per distinct content; an
    array changed in place, another dtype with other values, or another
    device is a new entry; the cache is bounded."""
    import torch

    from voxelproj_gb300 import wrappers as w

    w._ANGLE_CACHE.clear()
    a = np.linspace(0, np.pi, 7).astype(np.float32)
    t1 = w.cached_angles(a, "cpu")
    assert t1.dtype == torch.float32 and t1.shape == (7,)
    assert w.cached_angles(a.copy(), "cpu") is t1          # same bytes
    assert w.cached_angles(list(a), "cpu") is t1            # a list of the same values
    ta = torch.tensor(a)                                    # a tensor already on the device:
    assert torch.equal(w.cached_angles(ta, "cpu"), t1)      # used as it is, not cached
    a[3] += 1e-3                                            # changed in place
    t2 = w.cached_angles(a, "cpu")
    assert t2 is not t1 and float(t2[3]) == float(np.float32(a[3]))
    np.testing.assert_array_equal(t1.numpy()[[0, 1, 2, 4, 5, 6]], t2.numpy()[[0, 1, 2, 4, 5, 6]])
    b = a.astype(np.float64)                                # same float32 values
    assert w.cached_angles(b, "cpu") is t2
    for k in range(w._ANGLE_CACHE_SIZE + 5):
        w.cached_angles(np.full(3, k, np.float32), "cpu")
    assert len(w._ANGLE_CACHE) == w._ANGLE_CACHE_SIZE
    w._ANGLE_CACHE.clear()
