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
