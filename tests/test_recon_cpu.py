"""Host-side parts of the reconstruction layer (no GPU)."""

from __future__ import annotations

import torch

from voxelproj_gb300.recon import ellipsoid_phantom


def test_ellipsoid_phantom_cpu():
    ph = ellipsoid_phantom(32, count=20, seed=0, device="cpu")
    assert ph.shape == (32, 32, 32) and ph.dtype == torch.float32
    assert float(ph.min()) >= 0.0 and float(ph.max()) <= 20.0
    frac = float((ph > 0).float().mean())
    assert 0.01 < frac < 0.9
    # deterministic for a seed
    assert torch.equal(ph, ellipsoid_phantom(32, count=20, seed=0, device="cpu"))
