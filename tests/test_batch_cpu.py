"""Host side of the batches on CPU: the seeded uneven-cube workload and the
Python checks made before a problem reaches the C ABI."""

from __future__ import annotations

import pytest
import torch

from voxelproj_gb300.batch import _problem, uneven_cubes


def test_uneven_cubes_seeded_and_in_range():
    a = uneven_cubes()
    assert a == uneven_cubes()  # the same workload every run
    assert len(a) == 64
    sides = set(range(64, 385, 32))
    assert all(s in sides and 90 <= n <= 720 for s, n in a)
    assert len({s for s, _ in a}) > 5  # uneven: many sizes
    assert uneven_cubes(seed=1) != a


def test_uneven_cubes_custom_ranges():
    got = uneven_cubes(10, seed=3, sides=(32, 48), nmin=5, nmax=6)
    assert len(got) == 10
    assert all(s in (32, 48) and n in (5, 6) for s, n in got)


def _fake_cuda(t):
    """t as a CPU tensor that reports itself as a CUDA tensor, so that the
    check of another argument is the one that fails (defined when used, so
    that collecting this file needs nothing of torch's subclassing)."""

    class FakeCuda(torch.Tensor):
        @property
        def is_cuda(self):
            return True

    return t.as_subclass(FakeCuda)


@pytest.mark.parametrize("name", ["in", "out", "angles"])
def test_problem_rejects_host_tensors(name):
    """Batched problems live on the device: a CPU tensor is refused by name
    before any pointer is taken."""
    tensors = {"in": torch.zeros(4, 4, 4), "out": torch.zeros(3, 4, 4), "angles": torch.zeros(3)}
    args = [t if k == name else _fake_cuda(t) for k, t in tensors.items()]
    with pytest.raises(RuntimeError, match=f"batch {name} must be"):
        _problem("forward", *args, 0)


def test_problem_rejects_non_3d_arrays():
    x = _fake_cuda(torch.zeros(4, 16))
    y = _fake_cuda(torch.zeros(3, 4, 4))
    a = _fake_cuda(torch.zeros(3))
    with pytest.raises(RuntimeError, match="3-D"):
        _problem("forward", x, y, a, 0)
