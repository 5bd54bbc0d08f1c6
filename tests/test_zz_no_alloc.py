"""vp_forward_z2_noalloc: the z_order 2 forward projection that allocates no
device memory.

It exists for callers that may not allocate device memory while they run:
code that fixes its memory at start-up, or hosts whose own allocator owns
the device.  Its scratch is a fixed array inside the library, not a pool
allocation.  The tests drive it through the C ABI exactly as such a caller
would, with every buffer made beforehand.  They check that:
* two calls in a row give the result of the allocating entry point
  vp_forward_z2, bit for bit;
* what one call leaves in the shared array never reaches a later call's
  output: a call on a NaN volume fills most of the array, then a call with
  61 heights (padded to 64 inside the array, so pad heights hold NaN
  leftovers) and another geometry still matches vp_forward_z2 bit for bit;
* repeated calls allocate nothing: in a fresh process that never calls an
  allocating entry point, the device's free memory does not move across
  calls of growing size;
* a problem too large for the array is refused without touching the output.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

from tests import tolerances as tol
from tests.common import lin, rel_err, seeded

pytestmark = pytest.mark.gpu


def _call(fn, x, y, a):
    stream = torch.cuda.current_stream().cuda_stream
    return fn(x.data_ptr(), *x.shape, y.data_ptr(), *y.shape, a.data_ptr(), a.numel(), 0, stream)


def test_noalloc_matches_allocating_entry_point_twice():
    from voxelproj_gb300 import _lib

    # heights >= 32 take the transposed path, which is the one needing scratch
    H, SY, SX, n, PX = 64, 40, 48, 50, 60
    assert 0 < _lib.LIB.vp_z2_workspace_bytes(H, SY, SX, H, n, PX) <= _lib.VP_NOALLOC_SCRATCH_BYTES
    x = torch.tensor(seeded((H, SY, SX), 71), device="cuda")
    a = torch.tensor(lin(n, -0.3, 3.0), device="cuda")
    y0 = seeded((H, n, PX), 72)

    y_ref = torch.tensor(y0, device="cuda")
    assert _call(_lib.LIB.vp_forward_z2, x, y_ref, a) == _lib.VP_OK
    outs = [torch.tensor(y0, device="cuda") for _ in range(2)]
    for y in outs:  # two calls in a row, sharing the library's scratch array
        assert _call(_lib.LIB.vp_forward_z2_noalloc, x, y, a) == _lib.VP_OK
    torch.cuda.synchronize()
    ref = y_ref.cpu().numpy()
    for y in outs:
        got = y.cpu().numpy()
        assert rel_err(got - y0, ref - y0) <= tol.REF_VS_REFERENCE
        np.testing.assert_array_equal(got, ref)


def test_noalloc_leftovers_never_reach_the_output():
    from voxelproj_gb300 import _lib

    # fill most of the array with NaN: a NaN volume, transposed and projected
    H, SY, SX, n, PX = 96, 256, 256, 200, 256
    need = _lib.LIB.vp_z2_workspace_bytes(H, SY, SX, H, n, PX)
    assert _lib.VP_NOALLOC_SCRATCH_BYTES // 2 < need <= _lib.VP_NOALLOC_SCRATCH_BYTES
    x = torch.full((H, SY, SX), float("nan"), device="cuda")
    y = torch.zeros((H, n, PX), device="cuda")
    a = torch.tensor(lin(n), device="cuda")
    assert _call(_lib.LIB.vp_forward_z2_noalloc, x, y, a) == _lib.VP_OK
    torch.cuda.synchronize()
    assert bool(torch.isnan(y).any())

    # then heights not a multiple of 4 and another geometry
    H, SY, SX, n, PX = 61, 37, 45, 53, 70
    x = torch.tensor(seeded((H, SY, SX), 73), device="cuda")
    a = torch.tensor(lin(n, 0.1, 3.4), device="cuda")
    y0 = seeded((H, n, PX), 74)
    y_ref = torch.tensor(y0, device="cuda")
    assert _call(_lib.LIB.vp_forward_z2, x, y_ref, a) == _lib.VP_OK
    y = torch.tensor(y0, device="cuda")
    assert _call(_lib.LIB.vp_forward_z2_noalloc, x, y, a) == _lib.VP_OK
    torch.cuda.synchronize()
    assert bool(torch.isfinite(y).all())
    assert torch.equal(y, y_ref)


# Run in a fresh process: only the no-allocation entry point is called, so
# no library pool exists that could serve a hidden allocation unnoticed.
_FREE_MEMORY_PROBE = r"""
import ctypes, sys
import torch
sys.path.insert(0, sys.argv[1])
from voxelproj_gb300 import _lib
from tests.common import lin, seeded

def call(H, SY, SX, n, PX):
    x = torch.tensor(seeded((H, SY, SX), H), device="cuda")
    y = torch.zeros((H, n, PX), device="cuda")
    a = torch.tensor(lin(n), device="cuda")
    return x, y, a

problems = [call(*g) for g in [(32, 16, 16, 8, 16), (40, 64, 64, 90, 64),
                               (64, 128, 128, 180, 128), (96, 200, 200, 128, 220)]]
torch.cuda.synchronize()
stream = torch.cuda.current_stream().cuda_stream

def run(x, y, a):
    st = _lib.LIB.vp_forward_z2_noalloc(x.data_ptr(), *x.shape, y.data_ptr(), *y.shape,
                                        a.data_ptr(), a.numel(), 0, stream)
    assert st == 0, st

run(*problems[0])  # first call: the library's code and array load, address looked up
torch.cuda.synchronize()
free0, _ = torch.cuda.mem_get_info()
for p in problems * 2:  # growing sizes, twice
    run(*p)
torch.cuda.synchronize()
free1, _ = torch.cuda.mem_get_info()
print(free0, free1)
assert free1 == free0, (free0, free1)
"""


def test_noalloc_allocates_nothing_across_calls():
    root = Path(__file__).resolve().parent.parent
    # modules load eagerly, so that no kernel's first launch loads code mid-way
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    res = subprocess.run([sys.executable, "-c", _FREE_MEMORY_PROBE, str(root)], cwd=root,
                         capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stdout + res.stderr


def test_noalloc_refuses_problems_beyond_its_array():
    from voxelproj_gb300 import _lib

    H, SY, SX, n, PX = 256, 256, 256, 64, 256  # needs 80 MiB of scratch
    need = _lib.LIB.vp_z2_workspace_bytes(H, SY, SX, H, n, PX)
    assert need > _lib.VP_NOALLOC_SCRATCH_BYTES
    x = torch.zeros((H, SY, SX), device="cuda")
    y = torch.full((H, n, PX), 5.0, device="cuda")
    a = torch.tensor(lin(n), device="cuda")
    assert _call(_lib.LIB.vp_forward_z2_noalloc, x, y, a) == _lib.VP_ERR_SCRATCH_LIMIT
    torch.cuda.synchronize()
    assert bool((y == 5.0).all())
