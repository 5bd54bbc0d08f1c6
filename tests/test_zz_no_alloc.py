"""vp_forward_z2_noalloc: the z_order 2 forward projection that allocates no
device memory.

It exists for callers that may not allocate device memory while they run:
code that fixes its memory at start-up, or hosts whose own allocator owns
the device.  Its scratch is a fixed array inside the library, not a pool
allocation.  The test drives it through the C ABI exactly as such a caller
would.  All buffers are made beforehand.  It checks that two calls in a row
give the same result as the allocating entry point vp_forward_z2.  It also
checks that a problem too large for the array is refused without touching
the output.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""

from __future__ import annotations

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
