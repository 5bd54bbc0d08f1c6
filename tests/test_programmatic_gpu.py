"""Programmatic dependent launches between a call's slab launches (forward)
and class launches (run adjoint).

Every slab launch after the first of a forward call, and the class-1 launch
of the run adjoint, may start while the launch before it runs; its warps
wait for that launch only to add into the output.  The sums are the same as
with launches one after another, which the batched kernels (one persistent
launch, stages ordered by counters, the same slab plan) reproduce bit for
bit.  The calls also work inside a CUDA graph capture.
"""

from __future__ import annotations

import pytest
import torch

import voxelproj_gb300 as vp
from tests.common import lin, seeded
from voxelproj_gb300 import _lib
from voxelproj_gb300.batch import Batch

pytestmark = pytest.mark.gpu

# volumes whose 256-height chunks take several 64 MB class slabs (3 and 2
# slab launches), angle counts that are not a multiple of the block's 4
# angles.  (Heights in whole 256-height chunks: a 4-height remainder runs the
# default's own 4-height form, which a batched variant-16 problem does not.)
GEOMS = [(300, 280, 512, 101, 320), (200, 210, 512, 45, 230)]


def _data(geom, seed):
    SY, SX, H, n, PX = geom
    ang = torch.tensor(lin(n, -0.3, 3.4), device="cuda")
    x = torch.tensor(seeded((SY, SX, H), seed), device="cuda")
    y = torch.tensor(seeded((n, PX, H), seed + 1), device="cuda")
    y0 = torch.tensor(seeded((n, PX, H), seed + 2), device="cuda")
    x0 = torch.tensor(seeded((SY, SX, H), seed + 3), device="cuda")
    return ang, x, y, y0, x0


@pytest.mark.parametrize("geom", GEOMS, ids=lambda g: "x".join(map(str, g)))
def test_programmatic_launches_equal_ordered_stages(geom):
    ang, x, y, y0, x0 = _data(geom, 900)
    # single calls with the defaults: forward variant 16 (programmatic slab
    # launches), run adjoint (programmatic class-1 launch), adding into
    # non-zero outputs
    ys, xs = y0.clone(), x0.clone()
    vp._CU.forward_z0(x, ys, ang)
    vp._CU.backward_z0(y, xs, ang)
    # the same plans in one persistent launch per body
    yb, xb = y0.clone(), x0.clone()
    b = Batch([("forward", x, yb, ang, 16), ("backward", y, xb, ang, 0)])
    b.run()
    torch.cuda.synchronize()
    assert not b.error()
    b.close()
    assert torch.equal(ys, yb)
    assert torch.equal(xs, xb)


def test_programmatic_launches_in_a_cuda_graph():
    ang, x, y, y0, x0 = _data(GEOMS[0], 910)
    yo, xo = y0.clone(), x0.clone()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    before = _lib.LIB.vp_launch_count()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            vp._CU.forward_z0(x, yo, ang)
            vp._CU.backward_z0(y, xo, ang)
    torch.cuda.current_stream().wait_stream(s)
    captured = _lib.LIB.vp_launch_count() - before
    torch.cuda.synchronize()
    assert torch.equal(yo, y0) and torch.equal(xo, x0)  # capturing does not execute
    assert captured > 2  # several slab launches and two class launches
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    ye, xe = y0.clone(), x0.clone()
    for _ in range(2):
        vp._CU.forward_z0(x, ye, ang)
        vp._CU.backward_z0(y, xe, ang)
    torch.cuda.synchronize()
    assert torch.equal(yo, ye)
    assert torch.equal(xo, xe)
