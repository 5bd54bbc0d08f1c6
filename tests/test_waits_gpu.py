"""Bounded device waits driven to their limits, on purpose and without any fault.

Every wait in this library's kernels gives up after a bounded time, records
that it did, and the kernel goes on.  These tests lower the limits with
``vp_set_wait_limits`` so that waits run out:

* batch stage waits: every later-stage task waits for one completion more
  than the stage before it gives, a count that nothing reaches.  Each wait
  gives up after ~17 us; the plan's error flag reads 1, the kernel returns
  and the output is finite.
* the staged adjoint's copy waits (backward z0 variant 9): with zero polls
  every wait on a bulk copy gives up at once.  Each block falls back to
  plain loads, so the result is still the plain run adjoint's bit for bit,
  and ``vp_wait_timeouts`` counts the waits that gave up.

The default limits are restored afterwards, and a fresh run is clean.
"""

from __future__ import annotations

import pytest
import torch

import voxelproj_gb300 as vp
from tests.common import lin, seeded
from voxelproj_gb300 import _lib
from voxelproj_gb300.batch import FORWARD_DEFAULT, Batch

pytestmark = pytest.mark.gpu

WAIT_DEFAULT = 0xFFFFFFFF


def restore_defaults():
    assert _lib.LIB.vp_set_wait_limits(WAIT_DEFAULT, 0, 0) == 0


def _batch_problems():
    # forward: a volume of two class slabs of 256-height chunks (two stages);
    # adjoint: the run adjoint's two angle classes (two stages)
    geoms = [(200, 200, 132, 16, 200), (40, 40, 132, 61, 57)]
    problems, outs, refs = [], [], []
    for i, (SY, SX, H, n, PX) in enumerate(geoms):
        a = torch.tensor(lin(n, -0.4, 3.5), device="cuda")
        x = torch.tensor(seeded((SY, SX, H), 500 + i), device="cuda")
        y = torch.tensor(seeded((n, PX, H), 600 + i), device="cuda")
        yo = torch.zeros((n, PX, H), device="cuda")
        xo = torch.zeros((SY, SX, H), device="cuda")
        problems += [("forward", x, yo, a, 0), ("backward", y, xo, a, 0)]
        outs += [yo, xo]
        refs.append((x, y, a))
    return problems, outs, refs


def test_batch_stage_waits_run_out_and_report():
    problems, outs, refs = _batch_problems()
    b = Batch(problems)
    try:
        assert _lib.LIB.vp_set_wait_limits(WAIT_DEFAULT, 64, 1) == 0
        b.run()
        torch.cuda.synchronize()  # the kernels returned
    finally:
        restore_defaults()
    assert b.error(), "a stage wait that cannot be satisfied must report"
    for o in outs:
        assert torch.isfinite(o).all()
    b.close()

    # defaults back: a new plan of the same problems runs clean and equals
    # the single-problem calls
    for o in outs:
        o.zero_()
    b2 = Batch(problems)
    b2.run()
    torch.cuda.synchronize()
    assert not b2.error()
    _lib.LIB.vp_set_kernel_variant(0, FORWARD_DEFAULT)  # the batch's forward default
    try:
        for (x, y, a), yo, xo in zip(refs, outs[0::2], outs[1::2]):
            ys = torch.zeros_like(yo)
            xs = torch.zeros_like(xo)
            vp._CU.forward_z0(x, ys, a)
            vp._CU.backward_z0(y, xs, a)
            torch.cuda.synchronize()
            assert torch.equal(yo, ys) and torch.equal(xo, xs)
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
    b2.close()


@pytest.mark.parametrize("geom", [(48, 40, 512, 70, 52), (33, 29, 256, 45, 40)],
                         ids=lambda g: "x".join(map(str, g)))
def test_staged_adjoint_copy_waits_run_out_and_fall_back(geom):
    SY, SX, H, n, PX = geom
    ang = torch.tensor(lin(n, -0.3, 3.3), device="cuda")
    y = torch.tensor(seeded((n, PX, H), 700), device="cuda")
    x0 = torch.tensor(seeded((SY, SX, H), 701), device="cuda")
    outs = {}
    try:
        _lib.LIB.vp_set_kernel_variant(1, 7)
        xo = x0.clone()
        vp._CU.backward_z0(y, xo, ang)
        outs["plain"] = xo
        before = _lib.LIB.vp_wait_timeouts()
        _lib.LIB.vp_set_kernel_variant(1, 9)
        assert _lib.LIB.vp_set_wait_limits(0, 0, 0) == 0
        xo = x0.clone()
        vp._CU.backward_z0(y, xo, ang)
        torch.cuda.synchronize()  # the kernels returned
        outs["gave_up"] = xo
        gave_up = _lib.LIB.vp_wait_timeouts() - before
        restore_defaults()
        before = _lib.LIB.vp_wait_timeouts()
        xo = x0.clone()
        vp._CU.backward_z0(y, xo, ang)
        torch.cuda.synchronize()
        outs["staged"] = xo
        clean = _lib.LIB.vp_wait_timeouts() - before
    finally:
        restore_defaults()
        _lib.LIB.vp_set_kernel_variant(1, 0)
    print(f"\n[waits] {geom}: {gave_up} copy waits gave up with zero polls, {clean} with the "
          f"default")
    assert gave_up > 0
    assert clean == 0
    assert torch.equal(outs["gave_up"], outs["plain"])
    assert torch.equal(outs["staged"], outs["plain"])


def test_staged_forward_copy_waits_run_out_and_fall_back():
    """The staged forward (variant 17) with zero polls: every wait on a
    line's copy gives up at once, the block reads global memory instead, and
    the result is still variant 10's bit for bit."""
    SY, SX, H, n, PX = 96, 80, 256, 61, 100
    ang = torch.tensor(lin(n), device="cuda")
    x = torch.tensor(seeded((SY, SX, H), 702), device="cuda")
    y0 = torch.tensor(seeded((n, PX, H), 703), device="cuda")
    outs = {}
    try:
        _lib.LIB.vp_set_kernel_variant(0, 10)
        yo = y0.clone()
        vp._CU.forward_z0(x, yo, ang)
        outs["plain"] = yo
        _lib.LIB.vp_set_kernel_variant(0, 17)
        before = _lib.LIB.vp_wait_timeouts()
        assert _lib.LIB.vp_set_wait_limits(0, 0, 0) == 0
        yo = y0.clone()
        vp._CU.forward_z0(x, yo, ang)
        torch.cuda.synchronize()
        outs["gave_up"] = yo
        gave_up = _lib.LIB.vp_wait_timeouts() - before
        restore_defaults()
        before = _lib.LIB.vp_wait_timeouts()
        yo = y0.clone()
        vp._CU.forward_z0(x, yo, ang)
        torch.cuda.synchronize()
        outs["staged"] = yo
        clean = _lib.LIB.vp_wait_timeouts() - before
    finally:
        restore_defaults()
        _lib.LIB.vp_set_kernel_variant(0, 0)
    print(f"\n[waits] staged forward: {gave_up} copy waits gave up with zero polls, {clean} "
          f"with the default")
    assert gave_up > 0 and clean == 0
    assert torch.equal(outs["gave_up"], outs["plain"])
    assert torch.equal(outs["staged"], outs["plain"])
