"""Batched persistent launches, CUDA-graph replay and the autotuner."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import voxelproj_gb300 as vp
from oracle import oracle
from tests import tolerances as tol
from tests.common import lin, rel_err, seeded
from voxelproj_gb300 import _lib
from voxelproj_gb300.batch import FORWARD_DEFAULT, Batch, uneven_cubes

pytestmark = pytest.mark.gpu

# (SY, SX, H, n_ang, PX) per problem: uneven sizes, rectangular volumes,
# detectors wider and narrower, more than one height chunk
GEOMS = [(24, 32, 8, 45, 40), (40, 40, 132, 61, 57), (9, 6, 4, 20, 11), (64, 48, 16, 90, 64)]


def _inputs(geoms, seed):
    out = []
    for i, (SY, SX, H, n, PX) in enumerate(geoms):
        ang = lin(n, -0.4, 3.5)
        out.append(dict(geom=(SY, SX, H, n, PX), ang=ang,
                        x=seeded((SY, SX, H), seed + 3 * i), y=seeded((n, PX, H), seed + 3 * i + 1),
                        y0=seeded((n, PX, H), seed + 3 * i + 2)))
    return out


@pytest.mark.parametrize("vf,vb", [(1, 4), (1, 6), (0, 0), (10, 7), (5, 6), (12, 7), (21, 7),
                                   (16, 6), (3, 4), (22, 7)])
def test_batch_matches_single_problem_calls(vf, vb):
    """Same bodies, same slabs and stages, same order: the batch reproduces the
    single-problem kernels of the same variant bit for bit."""
    cases = _inputs(GEOMS, 100)
    problems, outs = [], []
    for c in cases:
        a = torch.tensor(c["ang"], device="cuda")
        x = torch.tensor(c["x"], device="cuda")
        y = torch.tensor(c["y"], device="cuda")
        yo = torch.tensor(c["y0"], device="cuda")  # accumulate into non-zero content
        xo = torch.zeros_like(x)
        problems += [("forward", x, yo, a, vf), ("backward", y, xo, a, vb)]
        outs.append((yo, xo))
    b = Batch(problems)
    b.run()
    torch.cuda.synchronize()
    assert not b.error()
    # the single-problem kernels of the same variants (a batched forward of
    # variant 0 runs FORWARD_DEFAULT)
    _lib.LIB.vp_set_kernel_variant(0, vf or FORWARD_DEFAULT)
    _lib.LIB.vp_set_kernel_variant(1, vb)
    try:
        for c, (yo, xo) in zip(cases, outs):
            SY, SX, H, n, PX = c["geom"]
            a = torch.tensor(c["ang"], device="cuda")
            xs = torch.zeros_like(xo)
            vp._CU.backward_z0(torch.tensor(c["y"], device="cuda"), xs, a)
            ys = torch.tensor(c["y0"], device="cuda")
            vp._CU.forward_z0(torch.tensor(c["x"], device="cuda"), ys, a)
            torch.cuda.synchronize()
            assert torch.equal(xo, xs)
            assert torch.equal(yo, ys)
            Ax = oracle.forward(c["x"], c["ang"], PX, 0)
            assert rel_err(yo.cpu().numpy() - c["y0"], Ax) <= tol.ref_vs_fp64(max(SY, SX, PX))
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
        _lib.LIB.vp_set_kernel_variant(1, 0)
    b.close()


def test_batch_stages_on_large_problems():
    """Problems with several volume slabs (forward stages) and both angle
    classes (adjoint stages) in one launch, 8 heights per lane on a whole
    256-height chunk (the constant-offset bodies) and a 4-height part for the
    last 4 heights, against single-problem calls."""
    probs, refs = [], []
    for side, n in [(320, 60), (200, 45), (96, 30)]:
        a = torch.linspace(0, np.pi, n + 1, device="cuda")[:-1].contiguous()
        x = torch.randn(side, side, 260, device="cuda")
        y = torch.randn(n, side, 260, device="cuda")
        yo = torch.zeros(n, side, 260, device="cuda")
        xo = torch.zeros(side, side, 260, device="cuda")
        probs += [("forward", x, yo, a), ("backward", y, xo, a)]
        refs.append((x, y, yo, xo, a))
    b = Batch(probs)
    b.run()
    b.run()  # runs accumulate: every output is now twice the operator
    torch.cuda.synchronize()
    assert not b.error()
    # default variants on both sides: the batch's forward default is
    # FORWARD_DEFAULT
    _lib.LIB.vp_set_kernel_variant(0, FORWARD_DEFAULT)
    try:
        for x, y, yo, xo, a in refs:
            ys = torch.zeros_like(yo)
            xs = torch.zeros_like(xo)
            for _ in range(2):
                vp._CU.forward_z0(x, ys, a)
                vp._CU.backward_z0(y, xs, a)
            torch.cuda.synchronize()
            assert torch.equal(yo, ys)
            assert torch.equal(xo, xs)
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
        _lib.LIB.vp_set_kernel_variant(1, 0)
    b.close()


def test_batch_graph_replays_accumulate():
    c = _inputs([(30, 30, 8, 40, 36)], 200)[0]
    a = torch.tensor(c["ang"], device="cuda")
    x = torch.tensor(c["x"], device="cuda")
    yo = torch.zeros(40, 36, 8, device="cuda")
    b = Batch([("forward", x, yo, a)])
    g = b.graph()
    torch.cuda.synchronize()
    assert float(yo.abs().sum()) == 0.0  # capturing does not execute
    g.replay()
    torch.cuda.synchronize()
    once = yo.clone()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert rel_err(yo.cpu().numpy(), 3 * once.cpu().numpy()) < 1e-6
    assert rel_err(once.cpu().numpy(), oracle.forward(c["x"], c["ang"], 36, 0)) <= tol.REF_VS_FP64
    b.close()


def test_batch_launches_one_kernel_per_body():
    """Problems of both directions and all height forms (4 per lane; 8 per
    lane on a part of whole 256-height chunks; 8 per lane on 200 heights):
    one persistent launch per body, six in all for any number of problems."""
    probs = []
    for side, H in [(40, 64), (36, 260), (48, 96), (30, 264), (28, 200)]:
        a = torch.linspace(0, np.pi, 20, device="cuda")
        x = torch.randn(side, side, H, device="cuda")
        y = torch.randn(20, side, H, device="cuda")
        probs += [("forward", x, torch.zeros_like(y), a), ("backward", y, torch.zeros_like(x), a)]
    b = Batch(probs)
    before = _lib.LIB.vp_launch_count()
    b.run()
    torch.cuda.synchronize()
    assert _lib.LIB.vp_launch_count() - before == 6
    assert not b.error()
    b.close()


def test_batch_one_launch_for_many_problems():
    shapes = uneven_cubes(6, seed=1, sides=(32, 64, 96), nmin=10, nmax=40)
    problems = []
    for side, n in shapes:
        a = torch.linspace(0, np.pi, n + 1, device="cuda")[:-1].contiguous()
        x = torch.randn(side, side, side, device="cuda")
        problems.append(("forward", x, torch.zeros(n, side, side, device="cuda"), a))
    b = Batch(problems)
    before = _lib.LIB.vp_launch_count()
    b.run()
    torch.cuda.synchronize()
    assert _lib.LIB.vp_launch_count() - before == 1
    assert b.work_items > len(problems)
    b.close()


def test_batch_rejects_unsupported_problems():
    a = torch.tensor(lin(10), device="cuda")
    x = torch.zeros(8, 8, 6, device="cuda")  # heights not a multiple of 4
    with pytest.raises(RuntimeError):
        Batch([("forward", x, torch.zeros(10, 8, 6, device="cuda"), a)])
    with pytest.raises(KeyError):
        Batch([("sideways", x, x, a)])
    # forward variant 13 (two warps per bin run) has no batched body: a
    # batch could not reproduce it bit for bit, so it is refused
    x4 = torch.zeros(8, 8, 8, device="cuda")
    with pytest.raises(RuntimeError):
        Batch([("forward", x4, torch.zeros(10, 8, 8, device="cuda"), a, 13)])
    empty = Batch([])
    empty.run()
    empty.close()


def test_autotuner_caches(tmp_path, monkeypatch):
    from voxelproj_gb300 import tune

    monkeypatch.setenv("VOXELPROJ_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    v = tune.batch_variant("forward", 64, 120)
    assert v in tune.BATCH_CANDIDATES["forward"]
    assert tune.batch_variant("forward", 64, 500) == v  # cached per side
    vb = tune.tune_single("backward", (48, 48, 128), (60, 48, 128))
    assert vb in tune.SINGLE_CANDIDATES["backward"]
    assert _lib.LIB.vp_get_kernel_variant(1) == vb
    _lib.LIB.vp_set_kernel_variant(1, 0)
    assert (tmp_path / "tune.json").exists()


def test_batch_update_replans_in_place():
    """vp_batch_update re-plans an existing plan for another set of problems:
    a larger set (buffers grow), a smaller one, and a set with an invalid
    problem (refused, plan unchanged).  Each run equals the single-problem
    calls; runs enqueued before an update keep their problems."""
    cases = _inputs(GEOMS, 300)

    def make(sel):
        probs, outs = [], []
        for i in sel:
            c = cases[i]
            a = torch.tensor(c["ang"], device="cuda")
            x = torch.tensor(c["x"], device="cuda")
            y = torch.tensor(c["y"], device="cuda")
            yo, xo = torch.zeros_like(y), torch.zeros_like(x)
            probs += [("forward", x, yo, a), ("backward", y, xo, a)]
            outs.append((x, y, a, yo, xo))
        return probs, outs

    def check(outs):
        _lib.LIB.vp_set_kernel_variant(0, FORWARD_DEFAULT)
        try:
            for x, y, a, yo, xo in outs:
                ys, xs = torch.zeros_like(yo), torch.zeros_like(xo)
                vp._CU.forward_z0(x, ys, a)
                vp._CU.backward_z0(y, xs, a)
                torch.cuda.synchronize()
                assert torch.equal(yo, ys) and torch.equal(xo, xs)
        finally:
            _lib.LIB.vp_set_kernel_variant(0, 0)

    p1, o1 = make([2])
    b = Batch(p1)
    b.run()                      # enqueued before the update: keeps problem 2
    p2, o2 = make([0, 1, 2, 3])  # more problems than the plan was made for
    b.update(p2)
    b.run()
    torch.cuda.synchronize()
    check(o1)
    check(o2)
    p3, o3 = make([1])
    b.update(p3)
    b.run()
    torch.cuda.synchronize()
    check(o3)
    bad = [("forward", p3[0][1], p3[0][2][:, :, :3].contiguous(), p3[0][3])]  # heights % 4
    with pytest.raises(RuntimeError):
        b.update(bad)
    for _, _, _, yo, xo in o3:
        yo.zero_()
        xo.zero_()
    b.run()                      # still the previous set
    torch.cuda.synchronize()
    check(o3)
    assert not b.error()
    b.close()
