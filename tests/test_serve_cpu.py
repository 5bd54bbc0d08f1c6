"""Admission rules of the reconstruction server (host only, no GPU)."""

from __future__ import annotations

import pytest
import torch

from voxelproj_gb300.serve import ReconstructionServer, Request


def _req(rid, side, n, method="sirt", arrival=0.0):
    b = torch.zeros(n, side, side)  # host tensor: only shapes matter here
    return Request(rid, b, torch.zeros(n), (side, side), 10, method, arrival=arrival)


def test_footprint_counts_resident_buffers():
    r = _req(0, 64, 100)
    nv, ns = 64 ** 3, 100 * 64 * 64
    assert r.footprint() == 4 * (4 * nv + 5 * ns)
    assert _req(1, 64, 100, "cgls").footprint() == 4 * (3 * nv + 3 * ns)


def test_submit_rejects_what_can_never_run():
    srv = ReconstructionServer(budget_bytes=1 << 20)
    with pytest.raises(ValueError):
        srv.submit(_req(0, 64, 100))  # larger than the whole budget
    with pytest.raises(ValueError):
        srv.submit(Request(1, torch.zeros(10, 8, 6), torch.zeros(10), (8, 8), 3))  # H % 4
    with pytest.raises(ValueError):
        srv.submit(_req(2, 8, 4, method="art"))


def test_queue_is_arrival_ordered():
    srv = ReconstructionServer(budget_bytes=1 << 30)
    for rid, t in [(0, 0.5), (1, 0.1), (2, 0.3)]:
        srv.submit(_req(rid, 8, 4, arrival=t))
    assert [q[2].rid for q in sorted(srv.queue)] == [1, 2, 0]


def test_admission_order_fifo_and_shortest_work_first():
    """fifo takes the earliest arrival; sjf the arrived request with the least
    total work (iterations x voxels x angles), arrival-independent."""
    reqs = [(_req(0, 32, 40, arrival=0.0), 0), (_req(1, 16, 20, arrival=0.1), 0),
            (_req(2, 8, 8, arrival=5.0), 0)]
    for policy, expect in (("fifo", 0), ("sjf", 1)):
        srv = ReconstructionServer(budget_bytes=1 << 34, policy=policy)
        for r, _ in reqs:
            srv.submit(r)
        i = srv._next(1.0)  # request 2 has not arrived yet
        assert srv.queue[i][2].rid == expect
    srv = ReconstructionServer(budget_bytes=1 << 34, policy="sjf")
    assert srv._next(0.0) is None
    assert ReconstructionServer.work(_req(3, 8, 4)) == 2 * 10 * 8 * 8 * 8 * 4
    with pytest.raises(ValueError):
        ReconstructionServer(budget_bytes=1, policy="lifo")
    with pytest.raises(ValueError):
        ReconstructionServer(budget_bytes=1, launch="never")
