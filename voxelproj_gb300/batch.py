"""Batched projections in persistent launches, replayable as a CUDA graph.

    b = Batch([("forward", x1, y1, angles1), ("backward", y2, x2, angles2, 4), ...])
    b.run()                 # one persistent launch per body present (at most 6)
    g = b.graph()           # CUDA graph of the same launches
    g.replay()

Each problem is (op, in, out, angles[, variant]): op "forward" adds A in to
out, "backward" adds A^T in to out.  The tensors are CUDA float32 in z_order 0
layout (x (SY, SX, H), y (n_ang, PX, H)) with H a multiple of 4; the batch
keeps references to them.  Variants are single-problem kernel variants
(None: the library default, for the forward FORWARD_DEFAULT; the benchmark
below asks the autotuner) and
select each problem's work-item body, heights per lane and volume slabs, so
a batched problem's result equals the single-problem call of that variant.
A body is the forward or the run adjoint with 4 or 8 heights per lane; each
body present runs as one persistent kernel over all its problems' work items.

    python -m voxelproj_gb300.batch

runs the uneven-batch workload: 64 cubes with sides drawn from
{64, 96, ..., 384} and U{90..720} angles each, A for every cube and A^T for
every sinogram, in persistent launches replayed as a CUDA graph, next to
the same work issued as sequential single-problem calls.  It prints one JSON
line.
"""

from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np
import torch

from . import _lib

_OPS = {"forward": _lib.VP_OP_FORWARD, "backward": _lib.VP_OP_BACKWARD}

# The single-problem forward variant that a batched forward problem of variant
# 0 (or None) runs, VP_BATCH_FORWARD_DEFAULT in the C header: its results
# equal single-problem calls of this variant bit for bit.
FORWARD_DEFAULT = 21


def _problem(op, inp, out, angles, variant):
    for t, name in ((inp, "in"), (out, "out"), (angles, "angles")):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32
                and t.is_contiguous()):
            raise RuntimeError(f"batch {name} must be a contiguous float32 CUDA tensor")
    if inp.dim() != 3 or out.dim() != 3:
        raise RuntimeError("batch in/out must be 3-D (z_order 0 layout)")
    p = _lib.BatchProblem()
    p.op = _OPS[op]
    p.flags = 0
    p.variant = int(variant or 0)
    p.in_ = inp.data_ptr()
    p.out = out.data_ptr()
    p.angles = angles.data_ptr()
    p.n_angles = angles.numel()
    p.in_dims[:] = list(inp.shape)
    p.out_dims[:] = list(out.shape)
    return p


class Batch:
    """A fixed batch of projection problems (see the module docstring)."""

    def __init__(self, problems, device=None):
        keep, arr, n = self._convert(problems)
        self._keep = keep
        self.device = torch.device(device) if device is not None else (
            keep[0][0].device if keep else torch.device("cuda"))
        self._plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.LIB.vp_batch_create(arr, n, ctypes.byref(self._plan)),
                       "batch_create")
        self.work_items = int(_lib.LIB.vp_batch_work_items(self._plan))

    @staticmethod
    def _convert(problems):
        keep, probs = [], []
        for spec in problems:
            op, inp, out, angles = spec[:4]
            variant = spec[4] if len(spec) > 4 else None
            if op not in _OPS:
                raise KeyError(op)
            probs.append(_problem(op, inp, out, angles, variant))
            keep.append((inp, out, angles))
        arr = (_lib.BatchProblem * max(1, len(probs)))(*probs)
        return keep, arr, len(probs)

    def update(self, problems, stream=None):
        """Replace the batch's problems (as given to the constructor) without
        synchronising (``vp_batch_update``): the new descriptors go up on
        `stream` (default: the current stream), after the runs already
        enqueued there and before the runs enqueued next."""
        keep, arr, n = self._convert(problems)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.LIB.vp_batch_update(self._plan, arr, n, s.cuda_stream),
                       "batch_update")
        self._keep = keep
        self.work_items = int(_lib.LIB.vp_batch_work_items(self._plan))

    def run(self, stream=None):
        """Enqueue the whole batch (one persistent launch per body present)
        on `stream` (default: the current stream)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.device(self.device):
            _lib.check(_lib.LIB.vp_batch_run(self._plan, s.cuda_stream), "batch_run")

    def graph(self) -> torch.cuda.CUDAGraph:
        """Capture one run in a CUDA graph; replay() re-executes the batch."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run(s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        return g

    def error(self) -> bool:
        """Synchronises; True if a run hit the bounded wait between stages
        (a dependency did not complete in time; results may be wrong)."""
        flag = ctypes.c_int(0)
        with torch.cuda.device(self.device):
            _lib.check(_lib.LIB.vp_batch_error(self._plan, ctypes.byref(flag)), "batch_error")
        return bool(flag.value)

    def close(self):
        if self._plan:
            _lib.LIB.vp_batch_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uneven_cubes(count=64, seed=2026, sides=tuple(range(64, 385, 32)), nmin=90, nmax=720):
    """(side, n_ang) of the uneven-batch workload, seeded."""
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(sides)), int(rng.integers(nmin, nmax + 1))) for _ in range(count)]


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--cubes", default=None,
                    help="explicit cubes as side:angles,... instead of the seeded workload")
    ap.add_argument("--only", choices=("both", "forward", "backward"), default="both",
                    help="batch A of every cube, A^T of every sinogram, or both")
    ap.add_argument("--forward-variant", type=int, default=None,
                    help="forward kernel variant of every problem, batched and sequential "
                         "(default: the autotuner's, or the library default with --no-tune)")
    args = ap.parse_args()
    from . import _CU, tune

    dev = torch.device("cuda")
    if args.cubes:
        shapes = [tuple(int(v) for v in c.split(":")) for c in args.cubes.split(",")]
    else:
        shapes = uneven_cubes(args.count)
    fwd, bwd = args.only in ("both", "forward"), args.only in ("both", "backward")
    g = torch.Generator(device=dev).manual_seed(7)
    problems, plain = [], []
    vu = 0
    for side, n in shapes:
        ang = torch.linspace(0, np.pi, n + 1, device=dev)[:-1].contiguous()
        x = torch.randn(side, side, side, device=dev, generator=g)
        y = torch.randn(n, side, side, device=dev, generator=g)
        y_out = torch.zeros(n, side, side, device=dev)
        x_out = torch.zeros(side, side, side, device=dev)
        vf = (args.forward_variant if args.forward_variant is not None
              else None if args.no_tune else tune.batch_variant("forward", side, n))
        vb = None if args.no_tune else tune.batch_variant("backward", side, n)
        if fwd:
            problems.append(("forward", x, y_out, ang, vf))
        if bwd:
            problems.append(("backward", y, x_out, ang, vb))
        plain.append((x, y_out, y, x_out, ang))
        vu += (int(fwd) + int(bwd)) * side**3 * n
    batch = Batch(problems)
    before = _lib.LIB.vp_launch_count()
    graph = batch.graph()
    launches = _lib.LIB.vp_launch_count() - before

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / args.reps

    t_graph = timed(graph.replay)

    def sequential():
        for x, y_out, y, x_out, ang in plain:
            if fwd:
                _CU.forward_z0(x, y_out, ang)
            if bwd:
                _CU.backward_z0(y, x_out, ang)

    if args.forward_variant is not None:  # the sequential calls run it too
        _lib.LIB.vp_set_kernel_variant(0, args.forward_variant)  # op 0: forward z0
    try:
        t_seq = timed(sequential)
        before = _lib.LIB.vp_launch_count()
        sequential()
        seq_launches = _lib.LIB.vp_launch_count() - before
    finally:
        if args.forward_variant is not None:
            _lib.LIB.vp_set_kernel_variant(0, 0)
    print(json.dumps({
        "workload": (f"cubes {args.cubes}" if args.cubes else
                     f"{args.count} cubes, sides {{64..384 step 32}}, U{{90..720}} angles each")
                    + {"both": "; A of every cube and A^T of every sinogram",
                       "forward": "; A of every cube", "backward": "; A^T of every sinogram"}[
                           args.only],
        "voxel_angle_updates": vu, "work_items": batch.work_items,
        "graph_ms": round(t_graph, 3), "graph_gvu_s": round(vu / t_graph / 1e6, 1),
        "sequential_ms": round(t_seq, 3), "sequential_gvu_s": round(vu / t_seq / 1e6, 1),
        "speedup_vs_sequential": round(t_seq / t_graph, 3),
        "launches_per_batch": int(launches), "sequential_launches": int(seq_launches),
    }))
    batch.close()


if __name__ == "__main__":
    main()
