"""Autotuner: picks kernel variants by timing them on the problem's shape.

Results are cached in a JSON file (``$VOXELPROJ_GB300_TUNE_CACHE``, default
``~/.cache/voxelproj_gb300/tune.json``) keyed by operation, layout and shape,
so a shape is timed once per machine.  The time of every kernel is linear in
the angle count, so shapes are tuned with at most 90 angles.

Two consumers:
* ``batch_variant(op, side, n_ang)`` chooses the work-item body and slab
  plan of a batched problem (forward: 8 heights per lane with class slabs or
  4 with row slabs; adjoint: runs with 8 or 4 heights per lane, or 2x2 voxel
  blocks), timed as a one-problem batch;
* ``tune_single(op, x_shape, y_shape)`` chooses the single-problem kernel
  variant and applies it with ``vp_set_kernel_variant``.

No counterpart in the reference, whose only knob is the fixed ``block_size``.
"""

from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import torch

from . import _lib

BATCH_CANDIDATES = {"forward": [16, 21, 10, 1], "backward": [7, 6, 4]}
SINGLE_CANDIDATES = {"forward": [16, 21, 10, 11, 13, 7, 1], "backward": [7, 6, 4, 1]}
TUNE_ANGLES = 90


def cache_path() -> Path:
    p = os.environ.get("VOXELPROJ_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "voxelproj_gb300" / "tune.json"


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except Exception:
        return {}


def _store(cache: dict) -> None:
    path = cache_path()
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only loses the cache


def _time(fn, reps: int = 3) -> float:
    fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(reps)]
    for a, b in ev:
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return float(np.median([a.elapsed_time(b) for a, b in ev]))


def batch_variant(op: str, side: int, n_ang: int, device="cuda") -> int:
    """Variant for a batched cube problem of this side (cached)."""
    key = f"batch/{op}/z0/{side}x{side}x{side}/px{side}"
    cache = _load()
    if key in cache:
        return int(cache[key]["variant"])
    if len(BATCH_CANDIDATES[op]) == 1:
        return BATCH_CANDIDATES[op][0]
    from .batch import Batch

    n = min(n_ang, TUNE_ANGLES)
    ang = torch.linspace(0, np.pi, n + 1, device=device)[:-1].contiguous()
    x = torch.randn(side, side, side, device=device)
    y = torch.randn(n, side, side, device=device)
    times = {}
    for v in BATCH_CANDIDATES[op]:
        out = torch.zeros_like(y if op == "forward" else x)
        b = Batch([(op, x if op == "forward" else y, out, ang, v)])
        times[v] = _time(b.run)
        b.close()
    best = min(times, key=times.get)
    cache[key] = {"variant": best, "ms": times}
    _store(cache)
    return best


def tune_single(op: str, x_shape, y_shape, device="cuda", apply: bool = True) -> int:
    """Times the single-problem z_order 0 variants for these shapes, caches the
    fastest and (by default) selects it for the process."""
    key = f"single/{op}/z0/{'x'.join(map(str, x_shape))}/{'x'.join(map(str, y_shape))}"
    op_id = 0 if op == "forward" else 1
    cache = _load()
    if key not in cache:
        from . import _CU

        n = min(y_shape[0], TUNE_ANGLES)
        ys = (n, y_shape[1], y_shape[2])
        ang = torch.linspace(0, np.pi, n + 1, device=device)[:-1].contiguous()
        x = torch.randn(tuple(x_shape), device=device)
        y = torch.randn(ys, device=device)
        times = {}
        prev = _lib.LIB.vp_get_kernel_variant(op_id)
        for v in SINGLE_CANDIDATES[op]:
            _lib.LIB.vp_set_kernel_variant(op_id, v)
            if op == "forward":
                out = torch.zeros(ys, device=device)
                times[v] = _time(lambda: _CU.forward_z0(x, out, ang))
            else:
                out = torch.zeros(tuple(x_shape), device=device)
                times[v] = _time(lambda: _CU.backward_z0(y, out, ang))
        _lib.LIB.vp_set_kernel_variant(op_id, prev)
        cache[key] = {"variant": min(times, key=times.get), "ms": times}
        _store(cache)
    best = int(cache[key]["variant"])
    if apply:
        _lib.LIB.vp_set_kernel_variant(op_id, best)
    return best
