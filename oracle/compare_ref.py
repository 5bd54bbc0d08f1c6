"""TEST INFRASTRUCTURE ONLY — times the reference's CUDA kernels beside this
library's on the same GPU.

The reference extension (``voxelproj._CU``) is built from the reference's
sources by ``oracle/build_ref.py``.  Both sides run A and A^T on the same
N(0, 1) float32 volume / sinogram on the device, with angles linspace(0, pi,
n), and are timed with CUDA events around each call (median of --reps after
one warm-up call).  The reference's calls include its per-call texture
staging (cudaMalloc3DArray, a device copy of the input into it,
cudaFreeArray; voxelproj/csrc/projectors.cu:57-103); its kernel-only time
comes from running this script under ncu (gpu__time_duration.sum of
sp_forward_z* / sp_backward_z*).  Its adjoint holds at most 512 angles
(sp_backward_z0.cuh:6), so larger angle counts run it in chunks of 512.

    python oracle/compare_ref.py --src DIR [--size 512] [--angles 192] [--z-order 0 2]

Prints one JSON line per (implementation, z_order, direction).
"""

from __future__ import annotations

import argparse
import json
import statistics
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--src", type=Path, default=None)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--angles", type=int, default=192)
    ap.add_argument("--z-order", type=int, nargs="+", default=[0, 2])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--impl", nargs="+", default=["reference", "ours"])
    args = ap.parse_args()
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import torch

    from oracle import build_ref

    ref = build_ref.build(args.src) if "reference" in args.impl else None
    import voxelproj_gb300 as vp

    N, n = args.size, args.angles
    dev = "cuda"
    g = torch.Generator(device=dev).manual_seed(0)
    ang = torch.tensor(np.linspace(0, np.pi, n).astype(np.float32), device=dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    for z in args.z_order:
        xs = (N, N, N)
        ys = (n, N, N) if z == 0 else (N, n, N)
        x = torch.randn(xs, generator=g, device=dev)
        y = torch.randn(ys, generator=g, device=dev)
        yo = torch.zeros(ys, device=dev)
        xo = torch.zeros(xs, device=dev)
        for impl in args.impl:
            mod = ref if impl == "reference" else vp._CU
            fwd = mod.forward_z0 if z == 0 else mod.forward_z2
            bwd = mod.backward_z0 if z == 0 else mod.backward_z2

            def run_bwd():
                if impl == "reference" and n > 512:
                    for a0 in range(0, n, 512):
                        a1 = min(n, a0 + 512)
                        yc = (y[a0:a1] if z == 0 else y[:, a0:a1]).contiguous()
                        bwd(yc, xo, ang[a0:a1].contiguous())
                else:
                    bwd(y, xo, ang)

            tf = timed(lambda: fwd(x, yo, ang))
            tb = timed(run_bwd)
            vu = float(N) ** 3 * n
            for d, t in (("A", tf), ("AT", tb)):
                print(json.dumps({"impl": impl, "z_order": z, "op": d, "size": N, "angles": n,
                                  "ms": round(t, 4), "gvu_s": round(vu / t / 1e6, 1)}),
                      flush=True)
        del x, y, yo, xo
        torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
