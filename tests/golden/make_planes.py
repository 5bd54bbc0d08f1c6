"""Records the reference's own outputs on height planes of the benchmark
configurations (needs a CUDA GPU and the reference's sources).

The projector's weights do not depend on the height index, and the
reference's kernels compute every height on its own (one thread per output
element, texture fetches at that height), so its result on a few height
planes of a volume equals those planes of its result on the whole volume.
This script runs the reference's kernels (``voxelproj._CU``, built from its
sources by ``oracle/build_ref.py``) on the planes only and stores the outputs;
the inputs are the hashed synthetic arrays of ``tests/golden/hashed.py``, which
the GPU tests regenerate whole, bit for bit, to run this library on the full
problem and compare the same planes.

Configurations (angles linspace(0, pi, n) in float32, detector width the
reference wrapper's default max(SY, SX)):
  c1_z{0,2}        128^3 volume, 192 angles, 128 bins
  c2_n192_z{0,2}   512^3 volume, 192 angles, 512 bins
  c2_n1024_z{0,2}  512^3 volume, 1024 angles, 512 bins
The reference's adjoint holds per-angle tables for at most 512 angles in
shared memory (sp_backward_z0.cuh:6,29-45), so 1024 angles are backprojected
in two chunks of 512 into the same output, which its accumulate semantics
(sp_backward_z0.cuh:98) make exact up to float summation order.

    python oracle/build_ref.py --src <dir holding voxelproj.cpp, projectors.cu>
    python tests/golden/make_planes.py --src <same dir>

Each case ``<name>`` stores:
  <name>/meta     int64 [z_order, SY, SX, H, n_ang, PX, seed_x, seed_y]
  <name>/heights  int64 height indices of the stored planes
  <name>/angles   float32 (n_ang,)
  <name>/fwd      A x on those planes, z_order layout with the planes as heights
  <name>/bwd      A^T y likewise
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "reference_planes.npz"
MAX_REF_BACKWARD_ANGLES = 512


def cases():
    out = []
    for z in (0, 2):
        hz = [3, 300] if z == 0 else [300]
        out.append(dict(name=f"c1_z{z}", z=z, N=128, n=192, PX=128,
                        heights=[3, 100] if z == 0 else [100], seed_x=101, seed_y=102))
        out.append(dict(name=f"c2_n192_z{z}", z=z, N=512, n=192, PX=512, heights=hz,
                        seed_x=201, seed_y=202))
        out.append(dict(name=f"c2_n1024_z{z}", z=z, N=512, n=1024, PX=512, heights=hz,
                        seed_x=301, seed_y=302))
    return out


def angles(n: int) -> np.ndarray:
    return np.linspace(0.0, np.pi, n).astype(np.float32)


def plane_inputs(c):
    """x and y on the case's height planes, in its z_order layout."""
    from tests.golden import hashed

    N, n, PX, z = c["N"], c["n"], c["PX"], c["z"]
    xc = hashed.canonical_numpy(c["seed_x"], (N, N, N), c["heights"])
    yc = hashed.canonical_numpy(c["seed_y"], (N, n, PX), c["heights"])
    return hashed.layout_numpy(xc, z), hashed.layout_numpy(yc, z)


def run_reference(_CU, c, x, y):
    import torch

    z = c["z"]
    fwd_fn = _CU.forward_z0 if z == 0 else _CU.forward_z2
    bwd_fn = _CU.backward_z0 if z == 0 else _CU.backward_z2
    ang = torch.tensor(angles(c["n"]), device="cuda")
    xg = torch.tensor(x, device="cuda")
    yg = torch.tensor(y, device="cuda")
    yout = torch.zeros_like(yg)
    fwd_fn(xg, yout, ang)
    xout = torch.zeros_like(xg)
    n = c["n"]
    for a0 in range(0, n, MAX_REF_BACKWARD_ANGLES):
        a1 = min(n, a0 + MAX_REF_BACKWARD_ANGLES)
        ychunk = (yg[a0:a1] if z == 0 else yg[:, a0:a1, :]).contiguous()
        bwd_fn(ychunk, xout, ang[a0:a1].contiguous())
    torch.cuda.synchronize()
    return yout.cpu().numpy(), xout.cpu().numpy()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--src", type=Path, default=None,
                    help="directory with the reference's voxelproj.cpp and projectors.cu")
    ap.add_argument("--out", type=Path, default=OUT)
    args = ap.parse_args()
    sys.path.insert(0, str(ROOT))
    from oracle import build_ref

    _CU = build_ref.build(args.src)
    store = {}
    for c in cases():
        x, y = plane_inputs(c)
        fwd, bwd = run_reference(_CU, c, x, y)
        k = c["name"]
        store[f"{k}/meta"] = np.array([c["z"], c["N"], c["N"], c["N"], c["n"], c["PX"],
                                       c["seed_x"], c["seed_y"]], np.int64)
        store[f"{k}/heights"] = np.array(c["heights"], np.int64)
        store[f"{k}/angles"] = angles(c["n"])
        store[f"{k}/fwd"] = fwd
        store[f"{k}/bwd"] = bwd
        print(f"{k}: fwd {fwd.shape} |max| {np.abs(fwd).max():.4g}  "
              f"bwd {bwd.shape} |max| {np.abs(bwd).max():.4g}", flush=True)
    args.out.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(args.out, **store)
    print(f"wrote {args.out} ({args.out.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
