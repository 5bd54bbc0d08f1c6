"""Records the reference's own outputs as golden fixtures (needs a CUDA GPU).

Runs the reference voxelproj CUDA kernels (``voxelproj._CU``, built from the
reference's sources by ``oracle/build_ref.py``) on small seeded inputs and
writes ``tests/golden/reference_outputs.npz``.  The fixtures pin the oracle
and the GB300 kernels to the reference (``tests/test_golden.py``: the oracle
on CPU, the kernels under the ``gpu`` mark).

    python oracle/build_ref.py --src <dir holding voxelproj.cpp, projectors.cu>
    python tests/golden/make_golden.py --src <same dir>

Inputs stay inside what the reference handles: its adjoint keeps per-angle
tables for at most 512 angles in shared memory (sp_backward_z0.cuh:6,29-45),
so larger angle sets are backprojected in chunks of <= 512 into the same
output, which its accumulate semantics make exact; the output's angle extent
always equals the number of angles passed (the reference reads angles[0..n)
with n taken from the output, sp_forward_z0.cuh:113-136).

Each case ``<name>`` stores:
  <name>/meta   int64 [z_order, SY, SX, Hx, n_ang, PX, Hy]
  <name>/angles float32 (n_ang,)
  <name>/x, <name>/y        inputs of A and A^T (layout of z_order)
  <name>/y0, <name>/x0      initial outputs (zeros unless the case accumulates)
  <name>/fwd = y0 + A x,  <name>/bwd = x0 + A^T y      (reference results)
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "reference_outputs.npz"
MAX_REF_BACKWARD_ANGLES = 512


def lin(n, lo=0.0, hi=np.pi):
    return np.linspace(lo, hi, n).astype(np.float32)


def cases():
    rng = np.random.default_rng(20261203)
    out = []
    for z in (0, 2):
        out += [
            dict(name=f"adj_full_z{z}", z=z, SY=6, SX=5, H=3, ang=lin(31), PX=11),
            dict(name=f"adj_interior_z{z}", z=z, SY=6, SX=5, H=3, ang=lin(31), PX=4),
            dict(name=f"identity_z{z}", z=z, SY=6, SX=5, H=3, ang=lin(7), PX=11),
            dict(name=f"rect_full_z{z}", z=z, SY=24, SX=32, H=5,
                 ang=lin(45, -np.pi / 2, 3 * np.pi / 2), PX=40),
            dict(name=f"rect_cut_z{z}", z=z, SY=24, SX=32, H=8,
                 ang=lin(45, -np.pi / 2, 3 * np.pi / 2), PX=20),
            dict(name=f"rand_angles_z{z}", z=z, SY=48, SX=48, H=2,
                 ang=rng.uniform(-2 * np.pi, 4 * np.pi, 64).astype(np.float32), PX=68),
            dict(name=f"accumulate_z{z}", z=z, SY=16, SX=20, H=4, ang=lin(24), PX=26,
                 accumulate=True),
            dict(name=f"odd_h_z{z}", z=z, SY=9, SX=11, H=7, ang=lin(33), PX=15),
            dict(name=f"c1lite_z{z}", z=z, SY=64, SX=64, H=4, ang=lin(192), PX=64),
            dict(name=f"many_angles_z{z}", z=z, SY=12, SX=10, H=2, ang=lin(600), PX=16),
            dict(name=f"hmismatch_z{z}", z=z, SY=10, SX=12, H=6, Hy=4, ang=lin(20), PX=14,
                 accumulate=True),
        ]
    for c in out:
        c.setdefault("Hy", c["H"])
        c.setdefault("accumulate", False)
    return out, rng


def shapes(c):
    z, SY, SX, Hx, n, PX, Hy = c["z"], c["SY"], c["SX"], c["H"], len(c["ang"]), c["PX"], c["Hy"]
    xs = (SY, SX, Hx) if z == 0 else (Hx, SY, SX)
    ys = (n, PX, Hy) if z == 0 else (Hy, n, PX)
    return xs, ys


def run_reference(_CU, c, x, y, y0, x0):
    import torch

    z = c["z"]
    dev = "cuda"
    fwd_fn = _CU.forward_z0 if z == 0 else _CU.forward_z2
    bwd_fn = _CU.backward_z0 if z == 0 else _CU.backward_z2
    ang = torch.tensor(c["ang"], device=dev)
    xg = torch.tensor(x, device=dev)
    yg = torch.tensor(y, device=dev)
    yout = torch.tensor(y0, device=dev)
    fwd_fn(xg, yout, ang)
    xout = torch.tensor(x0, device=dev)
    n = len(c["ang"])
    for a0 in range(0, n, MAX_REF_BACKWARD_ANGLES):
        a1 = min(n, a0 + MAX_REF_BACKWARD_ANGLES)
        ychunk = (yg[a0:a1] if z == 0 else yg[:, a0:a1, :]).contiguous()
        assert ychunk.shape[0 if z == 0 else 1] <= MAX_REF_BACKWARD_ANGLES
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
    cs, rng = cases()
    store = {}
    for c in cs:
        xs, ys = shapes(c)
        x = rng.standard_normal(xs).astype(np.float32)
        y = rng.standard_normal(ys).astype(np.float32)
        y0 = rng.standard_normal(ys).astype(np.float32) if c["accumulate"] else np.zeros(ys, np.float32)
        x0 = rng.standard_normal(xs).astype(np.float32) if c["accumulate"] else np.zeros(xs, np.float32)
        fwd, bwd = run_reference(_CU, c, x, y, y0, x0)
        k = c["name"]
        store[f"{k}/meta"] = np.array([c["z"], c["SY"], c["SX"], c["H"], len(c["ang"]), c["PX"],
                                       c["Hy"]], np.int64)
        store[f"{k}/angles"] = c["ang"]
        store[f"{k}/x"] = x
        store[f"{k}/y"] = y
        store[f"{k}/y0"] = y0
        store[f"{k}/x0"] = x0
        store[f"{k}/fwd"] = fwd
        store[f"{k}/bwd"] = bwd
        print(f"{k}: x{xs} y{ys} |fwd|max={np.abs(fwd).max():.4g} |bwd|max={np.abs(bwd).max():.4g}")
    np.savez_compressed(args.out, **store)
    print(f"wrote {args.out} ({args.out.stat().st_size} bytes, {len(cs)} cases)")


if __name__ == "__main__":
    main()
