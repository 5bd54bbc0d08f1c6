"""Parity at the benchmark configurations.

  C1: 128^3 volume, 192 angles, 128 bins
  C2: 512^3 volume, 192 and 1024 angles, 512 bins, output written in place
both z_orders, angles linspace(0, pi, n) in float32.

The inputs are the hashed synthetic arrays of ``tests/golden/hashed.py``
(N(0, 1)-like, bounded), which any machine regenerates bit for bit.  The
GPU tests run the whole problem through the public API
(``voxelproj_gb300.forward`` / ``backward`` into preallocated zero outputs)
with the default kernels, and compare a few height planes of the results:

  * against the reference's own CUDA kernels, recorded on those planes by
    ``tests/golden/make_planes.py`` (``tests/golden/reference_planes.npz``);
  * against the FP64 oracle on the same planes.

Size-independent properties are checked on the whole result: the adjoint
identity with FP64 inner products, and z_order 2 equal to z_order 0 bit for
bit (z_order 2 runs the z_order 0 kernels between transposes).

The CPU test pins how far the reference itself is from the exact operator at
these sizes, which sets the bound for A (its rays are marched with an
accumulated float position, sp_forward_z0.cuh:33,53).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle
from tests import tolerances as tol
from tests.common import rel_err
from tests.golden import hashed

PLANES = Path(__file__).resolve().parent / "golden" / "reference_planes.npz"


def load_cases():
    if not PLANES.exists():
        return {}
    data = np.load(PLANES)
    cases = {}
    for key in data.files:
        name, field = key.split("/")
        cases.setdefault(name, {})[field] = data[key]
    return cases


CASES = load_cases()
NAMES = sorted(CASES)


def meta(c):
    z, SY, SX, H, n, PX, sx, sy = (int(v) for v in c["meta"])
    return z, SY, SX, H, n, PX, sx, sy


def compact_y(yp, z):
    """Planes of y in the z_order layout -> (n_h, n_ang, PX)."""
    return np.ascontiguousarray(yp.transpose(2, 0, 1)) if z == 0 else yp


def compact_x(xp, z):
    """Planes of x in the z_order layout -> (n_h, SY, SX)."""
    return np.ascontiguousarray(xp.transpose(2, 0, 1)) if z == 0 else xp


def plane_inputs(c):
    z, SY, SX, H, n, PX, sx, sy = meta(c)
    hs = c["heights"]
    xc = hashed.canonical_numpy(sx, (H, SY, SX), hs)
    yc = hashed.canonical_numpy(sy, (H, n, PX), hs)
    return hashed.layout_numpy(xc, z), hashed.layout_numpy(yc, z)


_ORACLE_CACHE: dict = {}


def oracle_planes(name):
    """FP64 A x and A^T y on the case's planes, compact."""
    if name not in _ORACLE_CACHE:
        c = CASES[name]
        z, SY, SX, H, n, PX, _, _ = meta(c)
        xp, yp = plane_inputs(c)
        _ORACLE_CACHE[name] = (oracle.forward_f64(xp, c["angles"], PX, z),
                               oracle.backward_f64(yp, c["angles"], SY, SX, z))
    return _ORACLE_CACHE[name]


def test_plane_fixtures_present():
    assert PLANES.exists(), "run tests/golden/make_planes.py on a GPU machine"
    assert {"c1_z0", "c1_z2", "c2_n192_z0", "c2_n192_z2", "c2_n1024_z0",
            "c2_n1024_z2"} <= set(NAMES)


def test_hashed_inputs_match_fixture_shapes():
    for name in NAMES:
        c = CASES[name]
        z, SY, SX, H, n, PX, _, _ = meta(c)
        xp, yp = plane_inputs(c)
        assert c["fwd"].shape == yp.shape and c["bwd"].shape == xp.shape
        assert c["angles"].shape == (n,)
        np.testing.assert_array_equal(c["angles"], np.linspace(0, np.pi, n).astype(np.float32))


@pytest.mark.parametrize("name", NAMES)
def test_reference_vs_fp64_on_planes(name):
    """How far the reference's kernels are from the exact (FP64) operator on
    the benchmark planes.  A^T (closed-form weights, hardware sin/cos) stays
    near the trig floor.  A's rays are marched with an accumulated float
    position and clipped in float (sp_forward_z0.cuh:33,53;
    projection_common.cuh:194-272), and at 512 voxels it is several 1e-3
    away: the 1e-5 target cannot hold for A against the reference, which is
    why A is bounded by the reference's own distance to FP64."""
    c = CASES[name]
    z, SY, SX, H, n, PX, _, _ = meta(c)
    A64, B64 = oracle_planes(name)
    ea = rel_err(compact_y(c["fwd"], z), A64)
    eb = rel_err(compact_x(c["bwd"], z), B64)
    print(f"\n[reference vs FP64] {name}: A {ea:.3e}  A^T {eb:.3e}")
    assert eb <= tol.ref_vs_fp64(max(SY, SX, PX))
    if SY >= 512:
        assert 1e-4 < ea < 3e-2  # the reference's forward misses 1e-5 by far
    else:
        assert ea < 3e-3


# ------------------------------------------------------------------ GPU ---

def run_full(c, trig="reference", z_order=None):
    """The whole problem through the public API, into zero outputs; returns
    (y, x) as device tensors in the z_order layout."""
    import voxelproj_gb300 as vp

    z, SY, SX, H, n, PX, sx, sy = meta(c)
    z = z if z_order is None else z_order
    dev = "cuda"
    x = hashed.layout_torch(hashed.canonical_torch(sx, (H, SY, SX), dev), z)
    ys = (n, PX, H) if z == 0 else (H, n, PX)
    y_in = hashed.layout_torch(hashed.canonical_torch(sy, (H, n, PX), dev), z)
    ang = torch.tensor(c["angles"], device=dev)
    yo = torch.zeros(ys, device=dev)
    xo = torch.zeros_like(x)
    vp.set_trig_mode(trig)
    try:
        r1 = vp.forward(x, ang, yo, z_order=z)
        r2 = vp.backward(y_in, ang, xo, z_order=z)
        torch.cuda.synchronize()
    finally:
        vp.set_trig_mode("reference")
    assert r1 is yo and r2 is xo  # written in place, same objects returned
    return x, y_in, yo, xo


def planes_of(t, heights, z):
    idx = torch.as_tensor(heights, device=t.device)
    p = t.index_select(2, idx) if z == 0 else t.index_select(0, idx)
    return p.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_config_matches_reference_and_fp64(name):
    """Default kernels on the full configuration, compared on the recorded
    planes.  A^T: within 1e-5 of the reference's kernels.  A: no further from
    the reference than the reference is from FP64, plus our own FP64 error.
    Both: within the TRIG_REF bound of the FP64 operator.  Whole result: the
    adjoint identity with FP64 inner products."""
    c = CASES[name]
    z, SY, SX, H, n, PX, _, _ = meta(c)
    hs = c["heights"]
    x, y_in, yo, xo = run_full(c)
    got_a = compact_y(planes_of(yo, hs, z), z)
    got_b = compact_x(planes_of(xo, hs, z), z)
    ref_a = compact_y(c["fwd"], z)
    ref_b = compact_x(c["bwd"], z)
    A64, B64 = oracle_planes(name)
    e_ref_a = rel_err(got_a, ref_a)
    e_ref_b = rel_err(got_b, ref_b)
    e64_a = rel_err(got_a, A64)
    e64_b = rel_err(got_b, B64)
    e_refref_a = rel_err(ref_a, A64)
    lhs = torch.dot(yo.double().flatten(), y_in.double().flatten()).item()
    rhs = torch.dot(x.double().flatten(), xo.double().flatten()).item()
    den = yo.double().norm().item() * y_in.double().norm().item()
    adj = abs(lhs - rhs) / den
    print(f"\n[config] {name}: A^T vs reference {e_ref_b:.3e}, vs FP64 {e64_b:.3e} | "
          f"A vs reference {e_ref_a:.3e} (reference vs FP64 {e_refref_a:.3e}), vs FP64 "
          f"{e64_a:.3e} | adjoint identity {adj:.3e}")
    bound64 = tol.ref_vs_fp64(max(SY, SX, PX))
    assert e_ref_b <= tol.REF_VS_REFERENCE
    assert e64_b <= bound64 and e64_a <= bound64
    assert e_ref_a <= e_refref_a + tol.REF_VS_FP64
    assert adj <= tol.ADJOINT


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if n.endswith("_z0") and n.startswith("c2_")])
def test_config_precise_trig_vs_fp64(name):
    """With accurate trig and a compensated detector coordinate, both
    operators are within the TRIG_PRECISE bound of FP64 at 512 voxels."""
    c = CASES[name]
    z, SY, SX, H, n, PX, _, _ = meta(c)
    hs = c["heights"]
    _, _, yo, xo = run_full(c, trig="precise")
    A64, B64 = oracle_planes(name)
    ea = rel_err(compact_y(planes_of(yo, hs, z), z), A64)
    eb = rel_err(compact_x(planes_of(xo, hs, z), z), B64)
    print(f"\n[config precise] {name}: A vs FP64 {ea:.3e}  A^T vs FP64 {eb:.3e}")
    bound = tol.precise_vs_fp64(max(SY, SX, PX))
    assert ea <= bound and eb <= bound


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", ["c1", "c2_n192", "c2_n1024"])
def test_config_z2_equals_z0(cfg):
    """The z_order 2 result is the z_order 0 result transposed, bit for bit,
    on the whole benchmark problem (same hashed data in both layouts)."""
    c = CASES[f"{cfg}_z0"]
    _, _, y0, x0 = run_full(c, z_order=0)
    y0 = y0.permute(2, 0, 1).contiguous()
    x0 = x0.permute(2, 0, 1).contiguous()
    _, _, y2, x2 = run_full(c, z_order=2)
    assert torch.equal(y0, y2)
    assert torch.equal(x0, x2)
