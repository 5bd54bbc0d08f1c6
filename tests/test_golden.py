"""Golden fixtures: outputs of the reference's own CUDA kernels.

``tests/golden/reference_outputs.npz`` holds the reference's outputs on
seeded inputs; ``tests/golden/make_golden.py`` regenerates them.
  * CPU: the FP64 oracle agrees with the reference (this pins the oracle);
  * GPU: the GB300 kernels agree with the reference.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle
from tests import tolerances as tol
from tests.common import rel_err

FIXTURES = Path(__file__).resolve().parent / "golden" / "reference_outputs.npz"


def load_cases():
    if not FIXTURES.exists():
        return {}
    data = np.load(FIXTURES)
    cases = {}
    for key in data.files:
        name, field = key.split("/")
        cases.setdefault(name, {})[field] = data[key]
    return cases


CASES = load_cases()
NAMES = sorted(CASES)


def test_fixtures_present():
    assert FIXTURES.exists(), "run tests/golden/make_golden.py on a GPU machine"
    assert len(NAMES) >= 20


def oracle_outputs(c):
    z, SY, SX, Hx, n, PX, Hy = (int(v) for v in c["meta"])
    H = min(Hx, Hy)
    x, y, ang = c["x"], c["y"], c["angles"]
    xh = x[:, :, :H] if z == 0 else x[:H]
    yh = y[:, :, :H] if z == 0 else y[:H]
    fwd = c["y0"].astype(np.float64).copy()
    bwd = c["x0"].astype(np.float64).copy()
    A = oracle.forward(np.ascontiguousarray(xh), ang, PX, z)
    B = oracle.backward(np.ascontiguousarray(yh), ang, SY, SX, z)
    if z == 0:
        fwd[:, :, :H] += A
        bwd[:, :, :H] += B
    else:
        fwd[:H] += A
        bwd[:H] += B
    return fwd, bwd


# How far the reference itself is from the exact operator at these sizes
# (fixtures up to 68 voxels wide; angles up to 4*pi in rand_angles):
#   A^T: closed-form 3-bin weights, but hardware sin/cos  -> ~1e-5
#   A:   rays marched with an accumulated float position
#        (sp_forward_z0.cuh:33,53) and clipped in float   -> ~1e-4
#        (it reaches 5.9e-3 at 512^3, measured on a GB300)
ORACLE_VS_REFERENCE = {"A": 1.5e-4, "AT": 2e-5}


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name):
    c = CASES[name]
    fwd, bwd = oracle_outputs(c)
    ef = rel_err(c["fwd"] - c["y0"], fwd - c["y0"])
    eb = rel_err(c["bwd"] - c["x0"], bwd - c["x0"])
    print(f"\n[oracle vs reference] {name}: A {ef:.3e}  A^T {eb:.3e}")
    assert ef <= ORACLE_VS_REFERENCE["A"] and eb <= ORACLE_VS_REFERENCE["AT"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_kernels_match_reference(name):
    """A^T: within the parity target (1e-5) of the reference's kernels.
    A: the reference's forward carries its own ray-march error, so the bound
    is: our distance to the reference is no more than the reference's
    distance to the FP64 operator plus our own (REF_VS_FP64)."""
    import voxelproj_gb300 as vp

    c = CASES[name]
    z = int(c["meta"][0])
    dev = "cuda"
    a = torch.tensor(c["angles"], device=dev)
    yo = torch.tensor(c["y0"], device=dev)
    (vp._CU.forward_z0 if z == 0 else vp._CU.forward_z2)(torch.tensor(c["x"], device=dev), yo, a)
    xo = torch.tensor(c["x0"], device=dev)
    (vp._CU.backward_z0 if z == 0 else vp._CU.backward_z2)(torch.tensor(c["y"], device=dev), xo, a)
    torch.cuda.synchronize()
    fwd64, _ = oracle_outputs(c)
    got_a = yo.cpu().numpy() - c["y0"]
    ref_a = c["fwd"] - c["y0"]
    exact_a = fwd64 - c["y0"]
    e_ref = rel_err(got_a, ref_a)
    e_ours64 = rel_err(got_a, exact_a)
    e_ref64 = rel_err(ref_a, exact_a)
    eb = rel_err(xo.cpu().numpy() - c["x0"], c["bwd"] - c["x0"])
    print(f"\n[kernels vs reference] {name}: A {e_ref:.3e} (ours vs FP64 {e_ours64:.3e}, "
          f"reference vs FP64 {e_ref64:.3e})  A^T {eb:.3e}")
    assert eb <= tol.REF_VS_REFERENCE
    assert e_ours64 <= tol.REF_VS_FP64
    assert e_ref <= e_ref64 + tol.REF_VS_FP64


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if not n.startswith("many_angles")])
def test_adjoint_bit_exact_variant(name):
    """With the variant that accumulates in the reference's order (z_order 0
    variant 4; the z_order 2 kernel for H < 32), A^T reproduces the
    reference's kernels bit for bit: same weights, same rounding order.  (The
    600-angle fixtures were recorded in two <= 512-angle chunks, which sums in
    another order, so they are left out.)"""
    import voxelproj_gb300 as vp
    from voxelproj_gb300 import _lib

    c = CASES[name]
    z = int(c["meta"][0])
    a = torch.tensor(c["angles"], device="cuda")
    xo = torch.tensor(c["x0"], device="cuda")
    _lib.LIB.vp_set_kernel_variant(1, 4)
    try:
        (vp._CU.backward_z0 if z == 0 else vp._CU.backward_z2)(
            torch.tensor(c["y"], device="cuda"), xo, a)
        torch.cuda.synchronize()
    finally:
        _lib.LIB.vp_set_kernel_variant(1, 0)
    np.testing.assert_array_equal(xo.cpu().numpy(), c["bwd"])
