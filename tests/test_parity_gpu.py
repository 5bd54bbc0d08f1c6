"""GPU kernels vs the FP64 oracle on seeded inputs (the parity tests proper).

Every case accumulates into a random initial output, so the accumulate
semantics of the reference (out += result) are checked together with the
values.  Geometries cover square and rectangular volumes, detectors wider and
narrower than the volume, heights that are and are not multiples of 4 (the
float4 and scalar paths), several height chunks, one voxel, long thin
volumes, angles inside and outside [0, pi] including the degenerate k*pi/2,
and more than 512 angles (the reference adjoint's limit).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import voxelproj_gb300 as vp
from oracle import oracle
from tests import tolerances as tol
from tests.common import lin, rel_err, seeded, x_shape, y_shape

pytestmark = pytest.mark.gpu

# (SY, SX, H, n_ang, PX, angle set)
GEOMS = [
    (6, 5, 3, 31, 11, "pi"),
    (6, 5, 3, 31, 4, "pi"),
    (24, 32, 5, 45, 40, "wide"),
    (24, 32, 8, 45, 20, "wide"),
    (33, 17, 1, 13, 50, "rand"),
    (16, 16, 128, 64, 16, "pi"),
    (64, 64, 4, 192, 64, "pi"),
    (40, 40, 12, 700, 57, "pi"),
    (7, 300, 2, 9, 310, "rand"),
    (1, 1, 5, 4, 1, "pi"),
    (50, 50, 132, 16, 72, "rand"),
    (50, 50, 130, 16, 72, "rand"),
    (48, 40, 16, 37, 64, "axes"),
]


def angle_set(kind, n, seed):
    if kind == "pi":
        return lin(n)
    if kind == "wide":
        return lin(n, -np.pi / 2, 3 * np.pi / 2)
    if kind == "axes":
        base = np.array([0, np.pi / 2, np.pi, 3 * np.pi / 2, -np.pi / 2, np.pi / 4, 3 * np.pi / 4],
                        np.float32)
        return np.resize(base, n).astype(np.float32)
    rng = np.random.default_rng(seed)
    return rng.uniform(-2 * np.pi, 4 * np.pi, n).astype(np.float32)


def run_ours(z, x, y, ang, y0, x0, trig):
    fwd = vp._CU.forward_z0 if z == 0 else vp._CU.forward_z2
    bwd = vp._CU.backward_z0 if z == 0 else vp._CU.backward_z2
    vp.set_trig_mode(trig)
    try:
        a = torch.tensor(ang, device="cuda")
        yo = torch.tensor(y0, device="cuda")
        fwd(torch.tensor(x, device="cuda"), yo, a)
        xo = torch.tensor(x0, device="cuda")
        bwd(torch.tensor(y, device="cuda"), xo, a)
        torch.cuda.synchronize()
    finally:
        vp.set_trig_mode("reference")
    return yo.cpu().numpy(), xo.cpu().numpy()


@pytest.mark.parametrize("trig", ["reference", "precise"])
@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("geom", GEOMS, ids=lambda g: "x".join(map(str, g[:5])) + g[5])
def test_matches_fp64_oracle(geom, z, trig):
    SY, SX, H, n, PX, kind = geom
    seed = hash((SY, SX, H, n, PX)) % 2**31
    ang = angle_set(kind, n, seed)
    x = seeded(x_shape(z, SY, SX, H), seed + 1)
    y = seeded(y_shape(z, n, PX, H), seed + 2)
    y0 = seeded(y_shape(z, n, PX, H), seed + 3)
    x0 = seeded(x_shape(z, SY, SX, H), seed + 4)
    got_f, got_b = run_ours(z, x, y, ang, y0, x0, trig)
    Ax = oracle.forward(x, ang, PX, z)
    ATy = oracle.backward(y, ang, SY, SX, z)
    ef = rel_err(got_f - y0, Ax)
    eb = rel_err(got_b - x0, ATy)
    n_ext = max(SY, SX, PX)
    bound = tol.precise_vs_fp64(n_ext) if trig == "precise" else tol.ref_vs_fp64(n_ext)
    print(f"\n[parity] z={z} {trig:9s} {geom}: A {ef:.3e}  A^T {eb:.3e}")
    assert ef <= bound and eb <= bound, (ef, eb)
    # accumulate semantics: the initial content is kept, not overwritten
    assert rel_err(got_f, y0 + Ax) <= bound * max(1.0, np.abs(Ax).max() / np.abs(y0 + Ax).max())


@pytest.mark.parametrize("z", [0, 2])
def test_adjoint_identity_gpu(z):
    SY, SX, H, n, PX = 37, 41, 9, 90, 60
    ang = lin(n)
    x = seeded(x_shape(z, SY, SX, H), 11, "uniform")
    y = seeded(y_shape(z, n, PX, H), 12, "uniform")
    Ax, ATy = run_ours(z, x, y, ang, np.zeros_like(y), np.zeros_like(x), "reference")
    lhs = np.vdot(Ax.astype(np.float64), y.astype(np.float64))
    rhs = np.vdot(x.astype(np.float64), ATy.astype(np.float64))
    den = np.linalg.norm(Ax.astype(np.float64)) * np.linalg.norm(y.astype(np.float64))
    print(f"\n[adjoint] z={z}: {abs(lhs - rhs) / den:.3e}")
    assert abs(lhs - rhs) / den <= tol.ADJOINT


def test_z0_and_z2_agree():
    SY, SX, H, n, PX = 30, 26, 6, 50, 44
    ang = lin(n)
    x0 = seeded((SY, SX, H), 21)
    y0 = seeded((n, PX, H), 22)
    A0, B0 = run_ours(0, x0, y0, ang, np.zeros((n, PX, H), np.float32),
                      np.zeros((SY, SX, H), np.float32), "reference")
    x2 = np.ascontiguousarray(x0.transpose(2, 0, 1))
    y2 = np.ascontiguousarray(y0.transpose(2, 0, 1))
    A2, B2 = run_ours(2, x2, y2, ang, np.zeros_like(y2), np.zeros_like(x2), "reference")
    assert rel_err(A2.transpose(1, 2, 0), A0) < 1e-6
    assert rel_err(B2.transpose(1, 2, 0), B0) < 1e-6


def test_weight_sum_single_voxel():
    """A lit voxel's projection sums to H at every angle; the reference's
    weight-sum study reports 1e-7..1e-6 for its kernels."""
    SY, SX, H, n = 9, 10, 4, 181
    ang = lin(n, 0, 2 * np.pi)
    for yi, xi in [(4, 5), (0, 0), (8, 9), (3, 7)]:
        x = np.zeros((SY, SX, H), np.float32)
        x[yi, xi] = 1
        y = vp.forward(torch.tensor(x, device="cuda"), ang, (n, 16, H))
        sums = y.sum(dim=(1, 2)).cpu().numpy() / H
        assert np.abs(sums - 1).max() < 2e-6


# Every kernel variant of the z_order 0 adjoint against the oracle (the
# autotuner may pick any of them): sizes that are not multiples of the block
# or run shape, degenerate angles, both signs of each step, several height
# chunks.
@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7, 9])
@pytest.mark.parametrize("geom", [(23, 37, 132, 61, 50, "wide"), (9, 6, 8, 40, 11, "axes"),
                                  (64, 64, 256, 96, 64, "rand"), (30, 21, 260, 33, 40, "rand")],
                         ids=lambda g: "x".join(map(str, g[:5])) + g[5])
def test_backward_variants(variant, geom):
    from voxelproj_gb300 import _lib

    SY, SX, H, n, PX, kind = geom
    ang = angle_set(kind, n, 99)
    y = seeded((n, PX, H), 31)
    x0 = seeded((SY, SX, H), 32)
    _lib.LIB.vp_set_kernel_variant(1, variant)
    try:
        xo = torch.tensor(x0, device="cuda")
        vp._CU.backward_z0(torch.tensor(y, device="cuda"), xo, torch.tensor(ang, device="cuda"))
        torch.cuda.synchronize()
    finally:
        _lib.LIB.vp_set_kernel_variant(1, 0)
    err = rel_err(xo.cpu().numpy() - x0, oracle.backward(y, ang, SY, SX, 0))
    print(f"\n[variant {variant}] {geom}: A^T {err:.3e}")
    assert err <= tol.ref_vs_fp64(max(SY, SX, PX))


@pytest.mark.parametrize("variant", [1, 4, 6, 7, 9])
@pytest.mark.parametrize("H", [36, 260])
def test_backward_variants_store_mode_via_z2(variant, H):
    """z_order 2 with H >= 32 runs the z_order 0 kernel in store mode into
    scratch; the result must not depend on the scratch's prior content."""
    from voxelproj_gb300 import _lib

    SY, SX, n, PX = 20, 26, 30, 34
    ang = lin(n)
    y = seeded((H, n, PX), 41)
    x0 = seeded((H, SY, SX), 42)
    _lib.LIB.vp_set_kernel_variant(1, variant)
    try:
        outs = []
        for _ in range(2):
            xo = torch.tensor(x0, device="cuda")
            vp._CU.backward_z2(torch.tensor(y, device="cuda"), xo, torch.tensor(ang, device="cuda"))
            torch.cuda.synchronize()
            outs.append(xo.cpu().numpy())
    finally:
        _lib.LIB.vp_set_kernel_variant(1, 0)
    np.testing.assert_array_equal(outs[0], outs[1])
    assert rel_err(outs[0] - x0, oracle.backward(y, ang, SY, SX, 2)) <= tol.ref_vs_fp64(PX)


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17,
                                     19, 21, 22, 23])
@pytest.mark.parametrize("geom", [(23, 37, 132, 61, 50, "wide"), (9, 6, 8, 40, 11, "axes"),
                                  (70, 64, 256, 96, 90, "rand"), (30, 21, 260, 33, 40, "rand"),
                                  (26, 31, 1024, 23, 36, "wide")],
                         ids=lambda g: "x".join(map(str, g[:5])) + g[5])
def test_forward_variants(variant, geom):
    """Every kernel variant of the z_order 0 forward against the oracle:
    bins per warp 4 / 8, heights per lane 4 / 8 (with half-filled height
    chunks), warps of a block on neighbouring bins / angles, angle counts that
    are not multiples of the group, degenerate angles."""
    from voxelproj_gb300 import _lib

    SY, SX, H, n, PX, kind = geom
    ang = angle_set(kind, n, 98)
    x = seeded((SY, SX, H), 33)
    y0 = seeded((n, PX, H), 34)
    _lib.LIB.vp_set_kernel_variant(0, variant)
    try:
        yo = torch.tensor(y0, device="cuda")
        vp._CU.forward_z0(torch.tensor(x, device="cuda"), yo, torch.tensor(ang, device="cuda"))
        torch.cuda.synchronize()
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
    err = rel_err(yo.cpu().numpy() - y0, oracle.forward(x, ang, PX, 0))
    print(f"\n[fwd variant {variant}] {geom}: A {err:.3e}")
    assert err <= tol.ref_vs_fp64(max(SY, SX, PX))


@pytest.mark.parametrize("variant", [1, 5, 7, 8, 9, 12, 13, 14, 16, 17, 19])
@pytest.mark.parametrize("H", [36, 260, 512])
def test_forward_variants_store_mode_via_z2(variant, H):
    """The forward's first slab launch writes the z_order 2 scratch in store
    mode; repeated calls must not depend on the scratch's prior content."""
    from voxelproj_gb300 import _lib

    SY, SX, n, PX = 40, 26, 30, 34
    ang = lin(n)
    x = seeded((H, SY, SX), 43)
    y0 = seeded((H, n, PX), 44)
    _lib.LIB.vp_set_kernel_variant(0, variant)
    try:
        outs = []
        for _ in range(2):
            yo = torch.tensor(y0, device="cuda")
            vp._CU.forward_z2(torch.tensor(x, device="cuda"), yo, torch.tensor(ang, device="cuda"))
            torch.cuda.synchronize()
            outs.append(yo.cpu().numpy())
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
    np.testing.assert_array_equal(outs[0], outs[1])
    assert rel_err(outs[0] - y0, oracle.forward(x, ang, PX, 2)) <= tol.ref_vs_fp64(PX)


@pytest.mark.parametrize("geom", [(48, 40, 512, 70, 52, "wide"), (33, 29, 256, 45, 40, "axes"),
                                  (40, 44, 772, 300, 47, "rand"), (16, 16, 264, 9, 20, "pi")],
                         ids=lambda g: "x".join(map(str, g[:5])) + g[5])
def test_adjoint_bulk_copy_variant_is_bit_identical(geom):
    """Variant 9 fetches the 8-height windows with bulk copies into shared
    memory; the arithmetic is variant 7's, so the results are equal bit for
    bit, and no bounded wait runs out.  Angle counts past one list pass
    (256) and past one table chunk, windows at the detector edge, heights
    with a 4-height remainder."""
    from voxelproj_gb300 import _lib

    SY, SX, H, n, PX, kind = geom
    ang = torch.tensor(angle_set(kind, n, 97), device="cuda")
    y = torch.tensor(seeded((n, PX, H), 35), device="cuda")
    x0 = torch.tensor(seeded((SY, SX, H), 36), device="cuda")
    before = _lib.LIB.vp_wait_timeouts()
    outs = {}
    try:
        for v in (7, 9):
            _lib.LIB.vp_set_kernel_variant(1, v)
            xo = x0.clone()
            vp._CU.backward_z0(y, xo, ang)
            torch.cuda.synchronize()
            outs[v] = xo
    finally:
        _lib.LIB.vp_set_kernel_variant(1, 0)
    assert torch.equal(outs[7], outs[9])
    assert _lib.LIB.vp_wait_timeouts() == before


@pytest.mark.parametrize("geom", [(64, 64, 256, 96, 64, "pi"), (70, 64, 260, 97, 90, "rand"),
                                  (40, 48, 512, 70, 52, "wide"), (128, 96, 384, 200, 130, "pi"),
                                  (33, 29, 132, 45, 40, "axes"), (96, 96, 256, 1024, 96, "pi"),
                                  (200, 180, 256, 13, 150, "pi")],
                         ids=lambda g: "x".join(map(str, g[:5])) + g[5])
@pytest.mark.parametrize("variant,plain", [(17, 10), (19, 10)])
def test_staged_forward_is_bit_identical(geom, variant, plain):
    """The aligned forms (four aligned neighbouring angles per block; 17
    stages the volume in shared memory by tensor copies, 19 loads it plainly)
    sum the same candidates in the same order as variant 10 with the same 64
    MB class slabs, so the results are equal bit for bit:
    sorted and unsorted angles, angle counts not a multiple of the group,
    partial height chunks, rectangular volumes, narrow and wide detectors."""
    from voxelproj_gb300 import _lib

    SY, SX, H, n, PX, kind = geom
    ang = torch.tensor(angle_set(kind, n, 96), device="cuda")
    x = torch.tensor(seeded((SY, SX, H), 37), device="cuda")
    y0 = torch.tensor(seeded((n, PX, H), 38), device="cuda")
    before = _lib.LIB.vp_wait_timeouts()
    outs = {}
    try:
        for v in (plain, variant):
            _lib.LIB.vp_set_kernel_variant(0, v)
            yo = y0.clone()
            vp._CU.forward_z0(x, yo, ang)
            torch.cuda.synchronize()
            outs[v] = yo
    finally:
        _lib.LIB.vp_set_kernel_variant(0, 0)
    assert torch.equal(outs[plain], outs[variant])
    assert _lib.LIB.vp_wait_timeouts() == before
