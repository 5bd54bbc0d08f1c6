"""The oracle against the mathematics it restates (CPU only).

These tests pin the FP64 oracle independently of any GPU code:
  * bin weights equal the area of the unit voxel falling in each detector bin
    (integrated over a fine grid of points of the rotated square);
  * weights sum to one (the reference's weight-sum study, WoxelWeight.ipynb);
  * closed-form answers at 0, pi/2 and pi/4;
  * A and A^T are exact transposes (adjoint identity to rounding);
  * computing a subset of heights equals the same slice of the full result;
  * the FP32 CPU port agrees with FP64.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests.common import lin, rel_err, seeded, x_shape, y_shape


def area_weights(phi: float, xp: float, n: int = 1500):
    """Fractions of a unit square centred at detector coordinate xp that fall
    in bins round(xp)-1, round(xp), round(xp)+1 at angle phi (midpoint grid)."""
    c, s = np.cos(np.float64(np.float32(phi))), np.sin(np.float64(np.float32(phi)))
    t = (np.arange(n) + 0.5) / n - 0.5
    u, v = np.meshgrid(t, t, indexing="ij")
    d = xp + u * c + v * s
    r = np.rint(xp)
    edges = np.array([r - 1.5, r - 0.5, r + 0.5, r + 1.5])
    hist, _ = np.histogram(d.ravel(), bins=edges)
    return int(r), hist / d.size


@pytest.mark.parametrize("phi", [0.0, 0.3, np.pi / 4, 1.0, np.pi / 2 - 0.05, 2.0, 2.9, -1.2, 5.5])
@pytest.mark.parametrize("xp", [10.0, 10.2, 10.49, 10.5001, 9.73])
def test_weights_are_voxel_area_per_bin(phi, xp):
    r, w = oracle.weights(phi, xp)
    r2, w2 = area_weights(phi, xp)
    assert r == r2
    # midpoint-grid quadrature of a piecewise-linear density: error ~ 1/n
    np.testing.assert_allclose(w, w2, atol=2e-3)
    assert abs(w.sum() - 1.0) < 1e-14


@pytest.mark.parametrize("phi", [0.0, 0.3, np.pi / 4, 1.0, np.pi / 2, 2.0, 3 * np.pi / 4, -1.2,
                                 5.5, 15.0])
def test_angle_params_trapezoid(phi):
    """Per-angle constants (sp_backward_z0.cuh:45-58): the unit square's
    footprint at angle phi is a trapezoid with plateau half-width a and foot
    half-width b, the two values |c -+ s| / 2 in increasing order, and height
    ymax = 1 / (a + b), so that its area is one."""
    k = oracle.angle_params(phi)
    p = np.float64(np.float32(phi))
    c, s = np.cos(p), np.sin(p)
    np.testing.assert_allclose([k["c"], k["s"]], [c, s], rtol=0, atol=1e-15)
    half = sorted([abs(c - s) / 2, abs(c + s) / 2])
    np.testing.assert_allclose([k["a"], k["b"]], half, rtol=0, atol=1e-15)
    assert 0.0 <= k["a"] <= k["b"]
    np.testing.assert_allclose(k["ymax"] * (k["a"] + k["b"]), 1.0, rtol=1e-15)
    # a + b = max(|c|, |s|): the footprint's foot is as wide as the square's
    # longer projected side
    np.testing.assert_allclose(k["a"] + k["b"], max(abs(c), abs(s)), rtol=1e-15)


def test_weights_closed_forms():
    # phi = 0: box of width 1 -> all weight in the nearest bin at integer xp
    r, w = oracle.weights(0.0, 7.0)
    assert r == 7 and np.allclose(w, [0, 1, 0], atol=0)
    # phi = pi/4: triangle of half-width b = sqrt(2)/2 and height 1/b; the
    # area beyond +-1/2 is (b - 1/2)^2 / (2 b^2) = (b - 1/2)^2 on each side
    b = np.sqrt(2) / 2
    r, w = oracle.weights(np.pi / 4, 7.0)
    edge = (b - 0.5) ** 2
    np.testing.assert_allclose(w, [edge, 1 - 2 * edge, edge], rtol=1e-6)
    # mirror symmetry of the footprint
    r1, w1 = oracle.weights(0.7, 7.3)
    r2, w2 = oracle.weights(0.7, 6.7)
    np.testing.assert_allclose(w1, w2[::-1], atol=1e-15)


def test_weight_sum_known_answer():
    """A single lit voxel projects to total weight H at every angle
    (reference study: WoxelWeight.ipynb, error ~1e-7..1e-6 in float)."""
    x = np.zeros((9, 10, 3), np.float32)
    x[4, 6, :] = 1.0
    ang = lin(181, 0, 2 * np.pi)
    Ax = oracle.forward(x, ang, 20, 0)
    np.testing.assert_allclose(Ax.sum(axis=(1, 2)), 3.0, atol=1e-12)


@pytest.mark.parametrize("z", [0, 2])
def test_angle_zero_is_column_sum(z):
    SY, SX, H = 7, 9, 4
    x = seeded(x_shape(z, SY, SX, H), 1)
    Ax = oracle.forward(x, np.zeros(1, np.float32), SX, z)
    xz0 = x if z == 0 else x.transpose(1, 2, 0)
    ref = xz0.astype(np.float64).sum(axis=0)  # (SX, H)
    got = Ax[0] if z == 0 else Ax[:, 0, :].T
    np.testing.assert_allclose(got, ref, atol=1e-12)


def test_angle_half_pi_is_row_sum():
    SY, SX, H = 8, 6, 2
    x = seeded((SY, SX, H), 2)
    Ax = oracle.forward(x, np.array([np.pi / 2], np.float32), SY, 0)
    np.testing.assert_allclose(Ax[0], x.astype(np.float64).sum(axis=1), atol=1e-6)


@pytest.mark.parametrize("z", [0, 2])
@pytest.mark.parametrize("PX", [11, 4, 17])
def test_adjoint_identity_fp64(z, PX):
    SY, SX, H, n = 6, 5, 3, 31
    ang = lin(n)
    x = seeded(x_shape(z, SY, SX, H), 3, "uniform")
    y = seeded(y_shape(z, n, PX, H), 4, "uniform")
    Ax = oracle.forward(x, ang, PX, z)
    ATy = oracle.backward(y, ang, SY, SX, z)
    lhs = np.vdot(Ax, y.astype(np.float64))
    rhs = np.vdot(x.astype(np.float64), ATy)
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


def test_height_subset_matches_full():
    SY, SX, H, n, PX = 12, 10, 9, 20, 16
    ang = lin(n)
    x = seeded((H, SY, SX), 5)
    y = seeded((H, n, PX), 6)
    hl = [0, 4, 8]
    full = oracle.forward_f64(x, ang, PX, 2)
    sub = oracle.forward_f64(x, ang, PX, 2, h_list=hl)
    np.testing.assert_array_equal(full[hl], sub)
    fullb = oracle.backward_f64(y, ang, SY, SX, 2)
    subb = oracle.backward_f64(y, ang, SY, SX, 2, h_list=hl)
    np.testing.assert_array_equal(fullb[hl], subb)


@pytest.mark.parametrize("z", [0, 2])
def test_fp32_port_matches_fp64(z):
    SY, SX, H, n, PX = 20, 24, 6, 45, 30
    ang = lin(n, -np.pi / 2, 3 * np.pi / 2)
    x = seeded(x_shape(z, SY, SX, H), 7)
    y = seeded(y_shape(z, n, PX, H), 8)
    y32 = np.zeros(y_shape(z, n, PX, H), np.float32)
    oracle.forward_f32_(x, y32, ang, z)
    x32 = np.zeros(x_shape(z, SY, SX, H), np.float32)
    oracle.backward_f32_(y, x32, ang, z)
    assert rel_err(y32, oracle.forward(x, ang, PX, z)) < 2e-6
    assert rel_err(x32, oracle.backward(y, ang, SY, SX, z)) < 2e-6


def test_degenerate_angles_finite():
    # k*pi/2 give a == b (empty quadratic pieces); results must stay finite
    ang = np.array([0, np.pi / 2, np.pi, 3 * np.pi / 2, -np.pi], np.float32)
    x = seeded((5, 5, 2), 9)
    Ax = oracle.forward(x, ang, 5, 0)
    assert np.isfinite(Ax).all()
    y = seeded((5, 5, 2), 10)
    assert np.isfinite(oracle.backward(y, ang, 5, 5, 0)).all()
