"""The forward's per-line candidate cap is never reached (CPU only).

fp_z0_warp lists, for each major line of a warp's slab, the minor-axis voxels
whose detector coordinate can fall in the warp's window of KW bins
(minor_range in vp_fp_z0.cuh), and clamps the count to Fp0Cap<KW>::value
entries per line: a count above the cap would drop candidates silently.  The
window is KW + 2b + 2·margin bins wide (b <= √½) and the minor step is at
least √½, so a line holds at most floor((KW + √2 + 2·margin) / √½) + 1
voxels.  This test restates minor_range in float32 (as the kernel computes
it) over square and rectangular volumes, wide and narrow detectors, and
angles including multiples of π/4, and checks the largest count against the
bound and the cap read from the kernel source.
"""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "voxelproj_gb300" / "csrc" / "vp_fp_z0.cuh"
F = np.float32


def kernel_constants():
    text = SRC.read_text()
    m = re.search(r"static constexpr int value = KW == 4 \? (\d+) : (\d+);", text)
    assert m, "Fp0Cap<KW>::value not found"
    margin = re.search(r"constexpr float kWindowMargin = ([0-9.e+-]+)f;", text)
    assert margin, "kWindowMargin not found"
    return {4: int(m.group(1)), 8: int(m.group(2))}, float(margin.group(1))


def max_line_count(SY, SX, PX, phi, KW, margin):
    """Largest candidate count over all lines and bin runs of one angle."""
    c, s = F(np.cos(F(phi))), F(np.sin(F(phi)))
    b = F(max(abs(c - s), abs(c + s)) / F(2))
    minor_x = abs(c) >= abs(s)
    n_major, n_minor = (SY, SX) if minor_x else (SX, SY)
    cent_major = F(0.5) * F((SY if minor_x else SX) - 1)
    cent_minor = F(0.5) * F((SX if minor_x else SY) - 1)
    sh_major = s if minor_x else c
    inv_sh_minor = F(1) / (c if minor_x else s)
    pcent = F(0.5) * F(PX - 1)
    i = np.arange(n_major, dtype=F)[:, None]
    p0 = np.arange(0, PX, KW, dtype=F)[None, :]
    t_lo = p0 - F(0.5) - b - F(margin)
    t_hi = p0 + F(KW) - F(0.5) + b + F(margin)
    K = (i - cent_major) * sh_major + pcent
    u1 = (t_lo - K) * inv_sh_minor + cent_minor
    u2 = (t_hi - K) * inv_sh_minor + cent_minor
    lo = np.maximum(0, np.ceil(np.minimum(u1, u2)))
    hi = np.minimum(n_minor - 1, np.floor(np.maximum(u1, u2)))
    return int(max(0, (hi - lo + 1).max()))


GEOMS = [(512, 512, 512), (64, 64, 64), (40, 72, 57), (100, 30, 160), (17, 200, 9)]
SPECIAL = [0.0, np.pi / 4, np.pi / 2, 3 * np.pi / 4, np.pi, -np.pi / 4, 5 * np.pi / 4,
           np.pi / 4 + 1e-6, np.pi / 4 - 1e-6, 7.0, -12.5]


@pytest.mark.parametrize("KW", [4, 8])
def test_line_counts_stay_below_cap(KW):
    caps, margin = kernel_constants()
    bound = int(np.floor((KW + np.sqrt(2) + 2 * margin) / np.sqrt(0.5))) + 1
    assert bound <= caps[KW]
    rng = np.random.default_rng(11)
    angles = SPECIAL + list(rng.uniform(-10, 10, 60))
    worst = 0
    for SY, SX, PX in GEOMS:
        for phi in angles:
            worst = max(worst, max_line_count(SY, SX, PX, phi, KW, margin))
    assert worst <= bound <= caps[KW]
    # the bound is reached near 45 degrees, so it is not loose by more than one
    assert worst >= bound - 1
