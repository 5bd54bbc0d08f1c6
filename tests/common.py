"""Shared helpers for the tests: geometries, seeded inputs, error metrics."""

from __future__ import annotations

import numpy as np


def x_shape(z, SY, SX, H):
    return (SY, SX, H) if z == 0 else (H, SY, SX)


def y_shape(z, n, PX, H):
    return (n, PX, H) if z == 0 else (H, n, PX)


def rel_err(got, ref) -> float:
    """max|got - ref| / max|ref| (the parity metric; 0 for an all-zero ref)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.abs(ref).max() if ref.size else 0.0
    num = np.abs(got - ref).max() if ref.size else 0.0
    return float(num / den) if den > 0 else float(num)


def seeded(shape, seed, kind="normal"):
    rng = np.random.default_rng(seed)
    if kind == "normal":
        return rng.standard_normal(shape).astype(np.float32)
    return rng.random(shape).astype(np.float32)


def lin(n, lo=0.0, hi=np.pi):
    return np.linspace(lo, hi, n).astype(np.float32)
