"""Seeded synthetic inputs that numpy (CPU) and torch (CPU or CUDA) produce
bit for bit alike, on any machine and any library version.

The parity tests at the full benchmark sizes (512^3 volumes, sinograms of up
to 1024 angles) need the same input on the machine that records the
reference's outputs and on the machine that checks against them, without
storing hundreds of MB.  A pseudo-random generator's stream is not promised
to stay the same across numpy / torch versions or CPU and GPU back ends, so
each value here is a pure function of (seed, index), computed with integer
arithmetic that never overflows int64:

  * a 32-bit integer hash (the "lowbias32" mixer: xor-shifts and two odd
    multipliers) of the element's flat index and the seed, twice;
  * four 16-bit uniforms u_i from the two hashes; their sum is exact;
  * v = (sum_i (u_i + 1/2) / 65536 - 2) * sqrt(3): an Irwin-Hall(4) variate
    scaled to unit variance, a bounded stand-in for N(0, 1) (|v| < 3.47),
    rounded once to float32.

The flat index is taken in a canonical (height, row, column) order, so the
z_order 0 and z_order 2 layouts of one seed hold the same values, transposed.
"""

from __future__ import annotations

import numpy as np

_M16 = 0xFFFF
_M32 = 0xFFFFFFFF
_C1 = 0x7FEB352D
_C2 = 0x846CA68B
_SCALE = float(np.sqrt(3.0)) / 65536.0


def _mul32(x, c: int):
    """(x * c) mod 2^32 for 0 <= x < 2^32, without leaving int64."""
    return (x * (c & _M16) + (((x * (c >> 16)) & _M16) << 16)) & _M32


def _hash32(x):
    x = x ^ (x >> 16)
    x = _mul32(x, _C1)
    x = x ^ (x >> 15)
    x = _mul32(x, _C2)
    return x ^ (x >> 16)


def _values(flat, seed: int, xp):
    """Values for int64 flat indices (numpy or torch array)."""
    s = (seed * 0x9E37 + 0x51ED) & _M32
    k0 = (flat * 2) & _M32
    h1 = _hash32(k0 ^ s)
    h2 = _hash32(((k0 + 1) & _M32) ^ s)
    tot = (h1 & _M16) + (h1 >> 16) + (h2 & _M16) + (h2 >> 16) - 131070
    if xp is np:
        return (tot.astype(np.float64) * _SCALE).astype(np.float32)
    import torch

    return (tot.to(torch.float64) * _SCALE).to(torch.float32)


def canonical_numpy(seed: int, dims, heights):
    """Values at (h, j, k) for h in `heights`, all j < dims[1], k < dims[2],
    of a canonical (H, D1, D2) array; returns float32 (len(heights), D1, D2)."""
    _, D1, D2 = dims
    h = np.asarray(heights, np.int64).reshape(-1, 1, 1)
    j = np.arange(D1, dtype=np.int64).reshape(1, -1, 1)
    k = np.arange(D2, dtype=np.int64).reshape(1, 1, -1)
    flat = (h * D1 + j) * D2 + k
    return _values(flat, seed, np)


def canonical_torch(seed: int, dims, device, h_chunk: int = 16):
    """The whole canonical (H, D1, D2) float32 array as a torch tensor on
    `device`, generated in chunks of heights to bound the int64 temporaries."""
    import torch

    H, D1, D2 = dims
    out = torch.empty((H, D1, D2), dtype=torch.float32, device=device)
    plane = (torch.arange(D1, dtype=torch.int64, device=device).view(-1, 1) * D2
             + torch.arange(D2, dtype=torch.int64, device=device).view(1, -1))
    for h0 in range(0, H, h_chunk):
        h1 = min(H, h0 + h_chunk)
        hs = torch.arange(h0, h1, dtype=torch.int64, device=device).view(-1, 1, 1)
        out[h0:h1] = _values(hs * (D1 * D2) + plane.unsqueeze(0), seed, torch)
    return out


def layout_numpy(canon, z_order: int):
    """(n_h, D1, D2) canonical planes -> the z_order layout (z0: (D1, D2, n_h))."""
    return np.ascontiguousarray(canon.transpose(1, 2, 0)) if z_order == 0 else canon


def layout_torch(canon, z_order: int):
    """Same for a torch tensor (a contiguous copy for z_order 0)."""
    return canon.permute(1, 2, 0).contiguous() if z_order == 0 else canon
