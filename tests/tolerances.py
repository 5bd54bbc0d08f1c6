"""Parity tolerances, with where they come from.

Metric: max|got - ref| / max|ref| over the whole output (the parity metric).

FP32 limits every result.  A detector coordinate xp = relx*c + rely*s + pcent
is off by its trig error times the lever arm |relx| + |rely| ~ N, plus a few
ulp of N.  A bin weight moves by up to sqrt(2) times that (the trapezoid's
largest height), and random inputs average part of it out.  So the bounds
grow with the largest extent N = max(SY, SX, PX):

* TRIG_PRECISE vs FP64: accurate sincosf and a compensated xp; the residue
  is the float rounding of sin/cos (~6e-8) times N.
  Measured: 1.7e-8..2.7e-8 * N at N = 50..512.
* TRIG_REF vs FP64: the hardware sin/cos of the reference's fast-math build
  have an absolute error near 4e-7 on [-pi, pi], growing outside it.
  Measured: 1.4e-7..4.2e-7 * N at N = 40..512, for angles up to 4*pi
  (the largest on a 30x21 volume with 40 bins and 33 random angles).
* vs the reference's own kernels (golden fixtures, TRIG_REF): the parity
  target, 1e-5 relative, for A^T.  The reference's A marches rays with an
  accumulated float position.  It is itself off the exact operator by more
  than that, so A is held to "no further from the reference than the
  reference is from FP64" (test_golden.py).
"""

# fixed bounds used by the small API tests (extents <= 64)
PRECISE_VS_FP64 = 5e-6
REF_VS_FP64 = 5e-5
# vs the reference's CUDA kernels (parity target)
REF_VS_REFERENCE = 1e-5
# adjoint identity |<Ax,y> - <x,A^T y>| / (||Ax|| ||y||), FP64 inner products
ADJOINT = 1e-6


def precise_vs_fp64(n: int) -> float:
    """Bound for TRIG_PRECISE results on a geometry of largest extent n."""
    return max(1e-6, 5e-8 * n)


def ref_vs_fp64(n: int) -> float:
    """Bound for TRIG_REF results on a geometry of largest extent n."""
    return max(5e-6, 5e-7 * n)
