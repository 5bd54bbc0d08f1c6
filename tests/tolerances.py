"""Parity tolerances, with where they come from.

Metric: max|got - ref| / max|ref| over the whole output (the north-star
parity metric).

FP32 sets the floor.  A detector coordinate xp ~ N/2 carries a rounding error
of a few ulp(N/2), i.e. ~1e-5 px at N = 512 and ~1.5e-6 px at N = 64.  That
moves a bin weight by up to 1.4x as much (the trapezoid height is at most
sqrt(2)), and random inputs average most of it out.

* TRIG_PRECISE vs FP64: accurate sincosf plus a compensated xp.  The error is
  a few 1e-7 from trig rounding times |xp - centre|, plus FP32 accumulation.
* TRIG_REF vs FP64: the reference's hardware sin/cos have an absolute error
  near 4e-7 on [-pi, pi] (more outside), which moves xp by ~4e-7 * N/2.
  That is ~2.5e-5 px at N = 128, i.e. a relative output error ~1e-5.
  It grows linearly with the volume size.
* vs the reference's own kernels (golden fixtures, TRIG_REF): the north-star
  bound, 1e-5 relative.
"""

# relative error bounds vs the FP64 oracle, for volumes up to ~64 voxels wide
PRECISE_VS_FP64 = 5e-6
REF_VS_FP64 = 5e-5
# vs the reference's CUDA kernels (spec parity target)
REF_VS_REFERENCE = 1e-5
# adjoint identity |<Ax,y> - <x,A^T y>| / (||Ax|| ||y||), FP64 inner products
ADJOINT = 1e-6
