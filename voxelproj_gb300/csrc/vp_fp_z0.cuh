// Per-warp body of the z_order 0 forward projection (detector-driven
// gather), shared by the single-problem kernel (vp_forward.cu) and the
// batched persistent kernel (vp_batch.cu).  See vp_forward.cu for the design.
#pragma once

#include "vp_common.cuh"

namespace vp {
namespace detail {

constexpr float kWindowMargin = 1e-3f;

// Minor-axis index range [lo, hi] (clamped to [0, n_minor)) of voxels on major
// line i whose detector coordinate can fall in [t_lo, t_hi].
struct MinorRange {
  int lo, hi;
};

__device__ __forceinline__ MinorRange minor_range(int i, float cent_major, float sh_major,
                                                  float cent_minor, float inv_sh_minor,
                                                  int min_lo, int min_hi, float pcent,
                                                  float t_lo, float t_hi) {
  const float K = ((float)i - cent_major) * sh_major + pcent;
  const float u1 = (t_lo - K) * inv_sh_minor + cent_minor;
  const float u2 = (t_hi - K) * inv_sh_minor + cent_minor;
  MinorRange m;
  m.lo = max(min_lo, (int)ceilf(fminf(u1, u2)));
  m.hi = min(min_hi, (int)floorf(fmaxf(u1, u2)));
  return m;
}

// ---------------------------------------------------------------------------
// z_order 0: x (SY, SX, H), y (n_ang, PX, H); heights contiguous.
// A warp owns angle a, KW consecutive bins and 32*R heights (lane <->
// heights; with R = 8 a lane holds two float4, 128 heights apart).  The voxels gathered are warp-uniform, so the warp enumerates
// them cooperatively: lane j takes major line i0+j, computes its candidate
// voxels and their bin weights into a per-warp shared list (offsets from a
// warp prefix sum), then all lanes stream the list with broadcast reads,
// UN candidates at a time so their loads overlap, and accumulate
// the KW bins in registers.  A candidate's three bins sit at run-relative
// offsets q-2, q-1, q (q = round(xp) - p0 + 1), dispatched with a
// warp-uniform switch.
//
// Cache locality: every angle touches the whole volume, so a launch is
// restricted to one slab of the volume (all launches add into y), and heights
// are the slowest grid axis.  Concurrently running blocks then share one slab
// x one height chunk, a few tens of MB that stay in L2 across all angles
// instead of being re-read from HBM per angle.  With row slabs, angles whose
// minor axis is y still walk every column per slab, mostly finding no
// candidate in it; class slabs give those angles a block of columns instead,
// so every warp walks only the major lines of its slab.
// With AGROUP the four warps of a block take four consecutive angles of the
// same bins, so their voxel strips overlap near the rotation centre (L1 hits
// of 46-58% at 512^3 against 10% for neighbouring bins): the default of the
// 8-height form.  In the 4-height form neighbouring bins measured faster.
// ---------------------------------------------------------------------------
constexpr int FP0_WARPS = 4;
constexpr int FP0_QBITS = 4;   // q in [0, KW + 1]
constexpr int FP0_UNROLL = 4;  // candidates whose loads are in flight together (R <= 4)

// Most candidates one major line can hold: the window [t_lo, t_hi] is
// KW + 2b + 2 * kWindowMargin bins wide with b <= sqrt(1/2), and neighbouring
// voxels on the minor axis are at least sqrt(1/2) bins apart, so a line holds
// at most floor((KW + sqrt(2) + 2 * margin) * sqrt(2)) + 1 of them (1.4142136
// rounds sqrt(2) up).  The list builder clamps a line's count to the cap; the
// assert below makes the clamp unreachable for every geometry, so no
// candidate can be dropped.
__host__ __device__ constexpr int fp0_line_bound(int KW) {
  return (int)(((float)KW + 1.4142136f + 2.0f * kWindowMargin) * 1.4142136f) + 1;
}

template <int KW>
struct Fp0Cap {
  static constexpr int value = KW == 4 ? 8 : 14;
  static_assert(value >= fp0_line_bound(KW), "a line's candidates must fit the list");
  // a warp's list: 32 lines of candidates, then padding for the loads of the
  // last group of FP0_UNROLL
  static constexpr int list = 32 * value + 4;
  static_assert(KW == 4 || KW == 8, "bins per warp: 4 or 8");
  static_assert(KW + 1 < (1 << FP0_QBITS), "q must fit its bits");
  static_assert(FP0_UNROLL <= 4, "list padding");
};

// Adds a candidate's weights to the run's accumulators: bin q-2 gets w0, q-1
// gets w1, q gets w2 (run-relative); bins outside [0, KW) are dropped.
template <int KW, int Q, typename V>
__device__ __forceinline__ void scatter3(V (&acc)[KW], const float4& e, const V& xv) {
  if constexpr (Q - 2 >= 0 && Q - 2 < KW) acc[Q - 2] = f4_fma(e.x, xv, acc[Q - 2]);
  if constexpr (Q - 1 >= 0 && Q - 1 < KW) acc[Q - 1] = f4_fma(e.y, xv, acc[Q - 1]);
  if constexpr (Q < KW) acc[Q] = f4_fma(e.z, xv, acc[Q]);
}

template <int KW, typename V>
__device__ __forceinline__ void scatter_q(V (&acc)[KW], const float4& e, const V& xv, int q) {
#define VP_Q_CASE(Q)                                            \
  case Q:                                                       \
    if constexpr (Q <= KW + 1) scatter3<KW, Q>(acc, e, xv);     \
    break;
  // the list builder clamps q to [0, KW + 1]: no range check needed
  __builtin_assume(q >= 0 && q <= KW + 1);
  switch (q) {
    VP_Q_CASE(0) VP_Q_CASE(1) VP_Q_CASE(2) VP_Q_CASE(3) VP_Q_CASE(4)
    VP_Q_CASE(5) VP_Q_CASE(6) VP_Q_CASE(7) VP_Q_CASE(8) VP_Q_CASE(9)
    default: break;
  }
#undef VP_Q_CASE
}

// The part of the volume one launch (or one batch stage) gathers from.
// Angles whose minor axis is x walk rows [y_lo, y_hi) (all columns); angles
// whose minor axis is y walk columns [x_lo, x_hi) within rows [yy_lo, yy_hi).
//   row slabs:   {y_lo, y_hi, 0, SX, y_lo, y_hi}  (one block of rows for all)
//   class slabs: {y_lo, y_hi, x_lo, x_hi, 0, SY}  (rows for one class,
//                                                  columns for the other)
// An empty range leaves that class's outputs untouched when adding (and
// writes zeros in store mode), so a launch can serve one class alone.
struct Slab {
  int y_lo, y_hi;
  int x_lo, x_hi;
  int yy_lo, yy_hi;
};

__host__ __device__ inline Slab row_slab(int y_lo, int y_hi, int SX) {
  return Slab{y_lo, y_hi, 0, SX, y_lo, y_hi};
}

// Slab k of a slab plan: row slabs of wy rows, or class slabs of wy rows and
// wx columns (ranges clamped to the volume).
__host__ __device__ inline Slab slab_of(int k, bool cls, int wy, int wx, int SY, int SX) {
  const int y_lo = k * wy < SY ? k * wy : SY;
  const int y_hi = y_lo + wy < SY ? y_lo + wy : SY;
  if (!cls) return row_slab(y_lo, y_hi, SX);
  const int x_lo = k * wx < SX ? k * wx : SX;
  const int x_hi = x_lo + wx < SX ? x_lo + wx : SX;
  return Slab{y_lo, y_hi, x_lo, x_hi, 0, SY};
}

// One warp: angle a, bins [p0, p0 + nb) (nb <= KW), this lane's heights from h (LaneH:
// R = 8 is [h, h + 4) and [h + 128, h + 132)), the voxels of slab s.  FULL:
// every lane's heights are inside [0, H).
// UN candidates are loaded together.  cand is this warp's shared candidate list of
// Fp0Cap<KW>::list entries.  All 32 lanes must call it together.
// wait() runs (by the whole warp) just before the outputs are written; with
// Wait::coherent the read of the output bypasses L1.
template <int R, int KW, int UN = FP0_UNROLL, class Wait = NoWait, bool FULL = false>
__device__ __forceinline__ void fp_z0_warp(const float* __restrict__ x, float* __restrict__ y,
                                           const float* __restrict__ angles, const Geom& g,
                                           int p0, int a, int h, const Slab& s,
                                           int accumulate, float4* cand,
                                           const Wait& wait = Wait(), int nb = KW) {
  using V = typename Vec<R>::T;
  constexpr int CAP = Fp0Cap<KW>::value;
  const int lane = threadIdx.x & 31;
  if (p0 >= g.PX || a >= g.n_ang) {  // warp-uniform
    wait();
    return;
  }
  const LaneH<R> lh(h, g.H);

  const AngleConst k = angle_const(__ldg(angles + a), g.trig);
  const bool minor_x = fabsf(k.c) >= fabsf(k.s);
  // major lines [maj_lo, maj_hi), minor indices [min_lo, min_hi], within the slab
  const int maj_lo = minor_x ? s.y_lo : s.x_lo;
  const int maj_hi = minor_x ? s.y_hi : s.x_hi;
  if (maj_lo >= maj_hi && accumulate) {  // warp-uniform: nothing of this slab to add
    wait();
    return;
  }
  const int min_lo = minor_x ? 0 : s.yy_lo;
  const int min_hi = minor_x ? g.SX - 1 : s.yy_hi - 1;
  const float cent_major = minor_x ? g.ycent : g.xcent;
  const float cent_minor = minor_x ? g.xcent : g.ycent;
  const float sh_major = minor_x ? k.s : k.c;
  const float inv_sh_minor = 1.0f / (minor_x ? k.c : k.s);
  const float t_lo = (float)p0 - 0.5f - k.b - kWindowMargin;
  const float t_hi = (float)(p0 + nb) - 0.5f + k.b + kWindowMargin;

  V acc[KW];
#pragma unroll
  for (int b = 0; b < KW; ++b) acc[b] = vzero<V>();
  const float* xs = x + lh.s0;

  for (int i0 = maj_lo; i0 < maj_hi; i0 += 32) {
    const int i = i0 + lane;
    int lo = 0, cnt = 0;
    if (i < maj_hi) {
      const MinorRange mr = minor_range(i, cent_major, sh_major, cent_minor, inv_sh_minor,
                                        min_lo, min_hi, g.pcent, t_lo, t_hi);
      lo = mr.lo;
      cnt = max(0, min(mr.hi - mr.lo + 1, CAP));
    }
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += n;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int start = incl - cnt;
    for (int t = 0; t < cnt; ++t) {
      const int m = lo + t;
      const int xi = minor_x ? m : i;
      const int yi = minor_x ? i : m;
      const BinWeights bw =
          voxel_weights((float)xi - g.xcent, (float)yi - g.ycent, k, g.pcent, g.trig);
      int q = bw.r - p0 + 1;
      float4 e = make_float4(bw.w0, bw.w1, bw.w2, 0.0f);
      if (q < 0 || q > KW + 1) {
        q = 0;
        e = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      const int vox = yi * g.SX + xi;
      e.w = __int_as_float((vox << FP0_QBITS) | q);
      cand[start + t] = e;
    }
    // padding after the list: voxel 0 with zero weights, so that the last
    // group's loads need no condition (its extra entries are not added)
    if (lane < UN) cand[total + lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    for (int c0 = 0; c0 < total; c0 += UN) {
      float4 e[UN];
      V xv[UN];
#pragma unroll
      for (int u = 0; u < UN; ++u) {
        e[u] = cand[c0 + u];
        const int vox = __float_as_int(e[u].w) >> FP0_QBITS;
        xv[u] = lh.template load<FULL>(xs + (size_t)vox * g.Hx);
      }
#pragma unroll
      for (int u = 0; u < UN; ++u) {
        if (c0 + u >= total) break;  // padding slots (warp-uniform)
        scatter_q<KW>(acc, e[u], xv[u], __float_as_int(e[u].w) & ((1 << FP0_QBITS) - 1));
      }
    }
    __syncwarp();
  }

  wait();
#pragma unroll
  for (int b = 0; b < KW; ++b) {
    const int p = p0 + b;
    if (p < g.PX && b < nb)
      store_lane<R, Wait::coherent>(y + ((size_t)a * g.PX + p) * g.Hy, lh, acc[b], accumulate);
  }
}

}  // namespace detail
}  // namespace vp
