// Shared device math of the exact-trapezoid parallel-beam projector pair.
//
// Geometry (reference voxelproj, sp_backward_z0.cuh:24-26 and :84): voxel and
// detector pitch are 1; the volume centre is ((SX-1)/2, (SY-1)/2), the
// detector centre (PX-1)/2, and voxel (xi, yi) lands on detector coordinate
//     xp = (xi - xcent) * cos(phi) + (yi - ycent) * sin(phi) + pcent.
// A unit voxel seen at angle phi is a trapezoid of area one with plateau
// half-width a = min(|c-s|, |c+s|)/2, base half-width b = max(...)/2 and
// height 1/(a+b) (sp_backward_z0.cuh:45-58).  Because b <= sqrt(2)/2 it covers
// at most the three bins round(xp)-1, round(xp), round(xp)+1 (:85-95), whose
// weights are differences of the trapezoid's piecewise-quadratic CDF
// (projection_common.cuh:139-166).
//
// The weights do not depend on the height index h, so every kernel computes
// them once per (voxel, angle) and applies them to a vector of heights.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vp {

// Trig used for the per-angle constants.
//   TRIG_REF:     the hardware approximations (__sincosf, approximate
//                 reciprocal) that the reference's --use_fast_math build uses
//                 for cos/sin/sincosf and '/', so results track its kernels.
//   TRIG_PRECISE: CUDA's accurate sincosf and IEEE division.
enum TrigMode : int { TRIG_REF = 0, TRIG_PRECISE = 1 };

// Per-angle constants: (c, s) and the CDF parameters (a, b, coeff, cd) with
// coeff = h/2 and cd = coeff/(b-a) (sp_backward_z0.cuh:45-58).  cd is set to
// zero when b == a (angles k*pi/2): the quadratic pieces are empty there, and
// a zero keeps every select in trap_cdf free of inf*0.
struct AngleConst {
  float c, s;
  float a, b, coeff, cd;
};

__device__ __forceinline__ AngleConst angle_const(float phi, int trig) {
  AngleConst k;
  float s, c;
  if (trig == TRIG_REF) {
    __sincosf(phi, &s, &c);
  } else {
    sincosf(phi, &s, &c);
  }
  k.c = c;
  k.s = s;
  const float cms = fabsf(0.5f * (c - s));
  const float cps = fabsf(0.5f * (c + s));
  const float a = fminf(cms, cps);
  const float b = fmaxf(cms, cps);
  const float den = (b - a) + 2.0f * a;
  float lmax, coeff, cd;
  if (trig == TRIG_REF) {
    lmax = __fdividef(1.0f, den);
    coeff = 0.5f * lmax;
    cd = (b > a) ? __fdividef(coeff, b - a) : 0.0f;
  } else {
    lmax = 1.0f / den;
    coeff = 0.5f * lmax;
    cd = (b > a) ? coeff / (b - a) : 0.0f;
  }
  k.a = a;
  k.b = b;
  k.coeff = coeff;
  k.cd = cd;
  return k;
}

// Trapezoid CDF F(x) for a footprint centred at 0 (projection_common.cuh:139-166):
//   0                          x <= -b
//   cd*(x+b)^2                 -b < x < -a
//   coeff*(b+a) + 2*coeff*x    -a <= x < a
//   1 - cd*(b-x)^2             a <= x < b
//   1                          x >= b
__device__ __forceinline__ float trap_cdf(float x, float a, float b, float coeff, float cd) {
  const float xl = __fadd_rn(x, b);
  const float xr = __fsub_rn(b, x);
  const float left = __fmul_rn(__fmul_rn(cd, xl), xl);
  const float mid = __fmaf_rn(coeff, __fadd_rn(b, a), __fmul_rn(__fmul_rn(2.0f, coeff), x));
  const float right = __fmaf_rn(-__fmul_rn(cd, xr), xr, 1.0f);
  float r = (x < b) ? right : 1.0f;
  r = (x < a) ? mid : r;
  r = (x < -a) ? left : r;
  r = (x <= -b) ? 0.0f : r;
  return r;
}

// Detector coordinate of a voxel with centred coordinates (relx, rely), with a
// fixed rounding order: xp = fma(relx, c, rely*s) + pcent.  Every kernel and
// both directions use it, so A and A^T carry bit-identical weights.  With the
// CDF below and TRIG_REF, A^T reproduces the reference's kernels bit for bit
// (checked against its recorded outputs).
__device__ __forceinline__ float det_coord(float relx, float rely, float c, float s, float pcent) {
  return __fadd_rn(__fmaf_rn(relx, c, __fmul_rn(rely, s)), pcent);
}

// Weights of bins r-1, r, r+1 for a voxel projecting to xp
// (sp_backward_z0.cuh:84-91): r = round-half-even(xp), xv = r - xp,
// w0 = F(xv-1/2), w1 = F(xv+1/2) - F(xv-1/2), w2 = 1 - F(xv+1/2).
struct BinWeights {
  int r;
  float w0, w1, w2;
};

__device__ __forceinline__ BinWeights weights_from_offset(int r, float xv, const AngleConst& k) {
  BinWeights o;
  o.r = r;
  const float v1 = trap_cdf(xv - 0.5f, k.a, k.b, k.coeff, k.cd);
  const float v2 = trap_cdf(xv + 0.5f, k.a, k.b, k.coeff, k.cd);
  o.w0 = v1;
  o.w1 = v2 - v1;
  o.w2 = 1.0f - v2;
  return o;
}

__device__ __forceinline__ BinWeights bin_weights(float xp, const AngleConst& k) {
  const int r = __float2int_rn(xp);
  return weights_from_offset(r, (float)r - xp, k);
}

// Error-free sum: s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

// Weights with the sub-bin offset xv = r - xp evaluated from an unrounded xp:
// the products and sums of xp are carried as (value, error) pairs with FMA
// and TwoSum, so at 512^3 the offset is not limited by the ~3e-5 px spacing
// of floats near 256.  Used by TRIG_PRECISE; TRIG_REF keeps the plain formula
// so that it rounds the way the reference does.
__device__ __forceinline__ BinWeights bin_weights_compensated(float relx, float rely,
                                                              const AngleConst& k,
                                                              float pcent) {
  const float p1 = __fmul_rn(relx, k.c);
  const float e1 = fmaf(relx, k.c, -p1);
  const float p2 = __fmul_rn(rely, k.s);
  const float e2 = fmaf(rely, k.s, -p2);
  float e3, e4;
  const float s1 = two_sum(p1, p2, e3);
  const float hi = two_sum(s1, pcent, e4);
  const float lo = (e1 + e2) + (e3 + e4);
  const int r = __float2int_rn(hi);
  const float xv = __fsub_rn((float)r, hi) - lo;
  return weights_from_offset(r, xv, k);
}

// The weights of voxel (relx, rely) at one angle, in the given trig mode.
__device__ __forceinline__ BinWeights voxel_weights(float relx, float rely, const AngleConst& k,
                                                    float pcent, int trig) {
  if (trig == TRIG_PRECISE) return bin_weights_compensated(relx, rely, k, pcent);
  return bin_weights(det_coord(relx, rely, k.c, k.s, pcent), k);
}

// acc + w * v per component, two components per instruction: the packed
// FP32 multiply-add of compute capability 10.x rounds each component as
// fmaf does, so results are those of four fmaf calls.
__device__ __forceinline__ float4 f4_fma(float w, float4 v, float4 acc) {
  const float2 ww = make_float2(w, w);
  const float2 lo = __ffma2_rn(ww, make_float2(v.x, v.y), make_float2(acc.x, acc.y));
  const float2 hi = __ffma2_rn(ww, make_float2(v.z, v.w), make_float2(acc.z, acc.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ float f4_fma(float w, float v, float acc) { return fmaf(w, v, acc); }

__device__ __forceinline__ float4 f4_add(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ float f4_add(float a, float b) { return a + b; }

template <typename T>
__device__ __forceinline__ T vzero();
template <>
__device__ __forceinline__ float vzero<float>() { return 0.0f; }
template <>
__device__ __forceinline__ float4 vzero<float4>() { return make_float4(0.f, 0.f, 0.f, 0.f); }

// Eight heights of one lane in two float4: [h, h + 4) and [h + 128, h + 132),
// so that each of the warp's two loads covers 512 contiguous bytes.
struct float4x2 {
  float4 a, b;
};
constexpr int kSecondHalf = 128;  // height offset of float4x2::b

__device__ __forceinline__ float4x2 f4_fma(float w, const float4x2& v, float4x2 acc) {
  acc.a = f4_fma(w, v.a, acc.a);
  acc.b = f4_fma(w, v.b, acc.b);
  return acc;
}
template <>
__device__ __forceinline__ float4x2 vzero<float4x2>() {
  return {vzero<float4>(), vzero<float4>()};
}

// Float vector of R heights per lane (R = 1, 4, or 8 as float4x2) and a
// guarded load of it.
template <int R>
struct Vec;
template <>
struct Vec<1> {
  using T = float;
};
template <>
struct Vec<4> {
  using T = float4;
};
template <>
struct Vec<8> {
  using T = float4x2;
};

// Height offsets of one lane: R = 1 or 4 heights from h; R = 8 as float4 at
// h and h + 128.  Lanes past H read offset 0 (always valid) and never store.
template <int R>
struct LaneH {
  static constexpr int NQ = R == 8 ? 2 : 1;  // float4 per lane
  int h, s0;
  int d[NQ];   // load offset of float4 k minus s0
  bool v[NQ];  // float4 k inside [0, H)
  __device__ __forceinline__ LaneH(int h_, int H) : h(h_) {
    s0 = h < H ? h : 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      v[k] = h + k * kSecondHalf < H;
      d[k] = (v[k] ? h + k * kSecondHalf : 0) - s0;
    }
  }
  // this lane's heights of a row, given q = row + s0.  FULL: every lane's
  // heights are inside [0, H) (whole chunks), so the second float4 is at the
  // constant offset kSecondHalf.
  template <bool FULL = false>
  __device__ __forceinline__ typename Vec<R>::T load(const float* q) const {
    if constexpr (R == 8) {
      float4x2 r;
      r.a = __ldg(reinterpret_cast<const float4*>(q));
      r.b = __ldg(reinterpret_cast<const float4*>(q + (FULL ? kSecondHalf : d[1])));
      return r;
    } else {
      return __ldg(reinterpret_cast<const typename Vec<R>::T*>(q));
    }
  }
};

template <typename V>
__device__ __forceinline__ V ld_or_zero(const float* p, bool ok) {
  return ok ? __ldg(reinterpret_cast<const V*>(p)) : vzero<V>();
}

// Geometry shared by all launches.  Volume (SY, SX) comes from x, detector
// (n_ang, PX) from y; H is min(Hx, Hy): heights past the shorter array read
// as zero in the reference (border-mode texture) and so leave the output
// unchanged, which computing only h < H reproduces.
struct Geom {
  int SY, SX;       // volume rows / columns
  int n_ang, PX;    // angles / detector bins
  int H;            // heights processed
  int Hx, Hy;       // height extent of x and of y (z_order 0 row strides)
  float xcent, ycent, pcent;
  int trig;
  int accumulate;   // 1: out += result (the reference's semantics); 0: out = result
};

// Epilogue: out (+)= acc.
__device__ __forceinline__ void store_out(float4* p, float4 v, int accumulate) {
  *p = accumulate ? f4_add(*p, v) : v;
}
__device__ __forceinline__ void store_out(float* p, float v, int accumulate) {
  *p = accumulate ? *p + v : v;
}

// Epilogue whose read bypasses L1 (ld.global.cg): for outputs that another
// block of the same launch, or the kernel before this one in a programmatic
// launch, wrote while this block ran, since L1 is not coherent across SMs.
__device__ __forceinline__ void store_out_coherent(float4* p, float4 v, int accumulate) {
  *p = accumulate ? f4_add(__ldcg(p), v) : v;
}
__device__ __forceinline__ void store_out_coherent(float* p, float v, int accumulate) {
  *p = accumulate ? __ldcg(p) + v : v;
}

// Epilogue of one lane's heights of the output row that starts at p.  With
// COHERENT the read of out bypasses L1 (accumulate only).
template <int R, bool COHERENT = false>
__device__ __forceinline__ void store_lane(float* p, const LaneH<R>& lh,
                                           const typename Vec<R>::T& v, int accumulate) {
  if constexpr (R == 8) {
    const float4* parts = reinterpret_cast<const float4*>(&v);
#pragma unroll
    for (int k = 0; k < LaneH<R>::NQ; ++k) {
      if (lh.v[k]) {
        float4* q = reinterpret_cast<float4*>(p + lh.h + k * kSecondHalf);
        if constexpr (COHERENT) store_out_coherent(q, parts[k], accumulate);
        else store_out(q, parts[k], accumulate);
      }
    }
  } else if (lh.v[0]) {
    auto* q = reinterpret_cast<typename Vec<R>::T*>(p + lh.h);
    if constexpr (COHERENT) store_out_coherent(q, v, accumulate); else store_out(q, v, accumulate);
  }
}

// One lane's heights of the output row at p: p = (p + v) + a when with_v,
// else p = p + a (a: the addend row, same layout).
template <int R>
__device__ __forceinline__ void add_lane(float* p, const float* a, const LaneH<R>& lh,
                                         const typename Vec<R>::T& v, bool with_v) {
  if constexpr (R == 8) {
    const float4* parts = reinterpret_cast<const float4*>(&v);
#pragma unroll
    for (int k = 0; k < LaneH<R>::NQ; ++k) {
      if (lh.v[k]) {
        float4* q = reinterpret_cast<float4*>(p + lh.h + k * kSecondHalf);
        const float4 c = __ldg(reinterpret_cast<const float4*>(a + lh.h + k * kSecondHalf));
        const float4 o = __ldcg(q);  // possibly written by the previous launch (PdlWait)
        const float4 t = with_v ? f4_add(o, parts[k]) : o;
        *q = f4_add(t, c);
      }
    }
  } else if (lh.v[0]) {
    using V = typename Vec<R>::T;
    V* q = reinterpret_cast<V*>(p + lh.h);
    const V c = *reinterpret_cast<const V*>(a + lh.h);
    const V o = __ldcg(q);
    const V t = with_v ? f4_add(o, v) : o;
    *q = f4_add(t, c);
  }
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization (launch_ex) may start while the kernel before it in its
// stream still runs.  pdl_trigger, run at the start of every block, lets such
// a successor start once every block of this kernel has begun; PdlWait, run
// by a warp just before it first reads back its outputs, holds until the
// kernels this one depends on have completed and their writes are visible.
// In a normally launched kernel, or one without a programmatic successor,
// both return at once.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// (the wait makes those writes visible to this grid, so the read-back needs
// no L1 bypass)
struct PdlWait {
  __device__ __forceinline__ void operator()() const {
    asm volatile("griddepcontrol.wait;" ::: "memory");
  }
  static constexpr bool coherent = false;
};

// Pre-store hook that does nothing (single-problem kernels).
struct NoWait {
  __device__ __forceinline__ void operator()() const {}
  static constexpr bool coherent = false;
};

// Pre-store hook of a block whose warps write the same outputs in two
// rounds: the second round waits at the block barrier that the first round
// reaches after writing (the writes are visible to the block after it).
struct HalfBarrier {
  bool second;
  __device__ __forceinline__ void operator()() const {
    if (second) __syncthreads();
  }
  static constexpr bool coherent = false;
};

}  // namespace vp
