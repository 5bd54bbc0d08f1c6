// Per-warp body of the z_order 0 register-blocked adjoint (BX x BY voxel
// block per warp, bin window per angle in registers), shared by the
// single-problem kernel (vp_backward.cu) and the batched persistent kernel
// (vp_batch.cu).  It accumulates in the reference's order: angles ascending,
// bins r-1, r, r+1 per angle.
#pragma once

#include "vp_common.cuh"

namespace vp {
namespace detail {

constexpr int BPB_WARPS = 4;
constexpr int BPB_CHUNK = 32;

constexpr int isqrt(int v) {
  int r = 0;
  while ((r + 1) * (r + 1) <= v) ++r;
  return r;
}

template <int BX, int BY>
struct BlockWindow {
  // |xp_i - xp_j| <= sqrt((BX-1)^2 + (BY-1)^2) over the block (Cauchy-Schwarz)
  // and |round(xp) - xp| <= 1/2, so round(xp) spans at most
  // floor(sqrt(D2) + 1) = isqrt(D2) + 1.
  static constexpr int D2 = (BX - 1) * (BX - 1) + (BY - 1) * (BY - 1);
  static constexpr int OMAX = isqrt(D2) + 1;  // largest window offset of a voxel
  static constexpr int WMAX = OMAX + 3;       // largest window
};

// acc += e.x * win[O] + e.y * win[O+1] + e.z * win[O+2] for the runtime offset
// held in e.w; the cases are generated up to OMAX.
template <int O, int OMAX, typename V>
__device__ __forceinline__ void apply_window(V& acc, const float4& e, const V* win, int o) {
  if constexpr (O <= OMAX) {
    if (o == O) {
      acc = f4_fma(e.x, win[O], acc);
      acc = f4_fma(e.y, win[O + 1], acc);
      acc = f4_fma(e.z, win[O + 2], acc);
    } else {
      apply_window<O + 1, OMAX>(acc, e, win, o);
    }
  }
}

// One warp: voxel block at (xi0, yi0), heights [h, h + 4) of this lane.
// tw (BPB_CHUNK x BX*BY entries) and tb (BPB_CHUNK entries) are this warp's
// shared tables.  All 32 lanes must call it together.
template <int BX, int BY>
__device__ __forceinline__ void bp_block_warp(const float* __restrict__ y, float* __restrict__ x,
                                              const float* __restrict__ angles, const Geom& g,
                                              int xi0, int yi0, int h, int accumulate,
                                              float4 (*tw)[BX * BY], int2* tb) {
  using V = float4;
  using BW = BlockWindow<BX, BY>;
  constexpr int NV = BX * BY;
  constexpr int OMAX = BW::OMAX;
  constexpr int WMAX = BW::WMAX;
  const int lane = threadIdx.x & 31;
  const bool hv = h < g.H;

  V acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = vzero<V>();

  const size_t yrow_stride = (size_t)g.PX * g.Hy;

  for (int a0 = 0; a0 < g.n_ang; a0 += BPB_CHUNK) {
    const int a = a0 + lane;
    if (a < g.n_ang) {
      const AngleConst k = angle_const(angles[a], g.trig);
      int rmin = 0x7fffffff, rmax = -0x7fffffff;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float relx = (float)(xi0 + v % BX) - g.xcent;
        const float rely = (float)(yi0 + v / BX) - g.ycent;
        const BinWeights bw = voxel_weights(relx, rely, k, g.pcent, g.trig);
        rmin = min(rmin, bw.r);
        rmax = max(rmax, bw.r);
        tw[lane][v] = make_float4(bw.w0, bw.w1, bw.w2, __int_as_float(bw.r));
      }
      // window [rmin - 1, rmin - 1 + W); a voxel's offset in it is r - rmin
      tb[lane] = make_int2(rmin, min(rmax - rmin + 3, WMAX));
    }
    __syncwarp();
    const int na = min(BPB_CHUNK, g.n_ang - a0);
    const float* yang = y + (size_t)a0 * yrow_stride + h;
    for (int j = 0; j < na; ++j) {
      const int2 bwin = tb[j];
      V win[WMAX];
#pragma unroll
      for (int jj = 0; jj < WMAX; ++jj) {
        const int bin = bwin.x - 1 + jj;
        win[jj] = ld_or_zero<V>(yang + (ptrdiff_t)bin * g.Hy,
                                hv && jj < bwin.y && (unsigned)bin < (unsigned)g.PX);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float4 e = tw[j][v];
        // offsets outside [0, OMAX] cannot occur (see BlockWindow) and would
        // match no case
        apply_window<0, OMAX>(acc[v], e, win, __float_as_int(e.w) - bwin.x);
      }
      yang += yrow_stride;
    }
    __syncwarp();
  }

  if (hv) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int xi = xi0 + v % BX;
      const int yi = yi0 + v / BX;
      if (xi < g.SX && yi < g.SY) {
        V* px = reinterpret_cast<V*>(x + ((size_t)yi * g.SX + xi) * g.Hx + h);
        store_out(px, acc[v], accumulate);
      }
    }
  }
}

}  // namespace detail
}  // namespace vp
