// Adjoint A^T (backprojection), voxel-driven, atomic-free.
//
// Replaces the reference kernels sp_backward_z0 (sp_backward_z0.cuh:8-100)
// and sp_backward_z2 (sp_backward_z2.cuh:8-101).  Those kernels run one thread
// per (voxel, height), rebuild a 512-entry angle table in every block (which
// overruns shared memory past 512 angles) and fetch the sinogram through a
// border-mode texture.  Here:
//   * angles are processed in chunks, so any angle count works;
//   * the three bin weights of a (voxel, angle) pair are computed once and
//     applied to a vector of heights held in registers;
//   * the sinogram is read straight from the caller's buffer; bins outside
//     [0, PX) read as zero, which is what the border-mode texture returned;
//   * all angles accumulate in registers and each voxel is updated with a
//     single read-modify-write at the end, so no atomics are needed.
#include <cuda_runtime.h>

#include "vp_common.cuh"
#include "vp_launch.h"

namespace vp {

namespace {

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

template <typename V>
__device__ __forceinline__ V ld_or_zero(const float* p, bool ok) {
  return ok ? __ldg(reinterpret_cast<const V*>(p)) : vzero<V>();
}

// ---------------------------------------------------------------------------
// z_order 0: x (SY, SX, H), y (n_ang, PX, H); the height axis is contiguous.
// A warp owns a run of BP0_RUN voxels along x and 32*R consecutive heights
// (lane <-> heights, R = 4 reads them as float4).  All lanes of a warp share
// the voxel run, so the per-(voxel, angle) weights are warp-uniform: lane j
// computes them for angle a0+j into a per-warp shared table and every lane
// then reads the table with broadcast loads.
// ---------------------------------------------------------------------------
constexpr int BP0_RUN = 4;
constexpr int BP0_WARPS = 4;
constexpr int BP0_CHUNK = 32;

template <int R>
__global__ void __launch_bounds__(32 * BP0_WARPS)
    bp_z0_kernel(const float* __restrict__ y, float* __restrict__ x,
                 const float* __restrict__ angles, Geom g) {
  using V = typename Vec<R>::T;
  __shared__ float4 tab[BP0_WARPS][BP0_CHUNK][BP0_RUN];

  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int h = (blockIdx.x * 32 + lane) * R;
  const int xi0 = blockIdx.y * BP0_RUN;
  const int yi = blockIdx.z * BP0_WARPS + w;
  if (yi >= g.SY) return;  // warp-uniform; the table is per warp
  const bool hv = h < g.H;

  V acc[BP0_RUN];
#pragma unroll
  for (int m = 0; m < BP0_RUN; ++m) acc[m] = vzero<V>();

  const float rely = (float)yi - g.ycent;
  const size_t yrow_stride = (size_t)g.PX * g.Hy;

  for (int a0 = 0; a0 < g.n_ang; a0 += BP0_CHUNK) {
    const int a = a0 + lane;
    if (a < g.n_ang) {
      const AngleConst k = angle_const(angles[a], g.trig);
#pragma unroll
      for (int m = 0; m < BP0_RUN; ++m) {
        const float relx = (float)(xi0 + m) - g.xcent;
        const BinWeights bw = voxel_weights(relx, rely, k, g.pcent, g.trig);
        tab[w][lane][m] = make_float4(bw.w0, bw.w1, bw.w2, __int_as_float(bw.r));
      }
    }
    __syncwarp();
    const int na = min(BP0_CHUNK, g.n_ang - a0);
    const float* yang = y + (size_t)a0 * yrow_stride + h;
    for (int j = 0; j < na; ++j) {
#pragma unroll
      for (int m = 0; m < BP0_RUN; ++m) {
        const float4 e = tab[w][j][m];
        const int r = __float_as_int(e.w);
        const float* yb = yang + (ptrdiff_t)r * g.Hy;
        const V v0 = ld_or_zero<V>(yb - g.Hy, hv && (unsigned)(r - 1) < (unsigned)g.PX);
        const V v1 = ld_or_zero<V>(yb, hv && (unsigned)r < (unsigned)g.PX);
        const V v2 = ld_or_zero<V>(yb + g.Hy, hv && (unsigned)(r + 1) < (unsigned)g.PX);
        acc[m] = f4_fma(e.x, v0, acc[m]);
        acc[m] = f4_fma(e.y, v1, acc[m]);
        acc[m] = f4_fma(e.z, v2, acc[m]);
      }
      yang += yrow_stride;
    }
    __syncwarp();
  }

  if (hv) {
#pragma unroll
    for (int m = 0; m < BP0_RUN; ++m) {
      const int xi = xi0 + m;
      if (xi < g.SX) {
        V* px = reinterpret_cast<V*>(x + ((size_t)yi * g.SX + xi) * g.Hx + h);
        *px = f4_add(*px, acc[m]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// z_order 2: x (H, SY, SX), y (H, n_ang, PX); x / PX are contiguous.
// A thread owns one voxel column (lane <-> xi, so loads and stores coalesce
// along x) and BP2_RH heights.  Weights are per thread (lanes hold different
// voxels) and are reused across the thread's heights.  Angle constants for a
// chunk of BP2_CHUNK angles are built once per block in shared memory.
// ---------------------------------------------------------------------------
constexpr int BP2_RH = 8;
constexpr int BP2_WARPS = 4;
constexpr int BP2_CHUNK = 32 * BP2_WARPS;

__global__ void __launch_bounds__(32 * BP2_WARPS)
    bp_z2_kernel(const float* __restrict__ y, float* __restrict__ x,
                 const float* __restrict__ angles, Geom g) {
  __shared__ float2 tcs[BP2_CHUNK];
  __shared__ float4 tpw[BP2_CHUNK];

  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int xi = blockIdx.x * 32 + lane;
  const int yi = blockIdx.y * BP2_WARPS + w;
  const int h0 = blockIdx.z * BP2_RH;
  const bool vv = xi < g.SX && yi < g.SY;

  float acc[BP2_RH];
#pragma unroll
  for (int i = 0; i < BP2_RH; ++i) acc[i] = 0.0f;

  const float relx = (float)xi - g.xcent;
  const float rely = (float)yi - g.ycent;
  const size_t yh_stride = (size_t)g.n_ang * g.PX;

  for (int a0 = 0; a0 < g.n_ang; a0 += BP2_CHUNK) {
    __syncthreads();
    const int tid = w * 32 + lane;
    if (a0 + tid < g.n_ang) {
      const AngleConst k = angle_const(angles[a0 + tid], g.trig);
      tcs[tid] = make_float2(k.c, k.s);
      tpw[tid] = make_float4(k.a, k.b, k.coeff, k.cd);
    }
    __syncthreads();
    if (!vv) continue;
    const int na = min(BP2_CHUNK, g.n_ang - a0);
    for (int j = 0; j < na; ++j) {
      const float2 cs = tcs[j];
      const float4 pw = tpw[j];
      AngleConst k;
      k.c = cs.x;
      k.s = cs.y;
      k.a = pw.x;
      k.b = pw.y;
      k.coeff = pw.z;
      k.cd = pw.w;
      const BinWeights bw = voxel_weights(relx, rely, k, g.pcent, g.trig);
      const bool ok0 = (unsigned)(bw.r - 1) < (unsigned)g.PX;
      const bool ok1 = (unsigned)bw.r < (unsigned)g.PX;
      const bool ok2 = (unsigned)(bw.r + 1) < (unsigned)g.PX;
      const float* yb = y + (size_t)(a0 + j) * g.PX + bw.r;
#pragma unroll
      for (int i = 0; i < BP2_RH; ++i) {
        const int h = h0 + i;
        if (h < g.H) {
          const float* p = yb + (size_t)h * yh_stride;
          const float v0 = ok0 ? __ldg(p - 1) : 0.0f;
          const float v1 = ok1 ? __ldg(p) : 0.0f;
          const float v2 = ok2 ? __ldg(p + 1) : 0.0f;
          acc[i] = fmaf(bw.w0, v0, acc[i]);
          acc[i] = fmaf(bw.w1, v1, acc[i]);
          acc[i] = fmaf(bw.w2, v2, acc[i]);
        }
      }
    }
  }

  if (vv) {
#pragma unroll
    for (int i = 0; i < BP2_RH; ++i) {
      const int h = h0 + i;
      if (h < g.H) {
        float* px = x + ((size_t)h * g.SY + yi) * g.SX + xi;
        *px += acc[i];
      }
    }
  }
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

cudaError_t launch_backward_z0(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream) {
  const bool vec4 = (g.Hx % 4 == 0) && (g.Hy % 4 == 0) &&
                    ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
  const int R = vec4 ? 4 : 1;
  dim3 block(32, BP0_WARPS);
  dim3 grid(ceil_div(g.H, 32 * R), ceil_div(g.SX, BP0_RUN), ceil_div(g.SY, BP0_WARPS));
  if (vec4)
    bp_z0_kernel<4><<<grid, block, 0, stream>>>(y, x, angles, g);
  else
    bp_z0_kernel<1><<<grid, block, 0, stream>>>(y, x, angles, g);
  return cudaGetLastError();
}

cudaError_t launch_backward_z2(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream) {
  dim3 block(32, BP2_WARPS);
  dim3 grid(ceil_div(g.SX, 32), ceil_div(g.SY, BP2_WARPS), ceil_div(g.H, BP2_RH));
  bp_z2_kernel<<<grid, block, 0, stream>>>(y, x, angles, g);
  return cudaGetLastError();
}

}  // namespace vp
