// Forward projection A, detector-driven gather.
//
// Replaces the reference kernels sp_forward_z0 (sp_forward_z0.cuh:107-185)
// and sp_forward_z2 (sp_forward_z2.cuh:102-174).  Those march each ray
// through a border-mode texture (ray clipped to an extended box,
// projection_common.cuh:194-272; minor-axis walk, sp_forward_z0.cuh:8-103) and
// re-evaluate two CDFs per visited voxel for every height.  Here a ray
// (angle, bin) gathers exactly the voxels whose three-bin footprint reaches
// it, with the same closed-form weights the adjoint uses, so A and A^T are
// the same matrix up to float summation order:
//   weight of bin p from voxel v = w_{p - round(xp_v) + 1}(v)   (bin_weights).
//
// Voxel enumeration: along the axis whose unit step moves xp by less
// ("major"), every index is visited; along the other ("minor", |shift| >=
// sqrt(1/2)) only the indices whose xp lies within b + 1/2 (+ a small margin)
// of the bins being gathered.  Voxels the margin admits needlessly get zero
// weight from the closed form, so the margin only costs time.
#include <cuda_runtime.h>

#include "vp_common.cuh"
#include "vp_fp_z0.cuh"
#include "vp_launch.h"

namespace vp {

namespace {

using namespace detail;

// ---------------------------------------------------------------------------
// z_order 0: x (SY, SX, H), y (n_ang, PX, H); heights contiguous.
// A warp owns angle a, KW consecutive bins and 32*R heights (lane <->
// heights).  The voxels gathered are warp-uniform, so the warp enumerates
// them cooperatively: lane j takes major line i0+j, computes its candidate
// voxels and their bin weights into a per-warp shared list (offsets from a
// warp prefix sum), then all lanes stream the list with broadcast reads,
// FP0_UNROLL candidates at a time so their loads overlap, and accumulate
// the KW bins in registers.  A candidate's three bins sit at run-relative
// offsets q-2, q-1, q (q = round(xp) - p0 + 1), dispatched with a
// warp-uniform switch.
//
// Cache locality: every angle touches the whole volume, so a launch is
// restricted to one slab of rows [y_lo, y_hi) of the volume (all launches add
// into y), and heights are the slowest grid axis.  Concurrently running
// blocks then share one slab x one 128-height chunk, a few tens of MB that
// stay in L2 across all angles instead of being re-read from HBM per angle.
// With AGROUP the four warps of a block take four consecutive angles of the
// same bins: their voxel strips largely coincide, so one warp's loads are L1
// hits for the others.
// ---------------------------------------------------------------------------
template <int R, int KW, bool AGROUP>
__global__ void __launch_bounds__(32 * FP0_WARPS)
    fp_z0_kernel(const float* __restrict__ x, float* __restrict__ y,
                 const float* __restrict__ angles, Geom g, int a_base, int y_lo, int y_hi,
                 int accumulate) {
  __shared__ float4 cand[FP0_WARPS][32 * Fp0Cap<KW>::value];
  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int p0 = (AGROUP ? blockIdx.x : blockIdx.x * FP0_WARPS + w) * KW;
  const int a = a_base + (AGROUP ? blockIdx.y * FP0_WARPS + w : blockIdx.y);
  const int h = (blockIdx.z * 32 + lane) * R;
  fp_z0_warp<R, KW>(x, y, angles, g, p0, a, h, y_lo, y_hi, accumulate, cand[w]);
}

// ---------------------------------------------------------------------------
// z_order 2: x (H, SY, SX), y (H, n_ang, PX); SX / PX contiguous.
// A thread owns one bin p (lane <-> p, so the output row is coalesced) of one
// angle and FP2_RH heights, walks the major axis, and gathers the candidate
// voxels of its bin; each weight is reused across the thread's heights.
// ---------------------------------------------------------------------------
constexpr int FP2_RH = 8;
constexpr int FP2_WARPS = 4;

__global__ void __launch_bounds__(32 * FP2_WARPS)
    fp_z2_kernel(const float* __restrict__ x, float* __restrict__ y,
                 const float* __restrict__ angles, Geom g, int a_base) {
  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int p = blockIdx.x * 32 + lane;
  const int a = a_base + blockIdx.y * FP2_WARPS + w;
  const int h0 = blockIdx.z * FP2_RH;
  if (a >= g.n_ang) return;  // warp-uniform
  const bool pv = p < g.PX;

  const AngleConst k = angle_const(__ldg(angles + a), g.trig);
  const bool minor_x = fabsf(k.c) >= fabsf(k.s);
  const int n_major = minor_x ? g.SY : g.SX;
  const int n_minor = minor_x ? g.SX : g.SY;
  const float cent_major = minor_x ? g.ycent : g.xcent;
  const float cent_minor = minor_x ? g.xcent : g.ycent;
  const float sh_major = minor_x ? k.s : k.c;
  const float inv_sh_minor = 1.0f / (minor_x ? k.c : k.s);
  const float t_lo = (float)p - 0.5f - k.b - kWindowMargin;
  const float t_hi = (float)p + 0.5f + k.b + kWindowMargin;
  const size_t xh_stride = (size_t)g.SY * g.SX;

  float acc[FP2_RH];
#pragma unroll
  for (int i = 0; i < FP2_RH; ++i) acc[i] = 0.0f;

  if (pv) {
    for (int i = 0; i < n_major; ++i) {
      const MinorRange mr = minor_range(i, cent_major, sh_major, cent_minor, inv_sh_minor,
                                        0, n_minor - 1, g.pcent, t_lo, t_hi);
      for (int m = mr.lo; m <= mr.hi; ++m) {
        const int xi = minor_x ? m : i;
        const int yi = minor_x ? i : m;
        const BinWeights bw =
            voxel_weights((float)xi - g.xcent, (float)yi - g.ycent, k, g.pcent, g.trig);
        const int q = p - bw.r + 1;
        const float wt = (q == 0) ? bw.w0 : (q == 1) ? bw.w1 : (q == 2) ? bw.w2 : 0.0f;
        if (wt != 0.0f) {
          const float* px = x + (size_t)yi * g.SX + xi;
#pragma unroll
          for (int r = 0; r < FP2_RH; ++r) {
            const int h = h0 + r;
            if (h < g.H) acc[r] = fmaf(wt, __ldg(px + (size_t)h * xh_stride), acc[r]);
          }
        }
      }
    }
    const size_t yh_stride = (size_t)g.n_ang * g.PX;
#pragma unroll
    for (int r = 0; r < FP2_RH; ++r) {
      const int h = h0 + r;
      if (h < g.H) store_out(y + (size_t)h * yh_stride + (size_t)a * g.PX + p, acc[r], g.accumulate);
    }
  }
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }
constexpr int kMaxGridYZ = 65535;

}  // namespace

// Rows per slab: about 32 MB of one 128-height chunk of the volume.
int fp0_slab_rows(const Geom& g) {
  const long long bytes_per_row = (long long)g.SX * 128 * 4;
  long long rows = (32ll << 20) / (bytes_per_row > 0 ? bytes_per_row : 1);
  if (rows < 8) rows = 8;
  return (int)(rows < g.SY ? rows : g.SY);
}

int launches_forward_z0(const Geom& g) {
  const int rows = fp0_slab_rows(g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const long long per = (v == 3 || v == 4) ? (long long)kMaxGridYZ * FP0_WARPS : kMaxGridYZ;
  return (int)(ceil_div(g.SY, rows) * ceil_div(g.n_ang, per));
}

int launches_forward_z2(const Geom& g) {
  return (int)ceil_div(g.n_ang, (long long)kMaxGridYZ * FP2_WARPS);
}

template <int R, int KW, bool AGROUP>
cudaError_t launch_fp_z0(const float* x, float* y, const float* angles, const Geom& g,
                         cudaStream_t stream) {
  const int rows = fp0_slab_rows(g);
  dim3 block(32, FP0_WARPS);
  bool first = true;
  const long long angles_per_launch = AGROUP ? (long long)kMaxGridYZ * FP0_WARPS : kMaxGridYZ;
  for (int y_lo = 0; y_lo < g.SY; y_lo += rows) {
    const int y_hi = y_lo + rows < g.SY ? y_lo + rows : g.SY;
    // the first slab applies the caller's mode; later slabs add to it
    const int accumulate = first ? g.accumulate : 1;
    first = false;
    for (long long a_base = 0; a_base < g.n_ang; a_base += angles_per_launch) {
      const long long na = g.n_ang - a_base < angles_per_launch ? g.n_ang - a_base
                                                                 : angles_per_launch;
      const unsigned gx = AGROUP ? ceil_div(g.PX, KW) : ceil_div(g.PX, KW * FP0_WARPS);
      const unsigned gy = AGROUP ? ceil_div(na, FP0_WARPS) : (unsigned)na;
      dim3 grid(gx, gy, ceil_div(g.H, 32 * R));
      fp_z0_kernel<R, KW, AGROUP><<<grid, block, 0, stream>>>(x, y, angles, g, (int)a_base, y_lo,
                                                              y_hi, accumulate);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <int R>
cudaError_t launch_fp_z0_variant(const float* x, float* y, const float* angles, const Geom& g,
                                 cudaStream_t stream, int variant) {
  switch (variant) {
    case 2: return launch_fp_z0<R, 8, false>(x, y, angles, g, stream);
    case 3: return launch_fp_z0<R, 4, true>(x, y, angles, g, stream);
    case 4: return launch_fp_z0<R, 8, true>(x, y, angles, g, stream);
    default: return launch_fp_z0<R, 4, false>(x, y, angles, g, stream);
  }
}

// Variants: 1 = 4 bins per warp, warps of a block on neighbouring bins
// (default, fastest at 512^3); 2 = 8 bins, neighbouring bins; 3 = 4 bins,
// warps of a block on neighbouring angles; 4 = 8 bins, neighbouring angles.
cudaError_t launch_forward_z0(const float* x, float* y, const float* angles, const Geom& g,
                              cudaStream_t stream) {
  const bool vec4 = (g.Hx % 4 == 0) && (g.Hy % 4 == 0) &&
                    ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
  const int variant = kernel_variant(OP_FORWARD_Z0);
  if (vec4) return launch_fp_z0_variant<4>(x, y, angles, g, stream, variant);
  return launch_fp_z0_variant<1>(x, y, angles, g, stream, variant);
}

cudaError_t launch_forward_z2(const float* x, float* y, const float* angles, const Geom& g,
                              cudaStream_t stream) {
  dim3 block(32, FP2_WARPS);
  const long long per_launch = (long long)kMaxGridYZ * FP2_WARPS;
  for (long long a_base = 0; a_base < g.n_ang; a_base += per_launch) {
    const long long na = g.n_ang - a_base < per_launch ? g.n_ang - a_base : per_launch;
    dim3 grid(ceil_div(g.PX, 32), ceil_div(na, FP2_WARPS), ceil_div(g.H, FP2_RH));
    fp_z2_kernel<<<grid, block, 0, stream>>>(x, y, angles, g, (int)a_base);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace vp
