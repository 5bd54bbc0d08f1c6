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
#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <type_traits>

#include "vp_common.cuh"
#include "vp_fp_staged.cuh"
#include "vp_fp_z0.cuh"
#include "vp_launch.h"

namespace vp {

namespace {

using namespace detail;

// z_order 0 kernel: one fp_z0_warp per warp (the design is described in
// vp_fp_z0.cuh).  Blocks of FP0_WARPS warps take neighbouring bin runs of one
// angle, or with AGROUP one bin run of neighbouring angles; blockIdx.z is the
// height chunk of 32 * R heights.
// The 8-height, 4-bin form is held to 7 resident blocks per SM (72
// registers), its fastest occupancy with 2 candidates in flight, and to 6
// (80 registers, no spills) with 3 in flight.
// PDL: the launch follows this call's previous slab launch programmatically
// (launch_ex), so its warps wait for that launch before they add into y.
// The first launch of a call keeps the form without the wait.
// With SPLIT a block takes 2 bin runs instead of 4, each by 2 warps that
// gather half of the slab's major lines each: twice the blocks, each half as
// long, so the last wave of a launch leaves less of the GPU idle.  The first
// half writes (in the caller's mode); after a block barrier the second adds.
template <int R, int KW, bool AGROUP, int UN, bool SPLIT = false, bool FULL = false,
          bool PDL = false>
__global__ void __launch_bounds__(32 * FP0_WARPS,
                                  SPLIT ? (R == 8 ? 7 : 8)
                                        : (R == 8 && KW == 4 ? (UN == 3 ? 6 : 7) : 0))
    fp_z0_kernel(const float* __restrict__ x, float* __restrict__ y,
                 const float* __restrict__ angles, Geom g, int a_base, Slab slab,
                 int accumulate) {
  __shared__ float4 cand[FP0_WARPS][Fp0Cap<KW>::list];
  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int h = blockIdx.z * 32 * R + lane * (R == 8 ? 4 : R);
  if constexpr (SPLIT) {
    static_assert(!AGROUP && FP0_WARPS == 4, "two bin runs x two halves");
    const int p0 = (blockIdx.x * 2 + (w & 1)) * KW;
    const int a = a_base + blockIdx.y;
    const int ym = slab.y_lo + (slab.y_hi - slab.y_lo) / 2;
    const int xm = slab.x_lo + (slab.x_hi - slab.x_lo) / 2;
    const bool second = w >= 2;
    const Slab hs = second ? Slab{ym, slab.y_hi, xm, slab.x_hi, slab.yy_lo, slab.yy_hi}
                           : Slab{slab.y_lo, ym, slab.x_lo, xm, slab.yy_lo, slab.yy_hi};
    fp_z0_warp<R, KW, UN>(x, y, angles, g, p0, a, h, hs, second ? 1 : accumulate, cand[w],
                          HalfBarrier{second});
    if (!second) __syncthreads();  // the second half adds after this one wrote
  } else {
    // a programmatic launch of the next slab may start as this one's last
    // blocks run
    pdl_trigger();
    const int p0 = (AGROUP ? blockIdx.x : blockIdx.x * FP0_WARPS + w) * KW;
    const int a = a_base + (AGROUP ? blockIdx.y * FP0_WARPS + w : blockIdx.y);
    using Wait = std::conditional_t<PDL, PdlWait, NoWait>;
    fp_z0_warp<R, KW, UN, Wait, FULL>(x, y, angles, g, p0, a, h, slab, accumulate, cand[w]);
  }
}

// The staged forward (vp_fp_staged.cuh): blocks of 4 compute warps on
// neighbouring angles (blockIdx.y = angle group) and a copy warp; blockIdx.x
// is the block's place on the group's aligned detector axis, offset by E
// blocks; blockIdx.z the 256-height chunk.  NBOX voxels per staged line,
// STAGES lines in flight; as many blocks per SM as shared memory holds (at
// most 4).
constexpr int fps_blocks_per_sm(size_t smem) {
  return (int)((227u * 1024u) / (smem + 1024u)) < 4 ? (int)((227u * 1024u) / (smem + 1024u)) : 4;
}

template <bool FULL, int NBOX, int STAGES>
__global__ void __launch_bounds__(FPS_THREADS,
                                  fps_blocks_per_sm(sizeof(FpsSmem<NBOX, STAGES>)))
    fp_z0_staged_kernel(const float* __restrict__ x, float* __restrict__ y,
                        const float* __restrict__ angles, Geom g, int a_base, Slab slab,
                        int accumulate, int E, unsigned long long* timeouts,
                        unsigned copy_polls, const __grid_constant__ CUtensorMap map_rows,
                        const __grid_constant__ CUtensorMap map_cols) {
  extern __shared__ __align__(1024) unsigned char fps_raw[];
  auto& sm = *reinterpret_cast<FpsSmem<NBOX, STAGES>*>(fps_raw);
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int a0 = a_base + (int)blockIdx.y * FPS_WARPS;
  const int h0 = (int)blockIdx.z * 256;
  const int bx = (int)blockIdx.x - E;
  const FpsGroup G = fps_group(angles, g, slab, a0);  // alike in every thread
  if (!G.aligned) {  // block-uniform: plain runs of 4 bins, as variant 10
    if (w >= FPS_WARPS || !G.valid[w] || bx < 0 || 4 * bx >= g.PX) return;
    fp_z0_warp<8, 4, 2, NoWait, FULL>(x, y, angles, g, 4 * bx, a0 + w, h0 + 4 * lane, slab,
                                      accumulate, sm.cand[w]);
    return;
  }
  fps_aligned_block<FULL, NBOX, STAGES>(x, y, angles, g, slab, accumulate, a0, h0, bx, -E,
                                        (int)gridDim.x - 1 - E, G, sm, &map_rows, &map_cols,
                                        timeouts, copy_polls);
}

// The aligned partition with plain loads (variant 19): 4 warps per block, no
// copy warp, 7 blocks per SM as variant 10.
template <bool FULL>
__global__ void __launch_bounds__(32 * FPS_WARPS, 7)
    fp_z0_aligned_kernel(const float* __restrict__ x, float* __restrict__ y,
                         const float* __restrict__ angles, Geom g, int a_base, Slab slab,
                         int accumulate, int E) {
  __shared__ float4 cand[FPS_WARPS][Fp0Cap<4>::list];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int a0 = a_base + (int)blockIdx.y * FPS_WARPS;
  const int h0 = (int)blockIdx.z * 256;
  const int bx = (int)blockIdx.x - E;
  const FpsGroup G = fps_group(angles, g, slab, a0);
  if (!G.aligned) {
    if (!G.valid[w] || bx < 0 || 4 * bx >= g.PX) return;
    fp_z0_warp<8, 4, 2, NoWait, FULL>(x, y, angles, g, 4 * bx, a0 + w, h0 + 4 * lane, slab,
                                      accumulate, cand[w]);
    return;
  }
  fps_plain_block<FULL>(x, y, angles, g, slab, accumulate, a0, h0, bx, -E,
                        (int)gridDim.x - 1 - E, G, cand[w]);
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

// Launch configuration of a forward variant for one problem.
struct Fp0Config {
  int R;          // heights per lane: 1, 4, or 8 (two float4)
  int KW;         // bins per warp
  bool agroup;    // warps of a block on neighbouring angles
  int un;         // candidates loaded together
  int slab_mb;    // volume bytes of one height chunk per slab launch
  bool cls;       // class slabs (rows for one angle class, columns for the other)
  bool split;     // two warps per bin run, each on half of the major lines
  int staged;     // aligned neighbouring-angle forms (vp_fp_staged.cuh), 8 heights per
                  // lane only: 1 = staged by tensor copies, 2 = plain loads; 0 = none
};

// Variants: 1 = 4 bins per warp, 4 heights per lane, warps of a block on
// neighbouring bins; 2 = 8 bins; 3 = 4 bins, warps of a block on
// neighbouring angles; 4 = 8 bins, neighbouring angles; 5 = 4 bins, 8
// heights per lane, 2 candidates in flight; 6 = as 5 with 4 in flight;
// 7 = as 5 with 64 MB slabs; 8 = 8 bins, 8 heights per lane; 9 / 10 / 11 =
// as 5 with class slabs of 32 / 64 / 128 MB; 12 = as 1
// with class slabs of 32 MB; 13 = as 10 with two warps per bin run, each on
// half of the slab's major lines (SPLIT); 14 / 15 = as 10 / 11 with 3
// candidates in flight at 6 blocks per SM; 16 = as 10 with the warps of a
// block on neighbouring angles; 17 = as 10, four aligned neighbouring angles
// per block, the volume staged through shared memory by tensor copies
// (vp_fp_staged.cuh); 19 = the aligned angle groups with plain loads; 21 /
// 22 / 23 = as 16 with 128 / 32 / 256 MB slabs.  The default (0) is 16 with
// 8 heights per lane and 10's layout (neighbouring bins) in the 4-height
// form.  Measured A per call with programmatic launches between the slab
// launches, variants 16 / 21 / 22 / 23: 512^3 and 192 angles 6.66 / 6.73 /
// 7.05 / 7.12 ms; 1024 angles 32.98 / 33.89 / 35.06 ms; 256^3 and 360 angles
// 1.534 / 1.585 / 1.551 ms; 384^3 and 641 angles 10.54 / 10.50 / 11.01 ms.
// (Without them 21 led: 6.94 against 7.02 ms at 512^3, the extra slab
// launches' tails costing more than the volume's better L2 residency.)
// Heights not in float4 run the scalar form of
// the same bin layout; 8-height variants on problems of at most 128 heights
// run the 4-height form.

// Whether the default's 4-height form takes two warps per bin run (SPLIT),
// for grids of less than two waves of blocks: when twice as many blocks of
// half the work take fewer half-waves than the blocks take waves, or when
// the blocks fill less than three quarters of one wave (smaller blocks then
// balance the SMs better).  Measured A per call (192 angles, default /
// split): 128^3 0.212 / 0.188 ms (1.26 waves of blocks); 96^3 0.114 /
// 0.114-0.117 ms (0.95 waves); 64^3 0.073 / 0.067 ms (0.63 waves).
// Without a device to ask, no.
bool fp0_split_pays(const Geom& g) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0) {
    cudaGetLastError();
    return false;
  }
  const double resident = 8.0 * sms;  // 4-height form: 8 blocks of 4 warps per SM
  const double blocks = (double)ceil_div(g.PX, 4 * FP0_WARPS) *
                        (g.n_ang < kMaxGridYZ ? g.n_ang : kMaxGridYZ) * ceil_div(g.H, 32 * 4);
  const double w = blocks / resident;
  if (w <= 0.0 || w >= 2.0) return false;
  return std::ceil(2.0 * w) < 2.0 * std::ceil(w) || w <= 0.75;
}

Fp0Config fp0_config(const Geom& g, bool vec4, int variant) {
  Fp0Config c{vec4 ? 4 : 1, 4, false, FP0_UNROLL, 32, false, false, 0};
  const bool dflt = variant == 0;
  if (dflt) variant = 16;  // the default
  switch (variant) {
    case 2: c.KW = 8; break;
    case 3: c.agroup = true; break;
    case 4: c.KW = 8; c.agroup = true; break;
    case 5: c.R = 8; c.un = 2; break;
    case 6: c.R = 8; break;
    case 7: c.R = 8; c.un = 2; c.slab_mb = 64; break;
    case 8: c.R = 8; c.KW = 8; c.un = 2; break;
    case 9: c.R = 8; c.un = 2; c.cls = true; break;
    case 10: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 64; break;
    case 11: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 128; break;
    case 12: c.cls = true; break;
    case 13: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 64; c.split = true; break;
    case 14: c.R = 8; c.un = 3; c.cls = true; c.slab_mb = 64; break;
    case 15: c.R = 8; c.un = 3; c.cls = true; c.slab_mb = 128; break;
    case 16: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 64; c.agroup = true; break;
    case 17: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 64; c.staged = 1; break;
    case 19: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 64; c.staged = 2; break;
    case 21: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 128; c.agroup = true; break;
    case 22: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 32; c.agroup = true; break;
    case 23: c.R = 8; c.un = 2; c.cls = true; c.slab_mb = 256; c.agroup = true; break;
    default: break;
  }
  if (c.R == 8 && (!vec4 || g.H <= 128)) {
    c.R = vec4 ? 4 : 1;
    c.un = FP0_UNROLL;
    c.staged = 0;
    // the default's 4-height form keeps neighbouring bins per block: angle
    // groups measured slower there (128^3, 192 angles: 0.223 against
    // 0.2095 ms); with few blocks it splits each bin run over two warps
    if (dflt) {
      c.agroup = false;
      c.split = vec4 && fp0_split_pays(g);
    }
  }
  return c;
}

// Slab launches of a call.  A row slab holds about slab_mb of one height
// chunk (at least 128 heights) of the volume, in whole rows (at least 8); a
// class slab's rows and columns together hold about as much, rows and
// columns split evenly over the slabs.
long long fp0_chunk_bytes(const Geom& g, const Fp0Config& c) {
  const long long chunk_h = 32 * c.R > 128 ? 32 * c.R : 128;
  return (long long)g.SY * g.SX * chunk_h * 4;
}

int fp0_slab_rows(const Geom& g, const Fp0Config& c) {
  const long long bytes_per_row = fp0_chunk_bytes(g, c) / (g.SY > 0 ? g.SY : 1);
  long long rows = ((long long)c.slab_mb << 20) / (bytes_per_row > 0 ? bytes_per_row : 1);
  if (rows < 8) rows = 8;
  return (int)(rows < g.SY ? rows : g.SY);
}

int fp0_slabs(const Geom& g, const Fp0Config& c) {
  if (!c.cls) return (int)ceil_div(g.SY, fp0_slab_rows(g, c));
  const long long budget = (long long)c.slab_mb << 20;
  long long n = (2 * fp0_chunk_bytes(g, c) + budget - 1) / budget;
  const long long nmax = ((g.SX < g.SY ? g.SX : g.SY) + 7) / 8;  // >= 8 lines per slab
  if (n > nmax) n = nmax;
  return (int)(n < 1 ? 1 : n);
}

// Rows (and, for class slabs, columns) per slab.
void fp0_slab_widths(const Geom& g, const Fp0Config& c, int n, int* wy, int* wx) {
  if (!c.cls) {
    *wy = fp0_slab_rows(g, c);
    *wx = g.SX;
  } else {
    *wy = (g.SY + n - 1) / n;
    *wx = (g.SX + n - 1) / n;
  }
}

Slab fp0_slab(const Geom& g, const Fp0Config& c, int k, int n) {
  int wy = 0, wx = 0;
  fp0_slab_widths(g, c, n, &wy, &wx);
  return slab_of(k, c.cls, wy, wx, g.SY, g.SX);
}

bool fp0_vec4(const float* x, const float* y, const Geom& g) {
  return (g.Hx % 4 == 0) && (g.Hy % 4 == 0) &&
         ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
}

int launches_forward_z0(const float* x, const float* y, const Geom& g);

int launches_forward_z2(const Geom& g) {
  return (int)ceil_div(g.n_ang, (long long)kMaxGridYZ * FP2_WARPS);
}

// One slab launch: slab, the caller's mode for it, and the angles [a_lo, a_hi)
// (the kernels index angles and y absolutely; g.n_ang is set to a_hi for
// their bound check).
struct SlabLaunch {
  const float* x;
  float* y;
  const float* angles;
  Geom g;
  Slab slab;
  int accumulate;
  int a_lo, a_hi;
  // the launch directly follows this call's previous slab launch on the
  // stream: it may start while that one runs (launch_ex)
  bool programmatic = false;
};

template <int R, int KW, bool AGROUP, int UN, bool SPLIT = false, bool FULL = false>
cudaError_t launch_slab(const SlabLaunch& L, cudaStream_t stream, int* launches) {
  dim3 block(32, FP0_WARPS);
  const long long per_launch = AGROUP ? (long long)kMaxGridYZ * FP0_WARPS : kMaxGridYZ;
  Geom g = L.g;
  g.n_ang = L.a_hi;
  for (long long a_base = L.a_lo; a_base < L.a_hi; a_base += per_launch) {
    const long long na = L.a_hi - a_base < per_launch ? L.a_hi - a_base : per_launch;
    const unsigned gx = AGROUP  ? ceil_div(g.PX, KW)
                        : SPLIT ? ceil_div(g.PX, KW * 2)
                                : ceil_div(g.PX, KW * FP0_WARPS);
    const unsigned gy = AGROUP ? ceil_div(na, FP0_WARPS) : (unsigned)na;
    dim3 grid(gx, gy, ceil_div(g.H, 32 * R));
    // Programmatic launches for the default 8-height form only: the wait
    // leaves its code as it was, where it costs the 4-height form 8 registers
    // and some of the opt-in forms spills.
    constexpr bool kPdlForm = R == 8 && KW == 4 && AGROUP && UN == 2 && !SPLIT;
    cudaError_t e;
    if constexpr (kPdlForm) {
      if (L.programmatic || a_base > L.a_lo)
        e = launch_ex(fp_z0_kernel<R, KW, AGROUP, UN, SPLIT, FULL, true>, grid, block, 0, stream,
                      true, L.x, L.y, L.angles, g, (int)a_base, L.slab, L.accumulate);
      else
        e = launch_ex(fp_z0_kernel<R, KW, AGROUP, UN, SPLIT, FULL, false>, grid, block, 0,
                      stream, false, L.x, L.y, L.angles, g, (int)a_base, L.slab, L.accumulate);
    } else {
      e = launch_ex(fp_z0_kernel<R, KW, AGROUP, UN, SPLIT, FULL, false>, grid, block, 0, stream,
                    false, L.x, L.y, L.angles, g, (int)a_base, L.slab, L.accumulate);
    }
    if (launches) ++*launches;
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <int R>
cudaError_t launch_slab_r(const Fp0Config& c, const SlabLaunch& L, cudaStream_t s, int* n) {
  if (c.KW == 8) {
    if (c.agroup) return launch_slab<R, 8, true, FP0_UNROLL>(L, s, n);
    return launch_slab<R, 8, false, FP0_UNROLL>(L, s, n);
  }
  if (c.agroup) return launch_slab<R, 4, true, FP0_UNROLL>(L, s, n);
  return launch_slab<R, 4, false, FP0_UNROLL>(L, s, n);
}

// The volume as a 3-D tensor (heights, columns, rows) with boxes of one
// staged line window: nbox voxels of a row (rows) or of a column (cols) x 256
// heights.
cudaError_t volume_tensor_maps(const float* x, const Geom& g, int nbox, CUtensorMap* rows,
                               CUtensorMap* cols) {
  const uint64_t dims[3] = {(uint64_t)g.Hx, (uint64_t)g.SX, (uint64_t)g.SY};
  const uint64_t strides[2] = {(uint64_t)g.Hx * sizeof(float),
                               (uint64_t)g.SX * g.Hx * sizeof(float)};
  const uint32_t box_rows[3] = {(uint32_t)FPS_LINE, (uint32_t)nbox, 1};
  const uint32_t box_cols[3] = {(uint32_t)FPS_LINE, 1, (uint32_t)nbox};
  cudaError_t e = tma::encode_3d_f32(rows, x, dims, strides, box_rows);
  if (e == cudaSuccess) e = tma::encode_3d_f32(cols, x, dims, strides, box_cols);
  return e;
}

// Grid of the aligned forms: the detector in blocks of FPS_W lead bins, with
// E blocks more on each side; angle groups; 256-height chunks.
struct AlignedGrid {
  int E;
  unsigned gx;
};
AlignedGrid aligned_grid(const Geom& g) {
  const int E = fps_margin(g.PX);
  return AlignedGrid{E, (unsigned)((float)g.PX / FPS_W) + 1 + 2 * (unsigned)E};
}

template <bool FULL, int NBOX, int STAGES>
cudaError_t launch_slab_staged(const SlabLaunch& L, cudaStream_t stream, int* launches) {
  using Smem = FpsSmem<NBOX, STAGES>;
  // per device, once: room for the kernel's dynamic shared memory
  static std::atomic<bool> configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || !configured[dev].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(reinterpret_cast<const void*>(fp_z0_staged_kernel<FULL, NBOX, STAGES>),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem));
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) configured[dev].store(true, std::memory_order_release);
  }
  CUtensorMap rows, cols;
  e = volume_tensor_maps(L.x, L.g, NBOX, &rows, &cols);
  if (e != cudaSuccess) return e;
  unsigned long long* timeouts = nullptr;
  e = wait_timeout_counter(&timeouts);
  if (e != cudaSuccess) return e;
  const unsigned polls = copy_wait_polls();
  Geom g = L.g;
  g.n_ang = L.a_hi;
  const AlignedGrid ag = aligned_grid(g);
  const long long per_launch = (long long)kMaxGridYZ * FPS_WARPS;
  for (long long a_base = L.a_lo; a_base < L.a_hi; a_base += per_launch) {
    const long long na = L.a_hi - a_base < per_launch ? L.a_hi - a_base : per_launch;
    dim3 grid(ag.gx, ceil_div(na, FPS_WARPS), ceil_div(g.H, 256));
    fp_z0_staged_kernel<FULL, NBOX, STAGES><<<grid, FPS_THREADS, sizeof(Smem), stream>>>(
        L.x, L.y, L.angles, g, (int)a_base, L.slab, L.accumulate, ag.E, timeouts, polls, rows,
        cols);
    if (launches) ++*launches;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <bool FULL>
cudaError_t launch_slab_aligned(const SlabLaunch& L, cudaStream_t stream, int* launches) {
  Geom g = L.g;
  g.n_ang = L.a_hi;
  const AlignedGrid ag = aligned_grid(g);
  const long long per_launch = (long long)kMaxGridYZ * FPS_WARPS;
  for (long long a_base = L.a_lo; a_base < L.a_hi; a_base += per_launch) {
    const long long na = L.a_hi - a_base < per_launch ? L.a_hi - a_base : per_launch;
    dim3 grid(ag.gx, ceil_div(na, FPS_WARPS), ceil_div(g.H, 256));
    fp_z0_aligned_kernel<FULL><<<grid, 32 * FPS_WARPS, 0, stream>>>(
        L.x, L.y, L.angles, g, (int)a_base, L.slab, L.accumulate, ag.E);
    if (launches) ++*launches;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_slab_config(const Fp0Config& c, const SlabLaunch& L, cudaStream_t s, int* n) {
  if (c.R == 8 && c.staged) {
    const bool full = L.g.H % 256 == 0;
    if (c.staged == 2)
      return full ? launch_slab_aligned<true>(L, s, n) : launch_slab_aligned<false>(L, s, n);
    return full ? launch_slab_staged<true, 12, 3>(L, s, n)
                : launch_slab_staged<false, 12, 3>(L, s, n);
  }
  if (c.R == 8) {
    if (c.KW == 8) return launch_slab<8, 8, false, 2>(L, s, n);
    if (c.un == 2 && c.agroup) {
      if (L.g.H % (32 * 8) == 0) return launch_slab<8, 4, true, 2, false, true>(L, s, n);
      return launch_slab<8, 4, true, 2>(L, s, n);
    }
    if (c.un == 2) {
      if (c.split) return launch_slab<8, 4, false, 2, true>(L, s, n);
      // whole chunks of 256 heights: the second float4 at a constant offset
      if (L.g.H % (32 * 8) == 0) return launch_slab<8, 4, false, 2, false, true>(L, s, n);
      return launch_slab<8, 4, false, 2>(L, s, n);
    }
    if (c.un == 3) {
      if (L.g.H % (32 * 8) == 0) return launch_slab<8, 4, false, 3, false, true>(L, s, n);
      return launch_slab<8, 4, false, 3>(L, s, n);
    }
    return launch_slab<8, 4, false, 4>(L, s, n);
  }
  if (c.R == 4 && c.split && c.KW == 4 && !c.agroup)
    return launch_slab<4, 4, false, FP0_UNROLL, true>(L, s, n);
  if (c.R == 4) return launch_slab_r<4>(c, L, s, n);
  return launch_slab_r<1>(c, L, s, n);
}

// Slabs [k0, k1) of the configuration's plan, all angles; the first slab
// applies the caller's mode, later slabs add to it.
cudaError_t launch_fp_z0_config(const float* x, float* y, const float* angles, const Geom& g,
                                const Fp0Config& c, int k0, int k1, cudaStream_t stream,
                                int* launches = nullptr) {
  const int nslabs = fp0_slabs(g, c);
  for (int k = k0; k < k1 && k < nslabs; ++k) {
    const SlabLaunch L{x, y, angles, g, fp0_slab(g, c, k, nslabs), k == 0 ? g.accumulate : 1,
                       0, g.n_ang, k > k0};
    const cudaError_t e = launch_slab_config(c, L, stream, launches);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The heights of a call as (first height, count) parts: one part, or with 8
// heights per lane an 8-height part and a 4-height remainder (r8_heights).
struct HeightParts {
  int n;
  Geom g[2];
  int h0[2];
};

HeightParts fp0_parts(const Geom& g, bool vec4, int variant) {
  HeightParts p{1, {g, g}, {0, 0}};
  if (fp0_config(g, vec4, variant).R == 8) {
    const int H8 = r8_heights(g.H);
    if (H8 < g.H) {
      p.n = 2;
      p.g[0].H = H8;
      p.g[1].H = g.H - H8;
      p.h0[1] = H8;
    }
  }
  return p;
}

cudaError_t launch_forward_z0(const float* x, float* y, const float* angles, const Geom& g,
                              cudaStream_t stream) {
  const bool vec4 = fp0_vec4(x, y, g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const HeightParts hp = fp0_parts(g, vec4, v);
  for (int i = 0; i < hp.n; ++i) {
    const Fp0Config c = fp0_config(hp.g[i], vec4, v);
    const cudaError_t e = launch_fp_z0_config(x + hp.h0[i], y + hp.h0[i], angles, hp.g[i], c, 0,
                                              1 << 30, stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

Fp0Plan forward_z0_plan(const Geom& g, bool vec4, int variant) {
  const Fp0Config c = fp0_config(g, vec4, variant);
  Fp0Plan p;
  p.R = c.R;
  p.KW = c.KW;
  p.un = c.un;
  p.agroup = c.agroup;
  p.staged = c.staged != 0;
  p.cls = c.cls;
  p.split = c.split;
  p.nslabs = fp0_slabs(g, c);
  fp0_slab_widths(g, c, p.nslabs, &p.wy, &p.wx);
  return p;
}

int launches_forward_z0(const float* x, const float* y, const Geom& g) {
  const bool vec4 = fp0_vec4(x, y, g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const HeightParts hp = fp0_parts(g, vec4, v);
  int n = 0;
  for (int i = 0; i < hp.n; ++i) {
    const Fp0Config c = fp0_config(hp.g[i], vec4, v);
    const long long per =
        (c.agroup || c.staged) ? (long long)kMaxGridYZ * FP0_WARPS : kMaxGridYZ;
    n += (int)(fp0_slabs(hp.g[i], c) * ceil_div(hp.g[i].n_ang, per));
  }
  return n;
}

// Streamed form for volumes that arrive in row order, on the main height
// part (launch_forward_z0_stream): while rows arrive, angles whose minor axis
// is x walk the rows that are in (the other class's range is empty); once
// all are in, the other angles walk blocks of columns.  Together these are
// the class slabs of the device path, spread over time.  The 4-height
// remainder of a split heights range runs whole at the end
// (launch_forward_z0_rest).
// Pieces of at most piece_mb MB of one height chunk (the caller's choice,
// and no more than the plan's slabs): pieces are copy and overlap units as
// well as slabs, and smaller ones start the kernels sooner.
int forward_z0_stream_rows(const float* x, const float* y, const Geom& g, int piece_mb) {
  const bool vec4 = fp0_vec4(x, y, g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const Geom gm = fp0_parts(g, vec4, v).g[0];
  Fp0Config c = fp0_config(gm, vec4, v);
  c.cls = false;  // rows of one class alone: the row-slab budget
  c.slab_mb = c.slab_mb < piece_mb ? c.slab_mb : piece_mb;
  return fp0_slab_rows(gm, c);
}

int forward_z0_stream_cols(const float* x, const float* y, const Geom& g, int piece_mb) {
  const bool vec4 = fp0_vec4(x, y, g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const Geom gm = fp0_parts(g, vec4, v).g[0];
  Fp0Config c = fp0_config(gm, vec4, v);
  c.cls = false;
  c.slab_mb = c.slab_mb < piece_mb ? c.slab_mb : piece_mb;
  Geom gt = gm;  // columns of the other class: rows and columns swapped
  gt.SY = gm.SX;
  gt.SX = gm.SY;
  return fp0_slab_rows(gt, c);
}

cudaError_t launch_forward_z0_stream(const float* x, float* y, const float* angles,
                                     const Geom& g, int rows_lo, int rows_hi, int cols_lo,
                                     int cols_hi, int a_lo, int a_hi, int accumulate,
                                     cudaStream_t stream, int* launches) {
  const bool vec4 = fp0_vec4(x, y, g);
  const int v = kernel_variant(OP_FORWARD_Z0);
  const Geom gm = fp0_parts(g, vec4, v).g[0];
  Fp0Config c = fp0_config(gm, vec4, v);
  c.cls = true;
  const SlabLaunch L{x, y, angles, gm, Slab{rows_lo, rows_hi, cols_lo, cols_hi, 0, g.SY},
                     accumulate, a_lo, a_hi};
  return launch_slab_config(c, L, stream, launches);
}

cudaError_t launch_forward_z0_rest(const float* x, float* y, const float* angles,
                                   const Geom& g, cudaStream_t stream, int* launches) {
  const bool vec4 = fp0_vec4(x, y, g);
  const HeightParts hp = fp0_parts(g, vec4, kernel_variant(OP_FORWARD_Z0));
  if (hp.n < 2) return cudaSuccess;
  const Fp0Config c = fp0_config(hp.g[1], vec4, kernel_variant(OP_FORWARD_Z0));
  return launch_fp_z0_config(x + hp.h0[1], y + hp.h0[1], angles, hp.g[1], c, 0, 1 << 30,
                             stream, launches);
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
