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
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <type_traits>

#include "vp_bp_block.cuh"
#include "vp_bp_runs.cuh"
#include "vp_bp_runs_tma.cuh"
#include "vp_common.cuh"
#include "vp_launch.h"

namespace vp {

namespace {

using namespace detail;

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
  const int xi0 = blockIdx.x * BP0_RUN;
  const int yi = blockIdx.y * BP0_WARPS + w;
  const int h = (blockIdx.z * 32 + lane) * R;
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
        store_out(px, acc[m], g.accumulate);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// z_order 0, register-blocked: a warp owns a BX x BY block of voxel columns
// and 128 heights (lane <-> 4 heights, float4).  At one angle the block's
// voxels land on bins [base, base + W) with W <= 3 + floor(dmax + 1), where
// dmax = sqrt((BX-1)^2 + (BY-1)^2) bounds the spread of xp over the block and
// the +1 covers rounding.  That window is loaded once into registers (about
// 7 float4 loads for 16 voxels instead of 48), and each voxel reads its
// three bins from it through a warp-uniform switch on its window offset
// o = round(xp) - base - 1, so every register index stays static.
//
// Per (voxel, angle) the lane-parallel table phase stores (w0, w1, w2, r);
// per angle it stores (rmin, W).
// ---------------------------------------------------------------------------
template <int BX, int BY>
__global__ void __launch_bounds__(32 * BPB_WARPS)
    bp_z0_block_kernel(const float* __restrict__ y, float* __restrict__ x,
                       const float* __restrict__ angles, Geom g, int nbx, int nblocks) {
  __shared__ float4 tw[BPB_WARPS][BPB_CHUNK][BX * BY];
  __shared__ int2 tb[BPB_WARPS][BPB_CHUNK];
  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int bidx = blockIdx.x * BPB_WARPS + w;
  const int h = (blockIdx.y * 32 + lane) * 4;
  if (bidx >= nblocks) return;  // warp-uniform; tables are per warp
  bp_block_warp<BX, BY>(y, x, angles, g, (bidx % nbx) * BX, (bidx / nbx) * BY, h, g.accumulate,
                        tw[w], tb[w]);
}

// ---------------------------------------------------------------------------
// z_order 0, run kernel.  Angles split in two classes: in class X (|c| <=
// |s|) one step along x moves xp by |c| <= sqrt(1/2), in class Y (|c| > |s|)
// one step along y moves it by |s| < sqrt(1/2).  One launch per class; in
// each, a warp owns RUN = 4 voxels along that axis and 128 heights (lane <->
// 4 heights) and visits only the angles of its class.
//
// Along the run xp advances by less than one bin per voxel, so round(xp)
// advances by 0 or 1 per voxel (mirrored when the step is negative: the
// window is then read in decreasing bin order and w0/w2 swap places).  The
// run's bins form a window of W = 3 + (number of advances) <= 6 bins that is
// loaded once, and the pattern of advances (3 bits) selects one of 8
// straight-line code paths with static register indices: one warp-uniform
// branch per run and angle.  Float noise can break monotonicity when xp sits
// on a half-integer and the step is tiny; such (run, angle) pairs take a
// generic path with three loads per voxel.
//
// Angles of a class are compacted per chunk (ballot + prefix count).  Table
// per (run, angle): 12 weights in window order, the 4 bins r, and
// (base bin, direction, pattern).  The second launch adds into x; a warp that
// saw no angle of its class leaves x untouched (in store mode the first launch
// always writes).
// ---------------------------------------------------------------------------
// PDL: the launch follows another run launch of the same call
// programmatically (launch_ex), so its warps wait for that launch before they
// add into x; a call's first launch keeps the form without the wait.
template <int PASS, int R, bool ADD = false, bool FULL = false, bool PDL = false>
__global__ void __launch_bounds__(32 * BPR_WARPS, R == 8 ? 5 : 0)
    bp_z0_runs_kernel(const float* __restrict__ y, float* __restrict__ x,
                      const float* __restrict__ angles, Geom g, int nrun_major, int run_base,
                      int run_end, int row_end, int accumulate,
                      const float* __restrict__ addend = nullptr) {
  __shared__ RunEntry tab[BPR_WARPS][BPR_CHUNK];
  __shared__ int alist[BPR_WARPS][BPR_LIST];
  const int lane = threadIdx.x;
  const int w = threadIdx.y;
  const int run = run_base + blockIdx.x * BPR_WARPS + w;
  // A programmatic launch of the next class may start as this one's last
  // blocks run; each warp waits for the launch before it only to add its
  // sums into x.  Warp 0 of every block has a run inside the range (the grid
  // covers [run_base, run_end) in blocks of 4 runs, and a block's first run,
  // or its band's first row, lies below row_end), so every block waits
  // before it ends.  (Waits
  // on the early returns below cost the 8-height form a register spill and
  // 4% of its time.)
  pdl_trigger();
  if (run >= run_end) return;  // warp-uniform; all shared state is per warp
  int xi0, yi0;
  run_origin<PASS>(run, nrun_major, &xi0, &yi0);
  if (yi0 >= row_end) return;
  using Wait = std::conditional_t<PDL, PdlWait, NoWait>;
  bp_runs_warp<PASS, R, Wait, ADD, FULL>(y, x, angles, g, xi0, yi0,
                                         blockIdx.y * 32 * R + lane * 4, accumulate, tab[w],
                                         alist[w], Wait(), addend);
}

// Bounded-wait timeouts of this library's kernels (0 in correct operation).
__device__ unsigned long long g_wait_timeouts = 0;

// Polls of a copy's completion barrier before a block of the bulk-copy
// adjoint falls back to plain loads (vp_set_wait_limits; tests lower it).
std::atomic<unsigned> g_copy_polls{tma::kTmaMaxPolls};

}  // namespace

void set_copy_wait_polls(unsigned polls, bool use_default) {
  g_copy_polls.store(use_default ? tma::kTmaMaxPolls : polls);
}

unsigned copy_wait_polls() { return g_copy_polls.load(); }

cudaError_t wait_timeout_counter(unsigned long long** out) {
  static std::atomic<unsigned long long*> addr[64] = {};
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  unsigned long long* p = addr[dev].load(std::memory_order_acquire);
  if (p == nullptr) {
    void* sym = nullptr;
    const cudaError_t e2 = cudaGetSymbolAddress(&sym, g_wait_timeouts);
    if (e2 != cudaSuccess) return e2;
    p = static_cast<unsigned long long*>(sym);
    addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return cudaSuccess;
}

namespace {

// The run adjoint with 8 heights per lane and each angle's bin window staged
// once per block by bulk copies (vp_bp_runs_tma.cuh): 4 compute warps on a
// 4 x 4 voxel tile (run_origin) and a copy warp.  Blocks that cannot stage (a
// partial height chunk, runs past the range) run bp_runs_warp instead.
constexpr size_t kTmaBlockSmem = sizeof(TmaBlockSmem);

template <int PASS>
__global__ void __launch_bounds__(TMA_THREADS, 4)
    bp_z0_runs_tma_kernel(const float* __restrict__ y, float* __restrict__ x,
                          const float* __restrict__ angles, Geom g, int nrun_major,
                          int run_base, int run_end, int row_end, int accumulate,
                          unsigned copy_polls, const __grid_constant__ CUtensorMap ymap) {
  extern __shared__ __align__(128) unsigned char tma_smem[];
  TmaBlockSmem& sm = *reinterpret_cast<TmaBlockSmem*>(tma_smem);
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int h0 = blockIdx.y * 32 * 8;
  // block-uniform: can every compute warp's run be staged?
  const int first = run_base + blockIdx.x * TMA_WARPS;
  bool staged = h0 + 32 * 8 <= g.H && first + TMA_WARPS <= run_end;
  if (staged) {
    int xo, yo;
    run_origin<PASS>(first + TMA_WARPS - 1, nrun_major, &xo, &yo);
    staged = yo < row_end;
    run_origin<PASS>(first, nrun_major, &xo, &yo);
    staged = staged && yo < row_end;
  }
  const int run = first + (w < TMA_WARPS ? w : 0);
  int xi0, yi0;
  run_origin<PASS>(run, nrun_major, &xi0, &yi0);
  if (staged) {
    bp_runs_tma_block<PASS>(y, x, angles, g, xi0, yi0, h0, accumulate, sm, &ymap,
                            &g_wait_timeouts, copy_polls);
    return;
  }
  if (w >= TMA_WARPS || run >= run_end || yi0 >= row_end) return;
  RunEntry* tab = reinterpret_cast<RunEntry*>(&sm.ring[0][0]) + w * BPR_CHUNK;
  int* alist = reinterpret_cast<int*>(reinterpret_cast<RunEntry*>(&sm.ring[0][0]) +
                                      TMA_WARPS * BPR_CHUNK) + w * BPR_LIST;
  bp_runs_warp<PASS, 8>(y, x, angles, g, xi0, yi0, h0 + lane * 4, accumulate, tab, alist);
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
        store_out(px, acc[i], g.accumulate);
      }
    }
  }
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

template <int BX, int BY>
cudaError_t launch_bp_z0_block(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream) {
  const int nbx = (g.SX + BX - 1) / BX;
  const int nby = (g.SY + BY - 1) / BY;
  const long long nblocks = (long long)nbx * nby;
  dim3 block(32, BPB_WARPS);
  // heights slowest, so blocks running together share one 128-height chunk
  dim3 grid(ceil_div(nblocks, BPB_WARPS), ceil_div(g.H, 128));
  bp_z0_block_kernel<BX, BY><<<grid, block, 0, stream>>>(y, x, angles, g, nbx, (int)nblocks);
  return cudaGetLastError();
}

// The sinogram as a 3-D tensor (heights, bins, angles) with boxes of 256
// heights x TMA_NBMAX bins x 1 angle, for the staged adjoint.
cudaError_t sinogram_tensor_map(const float* y, const Geom& g, CUtensorMap* map) {
  const uint64_t dims[3] = {(uint64_t)g.Hy, (uint64_t)g.PX, (uint64_t)g.n_ang};
  const uint64_t strides[2] = {(uint64_t)g.Hy * sizeof(float),
                               (uint64_t)g.PX * g.Hy * sizeof(float)};
  const uint32_t box[3] = {(uint32_t)TMA_BIN_FLOATS, (uint32_t)TMA_NBMAX, 1};
  return tma::encode_3d_f32(map, y, dims, strides, box);
}

cudaError_t launch_bp_z0_runs_tma(const float* y, float* x, const float* angles, const Geom& g,
                                  int row_lo, int row_hi, cudaStream_t stream) {
  CUtensorMap ymap;
  cudaError_t e0m = sinogram_tensor_map(y, g, &ymap);
  if (e0m != cudaSuccess) return e0m;
  // per device, once; two threads setting the same attributes at once is
  // harmless, and the flag is atomic
  static std::atomic<bool> configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || !configured[dev].load(std::memory_order_acquire)) {
    // the attribute is per device; setting it twice is harmless
    for (const void* k : {reinterpret_cast<const void*>(bp_z0_runs_tma_kernel<0>),
                          reinterpret_cast<const void*>(bp_z0_runs_tma_kernel<1>)}) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kTmaBlockSmem);
      if (e == cudaSuccess)  // room for four blocks per SM
        e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      if (e != cudaSuccess) return e;
    }
    if (dev >= 0 && dev < 64) configured[dev].store(true, std::memory_order_release);
  }
  dim3 block(TMA_THREADS);
  const unsigned hchunks = ceil_div(g.H, 32 * 8);
  const int nmaj0 = (int)ceil_div(g.SX, RUN);
  // class-0 runs in bands of RUN rows (run_origin): row_lo is a multiple of RUN
  const long long b0 = (long long)row_lo * nmaj0;
  const long long e0 = (long long)ceil_div(row_hi, RUN) * RUN * nmaj0;
  if (e0 > b0) {
    bp_z0_runs_tma_kernel<0><<<dim3(ceil_div(e0 - b0, TMA_WARPS), hchunks), block,
                               kTmaBlockSmem, stream>>>(y, x, angles, g, nmaj0, (int)b0,
                                                        (int)e0, row_hi, g.accumulate,
                                                        g_copy_polls.load(), ymap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const long long b1 = (long long)(row_lo / RUN) * g.SX;
  const long long e1 = (long long)ceil_div(row_hi, RUN) * g.SX;
  if (e1 > b1) {
    bp_z0_runs_tma_kernel<1><<<dim3(ceil_div(e1 - b1, TMA_WARPS), hchunks), block,
                               kTmaBlockSmem, stream>>>(y, x, angles, g, g.SX, (int)b1,
                                                        (int)e1, row_hi, 1,
                                                        g_copy_polls.load(), ymap);
    return cudaGetLastError();
  }
  return cudaSuccess;
}

// Both class launches for the voxel rows [row_lo, row_hi); row_lo is a
// multiple of RUN (class-1 runs span RUN rows).
// With addend, the class-1 launch also adds addend (same layout as x) into the
// rows it writes, after its own sums: x = (x + A^T y) + addend.
// programmatic: the first launch directly follows another run launch of the
// same call (launch_ex); the class-1 launch follows the class-0 one.
// addend_ready: an event the class-1 launch, which reads addend, waits for
// (the class-0 launch runs before the addend is in).
template <int R, bool FULL = false>
cudaError_t launch_bp_z0_runs_h(const float* y, float* x, const float* angles, const Geom& g,
                                int row_lo, int row_hi, cudaStream_t stream,
                                const float* addend = nullptr, bool programmatic = false,
                                cudaEvent_t addend_ready = nullptr) {
  dim3 block(32, BPR_WARPS);
  const unsigned hchunks = ceil_div(g.H, 32 * R);
  const int nmaj0 = (int)ceil_div(g.SX, RUN);
  // class-0 runs in bands of RUN rows (run_origin): row_lo is a multiple of RUN
  const long long b0 = (long long)row_lo * nmaj0;
  const long long e0 = (long long)ceil_div(row_hi, RUN) * RUN * nmaj0;
  const float* no_addend = nullptr;
  if (e0 > b0) {
    const dim3 grid(ceil_div(e0 - b0, BPR_WARPS), hchunks);
    cudaError_t e =
        programmatic
            ? launch_ex(bp_z0_runs_kernel<0, R, false, FULL, true>, grid, block, 0, stream,
                        true, y, x, angles, g, nmaj0, (int)b0, (int)e0, row_hi, g.accumulate,
                        no_addend)
            : launch_ex(bp_z0_runs_kernel<0, R, false, FULL, false>, grid, block, 0, stream,
                        false, y, x, angles, g, nmaj0, (int)b0, (int)e0, row_hi, g.accumulate,
                        no_addend);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    programmatic = true;
  }
  const long long b1 = (long long)(row_lo / RUN) * g.SX;
  const long long e1 = (long long)ceil_div(row_hi, RUN) * g.SX;
  if (e1 > b1) {
    const dim3 grid(ceil_div(e1 - b1, BPR_WARPS), hchunks);
    // the class-1 launch follows the class-0 one whenever there is one (an
    // ordinary launch after a wait for the addend)
    cudaError_t e;
    if (addend && addend_ready) {
      e = cudaStreamWaitEvent(stream, addend_ready, 0);
      if (e != cudaSuccess) return e;
      programmatic = false;
    }
    if (addend)
      e = programmatic ? launch_ex(bp_z0_runs_kernel<1, R, true, FULL, true>, grid, block, 0,
                                   stream, true, y, x, angles, g, g.SX, (int)b1, (int)e1,
                                   row_hi, 1, addend)
                       : launch_ex(bp_z0_runs_kernel<1, R, true, FULL, false>, grid, block, 0,
                                   stream, false, y, x, angles, g, g.SX, (int)b1, (int)e1,
                                   row_hi, 1, addend);
    else
      e = programmatic ? launch_ex(bp_z0_runs_kernel<1, R, false, FULL, true>, grid, block, 0,
                                   stream, true, y, x, angles, g, g.SX, (int)b1, (int)e1,
                                   row_hi, 1, no_addend)
                       : launch_ex(bp_z0_runs_kernel<1, R, false, FULL, false>, grid, block,
                                   0, stream, false, y, x, angles, g, g.SX, (int)b1, (int)e1,
                                   row_hi, 1, no_addend);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
  }
  return cudaSuccess;
}

// The run launches, with the constant-offset loads when every lane's heights
// are inside [0, H) (8 per lane and whole chunks of 256).
template <int R>
cudaError_t launch_bp_z0_runs(const float* y, float* x, const float* angles, const Geom& g,
                              int row_lo, int row_hi, cudaStream_t stream,
                              const float* addend = nullptr, bool programmatic = false,
                              cudaEvent_t addend_ready = nullptr) {
  if (R == 8 && g.H % (32 * 8) == 0)
    return launch_bp_z0_runs_h<R, true>(y, x, angles, g, row_lo, row_hi, stream, addend,
                                        programmatic, addend_ready);
  return launch_bp_z0_runs_h<R, false>(y, x, angles, g, row_lo, row_hi, stream, addend,
                                       programmatic, addend_ready);
}

// Runs with 8 heights per lane on heights [0, r8_heights(H)) and 4 on the
// rest (one part when H <= 128 or the split leaves no remainder).
int bp0_split(const Geom& g) { return g.H > 128 ? r8_heights(g.H) : 0; }

cudaError_t launch_bp_z0_runs_split(const float* y, float* x, const float* angles,
                                    const Geom& g, int row_lo, int row_hi,
                                    cudaStream_t stream, bool tma = false,
                                    const float* addend = nullptr,
                                    cudaEvent_t addend_ready = nullptr) {
  const int H8 = bp0_split(g);
  if (H8 > 0) {
    Geom g8 = g;
    g8.H = H8;
    const cudaError_t e =
        tma ? launch_bp_z0_runs_tma(y, x, angles, g8, row_lo, row_hi, stream)
            : launch_bp_z0_runs<8>(y, x, angles, g8, row_lo, row_hi, stream, addend, false,
                                   addend_ready);
    if (e != cudaSuccess || H8 == g.H) return e;
  }
  Geom g4 = g;
  g4.H = g.H - H8;
  // after the 8-height part's run launches (the bulk-copy form has no
  // programmatic wait, so a launch after it is an ordinary one); the addend
  // wait was taken there, if there was one
  return launch_bp_z0_runs<4>(y + H8, x + H8, angles, g4, row_lo, row_hi, stream,
                              addend ? addend + H8 : nullptr, H8 > 0 && !tma,
                              H8 > 0 ? nullptr : addend_ready);
}

bool bp0_vec4(const float* y, const float* x, const Geom& g) {
  return (g.Hx % 4 == 0) && (g.Hy % 4 == 0) &&
         ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15) == 0;
}

int launches_backward_z0(const float* y, const float* x, const Geom& g) {
  const int v = kernel_variant(OP_BACKWARD_Z0);
  if (!bp0_vec4(y, x, g) || (v >= 1 && v <= 5)) return 1;
  const int H8 = bp0_split(g);  // runs: two launches per height part
  return (v != 6 && H8 > 0 && H8 < g.H) ? 4 : 2;
}

// Variants: 1 = one voxel run per warp (bp_z0_kernel); 2 = 4x4 register
// block; 3 = 4x2; 4 = 2x2 (accumulates in the reference's order, so its
// results equal the reference's bit for bit); 5 = 8x2; 6 = runs along the
// axis of smaller step, two launches (bp_z0_runs_kernel); 7 = runs with 8
// heights per lane (two float4, 128 heights apart; problems of at most 128
// heights run 6, and a last chunk of at most 128 heights runs with 4 per
// lane); 9 = as 7 with each angle's windows staged per block by bulk copies
// (bp_z0_runs_tma_kernel).  The default when heights come in float4 is 7.
cudaError_t launch_backward_z0(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream) {
  const bool vec4 = bp0_vec4(y, x, g);
  const int variant = kernel_variant(OP_BACKWARD_Z0);
  if (vec4 && variant != 1) {
    switch (variant) {
      case 2: return launch_bp_z0_block<4, 4>(y, x, angles, g, stream);
      case 3: return launch_bp_z0_block<4, 2>(y, x, angles, g, stream);
      case 4: return launch_bp_z0_block<2, 2>(y, x, angles, g, stream);
      case 5: return launch_bp_z0_block<8, 2>(y, x, angles, g, stream);
      case 6: return launch_bp_z0_runs<4>(y, x, angles, g, 0, g.SY, stream);
      case 9: return launch_bp_z0_runs_split(y, x, angles, g, 0, g.SY, stream, true);
      default: return launch_bp_z0_runs_split(y, x, angles, g, 0, g.SY, stream);
    }
  }
  const int R = vec4 ? 4 : 1;
  dim3 block(32, BP0_WARPS);
  dim3 grid(ceil_div(g.SX, BP0_RUN), ceil_div(g.SY, BP0_WARPS), ceil_div(g.H, 32 * R));
  if (vec4)
    bp_z0_kernel<4><<<grid, block, 0, stream>>>(y, x, angles, g);
  else
    bp_z0_kernel<1><<<grid, block, 0, stream>>>(y, x, angles, g);
  return cudaGetLastError();
}

unsigned long long wait_timeouts() {
  unsigned long long n = 0;
  if (cudaMemcpyFromSymbol(&n, g_wait_timeouts, sizeof(n)) != cudaSuccess) return ~0ull;
  return n;
}

int backward_z0_row_step(const float* y, const float* x, const Geom& g) {
  const int v = kernel_variant(OP_BACKWARD_Z0);
  return (bp0_vec4(y, x, g) && (v < 1 || v > 5)) ? RUN : 0;
}

cudaError_t launch_backward_z0_rows(const float* y, float* x, const float* angles,
                                    const Geom& g, int row_lo, int row_hi,
                                    cudaStream_t stream) {
  if (row_lo == 0 && row_hi == g.SY) return launch_backward_z0(y, x, angles, g, stream);
  if (backward_z0_row_step(y, x, g) == 0 || row_lo % RUN != 0) return cudaErrorInvalidValue;
  const int v = kernel_variant(OP_BACKWARD_Z0);
  if (v == 6) return launch_bp_z0_runs<4>(y, x, angles, g, row_lo, row_hi, stream);
  return launch_bp_z0_runs_split(y, x, angles, g, row_lo, row_hi, stream, v == 9);
}

bool backward_z0_rows_can_add(const float* y, const float* x, const Geom& g) {
  const int v = kernel_variant(OP_BACKWARD_Z0);
  return bp0_vec4(y, x, g) && (v == 0 || v == 6 || v == 7);
}

cudaError_t launch_backward_z0_rows_add(const float* y, float* x, const float* angles,
                                        const Geom& g, int row_lo, int row_hi,
                                        const float* addend, cudaStream_t stream,
                                        cudaEvent_t addend_ready) {
  if (!backward_z0_rows_can_add(y, x, g) || row_lo % RUN != 0) return cudaErrorInvalidValue;
  if (kernel_variant(OP_BACKWARD_Z0) == 6)
    return launch_bp_z0_runs<4>(y, x, angles, g, row_lo, row_hi, stream, addend, false,
                                addend_ready);
  return launch_bp_z0_runs_split(y, x, angles, g, row_lo, row_hi, stream, false, addend,
                                 addend_ready);
}

cudaError_t launch_backward_z2(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream) {
  dim3 block(32, BP2_WARPS);
  dim3 grid(ceil_div(g.SX, 32), ceil_div(g.SY, BP2_WARPS), ceil_div(g.H, BP2_RH));
  bp_z2_kernel<<<grid, block, 0, stream>>>(y, x, angles, g);
  return cudaGetLastError();
}

}  // namespace vp
