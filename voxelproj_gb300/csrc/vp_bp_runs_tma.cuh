// Run adjoint (z_order 0) with each angle's bin window staged once per block
// by bulk copies (TMA) into a shared-memory ring.
//
// A block is 4 compute warps and 1 copy warp.  The compute warps own the runs
// of a 4 x 4 voxel tile: the same 4-voxel run in 4 neighbouring rows (angle
// class 0, runs along x) or columns (class 1, runs along y), and one full
// chunk of 256 heights (8 per lane).  Every warp works through the same
// angles in the same order, so at angle a their windows are a fraction of a
// bin apart: their union is at most ~8 bins, against 3..6 per warp.  The copy
// warp stages that union with one tensor copy (a box of 8 bins x 256 heights
// of the sinogram, 8 KB; bins past the detector read as zero) into one ring
// stage and arms the stage's `full` mbarrier with its byte count; the compute
// warps read
// their window from the stage and release it on the stage's `empty` mbarrier.
// TMA_STAGES angles are in flight.  Tables, windows and arithmetic are those
// of bp_runs_warp with 8 heights per lane, so the results are bit-identical to
// it.  Windows on the generic path (detector edge) and windows a stage could
// not hold are read from global memory.
//
// Every wait is bounded (tma::mbar_wait).  When one runs out the block sets a
// shared flag: no more copies are issued, every warp computes the rest from
// global memory (results stay right), waits still in progress give up, and
// before the block exits the copy warp waits once more, bounded, for the
// stages with copies outstanding.  A compute warp's wait for a stage's copy
// polls at most copy_polls times (the kernel's argument).
#pragma once

#include "vp_bp_runs.cuh"
#include "vp_common.cuh"
#include "vp_tma.cuh"

namespace vp {
namespace detail {

constexpr int TMA_STAGES = 4;         // angles in flight per block
constexpr int TMA_NBMAX = 8;          // bins of a stage: the tensor map's box
constexpr int TMA_BIN_FLOATS = 256;   // one bin's 256 heights (8 per lane)
constexpr int TMA_LIST = 256;         // class angles listed per pass over the angle axis
constexpr int TMA_WARPS = BPR_WARPS;  // compute warps; one more copies
constexpr int TMA_THREADS = 32 * (TMA_WARPS + 1);

struct TmaBlockSmem {
  float ring[TMA_STAGES][TMA_NBMAX * TMA_BIN_FLOATS];  // 32 KB, 1 KB-aligned bins
  uint64_t full[TMA_STAGES];   // bytes of the stage landed (1 arrival + tx)
  uint64_t empty[TMA_STAGES];  // the compute warps are done with it (TMA_WARPS arrivals)
  int lo[TMA_STAGES];          // first staged bin, or -1: nothing staged
  int nb[TMA_STAGES];          // staged bins
  RunEntry tab[TMA_WARPS][BPR_CHUNK];
  int alist[TMA_WARPS + 1][TMA_LIST];
  int broken;                  // a wait ran out: no more copies, global loads only
};
// The fallback for blocks that cannot stage (bp_runs_warp) takes a table and
// a BPR_LIST angle list per compute warp from the ring.
static_assert(sizeof(float) * TMA_STAGES * TMA_NBMAX * TMA_BIN_FLOATS >=
                  TMA_WARPS * (sizeof(RunEntry) * BPR_CHUNK + sizeof(int) * BPR_LIST),
              "the ring must hold the fallback's tables and angle lists");

// Fast path of pattern PAT, the window's bin u read from stage bin
// (base - lo) + dir * u: the same loads-then-FMAs order as run_window<PAT, 8>.
template <int PAT>
__device__ __forceinline__ void run_window_staged(float4x2 (&acc)[RUN], const float4 (&wv)[3],
                                                  const float* first_bin, int dir, int lane) {
  constexpr int o1 = (PAT & 1);
  constexpr int o2 = o1 + ((PAT >> 1) & 1);
  constexpr int o3 = o2 + ((PAT >> 2) & 1);
  constexpr int W = 3 + o3;
  float4x2 win[W];
#pragma unroll
  for (int u = 0; u < W; ++u) {
    const float* b = first_bin + dir * u * TMA_BIN_FLOATS;
    win[u].a = *reinterpret_cast<const float4*>(b + 4 * lane);
    win[u].b = *reinterpret_cast<const float4*>(b + kSecondHalf + 4 * lane);
  }
  const float ws[12] = {wv[0].x, wv[0].y, wv[0].z, wv[0].w, wv[1].x, wv[1].y,
                        wv[1].z, wv[1].w, wv[2].x, wv[2].y, wv[2].z, wv[2].w};
  constexpr int off[RUN] = {0, o1, o2, o3};
#pragma unroll
  for (int m = 0; m < RUN; ++m) {
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[m] = f4_fma(ws[3 * m + k], win[off[m] + k], acc[m]);
  }
}

// Window bins [first, last] (ascending) of a fast entry.
__device__ __forceinline__ void window_bins(const RunEntry& e, int* first, int* last) {
  const int dir = e.meta.z >= 0 ? 1 : -1;
  const int base = e.r.x - dir;
  const int end = base + dir * (2 + __popc(e.meta.w));
  *first = min(base, end);
  *last = max(base, end);
}

// Copy warp: stages entry j (angle a) of the current chunk into stage s: the
// box of bins [lo, lo + TMA_NBMAX) at heights [h0, h0 + 256) of angle a.
__device__ __forceinline__ void stage_entry(TmaBlockSmem& sm, int j, int a, int s, int h0,
                                            const CUtensorMap* ymap) {
  const int lane = threadIdx.x & 31;
  // union of the compute warps' fast windows: lanes 0..TMA_WARPS-1 look at one each
  int lo = 1 << 30, hi = -1;
  if (lane < TMA_WARPS) {
    const RunEntry& e = sm.tab[lane][j];
    if (e.meta.w < BPR_GENERIC) window_bins(e, &lo, &hi);
  }
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, d));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, d));
  }
  const int nb = hi - lo + 1;
  const bool stage = hi >= lo && nb <= TMA_NBMAX;
  if (lane == 0) {
    sm.lo[s] = stage ? lo : -1;
    sm.nb[s] = stage ? nb : 0;
    if (stage) {
      tma::mbar_arrive_expect_tx(&sm.full[s],
                                 (unsigned)(TMA_NBMAX * TMA_BIN_FLOATS * sizeof(float)));
      tma::tensor3d_g2s(&sm.ring[s][0], ymap, h0, lo, a, &sm.full[s]);
    } else {
      tma::mbar_arrive(&sm.full[s]);
    }
  }
}

__device__ __forceinline__ bool block_broken(TmaBlockSmem& sm) {
  return *reinterpret_cast<volatile int*>(&sm.broken) != 0;
}

__device__ __forceinline__ void set_broken(TmaBlockSmem& sm) {
  *reinterpret_cast<volatile int*>(&sm.broken) = 1;
}

// The whole block: compute warps 0..TMA_WARPS-1 (this warp's run at (xi0,
// yi0)), copy warp TMA_WARPS; heights [h0, h0 + 256), a full chunk.
template <int PASS>
__device__ __forceinline__ void bp_runs_tma_block(const float* __restrict__ y,
                                                  float* __restrict__ x,
                                                  const float* __restrict__ angles,
                                                  const Geom& g, int xi0, int yi0, int h0,
                                                  int accumulate, TmaBlockSmem& sm,
                                                  const CUtensorMap* ymap,
                                                  unsigned long long* timeouts,
                                                  unsigned copy_polls) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool copier = w == TMA_WARPS;
  const LaneH<8> lh(h0 + 4 * lane, g.H);
  const int dx = PASS == 0 ? 1 : 0;
  const int dy = PASS == 0 ? 0 : 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < TMA_STAGES; ++s) {
      tma::mbar_init(&sm.full[s], 1);
      tma::mbar_init(&sm.empty[s], TMA_WARPS);
    }
    sm.broken = 0;
    tma::fence_mbar_init();
  }
  __syncthreads();

  float4x2 acc[RUN];
#pragma unroll
  for (int m = 0; m < RUN; ++m) acc[m] = vzero<float4x2>();
  unsigned full_ph = 0, empty_ph = 0;  // per stage: parity of the next phase
  unsigned armed = 0;                  // copy warp: stages whose copies were issued
  unsigned used = 0;                   // copy warp: stages used at least once
  unsigned next_ph = 0;                // copy warp: parity of each stage's next arming
  int slot = 0;                        // ring stage of the next entry
  int seen = 0;

  for (int w0 = 0; w0 < g.n_ang; w0 += TMA_LIST) {
    const int wend = min(g.n_ang, w0 + TMA_LIST);
    int* list = sm.alist[w];
    const int nlist = list_class_angles<PASS>(angles, w0, wend, g.trig, list);
    for (int c0 = 0; c0 < nlist; c0 += BPR_CHUNK) {
      const int count = min(BPR_CHUNK, nlist - c0);
      if (!copier && lane < count)
        sm.tab[w][lane] = run_entry<PASS>(angles, list[c0 + lane], g, xi0, yi0);
      __syncthreads();  // tables of this chunk are complete

      if (copier) {
        for (int j = 0; j < count; ++j) {
          const int s = (slot + j) % TMA_STAGES;
          if (block_broken(sm)) break;
          if (used & (1u << s)) {  // wait until the compute warps released stage s
            const bool ok = __all_sync(
                0xffffffffu, tma::mbar_wait(&sm.empty[s], (empty_ph >> s) & 1u, timeouts,
                                            tma::kTmaMaxPolls, &sm.broken));
            if (!ok) {
              set_broken(sm);
              break;
            }
            empty_ph ^= 1u << s;
            armed &= ~(1u << s);  // its copies landed: the compute warps read them
          }
          if (lane == 0) tma::fence_proxy_async_smem();
          __syncwarp();
          stage_entry(sm, j, list[c0 + j], s, h0, ymap);
          used |= 1u << s;
          armed |= 1u << s;
          next_ph ^= 1u << s;
        }
      } else {
        const RunEntry* tab = sm.tab[w];
        for (int j = 0; j < count; ++j) {
          const int s = (slot + j) % TMA_STAGES;
          bool staged = false;
          if (!block_broken(sm)) {
            staged = __all_sync(0xffffffffu,
                                tma::mbar_wait(&sm.full[s], (full_ph >> s) & 1u, timeouts,
                                               copy_polls, &sm.broken));
            if (staged)
              full_ph ^= 1u << s;
            else
              set_broken(sm);
          }
          const RunEntry& e = tab[j];
          const int4 meta = e.meta;
          const float4 wv[3] = {e.w[0], e.w[1], e.w[2]};
          const long long off = (long long)(unsigned)meta.x | ((long long)meta.y << 32);
          const float* p = y + off + lh.s0;  // for the global-memory paths
          const ptrdiff_t stride = meta.z;
          const int lo = staged ? sm.lo[s] : -1;
          if (meta.w < BPR_GENERIC) {
            const int dir = meta.z >= 0 ? 1 : -1;
            const int base = e.r.x - dir;
            if (lo >= 0) {
              const float* fb = sm.ring[s] + (base - lo) * TMA_BIN_FLOATS;
              switch (meta.w) {
                case 0: run_window_staged<0>(acc, wv, fb, dir, lane); break;
                case 1: run_window_staged<1>(acc, wv, fb, dir, lane); break;
                case 2: run_window_staged<2>(acc, wv, fb, dir, lane); break;
                case 3: run_window_staged<3>(acc, wv, fb, dir, lane); break;
                case 4: run_window_staged<4>(acc, wv, fb, dir, lane); break;
                case 5: run_window_staged<5>(acc, wv, fb, dir, lane); break;
                case 6: run_window_staged<6>(acc, wv, fb, dir, lane); break;
                default: run_window_staged<7>(acc, wv, fb, dir, lane); break;
              }
            } else {
              switch (meta.w) {
                case 0: run_window<0, 8>(acc, wv, p, stride, lh); break;
                case 1: run_window<1, 8>(acc, wv, p, stride, lh); break;
                case 2: run_window<2, 8>(acc, wv, p, stride, lh); break;
                case 3: run_window<3, 8>(acc, wv, p, stride, lh); break;
                case 4: run_window<4, 8>(acc, wv, p, stride, lh); break;
                case 5: run_window<5, 8>(acc, wv, p, stride, lh); break;
                case 6: run_window<6, 8>(acc, wv, p, stride, lh); break;
                default: run_window<7, 8>(acc, wv, p, stride, lh); break;
              }
            }
          } else {
            // generic path: three guarded global loads per voxel
            const int dir = meta.z >= 0 ? 1 : -1;
            const int rr[RUN] = {e.r.x, e.r.y, e.r.z, e.r.w};
            const int base = rr[0] - dir;
            const float ws[12] = {wv[0].x, wv[0].y, wv[0].z, wv[0].w, wv[1].x, wv[1].y,
                                  wv[1].z, wv[1].w, wv[2].x, wv[2].y, wv[2].z, wv[2].w};
#pragma unroll
            for (int m = 0; m < RUN; ++m) {
#pragma unroll
              for (int kk = 0; kk < 3; ++kk) {
                const int bin = rr[m] + dir * (kk - 1);
                const float4x2 v = (unsigned)bin < (unsigned)g.PX
                                       ? lh.load(p + (ptrdiff_t)(bin - base) * g.Hy)
                                       : vzero<float4x2>();
                acc[m] = f4_fma(ws[3 * m + kk], v, acc[m]);
              }
            }
          }
          __syncwarp();  // every lane is done with stage s
          if (staged && lane == 0) tma::mbar_arrive(&sm.empty[s]);
        }
      }
      slot = (slot + count) % TMA_STAGES;
      __syncthreads();  // the tables are rebuilt for the next chunk
    }
    seen += nlist;
  }

  if (copier) {
    // after a wait ran out, stages whose copies were issued may still have
    // bytes in flight: let them land (bounded) before the block's shared
    // memory goes
    if (block_broken(sm)) {
      for (int s = 0; s < TMA_STAGES; ++s)  // the phase of the last arming
        if (armed & (1u << s)) tma::mbar_wait(&sm.full[s], ((next_ph >> s) & 1u) ^ 1u, timeouts);
    }
    return;
  }
  if (lh.v[0] && (seen > 0 || !accumulate)) {
#pragma unroll
    for (int m = 0; m < RUN; ++m) {
      const int xi = xi0 + m * dx;
      const int yi = yi0 + m * dy;
      if (xi < g.SX && yi < g.SY)
        store_lane<8>(x + ((size_t)yi * g.SX + xi) * g.Hx, lh, acc[m], accumulate);
    }
  }
}

}  // namespace detail
}  // namespace vp
