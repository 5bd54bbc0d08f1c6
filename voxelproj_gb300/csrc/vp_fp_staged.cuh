// Forward projection A (z_order 0) with the volume staged in shared memory by
// tensor copies, shared by four neighbouring angles.
//
// The gather of fp_z0_warp brings every candidate voxel's heights into
// registers from L2.  With 72 registers and 7 blocks per SM, the bytes a
// warp can hold in flight bound the kernel: it waits on its loads (long
// scoreboard) with half of its issue slots idle.  Two changes here:
//
// 1. The four compute warps of a block take four neighbouring angles of the
//    same angle class, each on a run of at most 4 bins, and the runs are
//    aligned: a bin p of angle k maps to the lead angle's detector through
//    the point where its ray crosses the slab's middle line,
//        t_k(p) = (p - pcent) * coef_k + off_k,
//    coef_k = shn_lead / shn_k, off_k = m * (shm_lead - shm_k * coef_k)
//    (shn / shm: the detector step per voxel along the minor / major axis,
//    m: the middle line's centred index, lead: the angle of largest |shn|),
//    and block b takes the bins with floor((t_k(p) + pcent + 1/2) / W) = b,
//    W = 3.99 lead bins.  coef_k >= 1, so no block holds more than 4 bins of
//    an angle, and every bin of every angle belongs to exactly one block
//    (blocks past the grid's ends are clamped onto its end blocks).  The four
//    warps' voxel strips then coincide on the middle line and part only
//    slowly away from it: on 512^3 with 192 angles a staged voxel serves 3.4
//    warp candidates on average, against 1.2 for neighbouring bins of one
//    angle.
// 2. A fifth warp copies, for every major line of the slab, the union of the
//    four warps' candidate windows (NBOX voxels x 256 heights) into a ring
//    of STAGES shared-memory stages with one 3-D tensor copy (TMA), under
//    full / empty mbarriers.  The compute warps read their candidates from
//    the stage; candidates past the box read global memory.  Bytes in flight
//    sit in shared memory, not registers.
//
// Candidates, their weights, the order in which each bin sums them (lines in
// order, candidates of a line in minor order) and the slabs are those of
// fp_z0_warp with 8 heights per lane, so the results are equal to variant 10
// bit for bit: a window that differs only adds or drops zero products.
// Groups whose angles are not close (another class, another sign of the
// minor step, a step ratio above 1.06 or a middle-line shift above
// 6% of the detector) run plain fp_z0_warp on runs of 4 bins.
//
// Every wait is bounded (tma::mbar_wait).  When one runs out the block sets a
// shared flag: no more copies are issued, every warp reads the rest from
// global memory (results stay right), and before the block exits the copy
// warp waits once more, bounded, for copies still in flight.
//
// fps_plain_block is the aligned partition alone: the four warps gather with
// plain loads and meet in L1.
//
// Measured on 512^3 with 192 angles, against 0.86 ms per slab launch for
// variant 10: both forms reuse as designed, and neither is faster, so both
// stay opt-in (forward variants 17 and 19).
//   - aligned, plain loads: L1 hit rate 68% (10%), L2 throughput 22% (63%),
//     0.93 ms: the same issue rate (50%) on 10% more instructions;
//   - staged: L2 throughput 20%, 1.72 ms: 2.2x the instructions, mostly
//     compute warps polling their stage's barrier; three lines in flight
//     per block do not cover the copies' latency, and more stages cost
//     occupancy (8-voxel boxes x 6 stages: 2.0 ms).
#pragma once

#include <stdint.h>

#include "vp_common.cuh"
#include "vp_fp_z0.cuh"
#include "vp_tma.cuh"

namespace vp {
namespace detail {

constexpr int FPS_WARPS = 4;                       // compute warps: neighbouring angles
constexpr int FPS_THREADS = 32 * (FPS_WARPS + 1);  // and a copy warp
constexpr int FPS_LINE = 256;                      // floats of one voxel's 256 heights
constexpr float FPS_W = 3.99f;                     // block width, lead bins
constexpr float FPS_MAX_COEF = 1.06f;
constexpr float FPS_MAX_SHIFT = 0.06f;             // of the detector, plus 4 bins

// NBOX voxels per staged line window, STAGES lines in flight.
template <int NBOX, int STAGES>
struct FpsSmem {
  float ring[STAGES][NBOX * FPS_LINE];  // 1 KB-aligned stages
  float4 cand[FPS_WARPS][Fp0Cap<4>::list];
  int rlo[FPS_WARPS][32];   // a warp's candidate window on each line of the batch
  int rhi[FPS_WARPS][32];
  int ulo[32];              // first voxel of each line's staged box, -1: none
  int nbw[FPS_WARPS];       // bins of each warp in this block
  uint64_t full[STAGES];
  uint64_t empty[STAGES];
  int broken;
};

// A group of FPS_WARPS neighbouring angles [a0, a0 + FPS_WARPS) on one slab,
// as every thread of a block computes it alike: the angles' constants, the
// group's class, whether it aligns, and each angle's map onto the lead's
// detector (coef, off2 as fps_block_of).
struct FpsGroup {
  AngleConst K[FPS_WARPS];
  bool valid[FPS_WARPS];
  bool mx;        // minor axis x (the class of the first angle)
  bool aligned;
  float coef[FPS_WARPS], off2[FPS_WARPS];
};

__device__ __forceinline__ FpsGroup fps_group(const float* __restrict__ angles, const Geom& g,
                                              const Slab& slab, int a0) {
  FpsGroup G;
#pragma unroll
  for (int k = 0; k < FPS_WARPS; ++k) {
    G.valid[k] = a0 + k < g.n_ang;
    G.K[k] = G.valid[k] ? angle_const(__ldg(angles + a0 + k), g.trig)
                        : AngleConst{1, 0, 0, 0, 0, 0};
  }
  G.mx = fabsf(G.K[0].c) >= fabsf(G.K[0].s);
  float shn[FPS_WARPS], shm[FPS_WARPS];
  G.aligned = true;
  int lead = 0;
#pragma unroll
  for (int k = 0; k < FPS_WARPS; ++k) {
    shn[k] = G.mx ? G.K[k].c : G.K[k].s;
    shm[k] = G.mx ? G.K[k].s : G.K[k].c;
    if (!G.valid[k]) continue;
    G.aligned = G.aligned && ((fabsf(G.K[k].c) >= fabsf(G.K[k].s)) == G.mx) &&
                ((shn[k] > 0.0f) == (shn[0] > 0.0f)) && shn[k] != 0.0f;
    if (fabsf(shn[k]) > fabsf(shn[lead])) lead = k;
  }
  const int maj_lo = G.mx ? slab.y_lo : slab.x_lo;
  const int maj_hi = G.mx ? slab.y_hi : slab.x_hi;
  const float m = 0.5f * (float)(maj_lo + maj_hi - 1) - (G.mx ? g.ycent : g.xcent);
#pragma unroll
  for (int k = 0; k < FPS_WARPS; ++k) {
    G.coef[k] = 1.0f;
    G.off2[k] = g.pcent + 0.5f;
    if (!G.valid[k] || !G.aligned) continue;
    G.coef[k] = __fdiv_rn(shn[lead], shn[k]);
    const float off = __fmul_rn(m, __fsub_rn(shm[lead], __fmul_rn(shm[k], G.coef[k])));
    G.off2[k] = __fadd_rn(__fadd_rn(off, g.pcent), 0.5f);
    G.aligned = G.aligned && G.coef[k] <= FPS_MAX_COEF &&
                fabsf(off) <= FPS_MAX_SHIFT * (float)g.PX + 4.0f;
  }
  return G;
}

// Grid margin (blocks on each side of the detector) for aligned groups: the
// bins of the non-lead angles reach past the lead's detector by at most
// PX/2 * (FPS_MAX_COEF - 1) + the shift bound.
__host__ __device__ inline int fps_margin(int PX) {
  return (int)((0.09f * (float)PX + 4.0f) / FPS_W) + 2;
}

// The block of bin p of an angle with coefficients (coef, off2), before
// clamping: floor(((p - pcent) * coef + off2) / W), off2 = off + pcent + 1/2.
__device__ __forceinline__ int fps_block_of(int p, float pcent, float coef, float off2) {
  const float t = __fmaf_rn(__fsub_rn((float)p, pcent), coef, off2);
  return (int)floorf(__fdiv_rn(t, FPS_W));
}

// The block's flag as lane 0 of the calling warp reads it (warp-uniform).
__device__ __forceinline__ bool fps_broken(const int& broken) {
  const int v = *reinterpret_cast<const volatile int*>(&broken);
  return __shfl_sync(0xffffffffu, v, 0) != 0;
}
__device__ __forceinline__ void fps_set_broken(int& broken) {
  *reinterpret_cast<volatile int*>(&broken) = 1;
}

// The bins [*first, *first + *nb) of block bx (clamped into [bmin, bmax]) of
// one angle, found by the whole warp: the block index is monotone in p, so
// the bins form one run; the scan starts a little before its estimate.
__device__ __forceinline__ void fps_range(int bx, int bmin, int bmax, int PX, float pcent,
                                          float coef, float off2, int* first, int* nb) {
  const int lane = threadIdx.x & 31;
  auto blk = [&](int p) {
    return min(max(fps_block_of(p, pcent, coef, off2), bmin), bmax);
  };
  // estimate: t = bx * W  ->  p = pcent + (bx * W - off2) / coef
  int p = (int)floorf(pcent + ((float)bx * FPS_W - off2) / coef) - 2;
  p = max(0, min(p, PX - 1));
  if (p > 0 && blk(p) >= bx) p = 0;  // estimate too high: scan from the start
  int f = -1, n = 0;
  for (; p < PX; p += 32) {
    const int q = p + lane;
    const int b = q < PX ? blk(q) : bmax + 1;
    const unsigned in = __ballot_sync(0xffffffffu, b == bx);
    const unsigned past = __ballot_sync(0xffffffffu, b > bx);
    if (in) {
      if (f < 0) f = p + __ffs(in) - 1;
      n += __popc(in);
    }
    if (past) break;
  }
  *first = f < 0 ? 0 : f;
  *nb = n;
}

// One aligned block (FULL: whole 256-height chunks) of group G.  Compute
// warps own bins [first, first + nb) of angle a0 + w.
template <bool FULL, int NBOX, int STAGES>
__device__ __forceinline__ void fps_aligned_block(
    const float* __restrict__ x, float* __restrict__ y, const float* __restrict__ angles,
    const Geom& g, const Slab& s, int accumulate, int a0, int h0, int bx, int bmin, int bmax,
    const FpsGroup& G, FpsSmem<NBOX, STAGES>& sm, const CUtensorMap* map_rows,
    const CUtensorMap* map_cols, unsigned long long* timeouts, unsigned copy_polls) {
  const AngleConst(&K)[FPS_WARPS] = G.K;
  const bool(&valid)[FPS_WARPS] = G.valid;
  const bool mx = G.mx;
  const float(&coef)[FPS_WARPS] = G.coef;
  const float(&off2)[FPS_WARPS] = G.off2;
  constexpr int CAP = Fp0Cap<4>::value;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const bool copier = w == FPS_WARPS;

  int first = 0, nb = 0;
  if (!copier && valid[w])
    fps_range(bx, bmin, bmax, g.PX, g.pcent, coef[w], off2[w], &first, &nb);
  if (!copier && lane == 0) sm.nbw[w] = nb;
  if (threadIdx.x == 0) sm.broken = 0;
  __syncthreads();
  int n_active = 0;
#pragma unroll
  for (int k = 0; k < FPS_WARPS; ++k) n_active += (sm.nbw[k] >= 1 && sm.nbw[k] <= 4) ? 1 : 0;
  if (threadIdx.x == 0 && n_active > 0) {
    for (int st = 0; st < STAGES; ++st) {
      tma::mbar_init(&sm.full[st], 1);
      tma::mbar_init(&sm.empty[st], (unsigned)n_active);
    }
    tma::fence_mbar_init();
  }
  __syncthreads();

  const LaneH<8> lh(h0 + 4 * lane, g.H);
  if (!copier && nb > 4) {
    // a clamped end block: its wide run goes through the plain gather, in
    // runs of up to 4 bins
    for (int p = first; p < first + nb; p += 4)
      fp_z0_warp<8, 4, 2, NoWait, FULL>(x, y, angles, g, p, a0 + w, h0 + 4 * lane, s,
                                        accumulate, sm.cand[w], NoWait(),
                                        min(4, first + nb - p));
    return;
  }
  if (n_active == 0 || (!copier && nb == 0)) return;
  const unsigned nbar = (unsigned)(n_active + 1) * 32u;

  // the group's slab lines (one class for the whole group)
  const int maj_lo = mx ? s.y_lo : s.x_lo;
  const int maj_hi = mx ? s.y_hi : s.x_hi;
  const int min_lo = mx ? 0 : s.yy_lo;
  const int min_hi = mx ? g.SX - 1 : s.yy_hi - 1;
  const float cent_major = mx ? g.ycent : g.xcent;
  const float cent_minor = mx ? g.xcent : g.ycent;

  if (copier) {
    unsigned armed = 0, next_ph = 0;  // stages with a copy issued; parity of their next arming
    unsigned gl = 0;                  // lines issued
    for (int i0 = maj_lo; i0 < maj_hi; i0 += 32) {
      const int nl = min(32, maj_hi - i0);
      asm volatile("bar.sync 1, %0;" ::"r"(nbar) : "memory");  // windows of this batch ready
      int ulo = 1 << 30, uhi = -1;
#pragma unroll
      for (int k = 0; k < FPS_WARPS; ++k) {
        const int n = sm.nbw[k];
        if (n >= 1 && n <= 4 && sm.rlo[k][lane] <= sm.rhi[k][lane]) {
          ulo = min(ulo, sm.rlo[k][lane]);
          uhi = max(uhi, sm.rhi[k][lane]);
        }
      }
      sm.ulo[lane] = uhi >= ulo ? ulo : -1;
      __syncwarp();
      for (int j = 0; j < nl; ++j, ++gl) {
        const int st = (int)(gl % STAGES);
        const unsigned use = gl / STAGES;
        if (use > 0) {  // the compute warps released the stage's previous line
          const bool ok = fps_broken(sm.broken) ? false
                          : __all_sync(0xffffffffu,
                                       tma::mbar_wait(&sm.empty[st], (use - 1) & 1u, timeouts,
                                                      tma::kTmaMaxPolls, &sm.broken));
          if (!ok) {
            fps_set_broken(sm.broken);
          } else {
            armed &= ~(1u << st);  // that line's copy landed before its release
          }
        }
        if (fps_broken(sm.broken)) continue;  // warp-uniform (read by lane 0)
        // The compute warps' reads of the stage's previous line completed
        // before their release (the loaded values fed their sums), so the
        // copy may overwrite it without a proxy fence.
        if (lane == 0) {
          const int u = sm.ulo[j];
          if (u >= 0) {
            tma::mbar_arrive_expect_tx(&sm.full[st],
                                       (unsigned)(NBOX * FPS_LINE * sizeof(float)));
            if (mx)
              tma::tensor3d_g2s(&sm.ring[st][0], map_rows, h0, u, i0 + j, &sm.full[st]);
            else
              tma::tensor3d_g2s(&sm.ring[st][0], map_cols, h0, i0 + j, u, &sm.full[st]);
          } else {
            tma::mbar_arrive(&sm.full[st]);
          }
        }
        __syncwarp();
        armed |= 1u << st;
        next_ph ^= 1u << st;
      }
    }
    if (fps_broken(sm.broken)) {
      // copies issued may still be landing: let them, bounded, before the
      // block's shared memory goes
      for (int st = 0; st < STAGES; ++st)
        if (armed & (1u << st))
          tma::mbar_wait(&sm.full[st], ((next_ph >> st) & 1u) ^ 1u, timeouts);
    }
    return;
  }

  // ---- compute warp: angle a0 + w, bins [first, first + nb) ----
  const int a = a0 + w;
  const AngleConst k = K[w];
  const float sh_major = mx ? k.s : k.c;
  const float inv_sh_minor = 1.0f / (mx ? k.c : k.s);
  const float t_lo = (float)first - 0.5f - k.b - kWindowMargin;
  const float t_hi = (float)(first + nb) - 0.5f + k.b + kWindowMargin;
  float4* cand = sm.cand[w];
  const float* xs = x + lh.s0;

  float4x2 acc[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) acc[b] = vzero<float4x2>();

  unsigned gl = 0;
  for (int i0 = maj_lo; i0 < maj_hi; i0 += 32) {
    const int nl = min(32, maj_hi - i0);
    const int i = i0 + lane;
    int lo = 0, cnt = 0;
    if (lane < nl) {
      const MinorRange mr = minor_range(i, cent_major, sh_major, cent_minor, inv_sh_minor,
                                        min_lo, min_hi, g.pcent, t_lo, t_hi);
      lo = mr.lo;
      cnt = max(0, min(mr.hi - mr.lo + 1, CAP));
    }
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    const int start = incl - cnt;
    for (int t = 0; t < cnt; ++t) {
      const int mm = lo + t;
      const int xi = mx ? mm : i;
      const int yi = mx ? i : mm;
      const BinWeights bw =
          voxel_weights((float)xi - g.xcent, (float)yi - g.ycent, k, g.pcent, g.trig);
      int q = bw.r - first + 1;
      float4 e = make_float4(bw.w0, bw.w1, bw.w2, 0.0f);
      if (q < 0 || q > 5) {
        q = 0;
        e = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      e.w = __int_as_float((mm << FP0_QBITS) | q);
      cand[start + t] = e;
    }
    sm.rlo[w][lane] = cnt > 0 ? lo : 1 << 30;
    sm.rhi[w][lane] = cnt > 0 ? lo + cnt - 1 : -1;
    __syncwarp();
    asm volatile("bar.sync 1, %0;" ::"r"(nbar) : "memory");

    for (int j = 0; j < nl; ++j, ++gl) {
      const int st = (int)(gl % STAGES);
      const unsigned use = gl / STAGES;
      const int c0 = __shfl_sync(0xffffffffu, start, j);
      const int c1 = c0 + __shfl_sync(0xffffffffu, cnt, j);
      bool staged = false;
      if (!fps_broken(sm.broken)) {
        staged = __all_sync(0xffffffffu, tma::mbar_wait(&sm.full[st], use & 1u, timeouts,
                                                       copy_polls, &sm.broken));
        if (!staged) fps_set_broken(sm.broken);
      }
      const int ul = staged ? sm.ulo[j] : -1;
      const float* stage = &sm.ring[st][0] + 4 * lane;
      const int line = i0 + j;
      for (int c = c0; c < c1; c += 2) {
        float4 e[2];
        float4x2 v[2];
        const bool two = c + 1 < c1;  // warp-uniform
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          e[u] = (u == 0 || two) ? cand[c + u] : make_float4(0.f, 0.f, 0.f, 0.f);
          const int mm = __float_as_int(e[u].w) >> FP0_QBITS;
          const unsigned off = (unsigned)(mm - ul);
          if (ul >= 0 && off < (unsigned)NBOX) {
            const float* b = stage + off * FPS_LINE;
            v[u].a = *reinterpret_cast<const float4*>(b);
            v[u].b = *reinterpret_cast<const float4*>(b + kSecondHalf);
          } else {
            const int vox = mx ? line * g.SX + mm : mm * g.SX + line;
            v[u] = lh.template load<FULL>(xs + (size_t)vox * g.Hx);
          }
        }
        scatter_q<4>(acc, e[0], v[0], __float_as_int(e[0].w) & ((1 << FP0_QBITS) - 1));
        if (two) scatter_q<4>(acc, e[1], v[1], __float_as_int(e[1].w) & ((1 << FP0_QBITS) - 1));
      }
      __syncwarp();
      if (staged && lane == 0) tma::mbar_arrive(&sm.empty[st]);
    }
  }

#pragma unroll
  for (int b = 0; b < 4; ++b)
    if (b < nb)
      store_lane<8>(y + ((size_t)a * g.PX + first + b) * g.Hy, lh, acc[b], accumulate);
}

// The aligned partition without staging: each warp of a 4-warp block gathers
// its run of at most 4 bins with plain loads (fp_z0_warp), so the four
// aligned windows meet in L1 instead of a staged box.
template <bool FULL>
__device__ __forceinline__ void fps_plain_block(const float* __restrict__ x, float* __restrict__ y,
                                                const float* __restrict__ angles, const Geom& g,
                                                const Slab& s, int accumulate, int a0, int h0,
                                                int bx, int bmin, int bmax, const FpsGroup& G,
                                                float4* cand) {
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  if (!G.valid[w]) return;
  int first = 0, nb = 0;
  fps_range(bx, bmin, bmax, g.PX, g.pcent, G.coef[w], G.off2[w], &first, &nb);
  for (int p = first; p < first + nb; p += 4)
    fp_z0_warp<8, 4, 2, NoWait, FULL>(x, y, angles, g, p, a0 + w, h0 + 4 * lane, s, accumulate,
                                      cand, NoWait(), min(4, first + nb - p));
}

}  // namespace detail
}  // namespace vp
