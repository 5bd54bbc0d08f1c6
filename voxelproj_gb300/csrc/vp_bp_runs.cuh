// Per-warp body of the z_order 0 run adjoint (two angle classes, 4-voxel runs
// along the axis of smaller step, bin window per (run, angle) in registers),
// shared by the single-problem kernel (vp_backward.cu) and the batched
// persistent kernel (vp_batch.cu).  See vp_backward.cu for the design.
#pragma once

#include "vp_common.cuh"

namespace vp {
namespace detail {

constexpr int RUN = 4;
constexpr int BPR_WARPS = 4;
constexpr int BPR_CHUNK = 32;
constexpr int BPR_LIST = 1024;  // class angles listed per window of the angle axis
constexpr int BPR_GENERIC = 8;  // pattern value of the generic path
constexpr int BPR_SKIP = 9;     // pattern value of a window wholly off the detector

struct RunEntry {
  float4 w[3];  // weights of voxels 0..3, 3 each, in window order
  int4 r;       // bin round(xp) of each voxel
  int4 meta;    // element offset of the window's first bin (lo, hi), signed
                // element step between window bins, pattern
};

// Fast path for advance pattern PAT: loads the W = 3 + popcount(PAT) window
// bins with no predicates (the table phase routed windows that leave the
// detector to the generic path, and windows wholly off it to no path at all),
// then applies the four voxels' weights.
// p points at the window's first bin at this lane's first height (lh.s0);
// stride is the signed distance between consecutive window bins.
template <int PAT, int R, bool FULL = false>
__device__ __forceinline__ void run_window(typename Vec<R>::T (&acc)[RUN], const float4 (&wv)[3],
                                           const float* p, ptrdiff_t stride, const LaneH<R>& lh) {
  constexpr int o1 = (PAT & 1);
  constexpr int o2 = o1 + ((PAT >> 1) & 1);
  constexpr int o3 = o2 + ((PAT >> 2) & 1);
  constexpr int W = 3 + o3;
  typename Vec<R>::T win[W];
#pragma unroll
  for (int u = 0; u < W; ++u) win[u] = lh.template load<FULL>(p + u * stride);
  const float ws[12] = {wv[0].x, wv[0].y, wv[0].z, wv[0].w, wv[1].x, wv[1].y,
                        wv[1].z, wv[1].w, wv[2].x, wv[2].y, wv[2].z, wv[2].w};
  constexpr int off[RUN] = {0, o1, o2, o3};
#pragma unroll
  for (int m = 0; m < RUN; ++m) {
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[m] = f4_fma(ws[3 * m + k], win[off[m] + k], acc[m]);
  }
}

// Origin of run `run` of class PASS.  Class 1 runs go along y (RUN rows) and
// are numbered along x, so the warps of a block take neighbouring columns.
// Class 0 runs go along x; they are numbered in bands of RUN rows, x-run
// major, so the warps of a block take the same x-run in RUN neighbouring
// rows.  Either way the four warps' windows at one angle are a fraction of a
// bin apart and mostly shared through L1.
template <int PASS>
__device__ __forceinline__ void run_origin(int run, int nrun_major, int* xi0, int* yi0) {
  if (PASS == 0) {
    const int band = run / (RUN * nrun_major);
    const int q = run - band * RUN * nrun_major;
    *xi0 = (q / RUN) * RUN;
    *yi0 = band * RUN + q % RUN;
  } else {
    *xi0 = run % nrun_major;
    *yi0 = (run / nrun_major) * RUN;
  }
}

template <int PASS>
__device__ __forceinline__ bool in_class(float phi, int trig) {
  float s, c;
  if (trig == TRIG_REF) {
    __sincosf(phi, &s, &c);
  } else {
    sincosf(phi, &s, &c);
  }
  return (PASS == 0) == (fabsf(c) <= fabsf(s));
}

// The class's angles in [w0, wend), ascending, into list; returns the count.
template <int PASS>
__device__ __forceinline__ int list_class_angles(const float* angles, int w0, int wend,
                                                 int trig, int* list) {
  const int lane = threadIdx.x & 31;
  int nlist = 0;
  for (int a1 = w0; a1 < wend; a1 += 32) {
    const int a = a1 + lane;
    const bool mine = a < wend && in_class<PASS>(angles[a], trig);
    const unsigned mask = __ballot_sync(0xffffffffu, mine);
    if (mine) list[nlist + __popc(mask & ((1u << lane) - 1u))] = a;
    nlist += __popc(mask);
  }
  __syncwarp();
  return nlist;
}

// The table entry of bp_runs_warp for angle a and the run at (xi0, yi0).
template <int PASS>
__device__ __forceinline__ RunEntry run_entry(const float* angles, int a, const Geom& g,
                                              int xi0, int yi0) {
  const int dx = PASS == 0 ? 1 : 0;
  const int dy = PASS == 0 ? 0 : 1;
  const AngleConst k = angle_const(angles[a], g.trig);
  BinWeights bw[RUN];
#pragma unroll
  for (int m = 0; m < RUN; ++m) {
    const float relx = (float)(xi0 + m * dx) - g.xcent;
    const float rely = (float)(yi0 + m * dy) - g.ycent;
    bw[m] = voxel_weights(relx, rely, k, g.pcent, g.trig);
  }
  const float step = PASS == 0 ? k.c : k.s;
  const int dir = step >= 0.0f ? 1 : -1;
  int pattern = 0;
  bool ok = true;
#pragma unroll
  for (int m = 0; m + 1 < RUN; ++m) {
    const int d = dir * (bw[m + 1].r - bw[m].r);
    ok = ok && (d == 0 || d == 1);
    pattern |= (d == 1 ? 1 : 0) << m;
  }
  const int base = bw[0].r - dir;
  const int last = base + dir * (2 + __popc(pattern));
  ok = ok && (unsigned)base < (unsigned)g.PX && (unsigned)last < (unsigned)g.PX;
  // every bin of every voxel off the detector: the run adds nothing at this
  // angle (adding the zero products would leave the sums unchanged, bit for
  // bit, since a sum that starts at +0 never becomes -0)
  const int rmin = min(min(bw[0].r, bw[1].r), min(bw[2].r, bw[3].r));
  const int rmax = max(max(bw[0].r, bw[1].r), max(bw[2].r, bw[3].r));
  const bool off_detector = rmax + 1 < 0 || rmin - 1 >= g.PX;
  float ws[12];
#pragma unroll
  for (int m = 0; m < RUN; ++m) {
    ws[3 * m + 0] = dir > 0 ? bw[m].w0 : bw[m].w2;
    ws[3 * m + 1] = bw[m].w1;
    ws[3 * m + 2] = dir > 0 ? bw[m].w2 : bw[m].w0;
  }
  RunEntry e;
  e.w[0] = make_float4(ws[0], ws[1], ws[2], ws[3]);
  e.w[1] = make_float4(ws[4], ws[5], ws[6], ws[7]);
  e.w[2] = make_float4(ws[8], ws[9], ws[10], ws[11]);
  e.r = make_int4(bw[0].r, bw[1].r, bw[2].r, bw[3].r);
  const long long off = (long long)a * g.PX * g.Hy + (long long)base * g.Hy;
  e.meta = make_int4((int)(unsigned)(off & 0xffffffffll), (int)(off >> 32), dir * g.Hy,
                     off_detector ? BPR_SKIP : ok ? pattern : BPR_GENERIC);
  return e;
}

// One warp: the run of class PASS starting at voxel (xi0, yi0), this lane's
// heights from h (R = 4: [h, h + 4); R = 8: also [h + 128, h + 132); FULL:
// all of them inside [0, H)).  tab
// (BPR_CHUNK entries) and alist (BPR_LIST ints) are this warp's shared
// tables.  All 32 lanes must call it together.  wait() runs (by the whole
// warp) just before the outputs are written; with Wait::coherent the read of
// the output bypasses L1.
template <int PASS, int R = 4, class Wait = NoWait, bool ADD = false, bool FULL = false>
__device__ __forceinline__ void bp_runs_warp(const float* __restrict__ y, float* __restrict__ x,
                                             const float* __restrict__ angles, const Geom& g,
                                             int xi0, int yi0, int h, int accumulate,
                                             RunEntry* tab, int* alist,
                                             const Wait& wait = Wait(),
                                             const float* __restrict__ addend = nullptr) {
  using V = typename Vec<R>::T;
  static_assert(R == 4 || R == 8, "heights per lane: 4 or 8");
  const int lane = threadIdx.x & 31;
  const LaneH<R> lh(h, g.H);
  const int dx = PASS == 0 ? 1 : 0;
  const int dy = PASS == 0 ? 0 : 1;

  V acc[RUN];
#pragma unroll
  for (int m = 0; m < RUN; ++m) acc[m] = vzero<V>();

  int seen = 0;
  const float* ys = y + lh.s0;  // this lane's heights of bin 0 of angle 0

  for (int w0 = 0; w0 < g.n_ang; w0 += BPR_LIST) {
    // this warp's list of the class's angles in [w0, w0 + BPR_LIST), ascending
    const int nlist =
        list_class_angles<PASS>(angles, w0, min(g.n_ang, w0 + BPR_LIST), g.trig, alist);

    for (int c0 = 0; c0 < nlist; c0 += BPR_CHUNK) {
      const int count = min(BPR_CHUNK, nlist - c0);
      if (lane < count) tab[lane] = run_entry<PASS>(angles, alist[c0 + lane], g, xi0, yi0);
      __syncwarp();
      for (int j = 0; j < count; ++j) {
        const RunEntry& e = tab[j];
        const int4 meta = e.meta;
        const float4 wv[3] = {e.w[0], e.w[1], e.w[2]};
        const long long off =
            (long long)(unsigned)meta.x | ((long long)meta.y << 32);
        const float* p = ys + off;
        const ptrdiff_t stride = meta.z;
        // run_entry writes a pattern, BPR_GENERIC or BPR_SKIP
        __builtin_assume(meta.w >= 0 && meta.w <= BPR_SKIP);
        switch (meta.w) {
          case 0: run_window<0, R, FULL>(acc, wv, p, stride, lh); break;
          case 1: run_window<1, R, FULL>(acc, wv, p, stride, lh); break;
          case 2: run_window<2, R, FULL>(acc, wv, p, stride, lh); break;
          case 3: run_window<3, R, FULL>(acc, wv, p, stride, lh); break;
          case 4: run_window<4, R, FULL>(acc, wv, p, stride, lh); break;
          case 5: run_window<5, R, FULL>(acc, wv, p, stride, lh); break;
          case 6: run_window<6, R, FULL>(acc, wv, p, stride, lh); break;
          case 7: run_window<7, R, FULL>(acc, wv, p, stride, lh); break;
          case BPR_SKIP: break;
          default: {
            // generic path: three guarded loads per voxel, bins relative to
            // the window start (p), whose bin is r0 - dir
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
                const V v = (unsigned)bin < (unsigned)g.PX
                                ? lh.template load<FULL>(p + (ptrdiff_t)(bin - base) * g.Hy)
                                : vzero<V>();
                acc[m] = f4_fma(ws[3 * m + kk], v, acc[m]);
              }
            }
            break;
          }
        }
      }
      __syncwarp();
    }
    seen += nlist;
  }

  wait();
  if constexpr (ADD) {
    // adding into x, then adding addend (same layout as x): (x + sums) + addend,
    // as a write of the sums followed by a separate add of addend
    if (lh.v[0]) {
#pragma unroll
      for (int m = 0; m < RUN; ++m) {
        const int xi = xi0 + m * dx;
        const int yi = yi0 + m * dy;
        if (xi < g.SX && yi < g.SY) {
          const size_t o = ((size_t)yi * g.SX + xi) * g.Hx;
          add_lane<R>(x + o, addend + o, lh, acc[m], seen > 0);
        }
      }
    }
  } else if (lh.v[0] && (seen > 0 || !accumulate)) {  // a lane past H has no second half either
#pragma unroll
    for (int m = 0; m < RUN; ++m) {
      const int xi = xi0 + m * dx;
      const int yi = yi0 + m * dy;
      if (xi < g.SX && yi < g.SY)
        store_lane<R, Wait::coherent>(x + ((size_t)yi * g.SX + xi) * g.Hx, lh, acc[m],
                                      accumulate);
    }
  }
}

}  // namespace detail
}  // namespace vp
