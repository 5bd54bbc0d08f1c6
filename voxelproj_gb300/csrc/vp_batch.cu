// Batched projections: many problems of different sizes and angle counts,
// A and A^T mixed, in one persistent launch per body (at most six).
//
// vp_batch_create validates the problems, splits each into work items and
// uploads a descriptor table (the only allocations: the table, the stage
// counters and an error flag).  vp_batch_run resets the counters and, for
// each body present (forward or run adjoint, 4 or 8 heights per lane, the
// 8-height forms also on whole 256-height chunks), launches one persistent kernel with a full wave of blocks (SMs x resident
// blocks).
// Each block repeatedly takes the next item from a global counter, finds its
// problem by binary search and runs the same per-warp bodies, with the same
// heights per lane and the same volume slabs, as the single-problem kernel
// of the problem's variant:
//   forward item = (problem, height chunk, volume slab, angle, 4 bin runs)
//   adjoint item = (problem, height chunk, angle class, 4 voxel runs)
//                  or, variant 4, (problem, chunk, 4 voxel blocks of 2x2)
// A height chunk is 32 lanes x 4 or 8 heights.  Items are numbered problem
// by problem, heights slowest, so blocks running together share one problem
// and height chunk and its working set stays in L2 (as the single-problem
// kernels' slabs and height ordering do); the dynamic counter balances
// problems of very different sizes.
//
// Stages.  The forward's volume slabs all add into the same sinogram bins,
// and the run adjoint's two angle classes into the same voxels.  Within a
// (problem, height chunk) these are numbered stages; every warp task counts
// itself done after writing, and a task of stage s > 0 waits, just before its
// read-modify-write, until what it adds to is complete, then reads the output
// past L1: for the forward, the same output tile (height chunk, angle, bin
// group) at stage s-1, on the tile's counter; for the adjoint, all of stage
// s-1, on the stage's counter.  Items are taken in increasing order, so every
// task a waiter depends on was taken earlier by a block that is already
// running: the wait always ends.  It is bounded anyway: after ~4 s of spinning
// it records an error (vp_batch_error) and writes regardless.  The bound is a
// kernel argument; vp_set_wait_limits lowers it, or makes every stage wait
// need one completion more than its stage gives, so that tests can drive the
// error path without any fault.
//
// A run allocates and synchronises nothing, so it can be captured in a CUDA
// graph and replayed.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/voxelproj_gb300.h"
#include "vp_bp_block.cuh"
#include "vp_bp_runs.cuh"
#include "vp_common.cuh"
#include "vp_fp_z0.cuh"
#include "vp_launch.h"

namespace vp {
namespace {

using namespace detail;

constexpr int BATCH_THREADS = 128;  // 4 warps
constexpr int BATCH_WARPS = BATCH_THREADS / 32;
static_assert(BATCH_WARPS == FP0_WARPS && BATCH_WARPS == BPB_WARPS &&
                  BATCH_WARPS == BPR_WARPS, "4 warps per block");
constexpr unsigned kMaxSpins = 1u << 24;  // x ~256 ns sleeps: ~4 s

// Stage-wait limits of a run: sleeps before giving up, and completions a
// stage waits for beyond what its previous stage gives (0 in operation).
struct WaitLimits {
  unsigned spins;
  unsigned extra;
};

enum BatchKind : int { K_FWD = 0, K_BWD_RUNS = 1, K_BWD_BLOCK = 2 };

struct BatchDesc {
  const float* in;
  float* out;
  const float* angles;
  Geom g;
  long long begin;      // first global item of this problem
  long long per_chunk;  // items per height chunk
  int kind;
  int R;                // heights per lane: 4, or 8 as two float4 128 apart
  int nstages;          // stages per chunk
  int counter_base;     // first counter of this problem (forward: per tile; run adjoint:
                        // per class-0 item; block adjoint: per stage, unused)
  // forward: slab plan (class slabs, rows and columns per slab); an item
  // row is an angle (its bins in groups of 4 runs, one per warp) or, with
  // agroup, a group of 4 neighbouring angles (one per warp, on the same
  // 4-bin run); units: item columns per row
  int cls, wy, wx, units, agroup, rows;
  // run adjoint: runs and run groups of each class
  int nruns0, groups0, nruns1, groups1;
  // block adjoint: blocks along x, blocks, block groups
  int nbx, nblocks, bgroups;
};

// Shared memory of each body: the forward bodies hold only their candidate
// lists (as the single-problem forward, leaving the rest of the SM's unified
// storage to L1); the adjoint bodies their run tables, or the 2x2 block
// tables where the 4-height adjoint carries that variant too.
struct FwdSmem {
  float4 cand[BATCH_WARPS][Fp0Cap<4>::list];
};
struct RunsSmem {
  RunEntry tab[BATCH_WARPS][BPR_CHUNK];
  int alist[BATCH_WARPS][BPR_LIST];
};
union Bwd4Smem {
  RunsSmem runs;
  struct {
    float4 tw[BATCH_WARPS][BPB_CHUNK][4];
    int2 tb[BATCH_WARPS][BPB_CHUNK];
  } blk;
};

// Waits (bounded) until the previous stage's counter reaches its target.
struct StageWait {
  const unsigned* counter;
  unsigned target;
  int* error;
  unsigned limit;  // sleeps before giving up
  static constexpr bool coherent = true;
  __device__ __forceinline__ void operator()() const {
    if ((threadIdx.x & 31) == 0) {
      unsigned spins = 0;
      while (*(volatile const unsigned*)counter < target) {
        if (++spins > limit) {
          atomicExch(error, 1);
          break;
        }
        __nanosleep(256);
      }
      __threadfence();
    }
    __syncwarp();
  }
};

// A warp's wait state parked in shared memory while its body runs, so that
// the gather does not hold it in registers.
struct WaitSlot {
  unsigned* counter;
  int* error;
  unsigned target;  // 0: no wait (the first stage)
  unsigned limit;
};

struct SlotWait {
  const WaitSlot* slot;
  static constexpr bool coherent = true;
  __device__ __forceinline__ void operator()() const {
    if (slot->target > 0) StageWait{slot->counter, slot->target, slot->error, slot->limit}();
  }
};

__device__ __forceinline__ void signal_done(unsigned* counter) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    __threadfence();  // this task's outputs before its count
    atomicAdd(counter, 1u);
  }
}

// A forward item's outputs are one (height chunk, item row, item column)
// tile: 16 neighbouring bins of one angle, or with agroup 4 neighbouring bins
// of 4 neighbouring angles; one item per stage writes it.  Its counter counts
// the warps done on the tile, so a stage waits for the tile's previous stage
// alone.
// FULL: the part's heights are whole 256-height chunks (R = 8).
// Out of line: its own register allocation, apart from the persistent loop's
// state (on the 64-cube workload the batched forward took 169.8 against
// 179.2 ms inlined).
template <int R, bool FULL>
__device__ __noinline__ void run_fwd_item(const BatchDesc& d, int stage, int in_stage,
                                             int hc, FwdSmem& sm, WaitSlot* slot, int w,
                                             int lane, unsigned* counters, int* error,
                                             const WaitLimits& lim) {
  constexpr int UN = R == 8 ? 2 : FP0_UNROLL;  // as the single-problem kernels
  const int row = in_stage / d.units;
  const int u = in_stage - row * d.units;
  const Slab slab = slab_of(stage, d.cls, d.wy, d.wx, d.g.SY, d.g.SX);
  // one counter per item tile: its 4 warps count themselves done on it
  if (lane == 0)
    *slot = WaitSlot{counters + d.counter_base + ((size_t)hc * d.rows + row) * d.units + u,
                     error, stage > 0 ? (unsigned)(stage * BATCH_WARPS) + lim.extra : 0u,
                     lim.spins};
  __syncwarp();
  const int a = d.agroup ? row * BATCH_WARPS + w : row;
  const int p0 = d.agroup ? u * 4 : (u * BATCH_WARPS + w) * 4;
  const int h = hc * 32 * R + lane * 4;
  fp_z0_warp<R, 4, UN, SlotWait, FULL>(d.in, d.out, d.angles, d.g, p0, a, h, slab, 1,
                                       sm.cand[w], SlotWait{slot});
  signal_done(slot->counter);
}

// A class-0 item (group grp) is the 4 x 4 voxel tile of band grp / nmaj
// (rows 4 * band ..) and columns 4 * (grp % nmaj) .., one row per warp
// (run_origin<0>); its counter counts its warps done.  A class-1 run (column
// x, band b) adds into the 4 voxels that class-0 group b * nmaj + x / 4 wrote,
// so each class-1 warp waits for that group alone (with columns a multiple of
// 4, class-1 group g waits for class-0 group g).  Before, class-1 items
// waited for every class-0 item of their height chunk, and the blocks that
// took a chunk's first class-1 items spun while its last class-0 items ran.
// FULL: the part's heights are whole 256-height chunks (R = 8).
template <int R, bool FULL>
__device__ __forceinline__ void run_bwd_runs_item(const BatchDesc& d, int stage, int grp,
                                                  int hc, RunsSmem& sm, int w, int lane,
                                                  unsigned* counters, int* error,
                                                  const WaitLimits& lim) {
  unsigned* tiles = counters + d.counter_base + (size_t)hc * d.groups0;
  const int run = grp * BATCH_WARPS + w;
  const int h = hc * 32 * R + lane * 4;
  const int nmaj = (d.g.SX + RUN - 1) / RUN;
  if (stage == 0) {
    int xi0, yi0;
    run_origin<0>(run, nmaj, &xi0, &yi0);
    if (run < d.nruns0 && yi0 < d.g.SY)
      bp_runs_warp<0, R, NoWait, false, FULL>(d.in, d.out, d.angles, d.g, xi0, yi0, h, 1,
                                              sm.tab[w], sm.alist[w]);
    signal_done(tiles + grp);
  } else if (run < d.nruns1) {
    const int x = run % d.g.SX;
    const int band = run / d.g.SX;
    const StageWait wt{tiles + band * nmaj + x / RUN, (unsigned)BATCH_WARPS + lim.extra, error,
                       lim.spins};
    bp_runs_warp<1, R, StageWait, false, FULL>(d.in, d.out, d.angles, d.g, x, band * RUN, h, 1,
                                               sm.tab[w], sm.alist[w], wt);
  }
}

// One kernel instance per body: the forward or the run adjoint with 4 or 8
// heights per lane (the 2x2 block adjoint rides with the 4-height adjoint),
// and the 8-height forms again for parts of whole 256-height chunks, whose
// second float4 is at a constant offset (FWD8F, BWD8F), as in the
// single-problem launches.
// Each instance gets the register allocation of its single-problem kernel, so
// no body runs at another body's occupancy; a plan launches the instances of
// the bodies it holds, one persistent launch each.
// Forward variant of a batched problem that asks for the default (0):
// VP_BATCH_FORWARD_DEFAULT = 21, the single-problem default's angle groups
// (in the 4-height form too) with 128 MB class slabs, whose fewer stages wait
// less in a batch.  On the 64-cube
// workload the batched forward took 151.5 ms with them against 154.8 ms with
// the single-problem default's 64 MB slabs (sequential calls: 156.4 ms); the
// single-problem calls gain more from 64 MB slabs, whose extra launches
// overlap there.
constexpr int kBatchForwardDefault = VP_BATCH_FORWARD_DEFAULT;

constexpr int B_FWD4 = 0, B_FWD8 = 1, B_BWD4 = 2, B_BWD8 = 3, B_FWD8F = 4, B_BWD8F = 5,
              NBODIES = 6;

__host__ __device__ inline int body_of(const BatchDesc& d) {
  if (d.kind == K_FWD) return d.R == 8 ? (d.g.H % 256 == 0 ? B_FWD8F : B_FWD8) : B_FWD4;
  if (d.kind == K_BWD_RUNS && d.R == 8) return d.g.H % 256 == 0 ? B_BWD8F : B_BWD8;
  return B_BWD4;
}

// Resident blocks per SM the registers must allow, so that each body keeps
// its single-problem kernel's occupancy despite the item bookkeeping:
// 8-height forwards 7 (72 registers, a few spilled; at 6 blocks the 64-cube
// batch took 332 ms instead of 322), 4-height forward 8 (64, as the
// single-problem 4-height kernel; at 7 blocks and 72 registers it ran 1.7%
// slower than its single calls), 8-height run adjoints 5 (96); the 4-height
// adjoints as the compiler chooses (72).
constexpr int batch_min_blocks(int body) {
  return body == B_FWD4 ? 8 : (body == B_FWD8 || body == B_FWD8F) ? 7
         : (body == B_BWD8 || body == B_BWD8F)                  ? 5
                                                                : 0;
}

template <int BODY>
struct BodySmem {
  using T = Bwd4Smem;
};
template <>
struct BodySmem<B_FWD4> {
  using T = FwdSmem;
};
template <>
struct BodySmem<B_FWD8> {
  using T = FwdSmem;
};
template <>
struct BodySmem<B_FWD8F> {
  using T = FwdSmem;
};
template <>
struct BodySmem<B_BWD8> {
  using T = RunsSmem;
};
template <>
struct BodySmem<B_BWD8F> {
  using T = RunsSmem;
};

__device__ __forceinline__ RunsSmem& runs_of(RunsSmem& sm) { return sm; }
__device__ __forceinline__ RunsSmem& runs_of(Bwd4Smem& sm) { return sm.runs; }

// Each block takes items from the body's counter; thread 0 finds the item's
// problem and keeps its descriptor in shared memory, so the bodies read the
// geometry from there instead of holding it in registers through the
// gather.  Items are taken in increasing order, so a block's problem index
// only moves forward and is looked up again only when the item leaves it.
template <int BODY>
__global__ void __launch_bounds__(BATCH_THREADS, batch_min_blocks(BODY))
    batch_kernel(const BatchDesc* __restrict__ descs, int ndesc, long long total,
                 unsigned long long* __restrict__ next, unsigned* __restrict__ counters,
                 int* __restrict__ error, WaitLimits lim) {
  __shared__ typename BodySmem<BODY>::T sm;
  __shared__ WaitSlot slots[BATCH_WARPS];
  __shared__ BatchDesc s_desc;        // the current item's problem
  __shared__ long long s_item;
  __shared__ long long s_next_begin;  // first item of the problem after s_desc's
  __shared__ int s_lo;                // index of s_desc, -1: none yet
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) s_lo = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const long long it = (long long)atomicAdd(next, 1ull);
      s_item = it;
      if (it < total && (s_lo < 0 || it >= s_next_begin)) {
        int lo = s_lo < 0 ? 0 : s_lo, hi = ndesc - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (descs[mid].begin <= it) lo = mid; else hi = mid - 1;
        }
        s_lo = lo;
        s_desc = descs[lo];
        s_next_begin = lo + 1 < ndesc ? descs[lo + 1].begin : total;
      }
    }
    __syncthreads();
    // the same for every lane: broadcast within the warp so that it is
    // warp-uniform to the compiler as well
    const long long item = __shfl_sync(0xffffffffu, s_item, 0);
    if (item >= total) return;  // block-uniform
    const BatchDesc& d = s_desc;
    // 32-bit index arithmetic: a problem's items fit in an int (checked when
    // the plan is made)
    const int local = (int)(item - d.begin);
    const int hc = local / (int)d.per_chunk;
    const int in_chunk = local - hc * (int)d.per_chunk;
    if constexpr (BODY == B_FWD4 || BODY == B_FWD8 || BODY == B_FWD8F) {
      constexpr int R = BODY == B_FWD4 ? 4 : 8;
      const int per_stage = d.rows * d.units;
      const int stage = in_chunk / per_stage;
      run_fwd_item<R, BODY == B_FWD8F>(d, stage, in_chunk - stage * per_stage, hc, sm,
                                       &slots[w], w, lane, counters, error, lim);
    } else {
      // the adjoint bodies run faster on a register copy of the descriptor
      // (108.3 against 110.6 ms on the 64-cube workload)
      const BatchDesc dr = s_desc;
      if (BODY == B_BWD8 || BODY == B_BWD8F || dr.kind == K_BWD_RUNS) {
        constexpr int R = (BODY == B_BWD8 || BODY == B_BWD8F) ? 8 : 4;
        const bool first = in_chunk < dr.groups0;
        run_bwd_runs_item<R, BODY == B_BWD8F>(dr, first ? 0 : 1,
                                              first ? in_chunk : in_chunk - dr.groups0, hc,
                                              runs_of(sm), w, lane, counters, error, lim);
      } else if constexpr (BODY == B_BWD4) {
        const int bidx = in_chunk * BATCH_WARPS + w;
        if (bidx < dr.nblocks)
          bp_block_warp<2, 2>(dr.in, dr.out, dr.angles, dr.g, (bidx % dr.nbx) * 2,
                              (bidx / dr.nbx) * 2, (hc * 32 + lane) * 4, 1,
                              reinterpret_cast<float4(*)[4]>(&sm.blk.tw[w][0][0]),
                              sm.blk.tb[w]);
      }
    }
    __syncthreads();  // shared memory and the item are reused by the next item
  }
}

unsigned ceil_div_u(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

using BatchKernelFn = void (*)(const BatchDesc*, int, long long, unsigned long long*, unsigned*,
                               int*, WaitLimits);

const void* batch_kernel_for(int body) {
  static const BatchKernelFn fns[NBODIES] = {batch_kernel<B_FWD4>, batch_kernel<B_FWD8>,
                                             batch_kernel<B_BWD4>, batch_kernel<B_BWD8>,
                                             batch_kernel<B_FWD8F>, batch_kernel<B_BWD8F>};
  return reinterpret_cast<const void*>(fns[body]);
}

}  // namespace

// Stage-wait limits of the runs enqueued from now on (set_stage_wait_limits).
std::atomic<unsigned> g_stage_spins{kMaxSpins};
std::atomic<unsigned> g_stage_extra{0};

void set_stage_wait_limits(unsigned spins, unsigned extra) {
  g_stage_spins.store(spins ? spins : kMaxSpins);
  g_stage_extra.store(extra);
}

}  // namespace vp

struct vp_batch_plan {
  int device = 0;
  vp::BatchDesc* d_descs = nullptr;     // grouped by body, problem order within a body
  unsigned long long* d_next = nullptr;  // one item counter per body
  unsigned* d_counters = nullptr;
  int* d_error = nullptr;
  int ncounters = 0;
  long long total = 0;
  // per body: first descriptor, descriptors, items, grid (0: body absent)
  int first[vp::NBODIES] = {};
  int ndesc[vp::NBODIES] = {};
  long long items[vp::NBODIES] = {};
  int grid[vp::NBODIES] = {};
  // room of the device buffers, and whether they came from the stream-ordered
  // allocator (grown by vp_batch_update) rather than cudaMalloc
  size_t desc_cap = 0, counter_cap = 0;
  bool descs_async = false, counters_async = false;
  // vp_batch_update: two page-locked staging buffers for descriptor uploads,
  // used in turn, each with the event of its last upload
  vp::BatchDesc* staging[2] = {nullptr, nullptr};
  size_t staging_cap[2] = {0, 0};
  cudaEvent_t uploaded[2] = {nullptr, nullptr};
  bool upload_pending[2] = {false, false};
  int next_staging = 0;
};

namespace {

// Work items of one height part: heights [0, g.H) of in / out, R heights
// per lane for the runs adjoint (the forward takes R from its plan).
int part_desc(const vp_batch_problem& p, const vp::Geom& g, const float* in, float* out, int R,
              vp::BatchDesc* d) {
  std::memset(d, 0, sizeof(*d));
  d->g = g;
  d->in = in;
  d->out = out;
  d->angles = p.angles;
  if (p.op == VP_OP_FORWARD) {
    // the single-problem forward's plan for this variant (0: the batch's
    // default, kBatchForwardDefault)
    const vp::Fp0Plan pl =
        vp::forward_z0_plan(g, true, p.variant ? p.variant : vp::kBatchForwardDefault);
    if (pl.KW != 4 || pl.split || pl.staged ||
        (pl.R == 8 ? pl.un != 2 : pl.un != vp::detail::FP0_UNROLL))
      return VP_ERR_BATCH;  // bodies the batch does not carry
    d->kind = vp::K_FWD;
    d->R = pl.R;
    d->cls = pl.cls ? 1 : 0;
    d->wy = pl.wy;
    d->wx = pl.wx;
    d->nstages = pl.nslabs;
    d->agroup = pl.agroup ? 1 : 0;
    d->rows = pl.agroup ? (int)vp::ceil_div_u(g.n_ang, vp::BATCH_WARPS) : g.n_ang;
    d->units = (int)vp::ceil_div_u(g.PX, pl.agroup ? 4ll : 4ll * vp::BATCH_WARPS);
    d->per_chunk = (long long)d->nstages * d->rows * d->units;
  } else if (p.variant == 0 || p.variant == 6 || p.variant == 7) {
    d->kind = vp::K_BWD_RUNS;
    d->R = R;
    d->nstages = 2;
    // class-0 runs in bands of RUN rows (run_origin), rows padded to the band
    d->nruns0 = (int)vp::ceil_div_u(g.SX, vp::detail::RUN) *
                (int)vp::ceil_div_u(g.SY, vp::detail::RUN) * vp::detail::RUN;
    d->nruns1 = g.SX * (int)vp::ceil_div_u(g.SY, vp::detail::RUN);
    d->groups0 = (int)vp::ceil_div_u(d->nruns0, vp::BATCH_WARPS);
    d->groups1 = (int)vp::ceil_div_u(d->nruns1, vp::BATCH_WARPS);
    d->per_chunk = (long long)d->groups0 + d->groups1;
  } else if (p.variant == 4) {
    d->kind = vp::K_BWD_BLOCK;
    d->R = 4;
    d->nstages = 1;
    d->nbx = (int)vp::ceil_div_u(g.SX, 2);
    d->nblocks = d->nbx * (int)vp::ceil_div_u(g.SY, 2);
    d->bgroups = (int)vp::ceil_div_u(d->nblocks, vp::BATCH_WARPS);
    d->per_chunk = d->bgroups;
  } else {
    return VP_ERR_BATCH;
  }
  const long long hch = (g.H + 32 * d->R - 1) / (32 * d->R);
  if (hch * d->per_chunk >= (1ll << 31)) return VP_ERR_BATCH;  // items indexed as int
  d->begin = hch * d->per_chunk;  // item count, turned into offsets later
  // counter count, turned into offsets later: one per forward tile, one per
  // class-0 item of the run adjoint
  const long long nctr = d->kind == vp::K_FWD        ? hch * d->rows * d->units
                         : d->kind == vp::K_BWD_RUNS ? hch * d->groups0
                                                     : hch * d->nstages;
  if (nctr >= (1ll << 31)) return VP_ERR_BATCH;
  d->counter_base = (int)nctr;
  return VP_OK;
}

// The problem's descriptors: one per height part.  With 8 heights per lane a
// last chunk of at most 128 heights is a second part with 4 per lane, as in
// the single-problem launchers (r8_heights).
int batch_desc(const vp_batch_problem& p, std::vector<vp::BatchDesc>* out) {
  if (p.op != VP_OP_FORWARD && p.op != VP_OP_BACKWARD) return VP_ERR_BATCH;
  if (p.flags & ~VP_FLAG_TRIG_PRECISE) return VP_ERR_BAD_FLAGS;
  const bool fwd = p.op == VP_OP_FORWARD;
  const int64_t* xd = fwd ? p.in_dims : p.out_dims;
  const int64_t* yd = fwd ? p.out_dims : p.in_dims;
  for (int i = 0; i < 3; ++i)
    if (xd[i] < 0 || yd[i] < 0 || xd[i] >= (1 << 30) || yd[i] >= (1 << 30)) return VP_ERR_BAD_SHAPE;
  if (xd[0] * xd[1] >= ((int64_t)1 << 27)) return VP_ERR_BAD_SHAPE;
  if (yd[0] > 0 && p.n_angles < yd[0]) return VP_ERR_ANGLES;
  const int64_t H = xd[2] < yd[2] ? xd[2] : yd[2];
  if (xd[0] == 0 || xd[1] == 0 || yd[0] == 0 || yd[1] == 0 || H == 0) return VP_OK;  // empty
  if (!p.in || !p.out || !p.angles) return VP_ERR_NULL_POINTER;
  // the batched bodies read and write heights as float4
  if ((xd[2] % 4) || (yd[2] % 4) ||
      ((reinterpret_cast<uintptr_t>(p.in) | reinterpret_cast<uintptr_t>(p.out)) & 15))
    return VP_ERR_BATCH;
  vp::Geom g;
  g.SY = (int)xd[0];
  g.SX = (int)xd[1];
  g.Hx = (int)xd[2];
  g.n_ang = (int)yd[0];
  g.PX = (int)yd[1];
  g.Hy = (int)yd[2];
  g.H = (int)H;
  g.xcent = 0.5f * (float)(g.SX - 1);
  g.ycent = 0.5f * (float)(g.SY - 1);
  g.pcent = 0.5f * (float)(g.PX - 1);
  g.trig = (p.flags & VP_FLAG_TRIG_PRECISE) ? vp::TRIG_PRECISE : vp::TRIG_REF;
  g.accumulate = 1;
  // heights per lane of the first part
  int R = 4;
  if (fwd)
    R = vp::forward_z0_plan(g, true, p.variant ? p.variant : vp::kBatchForwardDefault).R;
  else if ((p.variant == 0 || p.variant == 7) && H > 128)
    R = 8;
  const int H8 = R == 8 ? vp::r8_heights(g.H) : g.H;
  vp::BatchDesc d;
  vp::Geom g0 = g;
  g0.H = H8;
  if (int st = part_desc(p, g0, p.in, p.out, R, &d)) return st;
  out->push_back(d);
  if (H8 < g.H) {
    vp::Geom g1 = g;
    g1.H = g.H - H8;
    if (int st = part_desc(p, g1, p.in + H8, p.out + H8, 4, &d)) return st;
    out->push_back(d);
  }
  return VP_OK;
}

// A plan's descriptors and bookkeeping for a set of problems: descriptors
// grouped by body, items numbered from 0 within each body, a persistent
// grid of one full wave per body present.
struct Layout {
  std::vector<vp::BatchDesc> descs;
  int first[vp::NBODIES] = {};
  int ndesc[vp::NBODIES] = {};
  long long items[vp::NBODIES] = {};
  int grid[vp::NBODIES] = {};
  long long total = 0;
  long long ncounters = 0;
};

// Resident blocks per SM of each body on the current device (cached).
cudaError_t blocks_per_sm(int device, int (&per_sm)[vp::NBODIES], int* sms) {
  static std::mutex mu;
  static int cached[64][vp::NBODIES + 1];
  static bool have[64] = {};
  std::lock_guard<std::mutex> lock(mu);
  if (device >= 0 && device < 64 && have[device]) {
    for (int b = 0; b < vp::NBODIES; ++b) per_sm[b] = cached[device][b];
    *sms = cached[device][vp::NBODIES];
    return cudaSuccess;
  }
  cudaError_t e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device);
  for (int b = 0; b < vp::NBODIES && e == cudaSuccess; ++b)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[b], vp::batch_kernel_for(b),
                                                      vp::BATCH_THREADS, 0);
  if (e == cudaSuccess && device >= 0 && device < 64) {
    for (int b = 0; b < vp::NBODIES; ++b) cached[device][b] = per_sm[b];
    cached[device][vp::NBODIES] = *sms;
    have[device] = true;
  }
  return e;
}

// Validates the problems and lays out their descriptors (no CUDA call).
int make_layout(const vp_batch_problem* problems, int count, Layout* L) {
  std::vector<vp::BatchDesc> by_body[vp::NBODIES];
  std::vector<vp::BatchDesc> parts;
  for (int i = 0; i < count; ++i) {
    parts.clear();
    if (int s = batch_desc(problems[i], &parts)) return s;
    for (const vp::BatchDesc& d : parts) by_body[vp::body_of(d)].push_back(d);
  }
  L->descs.reserve(2 * (size_t)count);
  for (int b = 0; b < vp::NBODIES; ++b) {
    L->first[b] = (int)L->descs.size();
    long long items = 0;
    for (vp::BatchDesc d : by_body[b]) {
      const long long n = d.begin;
      d.begin = items;
      items += n;
      const long long nc = d.counter_base;
      d.counter_base = (int)L->ncounters;
      L->ncounters += nc;
      L->descs.push_back(d);
    }
    L->ndesc[b] = (int)by_body[b].size();
    L->items[b] = items;
    L->total += items;
  }
  if (L->ncounters >= (1ll << 31)) return VP_ERR_BATCH;
  return VP_OK;
}

// One full wave of blocks per body present, on `device`.
int fill_grid(int device, Layout* L) {
  int per_sm[vp::NBODIES] = {}, sms = 0;
  const cudaError_t e = blocks_per_sm(device, per_sm, &sms);
  if (e != cudaSuccess) return vp::record_cuda_error(e);
  for (int b = 0; b < vp::NBODIES; ++b) {
    if (L->items[b] == 0) continue;
    const long long wave = (long long)sms * (per_sm[b] > 0 ? per_sm[b] : 1);
    L->grid[b] = (int)(L->items[b] < wave ? L->items[b] : wave);
  }
  return VP_OK;
}

void adopt_layout(vp_batch_plan* pl, const Layout& L) {
  for (int b = 0; b < vp::NBODIES; ++b) {
    pl->first[b] = L.first[b];
    pl->ndesc[b] = L.ndesc[b];
    pl->items[b] = L.items[b];
    pl->grid[b] = L.grid[b];
  }
  pl->total = L.total;
  pl->ncounters = (int)L.ncounters;
}

// Grows a stream-ordered device buffer to at least `need` elements of `size`
// bytes (by half again), freeing the old one in stream order.
cudaError_t grow(void** buf, size_t* cap, bool* async, size_t need, size_t size,
                 cudaStream_t st) {
  if (need <= *cap) return cudaSuccess;
  const size_t n = need + need / 2;
  void* fresh = nullptr;
  cudaError_t e = cudaMallocAsync(&fresh, n * size, st);
  if (e != cudaSuccess) return e;
  if (*buf) e = *async ? cudaFreeAsync(*buf, st) : cudaFree(*buf);
  *buf = fresh;
  *cap = n;
  *async = true;
  return e;
}

}  // namespace

extern "C" {

int vp_batch_create(const vp_batch_problem* problems, int count, vp_batch_plan** plan) {
  if (plan == nullptr || (count > 0 && problems == nullptr)) return VP_ERR_NULL_POINTER;
  if (count < 0) return VP_ERR_BATCH;
  *plan = nullptr;
  Layout L;
  if (int s = make_layout(problems, count, &L)) return s;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return vp::record_cuda_error(e);
  if (int s = fill_grid(device, &L)) return s;
  vp_batch_plan* pl = new (std::nothrow) vp_batch_plan;
  if (pl == nullptr) return VP_ERR_BATCH;
  pl->device = device;
  adopt_layout(pl, L);
  const std::vector<vp::BatchDesc>& descs = L.descs;
  if (!descs.empty()) e = cudaMalloc(&pl->d_descs, descs.size() * sizeof(vp::BatchDesc));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_next, vp::NBODIES * sizeof(unsigned long long));
  if (e == cudaSuccess && L.ncounters > 0)
    e = cudaMalloc(&pl->d_counters, L.ncounters * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_error, sizeof(int));
  if (e == cudaSuccess && !descs.empty())
    e = cudaMemcpy(pl->d_descs, descs.data(), descs.size() * sizeof(vp::BatchDesc),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(pl->d_error, 0, sizeof(int));
  if (e != cudaSuccess) {
    vp_batch_destroy(pl);
    return vp::record_cuda_error(e);
  }
  pl->desc_cap = descs.size();
  pl->counter_cap = (size_t)L.ncounters;
  *plan = pl;
  return VP_OK;
}

int vp_batch_update(vp_batch_plan* plan, const vp_batch_problem* problems, int count,
                    void* stream) {
  if (plan == nullptr || (count > 0 && problems == nullptr)) return VP_ERR_NULL_POINTER;
  if (count < 0) return VP_ERR_BATCH;
  Layout L;
  if (int s = make_layout(problems, count, &L)) return s;  // plan unchanged
  if (int s = fill_grid(plan->device, &L)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t nd = L.descs.size();
  cudaError_t e = grow(reinterpret_cast<void**>(&plan->d_descs), &plan->desc_cap,
                       &plan->descs_async, nd, sizeof(vp::BatchDesc), st);
  if (e == cudaSuccess)
    e = grow(reinterpret_cast<void**>(&plan->d_counters), &plan->counter_cap,
             &plan->counters_async, (size_t)L.ncounters, sizeof(unsigned), st);
  if (e == cudaSuccess && nd > 0) {
    // the staging buffer used two updates ago: wait for its upload to leave it
    const int k = plan->next_staging;
    plan->next_staging ^= 1;
    if (plan->upload_pending[k]) e = cudaEventSynchronize(plan->uploaded[k]);
    if (e == cudaSuccess && plan->uploaded[k] == nullptr)
      e = cudaEventCreateWithFlags(&plan->uploaded[k], cudaEventDisableTiming);
    if (e == cudaSuccess && plan->staging_cap[k] < nd) {
      if (plan->staging[k]) e = cudaFreeHost(plan->staging[k]);
      plan->staging[k] = nullptr;
      plan->staging_cap[k] = 0;
      const size_t n = nd + nd / 2;
      if (e == cudaSuccess)
        e = cudaMallocHost(reinterpret_cast<void**>(&plan->staging[k]),
                           n * sizeof(vp::BatchDesc));
      if (e == cudaSuccess) plan->staging_cap[k] = n;
    }
    if (e == cudaSuccess) {
      std::memcpy(plan->staging[k], L.descs.data(), nd * sizeof(vp::BatchDesc));
      e = cudaMemcpyAsync(plan->d_descs, plan->staging[k], nd * sizeof(vp::BatchDesc),
                          cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(plan->uploaded[k], st);
    if (e == cudaSuccess) plan->upload_pending[k] = true;
  }
  if (e != cudaSuccess) return vp::record_cuda_error(e);
  adopt_layout(plan, L);
  return VP_OK;
}

int vp_batch_run(vp_batch_plan* plan, void* stream) {
  if (plan == nullptr) return VP_ERR_NULL_POINTER;
  if (plan->total == 0) return VP_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(plan->d_next, 0, vp::NBODIES * sizeof(unsigned long long), st);
  if (e == cudaSuccess && plan->ncounters > 0)
    e = cudaMemsetAsync(plan->d_counters, 0, (size_t)plan->ncounters * sizeof(unsigned), st);
  vp::WaitLimits lim{vp::g_stage_spins.load(), vp::g_stage_extra.load()};
  int launched = 0;
  for (int b = 0; b < vp::NBODIES && e == cudaSuccess; ++b) {
    if (plan->items[b] == 0) continue;
    const vp::BatchDesc* descs = plan->d_descs + plan->first[b];
    unsigned long long* next = plan->d_next + b;
    void* args[] = {&descs, &plan->ndesc[b], &plan->items[b], &next, &plan->d_counters,
                    &plan->d_error, &lim};
    e = cudaLaunchKernel(vp::batch_kernel_for(b), dim3(plan->grid[b]), dim3(vp::BATCH_THREADS),
                         args, 0, st);
    ++launched;
  }
  vp::count_launches(launched);
  return e == cudaSuccess ? VP_OK : vp::record_cuda_error(e);
}

int vp_batch_error(vp_batch_plan* plan, int* error) {
  if (plan == nullptr || error == nullptr) return VP_ERR_NULL_POINTER;
  *error = 0;
  if (plan->d_error == nullptr) return VP_OK;
  const cudaError_t e = cudaMemcpy(error, plan->d_error, sizeof(int), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? VP_OK : vp::record_cuda_error(e);
}

int64_t vp_batch_work_items(const vp_batch_plan* plan) { return plan ? plan->total : 0; }

int vp_batch_destroy(vp_batch_plan* plan) {
  if (plan == nullptr) return VP_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(plan->device);
  // buffers grown by vp_batch_update came from the stream-ordered allocator
  if (plan->d_descs) plan->descs_async ? cudaFreeAsync(plan->d_descs, nullptr) : cudaFree(plan->d_descs);
  if (plan->d_next) cudaFree(plan->d_next);
  if (plan->d_counters)
    plan->counters_async ? cudaFreeAsync(plan->d_counters, nullptr) : cudaFree(plan->d_counters);
  if (plan->d_error) cudaFree(plan->d_error);
  for (int k = 0; k < 2; ++k) {
    if (plan->uploaded[k]) {
      cudaEventSynchronize(plan->uploaded[k]);
      cudaEventDestroy(plan->uploaded[k]);
    }
    if (plan->staging[k]) cudaFreeHost(plan->staging[k]);
  }
  cudaSetDevice(prev);
  delete plan;
  return VP_OK;
}

}  // extern "C"
