// Batched projections: many problems of different sizes and angle counts,
// A and A^T mixed, in one persistent launch.
//
// vp_batch_create validates the problems, splits each into work items and
// uploads a descriptor table (the only allocations: the table, the stage
// counters and an error flag).  vp_batch_run resets the counters and launches
// one persistent kernel with a full wave of blocks (SMs x resident blocks).
// Each block repeatedly takes the next item from a global counter, finds its
// problem by binary search and runs the same per-warp bodies as the
// single-problem kernels:
//   forward item = (problem, 128-height chunk, volume slab, angle, 4 bin runs)
//   adjoint item = (problem, 128-height chunk, angle class, 4 voxel runs)
//                  or, variant 4, (problem, chunk, 4 voxel blocks of 2x2)
// Items are numbered problem by problem, heights slowest, so blocks running
// together share one problem and height chunk and its working set stays in
// L2 (as the single-problem kernels' slabs and height ordering do); the
// dynamic counter balances problems of very different sizes.
//
// Stages.  The forward's volume slabs all add into the same sinogram bins,
// and the run adjoint's two angle classes into the same voxels.  Within a
// (problem, height chunk) these are numbered stages; every warp task counts
// itself done on its stage's counter after writing, and a task of stage s > 0
// waits, just before its read-modify-write, until stage s-1 is complete, then
// reads the output past L1.  Items are taken in increasing order, so every
// task a waiter depends on was taken earlier by a block that is already
// running: the wait always ends.  It is bounded anyway: after ~4 s of spinning
// it records an error (vp_batch_error) and writes regardless.
//
// A run allocates and synchronises nothing, so it can be captured in a CUDA
// graph and replayed.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
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

enum BatchKind : int { K_FWD = 0, K_BWD_RUNS = 1, K_BWD_BLOCK = 2 };

struct BatchDesc {
  const float* in;
  float* out;
  const float* angles;
  Geom g;
  long long begin;      // first global item of this problem
  long long per_chunk;  // items per 128-height chunk
  int kind;
  int nstages;          // stages per chunk
  int counter_base;     // first stage counter of this problem
  // forward: slab rows, bin groups per angle
  int slab_rows, units;
  // run adjoint: runs and run groups of each class
  int nruns0, groups0, nruns1, groups1;
  // block adjoint: blocks along x, blocks, block groups
  int nbx, nblocks, bgroups;
};

union BatchSmem {
  float4 cand[BATCH_WARPS][32 * Fp0Cap<4>::value];
  struct {
    RunEntry tab[BATCH_WARPS][BPR_CHUNK];
    int alist[BATCH_WARPS][BPR_LIST];
  } runs;
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
  static constexpr bool coherent = true;
  __device__ __forceinline__ void operator()() const {
    if ((threadIdx.x & 31) == 0) {
      unsigned spins = 0;
      while (*(volatile const unsigned*)counter < target) {
        if (++spins > kMaxSpins) {
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

__device__ __forceinline__ void signal_done(unsigned* counter) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    __threadfence();  // this task's outputs before its count
    atomicAdd(counter, 1u);
  }
}

__device__ __forceinline__ void run_fwd_item(const BatchDesc& d, long long local, int stage,
                                             long long in_stage, int hc, BatchSmem& sm, int w,
                                             int lane, unsigned* counters, int* error) {
  const int a = (int)(in_stage / d.units);
  const int bg = (int)(in_stage % d.units);
  const int y_lo = stage * d.slab_rows;
  const int y_hi = min(d.g.SY, y_lo + d.slab_rows);
  unsigned* ctr = counters + d.counter_base + hc * d.nstages + stage;
  const int p0 = (bg * BATCH_WARPS + w) * 4;
  const int h = (hc * 32 + lane) * 4;
  if (stage == 0) {
    fp_z0_warp<4, 4>(d.in, d.out, d.angles, d.g, p0, a, h, row_slab(y_lo, y_hi, d.g.SX), 1,
                     sm.cand[w]);
  } else {
    const StageWait wt{ctr - 1, (unsigned)(d.g.n_ang * d.units * BATCH_WARPS), error};
    fp_z0_warp<4, 4>(d.in, d.out, d.angles, d.g, p0, a, h, row_slab(y_lo, y_hi, d.g.SX), 1,
                     sm.cand[w], wt);
  }
  signal_done(ctr);
}

__device__ __forceinline__ void run_bwd_runs_item(const BatchDesc& d, int stage, long long grp,
                                                  int hc, BatchSmem& sm, int w, int lane,
                                                  unsigned* counters, int* error) {
  unsigned* ctr = counters + d.counter_base + hc * d.nstages + stage;
  const int run = (int)grp * BATCH_WARPS + w;
  const int h = (hc * 32 + lane) * 4;
  if (stage == 0) {
    if (run < d.nruns0) {
      const int nmaj = (d.g.SX + RUN - 1) / RUN;
      bp_runs_warp<0>(d.in, d.out, d.angles, d.g, (run % nmaj) * RUN, run / nmaj, h, 1,
                      sm.runs.tab[w], sm.runs.alist[w]);
    }
  } else if (run < d.nruns1) {
    const StageWait wt{ctr - 1, (unsigned)(d.groups0 * BATCH_WARPS), error};
    bp_runs_warp<1>(d.in, d.out, d.angles, d.g, run % d.g.SX, (run / d.g.SX) * RUN, h, 1,
                    sm.runs.tab[w], sm.runs.alist[w], wt);
  }
  signal_done(ctr);
}

// 7 resident blocks per SM (72 registers), the occupancy of the
// single-problem run adjoint; the few spilled values are item bookkeeping.
__global__ void __launch_bounds__(BATCH_THREADS, 7)
    batch_kernel(const BatchDesc* __restrict__ descs, int ndesc, long long total,
                 unsigned long long* __restrict__ next, unsigned* __restrict__ counters,
                 int* __restrict__ error) {
  __shared__ BatchSmem sm;
  __shared__ long long s_item;
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(next, 1ull);
    __syncthreads();
    const long long item = s_item;
    if (item >= total) return;  // block-uniform
    int lo = 0, hi = ndesc - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (descs[mid].begin <= item) lo = mid; else hi = mid - 1;
    }
    const BatchDesc d = descs[lo];
    const long long local = item - d.begin;
    const int hc = (int)(local / d.per_chunk);
    const long long in_chunk = local % d.per_chunk;
    if (d.kind == K_FWD) {
      const long long per_stage = (long long)d.g.n_ang * d.units;
      run_fwd_item(d, local, (int)(in_chunk / per_stage), in_chunk % per_stage, hc, sm, w, lane,
                   counters, error);
    } else if (d.kind == K_BWD_RUNS) {
      const bool first = in_chunk < d.groups0;
      run_bwd_runs_item(d, first ? 0 : 1, first ? in_chunk : in_chunk - d.groups0, hc, sm, w,
                        lane, counters, error);
    } else {
      const int bidx = (int)in_chunk * BATCH_WARPS + w;
      if (bidx < d.nblocks)
        bp_block_warp<2, 2>(d.in, d.out, d.angles, d.g, (bidx % d.nbx) * 2, (bidx / d.nbx) * 2,
                            (hc * 32 + lane) * 4, 1,
                            reinterpret_cast<float4(*)[4]>(&sm.blk.tw[w][0][0]), sm.blk.tb[w]);
    }
    __syncthreads();  // shared memory and s_item are reused by the next item
  }
}

unsigned ceil_div_u(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace
}  // namespace vp

struct vp_batch_plan {
  int device = 0;
  vp::BatchDesc* d_descs = nullptr;
  unsigned long long* d_next = nullptr;
  unsigned* d_counters = nullptr;
  int* d_error = nullptr;
  int ndesc = 0;
  int ncounters = 0;
  long long total = 0;
  int grid = 0;
};

namespace {

int batch_desc(const vp_batch_problem& p, vp::BatchDesc* d, bool* empty) {
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
  *empty = xd[0] == 0 || xd[1] == 0 || yd[0] == 0 || yd[1] == 0 || H == 0;
  if (*empty) return VP_OK;
  if (!p.in || !p.out || !p.angles) return VP_ERR_NULL_POINTER;
  // the batched bodies read and write heights as float4
  if ((xd[2] % 4) || (yd[2] % 4) ||
      ((reinterpret_cast<uintptr_t>(p.in) | reinterpret_cast<uintptr_t>(p.out)) & 15))
    return VP_ERR_BATCH;
  vp::Geom& g = d->g;
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
  d->in = p.in;
  d->out = p.out;
  d->angles = p.angles;
  const long long hch = (H + 127) / 128;
  if (fwd) {
    if (p.variant != 0 && p.variant != 1) return VP_ERR_BATCH;
    d->kind = vp::K_FWD;
    // about 32 MB of one 128-height chunk of the volume per slab
    long long rows = (32ll << 20) / ((long long)g.SX * 128 * 4);
    rows = rows < 8 ? 8 : rows;
    d->slab_rows = (int)(rows < g.SY ? rows : g.SY);
    d->nstages = (int)vp::ceil_div_u(g.SY, d->slab_rows);
    d->units = (int)vp::ceil_div_u(g.PX, 4ll * vp::BATCH_WARPS);
    d->per_chunk = (long long)d->nstages * g.n_ang * d->units;
  } else if (p.variant == 0 || p.variant == 6) {
    d->kind = vp::K_BWD_RUNS;
    d->nstages = 2;
    d->nruns0 = (int)vp::ceil_div_u(g.SX, vp::detail::RUN) * g.SY;
    d->nruns1 = g.SX * (int)vp::ceil_div_u(g.SY, vp::detail::RUN);
    d->groups0 = (int)vp::ceil_div_u(d->nruns0, vp::BATCH_WARPS);
    d->groups1 = (int)vp::ceil_div_u(d->nruns1, vp::BATCH_WARPS);
    d->per_chunk = (long long)d->groups0 + d->groups1;
  } else if (p.variant == 4) {
    d->kind = vp::K_BWD_BLOCK;
    d->nstages = 1;
    d->nbx = (int)vp::ceil_div_u(g.SX, 2);
    d->nblocks = d->nbx * (int)vp::ceil_div_u(g.SY, 2);
    d->bgroups = (int)vp::ceil_div_u(d->nblocks, vp::BATCH_WARPS);
    d->per_chunk = d->bgroups;
  } else {
    return VP_ERR_BATCH;
  }
  d->begin = hch * d->per_chunk;  // item count, turned into offsets later
  d->counter_base = (int)(hch * d->nstages);  // counter count, turned into offsets later
  return VP_OK;
}

}  // namespace

extern "C" {

int vp_batch_create(const vp_batch_problem* problems, int count, vp_batch_plan** plan) {
  if (plan == nullptr || (count > 0 && problems == nullptr)) return VP_ERR_NULL_POINTER;
  if (count < 0) return VP_ERR_BATCH;
  *plan = nullptr;
  std::vector<vp::BatchDesc> descs;
  descs.reserve(count);
  long long total = 0;
  long long ncounters = 0;
  for (int i = 0; i < count; ++i) {
    vp::BatchDesc d;
    std::memset(&d, 0, sizeof(d));
    bool empty = false;
    if (int s = batch_desc(problems[i], &d, &empty)) return s;
    if (empty) continue;
    const long long n = d.begin;
    d.begin = total;
    total += n;
    const long long nc = d.counter_base;
    d.counter_base = (int)ncounters;
    ncounters += nc;
    descs.push_back(d);
  }
  if (ncounters >= (1ll << 31)) return VP_ERR_BATCH;
  vp_batch_plan* pl = new (std::nothrow) vp_batch_plan;
  if (pl == nullptr) return VP_ERR_BATCH;
  cudaError_t e = cudaGetDevice(&pl->device);
  int sms = 0, per_sm = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pl->device);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vp::batch_kernel,
                                                      vp::BATCH_THREADS, 0);
  if (e == cudaSuccess && !descs.empty())
    e = cudaMalloc(&pl->d_descs, descs.size() * sizeof(vp::BatchDesc));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_next, sizeof(unsigned long long));
  if (e == cudaSuccess && ncounters > 0) e = cudaMalloc(&pl->d_counters, ncounters * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_error, sizeof(int));
  if (e == cudaSuccess && !descs.empty())
    e = cudaMemcpy(pl->d_descs, descs.data(), descs.size() * sizeof(vp::BatchDesc),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(pl->d_error, 0, sizeof(int));
  if (e != cudaSuccess) {
    vp_batch_destroy(pl);
    return vp::record_cuda_error(e);
  }
  pl->ndesc = (int)descs.size();
  pl->ncounters = (int)ncounters;
  pl->total = total;
  const long long wave = (long long)sms * (per_sm > 0 ? per_sm : 1);
  pl->grid = (int)(total < wave ? total : wave);
  *plan = pl;
  return VP_OK;
}

int vp_batch_run(vp_batch_plan* plan, void* stream) {
  if (plan == nullptr) return VP_ERR_NULL_POINTER;
  if (plan->total == 0) return VP_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(plan->d_next, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess && plan->ncounters > 0)
    e = cudaMemsetAsync(plan->d_counters, 0, (size_t)plan->ncounters * sizeof(unsigned), st);
  if (e == cudaSuccess) {
    vp::batch_kernel<<<plan->grid, vp::BATCH_THREADS, 0, st>>>(
        plan->d_descs, plan->ndesc, plan->total, plan->d_next, plan->d_counters, plan->d_error);
    e = cudaGetLastError();
  }
  vp::count_launches(1);
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
  if (plan->d_descs) cudaFree(plan->d_descs);
  if (plan->d_next) cudaFree(plan->d_next);
  if (plan->d_counters) cudaFree(plan->d_counters);
  if (plan->d_error) cudaFree(plan->d_error);
  cudaSetDevice(prev);
  delete plan;
  return VP_OK;
}

}  // extern "C"
