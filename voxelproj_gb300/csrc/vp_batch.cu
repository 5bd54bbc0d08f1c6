// Batched projections: many problems of different sizes and angle counts,
// A and A^T mixed, in one persistent launch.
//
// vp_batch_create validates the problems, splits each into work items and
// uploads a descriptor table (the only allocation).  vp_batch_run resets the
// work counter and launches one persistent kernel with a full wave of blocks
// (SMs x resident blocks).  Each block repeatedly takes the next item from a
// global counter, finds its problem by binary search over the table and runs
// the same per-warp bodies as the single-problem kernels:
//   forward item  = (problem, 128-height chunk, angle, group of 4 bin runs)
//   adjoint item  = (problem, 128-height chunk, group of 4 voxel blocks)
// Items are numbered problem by problem with heights slowest, so blocks that
// run together share one problem and one height chunk (cache locality), and
// the dynamic counter balances problems of very different sizes.
//
// Every item of the adjoint owns its voxels for all angles (register-blocked
// 2x2 or 4x2 voxel blocks), and every forward item owns its bins for the
// whole volume (no slabs), so no two items write the same output element and
// no ordering between items is needed.  A run allocates and synchronises
// nothing, so it can be captured in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/voxelproj_gb300.h"
#include "vp_bp_block.cuh"
#include "vp_common.cuh"
#include "vp_fp_z0.cuh"
#include "vp_launch.h"

namespace vp {
namespace {

using namespace detail;

constexpr int BATCH_THREADS = 128;  // 4 warps
constexpr int BATCH_WARPS = BATCH_THREADS / 32;
static_assert(BATCH_WARPS == FP0_WARPS && BATCH_WARPS == BPB_WARPS, "4 warps per block");

enum BatchKind : int { K_FWD4 = 0, K_FWD8 = 1, K_BWD22 = 2, K_BWD42 = 3 };

struct BatchDesc {
  const float* in;
  float* out;
  const float* angles;
  Geom g;
  long long begin;  // first global item of this problem
  int kind;
  int units;        // forward: bin groups per angle; adjoint: voxel-block groups
  int nbx;          // adjoint: blocks along x
  int nblocks;      // adjoint: blocks in total
};

union BatchSmem {
  float4 cand[BATCH_WARPS][32 * Fp0Cap<8>::value];
  struct {
    float4 tw[BATCH_WARPS][BPB_CHUNK][8];
    int2 tb[BATCH_WARPS][BPB_CHUNK];
  } blk;
};

template <int BX, int BY>
__device__ __forceinline__ void run_bwd_item(const BatchDesc& d, long long local, BatchSmem& sm,
                                             int w, int lane) {
  const int hc = (int)(local / d.units);
  const int grp = (int)(local % d.units);
  const int bidx = grp * BATCH_WARPS + w;
  if (bidx >= d.nblocks) return;
  auto* tw = reinterpret_cast<float4(*)[BX * BY]>(&sm.blk.tw[w][0][0]);
  bp_block_warp<BX, BY>(d.in, d.out, d.angles, d.g, (bidx % d.nbx) * BX, (bidx / d.nbx) * BY,
                        (hc * 32 + lane) * 4, 1, tw, sm.blk.tb[w]);
}

template <int KW>
__device__ __forceinline__ void run_fwd_item(const BatchDesc& d, long long local, BatchSmem& sm,
                                             int w, int lane) {
  const long long per_hc = (long long)d.g.n_ang * d.units;
  const int hc = (int)(local / per_hc);
  const long long rem = local % per_hc;
  const int a = (int)(rem / d.units);
  const int bg = (int)(rem % d.units);
  fp_z0_warp<4, KW>(d.in, d.out, d.angles, d.g, (bg * BATCH_WARPS + w) * KW, a,
                    (hc * 32 + lane) * 4, 0, d.g.SY, 1, sm.cand[w]);
}

__global__ void __launch_bounds__(BATCH_THREADS)
    batch_kernel(const BatchDesc* __restrict__ descs, int ndesc, long long total,
                 unsigned long long* __restrict__ counter) {
  __shared__ BatchSmem sm;
  __shared__ long long s_item;
  const int w = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(counter, 1ull);
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
    switch (d.kind) {
      case K_FWD4: run_fwd_item<4>(d, local, sm, w, lane); break;
      case K_FWD8: run_fwd_item<8>(d, local, sm, w, lane); break;
      case K_BWD42: run_bwd_item<4, 2>(d, local, sm, w, lane); break;
      default: run_bwd_item<2, 2>(d, local, sm, w, lane); break;
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
  unsigned long long* d_counter = nullptr;
  int ndesc = 0;
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
    d->kind = p.variant == 2 ? vp::K_FWD8 : vp::K_FWD4;
    const int kw = d->kind == vp::K_FWD8 ? 8 : 4;
    d->units = (int)vp::ceil_div_u(g.PX, (long long)kw * vp::BATCH_WARPS);
    d->nbx = d->nblocks = 0;
    d->begin = hch * g.n_ang * d->units;  // item count, turned into offsets later
  } else {
    d->kind = p.variant == 3 ? vp::K_BWD42 : vp::K_BWD22;
    const int bx = d->kind == vp::K_BWD42 ? 4 : 2, by = 2;
    d->nbx = (int)vp::ceil_div_u(g.SX, bx);
    d->nblocks = d->nbx * (int)vp::ceil_div_u(g.SY, by);
    d->units = (int)vp::ceil_div_u(d->nblocks, vp::BATCH_WARPS);
    d->begin = hch * d->units;
  }
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
  for (int i = 0; i < count; ++i) {
    vp::BatchDesc d;
    std::memset(&d, 0, sizeof(d));
    bool empty = false;
    if (int s = batch_desc(problems[i], &d, &empty)) return s;
    if (empty) continue;
    const long long n = d.begin;
    d.begin = total;
    total += n;
    descs.push_back(d);
  }
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
  if (e == cudaSuccess) e = cudaMalloc(&pl->d_counter, sizeof(unsigned long long));
  if (e == cudaSuccess && !descs.empty())
    e = cudaMemcpy(pl->d_descs, descs.data(), descs.size() * sizeof(vp::BatchDesc),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    vp_batch_destroy(pl);
    return vp::record_cuda_error(e);
  }
  pl->ndesc = (int)descs.size();
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
  cudaError_t e = cudaMemsetAsync(plan->d_counter, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    vp::batch_kernel<<<plan->grid, vp::BATCH_THREADS, 0, st>>>(plan->d_descs, plan->ndesc,
                                                               plan->total, plan->d_counter);
    e = cudaGetLastError();
  }
  vp::count_launches(1);
  return e == cudaSuccess ? VP_OK : vp::record_cuda_error(e);
}

int64_t vp_batch_work_items(const vp_batch_plan* plan) { return plan ? plan->total : 0; }

int vp_batch_destroy(vp_batch_plan* plan) {
  if (plan == nullptr) return VP_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(plan->device);
  if (plan->d_descs) cudaFree(plan->d_descs);
  if (plan->d_counter) cudaFree(plan->d_counter);
  cudaSetDevice(prev);
  delete plan;
  return VP_OK;
}

}  // extern "C"
