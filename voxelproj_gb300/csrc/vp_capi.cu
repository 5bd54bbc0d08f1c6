// C ABI: argument validation, geometry setup and dispatch to the kernels.
// The reference's host launchers (voxelproj/csrc/projectors.cu:34-299) also
// copied the input into a cudaArray and bound a texture on every call; none
// of that exists here, so a call is validation plus one kernel launch.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>

#include "../../include/voxelproj_gb300.h"
#include "vp_common.cuh"
#include "vp_launch.h"

namespace {

thread_local int g_last_cuda_error = 0;
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_variant[vp::OP_COUNT] = {};

constexpr int64_t kMaxDim = (int64_t)1 << 30;
// fp_z0 packs the voxel index (yi*SX + xi) with 4 tag bits into an int.
constexpr int64_t kMaxVoxelsPerSlice = (int64_t)1 << 27;

int check_flags(int flags) { return (flags & ~VP_FLAG_TRIG_PRECISE) ? VP_ERR_BAD_FLAGS : VP_OK; }

bool dims_ok(int64_t a, int64_t b, int64_t c) {
  return a >= 0 && b >= 0 && c >= 0 && a < kMaxDim && b < kMaxDim && c < kMaxDim;
}

// Builds the geometry from x's (SY, SX, Hx) and y's (n_ang, PX, Hy) and
// validates pointers and the angle count.  Sets *empty when there is no work.
int make_geom(const void* xp, int64_t SY, int64_t SX, int64_t Hx, const void* yp, int64_t n_ang,
              int64_t PX, int64_t Hy, const float* angles, int64_t n_angles, int flags,
              vp::Geom* g, bool* empty) {
  if (int s = check_flags(flags)) return s;
  if (!dims_ok(SY, SX, Hx) || !dims_ok(n_ang, PX, Hy)) return VP_ERR_BAD_SHAPE;
  if (SY * SX >= kMaxVoxelsPerSlice) return VP_ERR_BAD_SHAPE;
  if (n_angles < 0) return VP_ERR_ANGLES;
  const int64_t H = Hx < Hy ? Hx : Hy;
  *empty = (SY == 0 || SX == 0 || n_ang == 0 || PX == 0 || H == 0);
  if (n_ang > 0 && n_angles < n_ang) return VP_ERR_ANGLES;
  if ((SY * SX * Hx > 0 && xp == nullptr) || (n_ang * PX * Hy > 0 && yp == nullptr) ||
      (n_ang > 0 && angles == nullptr))
    return VP_ERR_NULL_POINTER;
  g->SY = (int)SY;
  g->SX = (int)SX;
  g->n_ang = (int)n_ang;
  g->PX = (int)PX;
  g->H = (int)H;
  g->Hx = (int)Hx;
  g->Hy = (int)Hy;
  g->xcent = 0.5f * (float)(SX - 1);
  g->ycent = 0.5f * (float)(SY - 1);
  g->pcent = 0.5f * (float)(PX - 1);
  g->trig = (flags & VP_FLAG_TRIG_PRECISE) ? vp::TRIG_PRECISE : vp::TRIG_REF;
  g->accumulate = 1;
  return VP_OK;
}

// Library-private stream-ordered pool for z_order 2 scratch when the caller
// supplies none; it keeps freed memory (release threshold = max) so repeated
// calls do not go back to the driver.
constexpr int kMaxDevices = 64;
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[kMaxDevices] = {};

cudaError_t private_pool(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  if (g_pools[dev] == nullptr) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}

int finish(cudaError_t e, int launches) {
  g_launches.fetch_add((uint64_t)launches, std::memory_order_relaxed);
  if (e != cudaSuccess) {
    g_last_cuda_error = (int)e;
    return VP_ERR_CUDA;
  }
  return VP_OK;
}

}  // namespace

namespace vp {
int record_cuda_error(cudaError_t e) {
  g_last_cuda_error = (int)e;
  return VP_ERR_CUDA;
}

void count_launches(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

int kernel_variant(int op) {
  return (op >= 0 && op < OP_COUNT) ? g_variant[op].load(std::memory_order_relaxed) : 0;
}
}  // namespace vp

// Host-buffer entry points (vp_host.cu).  VP_FLAG_OVERWRITE is accepted here
// only.  An empty problem in overwrite mode still zeroes the output.
namespace {

cudaError_t zero_any(float* out, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  cudaMemPool_t pool;
  cudaError_t e = private_pool(&pool);
  if (e != cudaSuccess) return e;
  void* z = nullptr;
  const size_t bytes = (size_t)n * sizeof(float);
  if ((e = cudaMallocFromPoolAsync(&z, bytes, pool, s)) != cudaSuccess) return e;
  e = cudaMemsetAsync(z, 0, bytes, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, z, bytes, cudaMemcpyDefault, s);
  const cudaError_t f = cudaFreeAsync(z, s);
  return e != cudaSuccess ? e : f;
}

// x and y dims in the caller's order; z2: heights first (x (Hx, SY, SX),
// y (Hy, n_ang, PX)), else last.
template <class Run>
int host_entry(bool z2, const float* x, int64_t x0, int64_t x1, int64_t x2, const float* y,
               int64_t y0, int64_t y1, int64_t y2, float* out, int64_t out_elems,
               const float* angles, int64_t n_angles, int flags, void* stream, Run run) {
  const bool overwrite = (flags & VP_FLAG_OVERWRITE) != 0;
  vp::Geom g;
  bool empty = false;
  const int f = flags & ~VP_FLAG_OVERWRITE;
  if (int s = z2 ? make_geom(x, x1, x2, x0, y, y1, y2, y0, angles, n_angles, f, &g, &empty)
                 : make_geom(x, x0, x1, x2, y, y0, y1, y2, angles, n_angles, f, &g, &empty))
    return s;
  const cudaStream_t st = (cudaStream_t)stream;
  if (empty) return overwrite ? finish(zero_any(out, out_elems, st), 0) : VP_OK;
  g.accumulate = overwrite ? 0 : 1;
  cudaMemPool_t pool;
  cudaError_t e = private_pool(&pool);
  int launches = 0;
  if (e == cudaSuccess) e = run(g, pool, st, &launches);
  return finish(e, launches);
}

}  // namespace

extern "C" {

int vp_set_kernel_variant(int op, int variant) {
  if (op < 0 || op >= vp::OP_COUNT || variant < 0 || variant > 64) return VP_ERR_BAD_FLAGS;
  g_variant[op].store(variant, std::memory_order_relaxed);
  return VP_OK;
}

int vp_get_kernel_variant(int op) { return vp::kernel_variant(op); }


int vp_version(void) { return 100; }

const char* vp_error_string(int status) {
  switch (status) {
    case VP_OK: return "ok";
    case VP_ERR_NULL_POINTER: return "null pointer for a non-empty array";
    case VP_ERR_BAD_SHAPE: return "invalid array shape";
    case VP_ERR_ANGLES: return "fewer angles than the angle extent of the sinogram";
    case VP_ERR_CUDA: return "CUDA runtime error";
    case VP_ERR_BAD_FLAGS: return "unknown flag bits";
    case VP_ERR_BAD_Z_ORDER: return "z_order must be 0 or 2";
    case VP_ERR_WORKSPACE: return "workspace smaller than vp_z2_workspace_bytes()";
    case VP_ERR_BATCH:
      return "unsupported batch problem (z_order 0 with heights in multiples of 4 and "
             "16-byte aligned buffers, op VP_OP_FORWARD or VP_OP_BACKWARD)";
    case VP_ERR_SCRATCH_LIMIT:
      return "problem needs more scratch than the library's static array holds "
             "(VP_NOALLOC_SCRATCH_BYTES); use vp_forward_z2 or vp_forward_z2_ws";
    default: return "unknown status";
  }
}

int vp_last_cuda_error(void) { return g_last_cuda_error; }

uint64_t vp_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

uint64_t vp_wait_timeouts(void) { return vp::wait_timeouts(); }

int vp_set_wait_limits(uint32_t copy_polls, uint32_t stage_spins, uint32_t stage_extra) {
  vp::set_copy_wait_polls(copy_polls, copy_polls == VP_WAIT_DEFAULT);
  vp::set_stage_wait_limits(stage_spins, stage_extra);
  return VP_OK;
}

int vp_forward_z0(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y, int64_t y0,
                  int64_t y1, int64_t y2, const float* angles, int64_t n_angles, int flags,
                  void* stream) {
  vp::Geom g;
  bool empty = false;
  if (int s = make_geom(x, x0, x1, x2, y, y0, y1, y2, angles, n_angles, flags, &g, &empty))
    return s;
  if (empty) return VP_OK;
  return finish(vp::launch_forward_z0(x, y, angles, g, (cudaStream_t)stream),
                vp::launches_forward_z0(x, y, g));
}

int vp_backward_z0(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x, int64_t x0,
                   int64_t x1, int64_t x2, const float* angles, int64_t n_angles, int flags,
                   void* stream) {
  vp::Geom g;
  bool empty = false;
  if (int s = make_geom(x, x0, x1, x2, y, y0, y1, y2, angles, n_angles, flags, &g, &empty))
    return s;
  if (empty) return VP_OK;
  return finish(vp::launch_backward_z0(y, x, angles, g, (cudaStream_t)stream),
                vp::launches_backward_z0(y, x, g));
}

int vp_forward_z0_host(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y, int64_t y0,
                       int64_t y1, int64_t y2, const float* angles, int64_t n_angles, int flags,
                       void* stream) {
  return host_entry(false, x, x0, x1, x2, y, y0, y1, y2, y, y0 * y1 * y2, angles, n_angles,
                    flags, stream,
                    [&](const vp::Geom& g, cudaMemPool_t pool, cudaStream_t s, int* n) {
                      return vp::forward_z0_host(x, y, angles, g, pool, s, n);
                    });
}

int vp_backward_z0_host(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x, int64_t x0,
                        int64_t x1, int64_t x2, const float* angles, int64_t n_angles, int flags,
                        void* stream) {
  return host_entry(false, x, x0, x1, x2, y, y0, y1, y2, x, x0 * x1 * x2, angles, n_angles,
                    flags, stream,
                    [&](const vp::Geom& g, cudaMemPool_t pool, cudaStream_t s, int* n) {
                      return vp::backward_z0_host(y, x, angles, g, pool, s, n);
                    });
}

int vp_forward_z2_host(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y, int64_t y0,
                       int64_t y1, int64_t y2, const float* angles, int64_t n_angles, int flags,
                       void* stream) {
  return host_entry(true, x, x0, x1, x2, y, y0, y1, y2, y, y0 * y1 * y2, angles, n_angles,
                    flags, stream,
                    [&](const vp::Geom& g, cudaMemPool_t pool, cudaStream_t s, int* n) {
                      return vp::z2_host(true, x, y, angles, g, pool, s, n);
                    });
}

int vp_backward_z2_host(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x, int64_t x0,
                        int64_t x1, int64_t x2, const float* angles, int64_t n_angles, int flags,
                        void* stream) {
  return host_entry(true, x, x0, x1, x2, y, y0, y1, y2, x, x0 * x1 * x2, angles, n_angles,
                    flags, stream,
                    [&](const vp::Geom& g, cudaMemPool_t pool, cudaStream_t s, int* n) {
                      return vp::z2_host(false, y, x, angles, g, pool, s, n);
                    });
}

size_t vp_z2_workspace_bytes(int64_t x0, int64_t x1, int64_t x2, int64_t y0, int64_t y1,
                             int64_t y2) {
  vp::Geom g;
  bool empty = false;
  const float one = 0.f;
  // shapes only: dummy non-null pointers, all angles assumed present
  if (make_geom(&one, x1, x2, x0, &one, y1, y2, y0, &one, y1, 0, &g, &empty) != VP_OK || empty)
    return 0;
  return vp::z2_workspace_bytes(g);
}

}  // extern "C"

namespace {

// z_order 2 dispatch shared by the entry points with and without workspace.
int run_z2(bool forward, const float* in, float* out, const float* angles, const vp::Geom& g,
           void* ws, size_t ws_bytes, cudaStream_t stream) {
  if (!vp::z2_uses_transpose(g)) {
    cudaError_t e = forward ? vp::launch_forward_z2(in, out, angles, g, stream)
                            : vp::launch_backward_z2(in, out, angles, g, stream);
    return finish(e, vp::launches_z2(g, forward));
  }
  const size_t need = vp::z2_workspace_bytes(g);
  bool owned = false;
  if (ws == nullptr) {
    cudaMemPool_t pool;
    cudaError_t e = private_pool(&pool);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&ws, need, pool, stream);
    if (e != cudaSuccess) return finish(e, 0);
    owned = true;
  } else if (ws_bytes < need) {
    return VP_ERR_WORKSPACE;
  }
  cudaError_t e = forward
      ? vp::forward_z2_transposed(in, out, angles, g, static_cast<float*>(ws), stream)
      : vp::backward_z2_transposed(in, out, angles, g, static_cast<float*>(ws), stream);
  if (owned) {
    const cudaError_t f = cudaFreeAsync(ws, stream);
    if (e == cudaSuccess) e = f;
  }
  return finish(e, vp::launches_z2(g, forward));
}

}  // namespace

extern "C" {

int vp_forward_z2_ws(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y, int64_t y0,
                     int64_t y1, int64_t y2, const float* angles, int64_t n_angles, int flags,
                     void* workspace, size_t workspace_bytes, void* stream) {
  vp::Geom g;
  bool empty = false;
  // z_order 2: x (Hx, SY, SX), y (Hy, n_ang, PX)
  if (int s = make_geom(x, x1, x2, x0, y, y1, y2, y0, angles, n_angles, flags, &g, &empty))
    return s;
  if (empty) return VP_OK;
  return run_z2(true, x, y, angles, g, workspace, workspace_bytes, (cudaStream_t)stream);
}

int vp_backward_z2_ws(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x, int64_t x0,
                      int64_t x1, int64_t x2, const float* angles, int64_t n_angles, int flags,
                      void* workspace, size_t workspace_bytes, void* stream) {
  vp::Geom g;
  bool empty = false;
  if (int s = make_geom(x, x1, x2, x0, y, y1, y2, y0, angles, n_angles, flags, &g, &empty))
    return s;
  if (empty) return VP_OK;
  return run_z2(false, y, x, angles, g, workspace, workspace_bytes, (cudaStream_t)stream);
}

int vp_forward_z2(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y, int64_t y0,
                  int64_t y1, int64_t y2, const float* angles, int64_t n_angles, int flags,
                  void* stream) {
  return vp_forward_z2_ws(x, x0, x1, x2, y, y0, y1, y2, angles, n_angles, flags, nullptr, 0,
                          stream);
}

int vp_backward_z2(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x, int64_t x0,
                   int64_t x1, int64_t x2, const float* angles, int64_t n_angles, int flags,
                   void* stream) {
  return vp_backward_z2_ws(y, y0, y1, y2, x, x0, x1, x2, angles, n_angles, flags, nullptr, 0,
                           stream);
}

int vp_forward(const float* x, const int64_t x_dims[3], float* y, const int64_t y_dims[3],
               const float* angles, int64_t n_angles, int z_order, int flags, void* stream) {
  if (x_dims == nullptr || y_dims == nullptr) return VP_ERR_NULL_POINTER;
  if (z_order == 0)
    return vp_forward_z0(x, x_dims[0], x_dims[1], x_dims[2], y, y_dims[0], y_dims[1], y_dims[2],
                         angles, n_angles, flags, stream);
  if (z_order == 2)
    return vp_forward_z2(x, x_dims[0], x_dims[1], x_dims[2], y, y_dims[0], y_dims[1], y_dims[2],
                         angles, n_angles, flags, stream);
  return VP_ERR_BAD_Z_ORDER;
}

int vp_backward(const float* y, const int64_t y_dims[3], float* x, const int64_t x_dims[3],
                const float* angles, int64_t n_angles, int z_order, int flags, void* stream) {
  if (x_dims == nullptr || y_dims == nullptr) return VP_ERR_NULL_POINTER;
  if (z_order == 0)
    return vp_backward_z0(y, y_dims[0], y_dims[1], y_dims[2], x, x_dims[0], x_dims[1], x_dims[2],
                          angles, n_angles, flags, stream);
  if (z_order == 2)
    return vp_backward_z2(y, y_dims[0], y_dims[1], y_dims[2], x, x_dims[0], x_dims[1], x_dims[2],
                          angles, n_angles, flags, stream);
  return VP_ERR_BAD_Z_ORDER;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Forward projection in z_order 2 without any device allocation.
//
// Some callers may not allocate device memory once they are running: code
// that must not allocate after start-up (a real-time acquisition loop, a
// service with a fixed memory plan), or a host framework that owns all device
// memory through its own allocator and forbids outside cudaMalloc.
// vp_forward_z2 needs scratch for its transposed path and takes it from a
// pool; this entry point instead uses a fixed array compiled into the library.
//
// The array, g_noalloc_scratch, is a file-scope __device__ array of
// VP_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU that loads this library's
// code holds it until the process exits.  Host code cannot use the symbol
// itself as a device address (on the host it names a shadow object), so the
// first call on each device looks up the array's device address with
// cudaGetSymbolAddress, with that device current, and caches it.  Make that
// first call before any stream capture.
//
// All calls on a device share the array, and it keeps whatever the previous
// call left.  Nothing in this path reads scratch before writing it: the
// input is transposed into the array, the projector stores (not adds) its
// result there, and only those values are copied back.  Pad heights up to a
// multiple of 4 carry leftovers, but they are never copied out.  Two calls
// that overlap on the GPU (different streams, no ordering between them) race
// on the array and corrupt each other's results.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocScratchFloats = VP_NOALLOC_SCRATCH_BYTES / sizeof(float);
static __device__ __align__(256) float g_noalloc_scratch[kNoallocScratchFloats];

std::mutex g_noalloc_mutex;
float* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
cudaError_t noalloc_scratch(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_addr[dev] == nullptr) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[dev] = static_cast<float*>(ptr);
  }
  *out = g_noalloc_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int vp_forward_z2_noalloc(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y,
                                     int64_t y0, int64_t y1, int64_t y2, const float* angles,
                                     int64_t n_angles, int flags, void* stream) {
  vp::Geom g;
  bool empty = false;
  if (int s = make_geom(x, x1, x2, x0, y, y1, y2, y0, angles, n_angles, flags, &g, &empty))
    return s;
  if (empty) return VP_OK;
  const size_t need = vp::z2_workspace_bytes(g);
  if (need > VP_NOALLOC_SCRATCH_BYTES) return VP_ERR_SCRATCH_LIMIT;
  float* scratch = nullptr;
  if (need > 0) {
    const cudaError_t e = noalloc_scratch(&scratch);
    if (e != cudaSuccess) return finish(e, 0);
  }
  return run_z2(true, x, y, angles, g, scratch, VP_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
