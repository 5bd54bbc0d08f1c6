// Host-buffer projections (z_order 0): the caller's arrays stay in host
// memory, and the copies to and from the device overlap the kernels.
//
// Forward, y_host (+)= A x_host:
//   copy stream:  angles, x rows of slab 0, slab 1, ..., then the y container
//   main stream:  slab k of the row-slab forward as soon as its rows are in
//                 (slab 0 in store mode into a fresh device y), the heights
//                 of a 4-height remainder once all rows are in, then y += the
//                 container, then y back to the host
// The volume arrives while earlier slabs project, and the container while
// the projection runs; only the first slab's rows and the result's way back
// are exposed.
//
// Adjoint, x_host (+)= A^T y_host:
//   copy stream:  angles, y, then the x container
//   main stream:  the adjoint of voxel rows [r_k, r_k+1) per slab, in store
//                 mode into a fresh device x
//   out stream:   per slab, once computed: x rows += container rows, rows back
// The result leaves the device while later rows are still being computed.
//
// Device buffers come from the library's stream-ordered pool, so repeated
// calls reuse memory without going back to the driver.  Copies use
// cudaMemcpyDefault: page-locked host buffers give asynchronous copies that
// overlap; pageable ones are still correct, with less overlap.  The call is
// asynchronous on `stream`: the host result is complete once the stream is.
//
// No counterpart in the reference, whose wrappers copy the whole input to
// the device, project, and copy the whole result back, one after another
// (voxelproj/wrappers.py:10-25 and :57-73).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "vp_common.cuh"
#include "vp_launch.h"

namespace vp {
namespace {

constexpr int kMaxDevices = 64;
// Adjoint slabs: about this many rows of output each (and at least RUN).
constexpr int kAdjointSlabs = 8;

// Side streams and events of one device, created on first use and kept.
struct HostCtx {
  cudaStream_t copy_in = nullptr;
  cudaStream_t copy_out = nullptr;
  std::vector<cudaEvent_t> ev;
};
std::mutex g_mutex;  // one host-buffer call per process at a time
HostCtx g_ctx[kMaxDevices];

cudaError_t get_ctx(int nev, HostCtx** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  HostCtx& c = g_ctx[dev];
  if (c.copy_in == nullptr) {
    if ((e = cudaStreamCreateWithFlags(&c.copy_in, cudaStreamNonBlocking)) != cudaSuccess)
      return e;
    if ((e = cudaStreamCreateWithFlags(&c.copy_out, cudaStreamNonBlocking)) != cudaSuccess)
      return e;
  }
  while ((int)c.ev.size() < nev) {
    cudaEvent_t ev;
    if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    c.ev.push_back(ev);
  }
  *out = &c;
  return cudaSuccess;
}

// dst[i] += src[i], i < n.
__global__ void add_kernel(float* __restrict__ dst, const float* __restrict__ src, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
    const size_t n4 = n / 4;
    float4* d4 = reinterpret_cast<float4*>(dst);
    const float4* s4 = reinterpret_cast<const float4*>(src);
    for (size_t j = i; j < n4; j += stride) d4[j] = f4_add(d4[j], s4[j]);
    for (size_t j = 4 * n4 + i; j < n; j += stride) dst[j] += src[j];
  } else {
    for (size_t j = i; j < n; j += stride) dst[j] += src[j];
  }
}

cudaError_t launch_add(float* dst, const float* src, size_t n, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  size_t blocks = (n / 4 + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  add_kernel<<<(unsigned)blocks, 256, 0, s>>>(dst, src, n);
  return cudaGetLastError();
}

// Stream-ordered buffers of one call, freed (stream-ordered) on destruction.
struct Buffers {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit Buffers(cudaStream_t s_) : s(s_) {}
  cudaError_t get(cudaMemPool_t pool, size_t bytes, float** out) {
    void* p = nullptr;
    const cudaError_t e = cudaMallocFromPoolAsync(&p, bytes > 0 ? bytes : 16, pool, s);
    if (e != cudaSuccess) return e;
    ptrs.push_back(p);
    *out = static_cast<float*>(p);
    return cudaSuccess;
  }
  ~Buffers() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
};

bool is_device_pointer(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

#define VP_TRY(expr)                         \
  do {                                       \
    const cudaError_t e_ = (expr);           \
    if (e_ != cudaSuccess) return e_;        \
  } while (0)

// Angles on the device: the caller's pointer if it is device memory, else a
// buffer (allocated here, filled by copy_angles on the copy stream).
cudaError_t alloc_angles(const float* angles, const Geom& g, Buffers& buf, cudaMemPool_t pool,
                         const float** out, float** staged) {
  *staged = nullptr;
  if (is_device_pointer(angles)) {
    *out = angles;
    return cudaSuccess;
  }
  VP_TRY(buf.get(pool, (size_t)g.n_ang * sizeof(float), staged));
  *out = *staged;
  return cudaSuccess;
}

cudaError_t copy_angles(float* staged, const float* angles, const Geom& g, cudaStream_t copy) {
  if (staged == nullptr) return cudaSuccess;
  return cudaMemcpyAsync(staged, angles, (size_t)g.n_ang * sizeof(float), cudaMemcpyDefault,
                         copy);
}

// Runs body(); after an error, waits for the side streams so that the
// buffers, freed on s when `buf` goes, are no longer in use.
template <class F>
cudaError_t guarded(F body, cudaStream_t s) {
  const cudaError_t e = body();
  if (e != cudaSuccess) {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices &&
        g_ctx[dev].copy_in != nullptr) {
      cudaStreamSynchronize(g_ctx[dev].copy_in);
      cudaStreamSynchronize(g_ctx[dev].copy_out);
    }
    cudaStreamSynchronize(s);
  }
  return e;
}

}  // namespace

cudaError_t forward_z0_host(const float* x_host, float* y_host, const float* angles,
                            const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const size_t row_elems = (size_t)g.SX * g.Hx;
  const size_t x_elems = (size_t)g.SY * row_elems;
  const size_t y_elems = (size_t)g.n_ang * g.PX * g.Hy;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *xd = nullptr, *yd = nullptr, *yc = nullptr, *as = nullptr;
    const float* ad = nullptr;
    VP_TRY(buf.get(pool, x_elems * sizeof(float), &xd));
    VP_TRY(buf.get(pool, y_elems * sizeof(float), &yd));
    if (g.accumulate) VP_TRY(buf.get(pool, y_elems * sizeof(float), &yc));
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    // the slab plan depends on the device buffers' alignment, which is 16 bytes
    const int nslabs = forward_z0_row_slabs(xd, yd, g);
    HostCtx* c = nullptr;
    VP_TRY(get_ctx(nslabs + 2, &c));
    cudaEvent_t ev_alloc = c->ev[0], ev_cont = c->ev[1];
    cudaEvent_t* ev_slab = c->ev.data() + 2;

    // the copy stream starts after the allocations (and prior work) on s
    VP_TRY(cudaEventRecord(ev_alloc, s));
    VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_alloc, 0));
    VP_TRY(copy_angles(as, angles, g, c->copy_in));
    for (int k = 0; k < nslabs; ++k) {
      int lo = 0, hi = 0;
      forward_z0_row_slab(xd, yd, g, k, &lo, &hi);
      if (hi > lo)
        VP_TRY(cudaMemcpyAsync(xd + (size_t)lo * row_elems, x_host + (size_t)lo * row_elems,
                               (size_t)(hi - lo) * row_elems * sizeof(float),
                               cudaMemcpyDefault, c->copy_in));
      VP_TRY(cudaEventRecord(ev_slab[k], c->copy_in));
    }
    if (g.accumulate)
      VP_TRY(cudaMemcpyAsync(yc, y_host, y_elems * sizeof(float), cudaMemcpyDefault,
                             c->copy_in));
    VP_TRY(cudaEventRecord(ev_cont, c->copy_in));

    Geom gs = g;
    gs.accumulate = 0;
    if (g.H < g.Hy) {  // heights past x's extent are not written: start from zero
      VP_TRY(cudaMemsetAsync(yd, 0, y_elems * sizeof(float), s));
      gs.accumulate = 1;
    }
    for (int k = 0; k < nslabs; ++k) {
      VP_TRY(cudaStreamWaitEvent(s, ev_slab[k], 0));
      VP_TRY(launch_forward_z0_row_slab(xd, yd, ad, gs, k, s));
      *launches += forward_z0_row_slab_launches(xd, yd, g);
    }
    VP_TRY(launch_forward_z0_row_rest(xd, yd, ad, gs, s, launches));
    VP_TRY(cudaStreamWaitEvent(s, ev_cont, 0));
    if (g.accumulate) {
      VP_TRY(launch_add(yd, yc, y_elems, s));
      *launches += 1;
    }
    return cudaMemcpyAsync(y_host, yd, y_elems * sizeof(float), cudaMemcpyDefault, s);
  }, s);
}

cudaError_t backward_z0_host(const float* y_host, float* x_host, const float* angles,
                             const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const size_t row_elems = (size_t)g.SX * g.Hx;
  const size_t x_elems = (size_t)g.SY * row_elems;
  const size_t y_elems = (size_t)g.n_ang * g.PX * g.Hy;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *xd = nullptr, *yd = nullptr, *xc = nullptr, *as = nullptr;
    const float* ad = nullptr;
    VP_TRY(buf.get(pool, y_elems * sizeof(float), &yd));
    VP_TRY(buf.get(pool, x_elems * sizeof(float), &xd));
    if (g.accumulate) VP_TRY(buf.get(pool, x_elems * sizeof(float), &xc));
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    // rows per slab: a multiple of the adjoint's row step, about SY / kAdjointSlabs
    const int step = backward_z0_row_step(yd, xd, g);
    int rows = g.SY;
    if (step > 0) {
      rows = (g.SY + kAdjointSlabs - 1) / kAdjointSlabs;
      rows = (rows + step - 1) / step * step;
    }
    const int nslabs = (g.SY + rows - 1) / rows;
    HostCtx* c = nullptr;
    VP_TRY(get_ctx(nslabs + 4, &c));
    cudaEvent_t ev_alloc = c->ev[0], ev_in = c->ev[1], ev_cont = c->ev[2], ev_out = c->ev[3];
    cudaEvent_t* ev_rows = c->ev.data() + 4;

    VP_TRY(cudaEventRecord(ev_alloc, s));
    VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_alloc, 0));
    VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_alloc, 0));
    VP_TRY(copy_angles(as, angles, g, c->copy_in));
    VP_TRY(cudaMemcpyAsync(yd, y_host, y_elems * sizeof(float), cudaMemcpyDefault, c->copy_in));
    VP_TRY(cudaEventRecord(ev_in, c->copy_in));
    if (g.accumulate)
      VP_TRY(cudaMemcpyAsync(xc, x_host, x_elems * sizeof(float), cudaMemcpyDefault,
                             c->copy_in));
    VP_TRY(cudaEventRecord(ev_cont, c->copy_in));

    Geom gs = g;
    gs.accumulate = 0;
    if (g.H < g.Hx) {  // heights past y's extent are not written: start from zero
      VP_TRY(cudaMemsetAsync(xd, 0, x_elems * sizeof(float), s));
      gs.accumulate = 1;
    }
    VP_TRY(cudaStreamWaitEvent(s, ev_in, 0));
    VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_cont, 0));
    for (int k = 0; k < nslabs; ++k) {
      const int lo = k * rows;
      const int hi = lo + rows < g.SY ? lo + rows : g.SY;
      VP_TRY(launch_backward_z0_rows(yd, xd, ad, gs, lo, hi, s));
      *launches += launches_backward_z0(yd, xd, g);
      VP_TRY(cudaEventRecord(ev_rows[k], s));
      // rows [lo, hi) are final: add the container's rows and send them back
      VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_rows[k], 0));
      const size_t off = (size_t)lo * row_elems, n = (size_t)(hi - lo) * row_elems;
      if (g.accumulate) {
        VP_TRY(launch_add(xd + off, xc + off, n, c->copy_out));
        *launches += 1;
      }
      VP_TRY(cudaMemcpyAsync(x_host + off, xd + off, n * sizeof(float), cudaMemcpyDefault,
                             c->copy_out));
    }
    VP_TRY(cudaEventRecord(ev_out, c->copy_out));
    return cudaStreamWaitEvent(s, ev_out, 0);  // s ends after the last row is home
  }, s);
}

}  // namespace vp
