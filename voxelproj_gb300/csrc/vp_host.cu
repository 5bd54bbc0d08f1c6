// Host-buffer projections: the caller's arrays stay in host memory, and the
// copies to and from the device overlap the kernels.  The z_order 0
// pipelines below are templates over how the arrays move; z_order 2 forwards
// use them with strided copies and device transposes (z2_host).
//
// Forward, y_host (+)= A x_host, on row slabs of the forward's plan:
//   copy stream:  angles, the volume's rows piece by piece (a quarter of a
//                 slab first, so that the kernels start early), then the y
//                 container
//   kernel streams (two chains, one per half of the angles, which write
//                 disjoint rows of y; one chain's last wave overlaps the
//                 other's next launch): angles whose minor axis is x, on each
//                 piece of rows as soon as it is in (the first launch in
//                 store mode into a fresh device y); once all rows are in, a
//                 4-height remainder of split heights (main stream), then
//                 the other angles on blocks of columns, the last block in
//                 groups of those angles
//   out stream:   once all rows are in, the angles whose minor axis is x
//                 beyond doubt (final then); later per group of the last
//                 column block, once final: y rows of those angles +=
//                 container, and back to the host
//
// Adjoint, x_host (+)= A^T y_host:
//   copy stream:  angles, the first sixth of the angles' sinogram rows,
//                 the rest, then the x container slab by slab
//   main stream:  the adjoint of the first angles over the whole volume as
//                 soon as they are in (store mode into a fresh device x),
//                 then the remaining angles in row slabs, alternating with a
//                 second kernel stream so that one slab's last wave overlaps
//                 the next slab
//   out stream:   per row slab, once computed: x rows += container rows
//                 (done by the slab's last kernel with the run kernels), and
//                 back to the host
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

#include <cmath>
#include <cstdint>
#include <mutex>
#include <vector>

#include "vp_common.cuh"
#include "vp_launch.h"

namespace vp {
namespace {

constexpr int kMaxDevices = 64;
constexpr int kAdjointSlabs = 12;     // adjoint row slabs per call
constexpr int kZ2AdjointSlabs = 8;    // row slabs of the z_order 2 adjoint's last chunk
constexpr int kForwardAngleGroups = 4;  // groups of the forward's last slab
// Forward angles sent home early: |phi| at most this many radians, and
// |cos phi| - |sin phi| at least this margin, far above the error of the
// kernels' single-precision sin/cos in that range.
constexpr double kEarlyMaxRad = 16.0;
constexpr double kEarlyMargin = 1e-3;

// Side streams and events of one device, created on first use and kept.
struct HostCtx {
  cudaStream_t copy_in = nullptr;
  cudaStream_t copy_out = nullptr;
  cudaStream_t compute2 = nullptr;  // a second kernel stream for independent slabs
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
    // the out stream's small add kernels must not wait behind the projection's
    // blocks: highest priority
    int least = 0, greatest = 0;
    if ((e = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess) return e;
    if ((e = cudaStreamCreateWithPriority(&c.copy_out, cudaStreamNonBlocking, greatest)) !=
        cudaSuccess)
      return e;
    if ((e = cudaStreamCreateWithFlags(&c.compute2, cudaStreamNonBlocking)) != cudaSuccess)
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
      cudaStreamSynchronize(g_ctx[dev].compute2);
    }
    cudaStreamSynchronize(s);
  }
  return e;
}

// How a host-buffer forward moves its arrays; forward_pipeline does the
// rest.  rows_in brings volume rows [lo, hi), every height, into the device's
// z_order 0 x (on the copy stream); container_in brings in the caller's y
// when adding; send puts the final angles [a0, a1) home (on the out stream),
// the container added first.
struct FwdZ0IO {  // z_order 0 host arrays: contiguous row and angle blocks
  // volume pieces of at most this many MB of one height chunk (1-D copies):
  // at 512^3 with 192 angles a call took 7.57 ms against 7.73 ms with 64 MB
  // pieces, 7.80 with 24 or 48 and 7.87 with 16
  static constexpr int piece_mb = 32;
  const float* x_host;
  float* y_host;
  const Geom& g;
  float* xd;
  float* yd;
  float* yc;
  size_t row_elems() const { return (size_t)g.SX * g.Hx; }
  size_t ang_elems() const { return (size_t)g.PX * g.Hy; }
  cudaError_t rows_in(int lo, int hi, cudaStream_t copy) const {
    const size_t off = (size_t)lo * row_elems();
    return cudaMemcpyAsync(xd + off, x_host + off, (size_t)(hi - lo) * row_elems() * sizeof(float),
                           cudaMemcpyDefault, copy);
  }
  cudaError_t container_in(cudaStream_t copy) const {
    if (!g.accumulate) return cudaSuccess;
    return cudaMemcpyAsync(yc, y_host, (size_t)g.n_ang * ang_elems() * sizeof(float),
                           cudaMemcpyDefault, copy);
  }
  cudaError_t send(int a0, int a1, cudaStream_t out, int* launches) const {
    const size_t off = (size_t)a0 * ang_elems(), n = (size_t)(a1 - a0) * ang_elems();
    if (g.accumulate) {
      VP_TRY(launch_add(yd + off, yc + off, n, out));
      *launches += 1;
    }
    return cudaMemcpyAsync(y_host + off, yd + off, n * sizeof(float), cudaMemcpyDefault, out);
  }
};

struct FwdZ2IO {  // z_order 2 host arrays: strided blocks, transposed on the device
  // pieces of at most 64 MB: smaller ones make more, narrower 2-D copies and
  // transposes (3321 against 3437 GVU/s end to end with 32 MB pieces)
  static constexpr int piece_mb = 64;
  const float* x_host;  // (H, SY, SX)
  float* y_host;        // (>= H, n_ang, PX): heights [0, H) are written
  const Geom& g2;       // the z_order 2 problem (its H heights)
  float* xs;            // staging of x, (H, SY, SX)
  float* ws;            // the transposed form's workspace: xt, then yt
  float* ys;            // staging of y, (H, n_ang, PX): the container, then the result
  int* launches;        // counts the transposes on the copy stream
  size_t vox() const { return (size_t)g2.SY * g2.SX; }
  size_t bins() const { return (size_t)g2.n_ang * g2.PX; }
  cudaError_t rows_in(int lo, int hi, cudaStream_t copy) const {
    VP_TRY(cudaMemcpy2DAsync(xs + (size_t)lo * g2.SX, vox() * sizeof(float),
                             x_host + (size_t)lo * g2.SX, vox() * sizeof(float),
                             (size_t)(hi - lo) * g2.SX * sizeof(float), g2.H, cudaMemcpyDefault,
                             copy));
    *launches += 1;
    return z2_transpose_in_rows(xs, g2, ws, lo, hi, copy);
  }
  cudaError_t container_in(cudaStream_t copy) const {
    if (!g2.accumulate) return cudaSuccess;
    return cudaMemcpyAsync(ys, y_host, (size_t)g2.H * bins() * sizeof(float),
                           cudaMemcpyDefault, copy);
  }
  cudaError_t send(int a0, int a1, cudaStream_t out, int* launches) const {
    VP_TRY(z2_transpose_out_angles(ys, g2, ws, a0, a1, g2.accumulate ? 1 : 0, out));
    *launches += 1;
    return cudaMemcpy2DAsync(y_host + (size_t)a0 * g2.PX, bins() * sizeof(float),
                             ys + (size_t)a0 * g2.PX, bins() * sizeof(float),
                             (size_t)(a1 - a0) * g2.PX * sizeof(float), g2.H,
                             cudaMemcpyDefault, out);
  }
};

// The forward's pipeline on device x (xd) and y (yd) in z_order 0 layout of
// geometry g; io moves the host arrays.  Called under g_mutex.
template <class IO>
cudaError_t forward_pipeline(const IO& io, const float* angles, const Geom& g, float* xd,
                             float* yd, float* as, const float* ad, cudaStream_t s,
                             int* launches) {
  const size_t y_elems = (size_t)g.n_ang * g.PX * g.Hy;
  // row pieces: a quarter slab, the rest of the first slab, then whole
  // slabs of the plan (which depends on the device buffers' alignment);
  // column pieces of the plan
  const int rows = forward_z0_stream_rows(xd, yd, g, IO::piece_mb);
  const int cols = forward_z0_stream_cols(xd, yd, g, IO::piece_mb);
  std::vector<int> cut{0};
  const int quarter = rows / 4 >= 8 ? rows / 4 : rows;
  int r = quarter < g.SY ? quarter : g.SY;
  cut.push_back(r);
  if (r < g.SY && r < rows) {  // the rest of the first slab
    r = rows < g.SY ? rows : g.SY;
    cut.push_back(r);
  }
  while (r < g.SY) {
    r = r + rows < g.SY ? r + rows : g.SY;
    cut.push_back(r);
  }
  std::vector<int> ccut{0};
  for (int q = 0; q < g.SX;) {
    q = q + cols < g.SX ? q + cols : g.SX;
    ccut.push_back(q);
  }
  const int npieces = (int)cut.size() - 1;
  const int ncpieces = (int)ccut.size() - 1;
  // two independent chains of launches, one per half of the angles (they
  // write disjoint rows of y), on the two kernel streams: each chain's last
  // wave overlaps the other chain's next launch
  const int nhalves = g.n_ang >= 2 ? 2 : 1;
  const int ah[3] = {0, nhalves == 2 ? g.n_ang / 2 : g.n_ang, g.n_ang};
  // Angles whose minor axis is x beyond doubt are final once every row
  // piece and the remainder heights have run, so they go back while the
  // column blocks run; the others go back in groups of the last column
  // block.  The kernels classify with single-precision sin/cos, within far
  // less than the margin of double precision here.
  std::vector<char> early(g.n_ang, 0);
  if (!is_device_pointer(angles)) {
    for (int a = 0; a < g.n_ang; ++a) {
      const double phi = angles[a];
      if (std::fabs(phi) <= kEarlyMaxRad)
        early[a] = std::fabs(std::cos(phi)) - std::fabs(std::sin(phi)) >= kEarlyMargin;
    }
  }
  std::vector<int> late[2];
  for (int h = 0; h < nhalves; ++h)
    for (int a = ah[h]; a < ah[h + 1]; ++a)
      if (!early[a]) late[h].push_back(a);
  // output groups of the last column block, per half
  const int per_half = kForwardAngleGroups / 2;
  int ng[2] = {0, 0};
  for (int h = 0; h < nhalves; ++h)
    ng[h] = (int)late[h].size() < per_half ? (int)late[h].size() : per_half;
  HostCtx* c = nullptr;
  VP_TRY(get_ctx(npieces + ng[0] + ng[1] + 7, &c));
  cudaEvent_t ev_alloc = c->ev[0], ev_cont = c->ev[1], ev_out = c->ev[2], ev_c2 = c->ev[3],
              ev_rest = c->ev[4], ev_rows1 = c->ev[5], ev_c2end = c->ev[6];
  cudaEvent_t* ev_piece = c->ev.data() + 7;
  cudaEvent_t* ev_group = ev_piece + npieces;

  // the side streams start after the allocations (and prior work) on s
  VP_TRY(cudaEventRecord(ev_alloc, s));
  VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_alloc, 0));
  VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_alloc, 0));
  VP_TRY(copy_angles(as, angles, g, c->copy_in));
  for (int k = 0; k < npieces; ++k) {
    VP_TRY(io.rows_in(cut[k], cut[k + 1], c->copy_in));
    VP_TRY(cudaEventRecord(ev_piece[k], c->copy_in));
  }
  VP_TRY(io.container_in(c->copy_in));
  VP_TRY(cudaEventRecord(ev_cont, c->copy_in));
  VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_cont, 0));

  // angles [a0, a1) are final: add the container and send them home
  auto send = [&](int a0, int a1) -> cudaError_t {
    return io.send(a0, a1, c->copy_out, launches);
  };

  Geom gs = g;
  gs.accumulate = 0;
  if (g.H < g.Hy) {  // heights past x's extent are not written: start from zero
    VP_TRY(cudaMemsetAsync(yd, 0, y_elems * sizeof(float), s));
    gs.accumulate = 1;
  }
  const cudaStream_t st[2] = {s, c->compute2};
  VP_TRY(cudaEventRecord(ev_c2, s));
  VP_TRY(cudaStreamWaitEvent(c->compute2, ev_c2, 0));
  // angles whose minor axis is x, on each piece of rows as it arrives (the
  // first piece in the caller's mode writes every angle of its half)
  for (int k = 0; k < npieces; ++k)
    for (int h = 0; h < nhalves; ++h) {
      VP_TRY(cudaStreamWaitEvent(st[h], ev_piece[k], 0));
      VP_TRY(launch_forward_z0_stream(xd, yd, ad, gs, cut[k], cut[k + 1], 0, 0, ah[h],
                                      ah[h + 1], k == 0 ? gs.accumulate : 1, st[h],
                                      launches));
    }
  VP_TRY(cudaEventRecord(ev_rows1, c->compute2));
  // every row is in: the remainder heights (other heights than the chains
  // write), then the early angles go home
  VP_TRY(launch_forward_z0_rest(xd, yd, ad, gs, s, launches));
  VP_TRY(cudaEventRecord(ev_rest, s));
  VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_rest, 0));
  VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_rows1, 0));
  for (int a = 0; a < g.n_ang;) {
    if (!early[a]) {
      ++a;
      continue;
    }
    int e = a;
    while (e < g.n_ang && early[e]) ++e;
    VP_TRY(send(a, e));
    a = e;
  }
  // the other angles on blocks of columns
  for (int j = 0; j + 1 < ncpieces; ++j)
    for (int h = 0; h < nhalves; ++h)
      VP_TRY(launch_forward_z0_stream(xd, yd, ad, gs, 0, 0, ccut[j], ccut[j + 1], ah[h],
                                      ah[h + 1], 1, st[h], launches));
  // the last block by groups of the late angles (equal counts), each group
  // sent home once final (and once the remainder heights, on s, are
  // written)
  VP_TRY(cudaStreamWaitEvent(c->compute2, ev_rest, 0));
  int gi = 0;
  for (int j = 0; j < per_half; ++j)
    for (int h = 0; h < nhalves; ++h) {
      if (j >= ng[h]) continue;
      const int m = (int)late[h].size();
      const int i0 = (int)((long long)m * j / ng[h]);
      const int i1 = (int)((long long)m * (j + 1) / ng[h]);
      VP_TRY(launch_forward_z0_stream(xd, yd, ad, gs, 0, 0, ccut[ncpieces - 1],
                                      ccut[ncpieces], late[h][i0], late[h][i1 - 1] + 1, 1,
                                      st[h], launches));
      VP_TRY(cudaEventRecord(ev_group[gi], st[h]));
      VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_group[gi], 0));
      ++gi;
      for (int i = i0; i < i1;) {  // runs of consecutive late angles
        int e = i + 1;
        while (e < i1 && late[h][e] == late[h][e - 1] + 1) ++e;
        VP_TRY(send(late[h][i], late[h][e - 1] + 1));
        i = e;
      }
    }
  // s ends after the last angles are home and compute2's work is done
  VP_TRY(cudaEventRecord(ev_c2end, c->compute2));
  VP_TRY(cudaStreamWaitEvent(s, ev_c2end, 0));
  VP_TRY(cudaEventRecord(ev_out, c->copy_out));
  return cudaStreamWaitEvent(s, ev_out, 0);
}

// How a host-buffer adjoint moves its arrays; backward_pipeline does the
// rest.  angles_in brings the sinogram of angles [a0, a1) into the device's
// z_order 0 y (on the copy stream); container_rows_in brings the caller's x
// rows [lo, hi) when adding; addend is the container on the device if the
// kernels can add it themselves (else null); send_rows puts the final rows
// home (on the out stream), adding the container first unless done.
struct BwdZ0IO {  // z_order 0 host arrays: contiguous row and angle blocks
  const float* y_host;
  float* x_host;
  const Geom& g;
  float* yd;
  float* xd;
  float* xc;
  size_t row_elems() const { return (size_t)g.SX * g.Hx; }
  size_t ang_elems() const { return (size_t)g.PX * g.Hy; }
  cudaError_t angles_in(int a0, int a1, cudaStream_t copy) const {
    const size_t off = (size_t)a0 * ang_elems();
    return cudaMemcpyAsync(yd + off, y_host + off, (size_t)(a1 - a0) * ang_elems() * sizeof(float),
                           cudaMemcpyDefault, copy);
  }
  cudaError_t container_rows_in(int lo, int hi, cudaStream_t copy) const {
    if (!g.accumulate) return cudaSuccess;
    const size_t off = (size_t)lo * row_elems();
    return cudaMemcpyAsync(xc + off, x_host + off, (size_t)(hi - lo) * row_elems() * sizeof(float),
                           cudaMemcpyDefault, copy);
  }
  const float* addend() const { return g.accumulate ? xc : nullptr; }
  cudaError_t send_rows(int lo, int hi, bool added, cudaStream_t out, int* launches) const {
    const size_t off = (size_t)lo * row_elems(), n = (size_t)(hi - lo) * row_elems();
    if (g.accumulate && !added) {
      VP_TRY(launch_add(xd + off, xc + off, n, out));
      *launches += 1;
    }
    return cudaMemcpyAsync(x_host + off, xd + off, n * sizeof(float), cudaMemcpyDefault, out);
  }
};

// The adjoint's pipeline on device y (yd) and x (xd) in z_order 0 layout of
// geometry g; io moves the host arrays.  Called under g_mutex.
template <class IO>
cudaError_t backward_pipeline(const IO& io, const float* angles, const Geom& g, float* yd,
                              float* xd, float* as, const float* ad, cudaStream_t s,
                              int* launches) {
  const size_t ang_elems = (size_t)g.PX * g.Hy;
  const size_t x_elems = (size_t)g.SY * g.SX * g.Hx;
  // rows per slab: a multiple of the adjoint's row step, about SY / kAdjointSlabs
  const int step = backward_z0_row_step(yd, xd, g);
  int rows = g.SY;
  if (step > 0) {
    rows = (g.SY + kAdjointSlabs - 1) / kAdjointSlabs;
    rows = (rows + step - 1) / step * step;
  }
  const int nslabs = (g.SY + rows - 1) / rows;
  // the first sixth of the angles runs over the whole volume first, while
  // the rest of the sinogram arrives (at 512^3 with 192 angles, 12 slabs
  // and a sixth measured 6.22 ms per call; 16 and an eighth 6.37 ms; 8 and
  // a quarter 6.72 ms)
  const int a_split = g.n_ang >= 8 ? g.n_ang / 6 : 0;
  HostCtx* c = nullptr;
  VP_TRY(get_ctx(2 * nslabs + 6, &c));
  cudaEvent_t ev_alloc = c->ev[0], ev_in0 = c->ev[1], ev_in = c->ev[2], ev_out = c->ev[3],
              ev_first = c->ev[4], ev_c2 = c->ev[5];
  cudaEvent_t* ev_rows = c->ev.data() + 6;
  cudaEvent_t* ev_cont = ev_rows + nslabs;  // container rows of slab k are in

  VP_TRY(cudaEventRecord(ev_alloc, s));
  VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_alloc, 0));
  VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_alloc, 0));
  VP_TRY(copy_angles(as, angles, g, c->copy_in));
  const size_t y0 = (size_t)a_split * ang_elems;
  if (a_split > 0) VP_TRY(io.angles_in(0, a_split, c->copy_in));
  VP_TRY(cudaEventRecord(ev_in0, c->copy_in));
  VP_TRY(io.angles_in(a_split, g.n_ang, c->copy_in));
  VP_TRY(cudaEventRecord(ev_in, c->copy_in));
  // the container slab by slab, in the order the results leave
  for (int k = 0; k < nslabs; ++k) {
    const int lo = k * rows;
    const int hi = lo + rows < g.SY ? lo + rows : g.SY;
    VP_TRY(io.container_rows_in(lo, hi, c->copy_in));
    VP_TRY(cudaEventRecord(ev_cont[k], c->copy_in));
  }

  Geom gs = g;
  gs.accumulate = 0;
  if (g.H < g.Hx) {  // heights past y's extent are not written: start from zero
    VP_TRY(cudaMemsetAsync(xd, 0, x_elems * sizeof(float), s));
    gs.accumulate = 1;
  }
  // angles [0, a_split) over all rows; then angles [a_split, n) by row slabs
  Geom g1 = gs;
  if (a_split > 0) {
    Geom g0 = gs;
    g0.n_ang = a_split;
    VP_TRY(cudaStreamWaitEvent(s, ev_in0, 0));
    VP_TRY(launch_backward_z0_rows(yd, xd, ad, g0, 0, g.SY, s));
    *launches += launches_backward_z0(yd, xd, g0);
    g1.n_ang = g.n_ang - a_split;
    g1.accumulate = 1;
  }
  VP_TRY(cudaStreamWaitEvent(s, ev_in, 0));
  VP_TRY(cudaEventRecord(ev_first, s));  // y is in and the first angles are launched
  VP_TRY(cudaStreamWaitEvent(c->compute2, ev_first, 0));
  // the run kernels add the container's rows themselves, in the slab's last
  // launch (the same sums, in the same order, as a separate add)
  const float* addend = io.addend();
  const bool fused_add = addend != nullptr && backward_z0_rows_can_add(yd + y0, xd, g1);
  for (int k = 0; k < nslabs; ++k) {
    const int lo = k * rows;
    const int hi = lo + rows < g.SY ? lo + rows : g.SY;
    const cudaStream_t sk = (k & 1) ? c->compute2 : s;  // slabs write disjoint rows
    if (fused_add) {
      // the slab's class-1 launch adds the container rows: only it waits
      // for them, the class-0 launch starts as soon as the sinogram is in
      VP_TRY(launch_backward_z0_rows_add(yd + y0, xd, ad + a_split, g1, lo, hi, addend, sk,
                                         ev_cont[k]));
    } else {
      VP_TRY(launch_backward_z0_rows(yd + y0, xd, ad + a_split, g1, lo, hi, sk));
    }
    *launches += launches_backward_z0(yd, xd, g1);
    VP_TRY(cudaEventRecord(ev_rows[k], sk));
    // rows [lo, hi) are final: (add the container's rows and) send them back
    VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_rows[k], 0));
    VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_cont[k], 0));
    VP_TRY(io.send_rows(lo, hi, fused_add, c->copy_out, launches));
  }
  VP_TRY(cudaEventRecord(ev_c2, c->compute2));
  VP_TRY(cudaStreamWaitEvent(s, ev_c2, 0));
  VP_TRY(cudaEventRecord(ev_out, c->copy_out));
  return cudaStreamWaitEvent(s, ev_out, 0);  // s ends after the last row is home
}

}  // namespace

cudaError_t forward_z0_host(const float* x_host, float* y_host, const float* angles,
                            const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const size_t x_elems = (size_t)g.SY * g.SX * g.Hx;
  const size_t y_elems = (size_t)g.n_ang * g.PX * g.Hy;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *xd = nullptr, *yd = nullptr, *yc = nullptr, *as = nullptr;
    const float* ad = nullptr;
    VP_TRY(buf.get(pool, x_elems * sizeof(float), &xd));
    VP_TRY(buf.get(pool, y_elems * sizeof(float), &yd));
    if (g.accumulate) VP_TRY(buf.get(pool, y_elems * sizeof(float), &yc));
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    const FwdZ0IO io{x_host, y_host, g, xd, yd, yc};
    return forward_pipeline(io, angles, g, xd, yd, as, ad, s, launches);
  }, s);
}

cudaError_t backward_z0_host(const float* y_host, float* x_host, const float* angles,
                             const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches) {
  std::lock_guard<std::mutex> lock(g_mutex);
  const size_t x_elems = (size_t)g.SY * g.SX * g.Hx;
  const size_t y_elems = (size_t)g.n_ang * g.PX * g.Hy;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *xd = nullptr, *yd = nullptr, *xc = nullptr, *as = nullptr;
    const float* ad = nullptr;
    VP_TRY(buf.get(pool, y_elems * sizeof(float), &yd));
    VP_TRY(buf.get(pool, x_elems * sizeof(float), &xd));
    if (g.accumulate) VP_TRY(buf.get(pool, x_elems * sizeof(float), &xc));
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    const BwdZ0IO io{y_host, x_host, g, yd, xd, xc};
    return backward_pipeline(io, angles, g, yd, xd, as, ad, s, launches);
  }, s);
}

// The z_order 2 adjoint with host arrays, by chunks of heights, whose
// sinogram and volume blocks are contiguous: chunks of 256 heights (the
// 8-heights-per-lane kernels' chunk) from 512 heights up, else halves.  With
// the transposed path (32 heights and more):
//   copy stream:  the chunks' sinograms in order, each container after the
//                 next chunk's sinogram (a projection needs only its input)
//   kernel streams (alternating by chunk, one projection at a time): the
//                 sinogram to height-fastest order and the z_order 0 adjoint
//                 into the workspace; the last chunk by row slabs
//   out stream:   per chunk, once projected and its container is in, the
//                 transpose-add into the container and the copy home; the
//                 last chunk slab by slab, so that most of it is home when
//                 the kernels end
// Small heights run the native z_order 2 kernel per chunk on one stream.
// Called under g_mutex.
cudaError_t z2_backward_chunked(const float* y_host, float* x_host, const float* angles,
                                const Geom& g, cudaMemPool_t pool, cudaStream_t s,
                                int* launches) {
  const size_t vox = (size_t)g.SY * g.SX, bins = (size_t)g.n_ang * g.PX;
  const int H = g.H;
  int Hc = H;
  if (H >= 512) Hc = 256;
  else if (H > 64) Hc = ((H + 1) / 2 + 3) / 4 * 4;
  const int nchunks = (H + Hc - 1) / Hc;
  Geom gc = g;  // a full chunk
  gc.H = gc.Hx = gc.Hy = Hc;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *in_d[2] = {}, *out_d[2] = {}, *ws[2] = {}, *as = nullptr;
    const float* ad = nullptr;
    const bool pipelined = z2_uses_transpose(gc);
    const size_t ws_elems = z2_workspace_bytes(gc) / sizeof(float);
    const int slots = nchunks > 1 ? 2 : 1;
    for (int i = 0; i < slots; ++i) {
      VP_TRY(buf.get(pool, (size_t)Hc * bins * sizeof(float), &in_d[i]));
      VP_TRY(buf.get(pool, (size_t)Hc * vox * sizeof(float), &out_d[i]));
      if (ws_elems > 0) VP_TRY(buf.get(pool, ws_elems * sizeof(float), &ws[i]));
    }
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    auto chunk = [&](int k) {
      Geom gk = g;
      const int h0 = k * Hc;
      gk.H = gk.Hx = gk.Hy = h0 + Hc <= H ? Hc : H - h0;
      gk.accumulate = 1;
      return gk;
    };
    // row slabs of the last chunk
    std::vector<int> scut{0};
    if (pipelined) {
      Geom gl = chunk(nchunks - 1);
      gl.H = gl.Hx = gl.Hy = (int)(((size_t)gl.H + 3) / 4 * 4);
      const float* xtl = ws[(nchunks - 1) & 1];
      const int step = backward_z0_row_step(xtl + vox * gl.H, xtl, gl);
      int rows = g.SY;
      if (step > 0) {
        rows = (g.SY + kZ2AdjointSlabs - 1) / kZ2AdjointSlabs;
        rows = (rows + step - 1) / step * step;
      }
      for (int q = 0; q < g.SY;) {
        q = q + rows < g.SY ? q + rows : g.SY;
        scut.push_back(q);
      }
    }
    const int nslabs = (int)scut.size() - 1;
    HostCtx* c = nullptr;
    VP_TRY(get_ctx(4 * nchunks + 3 + nslabs, &c));
    cudaEvent_t ev_ready = c->ev[0], ev_c2 = c->ev[1], ev_out = c->ev[2];
    cudaEvent_t* ev_in = c->ev.data() + 3;      // chunk k's sinogram is in
    cudaEvent_t* ev_kern = ev_in + nchunks;     // chunk k's projection is in ws
    cudaEvent_t* ev_cont = ev_kern + nchunks;   // chunk k's container is in
    cudaEvent_t* ev_done = ev_cont + nchunks;   // chunk k is home
    cudaEvent_t* ev_slab = ev_done + nchunks;   // row slab r of the last chunk is computed
    VP_TRY(copy_angles(as, angles, g, s));
    VP_TRY(cudaEventRecord(ev_ready, s));  // buffers allocated, angles in
    VP_TRY(cudaStreamWaitEvent(c->compute2, ev_ready, 0));
    const cudaStream_t st[2] = {s, c->compute2};
    if (!pipelined) {
      for (int k = 0; k < nchunks; ++k) {
        const cudaStream_t t = st[k & 1];
        const Geom gk = chunk(k);
        const size_t h0 = (size_t)k * Hc, hc = (size_t)gk.H;
        VP_TRY(cudaMemcpyAsync(in_d[k & 1], y_host + h0 * bins, hc * bins * sizeof(float),
                               cudaMemcpyDefault, t));
        if (g.accumulate)
          VP_TRY(cudaMemcpyAsync(out_d[k & 1], x_host + h0 * vox, hc * vox * sizeof(float),
                                 cudaMemcpyDefault, t));
        else
          VP_TRY(cudaMemsetAsync(out_d[k & 1], 0, hc * vox * sizeof(float), t));
        VP_TRY(launch_backward_z2(in_d[k & 1], out_d[k & 1], ad, gk, t));
        *launches += launches_z2(gk, false);
        VP_TRY(cudaMemcpyAsync(x_host + h0 * vox, out_d[k & 1], hc * vox * sizeof(float),
                               cudaMemcpyDefault, t));
      }
    } else {
      VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_ready, 0));
      VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_ready, 0));
      const bool slabs_out = nslabs > 1;
      auto issue_cont = [&](int j) -> cudaError_t {
        if (!g.accumulate) return cudaSuccess;
        if (j >= 2) VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_done[j - 2], 0));  // slot free
        const size_t h0 = (size_t)j * Hc, hc = (size_t)chunk(j).H;
        VP_TRY(cudaMemcpyAsync(out_d[j & 1], x_host + h0 * vox, hc * vox * sizeof(float),
                               cudaMemcpyDefault, c->copy_in));
        return cudaEventRecord(ev_cont[j], c->copy_in);
      };
      auto issue_out = [&](int j) -> cudaError_t {
        const Geom gj = chunk(j);
        const size_t h0 = (size_t)j * Hc, hc = (size_t)gj.H;
        float* dst = out_d[j & 1];  // the container's chunk, or stored into
        if (g.accumulate) VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_cont[j], 0));
        if (slabs_out && j == nchunks - 1) {
          for (int r = 0; r < nslabs; ++r) {
            const int lo = scut[r], hi = scut[r + 1];
            VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_slab[r], 0));
            VP_TRY(z2_transpose_out_rows(dst, gj, ws[j & 1], lo, hi, g.accumulate ? 1 : 0,
                                         c->copy_out));
            *launches += 1;
            VP_TRY(cudaMemcpy2DAsync(x_host + h0 * vox + (size_t)lo * g.SX, vox * sizeof(float),
                                     dst + (size_t)lo * g.SX, vox * sizeof(float),
                                     (size_t)(hi - lo) * g.SX * sizeof(float), hc,
                                     cudaMemcpyDefault, c->copy_out));
          }
          return cudaEventRecord(ev_done[j], c->copy_out);
        }
        VP_TRY(cudaStreamWaitEvent(c->copy_out, ev_kern[j], 0));
        VP_TRY(z2_transpose_out(false, dst, gj, ws[j & 1], g.accumulate ? 1 : 0, c->copy_out));
        VP_TRY(cudaMemcpyAsync(x_host + h0 * vox, dst, hc * vox * sizeof(float),
                               cudaMemcpyDefault, c->copy_out));
        return cudaEventRecord(ev_done[j], c->copy_out);
      };
      for (int k = 0; k < nchunks; ++k) {
        const cudaStream_t t = st[k & 1];
        const Geom gk = chunk(k);
        const size_t h0 = (size_t)k * Hc, hc = (size_t)gk.H;
        // the sinogram slot is free once chunk k - 2 is home (its projection
        // read it)
        if (k >= 2) VP_TRY(cudaStreamWaitEvent(c->copy_in, ev_done[k - 2], 0));
        VP_TRY(cudaMemcpyAsync(in_d[k & 1], y_host + h0 * bins, hc * bins * sizeof(float),
                               cudaMemcpyDefault, c->copy_in));
        VP_TRY(cudaEventRecord(ev_in[k], c->copy_in));
        VP_TRY(cudaStreamWaitEvent(t, ev_in[k], 0));
        if (k >= 1) VP_TRY(cudaStreamWaitEvent(t, ev_kern[k - 1], 0));  // one at a time
        if (k >= 2) VP_TRY(cudaStreamWaitEvent(t, ev_done[k - 2], 0));  // workspace free
        if (slabs_out && k == nchunks - 1) {
          // by row slabs, each handed to the out stream once computed
          Geom gl = gk;
          gl.H = gl.Hx = gl.Hy = (int)(((size_t)gk.H + 3) / 4 * 4);
          gl.accumulate = 0;
          float* xtl = ws[k & 1];
          float* ytl = ws[k & 1] + vox * gl.H;
          VP_TRY(z2_transpose_in_angles(in_d[k & 1], gk, ws[k & 1], 0, g.n_ang, t));
          *launches += 1;  // the transposes back are counted per slab
          for (int r = 0; r < nslabs; ++r) {
            VP_TRY(launch_backward_z0_rows(ytl, xtl, ad, gl, scut[r], scut[r + 1], t));
            *launches += launches_backward_z0(ytl, xtl, gl);
            VP_TRY(cudaEventRecord(ev_slab[r], t));
          }
        } else {
          VP_TRY(z2_project(false, in_d[k & 1], ad, gk, ws[k & 1], t));
          *launches += launches_z2(gk, false);
        }
        VP_TRY(cudaEventRecord(ev_kern[k], t));
        if (k >= 1) {
          VP_TRY(issue_cont(k - 1));
          VP_TRY(issue_out(k - 1));
        }
      }
      VP_TRY(issue_cont(nchunks - 1));
      VP_TRY(issue_out(nchunks - 1));
      VP_TRY(cudaEventRecord(ev_out, c->copy_out));
      VP_TRY(cudaStreamWaitEvent(s, ev_out, 0));
    }
    if (!g.accumulate && g.Hx > H) {
      // heights of the output past the input's extent: zero (out = result)
      float* z = nullptr;
      const size_t n = (size_t)(g.Hx - H) * vox;
      VP_TRY(buf.get(pool, n * sizeof(float), &z));
      VP_TRY(cudaMemsetAsync(z, 0, n * sizeof(float), s));
      VP_TRY(cudaMemcpyAsync(x_host + (size_t)H * vox, z, n * sizeof(float), cudaMemcpyDefault,
                             s));
    }
    VP_TRY(cudaEventRecord(ev_c2, c->compute2));
    return cudaStreamWaitEvent(s, ev_c2, 0);  // s ends after both streams' chunks
  }, s);
}

// z_order 2 with host arrays.  The forward, from 32 heights up, runs the
// z_order 0 pipeline above on the transposed form's workspace: the volume
// rows and sinogram angles it moves are strided in z_order 2, so they travel
// as 2-D copies into heights-slowest staging buffers, transposed on the
// device (rows in) or transposed, added to the container and copied home
// (angles out).  Below 32 heights the native z_order 2 kernels run on one
// stream: copy in, project into the container (or zeros), copy home.  The
// adjoint runs by chunks of heights (z2_backward_chunked), whose sinogram
// and volume blocks are contiguous: in the z_order 0 pipeline its first
// angles and its row slabs would be 2-D copies of rows narrow enough (64 and
// 90 KB) to run at well under the link's speed.
cudaError_t z2_host(bool forward, const float* in_host, float* out_host, const float* angles,
                    const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches) {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!forward) return z2_backward_chunked(in_host, out_host, angles, g, pool, s, launches);
  const float* x_host = in_host;
  float* y_host = out_host;
  const size_t vox = (size_t)g.SY * g.SX, bins = (size_t)g.n_ang * g.PX;
  const int H = g.H;
  Buffers buf(s);
  return guarded([&]() -> cudaError_t {
    float *xs = nullptr, *ys = nullptr, *ws = nullptr, *as = nullptr;
    const float* ad = nullptr;
    VP_TRY(buf.get(pool, (size_t)H * vox * sizeof(float), &xs));
    VP_TRY(buf.get(pool, (size_t)H * bins * sizeof(float), &ys));
    VP_TRY(alloc_angles(angles, g, buf, pool, &ad, &as));
    Geom g2 = g;  // the heights computed, contiguous in the staging buffers
    g2.Hx = g2.Hy = H;
    if (z2_uses_transpose(g2)) {
      VP_TRY(buf.get(pool, z2_workspace_bytes(g2), &ws));
      // the z_order 0 view of the workspace (padding heights are computed
      // and never copied back)
      Geom gv = g2;
      gv.H = gv.Hx = gv.Hy = (H + 3) / 4 * 4;
      const FwdZ2IO io{x_host, y_host, g2, xs, ws, ys, launches};
      VP_TRY(forward_pipeline(io, angles, gv, ws, ws + vox * (size_t)gv.H, as, ad, s, launches));
    } else {
      VP_TRY(copy_angles(as, angles, g, s));
      VP_TRY(cudaMemcpyAsync(xs, x_host, (size_t)H * vox * sizeof(float), cudaMemcpyDefault, s));
      Geom gk = g2;
      gk.accumulate = 1;  // into the container, or zeros
      if (g.accumulate)
        VP_TRY(cudaMemcpyAsync(ys, y_host, (size_t)H * bins * sizeof(float), cudaMemcpyDefault,
                               s));
      else
        VP_TRY(cudaMemsetAsync(ys, 0, (size_t)H * bins * sizeof(float), s));
      VP_TRY(launch_forward_z2(xs, ys, ad, gk, s));
      *launches += launches_z2(gk, true);
      VP_TRY(cudaMemcpyAsync(y_host, ys, (size_t)H * bins * sizeof(float), cudaMemcpyDefault, s));
    }
    if (!g.accumulate && g.Hy > H) {
      // heights of the output past the input's extent: zero (out = result)
      float* z = nullptr;
      const size_t n = (size_t)(g.Hy - H) * bins;
      VP_TRY(buf.get(pool, n * sizeof(float), &z));
      VP_TRY(cudaMemsetAsync(z, 0, n * sizeof(float), s));
      VP_TRY(cudaMemcpyAsync(y_host + (size_t)H * bins, z, n * sizeof(float), cudaMemcpyDefault,
                             s));
    }
    return cudaSuccess;
  }, s);
}

}  // namespace vp
