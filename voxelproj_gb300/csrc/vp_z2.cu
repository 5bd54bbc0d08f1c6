// z_order 2 through the z_order 0 kernels.
//
// In z_order 2 the height axis is the slowest one: x (H, SY, SX) and
// y (H, n_ang, PX).  The projector's weights do not depend on the height,
// so the fast kernels put heights across the lanes of a warp; that needs
// heights contiguous.  For H >= 32 the z_order 2 operators therefore run as
//     transpose the input to height-fastest order  (HBM-bound tiled transpose)
//     z_order 0 kernel, storing (not accumulating) into scratch
//     transpose the result back, adding it to the caller's output
// which costs about 2 * (|x| + |y|) of extra HBM traffic, a fraction of a
// millisecond at 512^3 against several milliseconds of projector work, and
// keeps the reference's accumulate semantics.  Small H keeps the native
// z_order 2 kernels (lanes across x / PX).
//
// Scratch: SY*SX*Hp + n_ang*PX*Hp floats (Hp = H rounded up to 4), supplied by
// the caller (vp_*_z2_ws) or taken from a library-private stream-ordered pool.
#include <cuda_runtime.h>

#include <cstdint>

#include "vp_common.cuh"
#include "vp_launch.h"

namespace vp {

namespace {

constexpr int TT = 32;         // tile edge
constexpr int TROWS = 8;       // thread rows per tile (each thread moves TT/TROWS elements)
constexpr int KE = TT / TROWS;

// dst[c * dst_ld + r] (+)= src[r * src_ld + c] for r < rows, c < cols.
// Tiles are visited with a grid-stride loop so any matrix fits one launch.
// ADD: add into dst.  The adding form moves two neighbouring tiles per
// iteration and issues every load of them (the source rows into shared
// memory, the destination's current values into registers) before the first
// store: 16 loads in flight per thread.  With one element's read-add-write
// in turn it waited on each destination read (57% of the copy bandwidth
// against 65-68% for the storing form, which keeps one tile per iteration,
// 32 registers and 8 blocks per SM).
template <bool ADD>
__global__ void __launch_bounds__(TT * TROWS)
    transpose_kernel(const float* __restrict__ src, float* __restrict__ dst, long long rows,
                     long long cols, long long src_ld, long long dst_ld) {
  constexpr int TPI = ADD ? 2 : 1;  // tiles per iteration
  __shared__ float tile[TPI][TT][TT + 1];
  const long long tiles_c = (cols + TT - 1) / TT;
  const long long tiles_r = (rows + TT - 1) / TT;
  const long long ntiles = tiles_c * tiles_r;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (long long t0 = (long long)blockIdx.x * TPI; t0 < ntiles;
       t0 += (long long)gridDim.x * TPI) {
    float old[TPI][KE];
    (void)old;
#pragma unroll
    for (int j = 0; j < TPI; ++j) {
      const long long t = t0 + j;
      const long long r0 = (t / tiles_c) * TT;
      const long long c0 = (t % tiles_c) * TT;
      const bool tv = t < ntiles;
#pragma unroll
      for (int k = 0; k < KE; ++k) {
        const long long r = r0 + ty + k * TROWS;
        const long long c = c0 + tx;
        if (tv && r < rows && c < cols) tile[j][ty + k * TROWS][tx] = __ldg(src + r * src_ld + c);
      }
#pragma unroll
      for (int k = 0; k < KE; ++k) {
        const long long c = c0 + ty + k * TROWS;
        const long long r = r0 + tx;
        if constexpr (ADD) old[j][k] = (tv && r < rows && c < cols) ? dst[c * dst_ld + r] : 0.0f;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < TPI; ++j) {
      const long long t = t0 + j;
      const long long r0 = (t / tiles_c) * TT;
      const long long c0 = (t % tiles_c) * TT;
      const bool tv = t < ntiles;
#pragma unroll
      for (int k = 0; k < KE; ++k) {
        const long long c = c0 + ty + k * TROWS;
        const long long r = r0 + tx;
        if (tv && r < rows && c < cols) {
          const float v = tile[j][tx][ty + k * TROWS];
          if constexpr (ADD) dst[c * dst_ld + r] = old[j][k] + v;
          else dst[c * dst_ld + r] = v;
        }
      }
    }
    __syncthreads();  // the tiles are refilled next iteration
  }
}

cudaError_t transpose(const float* src, float* dst, long long rows, long long cols,
                      long long src_ld, long long dst_ld, int accumulate, cudaStream_t stream) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  const long long ntiles = ((rows + TT - 1) / TT) * ((cols + TT - 1) / TT);
  const long long iters = accumulate ? (ntiles + 1) / 2 : ntiles;
  // one resident wave of blocks (the tiles are dealt out by block index)
  int dev = 0, sms = 152, per_sm = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const void* fn = accumulate ? reinterpret_cast<const void*>(transpose_kernel<true>)
                              : reinterpret_cast<const void*>(transpose_kernel<false>);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, TT * TROWS, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  const long long cap = (long long)sms * per_sm;
  const unsigned grid = (unsigned)(iters < cap ? iters : cap);
  if (accumulate)
    transpose_kernel<true><<<grid, dim3(TT, TROWS), 0, stream>>>(src, dst, rows, cols, src_ld,
                                                                 dst_ld);
  else
    transpose_kernel<false><<<grid, dim3(TT, TROWS), 0, stream>>>(src, dst, rows, cols, src_ld,
                                                                  dst_ld);
  return cudaGetLastError();
}

inline long long round4(long long v) { return (v + 3) / 4 * 4; }

}  // namespace

bool z2_uses_transpose(const Geom& g) { return g.H >= 32; }

size_t z2_workspace_bytes(const Geom& g) {
  if (!z2_uses_transpose(g)) return 0;
  const long long Hp = round4(g.H);
  return (size_t)(((long long)g.SY * g.SX + (long long)g.n_ang * g.PX) * Hp) * sizeof(float);
}

int launches_z2(const Geom& g, bool forward) {
  if (!z2_uses_transpose(g)) return forward ? launches_forward_z2(g) : 1;
  // the transposed path runs the z_order 0 kernels on 16-byte aligned scratch
  // with a height extent that is a multiple of 4
  Geom g0 = g;
  g0.H = g0.Hx = g0.Hy = (int)round4(g.H);
  static const float aligned[4] = {};
  return 2 + (forward ? launches_forward_z0(aligned, aligned, g0)
                      : launches_backward_z0(aligned, aligned, g0));
}

// The first steps of the transposed form, into ws: the input to
// height-fastest order, then its z_order 0 projection (stored).
//   forward:  x (Hx, SY, SX) -> xt (SY, SX, Hp); yt = A xt
//   adjoint:  y (Hy, n, PX) -> yt (n, PX, Hp); xt = A^T yt
cudaError_t z2_project(bool forward, const float* in, const float* angles, const Geom& g,
                       float* ws, cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  const long long nbin = (long long)g.n_ang * g.PX;
  float* xt = ws;
  float* yt = ws + nvox * Hp;
  Geom g0 = g;
  g0.H = g0.Hx = g0.Hy = (int)Hp;
  g0.accumulate = 0;
  if (forward) {
    const cudaError_t e = transpose(in, xt, g.H, nvox, nvox, Hp, 0, stream);
    if (e != cudaSuccess) return e;
    return launch_forward_z0(xt, yt, angles, g0, stream);
  }
  const cudaError_t e = transpose(in, yt, g.H, nbin, nbin, Hp, 0, stream);
  if (e != cudaSuccess) return e;
  return launch_backward_z0(yt, xt, angles, g0, stream);
}

// The last step: out (+)= the projection in ws, back in heights-slowest
// order (add = 1 adds, 0 stores).
cudaError_t z2_transpose_out(bool forward, float* out, const Geom& g, const float* ws, int add,
                             cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  const long long nbin = (long long)g.n_ang * g.PX;
  if (forward) return transpose(ws + nvox * Hp, out, nbin, g.H, Hp, nbin, add, stream);
  return transpose(ws, out, nvox, g.H, Hp, nvox, add, stream);
}

// Volume rows [lo, hi) of a heights-slowest volume chunk in (g.H, SY, SX)
// into the transposed form's xt (SY, SX, Hp), stored.
cudaError_t z2_transpose_in_rows(const float* x, const Geom& g, float* ws, int lo, int hi,
                                 cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  return transpose(x + (long long)lo * g.SX, ws + (long long)lo * g.SX * Hp, g.H,
                   (long long)(hi - lo) * g.SX, nvox, Hp, 0, stream);
}

// Angles [a0, a1) of a heights-slowest sinogram in (g.H, n_ang, PX) into the
// transposed form's yt (n_ang, PX, Hp), stored.
cudaError_t z2_transpose_in_angles(const float* y, const Geom& g, float* ws, int a0, int a1,
                                   cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  const long long nbin = (long long)g.n_ang * g.PX;
  return transpose(y + (long long)a0 * g.PX, ws + nvox * Hp + (long long)a0 * g.PX * Hp, g.H,
                   (long long)(a1 - a0) * g.PX, nbin, Hp, 0, stream);
}

// Angles [a0, a1) of the forward's yt (n_ang, PX, Hp) in ws into a
// heights-slowest sinogram y (g.H, n_ang, PX): added (add = 1) or stored (0).
cudaError_t z2_transpose_out_angles(float* y, const Geom& g, const float* ws, int a0, int a1,
                                    int add, cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  const long long nbin = (long long)g.n_ang * g.PX;
  return transpose(ws + nvox * Hp + (long long)a0 * g.PX * Hp, y + (long long)a0 * g.PX,
                   (long long)(a1 - a0) * g.PX, g.H, Hp, nbin, add, stream);
}

// Volume rows [lo, hi) of the adjoint's xt (SY, SX, Hp) in ws into a
// heights-slowest chunk x (g.H, SY, SX): added (add = 1) or stored (0).
cudaError_t z2_transpose_out_rows(float* x, const Geom& g, const float* ws, int lo, int hi,
                                  int add, cudaStream_t stream) {
  const long long Hp = round4(g.H);
  const long long nvox = (long long)g.SY * g.SX;
  return transpose(ws + (long long)lo * g.SX * Hp, x + (long long)lo * g.SX,
                   (long long)(hi - lo) * g.SX, g.H, Hp, nvox, add, stream);
}

// x (Hx, SY, SX) -> xt (SY, SX, Hp); yt = A xt; y (Hy, n, PX) += yt^T.
cudaError_t forward_z2_transposed(const float* x, float* y, const float* angles, const Geom& g,
                                  float* ws, cudaStream_t stream) {
  const cudaError_t e = z2_project(true, x, angles, g, ws, stream);
  if (e != cudaSuccess) return e;
  return z2_transpose_out(true, y, g, ws, 1, stream);
}

// y (Hy, n, PX) -> yt (n, PX, Hp); xt = A^T yt; x (Hx, SY, SX) += xt^T.
cudaError_t backward_z2_transposed(const float* y, float* x, const float* angles, const Geom& g,
                                   float* ws, cudaStream_t stream) {
  const cudaError_t e = z2_project(false, y, angles, g, ws, stream);
  if (e != cudaSuccess) return e;
  return z2_transpose_out(false, x, g, ws, 1, stream);
}

}  // namespace vp
