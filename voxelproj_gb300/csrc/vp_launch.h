// Internal launch interface between the C-ABI layer (vp_capi.cu) and the
// kernel translation units.  Every launcher enqueues on `stream`, never
// synchronises, and returns the launch status.
#pragma once

#include <cuda_runtime.h>

#include "vp_common.cuh"

namespace vp {

// Launches kernel k; with programmatic set, with programmatic stream
// serialization, so that it may start while the kernel before it in the
// stream still runs (the kernel must run PdlWait, vp_common.cuh, before it
// reads back outputs that kernel writes).  Set only on a launch that directly
// follows one of this library's own kernels in the same call: the kernel
// before may then be running, but every operation before that one is done.
template <typename... KArgs, typename... Args>
cudaError_t launch_ex(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                      cudaStream_t stream, bool programmatic, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  if (programmatic) {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// y (z_order 0: (n_ang, PX, Hy), z_order 2: (Hy, n_ang, PX)) += A x.
cudaError_t launch_forward_z0(const float* x, float* y, const float* angles, const Geom& g,
                              cudaStream_t stream);
cudaError_t launch_forward_z2(const float* x, float* y, const float* angles, const Geom& g,
                              cudaStream_t stream);
// x (z_order 0: (SY, SX, Hx), z_order 2: (Hx, SY, SX)) += A^T y.
cudaError_t launch_backward_z0(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream);
cudaError_t launch_backward_z2(const float* y, float* x, const float* angles, const Geom& g,
                               cudaStream_t stream);

// Status bookkeeping shared by the C entry points (vp_capi.cu): records a
// CUDA error for vp_last_cuda_error() and returns VP_ERR_CUDA; counts launches
// for vp_launch_count().
int record_cuda_error(cudaError_t e);
void count_launches(int n);

// Kernel variant selection (0 = automatic), set through vp_set_kernel_variant.
enum Op : int { OP_FORWARD_Z0 = 0, OP_BACKWARD_Z0 = 1, OP_FORWARD_Z2 = 2, OP_BACKWARD_Z2 = 3,
                OP_COUNT = 4 };
int kernel_variant(int op);

// z_order 2 through the z_order 0 kernels (vp_z2.cu).
bool z2_uses_transpose(const Geom& g);
size_t z2_workspace_bytes(const Geom& g);
int launches_z2(const Geom& g, bool forward);
cudaError_t forward_z2_transposed(const float* x, float* y, const float* angles, const Geom& g,
                                  float* ws, cudaStream_t stream);
cudaError_t backward_z2_transposed(const float* y, float* x, const float* angles, const Geom& g,
                                   float* ws, cudaStream_t stream);
// The two halves of the transposed form: z2_project puts the input in
// height-fastest order and stores its z_order 0 projection, both in ws;
// z2_transpose_out adds (add = 1) or stores (0) that projection into the
// caller's heights-slowest output.
cudaError_t z2_project(bool forward, const float* in, const float* angles, const Geom& g,
                       float* ws, cudaStream_t stream);
cudaError_t z2_transpose_out(bool forward, float* out, const Geom& g, const float* ws, int add,
                             cudaStream_t stream);
// Row ranges of the same: volume rows [lo, hi) of a (g.H, SY, SX) chunk into
// the forward's height-fastest workspace (stored), and of the adjoint's
// workspace result back into a (g.H, SY, SX) chunk (add = 1 adds, 0 stores).
// The workspace's z_order 0 views are xt = ws, yt = ws + SY*SX*Hp (Hp = g.H
// rounded up to 4).
cudaError_t z2_transpose_in_rows(const float* x, const Geom& g, float* ws, int lo, int hi,
                                 cudaStream_t stream);
cudaError_t z2_transpose_out_rows(float* x, const Geom& g, const float* ws, int lo, int hi,
                                  int add, cudaStream_t stream);
// Angle ranges likewise: angles [a0, a1) of a (g.H, n_ang, PX) sinogram into
// the adjoint's workspace (stored), and of the forward's workspace result
// back into a (g.H, n_ang, PX) sinogram (add = 1 adds, 0 stores).
cudaError_t z2_transpose_in_angles(const float* y, const Geom& g, float* ws, int a0, int a1,
                                   cudaStream_t stream);
cudaError_t z2_transpose_out_angles(float* y, const Geom& g, const float* ws, int a0, int a1,
                                    int add, cudaStream_t stream);

// Height split of the 8-heights-per-lane forms: heights [0, r8_heights(H))
// run with 8 per lane (chunks of 256); a last chunk of at most 128 heights
// runs with 4 per lane instead, since 8 would leave half of it idle.
inline int r8_heights(int H) {
  const int full = H / 256 * 256;
  return (H - full > 128 || full == 0) ? H : full;
}

// Forward launch plan of a kernel variant (0 = default) for a geometry:
// heights per lane R, bins per warp KW, candidates in flight un, block on
// neighbouring angles, class slabs, and nslabs slabs of wy rows (and wx
// columns for class slabs; slab k as detail::slab_of).  The batched kernel
// follows the same plan, so its results equal the single-problem kernel's.
struct Fp0Plan {
  int R, KW, un;
  bool agroup, cls, split, staged;
  int nslabs, wy, wx;
};
Fp0Plan forward_z0_plan(const Geom& g, bool vec4, int variant);

// Streamed forms for host buffers.
// Forward, on the main height part: launch_forward_z0_stream gathers angles
// [a_lo, a_hi) from volume rows [rows_lo, rows_hi) for angles whose minor
// axis is x and from columns [cols_lo, cols_hi) for the others (an empty
// range skips that class when adding).  Rows in pieces of up to
// forward_z0_stream_rows (columns empty) as they arrive, then columns in
// pieces of up to forward_z0_stream_cols (rows empty), the first launch in
// the caller's mode and the rest adding, then launch_forward_z0_rest (the
// 4-height remainder of a split heights range, whole), give the full result.
// Adjoint: voxel rows [row_lo, row_hi) alone, row_lo a multiple of
// backward_z0_row_step() (0: rows cannot be split, launch [0, SY) only).
// Pieces hold at most piece_mb MB of one height chunk (and no more than the
// forward plan's slabs).
int forward_z0_stream_rows(const float* x, const float* y, const Geom& g, int piece_mb);
int forward_z0_stream_cols(const float* x, const float* y, const Geom& g, int piece_mb);
cudaError_t launch_forward_z0_stream(const float* x, float* y, const float* angles,
                                     const Geom& g, int rows_lo, int rows_hi, int cols_lo,
                                     int cols_hi, int a_lo, int a_hi, int accumulate,
                                     cudaStream_t stream, int* launches);
cudaError_t launch_forward_z0_rest(const float* x, float* y, const float* angles,
                                   const Geom& g, cudaStream_t stream, int* launches);
int backward_z0_row_step(const float* y, const float* x, const Geom& g);
// Bounded waits in this library's kernels that ran out (synchronising read).
unsigned long long wait_timeouts();
// Limits of the bounded waits for launches enqueued from now on
// (vp_set_wait_limits): polls of a bulk copy's barrier in the staged adjoint
// (the default with use_default), and a batch stage's sleeps (0: default) and
// extra completions waited for (0 in operation).
void set_copy_wait_polls(unsigned polls, bool use_default);
void set_stage_wait_limits(unsigned spins, unsigned extra);
// The current limit of copy waits, and the device address (current device)
// of the counter vp_wait_timeouts reads, for kernels of other units.
unsigned copy_wait_polls();
cudaError_t wait_timeout_counter(unsigned long long** out);
cudaError_t launch_backward_z0_rows(const float* y, float* x, const float* angles,
                                    const Geom& g, int row_lo, int row_hi,
                                    cudaStream_t stream);
// As launch_backward_z0_rows, and then adds addend (same layout as x) into
// those rows: x = (x + A^T y) + addend in adding mode, A^T y + addend in
// store mode, in the same order as a separate add after the projection.
// Only for the run variants (backward_z0_rows_can_add).  addend_ready (may
// be null): an event recorded once addend is in; the launches that read it
// wait for it, the ones before them do not.
bool backward_z0_rows_can_add(const float* y, const float* x, const Geom& g);
cudaError_t launch_backward_z0_rows_add(const float* y, float* x, const float* angles,
                                        const Geom& g, int row_lo, int row_hi,
                                        const float* addend, cudaStream_t stream,
                                        cudaEvent_t addend_ready = nullptr);

// Host-buffer projections (vp_host.cu): g.accumulate selects out += result
// (1) or out = result (0); *launches is incremented by the kernels launched.
cudaError_t forward_z0_host(const float* x_host, float* y_host, const float* angles,
                            const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches);
cudaError_t backward_z0_host(const float* y_host, float* x_host, const float* angles,
                             const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches);
// z_order 2 (heights slowest): in is x for the forward, y for the adjoint.
cudaError_t z2_host(bool forward, const float* in_host, float* out_host, const float* angles,
                    const Geom& g, cudaMemPool_t pool, cudaStream_t s, int* launches);

// Kernel launches the forward launchers issue for a geometry (grids are
// split past 65535 angle blocks).
int launches_forward_z0(const float* x, const float* y, const Geom& g);
int launches_backward_z0(const float* y, const float* x, const Geom& g);
int launches_forward_z2(const Geom& g);

}  // namespace vp
