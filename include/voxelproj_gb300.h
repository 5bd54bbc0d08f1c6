/*
 * voxelproj_gb300 — C ABI of the exact-trapezoid parallel-beam projector
 * pair for NVIDIA GB300 (sm_103a).
 *
 * The four projector entry points replace the reference's pybind functions
 * voxelproj._CU.forward_z0 / backward_z0 / forward_z2 / backward_z2
 * (voxelproj/csrc/voxelproj.cpp:15-33, implemented in
 * voxelproj/csrc/projectors.cu:34-299).  Argument meaning follows them:
 *
 *   forward_*(in = x, out = y, angles)    y += A x
 *   backward_*(in = y, out = x, angles)   x += A^T y
 *
 * Layouts (row-major, float32, contiguous):
 *   z_order 0: x (SY, SX, Hx), y (n_ang, PX, Hy)   heights contiguous
 *   z_order 2: x (Hx, SY, SX), y (Hy, n_ang, PX)   columns / bins contiguous
 *
 * The volume grid (SY, SX) is taken from x and the detector (n_ang, PX) from
 * y, as the reference takes them from whichever of in/out holds them.  Only
 * heights h < min(Hx, Hy) are computed: the reference reads heights past the
 * input's extent as zero through its border-mode texture, which leaves those
 * output heights unchanged, and so does this library.
 *
 * Semantics kept from the reference: results are ACCUMULATED into the output
 * (`out += ...`, sp_forward_z0.cuh:167,180; sp_backward_z0.cuh:98); angles are
 * radians and only the first n_ang entries are read.
 *
 * Differences from the reference, all of them additions:
 *   - any number of angles (the reference adjoint is limited to 512);
 *   - every argument is validated and an error code is returned instead of
 *     launching on bad input (the reference checked only `in`);
 *   - work is enqueued on the caller's stream and never synchronises (the
 *     reference ran on the legacy default stream and synchronised through
 *     cudaFreeArray);
 *   - no per-call allocation or staging copy of the input.
 *
 * All pointers are device pointers on the current CUDA device.  `stream` is a
 * cudaStream_t (NULL = legacy default stream).
 */
#ifndef VOXELPROJ_GB300_H
#define VOXELPROJ_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VP_API __attribute__((visibility("default")))
#else
#define VP_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define VP_OK 0
#define VP_ERR_NULL_POINTER 1   /* a pointer is NULL while its array is non-empty */
#define VP_ERR_BAD_SHAPE 2      /* negative or too large dimension */
#define VP_ERR_ANGLES 3         /* fewer angles than the angle extent of y */
#define VP_ERR_CUDA 4           /* a CUDA runtime call failed; see vp_last_cuda_error() */
#define VP_ERR_BAD_FLAGS 5      /* unknown bit in `flags` */
#define VP_ERR_BAD_Z_ORDER 6    /* z_order other than 0 or 2 */
#define VP_ERR_WORKSPACE 7      /* workspace smaller than vp_z2_workspace_bytes() */
#define VP_ERR_SCRATCH_LIMIT 8  /* problem too large for vp_forward_z2_noalloc's array */
#define VP_ERR_BATCH 9          /* a batch problem this library cannot batch (see vp_batch_create) */

/* Flags. */
#define VP_FLAG_TRIG_PRECISE 1  /* accurate sincosf / IEEE division for the per-angle
                                   constants; default is the hardware approximations
                                   that the reference's --use_fast_math build uses */
#define VP_FLAG_OVERWRITE 2     /* out = result instead of out += result; the output
                                   is not read (host-buffer entry points only) */

/* Library version, major*10000 + minor*100 + patch. */
VP_API int vp_version(void);

/* Static text for a status code. */
VP_API const char* vp_error_string(int status);

/* The cudaError_t of the last VP_ERR_CUDA returned on this host thread. */
VP_API int vp_last_cuda_error(void);

/* Number of kernels this library has launched in this process (all threads).
 * No counterpart in the reference; lets callers and benchmarks see how many
 * GPU launches a sequence of calls issued. */
VP_API uint64_t vp_launch_count(void);

/* Bounded waits in this library's kernels that ran out since the library was
 * loaded: 0 in correct operation.  Kernels that wait on asynchronous copies
 * give up after a bounded time instead of spinning on, count it here and
 * fall back to direct loads.  Synchronises the device. */
VP_API uint64_t vp_wait_timeouts(void);

/* Limits of this library's bounded device waits, for tests of their error
 * paths; no counterpart in the reference.  They apply process-wide to
 * launches enqueued from now on.  No wait can hang: each gives up at its
 * limit, records it, and the kernel goes on (vp_wait_timeouts,
 * vp_batch_error).
 *   copy_polls   polls of a bulk copy's completion barrier in the staged
 *                adjoint (backward z0 variant 9) before its block falls back
 *                to plain loads: VP_WAIT_DEFAULT for the default (2^22), 0 to
 *                make every such wait give up at once.
 *   stage_spins  ~256 ns sleeps a batch stage waits for the stage before it
 *                (0: the default, 2^24, about 4 s).
 *   stage_extra  completions a batch stage waits for beyond those its
 *                previous stage gives: 0 in operation; any other value makes
 *                every stage wait run out.
 * Returns VP_OK. */
#define VP_WAIT_DEFAULT 0xFFFFFFFFu
VP_API int vp_set_wait_limits(uint32_t copy_polls, uint32_t stage_spins, uint32_t stage_extra);

/* Kernel variant selection, used by the autotuner and for measurements.
 * op: 0 = forward z0, 1 = backward z0, 2 = forward z2, 3 = backward z2;
 * variant 0 = automatic (default).  Unknown variants fall back to automatic.
 * Process-wide; no counterpart in the reference (its only tuning knob,
 * block_size, is accepted and ignored by the Python layer). */
VP_API int vp_set_kernel_variant(int op, int variant);
VP_API int vp_get_kernel_variant(int op);

/* y += A x, z_order 0.  x (x0=SY, x1=SX, x2=Hx), y (y0=n_ang, y1=PX, y2=Hy).
 * Replaces voxelproj._CU.forward_z0 (voxelproj/csrc/projectors.cu:34-104). */
VP_API int vp_forward_z0(const float* x, int64_t x0, int64_t x1, int64_t x2,
                  float* y, int64_t y0, int64_t y1, int64_t y2,
                  const float* angles, int64_t n_angles, int flags, void* stream);

/* x += A^T y, z_order 0.  y (y0=n_ang, y1=PX, y2=Hy), x (x0=SY, x1=SX, x2=Hx).
 * Replaces voxelproj._CU.backward_z0 (voxelproj/csrc/projectors.cu:106-169). */
VP_API int vp_backward_z0(const float* y, int64_t y0, int64_t y1, int64_t y2,
                   float* x, int64_t x0, int64_t x1, int64_t x2,
                   const float* angles, int64_t n_angles, int flags, void* stream);

/* y += A x, z_order 2.  x (x0=Hx, x1=SY, x2=SX), y (y0=Hy, y1=n_ang, y2=PX).
 * Replaces voxelproj._CU.forward_z2 (voxelproj/csrc/projectors.cu:171-234). */
VP_API int vp_forward_z2(const float* x, int64_t x0, int64_t x1, int64_t x2,
                  float* y, int64_t y0, int64_t y1, int64_t y2,
                  const float* angles, int64_t n_angles, int flags, void* stream);

/* x += A^T y, z_order 2.  y (y0=Hy, y1=n_ang, y2=PX), x (x0=Hx, x1=SY, x2=SX).
 * Replaces voxelproj._CU.backward_z2 (voxelproj/csrc/projectors.cu:236-299). */
VP_API int vp_backward_z2(const float* y, int64_t y0, int64_t y1, int64_t y2,
                   float* x, int64_t x0, int64_t x1, int64_t x2,
                   const float* angles, int64_t n_angles, int flags, void* stream);

/* z_order 2 with caller-supplied scratch.  For H >= 32 the z_order 2
 * operators transpose to height-fastest order, run the z_order 0 kernels and
 * transpose back (adding into the output); they need
 * vp_z2_workspace_bytes(...) bytes of device scratch (0 when H < 32).  The
 * plain vp_forward_z2 / vp_backward_z2 take it from a library-private
 * stream-ordered pool; these variants use `workspace` instead and fail with
 * VP_ERR_WORKSPACE if it is too small.  No counterpart in the reference,
 * which staged its input through a per-call cudaArray. */
VP_API size_t vp_z2_workspace_bytes(int64_t x0, int64_t x1, int64_t x2,
                                    int64_t y0, int64_t y1, int64_t y2);
VP_API int vp_forward_z2_ws(const float* x, int64_t x0, int64_t x1, int64_t x2,
                            float* y, int64_t y0, int64_t y1, int64_t y2,
                            const float* angles, int64_t n_angles, int flags,
                            void* workspace, size_t workspace_bytes, void* stream);
VP_API int vp_backward_z2_ws(const float* y, int64_t y0, int64_t y1, int64_t y2,
                             float* x, int64_t x0, int64_t x1, int64_t x2,
                             const float* angles, int64_t n_angles, int flags,
                             void* workspace, size_t workspace_bytes, void* stream);

/* y += A x, z_order 2, allocating nothing: for callers that may not allocate
 * device memory while they run (code that fixes its memory at start-up,
 * hosts whose own allocator owns the device).  Same arguments and results as
 * vp_forward_z2, but its scratch is an array of VP_NOALLOC_SCRATCH_BYTES
 * (64 MiB) compiled into the library, held by every GPU that loads the
 * library until the process exits.  Problems needing more scratch than that
 * (vp_z2_workspace_bytes) return VP_ERR_SCRATCH_LIMIT and leave y unchanged.
 * The first call on a device looks up the array's address (make it before
 * any stream capture).  All calls share the array: calls that overlap on the
 * GPU race and must be ordered by the caller.  No counterpart in the
 * reference. */
#define VP_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
VP_API int vp_forward_z2_noalloc(const float* x, int64_t x0, int64_t x1, int64_t x2,
                                 float* y, int64_t y0, int64_t y1, int64_t y2,
                                 const float* angles, int64_t n_angles, int flags, void* stream);

/* ---- Batches -----------------------------------------------------------
 * Many problems of different sizes and angle counts, forward and adjoint
 * mixed, in one persistent kernel launch per body present: the forward and
 * the run adjoint with 4 or 8 heights per lane, the 8-height forms in two
 * bodies (whole 256-height chunks or not), so at most six launches however
 * many problems.  Each body keeps its single-problem kernel's register
 * budget.  No counterpart in the reference, which launches one kernel per
 * call.
 *
 * A problem is in z_order 0 layout (x (SY, SX, H), y (n_ang, PX, H)) with
 * heights a multiple of 4 and 16-byte aligned buffers; its output is
 * accumulated into, as for the single-problem calls.  Outputs of different
 * problems must not overlap.  Results equal the single-problem kernels of the
 * same variant, bit for bit. */
#define VP_OP_FORWARD 0   /* out (y) += A in (x) */
#define VP_OP_BACKWARD 1  /* out (x) += A^T in (y) */
/* The single-problem forward variant that a batched forward problem of
 * variant 0 runs: four neighbouring angles per block and 128 MB class slabs.
 * Batched, its fewer stages wait less than the single-problem default's
 * 64 MB slabs. */
#define VP_BATCH_FORWARD_DEFAULT 21

typedef struct vp_batch_problem {
  int op;                 /* VP_OP_FORWARD or VP_OP_BACKWARD */
  int flags;              /* VP_FLAG_* as for the single-problem calls */
  int variant;            /* the single-problem kernel variant whose body,
                             heights per lane and slabs the problem uses.
                             Forward: 0 (= VP_BATCH_FORWARD_DEFAULT) or
                             any variant with 4 bins per warp (1, 3, 5, 7, 9,
                             10, 11, 12, 16, 21, 22, 23).  Adjoint: 0 / 7 = runs in two angle
                             classes, 8 heights per lane past 128 heights
                             (default); 6 = runs, 4 heights per lane; 4 = 2x2
                             voxel blocks (accumulates in the reference's
                             order, bit-identical to it) */
  int reserved;
  const float* in;        /* x for a forward problem, y for an adjoint one */
  float* out;             /* y for a forward problem, x for an adjoint one */
  const float* angles;
  int64_t n_angles;
  int64_t in_dims[3];
  int64_t out_dims[3];
} vp_batch_problem;

typedef struct vp_batch_plan vp_batch_plan;

/* Validates the problems and uploads their descriptor table to the current
 * device (the only device allocation); *plan receives the plan. */
VP_API int vp_batch_create(const vp_batch_problem* problems, int count, vp_batch_plan** plan);
/* Re-plans `plan` for another set of problems (validated as by
 * vp_batch_create), without synchronising the device: the descriptors go up
 * by an asynchronous copy on `stream` from the plan's page-locked staging
 * (two buffers used in turn; an update waits only for the upload of two
 * updates before), and device buffers are reallocated in stream order only
 * when the new set needs more room than the plan has.  Runs enqueued before
 * on the same stream keep their problems, runs after see the new set: run
 * the plan on the stream it was updated on, or order the two.  On an invalid
 * problem the plan is left as it was.  For a scheduler whose set of problems
 * changes from one step to the next.  No counterpart in the reference. */
VP_API int vp_batch_update(vp_batch_plan* plan, const vp_batch_problem* problems, int count,
                           void* stream);
/* Enqueues the whole batch on `stream`: a counter reset and one persistent
 * launch per body present.  Allocates and synchronises nothing, so it can be
 * captured in a CUDA graph.  Runs of the same plan must not overlap on the
 * GPU. */
VP_API int vp_batch_run(vp_batch_plan* plan, void* stream);
/* Work items of the plan (blocks' units of work). */
VP_API int64_t vp_batch_work_items(const vp_batch_plan* plan);
/* Synchronises and reports whether a run hit its bounded wait between stages
 * (*error = 1: a dependency did not complete in ~4 s and the result may be
 * wrong).  Stays set for the plan's lifetime once raised. */
VP_API int vp_batch_error(vp_batch_plan* plan, int* error);
VP_API int vp_batch_destroy(vp_batch_plan* plan);

/* ---- Host buffers --------------------------------------------------------
 * y (+)= A x and x (+)= A^T y with x and y in host memory (any
 * memory cudaMemcpyDefault can address); angles in host or device memory.
 * Dims as for vp_forward_z0 / vp_backward_z0.  The library stages the arrays
 * through device buffers of its own pool and overlaps the copies with the
 * kernels: the forward starts on the first volume rows while the rest are in
 * flight, the adjoint sends finished voxel rows back while later rows are
 * computed.  Page-locked host buffers make the copies asynchronous; pageable
 * ones work with less overlap.  The call is asynchronous on `stream`: the
 * host output is complete when the stream is, and the host arrays must not
 * be modified before then.  Same results as the device entry points with the
 * same kernel variant, and the same per-slab summation; flags may add
 * VP_FLAG_OVERWRITE.  No counterpart in the reference, whose Python wrappers
 * copy the whole input in, project, and copy the result out one after
 * another (voxelproj/wrappers.py:10-25, :57-73). */
VP_API int vp_forward_z0_host(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y,
                              int64_t y0, int64_t y1, int64_t y2, const float* angles,
                              int64_t n_angles, int flags, void* stream);
VP_API int vp_backward_z0_host(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x,
                               int64_t x0, int64_t x1, int64_t x2, const float* angles,
                               int64_t n_angles, int flags, void* stream);
/* The same for z_order 2, dims as for vp_forward_z2 / vp_backward_z2.  Heights
 * are the slowest axis there, so the library works in chunks of heights (256
 * from 512 heights up), each an independent problem whose copies overlap the
 * other chunk's kernels. */
VP_API int vp_forward_z2_host(const float* x, int64_t x0, int64_t x1, int64_t x2, float* y,
                              int64_t y0, int64_t y1, int64_t y2, const float* angles,
                              int64_t n_angles, int flags, void* stream);
VP_API int vp_backward_z2_host(const float* y, int64_t y0, int64_t y1, int64_t y2, float* x,
                               int64_t x0, int64_t x1, int64_t x2, const float* angles,
                               int64_t n_angles, int flags, void* stream);

/* z_order dispatch, as voxelproj.wrappers.forward/backward select a kernel by
 * z_order (voxelproj/wrappers.py:44-47, :92-95); dims as for the
 * matching entry point above. */
VP_API int vp_forward(const float* x, const int64_t x_dims[3], float* y, const int64_t y_dims[3],
               const float* angles, int64_t n_angles, int z_order, int flags, void* stream);
VP_API int vp_backward(const float* y, const int64_t y_dims[3], float* x, const int64_t x_dims[3],
                const float* angles, int64_t n_angles, int z_order, int flags, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VOXELPROJ_GB300_H */
