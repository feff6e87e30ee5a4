/*
 * torchmorph_gb300 -- C ABI of the GB300 (sm_103a) morphology, distance
 * transform and Sinkhorn kernels.
 *
 * The library (libtmcore.so) is the drop-in replacement for the reference's
 * pybind11 module `torchmorph._C` (torchmorph/csrc/torchmorph.cpp:79-155).
 * Every entry point takes plain device pointers, sizes and a CUDA stream; no
 * torch types cross this boundary.  Each declaration names the reference
 * function it replaces.
 *
 * Conventions
 *   - An "item" is one (b, c) slice of the reference's (B, C, *spatial)
 *     tensors; `batch` = B*C items are laid out back to back, each a
 *     C-contiguous array of `ndim` (1..8) spatial dimensions `shape`.
 *   - Index outputs are int32 planes laid out (ndim, batch, *shape), the
 *     layout of the reference's `indices` tensors.
 *   - Structuring elements, footprints, origins and sampling are HOST
 *     arrays (the reference passes them as CPU tensors / Python lists).
 *   - Work is enqueued on `stream` of the CURRENT device; calls are
 *     asynchronous unless stated otherwise.  The caller selects the device.
 *   - Every function returns a tm_status; on failure tm_last_error() holds
 *     a message for the calling thread.
 *   - Functions that need temporary device memory take a caller-owned
 *     `workspace` of at least the size its *_workspace_size() companion
 *     returns; the library itself never allocates device memory.
 *   - Per-device state (kernel attributes, the tm_edt_noalloc scratch
 *     address) is cached for the life of the process: calling
 *     cudaDeviceReset() on a device while the library is loaded is not
 *     supported.
 */
#ifndef TORCHMORPH_GB300_H
#define TORCHMORPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *tm_stream_t; /* same type as cudaStream_t */

typedef enum tm_status {
    TM_OK = 0,
    TM_ERR_INVALID_ARGUMENT = 1, /* bad shape, pointer, origin, mode, ...   */
    TM_ERR_UNSUPPORTED = 2,      /* valid request the library does not serve */
    TM_ERR_CUDA = 3,             /* a CUDA runtime call or launch failed    */
    TM_ERR_TOO_LARGE = 4,        /* sizes overflow the kernel's index types */
    TM_ERR_WORKSPACE = 5,        /* workspace missing or too small          */
    TM_ERR_TIMEOUT = 6           /* a bounded device-side wait gave up       */
} tm_status;

/* Border modes of the grey operators (torchmorph/morphology/grey.py:8-14). */
typedef enum tm_border_mode {
    TM_MODE_CONSTANT = 0,
    TM_MODE_REFLECT = 1,
    TM_MODE_NEAREST = 2,
    TM_MODE_MIRROR = 3,
    TM_MODE_WRAP = 4
} tm_border_mode;

/* Element types accepted by the distance transforms' foreground input. */
typedef enum tm_dtype { TM_F32 = 0, TM_U8 = 1 } tm_dtype;

/* Chamfer metrics (torchmorph/distance_transform.py:121-123) plus the
 * weighted 3-4-5 chamfer, which the reference does not have. */
typedef enum tm_cdt_metric {
    TM_CDT_CHESSBOARD = 0,
    TM_CDT_TAXICAB = 1,
    TM_CDT_CHAMFER345 = 2
} tm_cdt_metric;

/* Brute-force metrics (torchmorph/csrc/bfdt_kernel.cu:167-171). */
typedef enum tm_bf_metric { TM_BF_EUCLIDEAN = 0, TM_BF_TAXICAB = 1, TM_BF_CHESSBOARD = 2 } tm_bf_metric;

const char *tm_status_string(int status);
const char *tm_last_error(void);
int tm_version(void);

/* Device-side status of the current device: 0 when no kernel has recorded a
 * failure, 1 when a bounded wait inside a kernel gave up (the kernel then
 * stopped early and its outputs are incomplete).  Synchronous; `reset`
 * clears the word.  No counterpart in the reference (its kernels have no
 * waits). */
int tm_device_error(int reset);

/* Poll budget of the grid barriers of the cooperative persistent kernels
 * (tm_pointcloud_sinkhorn, the FP32 Sinkhorn iterations): a CTA that waits
 * longer records a timeout in the device status word (tm_device_error) and
 * every CTA of the launch returns.  polls < 0 restores the default (2^26
 * polls of ~64 ns).  The waits that guard TMA copies and tensor-core work
 * keep their own fixed budget.  No counterpart in the reference. */
void tm_set_grid_wait_budget(int64_t polls);

/* ------------------------------------------------------------ autotuning --
 * Implementation variants of four operators, picked per work class by the
 * autotuner (torchmorph_gb300/autotune.py).  Every variant of an operator
 * computes bit-identical results; variant -1 restores the library's built-in
 * choice.  The table is process-wide (host memory), so a tuning applies to
 * every device of the process.  No counterpart in the reference (its block
 * sizes are compile-time constants, e.g. torchmorph/csrc/ot_kernel.cu:9).
 *   op 0  grey / binary flat 1-D / 2-D boxes: 0 TMA-staged persistent tiles,
 *         1 plain loads (one CTA per tile), 2 / 3 TMA tiles with at most 1 / 2
 *         CTAs per SM;                       class: log2(voxels)
 *   op 1  FP32 Sinkhorn: bit 0 = 64 pairs per tile (else 16), bit 1 = one CTA
 *         per SM (else two);                 class: 8 min(7, log2 n) + min(7, log2 d - 6)
 *   op 2  3-D exact EDT: 0 bitmap shell search first, 1 separable passes only;
 *                                             class: log2(voxels)
 *   op 3  3-D chamfer distances: 0 bitmap shell search first (persistent warps
 *         on a queue of 8-row units), 1 raster passes only, 2 shell search with
 *         one CTA per 32-row block;           class: log2(voxels)
 * tm_tune_class(op, a, b): the class of a call (a = voxels, or a = n pairs and
 * b = d points for op 1). */
int tm_tune_variants(int op);
int tm_tune_class(int op, int64_t a, int64_t b);
int tm_tune_set(int op, int cls, int variant);
int tm_tune_get(int op, int cls);

/* ------------------------------------------------------------------ grey --
 * Replaces grey_erosion_cuda / grey_dilation_cuda
 * (torchmorph/csrc/torchmorph.cpp:3-19, torchmorph/csrc/grey_kernel.cu:332-356).
 * structure: float32[prod(sshape)] host; footprint: uint8[prod(sshape)]
 * host or NULL (all active); origin: int64[ndim] host.
 * in/out: float32 device, batch*prod(shape) elements; out must not alias in.
 */
int tm_grey_erosion(const float *in, float *out, int64_t batch, int ndim,
                    const int64_t *shape, const float *structure, const uint8_t *footprint,
                    const int64_t *sshape, const int64_t *origin, int mode, float cval,
                    tm_stream_t stream);
int tm_grey_dilation(const float *in, float *out, int64_t batch, int ndim,
                     const int64_t *shape, const float *structure, const uint8_t *footprint,
                     const int64_t *sshape, const int64_t *origin, int mode, float cval,
                     tm_stream_t stream);

/* Opt-in backward of grey erosion / dilation, 1-3 spatial dimensions, at
 * most 255 active taps.  No counterpart in the reference (its operators are
 * not differentiable, torchmorph/morphology/grey.py:92-100).
 * *_arg: the forward (same arguments and output as tm_grey_erosion /
 * tm_grey_dilation) that also writes arg[i] = index of the first active tap,
 * in footprint raster order, attaining the extremum (255: none).
 * *_backward: grad_in[j] = sum of grad_out[o] over the outputs o whose
 * recorded tap reads j through the border mode (reads of the constant
 * border route nothing); deterministic gather, no atomics. */
int tm_grey_erosion_arg(const float *in, float *out, uint8_t *arg, int64_t batch, int ndim,
                        const int64_t *shape, const float *structure, const uint8_t *footprint,
                        const int64_t *sshape, const int64_t *origin, int mode, float cval,
                        tm_stream_t stream);
int tm_grey_dilation_arg(const float *in, float *out, uint8_t *arg, int64_t batch, int ndim,
                         const int64_t *shape, const float *structure, const uint8_t *footprint,
                         const int64_t *sshape, const int64_t *origin, int mode, float cval,
                         tm_stream_t stream);
int tm_grey_erosion_backward(const float *grad_out, const uint8_t *arg, float *grad_in,
                             int64_t batch, int ndim, const int64_t *shape,
                             const uint8_t *footprint, const int64_t *sshape,
                             const int64_t *origin, int mode, tm_stream_t stream);
int tm_grey_dilation_backward(const float *grad_out, const uint8_t *arg, float *grad_in,
                              int64_t batch, int ndim, const int64_t *shape,
                              const uint8_t *footprint, const int64_t *sshape,
                              const int64_t *origin, int mode, tm_stream_t stream);

/* One-pass grey composites of 2-D items (same arguments as tm_grey_dilation):
 * out = dilation - erosion (morphological_gradient,
 * torchmorph/morphology/grey.py:200-221) and out = (dilation + erosion) - 2 in
 * (morphological_laplace, grey.py:268-289), each value rounded as the
 * reference's elementwise float32 ops round it.  Elements of up to 64 active
 * taps whose offsets span at most 31 per axis; anything else returns
 * TM_ERR_UNSUPPORTED (the caller then composes the two operators). */
int tm_grey_gradient(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                     const float *structure, const uint8_t *footprint, const int64_t *sshape,
                     const int64_t *origin, int mode, float cval, tm_stream_t stream);
int tm_grey_laplace(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                    const float *structure, const uint8_t *footprint, const int64_t *sshape,
                    const int64_t *origin, int mode, float cval, tm_stream_t stream);

/* One-pass grey opening / closing and white / black top-hats of 1-D or 2-D
 * items with flat rectangular elements (footprint all active, one structure
 * value, up to 33 per axis): the first operator, the intermediate image's
 * border handling and the second operator (and the top-hat difference) in
 * one kernel per 32 x 128 output tile, bit-identical to the reference's
 * composition (torchmorph/morphology/grey.py:162-197, 224-265).  Arguments
 * as for tm_grey_dilation; TM_ERR_UNSUPPORTED outside these limits, where
 * the caller composes the operators. */
int tm_grey_opening(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                    const float *structure, const uint8_t *footprint, const int64_t *sshape,
                    const int64_t *origin, int mode, float cval, tm_stream_t stream);
int tm_grey_closing(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                    const float *structure, const uint8_t *footprint, const int64_t *sshape,
                    const int64_t *origin, int mode, float cval, tm_stream_t stream);
int tm_white_tophat(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                    const float *structure, const uint8_t *footprint, const int64_t *sshape,
                    const int64_t *origin, int mode, float cval, tm_stream_t stream);
int tm_black_tophat(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                    const float *structure, const uint8_t *footprint, const int64_t *sshape,
                    const int64_t *origin, int mode, float cval, tm_stream_t stream);

/* ---------------------------------------------------------------- binary --
 * Replaces binary_erosion_cuda / binary_dilation_cuda
 * (torchmorph/csrc/torchmorph.cpp:21-33, torchmorph/csrc/binary_kernel.cu:252-272).
 * in/out: uint8 (torch.bool) device arrays holding 0/1; structure: uint8 host.
 */
int tm_binary_erosion(const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
                      const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
                      const int64_t *origin, int border_value, tm_stream_t stream);
int tm_binary_dilation(const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
                       const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
                       const int64_t *origin, int border_value, tm_stream_t stream);

/* One-pass binary opening / closing (one iteration, no mask) of 1-D or 2-D
 * items on bit-packed tiles: the first operator over the tile grown by the
 * second's halo stays on chip, positions outside the item read border_value
 * in both operators -- equal to the reference's two calls
 * (torchmorph/morphology/binary.py:231-290).  Arguments as for
 * tm_binary_erosion; TM_ERR_UNSUPPORTED when a structure offset reaches
 * beyond 16 rows or 32 columns, where the caller composes the operators.
 * 1-D / 2-D tm_binary_erosion / tm_binary_dilation with elements other than
 * full boxes run on the same bit tiles. */
int tm_binary_opening(const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                      const uint8_t *structure, const int64_t *sshape, const int64_t *origin,
                      int border_value, tm_stream_t stream);
int tm_binary_closing(const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                      const uint8_t *structure, const int64_t *sshape, const int64_t *origin,
                      int border_value, tm_stream_t stream);

/* ------------------------------------------------------------------- edt --
 * Replaces edt_cuda (torchmorph/csrc/torchmorph.cpp:35-40,
 * torchmorph/csrc/edt_kernel.cu:904-958).
 * input: device array of `in_dtype`, nonzero = foreground.
 * sampling: float32[ndim] host or NULL (unit spacing).
 * dist: float32 device or NULL; indices: int32 (ndim, batch, *shape) or NULL;
 * sqdist: int32 squared distances (unit spacing only) or NULL -- an output
 * the reference does not have.  At least one output must be given.
 * Feature indices follow scipy.ndimage: nearest background voxel, ties to
 * the smallest last-axis coordinate, then the previous axis, and so on.
 */
size_t tm_edt_workspace_size(int64_t batch, int ndim, const int64_t *shape, const float *sampling);
int tm_edt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
           const float *sampling, float *dist, int32_t *indices, int32_t *sqdist,
           void *workspace, size_t workspace_bytes, tm_stream_t stream);

/* Allocation-free EDT.  No counterpart in the reference: this entry point
 * exists for callers that cannot hand the library a device workspace (for
 * example code paths where allocating device memory is not allowed, or C
 * callers without an allocator of their own).  It runs the same kernels as
 * tm_edt for 2-D and 3-D items with unit spacing, on a fixed 32 MiB scratch
 * area that the library keeps on every GPU that loads it until the process
 * exits; larger batches (above ~4M voxels of 3-D items or ~16M of 2-D items)
 * are rejected with TM_ERR_TOO_LARGE, other shapes with TM_ERR_UNSUPPORTED.
 * The first call on a device (2-D or 3-D alike: nothing else is set up
 * lazily on this path) looks up the scratch area's device address; make
 * that first call outside any CUDA stream capture.  All calls on a device
 * share the scratch: calls whose GPU work may overlap must be serialised by
 * the caller.  Outputs as for tm_edt.
 */
int tm_edt_noalloc(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
                   float *dist, int32_t *indices, int32_t *sqdist, tm_stream_t stream);

/* ------------------------------------------------------------------- cdt --
 * Replaces cdt_cuda (torchmorph/csrc/torchmorph.cpp:42-47,
 * torchmorph/csrc/cdt_kernel.cu:269-463).
 * dist: float32 (path cost; -1 where an item has no background) or NULL;
 * for TM_CDT_CHAMFER345 the cost is divided by 3.  indices as for tm_edt.
 */
size_t tm_cdt_workspace_size(int64_t batch, int ndim, const int64_t *shape);
int tm_cdt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
           int metric, float *dist, int32_t *indices, void *workspace, size_t workspace_bytes,
           tm_stream_t stream);

/* ------------------------------------------------------------------ bfdt --
 * Replaces bfdt_cuda (torchmorph/csrc/torchmorph.cpp:49-55,
 * torchmorph/csrc/bfdt_kernel.cu:154-297).
 */
size_t tm_bfdt_workspace_size(int64_t batch, int ndim, const int64_t *shape);
int tm_bfdt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
            int metric, const float *sampling, float *dist, int32_t *indices,
            void *workspace, size_t workspace_bytes, tm_stream_t stream);

/* ---------------------------------------------------------------- ragged --
 * Ragged batches: n_items 2-D images of different sizes packed in one
 * buffer (image i: heights[i] x widths[i] elements from element offsets[i],
 * row-major).  Each operator is ONE persistent launch over the 128 x 32
 * tiles of all images, taking tiles from a work queue in the plan; the
 * result per image equals the uniform-batch operator on that image
 * (tm_grey_erosion ... with batch 1, ndim 2), i.e. the reference's per-image
 * calls of grey_erosion_cuda ... (torchmorph/csrc/torchmorph.cpp:3-33).
 * No counterpart in the reference, which has no ragged batches.
 *
 * tm_ragged_plan writes the device descriptor table into `plan` (device,
 * 256-byte aligned, tm_ragged_plan_size(n_items) bytes); one plan serves
 * every operator and dtype on that layout, and may be reused across CUDA
 * graph replays.  Operators sharing a plan must not run concurrently.
 * Structures are 2-D, sizes 1..255 per axis; grey ops take the same
 * structure/footprint/origin/mode/cval as tm_grey_erosion, binary ops a
 * uint8 structure and border_value as tm_binary_erosion (one iteration). */
size_t tm_ragged_plan_size(int64_t n_items);
int tm_ragged_plan(int64_t n_items, const int64_t *heights, const int64_t *widths,
                   const int64_t *offsets, void *plan, size_t plan_bytes, tm_stream_t stream);
int tm_ragged_grey_erosion(const float *in, float *out, const void *plan, size_t plan_bytes,
                           int64_t n_items, const float *structure, const uint8_t *footprint,
                           const int64_t *sshape, const int64_t *origin, int mode, float cval,
                           tm_stream_t stream);
int tm_ragged_grey_dilation(const float *in, float *out, const void *plan, size_t plan_bytes,
                            int64_t n_items, const float *structure, const uint8_t *footprint,
                            const int64_t *sshape, const int64_t *origin, int mode, float cval,
                            tm_stream_t stream);
int tm_ragged_binary_erosion(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                             int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                             const int64_t *origin, int border_value, tm_stream_t stream);
int tm_ragged_binary_dilation(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                              int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                              const int64_t *origin, int border_value, tm_stream_t stream);
/* Ragged binary operators run on bit-packed tiles (as tm_binary_opening);
 * the opening / closing in one pass. */
int tm_ragged_binary_opening(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                             int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                             const int64_t *origin, int border_value, tm_stream_t stream);
int tm_ragged_binary_closing(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                             int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                             const int64_t *origin, int border_value, tm_stream_t stream);

/* Ragged batches of 3-D volumes (volume i: depths[i] x heights[i] x
 * widths[i] elements from element offsets[i]).  Each operator is ONE
 * persistent launch over the 4 x 8 x 32 output tiles of all volumes, taken
 * from the plan's work queue and computed from a shared-memory copy of the
 * tile's input region; per volume the result equals the uniform-batch
 * operator on that volume (batch 1, ndim 3), i.e. the reference's per-volume
 * calls of grey_erosion_cuda ... (torchmorph/csrc/torchmorph.cpp:3-33).
 * Structures up to 255 per axis and 1024 active taps.  Other arguments as
 * for the 2-D ragged operators. */
size_t tm_ragged3d_plan_size(int64_t n_items);
int tm_ragged3d_plan(int64_t n_items, const int64_t *depths, const int64_t *heights,
                     const int64_t *widths, const int64_t *offsets, void *plan, size_t plan_bytes,
                     tm_stream_t stream);
int tm_ragged3d_grey_erosion(const float *in, float *out, const void *plan, size_t plan_bytes,
                             int64_t n_items, const float *structure, const uint8_t *footprint,
                             const int64_t *sshape, const int64_t *origin, int mode, float cval,
                             tm_stream_t stream);
int tm_ragged3d_grey_dilation(const float *in, float *out, const void *plan, size_t plan_bytes,
                              int64_t n_items, const float *structure, const uint8_t *footprint,
                              const int64_t *sshape, const int64_t *origin, int mode, float cval,
                              tm_stream_t stream);
int tm_ragged3d_binary_erosion(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                               int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                               const int64_t *origin, int border_value, tm_stream_t stream);
int tm_ragged3d_binary_dilation(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                const int64_t *origin, int border_value, tm_stream_t stream);

/* Ragged exact EDT (unit spacing) of n_items 2-D or 3-D items (shapes:
 * int64[n_items * ndim] host, item i at element offsets[i] of the packed
 * input), in ONE cooperative persistent launch: the separable passes of
 * edt_cuda (torchmorph/csrc/edt_kernel.cu:904-958, scipy's tie rule) run for
 * all items at once, one grid-wide phase per axis.  Replaces the reference's
 * per-item calls of torchmorph/distance_transform.py:72-102.
 *   tm_ragged_edt_plan   builds the device descriptor table once per layout;
 *   tm_ragged_edt        input: float32 or uint8 (nonzero = foreground);
 *                        total = packed element count; max_line = longest
 *                        axis of any item; lines[a] = sum over items of
 *                        numel / shape[a]; dist float32[total], indices
 *                        int32 (ndim, total) (item-local coordinates), sqdist
 *                        int32[total], each optional; workspace of
 *                        tm_ragged_edt_workspace_size(total, max_line) bytes,
 *                        256-byte aligned.
 * Axes up to 32767 voxels, items below 2^31 voxels. */
size_t tm_ragged_edt_plan_size(int64_t n_items);
int tm_ragged_edt_plan(int64_t n_items, int ndim, const int64_t *shapes, const int64_t *offsets,
                       void *plan, size_t plan_bytes, tm_stream_t stream);
size_t tm_ragged_edt_workspace_size(int64_t total, int64_t max_line);
int tm_ragged_edt(const void *input, int in_dtype, const void *plan, size_t plan_bytes,
                  int64_t n_items, int ndim, int64_t total, int64_t max_line, const int64_t *lines,
                  float *dist, int32_t *indices, int32_t *sqdist, void *workspace,
                  size_t workspace_bytes, tm_stream_t stream);

/* -------------------------------------------------------------- sinkhorn --
 * FP32 Sinkhorn on the CUDA cores for n histogram pairs sharing one (d, d)
 * matrix.  Every call runs its iterations in ONE cooperative persistent
 * launch (tiles of 128 matrix rows x 16 or 64 pairs, bounded grid barriers
 * between half-steps); the workspace holds the launch's control block.
 *
 * Replaces sinkhorn_fastiter (torchmorph/csrc/torchmorph.cpp:58-66,
 * torchmorph/csrc/ot_kernel.cu:188-233): n_iter scaling iterations
 * u = a / (K v + 1e-12), v = b / (K^T u + 1e-12) on (n, d) batches sharing
 * K (d, d).  u and v are updated in place.  workspace: 16-byte aligned,
 * tm_sinkhorn_iter_workspace_size() bytes.
 */
size_t tm_sinkhorn_iter_workspace_size(void);
int tm_sinkhorn_fastiter(const float *a, const float *b, const float *K, const float *K_T,
                         float *u, float *v, int64_t n, int64_t d, int64_t n_iter,
                         void *workspace, size_t workspace_bytes, tm_stream_t stream);

/* Replaces sinkhorn_logiter (torchmorph/csrc/torchmorph.cpp:68-77,
 * torchmorph/csrc/ot_kernel.cu:235-283): n_iter log-domain iterations
 * log_u = log_a - LSE_j(-M_ij/eps + log_v_j), then the same for log_v with
 * M_T; -inf wherever every term is -inf.  Workspace as for fastiter.
 */
int tm_sinkhorn_logiter(const float *log_a, const float *log_b, const float *M,
                        const float *M_T, float *log_u, float *log_v, int64_t n, int64_t d,
                        int64_t n_iter, double epsilon, void *workspace, size_t workspace_bytes,
                        tm_stream_t stream);

/* A whole FP32 solve on the device.  Replaces the fused branch of
 * _scaling_iterations / _log_iterations and the plan materialisation of
 * _SinkhornDistance.forward (torchmorph/optimal_transport.py:38-144):
 * builds K = exp(-C/eps) and K^T (scaling form) or C^T (log form), starts
 * from u = v = 1 (log u = log v = 0), runs up to max_iter iterations in one
 * launch and, when threshold > 0, stops after the first iteration k with
 * (k + 1) % check_every == 0 at which every pair's L1 row-marginal residual
 * sum_i |a_i - (P 1)_i| of the plan that iteration started from is <=
 * threshold (decided on the device: no host round trip).  Outputs: log_u,
 * log_v (device fp32 (n, d), the reference's u.log() / log-potentials),
 * cost[b] = <P_b, C> and row_err[b] (fp64 [n], for the returned potentials,
 * P never materialised) and iterations (int32 scalar); cost, row_err and
 * iterations may be NULL.  a, b: fp32 (n, d) rows summing to 1; C: fp32
 * (d, d), or NULL for the cost |i - j| of d points on a line (the
 * reference's default build_cost_matrix((d,)) for p = 1 or 2), which is then
 * computed where it is used -- no (d, d) matrix is stored or read; the same
 * NULL is accepted by tm_sinkhorn_plan and tm_sinkhorn_cost_grad.
 * workspace: 256-byte aligned, tm_sinkhorn_f32_workspace_size bytes
 * (line_cost = 1 when C is NULL).
 * No counterpart in the reference's extension (it exposes the iterations
 * only). */
size_t tm_sinkhorn_f32_workspace_size(int64_t n, int64_t d, int log_space, int64_t max_iter,
                                      int64_t check_every, int line_cost);
int tm_sinkhorn_f32_solve(const float *a, const float *b, const float *C, int64_t n, int64_t d,
                          double epsilon, int log_space, int64_t max_iter, double threshold,
                          int64_t check_every, float *log_u, float *log_v, double *cost,
                          double *row_err, int32_t *iterations, void *workspace,
                          size_t workspace_bytes, tm_stream_t stream);

/* Transport plans plan[b, i, j] = exp((log_u[b, i] - C[i, j] / eps) +
 * log_v[b, j]) (device fp32 (n, d, d)) in one pass, with the operations and
 * rounding of SinkhornSolver.plan (torchmorph/optimal_transport.py:228-237).
 */
int tm_sinkhorn_plan(const float *log_u, const float *log_v, const float *C, int64_t n,
                     int64_t d, double epsilon, float *plan, tm_stream_t stream);

/* Gradient of sum_b grad_distance[b] * distance[b] with respect to the cost
 * matrix by the envelope theorem: grad_C = sum_b grad_distance[b] P_b, plan
 * entries recomputed from the log-potentials and never stored (device fp32
 * (d, d)).  The reference returns no cost gradient
 * (torchmorph/optimal_transport.py:146-150). */
int tm_sinkhorn_cost_grad(const float *log_u, const float *log_v, const float *C,
                          const float *grad_distance, int64_t n, int64_t d, double epsilon,
                          float *grad_C, tm_stream_t stream);

/* ------------------------------------------------ sinkhorn, tensor cores --
 * Shared-cost batched Sinkhorn on the tcgen05 tensor cores.  Replaces, for
 * n histogram pairs sharing one (d, d) cost, the iterations of
 * _scaling_iterations / _log_iterations (torchmorph/optimal_transport.py:
 * 71-125, fused path sinkhorn_fastiter / sinkhorn_logiter) and the plan
 * materialisation of _SinkhornDistance.forward (:136-144):
 *   init     builds K = exp(-C/eps), K^T and K o C (bf16 hi + lo) and sets
 *            log u = log v = 0 (the reference's start);
 *   iterate  runs n_iter iterations (u update, then v update); when row_err
 *            (device, fp64[n]) is given it receives the L1 row-marginal
 *            residual sum_i |a_i - (P 1)_i| of the plan the last iteration
 *            started from;
 *   finish   writes log_u, log_v (device fp32 (n, d)), cost[h] = <P_h, C>
 *            and row_err[h] (device fp64[n]) for the current potentials;
 *            any output may be NULL.
 * a, b: device fp32 (n, d), rows summing to 1; C: device fp32 (d, d).
 * The workspace (256-byte aligned, tm_sinkhorn_tc_workspace_size bytes)
 * holds the whole solver state between the calls.  No counterpart in the
 * reference's extension. */
size_t tm_sinkhorn_tc_workspace_size(int64_t n, int64_t d);
int tm_sinkhorn_tc_init(const float *a, const float *b, const float *C, int64_t n, int64_t d,
                        double epsilon, void *workspace, size_t workspace_bytes,
                        tm_stream_t stream);
int tm_sinkhorn_tc_iterate(int64_t n, int64_t d, int64_t n_iter, double *row_err,
                           void *workspace, size_t workspace_bytes, tm_stream_t stream);
int tm_sinkhorn_tc_finish(int64_t n, int64_t d, float *log_u, float *log_v, double *cost,
                          double *row_err, void *workspace, size_t workspace_bytes,
                          tm_stream_t stream);

/* ----------------------------------------------- sinkhorn, point clouds --
 * Ragged batch of OT problems between point clouds in R^3 with the
 * squared-Euclidean cost recomputed from the points: problem p has n[p]
 * source points (x, packed (sum n, 3) fp32) and m[p] target points (y),
 * log weights log_a / log_b (packed like the points).  Log-domain Sinkhorn
 * (the iteration of torchmorph/optimal_transport.py:96-125 without a cost
 * matrix) for all problems in ONE cooperative persistent launch; a problem
 * stops once the L1 column-marginal error of its plan is <= threshold
 * (checked every check_every iterations) or after max_iter iterations.
 * Outputs: potentials f (sum n), g (sum m) (fp32, the reference's
 * epsilon * log u / log v), cost[p] = <f, a> + <g, b> (the regularised
 * cost, fp64) and iterations[p] (both optional).  The workspace
 * (tm_pointcloud_sinkhorn_workspace_size bytes, 256-byte aligned) is
 * scratch.  No counterpart in the reference (no ragged OT API).
 *
 * tm_pointcloud_sinkhorn_grad: gradient of the regularised cost w.r.t. the
 * points (envelope theorem: d cost_p / d x_i = 2 sum_j P_ij (x_i - y_j),
 * plan entries recomputed from f, g), scaled by grad_cost[p] (device fp32);
 * grad_x / grad_y may be NULL; the workspace holds
 * tm_pointcloud_sinkhorn_grad_workspace_size(n_problems) bytes. */
size_t tm_pointcloud_sinkhorn_workspace_size(int64_t n_problems, const int64_t *n,
                                             const int64_t *m, int64_t max_iter);
int tm_pointcloud_sinkhorn(const float *x, const float *y, const float *log_a,
                           const float *log_b, int64_t n_problems, const int64_t *n,
                           const int64_t *m, double epsilon, int64_t max_iter, double threshold,
                           int64_t check_every, float *f, float *g, double *cost,
                           int32_t *iterations, void *workspace, size_t workspace_bytes,
                           tm_stream_t stream);
size_t tm_pointcloud_sinkhorn_grad_workspace_size(int64_t n_problems);
int tm_pointcloud_sinkhorn_grad(const float *x, const float *y, const float *log_a,
                                const float *log_b, const float *f, const float *g,
                                int64_t n_problems, const int64_t *n, const int64_t *m,
                                double epsilon, const float *grad_cost, float *grad_x,
                                float *grad_y, void *workspace, size_t workspace_bytes,
                                tm_stream_t stream);

/* Error-compensated BF16 tensor-core product D = A B^T in fp32, with
 * A = a_hi + a_lo (M x K) and B = b_hi + b_lo (N x K), all bf16 row-major
 * device arrays, D fp32 M x N row-major: three tcgen05 MMAs per k-step
 * (hi.hi + lo.hi + hi.lo).  M and N multiples of 128, K a multiple of 64,
 * pointers 16-byte aligned.  No counterpart in the reference: this is the
 * product the shared-cost Sinkhorn solver below runs on, exported so that
 * callers can test it on its own. */
int tm_gemm_bf16x3(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo,
                   float *d, int64_t M, int64_t N, int64_t K, tm_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* TORCHMORPH_GB300_H */
