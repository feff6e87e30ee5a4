// Opt-in backward of grey erosion / dilation (1-3 spatial dimensions).
//
// Forward with argument: the same taps as the forward operator
// (torchmorph/csrc/grey_kernel.cu:271-291; erosion reads x + delta and takes
// min(v - s), dilation reads x - delta and takes max(v + s)), evaluated in
// footprint (raster) order with a strict comparison, so the recorded
// argument is the FIRST tap attaining the extremum; the output value is the
// forward operator's, bit for bit.  255 means "no tap" (every tap gave the
// identity, e.g. all -inf for a dilation).
//
// Backward as a gather (deterministic, no atomics): input voxel j receives
// grad_out[o] from every output o whose recorded tap t reads j, i.e. whose
// coordinate o + off_t maps onto j through the border mode.  Per axis the
// coordinates y' that map onto j inside the window a tap can reach form at
// most two ranges (reflect / mirror: j and its mirror image; wrap: one
// point; nearest: a run at the edges; constant: j itself -- constant-border
// reads never route a gradient).  Interior voxels take a fast path over flat
// offsets.  Sums run in tap order, then coordinate order.
//
// The same 2-D tile machinery also runs the one-pass grey composites
// (morphological gradient and laplace, tm_grey_gradient / tm_grey_laplace).
#include <algorithm>
#include <cstring>
#include <vector>

#include "morph_tile.cuh"
#include "tm_common.cuh"
#include "vwalk.cuh"

namespace tmc {
namespace {

using namespace morph;

constexpr int kGradMaxDims = 3;
constexpr int kGradMaxTaps = 255;
constexpr uint8_t kNoTap = 255;
constexpr int kGradThreads = 256;

struct GradParams {
    int ndim, ntaps, mode;
    float cval;
    int64_t batch, numel_item;
    int shape[kGradMaxDims];
    int stride[kGradMaxDims];
    int halo[kGradMaxDims];  // max |offset| per axis
};

struct GradTaps {
    int32_t flat[kGradMaxTaps];
    int16_t off[kGradMaxTaps][kGradMaxDims];
    float val[kGradMaxTaps];
};

__device__ __forceinline__ void coords_of(int64_t sp, const GradParams &p, int *c) {
    for (int d = 0; d < kGradMaxDims; d++) {
        if (d < p.ndim) {
            c[d] = (int)(sp / p.stride[d]);
            sp -= (int64_t)c[d] * p.stride[d];
        } else {
            c[d] = 0;
        }
    }
}

template <bool MAX>
__global__ void __launch_bounds__(kGradThreads) morph_arg_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                                 uint8_t *__restrict__ arg, GradParams p,
                                                                 const __grid_constant__ GradTaps taps) {
    using Op = MorphOp<float, MAX>;
    const int64_t total = p.batch * p.numel_item;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = idx / p.numel_item;
        const int64_t sp = idx - item * p.numel_item;
        const float *src = in + item * p.numel_item;
        int c[kGradMaxDims];
        coords_of(sp, p, c);
        bool interior = true;
        for (int d = 0; d < p.ndim; d++) interior &= c[d] >= p.halo[d] && c[d] < p.shape[d] - p.halo[d];
        float best = Op::identity();
        int a = kNoTap;
        for (int t = 0; t < p.ntaps; t++) {
            float v;
            if (interior) {
                v = src[sp + taps.flat[t]];
            } else {
                int64_t f = 0;
                bool use_c = false;
                for (int d = 0; d < p.ndim; d++) {
                    const int m = map_coord(c[d] + taps.off[t][d], p.shape[d], p.mode);
                    if (m < 0) {
                        use_c = true;
                        break;
                    }
                    f += (int64_t)m * p.stride[d];
                }
                v = use_c ? p.cval : src[f];
            }
            v = Op::apply(v, taps.val[t]);
            if (MAX ? v > best : v < best) {
                best = v;
                a = t;
            }
        }
        out[idx] = best;
        arg[idx] = (uint8_t)a;
    }
}

__device__ __forceinline__ int pmod(int a, int m) {
    const int r = a % m;
    return r < 0 ? r + m : r;
}

// Coordinates y' in [lo, hi] (hi - lo + 1 == n) with map_coord(y') == c, as
// up to two ranges [a0, b0], [a1, b1] (an unused range has b < a).
struct Ranges {
    int a0, b0, a1, b1;
    __device__ __forceinline__ bool empty() const { return b0 < a0; }
    __device__ __forceinline__ int lo(int i) const { return i ? a1 : a0; }
    __device__ __forceinline__ int hi(int i) const { return i ? b1 : b0; }
};

__device__ __forceinline__ Ranges preimage_ranges(int c, int n, int mode, int lo, int hi) {
    Ranges r{0, -1, 0, -1};
    auto add = [&](int a, int b) {
        a = a > lo ? a : lo;
        b = b < hi ? b : hi;
        if (a > b) return;
        if (r.b0 < r.a0) {
            r.a0 = a;
            r.b0 = b;
        } else {
            r.a1 = a;
            r.b1 = b;
        }
    };
    switch (mode) {
    case TM_MODE_NEAREST:
        if (n == 1) add(lo, hi);
        else if (c == 0) add(lo, 0);
        else if (c == n - 1) add(n - 1, hi);
        else add(c, c);
        break;
    case TM_MODE_WRAP: {
        const int y = lo + pmod(c - lo, n);
        add(y, y);
        break;
    }
    case TM_MODE_REFLECT: {
        const int P = 2 * n;
        const int y1 = lo + pmod(c - lo, P), y2 = lo + pmod(-1 - c - lo, P);
        add(y1, y1);
        if (y2 != y1) add(y2, y2);
        break;
    }
    case TM_MODE_MIRROR: {
        if (n == 1) {
            add(lo, hi);
            break;
        }
        const int P = 2 * (n - 1);
        const int y1 = lo + pmod(c - lo, P), y2 = lo + pmod(-c - lo, P);
        add(y1, y1);
        if (y2 != y1) add(y2, y2);
        break;
    }
    default:  // constant: out-of-range reads are cval and carry no gradient
        add(c, c);
        break;
    }
    return r;
}

// grad_in of voxel sp (coordinates c) of one item: gather over taps and
// the coordinates' border preimages.
__device__ __forceinline__ float grad_voxel(const float *__restrict__ g, const uint8_t *__restrict__ a, int64_t sp,
                                            const int *c, const GradParams &p, const GradTaps &taps) {
    // interior: every tap's output o = j - off is in the image, and no
    // out-of-image coordinate a tap can reach maps onto j (mirror maps -h
    // onto h, hence the extra voxel)
    bool interior = true;
    for (int d = 0; d < p.ndim; d++) interior &= c[d] > p.halo[d] && c[d] < p.shape[d] - 1 - p.halo[d];
    float acc = 0.f;
    if (interior) {
        for (int t = 0; t < p.ntaps; t++) {
            const int64_t o = sp - taps.flat[t];
            if (a[o] == t) acc += g[o];
        }
        return acc;
    }
    for (int t = 0; t < p.ntaps; t++) {
        Ranges rg[kGradMaxDims];
        bool none = false;
        for (int d = 0; d < kGradMaxDims; d++) {
            if (d < p.ndim) {
                const int off = taps.off[t][d];
                rg[d] = preimage_ranges(c[d], p.shape[d], p.mode, off, off + p.shape[d] - 1);
                none |= rg[d].empty();
            } else {
                rg[d] = Ranges{0, 0, 0, -1};
            }
        }
        if (none) continue;
        for (int i0 = 0; i0 < 2; i0++)
            for (int y0 = rg[0].lo(i0); y0 <= rg[0].hi(i0); y0++)
                for (int i1 = 0; i1 < 2; i1++)
                    for (int y1 = rg[1].lo(i1); y1 <= rg[1].hi(i1); y1++)
                        for (int i2 = 0; i2 < 2; i2++)
                            for (int y2 = rg[2].lo(i2); y2 <= rg[2].hi(i2); y2++) {
                                const int y[3] = {y0, y1, y2};
                                int64_t o = 0;
                                for (int d = 0; d < p.ndim; d++) o += (int64_t)(y[d] - taps.off[t][d]) * p.stride[d];
                                if (a[o] == t) acc += g[o];
                            }
    }
    return acc;
}

// grad_voxel for a 2-D item, pixel (y, x) within the halo of the border:
// the same sums in the same order, ranges held in registers.
__device__ __forceinline__ float grad_pixel2d(const float *__restrict__ g, const uint8_t *__restrict__ a, int y, int x,
                                           const GradParams &p, const GradTaps &taps) {
    const int H = p.shape[0], W = p.shape[1];
    float acc = 0.f;
    for (int t = 0; t < p.ntaps; t++) {
        const int dy = taps.off[t][0], dx = taps.off[t][1];
        const Ranges ry = preimage_ranges(y, H, p.mode, dy, dy + H - 1);
        const Ranges rx = preimage_ranges(x, W, p.mode, dx, dx + W - 1);
#pragma unroll
        for (int i = 0; i < 2; i++)
            for (int yy = ry.lo(i); yy <= ry.hi(i); yy++)
#pragma unroll
                for (int k = 0; k < 2; k++)
                    for (int xx = rx.lo(k); xx <= rx.hi(k); xx++) {
                        const int64_t o = (int64_t)(yy - dy) * W + (xx - dx);
                        if (a[o] == t) acc += g[o];
                    }
    }
    return acc;
}

__global__ void __launch_bounds__(kGradThreads) morph_grad_kernel(const float *__restrict__ gout,
                                                                  const uint8_t *__restrict__ arg,
                                                                  float *__restrict__ gin, GradParams p,
                                                                  const __grid_constant__ GradTaps taps) {
    const int64_t total = p.batch * p.numel_item;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = idx / p.numel_item;
        const int64_t sp = idx - item * p.numel_item;
        int c[kGradMaxDims];
        coords_of(sp, p, c);
        gin[idx] = grad_voxel(gout + item * p.numel_item, arg + item * p.numel_item, sp, c, p, taps);
    }
}

// Frames of the float4 walkers (centred K x K flat boxes of 2-D items): the
// outputs (forward) or input pixels (backward) outside the walkers'
// rectangle, one thread each, with the per-voxel code above (same taps, same
// order).  Launched behind the walker (programmatic dependent launch); each
// finishes only once the walker has, so the stream's next work sees every
// output.
template <bool MAX>
__global__ void __launch_bounds__(256) arg_frame_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                        uint8_t *__restrict__ arg, GradParams p,
                                                        const __grid_constant__ GradTaps taps, vwalk::FrameRect fr) {
    using Op = MorphOp<float, MAX>;
    const int n = fr.count();
    for (int64_t item = blockIdx.y; item < p.batch; item += gridDim.y) {
        const float *src = in + item * p.numel_item;
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            int y, x;
            fr.at(k, y, x);
            float best = Op::identity();
            int a = kNoTap;
            for (int t = 0; t < p.ntaps; t++) {
                const int my = map_coord(y + taps.off[t][0], p.shape[0], p.mode);
                const int mx = map_coord(x + taps.off[t][1], p.shape[1], p.mode);
                const float v =
                    Op::apply((my < 0 || mx < 0) ? p.cval : src[(int64_t)my * p.shape[1] + mx], taps.val[t]);
                if (MAX ? v > best : v < best) {
                    best = v;
                    a = t;
                }
            }
            const int64_t o = item * p.numel_item + (int64_t)y * p.shape[1] + x;
            out[o] = best;
            arg[o] = (uint8_t)a;
        }
    }
    pdl_wait();
}

__global__ void __launch_bounds__(256) grad_frame_kernel(const float *__restrict__ gout,
                                                         const uint8_t *__restrict__ arg, float *__restrict__ gin,
                                                         GradParams p, const __grid_constant__ GradTaps taps,
                                                         vwalk::FrameRect fr) {
    const int n = fr.count();
    for (int64_t item = blockIdx.y; item < p.batch; item += gridDim.y) {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            int y, x;
            fr.at(k, y, x);
            gin[item * p.numel_item + (int64_t)y * p.shape[1] + x] =
                grad_pixel2d(gout + item * p.numel_item, arg + item * p.numel_item, y, x, p, taps);
        }
    }
    pdl_wait();
}

// The walkers' box: a full centred K x K footprint (K 3 or 5) of a 2-D item
// with one structure value (the backward needs no values); 0 otherwise.
int walk_box(const GradParams &p, const GradTaps &taps, const int64_t *sshape, const int64_t *origin,
             bool need_flat) {
    if (p.ndim != 2 || sshape[0] != sshape[1] || origin[0] != 0 || origin[1] != 0) return 0;
    const int k = (int)sshape[0];
    if ((k != 3 && k != 5) || p.ntaps != k * k) return 0;
    if (need_flat)
        for (int t = 1; t < p.ntaps; t++)
            if (std::memcmp(&taps.val[t], &taps.val[0], sizeof(float)) != 0) return 0;
    return k;
}

dim3 frame_grid(const vwalk::FrameRect &fr, int64_t batch) {
    const unsigned gy = (unsigned)std::min<int64_t>(batch, 65535);
    const int64_t want = std::max<int64_t>(1, (int64_t)sm_count() * 16 / gy);
    return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(fr.count(), 256), want)), gy);
}

// Forward with argument through the walkers; *done = false when they do not apply.
template <bool MAX>
int run_arg_walk(const float *in, float *out, uint8_t *arg, const GradParams &p, const GradTaps &taps, int k,
                 cudaStream_t s, bool *done) {
    *done = false;
    const int H = p.shape[0], W = p.shape[1];
    if (reinterpret_cast<uintptr_t>(arg) & 3) return TM_OK;
    static thread_local int cached_dev[2] = {-1, -1}, cached_blocks[2] = {0, 0};
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    const int ki = k == 3 ? 0 : 1;
    auto kern = k == 3 ? vwalk::vwalk_arg_kernel<MAX, 3> : vwalk::vwalk_arg_kernel<MAX, 5>;
    if (cached_dev[ki] != dev) {
        int per_sm = 0;
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, vwalk::kThreads, 0));
        cached_blocks[ki] = std::max(per_sm, 1) * sm_count();
        cached_dev[ki] = dev;
    }
    vwalk::Params wp;
    if (!vwalk::plan(H, W, p.batch, k, 1, in, out, (int64_t)cached_blocks[ki] * (vwalk::kThreads / 32), wp))
        return TM_OK;
    wp.sval = taps.val[0];
    *done = true;
    const int64_t blocks = std::min<int64_t>(ceil_div(wp.ntasks, vwalk::kThreads / 32), cached_blocks[ki]);
    if (wp.ntasks > 0)
        kern<<<(unsigned)blocks, vwalk::kThreads, 0, s>>>(in, out, reinterpret_cast<uint32_t *>(arg), wp);
    TM_LAUNCH_CHECK("vwalk_arg_kernel");
    const vwalk::FrameRect fr{H, W, wp.ry0, wp.ry1, 4, W - 4};
    TM_CHECK_CUDA(launch_pdl(arg_frame_kernel<MAX>, frame_grid(fr, p.batch), dim3(256), 0, s, in, out, arg, p, taps,
                             fr));
    return TM_OK;
}

// Backward through the walkers; *done = false when they do not apply.
int run_grad_walk(bool dilation, const float *gout, const uint8_t *arg, float *gin, const GradParams &p,
                  const GradTaps &taps, int k, cudaStream_t s, bool *done) {
    *done = false;
    const int H = p.shape[0], W = p.shape[1];
    if ((reinterpret_cast<uintptr_t>(arg) & 3) || (reinterpret_cast<uintptr_t>(gin) & 15)) return TM_OK;
    using KernT = void (*)(const float *, const uint32_t *, float *, vwalk::Params);
    const KernT kern = dilation ? (k == 3 ? vwalk::vwalk_grad_kernel<true, 3> : vwalk::vwalk_grad_kernel<true, 5>)
                                : (k == 3 ? vwalk::vwalk_grad_kernel<false, 3> : vwalk::vwalk_grad_kernel<false, 5>);
    static thread_local int cached_dev[4] = {-1, -1, -1, -1}, cached_blocks[4] = {0, 0, 0, 0};
    const int ki = (dilation ? 2 : 0) + (k == 3 ? 0 : 1);
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev[ki] != dev) {
        int per_sm = 0;
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, vwalk::kThreads, 0));
        cached_blocks[ki] = std::max(per_sm, 1) * sm_count();
        cached_dev[ki] = dev;
    }
    vwalk::Params wp;
    // input rows [h + 1, H - 1 - h): no border mapping routes a gradient there
    if (!vwalk::plan(H, W, p.batch, k, 1, gout, gin, (int64_t)cached_blocks[ki] * (vwalk::kThreads / 32), wp, 1))
        return TM_OK;
    wp.sval = 0.f;
    *done = true;
    const int64_t blocks = std::min<int64_t>(ceil_div(wp.ntasks, vwalk::kThreads / 32), cached_blocks[ki]);
    if (wp.ntasks > 0)
        kern<<<(unsigned)blocks, vwalk::kThreads, 0, s>>>(gout, reinterpret_cast<const uint32_t *>(arg), gin, wp);
    TM_LAUNCH_CHECK("vwalk_grad_kernel");
    const vwalk::FrameRect fr{H, W, wp.ry0, wp.ry1, 4, W - 4};
    TM_CHECK_CUDA(
        launch_pdl(grad_frame_kernel, frame_grid(fr, p.batch), dim3(256), 0, s, gout, arg, gin, p, taps, fr));
    return TM_OK;
}

// ------------------------------------------------------------- 2-D tiles
// 2-D items: 128 x 32 tiles, 256 threads, one column and 16 rows per
// thread.  The forward stages the input region the tile's taps read
// (borders mapped as in the forward operator); the backward stages
// (grad_out, argument) of the outputs its inputs can receive from.  Both run
// the taps in the outer loop over 16 unrolled rows, reading shared memory at
// a per-tap offset (computed on the host for the compile-time row pitch), so
// the per-output results and their order of evaluation are those of the
// per-voxel kernels above.  Backward pixels within the halo of the image
// border take grad_voxel.
constexpr int kT2W = 128, kT2H = 32, kT2Threads = 256, kT2Rows = 16;
constexpr int kT2MaxTaps = 64;
constexpr int kT2MaxExt = 30;  // tap offsets span at most 31 per axis

struct Taps2D {
    int n, min_dy, min_dx, ext_y, ext_x;  // offsets span [min, min + ext] per axis
    int soff[kT2MaxTaps];                 // shared-memory offset of tap t for row 0, column 0
    float val[kT2MaxTaps];
};

// Staging of a region of RH x RW elements (RW <= 160): warp w takes rows
// w, w + 8, ...; each lane issues the loads of RB rows x 5 column chunks
// before storing any of them, so a warp keeps up to 5 RB loads in flight
// instead of one.
constexpr int kT2ColChunks = 5;

template <int RB, class Load, class Store>
__device__ __forceinline__ void stage_region(int RH, int RW, Load load, Store store) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kT2Threads / 32;
    for (int rb = warp; rb < RH; rb += kWarps * RB) {
        decltype(load(0, 0)) v[RB][kT2ColChunks];
#pragma unroll
        for (int k = 0; k < RB; k++)
#pragma unroll
            for (int j = 0; j < kT2ColChunks; j++) {
                const int r = rb + kWarps * k, cc = lane + 32 * j;
                if (r < RH && cc < RW) v[k][j] = load(r, cc);
            }
#pragma unroll
        for (int k = 0; k < RB; k++)
#pragma unroll
            for (int j = 0; j < kT2ColChunks; j++) {
                const int r = rb + kWarps * k, cc = lane + 32 * j;
                if (r < RH && cc < RW) store(r, cc, v[k][j]);
            }
    }
}

template <bool MAX, int P>
__global__ void __launch_bounds__(kT2Threads, 4) morph_arg2d_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                                 uint8_t *__restrict__ arg, GradParams p,
                                                                 const __grid_constant__ Taps2D tp) {
    using Op = MorphOp<float, MAX>;
    extern __shared__ __align__(16) float stile[];
    const int H = p.shape[0], W = p.shape[1];
    const int RH = kT2H + tp.ext_y, RW = kT2W + tp.ext_x;
    const int x0 = blockIdx.x * kT2W, y0 = blockIdx.y * kT2H;
    const int gy0 = y0 + tp.min_dy, gx0 = x0 + tp.min_dx;
    const bool inner = gy0 >= 0 && gx0 >= 0 && gy0 + RH <= H && gx0 + RW <= W;
    const int c = threadIdx.x % kT2W, r0 = (threadIdx.x / kT2W) * kT2Rows;
    const int x = x0 + c;
    for (int64_t item = blockIdx.z; item < p.batch; item += gridDim.z) {
        const float *src = in + item * p.numel_item;
        const int mode = p.mode;
        const float cval = p.cval;
        auto put = [&](int r, int cc, float v) { stile[r * P + cc] = v; };
        if (inner)
            stage_region<2>(RH, RW, [&](int r, int cc) { return src[(int64_t)(gy0 + r) * W + gx0 + cc]; }, put);
        else
            stage_region<1>(
                RH, RW,
                [&](int r, int cc) {
                    const int my = map_coord(gy0 + r, H, mode), mx = map_coord(gx0 + cc, W, mode);
                    return (my < 0 || mx < 0) ? cval : src[(int64_t)my * W + mx];
                },
                put);
        __syncthreads();
        float best[kT2Rows];
        int ba[kT2Rows];
#pragma unroll
        for (int i = 0; i < kT2Rows; i++) {
            best[i] = Op::identity();
            ba[i] = kNoTap;
        }
        const float *base = stile + r0 * P + c;
        for (int t = 0; t < tp.n; t++) {
            const float *q = base + tp.soff[t];
            const float sv = tp.val[t];
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                const float v = Op::apply(q[i * P], sv);
                if (MAX ? v > best[i] : v < best[i]) {
                    best[i] = v;
                    ba[i] = t;
                }
            }
        }
        if (x < W) {
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                const int y = y0 + r0 + i;
                if (y < H) {
                    const int64_t o = item * p.numel_item + (int64_t)y * W + x;
                    out[o] = best[i];
                    arg[o] = (uint8_t)ba[i];
                }
            }
        }
        __syncthreads();
    }
}

template <int P>
__global__ void __launch_bounds__(kT2Threads, 3) morph_grad2d_kernel(const float *__restrict__ gout,
                                                                  const uint8_t *__restrict__ arg,
                                                                  float *__restrict__ gin, GradParams p,
                                                                  const __grid_constant__ GradTaps taps,
                                                                  const __grid_constant__ Taps2D tp) {
    extern __shared__ __align__(16) uint2 sga[];  // (grad_out bits, argument) per staged output
    const int H = p.shape[0], W = p.shape[1];
    // outputs o = j - off with off in [min, min + ext] per axis
    const int RH = kT2H + tp.ext_y, RW = kT2W + tp.ext_x;
    const int x0 = blockIdx.x * kT2W, y0 = blockIdx.y * kT2H;
    const int oy0 = y0 - tp.min_dy - tp.ext_y, ox0 = x0 - tp.min_dx - tp.ext_x;
    // every input of an inner tile is an interior voxel of grad_voxel
    const bool inner = y0 > p.halo[0] && y0 + kT2H - 1 < H - 1 - p.halo[0] && x0 > p.halo[1] &&
                       x0 + kT2W - 1 < W - 1 - p.halo[1];
    const int c = threadIdx.x % kT2W, r0 = (threadIdx.x / kT2W) * kT2Rows;
    const int x = x0 + c;
    // border pixels of an outer tile (within the halo of the image border)
    // as lists of rows and columns, so that all threads share their gathers:
    // (border rows x all columns) + (other rows x border columns)
    __shared__ int s_brow[kT2H], s_orow[kT2H], s_bcol[kT2W];
    __shared__ unsigned s_cmask[kT2W / 32];
    __shared__ int s_nb[2];
    const int ncols = min(kT2W, W - x0);
    int n_brow = 0, n_orow = 0, n_bcol = 0;
    if (!inner) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const unsigned lt = (1u << lane) - 1u;
        if (warp == 0) {
            const int y = y0 + lane;
            const bool in = y < H, br = in && (y <= p.halo[0] || y >= H - 1 - p.halo[0]);
            const unsigned mb = __ballot_sync(~0u, br), mo = __ballot_sync(~0u, in && !br);
            if (br) s_brow[__popc(mb & lt)] = lane;
            if (in && !br) s_orow[__popc(mo & lt)] = lane;
            if (lane == 0) {
                s_nb[0] = __popc(mb);
                s_nb[1] = __popc(mo);
            }
        }
        if (warp < kT2W / 32) {
            const int xc = x0 + warp * 32 + lane;
            const bool bc = xc < W && (xc <= p.halo[1] || xc >= W - 1 - p.halo[1]);
            s_cmask[warp] = __ballot_sync(~0u, bc);
        }
        __syncthreads();
        if (warp < kT2W / 32) {
            int before = 0;
            for (int w = 0; w < warp; w++) before += __popc(s_cmask[w]);
            if ((s_cmask[warp] >> lane) & 1u) s_bcol[before + __popc(s_cmask[warp] & lt)] = warp * 32 + lane;
        }
        n_brow = s_nb[0];
        n_orow = s_nb[1];
        for (int w = 0; w < kT2W / 32; w++) n_bcol += __popc(s_cmask[w]);
        __syncthreads();
    }
    for (int64_t item = blockIdx.z; item < p.batch; item += gridDim.z) {
        const float *g = gout + item * p.numel_item;
        const uint8_t *a = arg + item * p.numel_item;
        auto put = [&](int r, int cc, uint2 v) { sga[r * P + cc] = v; };
        if (inner)
            stage_region<2>(
                RH, RW,
                [&](int r, int cc) {
                    const int64_t k = (int64_t)(oy0 + r) * W + ox0 + cc;
                    return make_uint2(__float_as_uint(g[k]), a[k]);
                },
                put);
        else
            stage_region<1>(
                RH, RW,
                [&](int r, int cc) {
                    const int oy = oy0 + r, ox = ox0 + cc;
                    // outside the image: never a match
                    if ((unsigned)oy >= (unsigned)H || (unsigned)ox >= (unsigned)W) return make_uint2(0u, kNoTap);
                    const int64_t k = (int64_t)oy * W + ox;
                    return make_uint2(__float_as_uint(g[k]), a[k]);
                },
                put);
        __syncthreads();
        float acc[kT2Rows];
#pragma unroll
        for (int i = 0; i < kT2Rows; i++) acc[i] = 0.f;
        const uint2 *base = sga + r0 * P + c;
        for (int t = 0; t < tp.n; t++) {
            const uint2 *q = base + tp.soff[t];
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                const uint2 v = q[i * P];
                if (v.y == (unsigned)t) acc[i] += __uint_as_float(v.x);
            }
        }
        float *dst = gin + item * p.numel_item;
        if (x < W) {
            const bool col_edge = !inner && (x <= p.halo[1] || x >= W - 1 - p.halo[1]);
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                const int y = y0 + r0 + i;
                if (y < H && !(col_edge || (!inner && (y <= p.halo[0] || y >= H - 1 - p.halo[0]))))
                    dst[(int64_t)y * W + x] = acc[i];
            }
        }
        if (!inner) {
            const int n1 = n_brow * ncols, nb = n1 + n_orow * n_bcol;
            for (int k = threadIdx.x; k < nb; k += kT2Threads) {
                int y, xb;
                if (k < n1) {
                    y = y0 + s_brow[k / ncols];
                    xb = x0 + k % ncols;
                } else {
                    const int k2 = k - n1;
                    y = y0 + s_orow[k2 / n_bcol];
                    xb = x0 + s_bcol[k2 % n_bcol];
                }
                dst[(int64_t)y * W + xb] = grad_pixel2d(g, a, y, xb, p, taps);
            }
        }
        __syncthreads();
    }
}

// Row pitch (in staged elements) of the 2-D kernels for a tap extent.
int pitch2d(int ext_x) { return ext_x <= 8 ? 136 : 160; }

bool make_taps2d(const GradParams &p, const GradTaps &taps, bool backward, Taps2D *tp) {
    if (p.ndim != 2 || p.ntaps > kT2MaxTaps) return false;
    std::memset(tp, 0, sizeof(*tp));
    int mny = 0, mxy = 0, mnx = 0, mxx = 0;
    for (int t = 0; t < p.ntaps; t++) {
        mny = std::min(mny, (int)taps.off[t][0]);
        mxy = std::max(mxy, (int)taps.off[t][0]);
        mnx = std::min(mnx, (int)taps.off[t][1]);
        mxx = std::max(mxx, (int)taps.off[t][1]);
    }
    if (mxy - mny > kT2MaxExt || mxx - mnx > kT2MaxExt) return false;
    tp->n = p.ntaps;
    tp->min_dy = mny;
    tp->min_dx = mnx;
    tp->ext_y = mxy - mny;
    tp->ext_x = mxx - mnx;
    const int P = pitch2d(tp->ext_x);
    for (int t = 0; t < p.ntaps; t++) {
        const int dy = taps.off[t][0], dx = taps.off[t][1];
        // forward: input j = o + off at staged (row + dy - min_dy, col + dx - min_dx);
        // backward: output o = j - off at staged (row + ext_y + min_dy - dy, col + ext_x + min_dx - dx)
        tp->soff[t] = backward ? (tp->ext_y + mny - dy) * P + (tp->ext_x + mnx - dx) : (dy - mny) * P + (dx - mnx);
        tp->val[t] = taps.val[t];
    }
    return true;
}

// ------------------------------------------ fused 2-D composites, one pass
// morphological_gradient = dilation - erosion and morphological_laplace =
// (dilation + erosion) - 2 x of 2-D items (torchmorph/morphology/grey.py:
// 200-221, 268-289) in one read of the input and one write: the union of
// the dilation's and the erosion's tap regions is staged once; each tap list
// runs in raster order with a strict comparison (the first extremum wins,
// as in the forward-with-argument kernel, whose values equal the plain
// operators' bit for bit), and the combination is rounded like the
// reference's elementwise ops (no contraction).
struct Taps2DPair {
    int nd, ne, min_dy, min_dx, ext_y, ext_x, center;
    int soff_d[kT2MaxTaps], soff_e[kT2MaxTaps];
    float val_d[kT2MaxTaps], val_e[kT2MaxTaps];
};

template <int OP, int P, bool SYM>  // OP 0: gradient, 1: laplace; SYM: flat, same offsets for both
__global__ void __launch_bounds__(kT2Threads, 3) grey_composite2d_kernel(const float *__restrict__ in,
                                                                         float *__restrict__ out, GradParams p,
                                                                         const __grid_constant__ Taps2DPair tp) {
    extern __shared__ __align__(16) float stile[];
    const int H = p.shape[0], W = p.shape[1];
    const int RH = kT2H + tp.ext_y, RW = kT2W + tp.ext_x;
    const int x0 = blockIdx.x * kT2W, y0 = blockIdx.y * kT2H;
    const int gy0 = y0 + tp.min_dy, gx0 = x0 + tp.min_dx;
    const bool inner = gy0 >= 0 && gx0 >= 0 && gy0 + RH <= H && gx0 + RW <= W;
    const int c = threadIdx.x % kT2W, r0 = (threadIdx.x / kT2W) * kT2Rows;
    const int x = x0 + c;
    for (int64_t item = blockIdx.z; item < p.batch; item += gridDim.z) {
        const float *src = in + item * p.numel_item;
        const int mode = p.mode;
        const float cval = p.cval;
        auto put = [&](int r, int cc, float v) { stile[r * P + cc] = v; };
        if (inner)
            stage_region<2>(RH, RW, [&](int r, int cc) { return src[(int64_t)(gy0 + r) * W + gx0 + cc]; }, put);
        else
            stage_region<1>(
                RH, RW,
                [&](int r, int cc) {
                    const int my = map_coord(gy0 + r, H, mode), mx = map_coord(gx0 + cc, W, mode);
                    return (my < 0 || mx < 0) ? cval : src[(int64_t)my * W + mx];
                },
                put);
        __syncthreads();
        float dmax[kT2Rows], emin[kT2Rows];
#pragma unroll
        for (int i = 0; i < kT2Rows; i++) {
            dmax[i] = -INFINITY;
            emin[i] = INFINITY;
        }
        const float *base = stile + r0 * P + c;
        if (SYM) {
            // flat element whose dilation and erosion read the same offsets: one
            // load per offset feeds both extrema (their values do not depend on the
            // order); the flat taps' + 0 / - 0 is applied once at the end
            for (int t = 0; t < tp.nd; t++) {
                const float *q = base + tp.soff_d[t];
#pragma unroll
                for (int i = 0; i < kT2Rows; i++) {
                    const float v = q[i * P];
                    dmax[i] = fmaxf(dmax[i], v);
                    emin[i] = fminf(emin[i], v);
                }
            }
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                dmax[i] = __fadd_rn(dmax[i], 0.f);
                emin[i] = __fsub_rn(emin[i], 0.f);
            }
        } else {
            for (int t = 0; t < tp.nd; t++) {
                const float *q = base + tp.soff_d[t];
                const float sv = tp.val_d[t];
#pragma unroll
                for (int i = 0; i < kT2Rows; i++) {
                    const float v = q[i * P] + sv;
                    if (v > dmax[i]) dmax[i] = v;
                }
            }
            for (int t = 0; t < tp.ne; t++) {
                const float *q = base + tp.soff_e[t];
                const float sv = tp.val_e[t];
#pragma unroll
                for (int i = 0; i < kT2Rows; i++) {
                    const float v = q[i * P] - sv;
                    if (v < emin[i]) emin[i] = v;
                }
            }
        }
        if (x < W) {
#pragma unroll
            for (int i = 0; i < kT2Rows; i++) {
                const int y = y0 + r0 + i;
                if (y < H) {
                    float r;
                    if (OP == 0) r = __fsub_rn(dmax[i], emin[i]);
                    else r = __fsub_rn(__fadd_rn(dmax[i], emin[i]), __fmul_rn(2.f, base[tp.center + i * P]));
                    out[item * p.numel_item + (int64_t)y * W + x] = r;
                }
            }
        }
        __syncthreads();
    }
}

dim3 grid2d(const GradParams &p) {
    return dim3((unsigned)ceil_div(p.shape[1], kT2W), (unsigned)ceil_div(p.shape[0], kT2H),
                (unsigned)std::min<int64_t>(p.batch, 65535));
}

// Host: tap table of the operator (same construction as the forward).
int build_grad_taps(bool dilation, int64_t batch, int ndim, const int64_t *shape, const float *structure,
                    const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
                    GradParams *p, GradTaps *taps) {
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (ndim > kGradMaxDims) return fail(TM_ERR_UNSUPPORTED, "the grey backward supports 1-3 spatial dimensions");
    if (!sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "structure shape/origin is NULL");
    if (mode < 0 || mode > 4) return fail(TM_ERR_INVALID_ARGUMENT, "unknown border mode %d", mode);
    if (g.numel_item >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels");
    std::memset(p, 0, sizeof(*p));
    std::memset(taps, 0, sizeof(*taps));
    int64_t stotal = 1, sstride[kGradMaxDims];
    for (int d = 0; d < ndim; d++) {
        if (sshape[d] < 1 || sshape[d] > 4096)
            return fail(TM_ERR_INVALID_ARGUMENT, "structure size %d is %lld", d, (long long)sshape[d]);
        if (origin[d] < -(sshape[d] / 2) || origin[d] > (sshape[d] - 1) / 2)
            return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
        stotal *= sshape[d];
    }
    sstride[ndim - 1] = 1;
    for (int d = ndim - 2; d >= 0; d--) sstride[d] = sstride[d + 1] * sshape[d + 1];
    int n = 0;
    for (int64_t i = 0; i < stotal; i++) {
        if (footprint && !footprint[i]) continue;
        if (n == kGradMaxTaps)
            return fail(TM_ERR_UNSUPPORTED, "the grey backward supports at most %d active taps", kGradMaxTaps);
        int64_t rem = i, f = 0;
        for (int d = 0; d < ndim; d++) {
            const int64_t k = rem / sstride[d];
            rem %= sstride[d];
            const int64_t delta = k - (sshape[d] / 2 + origin[d]);
            const int off = (int)(dilation ? -delta : delta);
            taps->off[n][d] = (int16_t)off;
            f += (int64_t)off * g.stride[d];
            const int h = off < 0 ? -off : off;
            p->halo[d] = h > p->halo[d] ? h : p->halo[d];
        }
        taps->flat[n] = (int32_t)f;
        taps->val[n] = structure ? structure[i] : 0.f;
        n++;
    }
    if (n == 0) return fail(TM_ERR_INVALID_ARGUMENT, "footprint must contain at least one active position");
    p->ndim = ndim;
    p->ntaps = n;
    p->mode = mode;
    p->cval = cval;
    p->batch = batch;
    p->numel_item = g.numel_item;
    for (int d = 0; d < ndim; d++) {
        p->shape[d] = (int)shape[d];
        p->stride[d] = (int)g.stride[d];
    }
    return TM_OK;
}

unsigned grid_for(int64_t total) {
    const int64_t blocks = ceil_div(total, kGradThreads), cap = (int64_t)sm_count() * 16;
    return (unsigned)(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

template <bool MAX>
int run_arg(const float *in, float *out, uint8_t *arg, int64_t batch, int ndim, const int64_t *shape,
            const float *structure, const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode,
            float cval, cudaStream_t s) {
    if (!in || !out || !arg) return fail(TM_ERR_INVALID_ARGUMENT, "NULL input, output or argument buffer");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    GradParams p;
    GradTaps taps;
    int st = build_grad_taps(MAX, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval, &p, &taps);
    if (st != TM_OK) return st;
    if (const int k = walk_box(p, taps, sshape, origin, true)) {
        bool done = false;
        st = run_arg_walk<MAX>(in, out, arg, p, taps, k, s, &done);
        if (st != TM_OK || done) return st;
    }
    Taps2D tp;
    if (make_taps2d(p, taps, false, &tp)) {
        const int P = pitch2d(tp.ext_x);
        const size_t smem = (size_t)(kT2H + tp.ext_y) * P * sizeof(float);
        auto kern = P == 136 ? morph_arg2d_kernel<MAX, 136> : morph_arg2d_kernel<MAX, 160>;
        if (smem > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid2d(p), kT2Threads, smem, s>>>(in, out, arg, p, tp);
        TM_LAUNCH_CHECK("morph_arg2d_kernel");
        return TM_OK;
    }
    morph_arg_kernel<MAX><<<grid_for(p.batch * p.numel_item), kGradThreads, 0, s>>>(in, out, arg, p, taps);
    TM_LAUNCH_CHECK("morph_arg_kernel");
    return TM_OK;
}

int run_grad(bool dilation, const float *gout, const uint8_t *arg, float *gin, int64_t batch, int ndim,
             const int64_t *shape, const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode,
             cudaStream_t s) {
    if (!gout || !arg || !gin) return fail(TM_ERR_INVALID_ARGUMENT, "NULL gradient or argument buffer");
    if (gin == gout) return fail(TM_ERR_INVALID_ARGUMENT, "grad_input must not alias grad_output");
    GradParams p;
    GradTaps taps;
    int st = build_grad_taps(dilation, batch, ndim, shape, nullptr, footprint, sshape, origin, mode, 0.f, &p, &taps);
    if (st != TM_OK) return st;
    if (const int k = walk_box(p, taps, sshape, origin, false)) {
        bool done = false;
        st = run_grad_walk(dilation, gout, arg, gin, p, taps, k, s, &done);
        if (st != TM_OK || done) return st;
    }
    Taps2D tp;
    if (make_taps2d(p, taps, true, &tp)) {
        const int P = pitch2d(tp.ext_x);
        const size_t smem = (size_t)(kT2H + tp.ext_y) * P * sizeof(uint2);
        auto kern = P == 136 ? morph_grad2d_kernel<136> : morph_grad2d_kernel<160>;
        if (smem > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid2d(p), kT2Threads, smem, s>>>(gout, arg, gin, p, taps, tp);
        TM_LAUNCH_CHECK("morph_grad2d_kernel");
        return TM_OK;
    }
    morph_grad_kernel<<<grid_for(p.batch * p.numel_item), kGradThreads, 0, s>>>(gout, arg, gin, p, taps);
    TM_LAUNCH_CHECK("morph_grad_kernel");
    return TM_OK;
}

int run_composite(int op, const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                  const float *structure, const uint8_t *footprint, const int64_t *sshape, const int64_t *origin,
                  int mode, float cval, cudaStream_t s) {
    if (!in || !out) return fail(TM_ERR_INVALID_ARGUMENT, "NULL input or output");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    if (ndim != 2) return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take 2-D items");
    GradParams pd, pe;
    GradTaps td, te;
    int st = build_grad_taps(true, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval, &pd, &td);
    if (st != TM_OK) return st;
    st = build_grad_taps(false, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval, &pe, &te);
    if (st != TM_OK) return st;
    if (pd.ntaps > kT2MaxTaps) return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take up to %d taps", kT2MaxTaps);
    {
        // centred flat 3 x 3 / 5 x 5 box on 16-byte aligned rows: float4 register
        // walkers for the interior, one thread per output for the frame
        const int k = (int)sshape[0];
        bool flat = sshape[1] == k && (k == 3 || k == 5) && origin[0] == 0 && origin[1] == 0 && pd.ntaps == k * k;
        for (int t = 1; t < pd.ntaps && flat; t++) flat = std::memcmp(&td.val[t], &td.val[0], sizeof(float)) == 0;
        if (flat) {
            bool done = false;
            const int H = (int)shape[0], W = (int)shape[1];
            const float sv = td.val[0];
            if (op == 0)
                st = k == 3 ? vwalk::run<true, 1, 0, 3, vwalk::kGradient>(in, out, H, W, batch, mode, cval, sv, s, &done)
                            : vwalk::run<true, 1, 0, 5, vwalk::kGradient>(in, out, H, W, batch, mode, cval, sv, s, &done);
            else
                st = k == 3 ? vwalk::run<true, 1, 0, 3, vwalk::kLaplace>(in, out, H, W, batch, mode, cval, sv, s, &done)
                            : vwalk::run<true, 1, 0, 5, vwalk::kLaplace>(in, out, H, W, batch, mode, cval, sv, s, &done);
            if (st != TM_OK || done) return st;
        }
    }
    int mny = 0, mxy = 0, mnx = 0, mxx = 0;  // union of both tap regions (and the voxel itself)
    for (int t = 0; t < pd.ntaps; t++)
        for (const GradTaps *tt : {&td, &te}) {
            mny = std::min(mny, (int)tt->off[t][0]);
            mxy = std::max(mxy, (int)tt->off[t][0]);
            mnx = std::min(mnx, (int)tt->off[t][1]);
            mxx = std::max(mxx, (int)tt->off[t][1]);
        }
    if (mxy - mny > kT2MaxExt || mxx - mnx > kT2MaxExt)
        return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take tap offsets spanning up to %d", kT2MaxExt + 1);
    Taps2DPair *tp = new Taps2DPair;
    std::memset(tp, 0, sizeof(*tp));
    tp->nd = pd.ntaps;
    tp->ne = pe.ntaps;
    tp->min_dy = mny;
    tp->min_dx = mnx;
    tp->ext_y = mxy - mny;
    tp->ext_x = mxx - mnx;
    const int P = pitch2d(tp->ext_x);
    tp->center = (0 - mny) * P + (0 - mnx);
    for (int t = 0; t < pd.ntaps; t++) {
        tp->soff_d[t] = (td.off[t][0] - mny) * P + (td.off[t][1] - mnx);
        tp->val_d[t] = td.val[t];
        tp->soff_e[t] = (te.off[t][0] - mny) * P + (te.off[t][1] - mnx);
        tp->val_e[t] = te.val[t];
    }
    // flat element whose dilation and erosion offsets are the same set
    bool sym = true;
    for (int t = 0; t < pd.ntaps && sym; t++) sym = td.val[t] == 0.f;
    if (sym) {
        std::vector<int> od(pd.ntaps), oe(pd.ntaps);
        for (int t = 0; t < pd.ntaps; t++) {
            od[t] = tp->soff_d[t];
            oe[t] = tp->soff_e[t];
        }
        std::sort(od.begin(), od.end());
        std::sort(oe.begin(), oe.end());
        sym = od == oe;
    }
    const size_t smem = (size_t)(kT2H + tp->ext_y) * P * sizeof(float);
    using KernT = void (*)(const float *, float *, GradParams, const Taps2DPair);
    KernT kern;
    if (sym)
        kern = op == 0 ? (P == 136 ? grey_composite2d_kernel<0, 136, true> : grey_composite2d_kernel<0, 160, true>)
                       : (P == 136 ? grey_composite2d_kernel<1, 136, true> : grey_composite2d_kernel<1, 160, true>);
    else
        kern = op == 0 ? (P == 136 ? grey_composite2d_kernel<0, 136, false> : grey_composite2d_kernel<0, 160, false>)
                       : (P == 136 ? grey_composite2d_kernel<1, 136, false> : grey_composite2d_kernel<1, 160, false>);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        kern<<<grid2d(pd), kT2Threads, smem, s>>>(in, out, pd, *tp);
        e = cudaGetLastError();
    }
    delete tp;
    TM_CHECK_CUDA(e);
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" int tm_grey_erosion_arg(const float *in, float *out, uint8_t *arg, int64_t batch, int ndim,
                                   const int64_t *shape, const float *structure, const uint8_t *footprint,
                                   const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                   tm_stream_t stream) {
    return tmc::run_arg<false>(in, out, arg, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval,
                               (cudaStream_t)stream);
}

extern "C" int tm_grey_dilation_arg(const float *in, float *out, uint8_t *arg, int64_t batch, int ndim,
                                    const int64_t *shape, const float *structure, const uint8_t *footprint,
                                    const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                    tm_stream_t stream) {
    return tmc::run_arg<true>(in, out, arg, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval,
                              (cudaStream_t)stream);
}

extern "C" int tm_grey_erosion_backward(const float *grad_out, const uint8_t *arg, float *grad_in, int64_t batch,
                                        int ndim, const int64_t *shape, const uint8_t *footprint,
                                        const int64_t *sshape, const int64_t *origin, int mode, tm_stream_t stream) {
    return tmc::run_grad(false, grad_out, arg, grad_in, batch, ndim, shape, footprint, sshape, origin, mode,
                         (cudaStream_t)stream);
}

extern "C" int tm_grey_dilation_backward(const float *grad_out, const uint8_t *arg, float *grad_in, int64_t batch,
                                         int ndim, const int64_t *shape, const uint8_t *footprint,
                                         const int64_t *sshape, const int64_t *origin, int mode,
                                         tm_stream_t stream) {
    return tmc::run_grad(true, grad_out, arg, grad_in, batch, ndim, shape, footprint, sshape, origin, mode,
                         (cudaStream_t)stream);
}

extern "C" int tm_grey_gradient(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                                const float *structure, const uint8_t *footprint, const int64_t *sshape,
                                const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_composite(0, in, out, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval,
                              (cudaStream_t)stream);
}

extern "C" int tm_grey_laplace(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_composite(1, in, out, batch, ndim, shape, structure, footprint, sshape, origin, mode, cval,
                              (cudaStream_t)stream);
}
