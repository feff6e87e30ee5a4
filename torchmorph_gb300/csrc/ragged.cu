// Ragged batches: many 2-D images of different sizes, packed one after the
// other in one buffer, processed by ONE persistent launch per operator.
//
// A plan (built once per batch layout, reusable across operators and CUDA
// graph replays) holds a device table with one descriptor per image
// {element offset, H, W, first tile, tiles per row}.  The images' 128 x 32
// output tiles are numbered consecutively image after image; the persistent
// CTAs take tile numbers from an atomic counter in the plan (the work queue),
// find the image by binary search over the first-tile column, stage the
// tile plus halo in shared memory with the reference's border mapping and
// run the same tile code as the uniform-batch kernels (morph_tile.cuh).
// Per-image launches of small images are launch- and tail-bound; one launch
// over all tiles keeps every SM busy.
//
// Flat rectangular footprints use the separable row/column tile code
// (compile-time column walkers for 3x3, 5x5, 1x3, van Herk/Gil-Werman runs
// otherwise); other footprints (the binary cross, non-flat structures) use a
// tap loop over the staged tile.  Semantics are those of the uniform-batch
// operators (torchmorph/csrc/grey_kernel.cu:101-170, binary_kernel.cu:56-127)
// applied to each image on its own.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "bitmorph.cuh"
#include "morph_tile.cuh"
#include "tile_queue.cuh"
#include "tm_common.cuh"

namespace tmc {
namespace {

using namespace morph;

struct RaggedItem {
    int64_t off;  // first element of the image in the packed input and output
    int H, W;
    int tile_begin;  // number of the image's first tile
    int tiles_x;
    int pad[2];
};

struct PlanHeader {
    int queue;  // next tile to hand out (reset before every launch)
    int ntiles;
    int nitems;
    int pad[61];
};
static_assert(sizeof(PlanHeader) == 256, "plan header is 256 bytes");

struct RaggedWindow {
    int kh, kw, lo_y, lo_x, mode;
    float cval, sval;
};

constexpr int kMaxTaps = 256;

struct RaggedTaps {
    int n;
    int min_y, min_x, ext_y, ext_x;  // halo origin and extent of the staged region
    int8_t dy[kMaxTaps], dx[kMaxTaps];
    float val[kMaxTaps];
};

// Stage rows [gy0, gy0 + RH) x columns [gx0, gx0 + RW) of one image into
// shared memory (row stride ld), mapping out-of-image coordinates.  Warp w
// takes rows w, w + 8, ...; a lane issues the loads of 2 rows x up to 5
// column chunks before it stores any, so a warp keeps many loads in flight
// (tiles inside the image; border tiles map every coordinate, one row at a
// time).
template <typename T>
__device__ __forceinline__ void stage_tile(const T *src, int H, int W, int gy0, int gx0, int RH, int RW, int ld,
                                           int mode, T cval, T *tile) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int nwarps = kFlatThreads / 32, RB = 2, NC = 5;
    const bool interior = gy0 >= 0 && gx0 >= 0 && gy0 + RH <= H && gx0 + RW <= W;
    if (interior) {
        for (int rb = warp; rb < RH; rb += nwarps * RB)
            for (int cb = 0; cb < RW; cb += 32 * NC) {
                T v[RB][NC];
#pragma unroll
                for (int k = 0; k < RB; k++)
#pragma unroll
                    for (int j = 0; j < NC; j++) {
                        const int r = rb + nwarps * k, c = cb + lane + 32 * j;
                        if (r < RH && c < RW) v[k][j] = src[(int64_t)(gy0 + r) * W + gx0 + c];
                    }
#pragma unroll
                for (int k = 0; k < RB; k++)
#pragma unroll
                    for (int j = 0; j < NC; j++) {
                        const int r = rb + nwarps * k, c = cb + lane + 32 * j;
                        if (r < RH && c < RW) tile[r * ld + c] = v[k][j];
                    }
            }
        return;
    }
    for (int r = warp; r < RH; r += nwarps) {
        const int my = map_coord(gy0 + r, H, mode);
        for (int cb = 0; cb < RW; cb += 32 * NC) {
            T v[NC];
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const int c = cb + lane + 32 * j;
                if (c < RW) {
                    const int mx = map_coord(gx0 + c, W, mode);
                    v[j] = (my < 0 || mx < 0) ? cval : src[(int64_t)my * W + mx];
                }
            }
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const int c = cb + lane + 32 * j;
                if (c < RW) tile[r * ld + c] = v[j];
            }
        }
    }
}

template <typename T, bool MAX, int KH, int KW>
__global__ void __launch_bounds__(kFlatThreads) ragged_flat_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                                   PlanHeader *hdr, const RaggedItem *__restrict__ items,
                                                                   RaggedWindow w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_slot[2];
    __shared__ int s_tb[kQueueCache];
    const int RH = kTileH + w.kh - 1, RW = kTileW + w.kw - 1;
    const int RWp = stage_pitch(w.kw);
    T *tile = reinterpret_cast<T *>(smem_raw);
    T *rows = tile + RH * RWp;
    TileQueue<RaggedItem> q{&hdr->queue, hdr->ntiles, hdr->nitems, items, s_tb, s_slot, 0};
    q.init();
    while (q.take()) {
        const int t = s_slot[0], item = s_slot[1];
        const RaggedItem it = items[item];
        const int local = t - it.tile_begin;
        const int ty = local / it.tiles_x, tx = local - ty * it.tiles_x;
        const int x0 = tx * kTileW, y0 = ty * kTileH;
        Flat2DParams p;
        p.H = it.H;
        p.W = it.W;
        p.kh = w.kh;
        p.kw = w.kw;
        p.lo_y = w.lo_y;
        p.lo_x = w.lo_x;
        p.mode = w.mode;
        p.batch = 1;
        p.cval = w.cval;
        p.sval = w.sval;
        stage_tile<T>(in + it.off, it.H, it.W, y0 + w.lo_y, x0 + w.lo_x, RH, RW, RWp, w.mode, (T)w.cval, tile);
        __syncthreads();
        tile_compute<T, MAX, KH, KW>(tile, RWp, rows, p, out + it.off, x0, y0);
        __syncthreads();
    }
}

// Tap loop over a staged tile.  With a compile-time row pitch P (taps
// spanning at most 33 rows and P - 128 + 1 columns) a thread owns one column
// and 16 rows, runs the taps in the outer loop at one shared-memory offset
// each, and keeps the 16 results in registers; P = 0 is the general case
// (one output at a time).  Per output the taps combine in the same order.
template <typename T, bool MAX, int P>
__global__ void __launch_bounds__(kFlatThreads) ragged_taps_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                                   PlanHeader *hdr, const RaggedItem *__restrict__ items,
                                                                   const __grid_constant__ RaggedTaps taps, int mode,
                                                                   float cval) {
    using Op = MorphOp<T, MAX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_slot[2];
    __shared__ int s_tb[kQueueCache];
    const int RH = kTileH + taps.ext_y, RW = kTileW + taps.ext_x;
    const int ld = P ? P : RW;
    T *tile = reinterpret_cast<T *>(smem_raw);
    TileQueue<RaggedItem> q{&hdr->queue, hdr->ntiles, hdr->nitems, items, s_tb, s_slot, 0};
    q.init();
    while (q.take()) {
        const int t = s_slot[0], item = s_slot[1];
        const RaggedItem it = items[item];
        const int local = t - it.tile_begin;
        const int ty = local / it.tiles_x, tx = local - ty * it.tiles_x;
        const int x0 = tx * kTileW, y0 = ty * kTileH;
        stage_tile<T>(in + it.off, it.H, it.W, y0 + taps.min_y, x0 + taps.min_x, RH, RW, ld, mode, (T)cval, tile);
        __syncthreads();
        T *dst = out + it.off;
        if constexpr (P != 0) {
            constexpr int kRows = kTileH * kTileW / kFlatThreads;  // 16
            const int c = threadIdx.x % kTileW, r0 = (threadIdx.x / kTileW) * kRows;
            T acc[kRows];
#pragma unroll
            for (int i = 0; i < kRows; i++) acc[i] = Op::identity();
            const T *base = tile + r0 * P + c;
            for (int k = 0; k < taps.n; k++) {
                const T *q = base + (taps.dy[k] - taps.min_y) * P + (taps.dx[k] - taps.min_x);
                const float sv = taps.val[k];
#pragma unroll
                for (int i = 0; i < kRows; i++) acc[i] = Op::combine(acc[i], Op::apply(q[i * P], sv));
            }
            const int gx = x0 + c;
            if (gx < it.W) {
#pragma unroll
                for (int i = 0; i < kRows; i++) {
                    const int gy = y0 + r0 + i;
                    if (gy < it.H) dst[(int64_t)gy * it.W + gx] = acc[i];
                }
            }
        } else {
            for (int e = threadIdx.x; e < kTileH * kTileW; e += kFlatThreads) {
                const int r = e / kTileW, c = e % kTileW;
                const int gy = y0 + r, gx = x0 + c;
                if (gy >= it.H || gx >= it.W) continue;
                T acc = Op::identity();
                for (int k = 0; k < taps.n; k++)
                    acc = Op::combine(acc, Op::apply(tile[(r + taps.dy[k] - taps.min_y) * RW + c + taps.dx[k] - taps.min_x],
                                                     taps.val[k]));
                dst[(int64_t)gy * it.W + gx] = acc;
            }
        }
        __syncthreads();
    }
}

// Persistent grid: resident CTAs per SM x SMs, cached per kernel and size.
template <typename K>
int persistent_grid(K kernel, size_t smem, int *grid) {
    struct Entry {
        const void *fn;
        size_t smem;
        int dev, ctas;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const Entry &e : cache)
            if (e.fn == (const void *)kernel && e.smem == smem && e.dev == dev) {
                *grid = e.ctas;
                return TM_OK;
            }
    }
    // the attribute allows the largest tile on the device (minus the kernel's static
    // shared memory), so that a later launch with a larger tile than a cached one fits
    int optin = 0;
    TM_CHECK_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    TM_CHECK_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const int max_dynamic = optin - (int)fa.sharedSizeBytes;
    if (smem > (size_t)max_dynamic)
        return fail(TM_ERR_UNSUPPORTED, "ragged tile needs %zu bytes of shared memory", smem);
    TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic));
    int per_sm = 0;
    TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kFlatThreads, smem));
    if (per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "ragged tile does not fit on an SM");
    const int ctas = per_sm * sm_count();
    std::lock_guard<std::mutex> lock(mu);
    cache.push_back({(const void *)kernel, smem, dev, ctas});
    *grid = ctas;
    return TM_OK;
}

template <typename T, bool MAX, int KH, int KW>
int launch_ragged_flat(const T *in, T *out, PlanHeader *hdr, const RaggedItem *items, const RaggedWindow &w,
                       cudaStream_t s) {
    const int RH = kTileH + w.kh - 1, RWp = stage_pitch(w.kw);
    const size_t smem = (size_t)RH * RWp * sizeof(T) + (KH == 0 ? (size_t)RH * kRowsPitch * sizeof(T) : 0);
    auto kernel = ragged_flat_kernel<T, MAX, KH, KW>;
    int grid = 0;
    int st = persistent_grid(kernel, smem, &grid);
    if (st != TM_OK) return st;
    TM_CHECK_CUDA(cudaMemsetAsync(&hdr->queue, 0, sizeof(int), s));
    kernel<<<grid, kFlatThreads, smem, s>>>(in, out, hdr, items, w);
    TM_LAUNCH_CHECK("ragged_flat_kernel");
    return TM_OK;
}

template <typename T, bool MAX>
int run_ragged(const T *in, T *out, const void *plan, size_t plan_bytes, int64_t n_items, const float *structure,
               const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
               cudaStream_t s) {
    if (!in || !out || !plan) return fail(TM_ERR_INVALID_ARGUMENT, "NULL input, output or plan");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    if (n_items < 1) return fail(TM_ERR_INVALID_ARGUMENT, "a ragged batch needs at least one image");
    if (plan_bytes < sizeof(PlanHeader) + (size_t)n_items * sizeof(RaggedItem))
        return fail(TM_ERR_WORKSPACE, "ragged plan buffer too small for %lld images", (long long)n_items);
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    if (!sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "structure shape/origin is NULL");
    if (mode < 0 || mode > 4) return fail(TM_ERR_INVALID_ARGUMENT, "unknown border mode %d", mode);
    for (int d = 0; d < 2; d++) {
        if (sshape[d] < 1 || sshape[d] > 255)
            return fail(TM_ERR_UNSUPPORTED, "ragged structure sizes must be 1..255, got %lld", (long long)sshape[d]);
        if (origin[d] < -(sshape[d] / 2) || origin[d] > (sshape[d] - 1) / 2)
            return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
    }
    if constexpr (sizeof(T) == 1) {  // binary: bit-packed tiles (the same plan)
        bool done = false;
        const int st = bitmorph_ragged(MAX ? 1 : 0, in, out, plan, footprint, sshape, origin, cval != 0.0f, s, &done);
        if (st != TM_OK || done) return st;
    }
    auto *hdr = static_cast<PlanHeader *>(const_cast<void *>(plan));
    auto *items = reinterpret_cast<const RaggedItem *>(static_cast<const unsigned char *>(plan) + sizeof(PlanHeader));
    const int kh = (int)sshape[0], kw = (int)sshape[1];
    const int cy = kh / 2 + (int)origin[0], cx = kw / 2 + (int)origin[1];
    // taps (torchmorph/csrc/grey_kernel.cu:271-291): erosion reads x + (k - c), dilation x - (k - c)
    RaggedTaps taps;
    std::memset(&taps, 0, sizeof(taps));
    bool uniform = true;
    float first = 0.f;
    int n = 0;
    for (int ky = 0; ky < kh; ky++)
        for (int kx = 0; kx < kw; kx++) {
            const int i = ky * kw + kx;
            if (footprint && !footprint[i]) continue;
            const float v = structure ? structure[i] : 0.f;
            if (n == 0) first = v;
            uniform &= std::memcmp(&v, &first, sizeof(float)) == 0;
            if (n < kMaxTaps) {
                const int dy = MAX ? -(ky - cy) : ky - cy, dx = MAX ? -(kx - cx) : kx - cx;
                taps.dy[n] = (int8_t)dy;
                taps.dx[n] = (int8_t)dx;
                taps.val[n] = v;
            }
            n++;
        }
    if (n == 0) return fail(TM_ERR_INVALID_ARGUMENT, "footprint must contain at least one active position");
    if (n == kh * kw && uniform) {
        RaggedWindow w;
        w.kh = kh;
        w.kw = kw;
        w.lo_y = MAX ? cy - kh + 1 : -cy;
        w.lo_x = MAX ? cx - kw + 1 : -cx;
        w.mode = mode;
        w.cval = cval;
        w.sval = first;
        if (kh == 3 && kw == 3) return launch_ragged_flat<T, MAX, 3, 3>(in, out, hdr, items, w, s);
        if (kh == 5 && kw == 5) return launch_ragged_flat<T, MAX, 5, 5>(in, out, hdr, items, w, s);
        if (kh == 1 && kw == 3) return launch_ragged_flat<T, MAX, 1, 3>(in, out, hdr, items, w, s);
        return launch_ragged_flat<T, MAX, 0, 0>(in, out, hdr, items, w, s);
    }
    if (n > kMaxTaps) return fail(TM_ERR_UNSUPPORTED, "ragged footprints are limited to %d active taps", kMaxTaps);
    taps.n = n;
    int min_y = 0, max_y = 0, min_x = 0, max_x = 0;
    for (int k = 0; k < n; k++) {
        min_y = std::min(min_y, (int)taps.dy[k]);
        max_y = std::max(max_y, (int)taps.dy[k]);
        min_x = std::min(min_x, (int)taps.dx[k]);
        max_x = std::max(max_x, (int)taps.dx[k]);
    }
    taps.min_y = min_y;
    taps.min_x = min_x;
    taps.ext_y = max_y - min_y;
    taps.ext_x = max_x - min_x;
    // compile-time pitch for taps spanning up to 33 rows and 9 or 33 columns
    const int P = taps.ext_y > 32 ? 0 : taps.ext_x <= 8 ? 136 : taps.ext_x <= 32 ? 160 : 0;
    const size_t smem = (size_t)(kTileH + taps.ext_y) * (P ? P : kTileW + taps.ext_x) * sizeof(T);
    auto kernel = P == 136 ? ragged_taps_kernel<T, MAX, 136>
                  : P == 160 ? ragged_taps_kernel<T, MAX, 160>
                             : ragged_taps_kernel<T, MAX, 0>;
    int grid = 0;
    int st = persistent_grid(kernel, smem, &grid);
    if (st != TM_OK) return st;
    TM_CHECK_CUDA(cudaMemsetAsync(&hdr->queue, 0, sizeof(int), s));
    kernel<<<grid, kFlatThreads, smem, s>>>(in, out, hdr, items, taps, mode, cval);
    TM_LAUNCH_CHECK("ragged_taps_kernel");
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" size_t tm_ragged_plan_size(int64_t n_items) {
    if (n_items < 1) return 0;
    return sizeof(tmc::PlanHeader) + (size_t)n_items * sizeof(tmc::RaggedItem);
}

extern "C" int tm_ragged_plan(int64_t n_items, const int64_t *heights, const int64_t *widths, const int64_t *offsets,
                              void *plan, size_t plan_bytes, tm_stream_t stream) {
    using namespace tmc;
    if (n_items < 1 || n_items > (1 << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "n_items must be 1..2^30");
    if (!heights || !widths || !offsets || !plan) return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (plan_bytes < tm_ragged_plan_size(n_items))
        return fail(TM_ERR_WORKSPACE, "ragged plan needs %zu bytes", tm_ragged_plan_size(n_items));
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    std::vector<unsigned char> host(tm_ragged_plan_size(n_items), 0);
    auto *hdr = reinterpret_cast<PlanHeader *>(host.data());
    auto *items = reinterpret_cast<RaggedItem *>(host.data() + sizeof(PlanHeader));
    int64_t tiles = 0;
    for (int64_t i = 0; i < n_items; i++) {
        const int64_t H = heights[i], W = widths[i];
        if (H < 1 || W < 1) return fail(TM_ERR_INVALID_ARGUMENT, "image %lld is empty", (long long)i);
        if (H * W >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "image %lld has 2^31 or more pixels", (long long)i);
        if (offsets[i] < 0) return fail(TM_ERR_INVALID_ARGUMENT, "negative offset for image %lld", (long long)i);
        items[i].off = offsets[i];
        items[i].H = (int)H;
        items[i].W = (int)W;
        items[i].tiles_x = (int)ceil_div(W, kTileW);
        items[i].tile_begin = (int)tiles;
        tiles += (int64_t)items[i].tiles_x * ceil_div(H, kTileH);
        if (tiles >= ((int64_t)1 << 31) - 65536) return fail(TM_ERR_TOO_LARGE, "too many tiles in one ragged batch");
    }
    hdr->queue = 0;
    hdr->ntiles = (int)tiles;
    hdr->nitems = (int)n_items;
    // pageable source: the call returns once the bytes are staged, so the
    // host vector may go away
    TM_CHECK_CUDA(cudaMemcpyAsync(plan, host.data(), host.size(), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return TM_OK;
}

extern "C" int tm_ragged_grey_erosion(const float *in, float *out, const void *plan, size_t plan_bytes,
                                      int64_t n_items, const float *structure, const uint8_t *footprint,
                                      const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                      tm_stream_t stream) {
    return tmc::run_ragged<float, false>(in, out, plan, plan_bytes, n_items, structure, footprint, sshape, origin,
                                         mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_ragged_grey_dilation(const float *in, float *out, const void *plan, size_t plan_bytes,
                                       int64_t n_items, const float *structure, const uint8_t *footprint,
                                       const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                       tm_stream_t stream) {
    return tmc::run_ragged<float, true>(in, out, plan, plan_bytes, n_items, structure, footprint, sshape, origin,
                                        mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_ragged_binary_erosion(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                        int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                        const int64_t *origin, int border_value, tm_stream_t stream) {
    return tmc::run_ragged<uint8_t, false>(in, out, plan, plan_bytes, n_items, nullptr, structure, sshape, origin,
                                           TM_MODE_CONSTANT, border_value ? 1.f : 0.f, (cudaStream_t)stream);
}

extern "C" int tm_ragged_binary_dilation(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                         int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                         const int64_t *origin, int border_value, tm_stream_t stream) {
    return tmc::run_ragged<uint8_t, true>(in, out, plan, plan_bytes, n_items, nullptr, structure, sshape, origin,
                                          TM_MODE_CONSTANT, border_value ? 1.f : 0.f, (cudaStream_t)stream);
}
