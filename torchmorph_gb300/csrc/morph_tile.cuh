// Device building blocks shared by the uniform-batch morphology kernels
// (morphology.cu) and the ragged-batch ones (ragged.cu): operator traits, the
// reference's border mapping, and the separable min/max of one staged 2-D
// tile.
#pragma once

#include <cmath>

#include "tm_common.cuh"

namespace tmc {
namespace morph {

}  // namespace morph

// 3-D items on shared-memory tiles (stencil3d.cu).  Sets *done = false and
// returns TM_OK, launching nothing, when the element does not fit the tile
// kernel (more than 1024 active taps, or a tile beyond shared memory).
template <typename T, bool MAX>
int stencil3d_uniform(const T *in, T *out, int64_t batch, const int64_t *shape, const float *structure,
                      const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
                      cudaStream_t s, bool *done);

namespace morph {

// ---------------------------------------------------------------- op traits
template <typename T, bool MAX>
struct MorphOp;

template <>
struct MorphOp<float, false> {  // grey erosion
    __device__ __forceinline__ static float identity() { return INFINITY; }
    __device__ __forceinline__ static float combine(float a, float b) { return fminf(a, b); }
    __device__ __forceinline__ static float apply(float v, float s) { return v - s; }
};
template <>
struct MorphOp<float, true> {  // grey dilation
    __device__ __forceinline__ static float identity() { return -INFINITY; }
    __device__ __forceinline__ static float combine(float a, float b) { return fmaxf(a, b); }
    __device__ __forceinline__ static float apply(float v, float s) { return v + s; }
};
template <>
struct MorphOp<uint8_t, false> {  // binary erosion (AND)
    __device__ __forceinline__ static uint8_t identity() { return 1; }
    __device__ __forceinline__ static uint8_t combine(uint8_t a, uint8_t b) { return a < b ? a : b; }
    __device__ __forceinline__ static uint8_t apply(uint8_t v, float) { return v; }
};
template <>
struct MorphOp<uint8_t, true> {  // binary dilation (OR)
    __device__ __forceinline__ static uint8_t identity() { return 0; }
    __device__ __forceinline__ static uint8_t combine(uint8_t a, uint8_t b) { return a > b ? a : b; }
    __device__ __forceinline__ static uint8_t apply(uint8_t v, float) { return v; }
};

// Border mapping (torchmorph/csrc/grey_kernel.cu:63-97).  Returns -1 when
// the constant value must be used.
__host__ __device__ __forceinline__ int map_coord(int c, int n, int mode) {
    if ((unsigned)c < (unsigned)n) return c;
    switch (mode) {
    case TM_MODE_NEAREST:
        return c < 0 ? 0 : n - 1;
    case TM_MODE_REFLECT: {
        int period = 2 * n;
        int r = c % period;
        if (r < 0) r += period;
        return r >= n ? period - 1 - r : r;
    }
    case TM_MODE_MIRROR: {
        int period = 2 * (n - 1);
        if (period <= 0) return 0;
        int r = c % period;
        if (r < 0) r += period;
        return r >= n ? period - r : r;
    }
    case TM_MODE_WRAP: {
        int r = c % n;
        return r < 0 ? r + n : r;
    }
    default:
        return -1;
    }
}

// ------------------------------------------------------------ flat 2-D tile
constexpr int kTileW = 128;
constexpr int kTileH = 32;
constexpr int kFlatThreads = 256;
constexpr int kRun = 8;
// Row pitch of the row-pass buffer: odd, so that threads writing the same
// column of consecutive rows hit different banks.
constexpr int kRowsPitch = kTileW + 1;

// Row pitch of a staged tile for a window of kw columns: room for full runs
// past the last column, made odd so that consecutive rows start in different
// banks (the row pass gives consecutive rows to consecutive threads).
__host__ __device__ inline int stage_pitch(int kw) { return (kTileW + kw - 1 + (kRun - 1)) | 1; }

struct Flat2DParams {
    int H, W;        // item size (1-D items use H = 1)
    int kh, kw;      // window
    int lo_y, lo_x;  // window of output (y, x) covers rows y+lo_y .. y+lo_y+kh-1
    int mode;
    int64_t batch;
    float cval;
    float sval;  // constant structure value (flat footprint)
};


// One run of kRun consecutive outputs of a 1-D sliding window of width k
// over src[0 .. kRun + k - 2] (src elements `step` apart in shared memory).
template <typename T, bool MAX>
__device__ __forceinline__ void window_run(const T *src, int step, int k, T *res) {
    using Op = MorphOp<T, MAX>;
    if (k <= kRun) {
#pragma unroll
        for (int j = 0; j < kRun; j++) {
            T acc = src[j * step];
            for (int t = 1; t < k; t++) acc = Op::combine(acc, src[(j + t) * step]);
            res[j] = acc;
        }
        return;
    }
    // van Herk/Gil-Werman split: every window of the run contains the
    // block [kRun-1, k-1]; the left part is a suffix of [j, kRun-2] and the
    // right part a prefix of [k, j+k-1].
    T mid = src[(kRun - 1) * step];
    for (int t = kRun; t < k; t++) mid = Op::combine(mid, src[t * step]);
    T suf[kRun];
    suf[kRun - 1] = mid;
#pragma unroll
    for (int j = kRun - 2; j >= 0; j--) suf[j] = Op::combine(src[j * step], suf[j + 1]);
    T pre = src[k * step];
    res[0] = suf[0];
#pragma unroll
    for (int j = 1; j < kRun; j++) {
        res[j] = Op::combine(suf[j], pre);
        if (j + 1 < kRun) pre = Op::combine(pre, src[(k + j) * step]);
    }
}

// Row pass then column pass of one staged tile: `tile` points at the first
// input column the tile needs (row stride ld), `rows` receives the row-pass
// result (RH x kTileW at pitch kRowsPitch); outputs go to dst at (y0.., x0..).
template <typename T, bool MAX>
__device__ __forceinline__ void flat_tile_compute(const T *tile, int ld, T *rows, const Flat2DParams &p, T *dst,
                                                  int x0, int y0) {
    using Op = MorphOp<T, MAX>;
    const int RH = kTileH + p.kh - 1;
    if (p.kw <= kRun) {
        // narrow windows: one output per thread, adjacent lanes on adjacent
        // columns, so every shared-memory access of a warp is conflict free
        for (int w = threadIdx.x; w < RH * kTileW; w += kFlatThreads) {
            const int r = w / kTileW, c = w % kTileW;
            const T *src = tile + r * ld + c;
            T acc = src[0];
            for (int t = 1; t < p.kw; t++) acc = Op::combine(acc, src[t]);
            rows[r * kRowsPitch + c] = acc;
        }
    } else {
        const int runs_per_row = kTileW / kRun;
        // an odd row stride: consecutive threads take the same run of consecutive
        // rows (conflict-free); otherwise consecutive runs of one row
        const bool by_rows = (ld & 1) != 0;
        for (int w = threadIdx.x; w < RH * runs_per_row; w += kFlatThreads) {
            const int r = by_rows ? w % RH : w / runs_per_row;
            const int c = (by_rows ? w / RH : w % runs_per_row) * kRun;
            T res[kRun];
            window_run<T, MAX>(tile + r * ld + c, 1, p.kw, res);
#pragma unroll
            for (int j = 0; j < kRun; j++) rows[r * kRowsPitch + c + j] = res[j];
        }
    }
    __syncthreads();
    const int runs_per_col = kTileH / kRun;
    for (int w = threadIdx.x; w < kTileW * runs_per_col; w += kFlatThreads) {
        int c = w % kTileW, r = (w / kTileW) * kRun;
        int gx = x0 + c;
        // kTileH is a multiple of kRun, so the run reads rows
        // r .. r + kRun + kh - 2 <= RH - 1: always inside the row buffer
        T res[kRun];
        window_run<T, MAX>(rows + r * kRowsPitch + c, kRowsPitch, p.kh, res);
        if (gx < p.W) {
#pragma unroll
            for (int j = 0; j < kRun; j++) {
                int gy = y0 + r + j;
                if (gy < p.H) __stcs(dst + (int64_t)gy * p.W + gx, MorphOp<T, MAX>::apply(res[j], p.sval));
            }
        }
    }
}

// Compile-time window (KH x KW): each thread walks down one column of the
// tile (two threads per column, 16 output rows each), computes every input
// row's horizontal minimum/maximum once and keeps the last KH of them in
// registers, so one pass produces the outputs without a row buffer.
// Adjacent lanes own adjacent columns: conflict-free shared-memory reads and
// 128-byte global stores.
template <typename T, bool MAX, int KH, int KW>
__device__ __forceinline__ void flat_tile_walk(const T *tile, int ld, const Flat2DParams &p, T *dst, int x0,
                                               int y0) {
    using Op = MorphOp<T, MAX>;
    constexpr int kSegRows = kTileH / 2;
    const int c = threadIdx.x % kTileW, seg = threadIdx.x / kTileW;
    const int gx = x0 + c;
    if (gx >= p.W) return;
    const int r0 = seg * kSegRows;
    const T *src = tile + r0 * ld + c;
    T h[KH];
#pragma unroll
    for (int k = 0; k < KH - 1; k++) {
        T acc = src[k * ld];
#pragma unroll
        for (int t = 1; t < KW; t++) acc = Op::combine(acc, src[k * ld + t]);
        h[k] = acc;
    }
    T *o = dst + (int64_t)(y0 + r0) * p.W + gx;
    const int rows_left = p.H - (y0 + r0);
#pragma unroll 4
    for (int r = 0; r < kSegRows; r++) {
        const T *row = src + (r + KH - 1) * ld;
        T acc = row[0];
#pragma unroll
        for (int t = 1; t < KW; t++) acc = Op::combine(acc, row[t]);
        h[KH - 1] = acc;
        T v = h[0];
#pragma unroll
        for (int k = 1; k < KH; k++) v = Op::combine(v, h[k]);
        if (r < rows_left) __stcs(o + (int64_t)r * p.W, Op::apply(v, p.sval));  // outputs: streaming stores
#pragma unroll
        for (int k = 0; k < KH - 1; k++) h[k] = h[k + 1];
    }
}

template <typename T, bool MAX, int KH, int KW>
__device__ __forceinline__ void tile_compute(const T *tile, int ld, T *rows, const Flat2DParams &p, T *dst, int x0,
                                             int y0) {
    if constexpr (KH > 0)
        flat_tile_walk<T, MAX, KH, KW>(tile, ld, p, dst, x0, y0);
    else
        flat_tile_compute<T, MAX>(tile, ld, rows, p, dst, x0, y0);
}

}  // namespace morph
}  // namespace tmc
