// Grey and binary morphology for GB300 (sm_103a).
//
// Semantics follow the reference operators tap for tap
// (torchmorph/csrc/grey_kernel.cu:101-170 and binary_kernel.cu:56-127):
// tap k of a structure of size s with origin o has per-axis offset
// delta = k - (s//2 + o); erosion reads x + delta and computes min(v - s_k),
// dilation reads x - delta and computes max(v + s_k).  Binary erosion and
// dilation are the same min / max over {0,1} bytes with a constant border
// equal to border_value, so both operator families share these kernels.
//
// Kernels
//   flat2d_kernel  -- flat rectangular footprints in 1-D/2-D: a shared-memory
//                     tile with halo, separable row then column min/max.
//                     Windows wider than kRun use the van Herk/Gil-Werman
//                     split (shared middle block + register prefix/suffix
//                     runs), so the cost per output stays ~2 reads.
//   stencil_kernel -- everything else (non-flat values, arbitrary
//                     footprints, 3..8-D): one thread per output, taps from
//                     the launch parameters, an interior fast path with flat
//                     offsets and a per-tap border path.
#include <cmath>
#include <cstring>
#include <vector>

#include "tm_common.cuh"

namespace tmc {
namespace {

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
__device__ __forceinline__ int map_coord(int c, int n, int mode) {
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

template <typename T, bool MAX>
__global__ void __launch_bounds__(kFlatThreads) flat2d_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                              Flat2DParams p) {
    using Op = MorphOp<T, MAX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int RH = kTileH + p.kh - 1;      // loaded rows
    const int RW = kTileW + p.kw - 1;      // loaded columns
    const int RWp = RW + (kRun - 1);       // padded so full runs never read past a row
    T *tile = reinterpret_cast<T *>(smem_raw);
    T *rows = tile + RH * RWp;             // row-pass result, RH x kTileW (+ pad)
    const int x0 = blockIdx.x * kTileW;
    const int y0 = blockIdx.y * kTileH;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = kFlatThreads / 32;
    const T cval = (T)p.cval;

    for (int64_t item = blockIdx.z; item < p.batch; item += gridDim.z) {
        const T *src = in + item * (int64_t)p.H * p.W;
        T *dst = out + item * (int64_t)p.H * p.W;
        const int gy0 = y0 + p.lo_y, gx0 = x0 + p.lo_x;
        const bool interior = gy0 >= 0 && gx0 >= 0 && gy0 + RH <= p.H && gx0 + RW <= p.W;
        // 1. stage the input tile (coalesced along x), mapping borders
        for (int r = warp; r < RH; r += nwarps) {
            int gy = gy0 + r;
            int my = interior ? gy : map_coord(gy, p.H, p.mode);
            for (int c = lane; c < RW; c += 32) {
                int gx = gx0 + c;
                T v;
                if (interior) {
                    v = src[(int64_t)gy * p.W + gx];
                } else {
                    int mx = map_coord(gx, p.W, p.mode);
                    v = (my < 0 || mx < 0) ? cval : src[(int64_t)my * p.W + mx];
                }
                tile[r * RWp + c] = v;
            }
        }
        __syncthreads();
        // 2. row pass: RH rows x kTileW outputs, runs of kRun
        const int runs_per_row = kTileW / kRun;
        for (int w = threadIdx.x; w < RH * runs_per_row; w += kFlatThreads) {
            int r = w / runs_per_row, c = (w % runs_per_row) * kRun;
            T res[kRun];
            window_run<T, MAX>(tile + r * RWp + c, 1, p.kw, res);
#pragma unroll
            for (int j = 0; j < kRun; j++) rows[r * kTileW + c + j] = res[j];
        }
        __syncthreads();
        // 3. column pass and store: kTileH x kTileW outputs, runs down columns
        const int runs_per_col = kTileH / kRun;
        for (int w = threadIdx.x; w < kTileW * runs_per_col; w += kFlatThreads) {
            int c = w % kTileW, r = (w / kTileW) * kRun;
            int gx = x0 + c;
            // kTileH is a multiple of kRun, so the run reads rows
            // r .. r + kRun + kh - 2 <= RH - 1: always inside the row buffer
            T res[kRun];
            window_run<T, MAX>(rows + r * kTileW + c, kTileW, p.kh, res);
            if (gx < p.W) {
#pragma unroll
                for (int j = 0; j < kRun; j++) {
                    int gy = y0 + r + j;
                    if (gy < p.H) dst[(int64_t)gy * p.W + gx] = Op::apply(res[j], p.sval);
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- stencil N-D
constexpr int kStencilThreads = 256;
constexpr int kTapBytes = 24576;

struct StencilParams {
    int ndim;
    int ntaps;
    int mode;
    int accumulate;  // 1: combine with the existing output (tap chunks 2..n)
    int64_t batch;
    int64_t numel_item;
    float cval;
    int shape[TM_MAX_NDIM];
    FastDiv div[TM_MAX_NDIM];  // divisors = spatial strides
    int min_off[TM_MAX_NDIM];
    int max_off[TM_MAX_NDIM];
};

// Tap table in the launch parameters: [flat int32 x n][value f32 x n][off int16 x n x ndim]
struct TapTable {
    unsigned char data[kTapBytes];
};

inline int tap_capacity(int ndim) { return kTapBytes / (8 + 2 * ndim); }

template <typename T, bool MAX>
__global__ void __launch_bounds__(kStencilThreads) stencil_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                                  StencilParams p, TapTable taps) {
    using Op = MorphOp<T, MAX>;
    const int n = p.ntaps;
    const int32_t *flat = reinterpret_cast<const int32_t *>(taps.data);
    const float *val = reinterpret_cast<const float *>(taps.data + 4 * n);
    const int16_t *off = reinterpret_cast<const int16_t *>(taps.data + 8 * n);
    const T cval = (T)p.cval;
    const int64_t total = p.batch * p.numel_item;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = idx / p.numel_item;
        const uint32_t sp = (uint32_t)(idx - item * p.numel_item);
        const T *src = in + item * p.numel_item;
        int coord[TM_MAX_NDIM];
        uint32_t rem = sp;
        bool interior = true;
#pragma unroll
        for (int d = 0; d < TM_MAX_NDIM; d++) {
            if (d < p.ndim) {
                uint32_t q = fdiv(rem, p.div[d]);
                rem -= q * p.div[d].d;
                coord[d] = (int)q;
                interior &= (coord[d] + p.min_off[d] >= 0) && (coord[d] + p.max_off[d] < p.shape[d]);
            }
        }
        T acc = p.accumulate ? out[idx] : Op::identity();
        if (interior) {
            for (int t = 0; t < n; t++) acc = Op::combine(acc, Op::apply(src[(int64_t)sp + flat[t]], val[t]));
        } else {
            for (int t = 0; t < n; t++) {
                int64_t f = 0;
                bool use_c = false;
                for (int d = 0; d < p.ndim; d++) {
                    int m = map_coord(coord[d] + off[t * p.ndim + d], p.shape[d], p.mode);
                    if (m < 0) {
                        use_c = true;
                        break;
                    }
                    f += (int64_t)m * p.div[d].d;
                }
                T v = use_c ? cval : src[f];
                acc = Op::combine(acc, Op::apply(v, val[t]));
            }
        }
        out[idx] = acc;
    }
}

// --------------------------------------------------------------- host side
struct Tap {
    int off[TM_MAX_NDIM];
    float val;
};

template <typename T, bool MAX>
int run_morphology(const T *in, T *out, int64_t batch, int ndim, const int64_t *shape,
                   const float *structure, const uint8_t *footprint, const int64_t *sshape,
                   const int64_t *origin, int mode, float cval, cudaStream_t stream) {
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (!in || !out) return fail(TM_ERR_INVALID_ARGUMENT, "input/output pointer is NULL");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    if (!sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "structure shape/origin is NULL");
    if (mode < 0 || mode > 4) return fail(TM_ERR_INVALID_ARGUMENT, "unknown border mode %d", mode);
    if (g.numel_item >= ((int64_t)1 << 31))
        return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels are not supported");
    int64_t stotal = 1;
    for (int d = 0; d < ndim; d++) {
        if (sshape[d] < 1 || sshape[d] > 32767)
            return fail(TM_ERR_INVALID_ARGUMENT, "structure size %d is %lld (must be 1..32767)", d,
                        (long long)sshape[d]);
        int64_t lo = -(sshape[d] / 2), hi = (sshape[d] - 1) / 2;
        if (origin[d] < lo || origin[d] > hi) return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
        stotal *= sshape[d];
    }
    // tap table (torchmorph/csrc/grey_kernel.cu:271-291)
    std::vector<Tap> taps;
    int64_t sstride[TM_MAX_NDIM];
    sstride[ndim - 1] = 1;
    for (int d = ndim - 2; d >= 0; d--) sstride[d] = sstride[d + 1] * sshape[d + 1];
    bool uniform = true;
    float first_val = 0.0f;
    for (int64_t i = 0; i < stotal; i++) {
        if (footprint && !footprint[i]) continue;
        Tap t;
        int64_t rem = i;
        for (int d = 0; d < ndim; d++) {
            int64_t k = rem / sstride[d];
            rem %= sstride[d];
            int64_t delta = k - (sshape[d] / 2 + origin[d]);
            t.off[d] = (int)(MAX ? -delta : delta);
        }
        t.val = structure ? structure[i] : 0.0f;
        if (taps.empty()) first_val = t.val;
        uniform &= std::memcmp(&t.val, &first_val, sizeof(float)) == 0;
        taps.push_back(t);
    }
    if (taps.empty())
        return fail(TM_ERR_INVALID_ARGUMENT, "footprint must contain at least one active position");
    const bool box = (int64_t)taps.size() == stotal && uniform;
    const int sms = sm_count();

    if (box && ndim <= 2) {
        Flat2DParams p;
        p.H = ndim == 2 ? (int)shape[0] : 1;
        p.W = (int)shape[ndim - 1];
        p.kh = ndim == 2 ? (int)sshape[0] : 1;
        p.kw = (int)sshape[ndim - 1];
        int cy = ndim == 2 ? (int)(sshape[0] / 2 + origin[0]) : 0;
        int cx = (int)(sshape[ndim - 1] / 2 + origin[ndim - 1]);
        // erosion window [x - c, x - c + k - 1]; dilation [x + c - k + 1, x + c]
        p.lo_y = MAX ? cy - p.kh + 1 : -cy;
        p.lo_x = MAX ? cx - p.kw + 1 : -cx;
        p.mode = mode;
        p.batch = batch;
        p.cval = cval;
        p.sval = first_val;
        if (p.kh > 4096 || p.kw > 4096) goto stencil;  // tile would not fit on chip
        {
            const int RH = kTileH + p.kh - 1, RW = kTileW + p.kw - 1 + (kRun - 1);
            size_t smem = (size_t)RH * RW * sizeof(T) + (size_t)RH * kTileW * sizeof(T);
            if (smem > 200 * 1024) goto stencil;
            if (smem > 48 * 1024)
                TM_CHECK_CUDA(cudaFuncSetAttribute(flat2d_kernel<T, MAX>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            dim3 grid((unsigned)ceil_div(p.W, kTileW), (unsigned)ceil_div(p.H, kTileH),
                      (unsigned)(batch < 65535 ? batch : 65535));
            flat2d_kernel<T, MAX><<<grid, kFlatThreads, smem, stream>>>(in, out, p);
            TM_LAUNCH_CHECK("flat2d_kernel");
            return TM_OK;
        }
    }
stencil:
    {
        StencilParams p;
        std::memset(&p, 0, sizeof(p));
        p.ndim = ndim;
        p.mode = mode;
        p.batch = batch;
        p.numel_item = g.numel_item;
        p.cval = cval;
        for (int d = 0; d < TM_MAX_NDIM; d++) {
            p.shape[d] = d < ndim ? (int)shape[d] : 1;
            p.div[d] = make_fastdiv(d < ndim ? (uint32_t)g.stride[d] : 1u);
            p.min_off[d] = 0;
            p.max_off[d] = 0;
        }
        for (const Tap &t : taps)
            for (int d = 0; d < ndim; d++) {
                p.min_off[d] = t.off[d] < p.min_off[d] ? t.off[d] : p.min_off[d];
                p.max_off[d] = t.off[d] > p.max_off[d] ? t.off[d] : p.max_off[d];
            }
        const int cap = tap_capacity(ndim);
        int64_t blocks = ceil_div(g.numel, kStencilThreads);
        int64_t max_blocks = (int64_t)sms * 8;
        if (blocks > max_blocks) blocks = max_blocks;
        TapTable table;
        for (size_t first = 0; first < taps.size(); first += cap) {
            int n = (int)std::min<size_t>(cap, taps.size() - first);
            int32_t *flat = reinterpret_cast<int32_t *>(table.data);
            float *val = reinterpret_cast<float *>(table.data + 4 * n);
            int16_t *off = reinterpret_cast<int16_t *>(table.data + 8 * n);
            for (int t = 0; t < n; t++) {
                const Tap &tp = taps[first + t];
                int64_t f = 0;
                for (int d = 0; d < ndim; d++) {
                    f += (int64_t)tp.off[d] * g.stride[d];
                    off[t * ndim + d] = (int16_t)tp.off[d];
                }
                flat[t] = (int32_t)f;
                val[t] = tp.val;
            }
            p.ntaps = n;
            p.accumulate = first > 0;
            stencil_kernel<T, MAX><<<(unsigned)blocks, kStencilThreads, 0, stream>>>(in, out, p, table);
            TM_LAUNCH_CHECK("stencil_kernel");
        }
    }
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" int tm_grey_erosion(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    if (!structure) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "structure is NULL");
    return tmc::run_morphology<float, false>(in, out, batch, ndim, shape, structure, footprint, sshape,
                                            origin, mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_grey_dilation(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                                const float *structure, const uint8_t *footprint, const int64_t *sshape,
                                const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    if (!structure) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "structure is NULL");
    return tmc::run_morphology<float, true>(in, out, batch, ndim, shape, structure, footprint, sshape,
                                           origin, mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_binary_erosion(const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
                                 const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
                                 const int64_t *origin, int border_value, tm_stream_t stream) {
    if (!structure) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "structure is NULL");
    return tmc::run_morphology<uint8_t, false>(in, out, batch, ndim, shape, nullptr, structure, sshape,
                                              origin, TM_MODE_CONSTANT, border_value ? 1.0f : 0.0f,
                                              (cudaStream_t)stream);
}

extern "C" int tm_binary_dilation(const uint8_t *in, uint8_t *out, int64_t batch, int ndim,
                                  const int64_t *shape, const uint8_t *structure, const int64_t *sshape,
                                  const int64_t *origin, int border_value, tm_stream_t stream) {
    if (!structure) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "structure is NULL");
    return tmc::run_morphology<uint8_t, true>(in, out, batch, ndim, shape, nullptr, structure, sshape,
                                             origin, TM_MODE_CONSTANT, border_value ? 1.0f : 0.0f,
                                             (cudaStream_t)stream);
}
