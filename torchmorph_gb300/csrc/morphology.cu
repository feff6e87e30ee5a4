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

#include "bitmorph.cuh"
#include "morph_tile.cuh"
#include "tm_common.cuh"
#include "tm_tma.cuh"
#include "vwalk.cuh"

namespace tmc {
namespace {

using namespace morph;

template <typename T, bool MAX, int KH, int KW>
__global__ void __launch_bounds__(kFlatThreads) flat2d_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                              Flat2DParams p) {
    using Op = MorphOp<T, MAX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int RH = kTileH + p.kh - 1;      // loaded rows
    const int RW = kTileW + p.kw - 1;      // loaded columns
    const int RWp = stage_pitch(p.kw);     // padded so full runs never read past a row; odd
    T *tile = reinterpret_cast<T *>(smem_raw);
    T *rows = tile + RH * RWp;             // row-pass result, RH x kTileW at pitch kRowsPitch
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = kFlatThreads / 32;
    const T cval = (T)p.cval;

    const int x0 = blockIdx.x * kTileW;
    const int y0 = blockIdx.y * kTileH;
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
        tile_compute<T, MAX, KH, KW>(tile, RWp, rows, p, dst, x0, y0);
        __syncthreads();
    }
}

// ------------------------------------------------ flat 2-D tile, TMA staged
// Persistent kernel for the tiles whose input region lies inside the item
// (every tile of a large image but the outer ring).  Each CTA walks the
// interior tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...; thread 0 issues
// one TMA tensor copy per tile into one of two shared-memory buffers, so the
// next tile's load is in flight while the current one is computed.  The TMA
// box starts at the 16-byte-aligned column at or left of the tile's first
// input column; the compute reads from the offset inside the buffer.
struct TmaTileParams {
    int bw;     // box width in elements (multiple of align)
    int align;  // elements per 16 bytes
    int ntx, nty;
    int64_t ntiles;
    // interior tiles: rows [ya, yb) x columns [xa, xb) of every item; work
    // units 0 .. n_interior-1 are interior tiles, the rest the border ring
    int ya, yb, xa, xb;
    int64_t n_interior;
};

// Work unit u -> (item, tx, ty): interior tiles first, then each item's ring
// (full rows above ya and from yb on, then the side columns of the rows in
// between).
__device__ __forceinline__ void unit_to_tile(const TmaTileParams &tp, int64_t u, int64_t &item, int &tx, int &ty,
                                             bool &inner) {
    const int iw = tp.xb - tp.xa, ih = tp.yb - tp.ya;
    if (u < tp.n_interior) {
        const int64_t per = (int64_t)iw * ih;
        item = u / per;
        const int k = (int)(u - item * per);
        ty = tp.ya + k / iw;
        tx = tp.xa + k % iw;
        inner = true;
        return;
    }
    inner = false;
    const int64_t ring = (int64_t)tp.ntx * tp.nty - (int64_t)iw * ih;
    const int64_t v = u - tp.n_interior;
    item = v / ring;
    int i = (int)(v - item * ring);
    const int top = tp.ya * tp.ntx, bottom = (tp.nty - tp.yb) * tp.ntx, side = tp.xa + (tp.ntx - tp.xb);
    if (i < top) {
        ty = i / tp.ntx;
        tx = i % tp.ntx;
    } else if (i < top + bottom) {
        i -= top;
        ty = tp.yb + i / tp.ntx;
        tx = i % tp.ntx;
    } else {
        i -= top + bottom;
        ty = tp.ya + i / side;
        const int k = i % side;
        tx = k < tp.xa ? k : tp.xb + (k - tp.xa);
    }
}

__host__ __device__ __forceinline__ size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int kMaxStageCols = 8;  // TMA tiles are at most 256 columns wide

template <typename T, bool MAX, int KH, int KW>
__global__ void __launch_bounds__(kFlatThreads) flat2d_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                  const T *__restrict__ in, T *__restrict__ out,
                                                                  Flat2DParams p, TmaTileParams tp, int *status) {
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    // TMA destinations must be 128-byte aligned: round the dynamic base up (the
    // launch asks for 1 KB of slack)
    unsigned char *smem_raw = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~static_cast<uintptr_t>(1023));
    const int RH = kTileH + p.kh - 1;
    const int RW = kTileW + p.kw - 1;
    const size_t buf_bytes = round_up((size_t)RH * tp.bw * sizeof(T), 1024);
    T *buf[2] = {reinterpret_cast<T *>(smem_raw), reinterpret_cast<T *>(smem_raw + buf_bytes)};
    T *rows = reinterpret_cast<T *>(smem_raw + 2 * buf_bytes);
    const size_t rows_bytes = KH == 0 ? round_up((size_t)RH * kRowsPitch * sizeof(T), 16) : 0;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + 2 * buf_bytes + rows_bytes);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint32_t bytes = (uint32_t)(RH * tp.bw * sizeof(T));
    auto interior = [&](int64_t u) { return u < tp.n_interior; };
    auto issue = [&](int64_t u, int s) {
        int64_t item;
        int tx, ty;
        bool inner;
        unit_to_tile(tp, u, item, tx, ty, inner);
        const int gx0 = tx * kTileW + p.lo_x, gy0 = ty * kTileH + p.lo_y;
        mbar_arrive_expect_tx(&bar[s], bytes);
        tma_load_3d(buf[s], &tmap, gx0 & ~(tp.align - 1), gy0, (int)item, &bar[s]);
    };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T cval = (T)p.cval;
    uint32_t phase0 = 0, phase1 = 0;
    int64_t t = blockIdx.x;
    if (threadIdx.x == 0 && t < tp.ntiles && interior(t)) issue(t, 0);
    for (int it = 0; t < tp.ntiles; it++, t += gridDim.x) {
        const int s = it & 1;
        const int64_t tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < tp.ntiles && interior(tn)) issue(tn, s ^ 1);
        int64_t item;
        int tx, ty;
        bool inner;
        unit_to_tile(tp, t, item, tx, ty, inner);
        const int gx0 = tx * kTileW + p.lo_x, gy0 = ty * kTileH + p.lo_y;
        int off = 0;
        if (inner) {
            const uint32_t ph = s == 0 ? phase0 : phase1;
            const bool landed = mbar_wait(&bar[s], ph, status);
            if (s == 0)
                phase0 ^= 1;
            else
                phase1 ^= 1;
            if (__syncthreads_or(!landed)) {
                // give the copy already issued for the next tile a bounded chance to land
                if (threadIdx.x == 0 && tn < tp.ntiles && interior(tn))
                    mbar_wait(&bar[s ^ 1], s == 0 ? phase1 : phase0, status);
                return;
            }
            off = gx0 - (gx0 & ~(tp.align - 1));
        } else {
            // border tile: stage the mapped region by hand; each lane maps its
            // (at most kMaxStageCols) columns once
            const T *src = in + item * (int64_t)p.H * p.W;
            int mxs[kMaxStageCols];
#pragma unroll
            for (int k = 0; k < kMaxStageCols; k++) {
                const int c = lane + 32 * k;
                mxs[k] = c < RW ? map_coord(gx0 + c, p.W, p.mode) : -1;
            }
            for (int rr = warp; rr < RH; rr += kFlatThreads / 32) {
                const int my = map_coord(gy0 + rr, p.H, p.mode);
                const T *srow = src + (int64_t)(my < 0 ? 0 : my) * p.W;
#pragma unroll
                for (int k = 0; k < kMaxStageCols; k++) {
                    const int c = lane + 32 * k;
                    if (c < RW) buf[s][rr * tp.bw + c] = (my < 0 || mxs[k] < 0) ? cval : srow[mxs[k]];
                }
            }
            __syncthreads();
        }
        tile_compute<T, MAX, KH, KW>(buf[s] + off, tp.bw, rows, p, out + item * (int64_t)p.H * p.W, tx * kTileW,
                                     ty * kTileH);
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

// Flat 1-D/2-D box: the mapped-border kernel for every tile (or only the
// border ring when the TMA kernel takes the interior), then the TMA kernel.
template <typename T, bool MAX, int KH, int KW>
int launch_flat2d(const T *in, T *out, Flat2DParams p, int64_t batch, int sms, cudaStream_t stream) {
    const int RH = kTileH + p.kh - 1, RWp = stage_pitch(p.kw);
    const size_t rows_bytes = KH == 0 ? (size_t)RH * kRowsPitch * sizeof(T) : 0;
    const size_t smem = (size_t)RH * RWp * sizeof(T) + rows_bytes;
    if (smem > 48 * 1024)
        TM_CHECK_CUDA(cudaFuncSetAttribute(flat2d_kernel<T, MAX, KH, KW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    dim3 grid((unsigned)ceil_div(p.W, kTileW), (unsigned)ceil_div(p.H, kTileH),
              (unsigned)(batch < 65535 ? batch : 65535));
    // TMA path for the interior tiles: needs 16-byte aligned rows and a box of at most 256 x 256
    TmaTileParams tp;
    tp.align = 16 / (int)sizeof(T);
    tp.bw = (int)round_up((size_t)(kTileW + p.kw - 1 + tp.align - 1), (size_t)tp.align);
    tp.ntx = (int)grid.x;
    tp.nty = (int)grid.y;
    tp.ntiles = (int64_t)tp.ntx * tp.nty * batch;
    {
        // interior tile rows/columns: the region of tile t starts at
        // t * tile + lo and is RH (RW) long
        auto first_ge = [](int lo, int tile) { return lo >= 0 ? 0 : (-lo + tile - 1) / tile; };
        const int RW = kTileW + p.kw - 1;
        tp.ya = first_ge(p.lo_y, kTileH);
        tp.yb = (p.H - RH - p.lo_y) >= 0 ? (p.H - RH - p.lo_y) / kTileH + 1 : 0;
        tp.xa = first_ge(p.lo_x, kTileW);
        tp.xb = (p.W - RW - p.lo_x) >= 0 ? (p.W - RW - p.lo_x) / kTileW + 1 : 0;
        tp.yb = std::min(std::max(tp.yb, tp.ya), tp.nty);
        tp.xb = std::min(std::max(tp.xb, tp.xa), tp.ntx);
        tp.ya = std::min(tp.ya, tp.yb);
        tp.xa = std::min(tp.xa, tp.xb);
        tp.n_interior = (int64_t)(tp.yb - tp.ya) * (tp.xb - tp.xa) * batch;
    }
    // one persistent launch takes every tile (TMA for interior tiles) once a
    // batch has a few tiles per SM; otherwise the plain kernel does all
    // autotuned variant: 0 TMA-staged persistent tiles at full occupancy, 1 plain
    // loads (one CTA per tile), 2 / 3 TMA with at most 1 / 2 CTAs per SM
    const int variant = tune_variant(kTuneGreyFlat2D, tune_class(kTuneGreyFlat2D, batch * (int64_t)p.H * p.W, 0));
    const bool tma_ok = variant != 1 && (p.W % tp.align) == 0 && ((uintptr_t)in & 15) == 0 && tp.bw <= 256 &&
                        RH <= 256 && p.H >= RH && p.W >= tp.bw && tp.ntiles >= 2LL * sms &&
                        tp.ntiles < ((int64_t)1 << 31) && batch < ((int64_t)1 << 31);
    if (!tma_ok) {
        flat2d_kernel<T, MAX, KH, KW><<<grid, kFlatThreads, smem, stream>>>(in, out, p);
        TM_LAUNCH_CHECK("flat2d_kernel");
        return TM_OK;
    }
    CUtensorMap map;
    const uint64_t dims[3] = {(uint64_t)p.W, (uint64_t)p.H, (uint64_t)batch};
    const uint64_t strides[2] = {(uint64_t)p.W * sizeof(T), (uint64_t)p.W * p.H * sizeof(T)};
    const uint32_t box[3] = {(uint32_t)tp.bw, (uint32_t)RH, 1};
    int st = encode_tensor_map(&map, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                               3, in, dims, strides, box);
    if (st != TM_OK) return st;
    int *status = nullptr;
    st = device_status_word(&status);
    if (st != TM_OK) return st;
    const size_t tsmem = 2 * round_up((size_t)RH * tp.bw * sizeof(T), 1024) +
                         (KH == 0 ? round_up((size_t)RH * kRowsPitch * sizeof(T), 16) : 0) + 2 * sizeof(uint64_t) + 1024;
    if (tsmem > 220 * 1024) return fail(TM_ERR_UNSUPPORTED, "TMA tile does not fit in shared memory");
    // attribute + occupancy depend only on the instantiation and the smem size: cache the last answer
    static thread_local size_t cached_smem = 0;
    static thread_local int cached_dev = -1, cached_per_sm = 1;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_smem != tsmem || cached_dev != dev) {
        TM_CHECK_CUDA(cudaFuncSetAttribute(flat2d_tma_kernel<T, MAX, KH, KW>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem));
        int per_sm = 0;
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, flat2d_tma_kernel<T, MAX, KH, KW>,
                                                                    kFlatThreads, tsmem));
        cached_per_sm = per_sm < 1 ? 1 : per_sm;
        cached_smem = tsmem;
        cached_dev = dev;
    }
    const int per_sm = variant == 2 ? 1 : (variant == 3 ? std::min(cached_per_sm, 2) : cached_per_sm);
    const int64_t ctas = std::min<int64_t>(tp.ntiles, (int64_t)sms * per_sm);
    flat2d_tma_kernel<T, MAX, KH, KW><<<(unsigned)ctas, kFlatThreads, tsmem, stream>>>(map, in, out, p, tp, status);
    TM_LAUNCH_CHECK("flat2d_tma_kernel");
    return TM_OK;
}

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
    if constexpr (sizeof(T) == 1) {
        // binary, 1-D / 2-D, elements other than full boxes (the default cross,
        // footprints): bit-packed tiles
        if (!box && ndim <= 2) {
            bool done = false;
            st = bitmorph_uniform(MAX ? 1 : 0, in, out, batch, ndim, shape, footprint, sshape, origin, cval != 0.0f,
                                  stream, &done);
            if (st != TM_OK || done) return st;
        }
    }

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
            const int RH = kTileH + p.kh - 1, RW = stage_pitch(p.kw);
            if ((size_t)RH * RW * sizeof(T) + (size_t)RH * kRowsPitch * sizeof(T) > 200 * 1024) goto stencil;
            if constexpr (sizeof(T) == 4) {
                // centred 3 x 3 / 5 x 5 windows on 16-byte aligned rows: register
                // walkers for the interior, one thread per output for the frame
                if (ndim == 2 && p.kh == p.kw && (p.kh == 3 || p.kh == 5) && p.lo_y == -(p.kh / 2) &&
                    p.lo_x == -(p.kw / 2)) {
                    bool done = false;
                    st = p.kh == 3
                             ? vwalk::run<MAX, 1, 0, 3>(in, out, p.H, p.W, batch, mode, p.cval, p.sval, stream, &done)
                             : vwalk::run<MAX, 1, 0, 5>(in, out, p.H, p.W, batch, mode, p.cval, p.sval, stream, &done);
                    if (st != TM_OK || done) return st;
                }
            }
            if (p.kh == 3 && p.kw == 3) return launch_flat2d<T, MAX, 3, 3>(in, out, p, batch, sms, stream);
            if (p.kh == 5 && p.kw == 5) return launch_flat2d<T, MAX, 5, 5>(in, out, p, batch, sms, stream);
            if (p.kh == 1 && p.kw == 3) return launch_flat2d<T, MAX, 1, 3>(in, out, p, batch, sms, stream);
            return launch_flat2d<T, MAX, 0, 0>(in, out, p, batch, sms, stream);
        }
    }
stencil:
    if (ndim == 3 && g.numel_item < ((int64_t)1 << 31)) {  // 3-D items: shared-memory tiles
        bool done = false;
        st = stencil3d_uniform<T, MAX>(in, out, batch, shape, structure, footprint, sshape, origin, mode, cval,
                                       stream, &done);
        if (st != TM_OK || done) return st;
    }
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
