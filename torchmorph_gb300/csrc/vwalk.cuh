// Register walkers for centred 3 x 3 and 5 x 5 flat windows over float32
// items whose rows are 16-byte aligned (GB300, sm_103a): grey erosion and
// dilation, the morphological gradient and laplace (one stage) and the
// one-pass opening, closing and top-hats (two stages).  The walkers take
// the outputs whose whole footprint, and every intermediate value those
// outputs use, lies inside the item: rows [STAGES * h, H - STAGES * h) and
// columns [4, W - 4), h = K / 2.  The outputs outside that rectangle (a
// frame a few voxels wide) go to the frame kernel, which applies the border
// mode; it is launched behind the walkers with programmatic dependent launch
// in small blocks that fit beside the walkers' CTAs, so it runs while they
// stream.
//
// One warp walks down a strip of 128 input columns: lane l holds columns
// x0 + 4l .. x0 + 4l + 3 of each row as one float4 load, its horizontal
// neighbours (h on each side) come from lanes l - 1 and l + 1 by shuffles,
// and the vertical window is a shift register of the last K - 1 row results
// per stage.  Lanes 1 .. 30 write their four outputs with one float4 store;
// lanes 0 and 31 only feed their neighbours (their outer columns' windows
// reach outside the strip), so consecutive strips start 120 columns apart
// and re-read 8 columns of each other (L2 hits).  A task is a block of
// output rows of one strip; its input rows are loaded kChunk rows ahead.
//
// Semantics are the reference's operators (torchmorph/csrc/grey_kernel.cu:
// 101-170): erosion min(x) - s, dilation max(x) + s for a flat element of
// value s; min / max are fminf / fmaxf, exact and order-independent.  For
// two stages the second operator reads the first one's image, every read
// position of which lies inside the item here.
#pragma once

#include <algorithm>

#include "morph_tile.cuh"

namespace tmc {
namespace vwalk {

using morph::MorphOp;

constexpr int kLanesOut = 30;               // lanes 1 .. 30 write outputs
constexpr int kStrip = 4 * kLanesOut;       // output columns per strip
constexpr int kChunk = 4;                   // input rows in flight per warp
constexpr int kThreads = 256;
constexpr int kTophatNone = 0, kTophatWhite = 1, kTophatBlack = 2;
constexpr int kGradient = 1, kLaplace = 2;
constexpr uint32_t kNoArg = 255u;  // no tap (every tap gave the identity)

struct Params {
    int H, W;
    int64_t batch;
    int ry0, ry1;   // output rows taken
    int rows;       // output rows per task
    int nrb;        // row blocks per item
    int nstrips;    // strips per item
    int64_t ntasks;
    float sval;
};

// a[h + i] = v[i]; a[0 .. h - 1] and a[h + 4 ..] the columns left and right
// of the lane's four, from the adjacent lanes.
template <int h>
__device__ __forceinline__ void extend(const float (&v)[4], float (&a)[4 + 2 * h]) {
#pragma unroll
    for (int i = 0; i < 4; i++) a[h + i] = v[i];
#pragma unroll
    for (int j = 1; j <= h; j++) a[h - j] = __shfl_up_sync(0xffffffffu, v[4 - j], 1);
#pragma unroll
    for (int j = 0; j < h; j++) a[h + 4 + j] = __shfl_down_sync(0xffffffffu, v[j], 1);
}

// o[i] = Op over the columns i - h .. i + h.
template <class Op, int h>
__device__ __forceinline__ void row_window(const float (&a)[4 + 2 * h], float (&o)[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float m = a[i];
#pragma unroll
        for (int j = 1; j <= 2 * h; j++) m = Op::combine(m, a[i + j]);
        o[i] = m;
    }
}

// Both extrema over the columns i - h .. i + h.
template <int h>
__device__ __forceinline__ void row_window_both(const float (&a)[4 + 2 * h], float (&mx)[4], float (&mn)[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float hi = a[i], lo = a[i];
#pragma unroll
        for (int j = 1; j <= 2 * h; j++) {
            hi = fmaxf(hi, a[i + j]);
            lo = fminf(lo, a[i + j]);
        }
        mx[i] = hi;
        mn[i] = lo;
    }
}

// Vertical window: combine the K - 1 held rows with the new one, then shift.
template <class Op, int K>
__device__ __forceinline__ void col_window(float (&ring)[K - 1][4], const float (&hnew)[4], float (&o)[4]) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float m = hnew[i];
#pragma unroll
        for (int j = 0; j < K - 1; j++) m = Op::combine(m, ring[j][i]);
        o[i] = m;
    }
#pragma unroll
    for (int j = 0; j + 1 < K - 1; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) ring[j][i] = ring[j + 1][i];
#pragma unroll
    for (int i = 0; i < 4; i++) ring[K - 2][i] = hnew[i];
}

// Resident blocks per SM the register budget is set for: 3 x 3 walks get
// 80 registers (three blocks: the loads in flight of 24 warps matter more
// than a few spilled values) unless they hold input rows (laplace: 128),
// 5 x 5 one-stage walks 128, two stages of 5 x 5 more (one block).
constexpr int kMinBlocks(int stages, int k, int combine) {
    return k == 3 ? (combine == kLaplace ? 2 : 3) : (stages == 1 ? 2 : 1);
}

// One task: output rows [ya, yb) of the strip at the lane's columns.
template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE>
__device__ __forceinline__ void walk_task(const float4 *src, float4 *dst, int ya, int yb, bool loads, bool writes,
                                          const Params &p) {
    using Op1 = MorphOp<float, MAX1>;
    using Op2 = MorphOp<float, !MAX1>;
    constexpr int h = K / 2;
    constexpr int kLag = STAGES * h;        // output row = input row - kLag
    constexpr int kFill = 2 * kLag;         // input rows before the first output
    // the laplace holds its input rows in registers; the top-hats reload the
    // input row of the output (kLag rows back: an L1 hit) to stay in 80 registers
    constexpr bool kHoldX = COMBINE == kLaplace;
    constexpr int kXHold = kHoldX ? kLag : 1;
    const int rs = ya - kLag, re = yb - 1 + kLag;  // input rows
    const int wq = p.W >> 2;
    float ring1[K - 1][4], ring2[K - 1][4], xh[kXHold][4];
    float4 cur[kChunk], nxt[kChunk];
#pragma unroll
    for (int k = 0; k < kChunk; k++)
        cur[k] = (loads && rs + k <= re) ? __ldg(src + (int64_t)(rs + k) * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int r0 = rs; r0 <= re; r0 += kChunk) {
        if (r0 + kChunk <= re) {
#pragma unroll
            for (int k = 0; k < kChunk; k++) {
                const int r = r0 + kChunk + k;
                nxt[k] = (loads && r <= re) ? __ldg(src + (int64_t)r * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int k = 0; k < kChunk; k++) {
            const int r = r0 + k;
            if (r > re) continue;
            const float v[4] = {cur[k].x, cur[k].y, cur[k].z, cur[k].w};
            float a[4 + 2 * h];
            extend<h>(v, a);
            float hr[4], e[4], o[4];
            if constexpr (COMBINE != 0) {
                // ring1 holds the maxima, ring2 the minima; rounded like the
                // reference's elementwise ops on the two operator images
                float hl[4], d[4];
                row_window_both<h>(a, hr, hl);
                col_window<MorphOp<float, true>, K>(ring1, hr, d);
                col_window<MorphOp<float, false>, K>(ring2, hl, e);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float dv = __fadd_rn(d[i], p.sval), ev = __fsub_rn(e[i], p.sval);
                    o[i] = COMBINE == kGradient ? __fsub_rn(dv, ev)
                                                : __fsub_rn(__fadd_rn(dv, ev), __fmul_rn(2.f, xh[0][i]));
                }
            } else {
                row_window<Op1, h>(a, hr);
                col_window<Op1, K>(ring1, hr, e);
#pragma unroll
                for (int i = 0; i < 4; i++) e[i] = Op1::apply(e[i], p.sval);
                if constexpr (STAGES == 1) {
#pragma unroll
                    for (int i = 0; i < 4; i++) o[i] = e[i];
                } else {
                    float a2[4 + 2 * h], h2[4];
                    extend<h>(e, a2);
                    row_window<Op2, h>(a2, h2);
                    col_window<Op2, K>(ring2, h2, o);
#pragma unroll
                    for (int i = 0; i < 4; i++) o[i] = Op2::apply(o[i], p.sval);
                }
            }
            if constexpr (TOPHAT != kTophatNone) {
                if (r - rs >= kFill && writes) {
                    const float4 xv = __ldg(src + (int64_t)(r - kLag) * wq);
                    const float xa[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
                    for (int i = 0; i < 4; i++) o[i] = TOPHAT == kTophatWhite ? xa[i] - o[i] : o[i] - xa[i];
                }
            }
            if constexpr (kHoldX) {
                // xh holds input rows r - kLag .. r - 1
#pragma unroll
                for (int j = 0; j + 1 < kXHold; j++)
#pragma unroll
                    for (int i = 0; i < 4; i++) xh[j][i] = xh[j + 1][i];
#pragma unroll
                for (int i = 0; i < 4; i++) xh[kXHold - 1][i] = v[i];
            }
            if (r - rs >= kFill && writes) __stcs(dst + (int64_t)(r - kLag) * wq, make_float4(o[0], o[1], o[2], o[3]));
        }
#pragma unroll
        for (int k = 0; k < kChunk; k++) cur[k] = nxt[k];
    }
}

// COMBINE: 0 the operators alone; kGradient dilation - erosion, kLaplace
// (dilation + erosion) - 2 x, both of one stage over the same window.
template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE = 0>
__global__ void __launch_bounds__(kThreads, kMinBlocks(STAGES, K, COMBINE))
    vwalk_kernel(const float *__restrict__ in, float *__restrict__ out, Params p) {
    pdl_trigger();  // the frame kernel launched behind this grid may start now
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
    for (int64_t t = (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); t < p.ntasks; t += nwarps) {
        const int strip = (int)(t % p.nstrips);
        const int64_t rest = t / p.nstrips;
        const int rb = (int)(rest % p.nrb);
        const int64_t item = rest / p.nrb;
        const int c = strip * kStrip + 4 * lane;             // first column of the lane
        const bool loads = c < p.W;                          // W is a multiple of 4
        const bool writes = lane >= 1 && lane <= kLanesOut && c + 8 <= p.W;
        const int ya = p.ry0 + rb * p.rows;
        const int yb = min(ya + p.rows, p.ry1);
        const float4 *src = reinterpret_cast<const float4 *>(in + item * (int64_t)p.H * p.W) + (c >> 2);
        float4 *dst = reinterpret_cast<float4 *>(out + item * (int64_t)p.H * p.W) + (c >> 2);
        walk_task<MAX1, STAGES, TOPHAT, K, COMBINE>(src, dst, ya, yb, loads, writes, p);
    }
}

// ------------------------------------------ forward with argument, backward
// The opt-in backward of grey erosion / dilation for the same centred K x K
// flat boxes.  Tap t = K i + j of the footprint reads row y + dy_i and column
// x + dx_j, dy_i = MAX ? h - i : i - h (dx likewise: dilation reads x - delta).
//
// Forward: the operator's value and the FIRST tap (raster order, strict
// comparison) attaining it -- per input row the first column tap attaining
// the row's extremum, then over the K rows the first row attaining the
// overall one; the pair is the first tap overall.  Backward (gather): input
// pixel p receives grad_out[o] from each output o = p - off_t whose recorded
// tap is t, summed in tap order, for pixels no border mapping routes a
// gradient to (rows [h + 1, H - 1 - h), columns [4, W - 4)); arguments are
// read four to a 32-bit word (bytes).
template <bool MAX, int K>
__global__ void __launch_bounds__(kThreads, K == 3 ? 3 : 2)
    vwalk_arg_kernel(const float *__restrict__ in, float *__restrict__ out, uint32_t *__restrict__ arg, Params p) {
    using Op = MorphOp<float, MAX>;
    constexpr int h = K / 2;
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
    for (int64_t t = (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); t < p.ntasks; t += nwarps) {
        const int strip = (int)(t % p.nstrips);
        const int64_t rest = t / p.nstrips;
        const int rb = (int)(rest % p.nrb);
        const int64_t item = rest / p.nrb;
        const int c = strip * kStrip + 4 * lane;
        const bool loads = c < p.W;
        const bool writes = lane >= 1 && lane <= kLanesOut && c + 8 <= p.W;
        const int ya = p.ry0 + rb * p.rows;
        const int yb = min(ya + p.rows, p.ry1);
        const int rs = ya - h, re = yb - 1 + h;
        const int wq = p.W >> 2;
        const float4 *src = reinterpret_cast<const float4 *>(in + item * (int64_t)p.H * p.W) + (c >> 2);
        float4 *dst = reinterpret_cast<float4 *>(out + item * (int64_t)p.H * p.W) + (c >> 2);
        uint32_t *adst = arg + ((item * (int64_t)p.H * p.W + c) >> 2);
        float ring[K - 1][4];
        uint32_t ringa[K - 1];
        float4 cur[kChunk], nxt[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; k++)
            cur[k] = (loads && rs + k <= re) ? __ldg(src + (int64_t)(rs + k) * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int r0 = rs; r0 <= re; r0 += kChunk) {
            if (r0 + kChunk <= re) {
#pragma unroll
                for (int k = 0; k < kChunk; k++) {
                    const int r = r0 + kChunk + k;
                    nxt[k] = (loads && r <= re) ? __ldg(src + (int64_t)r * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
#pragma unroll
            for (int k = 0; k < kChunk; k++) {
                const int r = r0 + k;
                if (r > re) continue;
                const float v[4] = {cur[k].x, cur[k].y, cur[k].z, cur[k].w};
                float a[4 + 2 * h];
                extend<h>(v, a);
                // row pass: first column tap attaining the row's extremum
                float rb4[4];
                uint32_t ra = 0u;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    float b = Op::identity();
                    uint32_t bj = kNoArg;
#pragma unroll
                    for (int j = 0; j < K; j++) {
                        const int dx = MAX ? h - j : j - h;
                        const float val = Op::apply(a[q + h + dx], p.sval);
                        if (MAX ? val > b : val < b) {
                            b = val;
                            bj = (uint32_t)j;
                        }
                    }
                    rb4[q] = b;
                    ra |= bj << (8 * q);
                }
                if (r - rs >= 2 * h && writes) {
                    // rows r - 2h .. r: ring[0 .. K-2], then this row (window index w)
                    float o[4];
                    uint32_t oa = 0u;
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float B = Op::identity();
                        uint32_t A = kNoArg;
#pragma unroll
                        for (int i = 0; i < K; i++) {
                            const int w = MAX ? 2 * h - i : i;  // row y + dy_i, y = r - h
                            const float rv = w == K - 1 ? rb4[q] : ring[w][q];
                            const uint32_t rj = ((w == K - 1 ? ra : ringa[w]) >> (8 * q)) & 255u;
                            if (MAX ? rv > B : rv < B) {
                                B = rv;
                                A = (uint32_t)(K * i) + rj;
                            }
                        }
                        o[q] = B;
                        oa |= A << (8 * q);
                    }
                    __stcs(dst + (int64_t)(r - h) * wq, make_float4(o[0], o[1], o[2], o[3]));
                    __stcs(adst + (int64_t)(r - h) * wq, oa);
                }
#pragma unroll
                for (int j = 0; j + 1 < K - 1; j++) {
#pragma unroll
                    for (int q = 0; q < 4; q++) ring[j][q] = ring[j + 1][q];
                    ringa[j] = ringa[j + 1];
                }
#pragma unroll
                for (int q = 0; q < 4; q++) ring[K - 2][q] = rb4[q];
                ringa[K - 2] = ra;
            }
#pragma unroll
            for (int k = 0; k < kChunk; k++) cur[k] = nxt[k];
        }
    }
}

template <bool MAX, int K>
__global__ void __launch_bounds__(kThreads, K == 3 ? 2 : 1)
    vwalk_grad_kernel(const float *__restrict__ gout, const uint32_t *__restrict__ arg, float *__restrict__ gin,
                      Params p) {
    constexpr int h = K / 2;
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);
    for (int64_t t = (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); t < p.ntasks; t += nwarps) {
        const int strip = (int)(t % p.nstrips);
        const int64_t rest = t / p.nstrips;
        const int rb = (int)(rest % p.nrb);
        const int64_t item = rest / p.nrb;
        const int c = strip * kStrip + 4 * lane;
        const bool loads = c < p.W;
        const bool writes = lane >= 1 && lane <= kLanesOut && c + 8 <= p.W;
        const int ya = p.ry0 + rb * p.rows;  // input rows written
        const int yb = min(ya + p.rows, p.ry1);
        const int rs = ya - h, re = yb - 1 + h;  // output rows read
        const int wq = p.W >> 2;
        const int64_t base4 = (item * (int64_t)p.H * p.W + c) >> 2;
        const float4 *gsrc = reinterpret_cast<const float4 *>(gout) + base4;
        const uint32_t *asrc = arg + base4;
        float4 *dst = reinterpret_cast<float4 *>(gin) + base4;
        // window rows r - 2h .. r: gradients with h columns each side, and the
        // argument words of the lane and its two neighbours
        float rg[K - 1][4 + 2 * h];
        uint32_t raw[K - 1][3];
        float4 cg[kChunk], ng[kChunk];
        uint32_t ca[kChunk], na[kChunk];
#pragma unroll
        for (int k = 0; k < kChunk; k++) {
            const bool ok = loads && rs + k <= re;
            cg[k] = ok ? __ldg(gsrc + (int64_t)(rs + k) * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
            ca[k] = ok ? __ldg(asrc + (int64_t)(rs + k) * wq) : 0xffffffffu;
        }
        for (int r0 = rs; r0 <= re; r0 += kChunk) {
            if (r0 + kChunk <= re) {
#pragma unroll
                for (int k = 0; k < kChunk; k++) {
                    const int r = r0 + kChunk + k;
                    const bool ok = loads && r <= re;
                    ng[k] = ok ? __ldg(gsrc + (int64_t)r * wq) : make_float4(0.f, 0.f, 0.f, 0.f);
                    na[k] = ok ? __ldg(asrc + (int64_t)r * wq) : 0xffffffffu;
                }
            }
#pragma unroll
            for (int k = 0; k < kChunk; k++) {
                const int r = r0 + k;
                if (r > re) continue;
                const float v[4] = {cg[k].x, cg[k].y, cg[k].z, cg[k].w};
                float ge[4 + 2 * h];
                extend<h>(v, ge);
                const uint32_t aw[3] = {__shfl_up_sync(0xffffffffu, ca[k], 1), ca[k],
                                        __shfl_down_sync(0xffffffffu, ca[k], 1)};
                if (r - rs >= 2 * h && writes) {
                    // input row r - h: tap (i, j) came from output row
                    // r - h - dy_i (window index w) and column x - dx_j
                    float acc[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        float s = 0.f;
#pragma unroll
                        for (int i = 0; i < K; i++) {
                            const int w = MAX ? i : 2 * h - i;
#pragma unroll
                            for (int j = 0; j < K; j++) {
                                const int kx = q - (MAX ? h - j : j - h);  // column offset from c, in [-h, 3 + h]
                                const int word = kx < 0 ? 0 : (kx < 4 ? 1 : 2);
                                const int byte = kx - 4 * (word - 1);
                                const uint32_t wv = w == K - 1 ? aw[word] : raw[w][word];
                                const float gv = w == K - 1 ? ge[kx + h] : rg[w][kx + h];
                                if (((wv >> (8 * byte)) & 255u) == (uint32_t)(K * i + j)) s += gv;
                            }
                        }
                        acc[q] = s;
                    }
                    __stcs(dst + (int64_t)(r - h) * wq, make_float4(acc[0], acc[1], acc[2], acc[3]));
                }
#pragma unroll
                for (int j = 0; j + 1 < K - 1; j++) {
#pragma unroll
                    for (int q = 0; q < 4 + 2 * h; q++) rg[j][q] = rg[j + 1][q];
#pragma unroll
                    for (int q = 0; q < 3; q++) raw[j][q] = raw[j + 1][q];
                }
#pragma unroll
                for (int q = 0; q < 4 + 2 * h; q++) rg[K - 2][q] = ge[q];
#pragma unroll
                for (int q = 0; q < 3; q++) raw[K - 2][q] = aw[q];
            }
#pragma unroll
            for (int k = 0; k < kChunk; k++) {
                cg[k] = ng[k];
                ca[k] = na[k];
            }
        }
    }
}

// Outputs outside the walkers' rectangle [ry0, ry1) x [rx0, rx1) (a frame a
// few voxels wide), one thread each, straight from the definition with the
// border mode at both levels: the first operator over the input (rows
// y + lo1y .., columns x + lo1x ..), and for two stages the second operator
// over the intermediate image (rows y + lo2y .., positions outside the item
// taking cval or the intermediate value at the mapped position).  Window
// sizes are compile-time, so a window's loads are independent; where the
// rows (side bands) or the columns (top and bottom bands) of the whole
// footprint lie inside the item, the first operator runs separably over the
// 2K - 1 footprint rows (columns) shared by the intermediate positions.
struct FrameParams {
    int H, W;
    int64_t batch;
    int lo1y, lo1x, lo2y, lo2x;
    int mode;
    float cval, sval;
    int ry0, ry1, rx0, rx1;
};

__device__ __forceinline__ float frame_ld(const float *src, const FrameParams &f, int r, int c) {
    return (r < 0 || c < 0) ? f.cval : __ldg(src + (int64_t)r * f.W + c);
}

template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE>
__device__ __forceinline__ float frame_value(const float *src, const FrameParams &f, int y, int x) {
    using Op1 = MorphOp<float, MAX1>;
    using Op2 = MorphOp<float, !MAX1>;
    using morph::map_coord;
    if constexpr (STAGES == 1) {
        int R[K], C[K];
#pragma unroll
        for (int a = 0; a < K; a++) {
            R[a] = map_coord(y + f.lo1y + a, f.H, f.mode);
            C[a] = map_coord(x + f.lo1x + a, f.W, f.mode);
        }
        float acc = Op1::identity(), lo = INFINITY;
#pragma unroll
        for (int a = 0; a < K; a++)
#pragma unroll
            for (int b = 0; b < K; b++) {
                const float v = frame_ld(src, f, R[a], C[b]);
                acc = Op1::combine(acc, v);
                if (COMBINE != 0) lo = fminf(lo, v);
            }
        float o = Op1::apply(acc, f.sval);
        if (COMBINE != 0) {
            const float ev = __fsub_rn(lo, f.sval);
            o = COMBINE == kGradient ? __fsub_rn(o, ev)
                                     : __fsub_rn(__fadd_rn(o, ev), __fmul_rn(2.f, src[(int64_t)y * f.W + x]));
        }
        return o;
    } else {
        float acc2 = Op2::identity();
        const int by = y + f.lo2y + f.lo1y, bx = x + f.lo2x + f.lo1x;  // first footprint row / column
        if (by >= 0 && by + 2 * K - 2 < f.H) {
            // every row at both levels inside the item: per footprint row, the
            // first operator along each intermediate column's mapped window
            int C2[K], CC[K][K];
#pragma unroll
            for (int j = 0; j < K; j++) {
                C2[j] = map_coord(x + f.lo2x + j, f.W, f.mode);
#pragma unroll
                for (int b = 0; b < K; b++) CC[j][b] = C2[j] < 0 ? 0 : map_coord(C2[j] + f.lo1x + b, f.W, f.mode);
            }
            float rm[2 * K - 1][K];
#pragma unroll
            for (int r = 0; r < 2 * K - 1; r++)
#pragma unroll
                for (int j = 0; j < K; j++) {
                    float m = Op1::identity();
#pragma unroll
                    for (int b = 0; b < K; b++) m = Op1::combine(m, frame_ld(src, f, by + r, CC[j][b]));
                    rm[r][j] = m;
                }
#pragma unroll
            for (int i = 0; i < K; i++)
#pragma unroll
                for (int j = 0; j < K; j++) {
                    float m = rm[i][j];
#pragma unroll
                    for (int a = 1; a < K; a++) m = Op1::combine(m, rm[i + a][j]);
                    acc2 = Op2::combine(acc2, C2[j] < 0 ? f.cval : Op1::apply(m, f.sval));
                }
        } else if (bx >= 0 && bx + 2 * K - 2 < f.W) {
            // every column inside the item: the same with rows and columns swapped
            int R2[K], RR[K][K];
#pragma unroll
            for (int i = 0; i < K; i++) {
                R2[i] = map_coord(y + f.lo2y + i, f.H, f.mode);
#pragma unroll
                for (int a = 0; a < K; a++) RR[i][a] = R2[i] < 0 ? 0 : map_coord(R2[i] + f.lo1y + a, f.H, f.mode);
            }
            float cm[2 * K - 1][K];
#pragma unroll
            for (int c = 0; c < 2 * K - 1; c++)
#pragma unroll
                for (int i = 0; i < K; i++) {
                    float m = Op1::identity();
#pragma unroll
                    for (int a = 0; a < K; a++) m = Op1::combine(m, frame_ld(src, f, RR[i][a], bx + c));
                    cm[c][i] = m;
                }
#pragma unroll
            for (int i = 0; i < K; i++)
#pragma unroll
                for (int j = 0; j < K; j++) {
                    float m = cm[j][i];
#pragma unroll
                    for (int b = 1; b < K; b++) m = Op1::combine(m, cm[j + b][i]);
                    acc2 = Op2::combine(acc2, R2[i] < 0 ? f.cval : Op1::apply(m, f.sval));
                }
        } else {
            // corners: both axes mapped
#pragma unroll 1
            for (int i = 0; i < K; i++) {
                const int my = map_coord(y + f.lo2y + i, f.H, f.mode);
                int RR[K];
#pragma unroll
                for (int a = 0; a < K; a++) RR[a] = my < 0 ? 0 : map_coord(my + f.lo1y + a, f.H, f.mode);
#pragma unroll 1
                for (int j = 0; j < K; j++) {
                    const int mx = map_coord(x + f.lo2x + j, f.W, f.mode);
                    float e = f.cval;
                    if (my >= 0 && mx >= 0) {
                        float m = Op1::identity();
#pragma unroll
                        for (int b = 0; b < K; b++) {
                            const int cc = map_coord(mx + f.lo1x + b, f.W, f.mode);
#pragma unroll
                            for (int a = 0; a < K; a++) m = Op1::combine(m, frame_ld(src, f, RR[a], cc));
                        }
                        e = Op1::apply(m, f.sval);
                    }
                    acc2 = Op2::combine(acc2, e);
                }
            }
        }
        float o = Op2::apply(acc2, f.sval);
        if (TOPHAT != kTophatNone) {
            const float xv = src[(int64_t)y * f.W + x];
            o = TOPHAT == kTophatWhite ? xv - o : o - xv;
        }
        return o;
    }
}

// Position (y, x) of the k-th of the H x W positions outside the rectangle
// [ry0, ry1) x [rx0, rx1): the rows above, the side columns of the rows in
// between, the rows below.
struct FrameRect {
    int H, W, ry0, ry1, rx0, rx1;
    __host__ __device__ int count() const { return H * W - (ry1 - ry0) * (rx1 - rx0); }
    __device__ __forceinline__ void at(int k, int &y, int &x) const {
        const int side = rx0 + (W - rx1), top = ry0 * W, mid = (ry1 - ry0) * side;
        if (k < top) {
            y = k / W;
            x = k - y * W;
        } else if ((k -= top) < mid) {
            const int r = k / side;
            y = ry0 + r;
            x = k - r * side;
            if (x >= rx0) x += rx1 - rx0;
        } else {
            k -= mid;
            const int r = k / W;
            y = ry1 + r;
            x = k - r * W;
        }
    }
};

template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE>
__global__ void __launch_bounds__(256) frame_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                    FrameParams f) {
    const FrameRect fr{f.H, f.W, f.ry0, f.ry1, f.rx0, f.rx1};
    const int ring = fr.count();
    for (int64_t item = blockIdx.y; item < f.batch; item += gridDim.y) {
        const float *src = in + item * (int64_t)f.H * f.W;
        float *dst = out + item * (int64_t)f.H * f.W;
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ring; k += gridDim.x * blockDim.x) {
            int y, x;
            fr.at(k, y, x);
            dst[(int64_t)y * f.W + x] = frame_value<MAX1, STAGES, TOPHAT, K, COMBINE>(src, f, y, x);
        }
    }
    // launched behind the walkers (programmatic dependent launch): finish only
    // once they have, so the next work of the stream sees every output
    pdl_wait();
}

// Launches the frame kernel for the outputs outside the rectangle.  Right
// behind a walker launch it may start early (programmatic dependent launch:
// the frame reads only the input and writes only its own outputs); behind
// anything else it is an ordinary launch.
template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE = 0>
int launch_frame(const float *in, float *out, const FrameParams &f, cudaStream_t s, bool behind_walker) {
    const int64_t ring = (int64_t)f.H * f.W - (int64_t)(f.ry1 - f.ry0) * (f.rx1 - f.rx0);
    if (ring <= 0 || f.batch <= 0) return TM_OK;
    const unsigned gy = (unsigned)std::min<int64_t>(f.batch, 65535);
    if (behind_walker && STAGES == 1) {
        // one stage (9 or 25 loads per output): blocks of 64 threads fit beside
        // the walker's CTAs (in the registers a 3 x 3 walk leaves: 65536 -
        // 3 x 256 x 80 = 4096), so the frame is computed while the walker
        // streams: about one block per SM, at most 32 outputs per thread
        const int64_t want = std::max<int64_t>(sm_count(), ceil_div(ring * f.batch, 64 * 32));
        const unsigned gx = (unsigned)std::max<int64_t>(1, ceil_div(want, gy));
        TM_CHECK_CUDA(
            launch_pdl(frame_kernel<MAX1, STAGES, TOPHAT, K, COMBINE>, dim3(gx, gy), dim3(64), 0, s, in, out, f));
        return TM_OK;
    }
    // two stages (45 or more loads per output): a full wave of one output per
    // thread, behind the walker's last CTAs
    const int64_t want = std::max<int64_t>(1, (int64_t)sm_count() * 16 / gy);
    const unsigned gx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ring, 256), want));
    if (behind_walker) {
        TM_CHECK_CUDA(
            launch_pdl(frame_kernel<MAX1, STAGES, TOPHAT, K, COMBINE>, dim3(gx, gy), dim3(256), 0, s, in, out, f));
    } else {
        frame_kernel<MAX1, STAGES, TOPHAT, K, COMBINE><<<dim3(gx, gy), 256, 0, s>>>(in, out, f);
        TM_LAUNCH_CHECK("vwalk::frame_kernel");
    }
    return TM_OK;
}

// Plans the walk: false when the item does not fit (rows not 16-byte
// aligned, too narrow or too short).  resident_warps is the number of walker
// warps the device holds at once; the row block is chosen so the tasks fill
// whole waves of them.
// margin: rows kept out of the walk beyond the lag on each side.
inline bool plan(int H, int W, int64_t batch, int K, int stages, const void *in, const void *out,
                 int64_t resident_warps, Params &p, int margin = 0) {
    const int lag = stages * (K / 2);
    if (W % 4 != 0 || W < 16 || H < 2 * (lag + margin) + 1) return false;
    if ((reinterpret_cast<uintptr_t>(in) & 15) || (reinterpret_cast<uintptr_t>(out) & 15)) return false;
    p.H = H;
    p.W = W;
    p.batch = batch;
    p.ry0 = lag + margin;
    p.ry1 = H - lag - margin;
    p.nstrips = (W - 8 + kStrip - 1) / kStrip;
    const int rows = p.ry1 - p.ry0;
    // cost of a candidate row block: waves of tasks x rows each task reads
    double best = 0.0;
    p.rows = 0;
    for (int R = 8; R <= 64; R += 4) {
        const int nrb = (rows + R - 1) / R;
        const int64_t tasks = batch * nrb * (int64_t)p.nstrips;
        const double waves = std::ceil((double)tasks / (double)std::max<int64_t>(resident_warps, 1));
        const double cost = waves * (R + 2 * lag);
        if (p.rows == 0 || cost < best) {
            best = cost;
            p.rows = R;
        }
    }
    p.nrb = (rows + p.rows - 1) / p.rows;
    p.ntasks = batch * p.nrb * (int64_t)p.nstrips;
    return true;
}

// Centred K x K flat window (value sval) of float32 items: the walkers, then
// the frame kernel launched behind them.  Sets *done = false and launches
// nothing when the items do not fit the walkers.
template <bool MAX1, int STAGES, int TOPHAT, int K, int COMBINE = 0>
int run(const float *in, float *out, int H, int W, int64_t batch, int mode, float cval, float sval, cudaStream_t s,
        bool *done) {
    *done = false;
    static thread_local int cached_dev = -1, cached_per_sm = 1;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev != dev) {
        int per_sm = 0;
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, vwalk_kernel<MAX1, STAGES, TOPHAT, K, COMBINE>, kThreads, 0));
        cached_per_sm = std::max(per_sm, 1);
        cached_dev = dev;
    }
    const int64_t resident_blocks = (int64_t)sm_count() * cached_per_sm;
    Params p;
    if (!plan(H, W, batch, K, STAGES, in, out, resident_blocks * (kThreads / 32), p)) return TM_OK;
    p.sval = sval;
    *done = true;
    FrameParams f;
    f.H = H;
    f.W = W;
    f.batch = batch;
    f.lo1y = f.lo1x = f.lo2y = f.lo2x = -(K / 2);
    f.mode = mode;
    f.cval = cval;
    f.sval = sval;
    f.ry0 = p.ry0;
    f.ry1 = p.ry1;
    f.rx0 = 4;
    f.rx1 = W - 4;
    const int64_t blocks = std::min<int64_t>(ceil_div(p.ntasks, kThreads / 32), resident_blocks);
    if (p.ntasks > 0) vwalk_kernel<MAX1, STAGES, TOPHAT, K, COMBINE><<<(unsigned)blocks, kThreads, 0, s>>>(in, out, p);
    TM_LAUNCH_CHECK("vwalk_kernel");
    return launch_frame<MAX1, STAGES, TOPHAT, K, COMBINE>(in, out, f, s, p.ntasks > 0);
}

}  // namespace vwalk
}  // namespace tmc
