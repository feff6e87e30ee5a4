// One-pass grey opening, closing and top-hats of 1-D / 2-D items with flat
// rectangular elements (GB300, sm_103a).
//
// The reference composes two full operator launches and, for the top-hats,
// a torch subtraction (torchmorph/morphology/grey.py:162-197, 224-265): the
// intermediate image makes a round trip through HBM (opening 16 B/pixel,
// top-hat 28 B/pixel).  Here one CTA computes a 32 x 128 output tile from a
// shared-memory copy of its input region grown by twice the window: the
// first operator over the region the second one reads, then the second
// operator (and the top-hat difference) straight to the output -- 8 B/pixel.
//
// Both operators keep the reference's semantics exactly:
//   first  = erosion (opening) or dilation (closing) of the input, with the
//            input's border mode;
//   second = the other operator applied to the first one's IMAGE, whose own
//            border is again the mode: positions of the intermediate outside
//            the item take cval (constant) or the intermediate value at the
//            mapped position (reflect, mirror, nearest, wrap).  A mapped
//            position inside the tile's computed region is read from shared
//            memory; any other (tiles at the edge of small items, wrap) is
//            recomputed from the input in global memory.
// Flat elements with one structure value s: erosion min(x) - s, dilation
// max(x) + s, rounded as the reference's per-tap x -/+ s (both are monotone
// in x).  Top-hats: white = x - opening, black = closing - x, float32 as the
// reference's torch subtraction.
#include <algorithm>
#include <cstring>

#include "morph_tile.cuh"
#include "vwalk.cuh"

namespace tmc {
namespace {

using namespace morph;

constexpr int kOTileH = 32, kOTileW = 128, kOThreads = 256;
constexpr int kOMaxK = 33;  // windows up to 33 x 33

struct Open2DParams {
    int H, W, kh, kw;
    int lo1y, lo1x, lo2y, lo2x;  // windows: output (y, x) of an operator reads rows y + lo .. y + lo + k - 1
    int mode;
    float cval, sval;
    int64_t batch;
    // outputs computed by open2d_walk_kernel (the tile kernel skips them):
    // rows ry0 <= y < ry1, columns rx0 <= x < rx1 of every item (empty when ry0 >= ry1)
    int ry0, ry1, rx0, rx1;
    // tiles (32 x 128) inside that rectangle: tile rows [tr0, tr1), columns [tc0, tc1)
    int tr0, tr1, tc0, tc1;
};

enum { kTophatNone = 0, kTophatWhite = 1, kTophatBlack = 2 };

// The first operator at item position (y, x) (inside the item), from global memory.
template <bool MAX1>
__device__ float first_at(const float *src, const Open2DParams &p, int y, int x) {
    using Op = MorphOp<float, MAX1>;
    float acc = Op::identity();
    for (int i = 0; i < p.kh; i++) {
        const int my = map_coord(y + p.lo1y + i, p.H, p.mode);
        for (int j = 0; j < p.kw; j++) {
            const int mx = map_coord(x + p.lo1x + j, p.W, p.mode);
            const float v = (my < 0 || mx < 0) ? p.cval : src[(int64_t)my * p.W + mx];
            acc = Op::combine(acc, v);
        }
    }
    return Op::apply(acc, p.sval);
}

// MAX1: the first operator is a dilation (closing); else an erosion (opening).
template <bool MAX1, int TOPHAT>
__global__ void __launch_bounds__(kOThreads) open2d_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                           Open2DParams p) {
    using Op1 = MorphOp<float, MAX1>;
    using Op2 = MorphOp<float, !MAX1>;
    extern __shared__ __align__(16) float osm[];
    // region of the second operator's reads (the intermediate): rows y0 + lo2y .., RH1 x RW1
    const int RH1 = kOTileH + p.kh - 1, RW1 = kOTileW + p.kw - 1;
    // region of the first operator's reads: RH0 x RW0
    const int RH0 = RH1 + p.kh - 1, RW0 = RW1 + p.kw - 1;
    float *s0 = osm;                  // input region, RH0 x RW0
    float *rowb = s0 + RH0 * RW0;     // row pass of either operator, RH0 x RW1
    float *s1 = rowb + RH0 * RW1;     // intermediate, RH1 x RW1
    const int tiles_x = (p.W + kOTileW - 1) / kOTileW, tiles_y = (p.H + kOTileH - 1) / kOTileH;
    // this CTA's tile: the k-th of the item's tiles that the walkers do not cover
    // entirely (tile rows [tr0, tr1) and columns [tc0, tc1) are theirs)
    const int ring = tiles_x * tiles_y - (p.tr1 - p.tr0) * (p.tc1 - p.tc0);
    const int64_t item = blockIdx.x / ring;
    int k = (int)(blockIdx.x - item * ring), ty, tx;
    const int top = p.tr0 * tiles_x, side = p.tc0 + (tiles_x - p.tc1);
    if (k < top) {
        ty = k / tiles_x;
        tx = k % tiles_x;
    } else if ((k -= top) < (p.tr1 - p.tr0) * side) {
        ty = p.tr0 + k / side;
        tx = k % side;
        if (tx >= p.tc0) tx += p.tc1 - p.tc0;
    } else {
        k -= (p.tr1 - p.tr0) * side;
        ty = p.tr1 + k / tiles_x;
        tx = k % tiles_x;
    }
    const int y0 = ty * kOTileH, x0 = tx * kOTileW;
    const float *src = in + item * (int64_t)p.H * p.W;
    float *dst = out + item * (int64_t)p.H * p.W;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kOThreads / 32;
    const int iy0 = y0 + p.lo2y + p.lo1y, ix0 = x0 + p.lo2x + p.lo1x;  // item position of s0[0]
    const int my0 = y0 + p.lo2y, mx0 = x0 + p.lo2x;                    // item position of s1[0]
    // stage the input region, a warp per row and every load of a row chunk in
    // flight before its stores; the border mapping only for tiles that need it
    const bool interior = iy0 >= 0 && ix0 >= 0 && iy0 + RH0 <= p.H && ix0 + RW0 <= p.W;
    constexpr int kNC = 5;
    for (int r = warp; r < RH0; r += kWarps) {
        const int yy = interior ? iy0 + r : map_coord(iy0 + r, p.H, p.mode);
        const float *row = src + (int64_t)(yy < 0 ? 0 : yy) * p.W;
        for (int c0 = 0; c0 < RW0; c0 += 32 * kNC) {
            float v[kNC];
#pragma unroll
            for (int j = 0; j < kNC; j++) {
                const int c = c0 + lane + 32 * j;
                v[j] = p.cval;
                if (c < RW0) {
                    const int xx = interior ? ix0 + c : map_coord(ix0 + c, p.W, p.mode);
                    if (yy >= 0 && xx >= 0) v[j] = row[xx];
                }
            }
#pragma unroll
            for (int j = 0; j < kNC; j++) {
                const int c = c0 + lane + 32 * j;
                if (c < RW0) s0[r * RW0 + c] = v[j];
            }
        }
    }
    __syncthreads();
    // first operator: row pass (RH0 x RW1), then column pass (RH1 x RW1)
    for (int r = warp; r < RH0; r += kWarps)
        for (int c = lane; c < RW1; c += 32) {
            const float *row = s0 + r * RW0 + c;
            float acc = row[0];
            for (int j = 1; j < p.kw; j++) acc = Op1::combine(acc, row[j]);
            rowb[r * RW1 + c] = acc;
        }
    __syncthreads();
    for (int r = warp; r < RH1; r += kWarps)
        for (int c = lane; c < RW1; c += 32) {
            const float *col = rowb + r * RW1 + c;
            float acc = col[0];
            for (int j = 1; j < p.kh; j++) acc = Op1::combine(acc, col[j * RW1]);
            s1[r * RW1 + c] = Op1::apply(acc, p.sval);
        }
    __syncthreads();
    // the intermediate image's own border: positions outside the item take cval
    // or the value at the mapped position (inside the item); nothing to do when
    // the whole intermediate region lies inside the item
    if (!(my0 >= 0 && mx0 >= 0 && my0 + RH1 <= p.H && mx0 + RW1 <= p.W)) {
        for (int r = warp; r < RH1; r += kWarps)
            for (int c = lane; c < RW1; c += 32) {
                const int yy = my0 + r, xx = mx0 + c;
                if ((unsigned)yy < (unsigned)p.H && (unsigned)xx < (unsigned)p.W) continue;
                const int my = map_coord(yy, p.H, p.mode), mx = map_coord(xx, p.W, p.mode);
                float v;
                if (my < 0 || mx < 0) {
                    v = p.cval;
                } else {
                    const int rr = my - my0, cc = mx - mx0;
                    v = ((unsigned)rr < (unsigned)RH1 && (unsigned)cc < (unsigned)RW1)
                            ? s1[rr * RW1 + cc]
                            : first_at<MAX1>(src, p, my, mx);
                }
                rowb[r * RW1 + c] = v;  // staged apart: every in-item value above stays readable
            }
        __syncthreads();
        for (int r = warp; r < RH1; r += kWarps)
            for (int c = lane; c < RW1; c += 32) {
                const int yy = my0 + r, xx = mx0 + c;
                if (!((unsigned)yy < (unsigned)p.H && (unsigned)xx < (unsigned)p.W)) s1[r * RW1 + c] = rowb[r * RW1 + c];
            }
        __syncthreads();
    }
    // second operator: row pass (RH1 x 128), then the column pass to the outputs
    for (int r = warp; r < RH1; r += kWarps)
        for (int c = lane; c < kOTileW; c += 32) {
            const float *row = s1 + r * RW1 + c;
            float acc = row[0];
            for (int j = 1; j < p.kw; j++) acc = Op2::combine(acc, row[j]);
            rowb[r * kOTileW + c] = acc;
        }
    __syncthreads();
    for (int r = warp; r < kOTileH; r += kWarps) {
        const int yy = y0 + r;
        if (yy >= p.H) break;
        const bool row_in = yy >= p.ry0 && yy < p.ry1;
        for (int c = lane; c < kOTileW; c += 32) {
            const int xx = x0 + c;
            if (xx >= p.W) break;
            if (row_in && xx >= p.rx0 && xx < p.rx1) continue;  // written by the walkers
            const float *col = rowb + r * kOTileW + c;
            float acc = col[0];
            for (int j = 1; j < p.kh; j++) acc = Op2::combine(acc, col[j * kOTileW]);
            float v = Op2::apply(acc, p.sval);
            if (TOPHAT != kTophatNone) {
                const float x = s0[(yy - iy0) * RW0 + (xx - ix0)];  // the input at (yy, xx)
                v = TOPHAT == kTophatWhite ? x - v : v - x;
            }
            dst[(int64_t)yy * p.W + xx] = v;
        }
    }
}

// Outputs whose whole input footprint (and the intermediate values they use)
// lie inside the item, for compile-time KH x KW windows: each warp owns a strip
// of 32 - (KW - 1) output columns and walks kWalkRows rows down it.  Lane l
// holds the intermediate column x0 + lo2x + l: per input row it loads one input
// column (lanes < KW - 1 one more, 32 to the right) and takes the first
// operator's row window from the neighbouring lanes by shuffles (the loads of the
// next 8 input rows in flight while the current 8 are used), the column window
// over the last KH rows in registers; the
// second operator's row window for output column x0 + l reads lanes l .. l + KW - 1
// by warp shuffles, its column window is again a register window.  No border
// mapping anywhere: the rectangle excludes every output that would need it.
constexpr int kWalkRows = 64;
constexpr int kWalkChunk = 8;  // input rows per chunk (two chunks of loads in flight)

template <bool MAX1, int TOPHAT, int KH, int KW>
__global__ void __launch_bounds__(256) open2d_walk_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                          Open2DParams p) {
    using Op1 = MorphOp<float, MAX1>;
    using Op2 = MorphOp<float, !MAX1>;
    static_assert(KW <= 16 && KH >= 1, "window");
    constexpr int kSW = 32 - (KW - 1);  // output columns per strip
    const int lane = threadIdx.x & 31;
    const int strips = (p.rx1 - p.rx0 + kSW - 1) / kSW, rblocks = (p.ry1 - p.ry0 + kWalkRows - 1) / kWalkRows;
    const int64_t per_item = (int64_t)strips * rblocks;
    const int64_t ntasks = p.batch * per_item;
    for (int64_t task = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); task < ntasks;
         task += (int64_t)gridDim.x * (blockDim.x / 32)) {
        const int64_t item = task / per_item;
        const int rem = (int)(task - item * per_item);
        const int sx = rem % strips, by = rem / strips;
        const int x0 = p.rx0 + kSW * sx, ya = p.ry0 + kWalkRows * by;
        const int yb = min(ya + kWalkRows, p.ry1);
        const float *src = in + item * (int64_t)p.H * p.W;
        float *dst = out + item * (int64_t)p.H * p.W;
        // lane l loads input column x0 + lo2x + lo1x + l of each row (lanes < KW - 1
        // also the column 32 further right); the first operator's row window of
        // intermediate column x0 + lo2x + l is then lanes l .. l + KW - 1 of those
        // values, taken by shuffles.  Every input column a rectangle output uses is
        // inside the item; the others are clamped to its last column, so every load
        // stays inside the item and the values that matter are unchanged.
        const int c0 = x0 + p.lo2x + p.lo1x;
        const int ca = min(c0 + lane, p.W - 1), cb = min(c0 + 32 + lane, p.W - 1);
        const bool halo = lane < KW - 1;
        const int i0 = ya + p.lo2y;  // first intermediate row
        float h1[KH];  // the first operator's row results of the last KH input rows
        float v2[KH];  // the second operator's row results of the last KH intermediate rows
        auto row_window = [&](float a, float b) {  // all lanes together (shuffles)
            float acc = a;
#pragma unroll
            for (int j = 1; j < KW; j++) {
                const int sl = lane + j;
                const float va = __shfl_sync(~0u, a, sl & 31);
                const float vb = __shfl_sync(~0u, b, sl & 31);
                acc = Op1::combine(acc, sl < 32 ? va : vb);
            }
            return acc;
        };
#pragma unroll
        for (int k = 0; k < KH - 1; k++) {
            const float *r = src + (int64_t)(i0 + p.lo1y + k) * p.W;
            const float a = __ldg(r + ca), b = halo ? __ldg(r + cb) : 0.0f;
            h1[k] = row_window(a, b);
        }
        const int nint = (yb - ya) + KH - 1;            // intermediate rows to produce
        const int ylast = i0 + p.lo1y + nint + KH - 2;  // last input row read
        // the loads of the next chunk are issued before the current chunk is used
        // (two chunks in flight); rows past the end repeat the last row
        float na[kWalkChunk], nb[kWalkChunk];
#pragma unroll
        for (int u = 0; u < kWalkChunk; u++) {
            const float *r = src + (int64_t)min(i0 + p.lo1y + u + KH - 1, ylast) * p.W;
            na[u] = __ldg(r + ca);
            nb[u] = halo ? __ldg(r + cb) : 0.0f;
        }
        for (int t0 = 0; t0 < nint; t0 += kWalkChunk) {
            float ra[kWalkChunk], rb[kWalkChunk];
#pragma unroll
            for (int u = 0; u < kWalkChunk; u++) {
                ra[u] = na[u];
                rb[u] = nb[u];
            }
            if (t0 + kWalkChunk < nint) {
#pragma unroll
                for (int u = 0; u < kWalkChunk; u++) {
                    const float *r = src + (int64_t)min(i0 + p.lo1y + t0 + kWalkChunk + u + KH - 1, ylast) * p.W;
                    na[u] = __ldg(r + ca);
                    nb[u] = halo ? __ldg(r + cb) : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < kWalkChunk; u++) {
                const int t = t0 + u;
                if (t >= nint) continue;  // uniform; (not break: the loop stays unrolled)
                h1[KH - 1] = row_window(ra[u], rb[u]);
                float iv = h1[0];
#pragma unroll
                for (int k = 1; k < KH; k++) iv = Op1::combine(iv, h1[k]);
                iv = Op1::apply(iv, p.sval);
#pragma unroll
                for (int k = 0; k < KH - 1; k++) h1[k] = h1[k + 1];
                float acc = iv;
#pragma unroll
                for (int j = 1; j < KW; j++) acc = Op2::combine(acc, __shfl_down_sync(~0u, iv, j));
                v2[KH - 1] = acc;
                if (t >= KH - 1) {  // output row ya + t - (KH - 1)
                    float o = v2[0];
#pragma unroll
                    for (int k = 1; k < KH; k++) o = Op2::combine(o, v2[k]);
                    o = Op2::apply(o, p.sval);
                    const int y = ya + t - (KH - 1), x = x0 + lane;
                    if (lane < kSW && x < p.rx1) {
                        if (TOPHAT != kTophatNone) {
                            const float xv = __ldg(src + (int64_t)y * p.W + x);
                            o = TOPHAT == kTophatWhite ? xv - o : o - xv;
                        }
                        dst[(int64_t)y * p.W + x] = o;
                    }
                }
#pragma unroll
                for (int k = 0; k < KH - 1; k++) v2[k] = v2[k + 1];
            }
        }
    }
}

// The rectangle of outputs the walkers can take (see open2d_walk_kernel).
void walk_rect(Open2DParams &p) {
    // output y reads intermediate rows y + lo2y .. y + lo2y + kh - 1 (all inside the item)
    // and those read input rows + lo1y .. + lo1y + kh - 1 (all inside the item)
    auto range = [](int lo1, int lo2, int k, int n, int &a, int &b) {
        a = std::max(-lo2, -(lo2 + lo1));
        b = std::min(n - (lo2 + k - 1), n - (lo2 + lo1 + 2 * k - 2));
        if (b < a) b = a;
    };
    range(p.lo1y, p.lo2y, p.kh, p.H, p.ry0, p.ry1);
    range(p.lo1x, p.lo2x, p.kw, p.W, p.rx0, p.rx1);
    if (p.ry1 <= p.ry0 || p.rx1 <= p.rx0) p.ry0 = p.ry1 = p.rx0 = p.rx1 = 0;
}

size_t open2d_smem(int kh, int kw) {
    const size_t RH1 = kOTileH + kh - 1, RW1 = kOTileW + kw - 1;
    const size_t RH0 = RH1 + kh - 1, RW0 = RW1 + kw - 1;
    return (RH0 * RW0 + RH0 * RW1 + RH1 * RW1) * sizeof(float);
}

template <bool MAX1, int TOPHAT>
int run_open2d(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape, const float *structure,
               const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
               cudaStream_t s) {
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (!in || !out) return fail(TM_ERR_INVALID_ARGUMENT, "input/output pointer is NULL");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    if (!sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "structure shape/origin is NULL");
    if (mode < 0 || mode > 4) return fail(TM_ERR_INVALID_ARGUMENT, "unknown border mode %d", mode);
    if (ndim < 1 || ndim > 2)
        return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take 1-D or 2-D items (compose the operators)");
    int64_t stotal = 1;
    for (int d = 0; d < ndim; d++) {
        if (sshape[d] < 1 || sshape[d] > kOMaxK)
            return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take windows up to %d per axis", kOMaxK);
        if (origin[d] < -(sshape[d] / 2) || origin[d] > (sshape[d] - 1) / 2)
            return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
        stotal *= sshape[d];
    }
    float sval = structure ? structure[0] : 0.0f;
    for (int64_t i = 0; i < stotal; i++) {
        if (footprint && !footprint[i])
            return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take full rectangular footprints");
        if (structure && std::memcmp(&structure[i], &sval, sizeof(float)) != 0)
            return fail(TM_ERR_UNSUPPORTED, "the one-pass composites take flat (uniform) structures");
    }
    if (g.numel_item >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels");
    Open2DParams p;
    p.H = ndim == 2 ? (int)shape[0] : 1;
    p.W = (int)shape[ndim - 1];
    p.kh = ndim == 2 ? (int)sshape[0] : 1;
    p.kw = (int)sshape[ndim - 1];
    const int cy = ndim == 2 ? (int)(sshape[0] / 2 + origin[0]) : 0;
    const int cx = (int)(sshape[ndim - 1] / 2 + origin[ndim - 1]);
    // erosion window [x - c, x - c + k - 1]; dilation [x + c - k + 1, x + c]
    auto lo = [](bool dil, int c, int k) { return dil ? c - k + 1 : -c; };
    p.lo1y = lo(MAX1, cy, p.kh);
    p.lo1x = lo(MAX1, cx, p.kw);
    p.lo2y = lo(!MAX1, cy, p.kh);
    p.lo2x = lo(!MAX1, cx, p.kw);
    p.mode = mode;
    p.cval = cval;
    p.sval = sval;
    p.batch = batch;
    p.ry0 = p.ry1 = p.rx0 = p.rx1 = 0;
    const bool walk = ndim == 2 && ((p.kh == 3 && p.kw == 3) || (p.kh == 5 && p.kw == 5));
    if (walk && cy == p.kh / 2 && cx == p.kw / 2) {
        // centred windows on 16-byte aligned rows: float4 register walkers and a frame
        bool done = false;
        st = p.kh == 3 ? vwalk::run<MAX1, 2, TOPHAT, 3>(in, out, p.H, p.W, batch, mode, cval, p.sval, s, &done)
                       : vwalk::run<MAX1, 2, TOPHAT, 5>(in, out, p.H, p.W, batch, mode, cval, p.sval, s, &done);
        if (st != TM_OK || done) return st;
    }
    if (walk) walk_rect(p);
    if (p.ry1 > p.ry0) {
        const int sw = 32 - (p.kw - 1);
        const int64_t tasks = batch * (int64_t)((p.rx1 - p.rx0 + sw - 1) / sw) *
                              ((p.ry1 - p.ry0 + kWalkRows - 1) / kWalkRows);
        const int64_t blocks = std::min<int64_t>(ceil_div(tasks, 8), (int64_t)sm_count() * 8);
        if (p.kh == 3) open2d_walk_kernel<MAX1, TOPHAT, 3, 3><<<(unsigned)blocks, 256, 0, s>>>(in, out, p);
        else open2d_walk_kernel<MAX1, TOPHAT, 5, 5><<<(unsigned)blocks, 256, 0, s>>>(in, out, p);
        TM_LAUNCH_CHECK("open2d_walk_kernel");
    }
    // a thin frame outside the rectangle: one thread per output
    if (p.ry1 > p.ry0) {
        const int64_t frame = (int64_t)p.H * p.W - (int64_t)(p.ry1 - p.ry0) * (p.rx1 - p.rx0);
        if (frame * 16 <= (int64_t)p.H * p.W) {
            vwalk::FrameParams f;
            f.H = p.H;
            f.W = p.W;
            f.batch = batch;
            f.lo1y = p.lo1y;
            f.lo1x = p.lo1x;
            f.lo2y = p.lo2y;
            f.lo2x = p.lo2x;
            f.mode = p.mode;
            f.cval = p.cval;
            f.sval = p.sval;
            f.ry0 = p.ry0;
            f.ry1 = p.ry1;
            f.rx0 = p.rx0;
            f.rx1 = p.rx1;
            return p.kh == 3 ? vwalk::launch_frame<MAX1, 2, TOPHAT, 3>(in, out, f, s, false)
                             : vwalk::launch_frame<MAX1, 2, TOPHAT, 5>(in, out, f, s, false);
        }
    }
    // tiles entirely inside the walkers' rectangle are skipped by the tile kernel
    const int tiles_x = (int)ceil_div(p.W, kOTileW), tiles_y = (int)ceil_div(p.H, kOTileH);
    p.tr0 = p.tr1 = p.tc0 = p.tc1 = 0;
    if (p.ry1 > p.ry0) {
        p.tr0 = (int)ceil_div(p.ry0, kOTileH);
        p.tr1 = std::max(p.tr0, p.ry1 / kOTileH);
        p.tc0 = (int)ceil_div(p.rx0, kOTileW);
        p.tc1 = std::max(p.tc0, p.rx1 / kOTileW);
        if (p.tr1 == p.tr0 || p.tc1 == p.tc0) p.tr0 = p.tr1 = p.tc0 = p.tc1 = 0;
    }
    const size_t smem = open2d_smem(p.kh, p.kw);
    auto kernel = open2d_kernel<MAX1, TOPHAT>;
    if (smem > 48 * 1024)
        TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t ring = (int64_t)tiles_x * tiles_y - (int64_t)(p.tr1 - p.tr0) * (p.tc1 - p.tc0);
    const int64_t tiles = batch * ring;
    if (tiles >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many tiles");
    if (tiles > 0) kernel<<<(unsigned)tiles, kOThreads, smem, s>>>(in, out, p);
    TM_LAUNCH_CHECK("open2d_kernel");
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" int tm_grey_opening(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_open2d<false, tmc::kTophatNone>(in, out, batch, ndim, shape, structure, footprint, sshape, origin,
                                                    mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_grey_closing(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_open2d<true, tmc::kTophatNone>(in, out, batch, ndim, shape, structure, footprint, sshape, origin,
                                                   mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_white_tophat(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_open2d<false, tmc::kTophatWhite>(in, out, batch, ndim, shape, structure, footprint, sshape,
                                                     origin, mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_black_tophat(const float *in, float *out, int64_t batch, int ndim, const int64_t *shape,
                               const float *structure, const uint8_t *footprint, const int64_t *sshape,
                               const int64_t *origin, int mode, float cval, tm_stream_t stream) {
    return tmc::run_open2d<true, tmc::kTophatBlack>(in, out, batch, ndim, shape, structure, footprint, sshape,
                                                    origin, mode, cval, (cudaStream_t)stream);
}
