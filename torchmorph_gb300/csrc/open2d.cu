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
#include <cstring>

#include "morph_tile.cuh"

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
    const int64_t item = blockIdx.x / ((int64_t)tiles_x * tiles_y);
    const int rem = (int)(blockIdx.x - item * (int64_t)tiles_x * tiles_y);
    const int y0 = (rem / tiles_x) * kOTileH, x0 = (rem % tiles_x) * kOTileW;
    const float *src = in + item * (int64_t)p.H * p.W;
    float *dst = out + item * (int64_t)p.H * p.W;
    const int tid = threadIdx.x;
    const int iy0 = y0 + p.lo2y + p.lo1y, ix0 = x0 + p.lo2x + p.lo1x;  // item position of s0[0]
    const int my0 = y0 + p.lo2y, mx0 = x0 + p.lo2x;                    // item position of s1[0]
    // stage the input region with the border mapping
    for (int i = tid; i < RH0 * RW0; i += kOThreads) {
        const int r = i / RW0, c = i - r * RW0;
        const int yy = map_coord(iy0 + r, p.H, p.mode), xx = map_coord(ix0 + c, p.W, p.mode);
        s0[i] = (yy < 0 || xx < 0) ? p.cval : src[(int64_t)yy * p.W + xx];
    }
    __syncthreads();
    // first operator: row pass (RH0 x RW1), then column pass (RH1 x RW1)
    for (int i = tid; i < RH0 * RW1; i += kOThreads) {
        const int r = i / RW1, c = i - r * RW1;
        const float *row = s0 + r * RW0 + c;
        float acc = row[0];
        for (int j = 1; j < p.kw; j++) acc = Op1::combine(acc, row[j]);
        rowb[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < RH1 * RW1; i += kOThreads) {
        const int r = i / RW1, c = i - r * RW1;
        const float *col = rowb + r * RW1 + c;
        float acc = col[0];
        for (int j = 1; j < p.kh; j++) acc = Op1::combine(acc, col[j * RW1]);
        s1[i] = Op1::apply(acc, p.sval);
    }
    __syncthreads();
    // the intermediate image's own border: positions outside the item take cval
    // or the value at the mapped position (inside the item)
    for (int i = tid; i < RH1 * RW1; i += kOThreads) {
        const int r = i / RW1, c = i - r * RW1;
        const int yy = my0 + r, xx = mx0 + c;
        if ((unsigned)yy < (unsigned)p.H && (unsigned)xx < (unsigned)p.W) continue;
        const int my = map_coord(yy, p.H, p.mode), mx = map_coord(xx, p.W, p.mode);
        float v;
        if (my < 0 || mx < 0) {
            v = p.cval;
        } else {
            const int rr = my - my0, cc = mx - mx0;
            v = ((unsigned)rr < (unsigned)RH1 && (unsigned)cc < (unsigned)RW1) ? s1[rr * RW1 + cc]
                                                                               : first_at<MAX1>(src, p, my, mx);
        }
        rowb[i] = v;  // staged apart: every in-item value above stays readable
    }
    __syncthreads();
    for (int i = tid; i < RH1 * RW1; i += kOThreads) {
        const int r = i / RW1, c = i - r * RW1;
        const int yy = my0 + r, xx = mx0 + c;
        if (!((unsigned)yy < (unsigned)p.H && (unsigned)xx < (unsigned)p.W)) s1[i] = rowb[i];
    }
    __syncthreads();
    // second operator: row pass (RH1 x 128), then the column pass to the outputs
    for (int i = tid; i < RH1 * kOTileW; i += kOThreads) {
        const int r = i / kOTileW, c = i - r * kOTileW;
        const float *row = s1 + r * RW1 + c;
        float acc = row[0];
        for (int j = 1; j < p.kw; j++) acc = Op2::combine(acc, row[j]);
        rowb[r * kOTileW + c] = acc;
    }
    __syncthreads();
    for (int i = tid; i < kOTileH * kOTileW; i += kOThreads) {
        const int r = i / kOTileW, c = i - r * kOTileW;
        const int yy = y0 + r, xx = x0 + c;
        if (yy >= p.H || xx >= p.W) continue;
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
    const size_t smem = open2d_smem(p.kh, p.kw);
    auto kernel = open2d_kernel<MAX1, TOPHAT>;
    if (smem > 48 * 1024)
        TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t tiles = batch * ceil_div(p.W, kOTileW) * ceil_div(p.H, kOTileH);
    if (tiles >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many tiles");
    kernel<<<(unsigned)tiles, kOThreads, smem, s>>>(in, out, p);
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
