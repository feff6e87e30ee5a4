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
#include <cstring>
#include <vector>

#include "morph_tile.cuh"
#include "tm_common.cuh"

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
// up to two ranges r[0..1], r[2..3]; returns the number of ranges.
__device__ __forceinline__ int preimage_ranges(int c, int n, int mode, int lo, int hi, int *r) {
    int cnt = 0;
    auto add = [&](int a, int b) {
        a = a > lo ? a : lo;
        b = b < hi ? b : hi;
        if (a <= b) {
            r[2 * cnt] = a;
            r[2 * cnt + 1] = b;
            cnt++;
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
    return cnt;
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
        const float *g = gout + item * p.numel_item;
        const uint8_t *a = arg + item * p.numel_item;
        int c[kGradMaxDims];
        coords_of(sp, p, c);
        // interior: every tap's output o = j - off is in the image, and no
        // out-of-image coordinate a tap can reach maps onto j (mirror maps
        // -h onto h, hence the extra voxel)
        bool interior = true;
        for (int d = 0; d < p.ndim; d++) interior &= c[d] > p.halo[d] && c[d] < p.shape[d] - 1 - p.halo[d];
        float acc = 0.f;
        if (interior) {
            for (int t = 0; t < p.ntaps; t++) {
                const int64_t o = sp - taps.flat[t];
                if (a[o] == t) acc += g[o];
            }
        } else {
            for (int t = 0; t < p.ntaps; t++) {
                int rng[kGradMaxDims][4], nr[kGradMaxDims];
                bool none = false;
                for (int d = 0; d < kGradMaxDims; d++) {
                    if (d < p.ndim) {
                        const int off = taps.off[t][d];
                        nr[d] = preimage_ranges(c[d], p.shape[d], p.mode, off, off + p.shape[d] - 1, rng[d]);
                        none |= nr[d] == 0;
                    } else {
                        nr[d] = 1;
                        rng[d][0] = rng[d][1] = 0;
                    }
                }
                if (none) continue;
                for (int r0 = 0; r0 < nr[0]; r0++)
                    for (int y0 = rng[0][2 * r0]; y0 <= rng[0][2 * r0 + 1]; y0++)
                        for (int r1 = 0; r1 < nr[1]; r1++)
                            for (int y1 = rng[1][2 * r1]; y1 <= rng[1][2 * r1 + 1]; y1++)
                                for (int r2 = 0; r2 < nr[2]; r2++)
                                    for (int y2 = rng[2][2 * r2]; y2 <= rng[2][2 * r2 + 1]; y2++) {
                                        const int y[3] = {y0, y1, y2};
                                        int64_t o = 0;
                                        for (int d = 0; d < p.ndim; d++)
                                            o += (int64_t)(y[d] - taps.off[t][d]) * p.stride[d];
                                        if (a[o] == t) acc += g[o];
                                    }
            }
        }
        gin[idx] = acc;
    }
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
    morph_grad_kernel<<<grid_for(p.batch * p.numel_item), kGradThreads, 0, s>>>(gout, arg, gin, p, taps);
    TM_LAUNCH_CHECK("morph_grad_kernel");
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
