// Brute-force distance transform for GB300 (sm_103a).
//
// Replaces the reference's bfdt_cuda (torchmorph/csrc/bfdt_kernel.cu:154-297),
// which loops over the batch on the host with two torch::nonzero syncs per
// item.  Here the whole batch runs in two launches with no host sync:
//   bf_compact_kernel  -- each item's background voxels are appended to a
//                         per-item list (one atomic counter per item);
//   bf_search_kernel   -- one thread per voxel; background coordinates are
//                         staged through shared memory in tiles and every
//                         foreground voxel keeps its nearest background.
// The list order is irrelevant: ties go to the largest flat index, i.e.
// the last nearest background in raster order -- scipy.ndimage's
// distance_transform_bf rule.  Unit spacing is exact in integers; with
// sampling the metric is evaluated in float32 as in the reference.
// Items without background get +inf (euclidean) or 2^32-1 (other metrics)
// and zero indices (reference bfdt_kernel.cu:208-221).
#include <cmath>
#include <cstring>

#include "tm_common.cuh"

namespace tmc {
namespace {

constexpr int kBfThreads = 256;
constexpr int kBfTile = 512;

struct BfParams {
    int ndim;
    int metric;
    int sampled;
    int64_t batch;
    int64_t numel_item;
    FastDiv div[TM_MAX_NDIM];
    float sampling[TM_MAX_NDIM];
};

template <typename In>
__global__ void bf_compact_kernel(const In *__restrict__ in, int32_t *__restrict__ list, int *__restrict__ count,
                                  BfParams p) {
    const int64_t total = p.batch * p.numel_item;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = i / p.numel_item;
        const int32_t v = (int32_t)(i - item * p.numel_item);
        if (in[i] == (In)0) {
            int pos = atomicAdd(&count[item], 1);
            list[item * p.numel_item + pos] = v;
        }
    }
}

__device__ __forceinline__ void unravel(uint32_t f, const BfParams &p, int *c) {
#pragma unroll
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        if (d < p.ndim) {
            uint32_t q = fdiv(f, p.div[d]);
            f -= q * p.div[d].d;
            c[d] = (int)q;
        }
    }
}

template <typename In>
__global__ void __launch_bounds__(kBfThreads) bf_search_kernel(const In *__restrict__ in,
                                                               const int32_t *__restrict__ list,
                                                               const int *__restrict__ count,
                                                               float *__restrict__ dist,
                                                               int32_t *__restrict__ indices, BfParams p) {
    __shared__ int32_t tile_flat[kBfTile];
    __shared__ int16_t tile_c[kBfTile * TM_MAX_NDIM];
    const int64_t item = blockIdx.y;
    const int64_t numel = p.batch * p.numel_item;
    const int nbg = count[item];
    const int nd = p.ndim;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < p.numel_item;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = base + threadIdx.x;
        const bool active = v < p.numel_item;
        const int64_t gi = item * p.numel_item + v;
        const bool fg = active && in[gi] != (In)0;
        int xc[TM_MAX_NDIM];
        if (active) unravel((uint32_t)v, p, xc);
        long long best_i = 0x7fffffffffffffffLL;  // exact metric (unit spacing)
        float best_f = INFINITY;                   // sampled metric
        int32_t best = -1;
        const bool any_fg = __syncthreads_or(fg);
        if (any_fg && nbg > 0) {
            for (int t0 = 0; t0 < nbg; t0 += kBfTile) {
                const int tn = min(kBfTile, nbg - t0);
                __syncthreads();
                for (int k = threadIdx.x; k < tn; k += blockDim.x) {
                    const int32_t f = list[item * p.numel_item + t0 + k];
                    tile_flat[k] = f;
                    int c[TM_MAX_NDIM];
                    unravel((uint32_t)f, p, c);
                    for (int d = 0; d < nd; d++) tile_c[k * TM_MAX_NDIM + d] = (int16_t)c[d];
                }
                __syncthreads();
                if (fg) {
                    for (int k = 0; k < tn; k++) {
                        const int32_t f = tile_flat[k];
                        if (!p.sampled) {
                            long long m = 0;
                            for (int d = 0; d < nd; d++) {
                                int dd = xc[d] - tile_c[k * TM_MAX_NDIM + d];
                                if (p.metric == TM_BF_EUCLIDEAN)
                                    m += (long long)dd * dd;
                                else if (p.metric == TM_BF_TAXICAB)
                                    m += dd < 0 ? -dd : dd;
                                else
                                    m = max(m, (long long)(dd < 0 ? -dd : dd));
                            }
                            if (m < best_i || (m == best_i && f > best)) {
                                best_i = m;
                                best = f;
                            }
                        } else {
                            float m = 0.0f;
                            for (int d = 0; d < nd; d++) {
                                float dd = (float)(xc[d] - tile_c[k * TM_MAX_NDIM + d]) * p.sampling[d];
                                if (p.metric == TM_BF_EUCLIDEAN)
                                    m = fmaf(dd, dd, m);
                                else if (p.metric == TM_BF_TAXICAB)
                                    m += fabsf(dd);
                                else
                                    m = fmaxf(m, fabsf(dd));
                            }
                            if (m < best_f || (m == best_f && f > best)) {
                                best_f = m;
                                best = f;
                            }
                        }
                    }
                }
            }
        }
        if (!active) continue;
        float dval;
        int bc[TM_MAX_NDIM];
        if (!fg) {
            dval = 0.0f;
            for (int d = 0; d < nd; d++) bc[d] = xc[d];
        } else if (nbg == 0) {
            dval = p.metric == TM_BF_EUCLIDEAN ? INFINITY : 4294967296.0f;
            for (int d = 0; d < nd; d++) bc[d] = 0;
        } else {
            unravel((uint32_t)best, p, bc);
            if (!p.sampled) {
                if (p.metric == TM_BF_EUCLIDEAN)
                    dval = best_i < (1LL << 24) ? __fsqrt_rn((float)best_i) : (float)sqrt((double)best_i);
                else
                    dval = (float)best_i;
            } else {
                dval = p.metric == TM_BF_EUCLIDEAN ? __fsqrt_rn(best_f) : best_f;
            }
        }
        if (dist) dist[gi] = dval;
        if (indices)
            for (int d = 0; d < nd; d++) indices[(int64_t)d * numel + gi] = bc[d];
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

template <typename In>
int run_bf(const In *in, const Geometry &g, int metric, const float *sampling, float *dist, int32_t *indices,
           unsigned char *ws, cudaStream_t stream) {
    BfParams p;
    std::memset(&p, 0, sizeof(p));
    p.ndim = g.ndim;
    p.metric = metric;
    p.batch = g.batch;
    p.numel_item = g.numel_item;
    p.sampled = 0;
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        p.div[d] = make_fastdiv(d < g.ndim ? (uint32_t)g.stride[d] : 1u);
        p.sampling[d] = (sampling && d < g.ndim) ? sampling[d] : 1.0f;
        if (d < g.ndim && p.sampling[d] != 1.0f) p.sampled = 1;
    }
    int *count = reinterpret_cast<int *>(ws);
    int32_t *list = reinterpret_cast<int32_t *>(ws + align256((size_t)g.batch * 4));
    TM_CHECK_CUDA(cudaMemsetAsync(count, 0, (size_t)g.batch * 4, stream));
    const int sms = sm_count();
    unsigned cb = (unsigned)std::min<int64_t>(ceil_div(g.numel, 256), (int64_t)sms * 16);
    bf_compact_kernel<In><<<cb, 256, 0, stream>>>(in, list, count, p);
    TM_LAUNCH_CHECK("bf_compact_kernel");
    for (int64_t b0 = 0; b0 < g.batch; b0 += 65535) {
        // items are addressed through blockIdx.y; every pointer is shifted by
        // the chunk start, index planes keep their stride of batch * numel_item
        const int64_t nb = std::min<int64_t>(65535, g.batch - b0);
        BfParams q = p;
        dim3 grid((unsigned)std::min<int64_t>(ceil_div(g.numel_item, kBfThreads), (int64_t)sms * 8), (unsigned)nb);
        bf_search_kernel<In><<<grid, kBfThreads, 0, stream>>>(
            in + b0 * g.numel_item, list + b0 * g.numel_item, count + b0, dist ? dist + b0 * g.numel_item : nullptr,
            indices ? indices + b0 * g.numel_item : nullptr, q);
        TM_LAUNCH_CHECK("bf_search_kernel");
    }
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" size_t tm_bfdt_workspace_size(int64_t batch, int ndim, const int64_t *shape) {
    tmc::Geometry g;
    if (tmc::make_geometry(batch, ndim, shape, &g) != TM_OK) return 0;
    return tmc::align256((size_t)batch * 4) + tmc::align256((size_t)g.numel * 4);
}

extern "C" int tm_bfdt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape, int metric,
                       const float *sampling, float *dist, int32_t *indices, void *workspace, size_t workspace_bytes,
                       tm_stream_t stream) {
    using namespace tmc;
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (!input) return fail(TM_ERR_INVALID_ARGUMENT, "input is NULL");
    if (in_dtype != TM_F32 && in_dtype != TM_U8) return fail(TM_ERR_INVALID_ARGUMENT, "unknown input dtype %d", in_dtype);
    if (metric < 0 || metric > 2)
        return fail(TM_ERR_INVALID_ARGUMENT, "Unsupported metric type. Use 'euclidean', 'taxicab', or 'chessboard'.");
    if (!dist && !indices) return fail(TM_ERR_INVALID_ARGUMENT, "at least one output must be requested");
    for (int d = 0; d < ndim; d++)
        if (shape[d] > 32767) return fail(TM_ERR_TOO_LARGE, "brute-force DT supports spatial sizes up to 32767");
    if (sampling)
        for (int d = 0; d < ndim; d++)
            if (!(std::isfinite(sampling[d]) && sampling[d] > 0.0f))
                return fail(TM_ERR_INVALID_ARGUMENT, "sampling values must be finite and greater than zero");
    if (g.numel_item >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels are not supported");
    size_t need = tm_bfdt_workspace_size(batch, ndim, shape);
    if (!workspace || workspace_bytes < need)
        return fail(TM_ERR_WORKSPACE, "workspace of %zu bytes required, got %zu", need, workspace_bytes);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    cudaStream_t s = (cudaStream_t)stream;
    if (in_dtype == TM_F32) return run_bf<float>((const float *)input, g, metric, sampling, dist, indices, ws, s);
    return run_bf<uint8_t>((const uint8_t *)input, g, metric, sampling, dist, indices, ws, s);
}
