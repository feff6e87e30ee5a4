// Chamfer distance transforms for GB300 (sm_103a).
//
// Replaces the reference's cdt_cuda (torchmorph/csrc/cdt_kernel.cu:269-463).
// The reference approximates the chessboard metric with racy diagonal
// relaxations; this file computes the exact two-pass raster chamfer of
// scipy.ndimage.distance_transform_cdt (the reference's test oracle): a
// forward pass in raster order over the causal half of the 3^n
// neighbourhood (offsets in raster order, strict '<', so the first offset
// wins a tie), then the same pass over the flipped array.  The weighted
// 3-4-5 chamfer (face 3, edge 4, corner 5; not in the reference) uses the
// same two passes.
//
// Parallel schedule.  Split each item into rows along the last axis.  A row
// r = (r_0..r_{n-2}) depends only on rows r + o' with o' causal, and
// tau(r) = sum_d r_d * 2^(n-2-d) strictly decreases along every causal o',
// so all rows with the same tau (a wavefront) are independent.  One CTA per
// item walks the wavefronts; each warp owns a row.  Inside a row the only
// serial dependency is the chain x-1 -> x, which unrolls to
//     dt(x) = min_k V(k) + w (x - k),  ties to the largest k,
// where V(k) is the best candidate from every other offset -- a prefix
// minimum of V(k) - w k, evaluated as a warp-shuffle scan.  The result is
// therefore bit-identical to the sequential raster pass.
#include <algorithm>
#include <cstring>
#include <vector>

#include "edt_internal.cuh"
#include "tm_common.cuh"
#include "tm_tma.cuh"

namespace tmc {
namespace {

constexpr int kCdtThreads = 1024;
constexpr int kMaxCdtOffsets = 3280;  // causal half of the 8-D 3^n neighbourhood
constexpr int64_t kKeyInf = 0x7fffffffffffffffLL;

struct CdtParams {
    int ndim;
    int W;                // last-axis length
    int rows;             // rows per item
    int T;                // wavefronts
    int noff;             // offsets (without the chain offset)
    int wchain;           // chain weight
    int64_t batch;
    int64_t numel_item;
    int shape[TM_MAX_NDIM];
    int64_t stride[TM_MAX_NDIM];
    FastDiv row_div[TM_MAX_NDIM];  // strides of the row index space (dims 0..n-2)
};

struct CdtOffsets {
    int32_t flat[kMaxCdtOffsets];
    int16_t code[kMaxCdtOffsets];  // base-3 digits of (o_d + 1), dim 0 most significant
    uint8_t weight[kMaxCdtOffsets];
};

__device__ __forceinline__ int tau_of_row(uint32_t r, const CdtParams &p) {
    int tau = 0;
    for (int d = 0; d < p.ndim - 1; d++) {
        uint32_t q = fdiv(r, p.row_div[d]);
        r -= q * p.row_div[d].d;
        tau += (int)q << (p.ndim - 2 - d);
    }
    return tau;
}

__device__ void cdt_count(int *__restrict__ cnt, const CdtParams &p) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < p.rows; r += gridDim.x * blockDim.x)
        atomicAdd(&cnt[tau_of_row((uint32_t)r, p)], 1);
}

// Exclusive scan of T counters (one CTA); off[T] = total.
__device__ void cdt_scan(const int *__restrict__ cnt, int *__restrict__ off, int T) {
    __shared__ int carry;
    __shared__ int warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < T; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < T ? __ldcg(cnt + i) : 0;
        int x = v;
        for (int s = 1; s < 32; s <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, s);
            if (lane >= s) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
            for (int s = 1; s < 32; s <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, w, s);
                if (lane >= s) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        int incl = x + (warp > 0 ? warp_sums[warp - 1] : 0) + carry;
        if (i < T) off[i] = incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[T] = carry;
}

__device__ void cdt_scatter(const int *__restrict__ off, int *__restrict__ cursor, int *__restrict__ order,
                            const CdtParams &p) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < p.rows; r += gridDim.x * blockDim.x) {
        int t = tau_of_row((uint32_t)r, p);
        int pos = atomicAdd(&cursor[t], 1);
        order[__ldcg(off + t) + pos] = r;
    }
}

// todo (optional): 1 for the items the raster passes must compute; the
// others were finished by the bitmap shell search and are left alone.
template <typename In>
__device__ void cdt_init(const In *__restrict__ in, int32_t *__restrict__ dt, int32_t *__restrict__ ft,
                         int64_t numel, int64_t numel_item, const int *__restrict__ todo) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < numel;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (todo && !todo[i / numel_item]) continue;
        dt[i] = in[i] != (In)0 ? -1 : 0;
        ft[i] = (int32_t)(i % numel_item);
    }
}

// (key, feature) pair of the chain scan: smaller key wins; keys are unique
// per position so no further tie rule is needed.
struct ScanPair {
    long long key;
    int feat;
};

__device__ __forceinline__ ScanPair pmin(ScanPair a, ScanPair b) { return b.key < a.key ? b : a; }

template <bool BACKWARD>
__device__ void cdt_pass(int32_t *dt, int32_t *ft, const int *order, const int *woff, const CdtParams &p,
                         const CdtOffsets &offs, const int *__restrict__ todo) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int nd = p.ndim;
    const int sgn = BACKWARD ? -1 : 1;
    for (int64_t item = blockIdx.x; item < p.batch; item += gridDim.x) {
        if (todo && !todo[item]) continue;  // uniform per block
        int32_t *D = dt + item * p.numel_item;
        int32_t *F = ft + item * p.numel_item;
        for (int step = 0; step < p.T; step++) {
            const int t = BACKWARD ? p.T - 1 - step : step;
            const int r0 = __ldcg(woff + t), r1 = __ldcg(woff + t + 1);
            for (int ri = r0 + warp; ri < r1; ri += nwarps) {
                const int row = __ldcg(order + ri);
                // row coordinates (dims 0..n-2)
                int rc[TM_MAX_NDIM];
                uint32_t rem = (uint32_t)row;
                bool row_inner = true;
                for (int d = 0; d < nd - 1; d++) {
                    uint32_t q = fdiv(rem, p.row_div[d]);
                    rem -= q * p.row_div[d].d;
                    rc[d] = (int)q;
                    row_inner &= q >= 1 && (int)q <= p.shape[d] - 2;
                }
                const int64_t rbase = (int64_t)row * p.W;
                ScanPair carry{kKeyInf, 0};
                for (int c0 = 0; c0 < p.W; c0 += 32) {
                    const int j = c0 + lane;  // position along the scan direction
                    const bool valid = j < p.W;
                    const int x = BACKWARD ? p.W - 1 - j : j;
                    ScanPair mine{kKeyInf, 0};
                    if (valid) {
                        const int64_t e = rbase + x;
                        int best = __ldcg(D + e);
                        int64_t bi = -1;
                        if (best != 0) {
                            const bool inner = row_inner && x >= 1 && x <= p.W - 2;
                            for (int k = 0; k < p.noff; k++) {
                                int64_t nb;
                                if (inner) {
                                    nb = e + sgn * offs.flat[k];
                                } else {
                                    int code = offs.code[k];
                                    bool ok = true;
                                    nb = 0;
                                    for (int d = nd - 1; d >= 0; d--) {
                                        int o = (code % 3 - 1) * sgn;
                                        code /= 3;
                                        int c = (d == nd - 1 ? x : rc[d]) + o;
                                        if (c < 0 || c >= p.shape[d]) {
                                            ok = false;
                                            break;
                                        }
                                        nb += (int64_t)c * p.stride[d];
                                    }
                                    if (!ok) continue;
                                }
                                const int tv = __ldcg(D + nb);
                                if (tv < 0) continue;
                                const int cand = tv + offs.weight[k];
                                if (best < 0 || cand < best) {
                                    best = cand;
                                    bi = nb;
                                }
                            }
                        }
                        if (best >= 0) {
                            mine.key = (long long)(best - p.wchain * j) * 4294967296LL + (4294967295LL - j);
                            mine.feat = bi >= 0 ? __ldcg(F + bi) : __ldcg(F + e);
                        }
                    }
                    // inclusive warp min-scan over the chunk, then the carry
                    ScanPair acc = mine;
#pragma unroll
                    for (int s = 1; s < 32; s <<= 1) {
                        ScanPair o;
                        o.key = __shfl_up_sync(0xffffffffu, acc.key, s);
                        o.feat = __shfl_up_sync(0xffffffffu, acc.feat, s);
                        if (lane >= s) acc = pmin(o, acc);
                    }
                    acc = pmin(carry, acc);
                    carry.key = __shfl_sync(0xffffffffu, acc.key, 31);
                    carry.feat = __shfl_sync(0xffffffffu, acc.feat, 31);
                    if (valid) {
                        const int64_t e = rbase + x;
                        if (acc.key != kKeyInf) {
                            const long long v0 = acc.key >> 32;  // V(k*) - w k*
                            D[e] = (int)(v0 + (long long)p.wchain * j);
                            F[e] = acc.feat;
                        }
                    }
                }
            }
            __syncthreads();
        }
    }
}

__device__ void cdt_finalize(const int32_t *dt, const int32_t *ft, float *__restrict__ dist,
                             int32_t *__restrict__ indices, int64_t numel, int64_t numel_item, int ndim,
                             const CdtParams &p, float divisor, const int *__restrict__ todo) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < numel;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (todo && !todo[i / numel_item]) continue;
        const int v = __ldcg(dt + i);
        if (dist) dist[i] = v < 0 ? -1.0f : (float)v / divisor;
        if (indices) {
            int64_t f = __ldcg(ft + i);
            for (int d = 0; d < ndim; d++) {
                int64_t q = f / p.stride[d];
                f -= q * p.stride[d];
                indices[(int64_t)d * numel + i] = (int32_t)q;
            }
        }
    }
}

struct CdtRasterArgs {
    const void *in;
    int32_t *dt, *ft;
    int *order, *woff, *cnt, *cur;
    float *dist;
    int32_t *indices;
    int64_t numel;
    float divisor;
    const int *todo;  // per-item flags of the shell search (NULL: every item)
    const int *any;   // flag after them: some item is marked
    GridControl *ctl;
    int *status;
    long long spin_limit;
};

// The whole raster transform in ONE cooperative launch: wavefront counts,
// their scan, the row order and the initial costs, then for every item (one
// CTA per item) the forward and the backward pass, then the outputs -- with
// bounded grid barriers between the phases.  After the shell search, the
// launch returns at once unless some item was marked.
template <typename In>
__global__ void __launch_bounds__(kCdtThreads, 1) cdt_raster_kernel(CdtRasterArgs a, CdtParams p, CdtOffsets offs) {
    if (a.any && !*(volatile const int *)a.any) return;  // uniform: every CTA leaves
    cdt_count(a.cnt, p);
    if (!grid_barrier_bounded(a.ctl, gridDim.x, a.status, a.spin_limit)) return;
    if (blockIdx.x == 0) cdt_scan(a.cnt, a.woff, p.T);
    cdt_init(static_cast<const In *>(a.in), a.dt, a.ft, a.numel, p.numel_item, a.todo);
    if (!grid_barrier_bounded(a.ctl, gridDim.x, a.status, a.spin_limit)) return;
    cdt_scatter(a.woff, a.cur, a.order, p);
    if (!grid_barrier_bounded(a.ctl, gridDim.x, a.status, a.spin_limit)) return;
    // an item's two passes run on the same CTA: no grid barrier between them
    cdt_pass<false>(a.dt, a.ft, a.order, a.woff, p, offs, a.todo);
    cdt_pass<true>(a.dt, a.ft, a.order, a.woff, p, offs, a.todo);
    if (!grid_barrier_bounded(a.ctl, gridDim.x, a.status, a.spin_limit)) return;
    cdt_finalize(a.dt, a.ft, a.dist, a.indices, a.numel, p.numel_item, p.ndim, p, a.divisor, a.todo);
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct CdtPlan {
    int rows, T;
    size_t dt_off, ft_off, order_off, woff_off, cnt_off, cur_off, ctl_off, total;
};

CdtPlan plan_cdt(const Geometry &g) {
    CdtPlan pl;
    pl.rows = (int)(g.numel_item / g.shape[g.ndim - 1]);
    int64_t T = 1;
    for (int d = 0; d < g.ndim - 1; d++) T += (g.shape[d] - 1) << (g.ndim - 2 - d);
    pl.T = (int)T;
    size_t o = 0;
    pl.dt_off = o;
    o += align256((size_t)g.numel * 4);
    pl.ft_off = o;
    o += align256((size_t)g.numel * 4);
    pl.order_off = o;
    o += align256((size_t)pl.rows * 4);
    pl.woff_off = o;
    o += align256((size_t)(pl.T + 1) * 4);
    pl.cnt_off = o;
    o += align256((size_t)pl.T * 4);
    pl.cur_off = o;
    o += align256((size_t)pl.T * 4);
    pl.ctl_off = o;  // the raster launch's barrier block, right after the counters
    o += sizeof(GridControl);
    pl.total = o;
    return pl;
}

// Zero the wavefront counters and the barrier block of the raster launch
// (contiguous in the workspace: one memset).
cudaError_t clear_cdt_counters(unsigned char *ws, const CdtPlan &pl, cudaStream_t stream) {
    return cudaMemsetAsync(ws + pl.cnt_off, 0, pl.ctl_off + sizeof(GridControl) - pl.cnt_off, stream);
}

template <typename In>
int run_cdt(const In *in, const Geometry &g, int metric, float *dist, int32_t *indices, unsigned char *ws,
            const CdtPlan &pl, const int *todo, bool counters_cleared, cudaStream_t stream) {
    const int nd = g.ndim;
    CdtParams p;
    std::memset(&p, 0, sizeof(p));
    p.ndim = nd;
    p.W = (int)g.shape[nd - 1];
    p.rows = pl.rows;
    p.T = pl.T;
    p.batch = g.batch;
    p.numel_item = g.numel_item;
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        p.shape[d] = d < nd ? (int)g.shape[d] : 1;
        p.stride[d] = d < nd ? g.stride[d] : 0;
        p.row_div[d] = make_fastdiv(d < nd - 1 ? (uint32_t)(g.stride[d] / g.shape[nd - 1]) : 1u);
    }
    // causal offsets in raster order, without the chain offset (0,..,0,-1)
    CdtOffsets local;
    int total = 1;
    for (int d = 0; d < nd; d++) total *= 3;
    int n = 0;
    for (int jj = 0; jj < total / 2; jj++) {
        int rem = jj, nz = 0, o[TM_MAX_NDIM];
        for (int d = nd - 1; d >= 0; d--) {
            o[d] = rem % 3 - 1;
            rem /= 3;
            nz += o[d] != 0;
        }
        if (metric == TM_CDT_TAXICAB && nz != 1) continue;
        bool chain = nz == 1 && o[nd - 1] == -1;
        if (chain) continue;
        int64_t f = 0;
        for (int d = 0; d < nd; d++) f += (int64_t)o[d] * g.stride[d];
        local.flat[n] = (int32_t)f;
        local.code[n] = (int16_t)jj;
        local.weight[n] = (uint8_t)(metric == TM_CDT_CHAMFER345 ? (nz == 1 ? 3 : nz == 2 ? 4 : 5) : 1);
        n++;
    }
    p.noff = n;
    p.wchain = metric == TM_CDT_CHAMFER345 ? 3 : 1;
    CdtRasterArgs a;
    a.in = in;
    a.dt = reinterpret_cast<int32_t *>(ws + pl.dt_off);
    a.ft = reinterpret_cast<int32_t *>(ws + pl.ft_off);
    a.order = reinterpret_cast<int *>(ws + pl.order_off);
    a.woff = reinterpret_cast<int *>(ws + pl.woff_off);
    a.cnt = reinterpret_cast<int *>(ws + pl.cnt_off);
    a.cur = reinterpret_cast<int *>(ws + pl.cur_off);
    a.ctl = reinterpret_cast<GridControl *>(ws + pl.ctl_off);
    a.dist = dist;
    a.indices = indices;
    a.numel = g.numel;
    a.divisor = metric == TM_CDT_CHAMFER345 ? 3.0f : 1.0f;
    a.todo = todo;
    a.any = todo ? todo + g.batch : nullptr;  // the flag after the per-item flags
    int st = device_status_word(&a.status);
    if (st != TM_OK) return st;
    a.spin_limit = grid_wait_budget();
    if (!counters_cleared) TM_CHECK_CUDA(clear_cdt_counters(ws, pl, stream));
    static thread_local int cached_dev = -1, cached_per_sm = 0;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev != dev) {
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_per_sm, cdt_raster_kernel<In>,
                                                                    kCdtThreads, 0));
        cached_dev = dev;
    }
    if (cached_per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "raster chamfer kernel does not fit on an SM");
    const int64_t blocks = std::min<int64_t>((int64_t)cached_per_sm * sm_count(),
                                             std::max<int64_t>(g.batch, ceil_div(g.numel, kCdtThreads)));
    void *params[] = {&a, &p, &local};
    TM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void *)cdt_raster_kernel<In>, dim3((unsigned)blocks),
                                              dim3(kCdtThreads), params, 0, stream));
    TM_LAUNCH_CHECK("cdt_raster_kernel");
    return TM_OK;
}

}  // namespace
}  // namespace tmc

// Distances without indices of 3-D items with 128-wide rows first go
// through the bitmap shell search (edt_compact.cu); its workspace follows
// the raster passes' one.
static bool cdt_shell_shape(const tmc::Geometry &g) { return g.ndim == 3 && (g.shape[2] + 31) / 32 == 4 && g.shape[2] % 4 == 0; }

extern "C" size_t tm_cdt_workspace_size(int64_t batch, int ndim, const int64_t *shape) {
    tmc::Geometry g;
    if (tmc::make_geometry(batch, ndim, shape, &g) != TM_OK) return 0;
    size_t n = tmc::plan_cdt(g).total;
    if (cdt_shell_shape(g)) n += tmc::cdt_shell_workspace(g);
    return n;
}

extern "C" int tm_cdt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape, int metric,
                      float *dist, int32_t *indices, void *workspace, size_t workspace_bytes, tm_stream_t stream) {
    using namespace tmc;
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (!input) return fail(TM_ERR_INVALID_ARGUMENT, "input is NULL");
    if (in_dtype != TM_F32 && in_dtype != TM_U8) return fail(TM_ERR_INVALID_ARGUMENT, "unknown input dtype %d", in_dtype);
    if (metric < 0 || metric > 2) return fail(TM_ERR_INVALID_ARGUMENT, "metric must be 'chessboard' or 'taxicab'");
    if (metric == TM_CDT_CHAMFER345 && ndim > 3)
        return fail(TM_ERR_UNSUPPORTED, "the 3-4-5 chamfer is defined for 1 to 3 spatial dimensions");
    if (!dist && !indices)
        return fail(TM_ERR_INVALID_ARGUMENT, "At least one of return_distances or return_indices must be True");
    if (g.numel_item >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels are not supported");
    CdtPlan pl = plan_cdt(g);
    const size_t need = pl.total + (cdt_shell_shape(g) ? cdt_shell_workspace(g) : 0);
    if (!workspace || workspace_bytes < need)
        return fail(TM_ERR_WORKSPACE, "workspace of %zu bytes required, got %zu", need, workspace_bytes);
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    cudaStream_t s = (cudaStream_t)stream;
    int *todo = nullptr;
    bool cleared = false;
    // autotuned variants: 1 = the raster passes for every item (no shell search),
    // 2 = the shell search with one CTA per 32-row block instead of the warp queue
    const int variant = tune_variant(kTuneCdt3D, tune_class(kTuneCdt3D, g.numel, 0));
    const bool shell = variant != 1;
    if (shell && cdt_shell_shape(g) && cdt_shell_eligible(g, dist, indices)) {
        // counters first, so that nothing but kernels follows the shell search
        TM_CHECK_CUDA(clear_cdt_counters(ws, pl, s));
        cleared = true;
        st = cdt_shell_run(input, in_dtype, g, metric, dist, ws + pl.total, &todo, s, variant == 2);
        if (st != TM_OK) return st;
    }
    if (in_dtype == TM_F32)
        return run_cdt<float>((const float *)input, g, metric, dist, indices, ws, pl, todo, cleared, s);
    return run_cdt<uint8_t>((const uint8_t *)input, g, metric, dist, indices, ws, pl, todo, cleared, s);
}
