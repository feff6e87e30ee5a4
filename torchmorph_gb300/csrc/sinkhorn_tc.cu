// Shared-cost batched Sinkhorn on the tcgen05 tensor cores.
//
// n histogram pairs (a_h, b_h) of length d share one cost matrix C (d x d).
// The solver keeps the log-potentials log u, log v (n x d, fp32) and per
// half-iteration computes
//
//     log u_h = log a_h - m_h - log( K v'_h ),   v'_h = exp(log v_h - m_h),
//     m_h = max_j log v_{h,j}                                   (and the mirror
//                                                                 update of v)
//
// i.e. the scaling iteration of torchmorph/optimal_transport.py:71-93 with a
// per-histogram max shift, so v' lies in (0, 1] and neither K v' nor u
// overflows or underflows where the log-domain form
// (optimal_transport.py:96-125) would not.  K v' for all histograms at once is
// the product K (d x d) . V'^T (d x n): one call of the error-compensated BF16
// kernel of tc_gemm.cuh, with K = exp(-C/eps) split into bf16 hi + lo once per
// solve, V' split per half-iteration by ot_prep_kernel, and the log update
// done in the product's epilogue.  K^T is stored split as well, so the
// column update is the same kernel.
//
// FP64 is used only where the result is a sum over many terms: the L1 row
// marginal residual sum_i |a_i - u_i (K v)_i| (the stopping test) and the
// transport cost <P, C> = sum_i u_i ((K o C) v)_i, the latter as one more
// product with K o C split like K, so no plan is ever materialised.
//
// Padding: d and n are rounded up to multiples of 128 (the product's tile);
// padded rows of K and padded histograms are zero and their potentials
// -inf, so they contribute nothing and are never written back.
#include <cuda_bf16.h>

#include <cmath>

#include "tc_gemm.cuh"

namespace tmc {
namespace {

constexpr int64_t kTile = 128;

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

struct OtLayout {
    int64_t n, d, np, dp;
    size_t k[6];  // K hi/lo, K^T hi/lo, (K o C) hi/lo: bf16 dp x dp
    size_t u[2], v[2];  // scaled potentials hi/lo: bf16 np x dp
    size_t la, lb, ma, mb, lu, lv;  // fp32 np x dp
    size_t su, sv;  // fp32 np shifts
    size_t err, cost;  // fp64 np
    size_t total;
};

OtLayout ot_layout(int64_t n, int64_t d) {
    OtLayout L{};
    L.n = n;
    L.d = d;
    L.np = round_up(n, kTile);
    L.dp = round_up(d, kTile);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) / 256 * 256;
        return at;
    };
    const size_t kk = (size_t)L.dp * L.dp * 2, pb = (size_t)L.np * L.dp * 2, pf = (size_t)L.np * L.dp * 4;
    for (auto &o : L.k) o = take(kk);
    for (auto &o : L.u) o = take(pb);
    for (auto &o : L.v) o = take(pb);
    L.la = take(pf);
    L.lb = take(pf);
    L.ma = take(pf);
    L.mb = take(pf);
    L.lu = take(pf);
    L.lv = take(pf);
    L.su = take(L.np * 4);
    L.sv = take(L.np * 4);
    L.err = take(L.np * 8);
    L.cost = take(L.np * 8);
    L.total = off;
    return L;
}

template <typename T>
T *at(void *ws, size_t off) {
    return reinterpret_cast<T *>(static_cast<unsigned char *>(ws) + off);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

__device__ __forceinline__ uint32_t bits(__nv_bfloat162 v) {
    return (uint32_t)__bfloat16_as_ushort(__low2bfloat16(v)) | ((uint32_t)__bfloat16_as_ushort(__high2bfloat16(v)) << 16);
}

// K = exp(-C/eps), K o C and K^T, split into bf16 hi + lo, zero-padded to dp.
// 32 x 32 tiles; the transpose goes through shared memory.
__global__ void ot_build_kernel(const float *__restrict__ C, int64_t d, int64_t dp, float eps,
                                __nv_bfloat16 *kh, __nv_bfloat16 *kl, __nv_bfloat16 *kth, __nv_bfloat16 *ktl,
                                __nv_bfloat16 *kch, __nv_bfloat16 *kcl) {
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.y * 32, j0 = (int64_t)blockIdx.x * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r, j = j0 + tx;
        float k = 0.f, kc = 0.f;
        if (i < d && j < d) {
            const float c = C[i * d + j];
            k = expf(-(c / eps));
            kc = k * c;
        }
        const int64_t idx = i * dp + j;
        split_bf16(k, kh[idx], kl[idx]);
        split_bf16(kc, kch[idx], kcl[idx]);
        tile[r][tx] = k;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t j = j0 + r, i = i0 + tx;
        const int64_t idx = j * dp + i;
        split_bf16(tile[tx][r], kth[idx], ktl[idx]);
    }
}

// Padded marginals, their logs, and the initial potentials (0, the
// reference's log_u = log_v = 0; -inf on padding).
__global__ void ot_init_kernel(const float *__restrict__ a, const float *__restrict__ b, int64_t n, int64_t d,
                               int64_t dp, int64_t total, float *ma, float *mb, float *la, float *lb, float *lu,
                               float *lv) {
    const float ninf = -INFINITY;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t h = t / dp, i = t - h * dp;
        const bool valid = h < n && i < d;
        const float av = valid ? a[h * d + i] : 0.f, bv = valid ? b[h * d + i] : 0.f;
        ma[t] = av;
        mb[t] = bv;
        la[t] = logf(av);  // log 0 = -inf: the plan's row is zero
        lb[t] = logf(bv);
        lu[t] = valid ? 0.f : ninf;
        lv[t] = valid ? 0.f : ninf;
    }
}

// One histogram per block: shift m = max log p (0 when every entry is -inf),
// then p' = exp(log p - m) split into bf16 hi + lo.
constexpr int kPrepThreads = 256;

__global__ void __launch_bounds__(kPrepThreads) ot_prep_kernel(const float *__restrict__ logp, int64_t dp,
                                                               __nv_bfloat16 *hi, __nv_bfloat16 *lo,
                                                               float *shift) {
    __shared__ float red[kPrepThreads / 32];
    const int64_t h = blockIdx.x;
    const float4 *row = reinterpret_cast<const float4 *>(logp + h * dp);
    const int64_t nv = dp / 4;
    float m = -INFINITY;
    for (int64_t t = threadIdx.x; t < nv; t += kPrepThreads) {
        const float4 x = row[t];
        m = fmaxf(m, fmaxf(fmaxf(x.x, x.y), fmaxf(x.z, x.w)));
    }
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    m = red[0];
    for (int w = 1; w < kPrepThreads / 32; w++) m = fmaxf(m, red[w]);
    if (m == -INFINITY) m = 0.f;
    if (threadIdx.x == 0) shift[h] = m;
    uint2 *hrow = reinterpret_cast<uint2 *>(hi + h * dp);
    uint2 *lrow = reinterpret_cast<uint2 *>(lo + h * dp);
    for (int64_t t = threadIdx.x; t < nv; t += kPrepThreads) {
        const float4 x = row[t];
        const float e0 = expf(x.x - m), e1 = expf(x.y - m), e2 = expf(x.z - m), e3 = expf(x.w - m);
        const __nv_bfloat162 h01 = __floats2bfloat162_rn(e0, e1), h23 = __floats2bfloat162_rn(e2, e3);
        const float2 f01 = __bfloat1622float2(h01), f23 = __bfloat1622float2(h23);
        const __nv_bfloat162 l01 = __floats2bfloat162_rn(e0 - f01.x, e1 - f01.y);
        const __nv_bfloat162 l23 = __floats2bfloat162_rn(e2 - f23.x, e3 - f23.y);
        hrow[t] = make_uint2(bits(h01), bits(h23));
        lrow[t] = make_uint2(bits(l01), bits(l23));
    }
}

__device__ __forceinline__ double warp_sum(double x) {
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Pull the 32 rows x kBN histograms of `base` (row-major, `ld` floats per
// histogram) that a warp's epilogue reads towards L2: one 128-byte line per
// histogram, lane l takes histograms l, l+32, ...
__device__ __forceinline__ void prefetch_block(const float *base, int64_t ld, int row, int n0, int n, int d) {
    const int lane = threadIdx.x & 31;
    const int row0 = row - lane;
    if (row0 >= d) return;
    for (int c = lane; c < tc::kBN; c += 32)
        if (n0 + c < n) prefetch_l2(base + (int64_t)(n0 + c) * ld + row0);
}

// Epilogue of S = K v' (or K^T u'): for row i and histogram h,
//   err[h]    += |marg_{h,i} - exp(log_pot_{h,i} + shift_h) S|   (if err)
//   log_pot_{h,i} = log marg_{h,i} - shift_h - log S            (if update)
// The residual is evaluated in fp64 (exp of a potential near 20 in fp32
// would already be off by ~1e-6) and reduced over the warp's 32 rows before
// one atomic per histogram.
struct OtUpdateEpilogue {
    const float *log_marg, *marg, *shift;
    float *log_pot;
    double *err;
    int64_t ld;
    int n, d, update;
    __device__ __forceinline__ void prefetch(int row, int n0) const {
        prefetch_block(log_marg, ld, row, n0, n, d);
        if (err) {
            prefetch_block(marg, ld, row, n0, n, d);
            prefetch_block(log_pot, ld, row, n0, n, d);
        }
    }
    __device__ __forceinline__ void operator()(const float *tile, int row, int n0) const {
        const int lane = threadIdx.x & 31;
        const bool in_rows = row < d;
        const int cols = min(tc::kBN, n - n0);
        if (!err) {
            for (int c0 = 0; c0 < cols; c0 += 16) {
                float lm[16];
#pragma unroll
                for (int q = 0; q < 16; q++)
                    lm[q] = (in_rows && c0 + q < cols) ? log_marg[(int64_t)(n0 + c0 + q) * ld + row] : 0.f;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int c = c0 + q;
                    if (in_rows && c < cols)
                        log_pot[(int64_t)(n0 + c) * ld + row] =
                            lm[q] - shift[n0 + c] - logf(fmaxf(tile[c * 32 + lane], 1e-30f));
                }
            }
            return;
        }
#pragma unroll 2
        for (int c = 0; c < cols; c++) {
            const int h = n0 + c;
            const float S = tile[c * 32 + lane];
            const float sh = shift[h];
            double e = 0.0;
            if (in_rows) {
                const int64_t idx = (int64_t)h * ld + row;
                e = fabs((double)marg[idx] - exp((double)log_pot[idx] + (double)sh) * (double)S);
                if (update) log_pot[idx] = log_marg[idx] - sh - logf(fmaxf(S, 1e-30f));
            }
            e = warp_sum(e);
            if (lane == 0) atomicAdd(&err[h], e);
        }
    }
};

// Epilogue of D = (K o C) v': cost[h] += sum_i exp(log u_{h,i} + shift_h) D,
// each term in fp32 (its ~1e-6 relative error averages out over the sum),
// the sum in fp64.
struct OtCostEpilogue {
    const float *log_u, *shift;
    double *cost;
    int64_t ld;
    int n, d;
    __device__ __forceinline__ void prefetch(int row, int n0) const { prefetch_block(log_u, ld, row, n0, n, d); }
    __device__ __forceinline__ void operator()(const float *tile, int row, int n0) const {
        const int lane = threadIdx.x & 31;
        const bool in_rows = row < d;
        const int cols = min(tc::kBN, n - n0);
#pragma unroll 4
        for (int c = 0; c < cols; c++) {
            const int h = n0 + c;
            double t = 0.0;
            if (in_rows) t = (double)(expf(log_u[(int64_t)h * ld + row] + shift[h]) * tile[c * 32 + lane]);
            t = warp_sum(t);
            if (lane == 0) atomicAdd(&cost[h], t);
        }
    }
};

int check_ws(const OtLayout &L, void *ws, size_t bytes) {
    if (!ws || bytes < L.total)
        return fail(TM_ERR_WORKSPACE, "Sinkhorn workspace of %zu bytes needed, %zu given", L.total, bytes);
    if ((uintptr_t)ws & 255) return fail(TM_ERR_INVALID_ARGUMENT, "Sinkhorn workspace must be 256-byte aligned");
    return TM_OK;
}

int check_sizes(int64_t n, int64_t d) {
    if (n <= 0 || d <= 0) return fail(TM_ERR_INVALID_ARGUMENT, "n and d must be positive");
    if (n > (1 << 24) || d > (1 << 20)) return fail(TM_ERR_TOO_LARGE, "n or d too large");
    return TM_OK;
}

constexpr int kStages = 3;

int prep(const OtLayout &L, const float *logp, __nv_bfloat16 *hi, __nv_bfloat16 *lo, float *shift,
         cudaStream_t s) {
    ot_prep_kernel<<<(unsigned)L.np, kPrepThreads, 0, s>>>(logp, L.dp, hi, lo, shift);
    TM_LAUNCH_CHECK("ot_prep_kernel");
    return TM_OK;
}

// Row update (K, v -> u) or column update (K^T, u -> v).
int half_step(const OtLayout &L, void *ws, bool rows, double *err, bool update, cudaStream_t s) {
    using bf = __nv_bfloat16;
    const float *src_pot = at<float>(ws, rows ? L.lv : L.lu);
    bf *sh = at<bf>(ws, rows ? L.v[0] : L.u[0]), *sl = at<bf>(ws, rows ? L.v[1] : L.u[1]);
    float *shift = at<float>(ws, rows ? L.sv : L.su);
    int st = prep(L, src_pot, sh, sl, shift, s);
    if (st != TM_OK) return st;
    OtUpdateEpilogue epi{at<float>(ws, rows ? L.la : L.lb), at<float>(ws, rows ? L.ma : L.mb), shift,
                         at<float>(ws, rows ? L.lu : L.lv), err, L.dp, (int)L.n, (int)L.d, update ? 1 : 0};
    const bf *kh = at<bf>(ws, L.k[rows ? 0 : 2]), *kl = at<bf>(ws, L.k[rows ? 1 : 3]);
    return tc::launch_gemm3<kStages>(kh, kl, sh, sl, L.dp, L.np, L.dp, epi, s);
}

}  // namespace
}  // namespace tmc

extern "C" size_t tm_sinkhorn_tc_workspace_size(int64_t n, int64_t d) {
    if (n <= 0 || d <= 0) return 0;
    return tmc::ot_layout(n, d).total;
}

extern "C" int tm_sinkhorn_tc_init(const float *a, const float *b, const float *C, int64_t n, int64_t d,
                                   double epsilon, void *workspace, size_t workspace_bytes, tm_stream_t stream) {
    using namespace tmc;
    int st = check_sizes(n, d);
    if (st != TM_OK) return st;
    if (!a || !b || !C) return fail(TM_ERR_INVALID_ARGUMENT, "NULL a, b or cost");
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive");
    const OtLayout L = ot_layout(n, d);
    if ((st = check_ws(L, workspace, workspace_bytes)) != TM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    using bf = __nv_bfloat16;
    dim3 grid((unsigned)(L.dp / 32), (unsigned)(L.dp / 32));
    ot_build_kernel<<<grid, dim3(32, 8), 0, s>>>(C, d, L.dp, (float)epsilon, at<bf>(workspace, L.k[0]),
                                                 at<bf>(workspace, L.k[1]), at<bf>(workspace, L.k[2]),
                                                 at<bf>(workspace, L.k[3]), at<bf>(workspace, L.k[4]),
                                                 at<bf>(workspace, L.k[5]));
    TM_LAUNCH_CHECK("ot_build_kernel");
    const int64_t total = L.np * L.dp;
    const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
    ot_init_kernel<<<blocks, 256, 0, s>>>(a, b, n, d, L.dp, total, at<float>(workspace, L.ma),
                                          at<float>(workspace, L.mb), at<float>(workspace, L.la),
                                          at<float>(workspace, L.lb), at<float>(workspace, L.lu),
                                          at<float>(workspace, L.lv));
    TM_LAUNCH_CHECK("ot_init_kernel");
    return TM_OK;
}

extern "C" int tm_sinkhorn_tc_iterate(int64_t n, int64_t d, int64_t n_iter, double *row_err, void *workspace,
                                      size_t workspace_bytes, tm_stream_t stream) {
    using namespace tmc;
    int st = check_sizes(n, d);
    if (st != TM_OK) return st;
    if (n_iter < 0) return fail(TM_ERR_INVALID_ARGUMENT, "n_iter must be non-negative");
    const OtLayout L = ot_layout(n, d);
    if ((st = check_ws(L, workspace, workspace_bytes)) != TM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *err = at<double>(workspace, L.err);
    for (int64_t it = 0; it < n_iter; it++) {
        const bool check = row_err && it == n_iter - 1;
        if (check) TM_CHECK_CUDA(cudaMemsetAsync(err, 0, L.np * sizeof(double), s));
        if ((st = half_step(L, workspace, true, check ? err : nullptr, true, s)) != TM_OK) return st;
        if ((st = half_step(L, workspace, false, nullptr, true, s)) != TM_OK) return st;
    }
    if (row_err) {
        if (n_iter == 0) TM_CHECK_CUDA(cudaMemsetAsync(row_err, 0, n * sizeof(double), s));
        else TM_CHECK_CUDA(cudaMemcpyAsync(row_err, err, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    return TM_OK;
}

extern "C" int tm_sinkhorn_tc_finish(int64_t n, int64_t d, float *log_u, float *log_v, double *cost,
                                     double *row_err, void *workspace, size_t workspace_bytes, tm_stream_t stream) {
    using namespace tmc;
    using bf = __nv_bfloat16;
    int st = check_sizes(n, d);
    if (st != TM_OK) return st;
    const OtLayout L = ot_layout(n, d);
    if ((st = check_ws(L, workspace, workspace_bytes)) != TM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (row_err) {
        double *err = at<double>(workspace, L.err);
        TM_CHECK_CUDA(cudaMemsetAsync(err, 0, L.np * sizeof(double), s));
        if ((st = half_step(L, workspace, true, err, false, s)) != TM_OK) return st;
        TM_CHECK_CUDA(cudaMemcpyAsync(row_err, err, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    if (cost) {
        bf *vh = at<bf>(workspace, L.v[0]), *vl = at<bf>(workspace, L.v[1]);
        float *sv = at<float>(workspace, L.sv);
        if (!row_err && (st = prep(L, at<float>(workspace, L.lv), vh, vl, sv, s)) != TM_OK) return st;
        double *acc = at<double>(workspace, L.cost);
        TM_CHECK_CUDA(cudaMemsetAsync(acc, 0, L.np * sizeof(double), s));
        OtCostEpilogue epi{at<float>(workspace, L.lu), sv, acc, L.dp, (int)L.n, (int)L.d};
        st = tc::launch_gemm3<kStages>(at<bf>(workspace, L.k[4]), at<bf>(workspace, L.k[5]), vh, vl, L.dp, L.np,
                                       L.dp, epi, s);
        if (st != TM_OK) return st;
        TM_CHECK_CUDA(cudaMemcpyAsync(cost, acc, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    const size_t pitch = (size_t)L.dp * 4, width = (size_t)d * 4;
    if (log_u)
        TM_CHECK_CUDA(cudaMemcpy2DAsync(log_u, width, at<float>(workspace, L.lu), pitch, width, n,
                                        cudaMemcpyDeviceToDevice, s));
    if (log_v)
        TM_CHECK_CUDA(cudaMemcpy2DAsync(log_v, width, at<float>(workspace, L.lv), pitch, width, n,
                                        cudaMemcpyDeviceToDevice, s));
    return TM_OK;
}
