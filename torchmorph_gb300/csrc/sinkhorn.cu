// Sinkhorn iterations for GB300 (sm_103a): the plain FP32 path.
//
// Replaces sinkhorn_fastiter / sinkhorn_logiter
// (torchmorph/csrc/ot_kernel.cu:188-283) with the same arithmetic contract:
//   scaling form  out[b,i] = num[b,i] / (sum_j mat[i,j] * scale[b,j] + 1e-12)
//   log form      out[b,i] = lognum[b,i] - LSE_j(-cost[i,j]/eps + logscale[b,j])
// where the u-update passes (a, K|M, v) and the v-update (b, K^T|M^T, u).
// One CTA owns one matrix row and a tile of kBatchTile histograms, so each
// matrix row is streamed once per tile with 128-bit loads; the log form
// keeps an online (max, scaled sum) pair per histogram and merges the
// pairs with warp shuffles.  expf / logf are the correctly-rounded-ish
// library functions (no fast-math).
#include <cmath>

#include "tm_common.cuh"

namespace tmc {
namespace {

constexpr int kOtThreads = 256;
constexpr int kBatchTile = 8;

__device__ __forceinline__ void lse_merge(float &m, float &s, float mo, float so) {
    const float hi = fmaxf(m, mo);
    if (hi == -INFINITY) {
        m = -INFINITY;
        s = 0.0f;
        return;
    }
    s = (m == -INFINITY ? 0.0f : s * expf(m - hi)) + (mo == -INFINITY ? 0.0f : so * expf(mo - hi));
    m = hi;
}

template <int TB>
__global__ void __launch_bounds__(kOtThreads) ot_scaling_update(const float *__restrict__ num,
                                                                const float *__restrict__ mat,
                                                                const float *__restrict__ scale,
                                                                float *__restrict__ out, int d, int n) {
    const int row = blockIdx.x;
    const int b0 = blockIdx.y * TB;
    const int tb = min(TB, n - b0);
    const float *mrow = mat + (size_t)row * d;
    float acc[TB];
#pragma unroll
    for (int t = 0; t < TB; t++) acc[t] = 0.0f;
    const bool vec = (d % 4) == 0;
    if (vec) {
        const float4 *m4 = reinterpret_cast<const float4 *>(mrow);
        for (int j4 = threadIdx.x; j4 < d / 4; j4 += blockDim.x) {
            const float4 k = m4[j4];
#pragma unroll
            for (int t = 0; t < TB; t++) {
                if (t < tb) {
                    const float4 sc = reinterpret_cast<const float4 *>(scale + (size_t)(b0 + t) * d)[j4];
                    acc[t] = fmaf(k.x, sc.x, acc[t]);
                    acc[t] = fmaf(k.y, sc.y, acc[t]);
                    acc[t] = fmaf(k.z, sc.z, acc[t]);
                    acc[t] = fmaf(k.w, sc.w, acc[t]);
                }
            }
        }
    } else {
        for (int j = threadIdx.x; j < d; j += blockDim.x) {
            const float k = mrow[j];
#pragma unroll
            for (int t = 0; t < TB; t++)
                if (t < tb) acc[t] = fmaf(k, scale[(size_t)(b0 + t) * d + j], acc[t]);
        }
    }
    __shared__ float part[kOtThreads / 32][TB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < TB; t++) {
        float v = acc[t];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) part[warp][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < tb) {
        float tot = 0.0f;
        for (int w = 0; w < kOtThreads / 32; w++) tot += part[w][threadIdx.x];
        const size_t idx = (size_t)(b0 + threadIdx.x) * d + row;
        out[idx] = num[idx] / (tot + 1e-12f);
    }
}

template <int TB>
__global__ void __launch_bounds__(kOtThreads) ot_log_update(const float *__restrict__ lognum,
                                                            const float *__restrict__ cost,
                                                            const float *__restrict__ logscale,
                                                            float *__restrict__ out, int d, int n,
                                                            float inv_eps) {
    const int row = blockIdx.x;
    const int b0 = blockIdx.y * TB;
    const int tb = min(TB, n - b0);
    const float *crow = cost + (size_t)row * d;
    float m[TB], s[TB];
#pragma unroll
    for (int t = 0; t < TB; t++) {
        m[t] = -INFINITY;
        s[t] = 0.0f;
    }
    for (int j = threadIdx.x; j < d; j += blockDim.x) {
        const float c = -crow[j] * inv_eps;
#pragma unroll
        for (int t = 0; t < TB; t++) {
            if (t < tb) {
                const float z = c + logscale[(size_t)(b0 + t) * d + j];
                if (z > m[t]) {
                    s[t] = s[t] * expf(m[t] - z) + 1.0f;
                    m[t] = z;
                } else if (m[t] != -INFINITY) {
                    s[t] += expf(z - m[t]);
                }
            }
        }
    }
    __shared__ float pm[kOtThreads / 32][TB], ps[kOtThreads / 32][TB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < TB; t++) {
        float mm = m[t], ss = s[t];
        for (int o = 16; o > 0; o >>= 1) {
            const float mo = __shfl_down_sync(0xffffffffu, mm, o);
            const float so = __shfl_down_sync(0xffffffffu, ss, o);
            lse_merge(mm, ss, mo, so);
        }
        if (lane == 0) {
            pm[warp][t] = mm;
            ps[warp][t] = ss;
        }
    }
    __syncthreads();
    if (threadIdx.x < tb) {
        float mm = -INFINITY, ss = 0.0f;
        for (int w = 0; w < kOtThreads / 32; w++) lse_merge(mm, ss, pm[w][threadIdx.x], ps[w][threadIdx.x]);
        const size_t idx = (size_t)(b0 + threadIdx.x) * d + row;
        out[idx] = mm == -INFINITY ? -INFINITY : lognum[idx] - mm - logf(ss);
    }
}

int check_ot(const void *p, const char *name) {
    if (!p) return fail(TM_ERR_INVALID_ARGUMENT, "%s is NULL", name);
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" int tm_sinkhorn_fastiter(const float *a, const float *b, const float *K, const float *K_T, float *u,
                                    float *v, int64_t n, int64_t d, int64_t n_iter, tm_stream_t stream) {
    using namespace tmc;
    const void *ptrs[] = {a, b, K, K_T, u, v};
    const char *names[] = {"a", "b", "K", "K_T", "u", "v"};
    for (int i = 0; i < 6; i++)
        if (check_ot(ptrs[i], names[i]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    if (n < 1 || d < 1 || d > (1 << 30) || n > (1 << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "bad (n, d)");
    if (n_iter < 0) return fail(TM_ERR_INVALID_ARGUMENT, "n_iter must be >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 grid((unsigned)d, (unsigned)ceil_div(n, kBatchTile));
    for (int64_t it = 0; it < n_iter; it++) {
        ot_scaling_update<kBatchTile><<<grid, kOtThreads, 0, s>>>(a, K, v, u, (int)d, (int)n);
        ot_scaling_update<kBatchTile><<<grid, kOtThreads, 0, s>>>(b, K_T, u, v, (int)d, (int)n);
    }
    TM_LAUNCH_CHECK("ot_scaling_update");
    return TM_OK;
}

extern "C" int tm_sinkhorn_logiter(const float *log_a, const float *log_b, const float *M, const float *M_T,
                                   float *log_u, float *log_v, int64_t n, int64_t d, int64_t n_iter, double epsilon,
                                   tm_stream_t stream) {
    using namespace tmc;
    const void *ptrs[] = {log_a, log_b, M, M_T, log_u, log_v};
    const char *names[] = {"log_a", "log_b", "M", "M_T", "log_u", "log_v"};
    for (int i = 0; i < 6; i++)
        if (check_ot(ptrs[i], names[i]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive, got %g", epsilon);
    if (n < 1 || d < 1 || d > (1 << 30) || n > (1 << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "bad (n, d)");
    if (n_iter < 0) return fail(TM_ERR_INVALID_ARGUMENT, "n_iter must be >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    const float inv_eps = (float)(1.0 / epsilon);
    const dim3 grid((unsigned)d, (unsigned)ceil_div(n, kBatchTile));
    for (int64_t it = 0; it < n_iter; it++) {
        ot_log_update<kBatchTile><<<grid, kOtThreads, 0, s>>>(log_a, M, log_v, log_u, (int)d, (int)n, inv_eps);
        ot_log_update<kBatchTile><<<grid, kOtThreads, 0, s>>>(log_b, M_T, log_u, log_v, (int)d, (int)n, inv_eps);
    }
    TM_LAUNCH_CHECK("ot_log_update");
    return TM_OK;
}
