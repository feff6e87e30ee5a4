// FP32 Sinkhorn for batches of histogram pairs sharing one (d, d) matrix
// (GB300, sm_103a): the plain CUDA-core path next to the tensor-core solver.
//
// Every half-step of every pair is one contraction with the shared matrix:
//   scaling form  out[b,i] = num[b,i] / (sum_j K[i,j] s[b,j] + 1e-12)
//   log form      out[b,i] = num[b,i] - LSE_j(-M[i,j]/eps + s[b,j])
// (u-update: num = a | log a, matrix K | M, s = v | log v; v-update: b,
// K^T | M^T, u), the contract of the reference's fused iterations
// (torchmorph/csrc/ot_kernel.cu:188-283, torchmorph/optimal_transport.py:
// 71-125): u first, +1e-12 in the scaling denominators, -inf wherever every
// term of a log-sum-exp is -inf.
//
// Design.  Both forms are GEMM-shaped: the (d x d) matrix is shared by the n
// pairs, so a CTA owns a tile of 128 matrix rows x TB pairs and reuses every
// staged matrix entry for all TB pairs (the reference streams the matrix once
// per group of 8 pairs).  Matrix and scaling tiles are staged in shared
// memory 16 columns at a time (register prefetch of the next chunk, one
// barrier per chunk); each thread accumulates 8 rows x TB/16 pairs.  The log
// form works in base 2 (entries pre-scaled by log2(e) when staged) with a
// running maximum per output, rescaled only when a group of 4 terms raises it,
// so a term costs one add, one subtract and one ex2.
//
// The whole iteration loop is ONE cooperative persistent launch: all CTAs
// are co-resident and meet at bounded grid barriers between half-steps, so a
// solve of any length costs one launch (the reference enqueues two kernels
// per iteration and replays captured chunks of them).  With a threshold the
// u-update of every check_every-th iteration also sums the L1 row-marginal
// residual |a_i - u_i (K v)_i| of the plan that iteration started from (per
// 128-row block, in fixed order), the next phase reduces it per pair, and
// all CTAs stop together once every pair is at or below the threshold -- no
// host round trip.  A barrier wait that exceeds its poll budget records
// TM_DEV_ERR_TIMEOUT in the device status word and makes every CTA leave.
#include <cmath>

#include "tm_tma.cuh"

namespace tmc {
namespace {

constexpr int kSkThreads = 256;
constexpr int kSkRows = 128;       // matrix rows per tile
constexpr int kSkChunk = 16;       // contraction columns staged per step
constexpr int kSkPitch = kSkChunk + 4;  // padded row of a staged tile (floats)
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;
constexpr float kNoMax = -3.0e38f;  // running-maximum start (below every finite term)

__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Cost of the d points 0, 1, ..., d - 1 on a line, the reference's default
// cost (build_cost_matrix((d,), p) for p = 1 or 2): |i - j|, exact in float32.
// A NULL cost matrix selects it; entries are then computed where they are
// used and no (d, d) matrix is ever stored or read.
__device__ __forceinline__ float line_cost(int i, int j) { return (float)(i > j ? i - j : j - i); }

struct SkControl {
    unsigned barrier_count;
    unsigned barrier_gen;
    int abort;
    int iterations;  // iterations completed by the last launch
    int pad[60];
};
static_assert(sizeof(SkControl) == 256, "control block is 256 bytes");

struct SkArgs {
    const float *num_u, *num_v;  // a, b (scaling) or log a, log b (log form)
    const float *mat, *mat_t;    // K, K^T or M, M^T (row-major d x d)
    float *u, *v;                // scalings or log-scalings, updated in place
    int n, d;
    float mscale;                // log form: -log2(e) / eps applied to staged matrix entries
    float inv_eps;               // scaling form with the line cost: K = exp(-|i - j| * inv_eps)
    int max_iter, check_every;   // check_every = 0: no residual checks
    float threshold;
    double *partial;             // [row blocks][n] residual partial sums
    double *err;                 // [n] residual of the last check
    int *notconv;                // [checks] set when some pair is above the threshold
    SkControl *ctl;
    int *status;
    long long spin_limit;
    bool vec;                    // d % 4 == 0 and 16-byte aligned operands: float4 staging
};


struct SkStage {
    float mat[2][kSkRows * kSkPitch];
    float sc[2][64 * kSkPitch];
};

// One tile of one half-step: rows [i0, i0 + 128) of the matrix, pairs
// [b0, b0 + 16 * MB).  Thread layout: lane % 16 = row group tr (rows tr + 16 r,
// r < 8), lane / 16 + 2 * warp = pair group tb (pairs tb + 16 m, m < MB), so a
// staged matrix row is read by 16 lanes at 20-float pitch (two wavefronts) and
// a scaling row is broadcast to 16 lanes; outputs are written 16 consecutive
// rows at a time.
template <bool LOG, int MB>
__device__ void sk_tile(const SkArgs &A, SkStage &st, int i0, int b0, const float *__restrict__ num,
                        const float *__restrict__ mat, const float *scale, float *out, double *partial_row) {
    constexpr int TB = 16 * MB;
    const int n = A.n, d = A.d;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tr = lane & 15, tb = (lane >> 4) + 2 * warp;
    // entries beyond the matrix or the batch contribute nothing: a zero kernel
    // weight (scaling form), an infinite cost and a -inf log-scaling (log form;
    // the cost is scaled by the negative mscale when staged)
    const float fill = LOG ? INFINITY : 0.0f;
    const float sfill = LOG ? -INFINITY : 0.0f;
    const float mscale = A.mscale;

    // staging assignment: matrix tile 128 x 16 = 512 float4 (two per thread),
    // scaling tile TB x 16 = TB * 4 float4 (threads < TB * 4)
    float4 pm[2], ps;
    auto load = [&](int j0) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int f = tid + h * kSkThreads;
            const int row = f >> 2, q = f & 3;
            const int i = i0 + row, j = j0 + 4 * q;
            float4 x = make_float4(fill, fill, fill, fill);
            if (!mat) {  // the line cost (symmetric: the same for K and K^T)
                if (i < d) {
                    float c[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        c[e] = fill;
                        if (j + e < d) c[e] = LOG ? line_cost(i, j + e) : expf(-line_cost(i, j + e) * A.inv_eps);
                    }
                    x = make_float4(c[0], c[1], c[2], c[3]);
                }
            } else if (i < d) {
                const float *src = mat + (size_t)i * d + j;
                if (A.vec) {
                    if (j < d) x = *reinterpret_cast<const float4 *>(src);
                } else {
                    if (j < d) x.x = src[0];
                    if (j + 1 < d) x.y = src[1];
                    if (j + 2 < d) x.z = src[2];
                    if (j + 3 < d) x.w = src[3];
                }
            }
            pm[h] = x;
        }
        ps = make_float4(sfill, sfill, sfill, sfill);
        if (tid < TB * 4) {
            const int p = tid >> 2, q = tid & 3;
            const int b = b0 + p, j = j0 + 4 * q;
            if (b < n) {
                // u and v are rewritten by other CTAs during the launch: L2 loads, never L1
                const float *src = scale + (size_t)b * d + j;
                if (A.vec) {
                    if (j < d) ps = __ldcg(reinterpret_cast<const float4 *>(src));
                } else {
                    if (j < d) ps.x = __ldcg(src);
                    if (j + 1 < d) ps.y = __ldcg(src + 1);
                    if (j + 2 < d) ps.z = __ldcg(src + 2);
                    if (j + 3 < d) ps.w = __ldcg(src + 3);
                }
            }
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int f = tid + h * kSkThreads;
            float4 x = pm[h];
            if (LOG) {  // base-2 exponent of the matrix term; -inf stays -inf
                x.x *= mscale;
                x.y *= mscale;
                x.z *= mscale;
                x.w *= mscale;
            }
            *reinterpret_cast<float4 *>(&st.mat[buf][(f >> 2) * kSkPitch + 4 * (f & 3)]) = x;
        }
        if (tid < TB * 4) {
            float4 x = ps;
            if (LOG) {
                x.x *= kLog2e;
                x.y *= kLog2e;
                x.z *= kLog2e;
                x.w *= kLog2e;
            }
            *reinterpret_cast<float4 *>(&st.sc[buf][(tid >> 2) * kSkPitch + 4 * (tid & 3)]) = x;
        }
    };

    float acc[8][MB];  // scaling: sum; log: scaled sum
    float mx[LOG ? 8 : 1][LOG ? MB : 1];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int m = 0; m < MB; m++) {
            acc[r][m] = 0.0f;
            if (LOG) mx[LOG ? r : 0][LOG ? m : 0] = kNoMax;
        }

    const int nchunks = (d + kSkChunk - 1) / kSkChunk;
    load(0);
    __syncthreads();  // the previous tile's readers are done with buffer 0
    store(0);
    __syncthreads();
    for (int c = 0; c < nchunks; c++) {
        const int buf = c & 1;
        if (c + 1 < nchunks) load((c + 1) * kSkChunk);
        const float *ms = st.mat[buf];
        const float *ss = st.sc[buf];
#pragma unroll
        for (int jq = 0; jq < kSkChunk / 4; jq++) {
            float4 sv[MB];
#pragma unroll
            for (int m = 0; m < MB; m++)
                sv[m] = *reinterpret_cast<const float4 *>(&ss[(tb + 16 * m) * kSkPitch + 4 * jq]);
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const float4 kv = *reinterpret_cast<const float4 *>(&ms[(tr + 16 * r) * kSkPitch + 4 * jq]);
#pragma unroll
                for (int m = 0; m < MB; m++) {
                    if (!LOG) {
                        float a = acc[r][m];
                        a = fmaf(kv.x, sv[m].x, a);
                        a = fmaf(kv.y, sv[m].y, a);
                        a = fmaf(kv.z, sv[m].z, a);
                        a = fmaf(kv.w, sv[m].w, a);
                        acc[r][m] = a;
                    } else {
                        const float z0 = kv.x + sv[m].x, z1 = kv.y + sv[m].y;
                        const float z2 = kv.z + sv[m].z, z3 = kv.w + sv[m].w;
                        const float cm = fmaxf(fmaxf(z0, z1), fmaxf(z2, z3));
                        float &M = mx[LOG ? r : 0][LOG ? m : 0];
                        if (cm > M) {  // rare after the first chunks: rescale the sum
                            acc[r][m] *= ex2(M - cm);
                            M = cm;
                        }
                        acc[r][m] += (ex2(z0 - M) + ex2(z1 - M)) + (ex2(z2 - M) + ex2(z3 - M));
                    }
                }
            }
        }
        if (c + 1 < nchunks) store(buf ^ 1);
        __syncthreads();
    }

    // epilogue: outputs, and the residual partial of the plan this half-step starts from
#pragma unroll
    for (int m = 0; m < MB; m++) {
        const int b = b0 + tb + 16 * m;
        float res = 0.0f;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int i = i0 + tr + 16 * r;
            if (b < n && i < d) {
                const size_t idx = (size_t)b * d + i;
                const float nu = num[idx];
                float o;
                if (!LOG) {
                    if (partial_row) res += fabsf(nu - __ldcg(out + idx) * acc[r][m]);
                    o = nu / (acc[r][m] + 1e-12f);
                } else {
                    const float M = mx[LOG ? r : 0][LOG ? m : 0];
                    const bool none = !(M > kNoMax);  // every term was -inf
                    const float lse2 = M + log2f(acc[r][m]);
                    if (partial_row) {
                        const float old = __ldcg(out + idx);
                        const float plan_row = none ? 0.0f : ex2(fmaf(old, kLog2e, lse2));
                        res += fabsf(ex2(nu * kLog2e) - plan_row);
                    }
                    o = none ? -INFINITY : nu - lse2 * kLn2;
                }
                out[idx] = o;
            }
        }
        if (partial_row) {
            // the 16 lanes of this half-warp hold the 128 rows of pair b
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) res += __shfl_xor_sync(0xffffffffu, res, o);
            if (tr == 0 && b < n) partial_row[b] = (double)res;
        }
    }
}

template <bool LOG, int MB>
__global__ void __launch_bounds__(kSkThreads, 2) sk_solve_kernel(SkArgs A) {
    __shared__ __align__(16) SkStage st;
    constexpr int TB = 16 * MB;
    const int row_blocks = (A.d + kSkRows - 1) / kSkRows;
    const int pair_blocks = (A.n + TB - 1) / TB;
    const int tiles = row_blocks * pair_blocks;
    int check = 0;
    int it = 0;
    for (; it < A.max_iter; it++) {
        const bool checking = A.check_every > 0 && (it + 1) % A.check_every == 0;
        // u-update (tiles ordered row block major: CTAs running at once share matrix rows in L2)
        for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
            const int rb = t / pair_blocks, pb = t % pair_blocks;
            sk_tile<LOG, MB>(A, st, rb * kSkRows, pb * TB, A.num_u, A.mat, A.v, A.u,
                             checking ? A.partial + (size_t)rb * A.n : nullptr);
        }
        if (!grid_barrier_bounded(A.ctl, gridDim.x, A.status, A.spin_limit)) return;
        if (checking) {  // per-pair residual sums, one warp per pair, fixed order
            const int warps = gridDim.x * (kSkThreads / 32);
            const int lane = threadIdx.x & 31;
            for (int b = blockIdx.x * (kSkThreads / 32) + (threadIdx.x >> 5); b < A.n; b += warps) {
                double s = 0.0;
                for (int r = lane; r < row_blocks; r += 32) s += __ldcg(A.partial + (size_t)r * A.n + b);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) {
                    A.err[b] = s;
                    if (!(s <= (double)A.threshold)) atomicOr(&A.notconv[check], 1);
                }
            }
        }
        for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
            const int rb = t / pair_blocks, pb = t % pair_blocks;
            sk_tile<LOG, MB>(A, st, rb * kSkRows, pb * TB, A.num_v, A.mat_t, A.u, A.v, nullptr);
        }
        if (!grid_barrier_bounded(A.ctl, gridDim.x, A.status, A.spin_limit)) return;
        if (checking) {
            const bool stop = *((volatile int *)&A.notconv[check]) == 0;
            check++;
            if (stop) {
                it++;
                break;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) A.ctl->iterations = it;
}

// K = exp(-C / eps) and K^T (scaling form), or C^T alone (log form, EXP = false),
// through 32 x 32 shared-memory tiles so both writes are coalesced.  inv_eps is
// the float32 reciprocal of eps: torch evaluates a CUDA tensor divided by a
// scalar as the product with that reciprocal.
template <bool EXP>
__global__ void sk_prepare_kernel(const float *__restrict__ C, float *__restrict__ K, float *__restrict__ KT,
                                  int d, float inv_eps) {
    __shared__ float tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int i = by + r, j = bx + threadIdx.x;
        if (i < d && j < d) {
            float x = C[(size_t)i * d + j];
            if (EXP) {
                x = expf(-x * inv_eps);  // the reference's torch.exp(-cost_matrix / epsilon) on CUDA
                K[(size_t)i * d + j] = x;
            }
            tile[r][threadIdx.x] = x;
        }
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int j = bx + r, i = by + threadIdx.x;
        if (i < d && j < d) KT[(size_t)j * d + i] = tile[threadIdx.x][r];
    }
}

__global__ void sk_fill_kernel(float *__restrict__ x, float *__restrict__ y, size_t count, float value) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) {
        x[k] = value;
        y[k] = value;
    }
}

// y = log(x) elementwise (the reference's u.log(), a.log()), two arrays at once.
__global__ void sk_log_kernel(const float *__restrict__ x0, float *__restrict__ y0, const float *__restrict__ x1,
                              float *__restrict__ y1, size_t count) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < count; k += (size_t)gridDim.x * blockDim.x) {
        y0[k] = logf(x0[k]);
        y1[k] = logf(x1[k]);
    }
}

// ------------------------------------------------- transport cost and residual
// cost[b] = sum_ij P_ij C_ij and err[b] = sum_i |a_i - sum_j P_ij| with
// P_ij = exp((log u_i - C_ij / eps) + log v_j), the reference's plan
// (optimal_transport.py:136-144) without materialising it.  A CTA takes 128
// rows x 16 pairs; per row and pair, fp32 sums over 16-column chunks are
// added in fp64, and the row blocks are reduced in fixed order by
// sk_cost_reduce_kernel.
__global__ void __launch_bounds__(kSkThreads)
    sk_cost_kernel(const float *__restrict__ lu, const float *__restrict__ lv, const float *__restrict__ C,
                   const float *__restrict__ a, int n, int d, float inv_eps, double *__restrict__ cost_part,
                   double *__restrict__ err_part) {
    constexpr int TB = 16;
    __shared__ __align__(16) float sc[kSkRows * kSkPitch];
    __shared__ __align__(16) float sv[TB * kSkPitch];
    const int pair_blocks = (n + TB - 1) / TB;
    const int rb = blockIdx.x / pair_blocks, pb = blockIdx.x % pair_blocks;
    const int i0 = rb * kSkRows, b0 = pb * TB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tr = lane & 15, tb = (lane >> 4) + 2 * warp;
    const int b = b0 + tb;
    float lui[8];
    double cacc[8], racc[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int i = i0 + tr + 16 * r;
        lui[r] = (i < d && b < n) ? lu[(size_t)b * d + i] : -INFINITY;
        cacc[r] = racc[r] = 0.0;
    }
    for (int j0 = 0; j0 < d; j0 += kSkChunk) {
        __syncthreads();
        for (int f = tid; f < kSkRows * kSkChunk; f += kSkThreads) {
            const int row = f / kSkChunk, col = f % kSkChunk;
            const int i = i0 + row, j = j0 + col;
            sc[row * kSkPitch + col] = (i < d && j < d) ? (C ? C[(size_t)i * d + j] : line_cost(i, j)) : 0.0f;
        }
        for (int f = tid; f < TB * kSkChunk; f += kSkThreads) {
            const int p = f / kSkChunk, col = f % kSkChunk;
            const int bb = b0 + p, j = j0 + col;
            sv[p * kSkPitch + col] = (bb < n && j < d) ? lv[(size_t)bb * d + j] : -INFINITY;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; r++) {
            float cs = 0.0f, rs = 0.0f;
#pragma unroll
            for (int k = 0; k < kSkChunk; k++) {
                const float c = sc[(tr + 16 * r) * kSkPitch + k];
                const float p = expf((lui[r] - c * inv_eps) + sv[tb * kSkPitch + k]);
                cs = fmaf(p, c, cs);
                rs += p;
            }
            cacc[r] += (double)cs;
            racc[r] += (double)rs;
        }
    }
    double cs = 0.0, es = 0.0;
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int i = i0 + tr + 16 * r;
        if (i < d && b < n) {
            cs += cacc[r];
            es += fabs((double)a[(size_t)b * d + i] - racc[r]);
        }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
        cs += __shfl_xor_sync(0xffffffffu, cs, o);
        es += __shfl_xor_sync(0xffffffffu, es, o);
    }
    if (tr == 0 && b < n) {
        cost_part[(size_t)rb * n + b] = cs;
        err_part[(size_t)rb * n + b] = es;
    }
}

__global__ void sk_cost_reduce_kernel(const double *__restrict__ cost_part, const double *__restrict__ err_part,
                                      int n, int row_blocks, double *__restrict__ cost, double *__restrict__ err) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    double c = 0.0, e = 0.0;
    for (int r = 0; r < row_blocks; r++) {
        c += cost_part[(size_t)r * n + b];
        e += err_part[(size_t)r * n + b];
    }
    if (cost) cost[b] = c;
    if (err) err[b] = e;
}

// ---------------------------------------------------------------- the plan
// plan[b, i, j] = exp((log u[b,i] - C[i,j] / eps) + log v[b,j]) with the
// reference's operations and rounding on CUDA tensors (optimal_transport.py:
// 228-237): C / eps as torch evaluates a CUDA tensor divided by a scalar (a
// product with the float32 reciprocal of eps), then the two additions in that
// order, each rounded (explicit _rn operations: no multiply-add contraction).
// One pass that writes each plan entry once (HBM-write bound); C is re-read
// from L2 per pair.
__global__ void sk_plan_kernel(const float *__restrict__ lu, const float *__restrict__ lv, const float *__restrict__ C,
                               int n, int d, float inv_eps, bool vec, float *__restrict__ plan) {
    const int64_t rows = (int64_t)n * d;
    for (int64_t row = blockIdx.x; row < rows; row += gridDim.x) {
        const int b = (int)(row / d), i = (int)(row % d);
        const float x = lu[row];
        const float *crow = C ? C + (size_t)i * d : nullptr;
        const float *vrow = lv + (size_t)b * d;
        float *prow = plan + (size_t)row * d;
        if (vec) {
            for (int j = 4 * threadIdx.x; j < d; j += 4 * blockDim.x) {
                const float4 c = crow ? *reinterpret_cast<const float4 *>(crow + j)
                                      : make_float4(line_cost(i, j), line_cost(i, j + 1), line_cost(i, j + 2),
                                                    line_cost(i, j + 3));
                const float4 v = *reinterpret_cast<const float4 *>(vrow + j);
                float4 o;
                o.x = expf(__fadd_rn(__fsub_rn(x, __fmul_rn(c.x, inv_eps)), v.x));
                o.y = expf(__fadd_rn(__fsub_rn(x, __fmul_rn(c.y, inv_eps)), v.y));
                o.z = expf(__fadd_rn(__fsub_rn(x, __fmul_rn(c.z, inv_eps)), v.z));
                o.w = expf(__fadd_rn(__fsub_rn(x, __fmul_rn(c.w, inv_eps)), v.w));
                *reinterpret_cast<float4 *>(prow + j) = o;
            }
        } else {
            for (int j = threadIdx.x; j < d; j += blockDim.x) {
                const float c = crow ? crow[j] : line_cost(i, j);
                prow[j] = expf(__fadd_rn(__fsub_rn(x, __fmul_rn(c, inv_eps)), vrow[j]));
            }
        }
    }
}

// --------------------------------------------- gradient w.r.t. the cost
// grad_C[i, j] = sum_b g[b] P_b[i, j]: the envelope-theorem gradient of the
// regularised transport cost with respect to the cost matrix, scaled by the
// upstream gradient of each pair's distance.  A CTA owns a 64 x 64 block of
// (i, j) (each thread 4 x 4 entries) and walks the pairs, 8 at a time, with
// the block's log-potentials staged in shared memory; plan entries are
// recomputed (base 2) and never stored.
constexpr int kGradTile = 64;
constexpr int kGradPairs = 8;

__global__ void __launch_bounds__(kSkThreads)
    sk_cost_grad_kernel(const float *__restrict__ lu, const float *__restrict__ lv, const float *__restrict__ C,
                        const float *__restrict__ gout, int n, int d, float mscale, float *__restrict__ grad) {
    __shared__ float su[kGradPairs][kGradTile];
    __shared__ float sv[kGradPairs][kGradTile];
    __shared__ float sg[kGradPairs];
    const int i0 = blockIdx.y * kGradTile, j0 = blockIdx.x * kGradTile;
    const int tid = threadIdx.x;
    const int ti = tid / 16, tj = tid % 16;  // entries (i0 + ti + 16 r, j0 + tj + 16 s)
    float mc[4][4], acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const int i = i0 + ti + 16 * r, j = j0 + tj + 16 * s;
            mc[r][s] = (i < d && j < d) ? (C ? C[(size_t)i * d + j] : line_cost(i, j)) * mscale : -INFINITY;
            acc[r][s] = 0.0f;
        }
    for (int p0 = 0; p0 < n; p0 += kGradPairs) {
        __syncthreads();
        for (int f = tid; f < kGradPairs * kGradTile; f += kSkThreads) {
            const int p = f / kGradTile, x = f % kGradTile;
            const int b = p0 + p;
            su[p][x] = (b < n && i0 + x < d) ? lu[(size_t)b * d + i0 + x] * kLog2e : -INFINITY;
            sv[p][x] = (b < n && j0 + x < d) ? lv[(size_t)b * d + j0 + x] * kLog2e : -INFINITY;
        }
        if (tid < kGradPairs) sg[tid] = p0 + tid < n ? gout[p0 + tid] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int p = 0; p < kGradPairs; p++) {
            const float g = sg[p];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const float x = su[p][ti + 16 * r];
#pragma unroll
                for (int s = 0; s < 4; s++) acc[r][s] = fmaf(g, ex2(mc[r][s] + (x + sv[p][tj + 16 * s])), acc[r][s]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const int i = i0 + ti + 16 * r, j = j0 + tj + 16 * s;
            if (i < d && j < d) grad[(size_t)i * d + j] = acc[r][s];
        }
}

// ------------------------------------------------------------------ host
int check_ptr(const void *p, const char *name) {
    if (!p) return fail(TM_ERR_INVALID_ARGUMENT, "%s is NULL", name);
    return TM_OK;
}

int check_nd(int64_t n, int64_t d) {
    if (n < 1 || d < 1) return fail(TM_ERR_INVALID_ARGUMENT, "need n >= 1 pairs and d >= 1 points, got (%lld, %lld)",
                                    (long long)n, (long long)d);
    if (n > (1 << 24) || d > (1 << 20) || n * d > ((int64_t)1 << 31))
        return fail(TM_ERR_TOO_LARGE, "problem too large: (%lld, %lld)", (long long)n, (long long)d);
    return TM_OK;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

// The persistent solver on caller-provided state.  control: 256-byte control
// block; partial/err/notconv only when check_every > 0.
int sk_launch(bool log_form, SkArgs A, cudaStream_t s) {
    int *status = nullptr;
    int st = device_status_word(&status);
    if (st != TM_OK) return st;
    A.status = status;
    A.spin_limit = grid_wait_budget();
    // autotuned variant: bit 0 = 64 pairs per tile (else 16), bit 1 = one CTA per SM
    // (else two); built-in: 64 pairs per tile above 24 pairs, two CTAs per SM
    const int variant = tune_variant(kTuneSinkhornF32, tune_class(kTuneSinkhornF32, A.n, A.d));
    const bool wide = variant < 0 ? A.n > 24 : (variant & 1) != 0;
    const void *kern;
    if (log_form) kern = wide ? (const void *)sk_solve_kernel<true, 4> : (const void *)sk_solve_kernel<true, 1>;
    else kern = wide ? (const void *)sk_solve_kernel<false, 4> : (const void *)sk_solve_kernel<false, 1>;
    int per_sm = 0;
    TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSkThreads, 0));
    if (per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "Sinkhorn kernel does not fit on an SM");
    if (variant >= 0 && (variant & 2)) per_sm = 1;
    const int tb = wide ? 64 : 16;
    const int64_t tiles = ceil_div(A.d, kSkRows) * ceil_div(A.n, tb);
    const int blocks = (int)std::min<int64_t>(tiles, (int64_t)per_sm * sm_count());
    TM_CHECK_CUDA(cudaMemsetAsync(A.ctl, 0, sizeof(SkControl), s));
    void *params[] = {&A};
    TM_CHECK_CUDA(cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(kSkThreads), params, 0, s));
    TM_LAUNCH_CHECK("sk_solve_kernel");
    return TM_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SkLayout {
    size_t mat, mat_t, su, sv, partial, err, notconv, ctl, cost_part, err_part, total;
};

SkLayout sk_layout(int64_t n, int64_t d, bool log_form, int64_t max_iter, int64_t check_every, bool line) {
    SkLayout L{};
    const size_t dd = (size_t)d * d * sizeof(float), nd = (size_t)n * d * sizeof(float);
    const size_t rblocks = (size_t)ceil_div(d, kSkRows);
    const size_t checks = check_every > 0 ? (size_t)(max_iter / check_every) + 1 : 1;
    size_t off = 0;
    L.mat = off;
    off += (log_form || line) ? 0 : align256(dd);  // K (the log form reads C itself)
    L.mat_t = off;
    off += line ? 0 : align256(dd);  // the line cost is computed where it is used
    L.su = off;
    off += align256(nd);  // u (scaling) or log a
    L.sv = off;
    off += align256(nd);  // v (scaling) or log b
    L.partial = off;
    off += align256(rblocks * n * sizeof(double));
    L.err = off;
    off += align256(n * sizeof(double));
    L.notconv = off;
    off += align256(checks * sizeof(int));
    L.ctl = off;
    off += align256(sizeof(SkControl));
    L.cost_part = off;
    off += align256(rblocks * n * sizeof(double));
    L.err_part = off;
    off += align256(rblocks * n * sizeof(double));
    L.total = off;
    return L;
}

template <typename T>
T *ws_at(void *ws, size_t off) {
    return reinterpret_cast<T *>(static_cast<unsigned char *>(ws) + off);
}

unsigned grid_for(size_t count) {
    return (unsigned)std::min<size_t>((count + 255) / 256, (size_t)sm_count() * 8);
}

int sk_cost(const float *lu, const float *lv, const float *C, const float *a, int64_t n, int64_t d, double epsilon,
            double *cost_part, double *err_part, double *cost, double *err, cudaStream_t s) {
    const int64_t rblocks = ceil_div(d, kSkRows);
    const unsigned blocks = (unsigned)(rblocks * ceil_div(n, 16));
    sk_cost_kernel<<<blocks, kSkThreads, 0, s>>>(lu, lv, C, a, (int)n, (int)d, 1.0f / (float)epsilon, cost_part,
                                                 err_part);
    TM_LAUNCH_CHECK("sk_cost_kernel");
    sk_cost_reduce_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(cost_part, err_part, (int)n, (int)rblocks, cost,
                                                                     err);
    TM_LAUNCH_CHECK("sk_cost_reduce_kernel");
    return TM_OK;
}

}  // namespace
}  // namespace tmc

// ----------------------------------------------------------------- C ABI
extern "C" size_t tm_sinkhorn_iter_workspace_size(void) { return sizeof(tmc::SkControl); }

// The reference's fixed-count fused iterations, in place, on the caller's
// matrices: one persistent launch for all n_iter iterations.
static int sk_fixed(bool log_form, const float *num_u, const float *num_v, const float *mat, const float *mat_t,
                    float *u, float *v, int64_t n, int64_t d, int64_t n_iter, double epsilon, void *workspace,
                    size_t workspace_bytes, cudaStream_t s) {
    using namespace tmc;
    const void *ptrs[] = {num_u, num_v, mat, mat_t, u, v};
    const char *names[] = {"a", "b", "matrix", "transposed matrix", "u", "v"};
    for (int k = 0; k < 6; k++)
        if (check_ptr(ptrs[k], names[k]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    int st = check_nd(n, d);
    if (st != TM_OK) return st;
    if (n_iter < 0) return fail(TM_ERR_INVALID_ARGUMENT, "n_iter must be >= 0");
    if (n_iter > (1LL << 30)) return fail(TM_ERR_TOO_LARGE, "n_iter too large");
    if (!workspace || workspace_bytes < sizeof(SkControl) || !aligned16(workspace))
        return fail(TM_ERR_WORKSPACE, "Sinkhorn iterations need a 16-byte aligned workspace of %zu bytes",
                    sizeof(SkControl));
    if (n_iter == 0) return TM_OK;
    SkArgs A{};
    A.num_u = num_u;
    A.num_v = num_v;
    A.mat = mat;
    A.mat_t = mat_t;
    A.u = u;
    A.v = v;
    A.n = (int)n;
    A.d = (int)d;
    A.mscale = log_form ? (float)(-1.4426950408889634 / epsilon) : 0.0f;
    A.max_iter = (int)n_iter;
    A.check_every = 0;
    A.ctl = static_cast<SkControl *>(workspace);
    A.vec = (d % 4) == 0 && aligned16(mat) && aligned16(mat_t) && aligned16(u) && aligned16(v);
    return sk_launch(log_form, A, s);
}

extern "C" int tm_sinkhorn_fastiter(const float *a, const float *b, const float *K, const float *K_T, float *u,
                                    float *v, int64_t n, int64_t d, int64_t n_iter, void *workspace,
                                    size_t workspace_bytes, tm_stream_t stream) {
    return sk_fixed(false, a, b, K, K_T, u, v, n, d, n_iter, 1.0, workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" int tm_sinkhorn_logiter(const float *log_a, const float *log_b, const float *M, const float *M_T,
                                   float *log_u, float *log_v, int64_t n, int64_t d, int64_t n_iter, double epsilon,
                                   void *workspace, size_t workspace_bytes, tm_stream_t stream) {
    if (!(epsilon > 0)) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive, got %g", epsilon);
    return sk_fixed(true, log_a, log_b, M, M_T, log_u, log_v, n, d, n_iter, epsilon, workspace, workspace_bytes,
                    (cudaStream_t)stream);
}

extern "C" size_t tm_sinkhorn_f32_workspace_size(int64_t n, int64_t d, int log_space, int64_t max_iter,
                                                 int64_t check_every, int line_cost) {
    if (n < 1 || d < 1 || max_iter < 0) return 0;
    return tmc::sk_layout(n, d, log_space != 0, max_iter, check_every, line_cost != 0).total;
}

extern "C" int tm_sinkhorn_f32_solve(const float *a, const float *b, const float *C, int64_t n, int64_t d,
                                     double epsilon, int log_space, int64_t max_iter, double threshold,
                                     int64_t check_every, float *log_u, float *log_v, double *cost, double *row_err,
                                     int32_t *iterations, void *workspace, size_t workspace_bytes,
                                     tm_stream_t stream) {
    using namespace tmc;
    const void *ptrs[] = {a, b, log_u, log_v};
    const char *names[] = {"a", "b", "log_u", "log_v"};
    for (int k = 0; k < 4; k++)
        if (check_ptr(ptrs[k], names[k]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    int st = check_nd(n, d);
    if (st != TM_OK) return st;
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive, got %g", epsilon);
    if (max_iter < 1 || max_iter > (1LL << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "max_iter must be in [1, 2^30]");
    const bool line = C == nullptr;  // the cost of d points on a line, computed where used
    if (threshold < 0) return fail(TM_ERR_INVALID_ARGUMENT, "threshold must be >= 0");
    if (threshold > 0 && check_every < 1) return fail(TM_ERR_INVALID_ARGUMENT, "check_every must be >= 1");
    if (threshold == 0) check_every = 0;
    const bool log_form = log_space != 0;
    const SkLayout L = sk_layout(n, d, log_form, max_iter, check_every, line);
    if (!workspace || workspace_bytes < L.total || ((uintptr_t)workspace & 255))
        return fail(TM_ERR_WORKSPACE, "workspace must be 256-byte aligned and hold %zu bytes", L.total);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nd = (size_t)n * d;
    float *su = ws_at<float>(workspace, L.su), *sv = ws_at<float>(workspace, L.sv);
    float *mat_t = line ? nullptr : ws_at<float>(workspace, L.mat_t);
    const dim3 tgrid((unsigned)ceil_div(d, 32), (unsigned)ceil_div(d, 32)), tblock(32, 8);
    SkArgs A{};
    A.inv_eps = 1.0f / (float)epsilon;
    if (log_form) {
        if (!line) {
            sk_prepare_kernel<false><<<tgrid, tblock, 0, s>>>(C, nullptr, mat_t, (int)d, 0.0f);
            TM_LAUNCH_CHECK("sk_prepare_kernel");
        }
        sk_log_kernel<<<grid_for(nd), 256, 0, s>>>(a, su, b, sv, nd);  // log a, log b
        TM_LAUNCH_CHECK("sk_log_kernel");
        sk_fill_kernel<<<grid_for(nd), 256, 0, s>>>(log_u, log_v, nd, 0.0f);
        TM_LAUNCH_CHECK("sk_fill_kernel");
        A.num_u = su;
        A.num_v = sv;
        A.mat = C;
        A.u = log_u;
        A.v = log_v;
        A.mscale = (float)(-1.4426950408889634 / epsilon);
    } else {
        float *K = line ? nullptr : ws_at<float>(workspace, L.mat);
        if (!line) {
            sk_prepare_kernel<true><<<tgrid, tblock, 0, s>>>(C, K, mat_t, (int)d, 1.0f / (float)epsilon);
            TM_LAUNCH_CHECK("sk_prepare_kernel");
        }
        sk_fill_kernel<<<grid_for(nd), 256, 0, s>>>(su, sv, nd, 1.0f);
        TM_LAUNCH_CHECK("sk_fill_kernel");
        A.num_u = a;
        A.num_v = b;
        A.mat = K;
        A.u = su;
        A.v = sv;
    }
    A.mat_t = mat_t;
    A.n = (int)n;
    A.d = (int)d;
    A.max_iter = (int)max_iter;
    A.check_every = (int)check_every;
    A.threshold = (float)threshold;
    A.partial = ws_at<double>(workspace, L.partial);
    A.err = ws_at<double>(workspace, L.err);
    A.notconv = ws_at<int>(workspace, L.notconv);
    A.ctl = ws_at<SkControl>(workspace, L.ctl);
    A.vec = (d % 4) == 0 && aligned16(A.mat) && aligned16(A.u) && aligned16(A.v) && aligned16(A.num_u) &&
            aligned16(A.num_v);
    if (check_every > 0)
        TM_CHECK_CUDA(cudaMemsetAsync(A.notconv, 0, (size_t)(max_iter / check_every + 1) * sizeof(int), s));
    if ((st = sk_launch(log_form, A, s)) != TM_OK) return st;
    if (!log_form) {
        sk_log_kernel<<<grid_for(nd), 256, 0, s>>>(su, log_u, sv, log_v, nd);
        TM_LAUNCH_CHECK("sk_log_kernel");
    }
    if (iterations)
        TM_CHECK_CUDA(cudaMemcpyAsync(iterations, &A.ctl->iterations, sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
    if (cost || row_err)
        return sk_cost(log_u, log_v, C, a, n, d, epsilon, ws_at<double>(workspace, L.cost_part),
                       ws_at<double>(workspace, L.err_part), cost, row_err, s);
    return TM_OK;
}

extern "C" int tm_sinkhorn_plan(const float *log_u, const float *log_v, const float *C, int64_t n, int64_t d,
                                double epsilon, float *plan, tm_stream_t stream) {
    using namespace tmc;
    const void *ptrs[] = {log_u, log_v, plan};
    const char *names[] = {"log_u", "log_v", "plan"};
    for (int k = 0; k < 3; k++)
        if (check_ptr(ptrs[k], names[k]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    int st = check_nd(n, d);
    if (st != TM_OK) return st;
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive, got %g", epsilon);
    const bool vec = (d % 4) == 0 && aligned16(log_v) && aligned16(C) && aligned16(plan);
    const unsigned blocks = (unsigned)std::min<int64_t>(n * d, (int64_t)sm_count() * 32);
    const float inv_eps = 1.0f / (float)epsilon;  // torch: tensor / scalar = tensor * (1 / scalar) on CUDA
    sk_plan_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(log_u, log_v, C, (int)n, (int)d, inv_eps, vec, plan);
    TM_LAUNCH_CHECK("sk_plan_kernel");
    return TM_OK;
}

extern "C" int tm_sinkhorn_cost_grad(const float *log_u, const float *log_v, const float *C,
                                     const float *grad_distance, int64_t n, int64_t d, double epsilon,
                                     float *grad_C, tm_stream_t stream) {
    using namespace tmc;
    const void *ptrs[] = {log_u, log_v, grad_distance, grad_C};
    const char *names[] = {"log_u", "log_v", "grad_distance", "grad_C"};
    for (int k = 0; k < 4; k++)
        if (check_ptr(ptrs[k], names[k]) != TM_OK) return TM_ERR_INVALID_ARGUMENT;
    int st = check_nd(n, d);
    if (st != TM_OK) return st;
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive, got %g", epsilon);
    const dim3 grid((unsigned)ceil_div(d, kGradTile), (unsigned)ceil_div(d, kGradTile));
    if (grid.y > 65535) return fail(TM_ERR_TOO_LARGE, "d too large for the gradient kernel");
    sk_cost_grad_kernel<<<grid, kSkThreads, 0, (cudaStream_t)stream>>>(
        log_u, log_v, C, grad_distance, (int)n, (int)d, (float)(-1.4426950408889634 / epsilon), grad_C);
    TM_LAUNCH_CHECK("sk_cost_grad_kernel");
    return TM_OK;
}
