// Ragged point-cloud Sinkhorn: many OT problems of uneven sizes (n_p source
// and m_p target points in R^3, squared-Euclidean cost) solved together in
// ONE cooperative persistent launch, and the gradient of the regularised
// cost w.r.t. the points.
//
// Per problem, log-domain Sinkhorn iterations (the form of
// torchmorph/optimal_transport.py:96-125, with the cost recomputed from the
// points instead of read from a matrix):
//
//   f_i = -eps LSE_j( (g_j - C_ij)/eps + log b_j ),
//   g_j = -eps LSE_i( (f_i - C_ij)/eps + log a_i ),   C_ij = |x_i - y_j|^2.
//
// Work: the rows of all problems form 128-row tiles (the f-update), the
// columns 128-column tiles (the g-update).  The persistent CTAs take tiles
// from one queue per phase; a grid barrier separates the phases.  Inside a
// tile (32 own points x 8 lanes) each lane keeps an online log-sum-exp in
// base 2 (one ex2 per pair) over every 8th partner point, partners staged
// in shared memory 256 at a time; the lanes merge by shuffles.  Small tiles
// keep many CTAs busy when only a few slow problems are still iterating.
//
// Potentials use the dual form f = eps (log u - log a), g = eps (log v -
// log b) of the reference's log_u / log_v and start where log_u = log_v = 0.
//
// Stopping: on check iterations the g-update also accumulates, per problem,
// sum_j b_j |exp((g_old_j - g_new_j)/eps) - 1|, the L1 column-marginal
// error of the plan (f, g_old) whose rows the f-update just made exact;
// problems at or below the threshold stop and their tiles are skipped
// (threshold <= 0: every problem runs max_iter iterations, as the
// reference's threshold = 0).
//
// Every wait in the grid barrier is bounded; a barrier that gives up sets
// the library's device status word and an abort flag that makes every CTA
// leave.  The launch is cooperative, so all CTAs are co-resident.
#include <algorithm>
#include <cmath>
#include <vector>

#include "tm_common.cuh"
#include "tm_tma.cuh"

namespace tmc {
namespace {

constexpr int kPcThreads = 256;
constexpr int kPcLanes = 16;                      // threads sharing one group of own points
constexpr int kPcRep = 4;                         // own points per thread
constexpr int kPcGroups = kPcThreads / kPcLanes;  // 16 groups
constexpr int kPcTile = kPcGroups * kPcRep;       // 64 own points per tile
constexpr int kPcChunk = 256;                     // partner points staged per pass
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;

struct PcProblem {
    int64_t x0, y0;  // first source / target point (packed arrays)
    int n, m;
    int row_tile0, col_tile0;  // first row tile / column tile of the problem
    float ox, oy, oz;          // centroid of both clouds (the kernels work in centred coordinates)
    int pad;
};

// 2^x with the hardware approximation (MUFU.EX2, ~2 ulp, subnormal results
// flushed: they are below 2^-126 of the running maximum and cannot change a
// float32 sum).
__device__ __forceinline__ float fast_exp2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct PcControl {
    unsigned barrier_count;
    unsigned barrier_gen;
    int n_active;
    int abort;
    int iterations;  // iterations run (all problems)
    int n_row_list, n_col_list;  // tiles of the still-active problems
    int pad[57];
};
static_assert(sizeof(PcControl) == 256, "control block is 256 bytes");

struct PcArgs {
    const float *x, *y;    // (Nx, 3), (Ny, 3)
    const float *la, *lb;  // log weights (Nx), (Ny)
    float *f, *g;          // potentials (Nx), (Ny)
    const PcProblem *prob;
    int nprob, row_tiles, col_tiles;
    float *err;       // per problem: marginal error being accumulated
    int *active;      // per problem: 1 while iterating
    int *iters;       // per problem: iterations when it stopped
    int *queue;       // 2 * max_iter tile counters
    const int *tile_prob;     // problem of every row tile, then of every column tile
    int *row_list, *col_list;  // tiles of the active problems (rebuilt on check iterations)
    PcControl *ctl;
    int *status;
    float eps, threshold;
    int max_iter, check_every;
    long long spin_limit;  // polls a barrier wait may take (tm_set_grid_wait_budget)
};


__device__ __forceinline__ int find_problem(const PcProblem *prob, int nprob, int tile, bool rows) {
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((rows ? prob[mid].row_tile0 : prob[mid].col_tile0) <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One tile of one half-iteration.  "Own" side: the 64 points being updated
// (rows for the f-update); "other" side: all points of the partner cloud.
// Thread t is lane t % 16 of group t / 16; the group owns points
// group + 16 q (q < 4) and each lane visits every 16th partner, so one
// 16-byte shared-memory read of a partner feeds four pairs.
//
// In base 2, with x^ = x - o, y^ = y - o (o the problem's centroid) and
// k = log2(e) / eps, the exponent of a pair is
//   z_ij = w_j - k |x^_i - y^_j|^2 = [w_j - k |y^_j|^2] + (2k x^_i) . y^_j - k |x^_i|^2,
// w_j = (pot_j / eps + log weight_j) log2(e): three FMAs per pair on a staged
// record (y^_j, w_j - k |y^_j|^2); the last term is added once per own point.
// Centring keeps |y^|^2 small, so the expansion loses ~1e-5 relative at most.
// Each lane keeps a running maximum (updated once per 4 partners) and a sum
// of 2^(z - max); the 16 lanes of an own point merge by shuffles.
__device__ void update_tile(const float *own_pts, const float *other_pts, const float *other_pot,
                            const float *other_lw, float *own_pot, int own0, int n_own, int n_other, float eps,
                            float3 o, float *err_acc, const float *own_lw, float4 *s_part) {
    const int grp = threadIdx.x / kPcLanes, lane = threadIdx.x % kPcLanes;
    const float k = kLog2e / eps, inv_eps = 1.f / eps;
    float qx[kPcRep], qy[kPcRep], qz[kPcRep], rr[kPcRep], mx[kPcRep], sum[kPcRep];
#pragma unroll
    for (int q = 0; q < kPcRep; q++) {
        const int i = own0 + grp + kPcGroups * q;
        const bool v = i < n_own;
        const float xx = v ? own_pts[3 * i] - o.x : 0.f, xy = v ? own_pts[3 * i + 1] - o.y : 0.f,
                    xz = v ? own_pts[3 * i + 2] - o.z : 0.f;
        qx[q] = 2.f * k * xx;
        qy[q] = 2.f * k * xy;
        qz[q] = 2.f * k * xz;
        rr[q] = -k * fmaf(xx, xx, fmaf(xy, xy, xz * xz));
        mx[q] = -1e30f;
        sum[q] = 0.f;
    }
    // partner records: (y^, w - k |y^|^2); padding contributes 2^-inf = 0
    auto record = [&](int j) {
        if (j >= n_other) return make_float4(0.f, 0.f, 0.f, -INFINITY);
        const float yx = other_pts[3 * j] - o.x, yy = other_pts[3 * j + 1] - o.y, yz = other_pts[3 * j + 2] - o.z;
        const float w = fmaf(other_pot[j], inv_eps, other_lw[j]) * kLog2e;
        return make_float4(yx, yy, yz, fmaf(-k, fmaf(yx, yx, fmaf(yy, yy, yz * yz)), w));
    };
    static_assert(kPcChunk == kPcThreads, "one partner record per thread and chunk");
    // two staging buffers: the next chunk's global loads are in flight while
    // the current chunk is computed, and one barrier per chunk suffices
    float4 next = record(threadIdx.x);
    int buf = 0;
    for (int j0 = 0; j0 < n_other; j0 += kPcChunk, buf ^= 1) {
        const int cnt = min(kPcChunk, n_other - j0);
        float4 *sp = s_part + buf * kPcChunk;
        sp[threadIdx.x] = next;
        __syncthreads();
        if (j0 + kPcChunk < n_other) next = record(j0 + kPcChunk + threadIdx.x);
        const int rounds = (cnt + 4 * kPcLanes - 1) / (4 * kPcLanes);
        for (int rd = 0; rd < rounds; rd++) {
            float4 pt[4];
#pragma unroll
            for (int u = 0; u < 4; u++) pt[u] = sp[rd * 4 * kPcLanes + u * kPcLanes + lane];
#pragma unroll
            for (int q = 0; q < kPcRep; q++) {
                float z[4];
#pragma unroll
                for (int u = 0; u < 4; u++) z[u] = fmaf(qx[q], pt[u].x, fmaf(qy[q], pt[u].y, fmaf(qz[q], pt[u].z, pt[u].w)));
                const float bm = fmaxf(fmaxf(z[0], z[1]), fmaxf(z[2], z[3]));
                if (bm > mx[q]) {
                    sum[q] *= fast_exp2(mx[q] - bm);
                    mx[q] = bm;
                }
#pragma unroll
                for (int u = 0; u < 4; u++) sum[q] += fast_exp2(z[u] - mx[q]);
            }
        }
    }
    __syncthreads();  // the staging buffers are reused by the next tile
#pragma unroll
    for (int q = 0; q < kPcRep; q++) {
#pragma unroll
        for (int o2 = 1; o2 < kPcLanes; o2 <<= 1) {
            const float m2 = __shfl_xor_sync(0xffffffffu, mx[q], o2), s2 = __shfl_xor_sync(0xffffffffu, sum[q], o2);
            const float m = fmaxf(mx[q], m2);
            sum[q] = sum[q] * fast_exp2(mx[q] - m) + s2 * fast_exp2(m2 - m);
            mx[q] = m;
        }
        const int i = own0 + grp + kPcGroups * q;
        if (lane == 0 && i < n_own) {
            // pot = -eps * ln(sum 2^z) = -eps ln2 (m + log2 s + r)
            const float pot = -eps * kLn2 * (mx[q] + log2f(sum[q]) + rr[q]);
            if (err_acc) {
                const float d = (own_pot[i] - pot) / eps;
                *err_acc += expf(own_lw[i]) * fabsf(expm1f(d));
            }
            own_pot[i] = pot;
        }
    }
}

// Block-wide exclusive scan of one int per thread; returns the prefix and
// sets *total.
__device__ int block_exclusive_scan(int v, int *total, int *s_scan) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_scan[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < kPcThreads / 32; w++) {
            const int t = s_scan[w];
            s_scan[w] = run;
            run += t;
        }
        s_scan[kPcThreads / 32] = run;
    }
    __syncthreads();
    const int res = s_scan[warp] + x - v;
    *total = s_scan[kPcThreads / 32];
    __syncthreads();
    return res;
}

// Rebuild the row/column tile lists of the active problems (one CTA).
__device__ void rebuild_lists(const PcArgs &a, int *s_scan) {
    int rows_run = 0, cols_run = 0;
    for (int base = 0; base < a.nprob; base += kPcThreads) {
        const int p = base + threadIdx.x;
        int nr = 0, nc = 0;
        PcProblem P{};
        if (p < a.nprob && a.active[p]) {
            P = a.prob[p];
            nr = (P.n + kPcTile - 1) / kPcTile;
            nc = (P.m + kPcTile - 1) / kPcTile;
        }
        int tr = 0, tc = 0;
        const int orr = block_exclusive_scan(nr, &tr, s_scan);
        const int oc = block_exclusive_scan(nc, &tc, s_scan);
        for (int q = 0; q < nr; q++) a.row_list[rows_run + orr + q] = P.row_tile0 + q;
        for (int q = 0; q < nc; q++) a.col_list[cols_run + oc + q] = P.col_tile0 + q;
        rows_run += tr;
        cols_run += tc;
    }
    if (threadIdx.x == 0) {
        a.ctl->n_row_list = rows_run;
        a.ctl->n_col_list = cols_run;
    }
}

__global__ void __launch_bounds__(kPcThreads) pc_sinkhorn_kernel(PcArgs a) {
    __shared__ float4 s_part[2 * kPcChunk];
    __shared__ int s_tile;
    __shared__ float s_err;
    __shared__ int s_scan[kPcThreads / 32 + 1];
    const unsigned nblocks = gridDim.x;
    int it = 0;
    for (; it < a.max_iter; it++) {
        // f-update over the row tiles of the active problems
        const int nrow = *(volatile int *)&a.ctl->n_row_list;
        for (;;) {
            if (threadIdx.x == 0) s_tile = atomicAdd(&a.queue[2 * it], 1);
            __syncthreads();
            const int ticket = s_tile;
            __syncthreads();
            if (ticket >= nrow) break;
            const int tile = a.row_list[ticket];
            const PcProblem P = a.prob[a.tile_prob[tile]];
            update_tile(a.x + 3 * P.x0, a.y + 3 * P.y0, a.g + P.y0, a.lb + P.y0, a.f + P.x0,
                        (tile - P.row_tile0) * kPcTile, P.n, P.m, a.eps, make_float3(P.ox, P.oy, P.oz), nullptr,
                        nullptr, s_part);
        }
        if (!grid_barrier_bounded(a.ctl, nblocks, a.status, a.spin_limit)) return;
        const bool check = ((it + 1) % a.check_every == 0) || it + 1 == a.max_iter;
        // g-update over the column tiles (+ the column-marginal error on check iterations)
        const int ncol = *(volatile int *)&a.ctl->n_col_list;
        for (;;) {
            if (threadIdx.x == 0) {
                s_tile = atomicAdd(&a.queue[2 * it + 1], 1);
                s_err = 0.f;
            }
            __syncthreads();
            const int ticket = s_tile;
            __syncthreads();
            if (ticket >= ncol) break;
            const int tile = a.col_list[ticket];
            const int p = a.tile_prob[a.row_tiles + tile];
            const PcProblem P = a.prob[p];
            float e = 0.f;
            update_tile(a.y + 3 * P.y0, a.x + 3 * P.x0, a.f + P.x0, a.la + P.x0, a.g + P.y0,
                        (tile - P.col_tile0) * kPcTile, P.m, P.n, a.eps, make_float3(P.ox, P.oy, P.oz),
                        check ? &e : nullptr, a.lb + P.y0, s_part);
            if (check) {
                for (int o = 16; o; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
                if ((threadIdx.x & 31) == 0 && e != 0.f) atomicAdd(&s_err, e);
                __syncthreads();
                if (threadIdx.x == 0) atomicAdd(&a.err[p], s_err);
            }
        }
        if (!grid_barrier_bounded(a.ctl, nblocks, a.status, a.spin_limit)) return;
        if (check) {
            if (blockIdx.x == 0) {
                for (int p = threadIdx.x; p < a.nprob; p += kPcThreads) {
                    if (a.active[p] && ((a.threshold > 0.f && a.err[p] <= a.threshold) || it + 1 == a.max_iter)) {
                        a.active[p] = 0;
                        a.iters[p] = it + 1;
                        atomicSub(&a.ctl->n_active, 1);
                    }
                    a.err[p] = 0.f;
                }
                __syncthreads();
                rebuild_lists(a, s_scan);
                __threadfence();
            }
            if (!grid_barrier_bounded(a.ctl, nblocks, a.status, a.spin_limit)) return;
            if (*(volatile int *)&a.ctl->n_active <= 0) {
                it++;
                break;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl->iterations = it;
}

// Start of the reference's iteration, log_u = log_v = 0, in dual-potential
// form: f = -eps log a, g = -eps log b.
__global__ void pc_init_kernel(const float *lw, float *pot, int64_t count, float eps) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        pot[i] = -eps * lw[i];
}

// Centroid of both clouds of every problem (one CTA per problem).
__global__ void __launch_bounds__(kPcThreads) pc_center_kernel(const float *x, const float *y, PcProblem *prob) {
    __shared__ float red[3][kPcThreads / 32];
    PcProblem &P = prob[blockIdx.x];
    float s[3] = {0.f, 0.f, 0.f};
    for (int i = threadIdx.x; i < P.n; i += kPcThreads)
        for (int d = 0; d < 3; d++) s[d] += x[3 * (P.x0 + i) + d];
    for (int j = threadIdx.x; j < P.m; j += kPcThreads)
        for (int d = 0; d < 3; d++) s[d] += y[3 * (P.y0 + j) + d];
    for (int d = 0; d < 3; d++) {
        for (int o = 16; o; o >>= 1) s[d] += __shfl_xor_sync(0xffffffffu, s[d], o);
        if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = s[d];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float t[3] = {0.f, 0.f, 0.f};
        for (int w = 0; w < kPcThreads / 32; w++)
            for (int d = 0; d < 3; d++) t[d] += red[d][w];
        const float inv = 1.f / (float)(P.n + P.m);
        P.ox = t[0] * inv;
        P.oy = t[1] * inv;
        P.oz = t[2] * inv;
    }
}

// Regularised cost per problem: sum_i a_i f_i + sum_j b_j g_j (fp64 sums).
__global__ void __launch_bounds__(kPcThreads) pc_cost_kernel(const float *f, const float *g, const float *la,
                                                             const float *lb, const PcProblem *prob, double *cost) {
    __shared__ double red[kPcThreads / 32];
    const PcProblem P = prob[blockIdx.x];
    double s = 0.0;
    for (int i = threadIdx.x; i < P.n; i += kPcThreads) s += exp((double)la[P.x0 + i]) * f[P.x0 + i];
    for (int j = threadIdx.x; j < P.m; j += kPcThreads) s += exp((double)lb[P.y0 + j]) * g[P.y0 + j];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kPcThreads / 32; w++) t += red[w];
        cost[blockIdx.x] = t;
    }
}

// Gradient of the regularised cost w.r.t. one cloud (envelope theorem):
// d/dp_i = scale_p * 2 sum_j P_ij (p_i - q_j), P_ij = exp((f_i + g_j - C_ij)/eps
// + log a_i + log b_j) recomputed per pair.  Same 32 x 8 tiles as the
// iterations, partner points staged in shared memory.
__global__ void __launch_bounds__(kPcThreads) pc_grad_kernel(const float *own_pts, const float *other_pts,
                                                             const float *own_pot, const float *other_pot,
                                                             const float *own_lw, const float *other_lw,
                                                             const PcProblem *prob, int nprob, int tiles, bool rows,
                                                             float eps, const float *scale, float *grad) {
    __shared__ float4 s_part[kPcChunk];
    const float k = kLog2e / eps;
    const int grp = threadIdx.x / kPcLanes, lane = threadIdx.x % kPcLanes;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int p = find_problem(prob, nprob, tile, rows);
        const PcProblem P = prob[p];
        const int64_t o0 = rows ? P.x0 : P.y0, q0 = rows ? P.y0 : P.x0;
        const int n_own = rows ? P.n : P.m, n_other = rows ? P.m : P.n;
        const int first = (tile - (rows ? P.row_tile0 : P.col_tile0)) * kPcTile;
        float px[kPcRep], py[kPcRep], pz[kPcRep], base[kPcRep], ax[kPcRep], ay[kPcRep], az[kPcRep];
#pragma unroll
        for (int q = 0; q < kPcRep; q++) {
            const int i = first + grp + kPcGroups * q;
            const bool v = i < n_own;
            px[q] = v ? own_pts[3 * (o0 + i)] : 0.f;
            py[q] = v ? own_pts[3 * (o0 + i) + 1] : 0.f;
            pz[q] = v ? own_pts[3 * (o0 + i) + 2] : 0.f;
            base[q] = v ? (own_pot[o0 + i] / eps + own_lw[o0 + i]) * kLog2e : -INFINITY;
            ax[q] = ay[q] = az[q] = 0.f;
        }
        for (int j0 = 0; j0 < n_other; j0 += kPcChunk) {
            const int cnt = min(kPcChunk, n_other - j0);
            for (int t = threadIdx.x; t < cnt; t += kPcThreads) {
                const int64_t j = q0 + j0 + t;
                s_part[t] = make_float4(other_pts[3 * j], other_pts[3 * j + 1], other_pts[3 * j + 2],
                                        (other_pot[j] / eps + other_lw[j]) * kLog2e);
            }
            __syncthreads();
            for (int t = lane; t < cnt; t += kPcLanes) {
                const float4 pt = s_part[t];
#pragma unroll
                for (int q = 0; q < kPcRep; q++) {
                    const float dx = px[q] - pt.x, dy = py[q] - pt.y, dz = pz[q] - pt.z;
                    const float c = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const float pij = exp2f(fmaf(-k, c, base[q] + pt.w));
                    ax[q] = fmaf(pij, dx, ax[q]);
                    ay[q] = fmaf(pij, dy, ay[q]);
                    az[q] = fmaf(pij, dz, az[q]);
                }
            }
            __syncthreads();
        }
        const float sc = 2.f * scale[p];
#pragma unroll
        for (int q = 0; q < kPcRep; q++) {
#pragma unroll
            for (int o = 1; o < kPcLanes; o <<= 1) {
                ax[q] += __shfl_xor_sync(0xffffffffu, ax[q], o);
                ay[q] += __shfl_xor_sync(0xffffffffu, ay[q], o);
                az[q] += __shfl_xor_sync(0xffffffffu, az[q], o);
            }
            const int i = first + grp + kPcGroups * q;
            if (lane == 0 && i < n_own) {
                grad[3 * (o0 + i)] = sc * ax[q];
                grad[3 * (o0 + i) + 1] = sc * ay[q];
                grad[3 * (o0 + i) + 2] = sc * az[q];
            }
        }
    }
}

struct PcLayout {
    size_t prob, err, active, iters, queue, ctl, tile_prob, row_list, col_list, total;
};

PcLayout pc_layout(int64_t nprob, int64_t max_iter, int64_t row_tiles, int64_t col_tiles) {
    PcLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) / 256 * 256;
        return at;
    };
    L.ctl = take(sizeof(PcControl));
    L.prob = take((size_t)nprob * sizeof(PcProblem));
    L.err = take((size_t)nprob * 4);
    L.active = take((size_t)nprob * 4);
    L.iters = take((size_t)nprob * 4);
    L.queue = take((size_t)max_iter * 2 * 4);
    L.tile_prob = take((size_t)(row_tiles + col_tiles) * 4);
    L.row_list = take((size_t)row_tiles * 4);
    L.col_list = take((size_t)col_tiles * 4);
    L.total = off;
    return L;
}

template <typename T>
T *ws_at(void *ws, size_t off) {
    return reinterpret_cast<T *>(static_cast<unsigned char *>(ws) + off);
}

int build_problems(int64_t nprob, const int64_t *n, const int64_t *m, std::vector<PcProblem> &out, int *row_tiles,
                   int *col_tiles, int64_t *nx, int64_t *ny) {
    out.resize(nprob);
    int64_t x0 = 0, y0 = 0, rt = 0, ct = 0;
    for (int64_t p = 0; p < nprob; p++) {
        if (n[p] < 1 || m[p] < 1) return fail(TM_ERR_INVALID_ARGUMENT, "problem %lld has an empty cloud", (long long)p);
        if (n[p] > (1 << 24) || m[p] > (1 << 24)) return fail(TM_ERR_TOO_LARGE, "clouds are limited to 2^24 points");
        out[p].x0 = x0;
        out[p].y0 = y0;
        out[p].n = (int)n[p];
        out[p].m = (int)m[p];
        out[p].row_tile0 = (int)rt;
        out[p].col_tile0 = (int)ct;
        x0 += n[p];
        y0 += m[p];
        rt += ceil_div(n[p], kPcTile);
        ct += ceil_div(m[p], kPcTile);
        if (rt >= (1 << 30) || ct >= (1 << 30)) return fail(TM_ERR_TOO_LARGE, "too many tiles");
    }
    *row_tiles = (int)rt;
    *col_tiles = (int)ct;
    *nx = x0;
    *ny = y0;
    return TM_OK;
}

}  // namespace
}  // namespace tmc

extern "C" size_t tm_pointcloud_sinkhorn_workspace_size(int64_t n_problems, const int64_t *n, const int64_t *m,
                                                        int64_t max_iter) {
    using namespace tmc;
    if (n_problems < 1 || max_iter < 1 || !n || !m) return 0;
    int64_t rt = 0, ct = 0;
    for (int64_t p = 0; p < n_problems; p++) {
        rt += ceil_div(n[p] > 0 ? n[p] : 0, kPcTile);
        ct += ceil_div(m[p] > 0 ? m[p] : 0, kPcTile);
    }
    return pc_layout(n_problems, max_iter, rt, ct).total;
}

extern "C" int tm_pointcloud_sinkhorn(const float *x, const float *y, const float *log_a, const float *log_b,
                                      int64_t n_problems, const int64_t *n, const int64_t *m, double epsilon,
                                      int64_t max_iter, double threshold, int64_t check_every, float *f, float *g,
                                      double *cost, int32_t *iterations, void *workspace, size_t workspace_bytes,
                                      tm_stream_t stream) {
    using namespace tmc;
    if (!x || !y || !log_a || !log_b || !f || !g || !n || !m)
        return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n_problems < 1 || n_problems > (1 << 24)) return fail(TM_ERR_INVALID_ARGUMENT, "n_problems must be 1..2^24");
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive");
    if (max_iter < 1 || max_iter > (1 << 24)) return fail(TM_ERR_INVALID_ARGUMENT, "max_iter must be 1..2^24");
    if (check_every < 1) return fail(TM_ERR_INVALID_ARGUMENT, "check_every must be positive");
    std::vector<PcProblem> probs;
    int row_tiles = 0, col_tiles = 0;
    int64_t nx = 0, ny = 0;
    int st = build_problems(n_problems, n, m, probs, &row_tiles, &col_tiles, &nx, &ny);
    if (st != TM_OK) return st;
    const PcLayout L = pc_layout(n_problems, max_iter, row_tiles, col_tiles);
    if (!workspace || workspace_bytes < L.total)
        return fail(TM_ERR_WORKSPACE, "point-cloud Sinkhorn workspace of %zu bytes needed", L.total);
    if ((uintptr_t)workspace & 255) return fail(TM_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    // control block, errors, iteration counts and queues start at zero; every problem active,
    // every tile in the work lists
    TM_CHECK_CUDA(cudaMemsetAsync(workspace, 0, L.total, s));
    PcControl ctl{};
    ctl.n_active = (int)n_problems;
    ctl.n_row_list = row_tiles;
    ctl.n_col_list = col_tiles;
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<PcControl>(workspace, L.ctl), &ctl, sizeof(ctl), cudaMemcpyHostToDevice, s));
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<PcProblem>(workspace, L.prob), probs.data(), probs.size() * sizeof(PcProblem),
                                  cudaMemcpyHostToDevice, s));
    std::vector<int> ones((size_t)n_problems, 1);
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<int>(workspace, L.active), ones.data(), ones.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, s));
    std::vector<int> tile_prob((size_t)row_tiles + col_tiles), lists((size_t)row_tiles + col_tiles);
    for (int64_t p = 0; p < n_problems; p++) {
        for (int t = 0; t < (int)ceil_div(n[p], kPcTile); t++) tile_prob[probs[p].row_tile0 + t] = (int)p;
        for (int t = 0; t < (int)ceil_div(m[p], kPcTile); t++) tile_prob[row_tiles + probs[p].col_tile0 + t] = (int)p;
    }
    for (int t = 0; t < row_tiles; t++) lists[t] = t;
    for (int t = 0; t < col_tiles; t++) lists[row_tiles + t] = t;
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<int>(workspace, L.tile_prob), tile_prob.data(), tile_prob.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, s));
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<int>(workspace, L.row_list), lists.data(), (size_t)row_tiles * sizeof(int),
                                  cudaMemcpyHostToDevice, s));
    TM_CHECK_CUDA(cudaMemcpyAsync(ws_at<int>(workspace, L.col_list), lists.data() + row_tiles,
                                  (size_t)col_tiles * sizeof(int), cudaMemcpyHostToDevice, s));
    // potentials start where the reference's log_u = log_v = 0 does
    const unsigned init_blocks = (unsigned)std::min<int64_t>(ceil_div(nx > ny ? nx : ny, 256), 1024);
    pc_init_kernel<<<init_blocks, 256, 0, s>>>(log_a, f, nx, (float)epsilon);
    pc_init_kernel<<<init_blocks, 256, 0, s>>>(log_b, g, ny, (float)epsilon);
    TM_LAUNCH_CHECK("pc_init_kernel");
    pc_center_kernel<<<(unsigned)n_problems, kPcThreads, 0, s>>>(x, y, ws_at<PcProblem>(workspace, L.prob));
    TM_LAUNCH_CHECK("pc_center_kernel");
    int *status = nullptr;
    if ((st = device_status_word(&status)) != TM_OK) return st;
    int per_sm = 0;
    TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pc_sinkhorn_kernel, kPcThreads, 0));
    if (per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "point-cloud kernel does not fit on an SM");
    per_sm = per_sm > 4 ? 4 : per_sm;  // fewer CTAs make the grid barrier cheaper
    const int blocks = per_sm * sm_count();
    PcArgs args;
    args.x = x;
    args.y = y;
    args.la = log_a;
    args.lb = log_b;
    args.f = f;
    args.g = g;
    args.prob = ws_at<PcProblem>(workspace, L.prob);
    args.nprob = (int)n_problems;
    args.row_tiles = row_tiles;
    args.col_tiles = col_tiles;
    args.err = ws_at<float>(workspace, L.err);
    args.active = ws_at<int>(workspace, L.active);
    args.iters = ws_at<int>(workspace, L.iters);
    args.queue = ws_at<int>(workspace, L.queue);
    args.tile_prob = ws_at<int>(workspace, L.tile_prob);
    args.row_list = ws_at<int>(workspace, L.row_list);
    args.col_list = ws_at<int>(workspace, L.col_list);
    args.ctl = ws_at<PcControl>(workspace, L.ctl);
    args.status = status;
    args.eps = (float)epsilon;
    args.threshold = (float)threshold;
    args.max_iter = (int)max_iter;
    args.check_every = (int)check_every;
    args.spin_limit = grid_wait_budget();
    void *params[] = {&args};
    TM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void *)pc_sinkhorn_kernel, dim3(blocks), dim3(kPcThreads), params,
                                              0, s));
    TM_LAUNCH_CHECK("pc_sinkhorn_kernel");
    if (cost) {
        pc_cost_kernel<<<(unsigned)n_problems, kPcThreads, 0, s>>>(f, g, log_a, log_b, args.prob, cost);
        TM_LAUNCH_CHECK("pc_cost_kernel");
    }
    if (iterations)
        TM_CHECK_CUDA(cudaMemcpyAsync(iterations, args.iters, (size_t)n_problems * sizeof(int32_t),
                                      cudaMemcpyDeviceToDevice, s));
    return TM_OK;
}

extern "C" size_t tm_pointcloud_sinkhorn_grad_workspace_size(int64_t n_problems) {
    return n_problems < 1 ? 0 : (size_t)n_problems * sizeof(tmc::PcProblem);
}

extern "C" int tm_pointcloud_sinkhorn_grad(const float *x, const float *y, const float *log_a, const float *log_b,
                                           const float *f, const float *g, int64_t n_problems, const int64_t *n,
                                           const int64_t *m, double epsilon, const float *grad_cost, float *grad_x,
                                           float *grad_y, void *workspace, size_t workspace_bytes,
                                           tm_stream_t stream) {
    using namespace tmc;
    if (!x || !y || !log_a || !log_b || !f || !g || !n || !m || !grad_cost)
        return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n_problems < 1 || n_problems > (1 << 24)) return fail(TM_ERR_INVALID_ARGUMENT, "n_problems must be 1..2^24");
    if (!(epsilon > 0)) return fail(TM_ERR_INVALID_ARGUMENT, "epsilon must be positive");
    const size_t need = (size_t)n_problems * sizeof(PcProblem);
    if (!workspace || workspace_bytes < need) return fail(TM_ERR_WORKSPACE, "gradient workspace of %zu bytes needed", need);
    std::vector<PcProblem> probs;
    int row_tiles = 0, col_tiles = 0;
    int64_t nx = 0, ny = 0;
    int st = build_problems(n_problems, n, m, probs, &row_tiles, &col_tiles, &nx, &ny);
    if (st != TM_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    auto *dprob = static_cast<PcProblem *>(workspace);
    TM_CHECK_CUDA(cudaMemcpyAsync(dprob, probs.data(), need, cudaMemcpyHostToDevice, s));
    const int cap = sm_count() * 8;
    if (grad_x) {
        pc_grad_kernel<<<row_tiles < cap ? row_tiles : cap, kPcThreads, 0, s>>>(
            x, y, f, g, log_a, log_b, dprob, (int)n_problems, row_tiles, true, (float)epsilon, grad_cost, grad_x);
        TM_LAUNCH_CHECK("pc_grad_kernel");
    }
    if (grad_y) {
        pc_grad_kernel<<<col_tiles < cap ? col_tiles : cap, kPcThreads, 0, s>>>(
            y, x, g, f, log_b, log_a, dprob, (int)n_problems, col_tiles, false, (float)epsilon, grad_cost, grad_y);
        TM_LAUNCH_CHECK("pc_grad_kernel");
    }
    return TM_OK;
}
