// Exact EDT fast path for 2-D and 3-D items with unit spacing (GB300, sm_103a).
//
// Same result as the generic separable passes in edt.cu (scipy's feature
// tie rule), restructured around three facts of the workload:
//
//  * Compact features.  After pass 0 a voxel's nearest site so far is
//    (f0, own y, own x) and after pass 1 it is (f0, f1, own x), so the
//    intermediate state is one int16 (f0) or one packed int16x2 (f0, f1)
//    per voxel; squared distances are recomputed on chip instead of being
//    stored: 2 + 4 bytes of intermediates per voxel.
//
//  * Bounded windows.  d(q) = min_p (q-p)^2 + g(p) is at most the best
//    value found among p = q-K .. q+K, and every minimiser -- ties included
//    -- lies within |q-p| <= isqrt(d(q)).  So the (2K+1)-candidate window
//    (constant offsets k^2, evaluated in increasing p with a strict '<' so
//    the lowest position wins a tie) is exact whenever its best value is
//    below (K+1)^2, and is widened to the exact radius otherwise (K = 4 in
//    pass 1, 2 in pass 2).  Lines that would need a radius above kFar run
//    the Felzenszwalb-Huttenlocher lower envelope instead, so sparse inputs
//    keep O(L) work per line.
//
//  * Coalescing and occupancy.  Passes 0 and 1 run along non-contiguous axes:
//    a block stages a tile of 128 adjacent lines in shared memory with
//    vectorised row loads, and adjacent threads own adjacent lines, so every
//    store is a full row.  Pass 1 splits each line over 4 threads.  Pass 2
//    runs along the contiguous axis with one warp per line.
#include <cmath>
#include <cstring>

#include "edt_internal.cuh"

namespace tmc {
namespace {

constexpr int32_t kBig = 1 << 30;  // "no site"; eligible shapes keep every real value below it
constexpr int kCols = 128;         // lines per block in passes 0 and 1
constexpr int kSegs = 4;           // threads per line in pass 1
constexpr int kC2Warps = 8;        // lines per block in pass 2
constexpr int kFar = 24;           // widest exact window before a line uses the envelope
constexpr int kNear1 = 4;          // first window of pass 1: q-4 .. q+4
constexpr int kNear2 = 2;          // first window of pass 2: q-2 .. q+2
constexpr int kMaxL0Smem = 256;    // pass 0 stages lines up to this length
constexpr int kMaxL1 = 768;        // pass 1 tile: (L1 + 8) x 128 int16
constexpr int kMaxL2 = 4096;       // pass 2 line: (L + 4) x 8 + L x 2 bytes per warp

struct CompactParams {
    int ndim;        // 2 or 3
    int L0, L1, L2;  // sizes (2-D: L0 = H, L1 = W, L2 = 1)
    int64_t batch;
    int64_t numel;   // batch * numel_item
    int64_t numel_item;
};

// floor(sqrt(u)) for 0 <= u < 2^31 (the float estimate is off by at most one).
__device__ __forceinline__ int isqrt_floor(int32_t u) {
    long long r = (long long)sqrtf((float)u);
    while ((r + 1) * (r + 1) <= u) r++;
    while (r * r > u) r--;
    return (int)r;
}

// Best of the 2K+1 candidates q-K .. q+K given their values g[0..2K]: in
// increasing position with a strict '<', so the lowest position wins a tie.
template <int K>
__device__ __forceinline__ void best_window(const int32_t *g, int32_t &best, int &bi) {
    best = g[0] + K * K;
    bi = 0;
#pragma unroll
    for (int k = 1; k <= 2 * K; k++) {
        const int32_t v = g[k] + (k - K) * (k - K);
        if (v < best) {
            best = v;
            bi = k;
        }
    }
}

// Widen the search of position q from the first window |q-p| <= K to the
// exact radius isqrt(best).  G(p) reads the line (valid for 0 <= p < L).
// Returns false when the radius exceeds kFar.
template <int K, typename GF>
__device__ __forceinline__ bool widen(int q, int L, GF G, int32_t &best, int &bp) {
    const int r = best >= kBig ? L : isqrt_floor(best);
    if (r > kFar) return false;
    const int lo = q - r < 0 ? 0 : q - r, hi = q + r >= L ? L - 1 : q + r;
    for (int pp = lo; pp < q - K; pp++) {
        const int32_t v = (q - pp) * (q - pp) + G(pp);
        if (v < best || (v == best && pp < bp)) {
            best = v;
            bp = pp;
        }
    }
    for (int pp = q + K + 1; pp <= hi; pp++) {
        const int32_t v = (q - pp) * (q - pp) + G(pp);
        if (v < best) {
            best = v;
            bp = pp;
        }
    }
    return true;
}

// ------------------------------------------------------------------ pass 0
// Nearest background along axis 0, written as its position f0 (-1: none).
// Staged variant: a block owns 128 adjacent columns of one item.
template <typename In>
__global__ void __launch_bounds__(kCols) edt_c0_smem_kernel(const In *__restrict__ in, int16_t *__restrict__ c1,
                                                            CompactParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = p.L0;
    const int64_t inner = p.numel_item / L;
    uint8_t *fg = smem_raw;                                             // [L][kCols]
    int16_t *prev = reinterpret_cast<int16_t *>(smem_raw + L * kCols);  // [L][kCols]
    const int64_t cblocks = (inner + kCols - 1) / kCols;
    const int64_t item = blockIdx.x / cblocks;
    const int64_t c0 = (blockIdx.x - item * cblocks) * kCols;
    const int64_t base = item * p.numel_item + c0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // stage: warp w takes rows w, w+4, ...; lane covers columns 4*lane .. 4*lane+3
    for (int y0 = warp; y0 < L; y0 += 4 * 8) {
        In v[8][4];
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int y = y0 + 4 * r;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int64_t c = c0 + 4 * lane + k;
                v[r][k] = (y < L && c < inner) ? in[base + (int64_t)y * inner + 4 * lane + k] : (In)1;
            }
        }
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int y = y0 + 4 * r;
            if (y < L) {
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) word |= (uint32_t)(v[r][k] != (In)0) << (8 * k);
                reinterpret_cast<uint32_t *>(fg + y * kCols)[lane] = word;
            }
        }
    }
    __syncthreads();
    const bool active = c0 + tid < inner;
    int last = -1;
    for (int y = 0; y < L; y++) {
        if (fg[y * kCols + tid] == 0) last = y;
        prev[y * kCols + tid] = (int16_t)last;
    }
    int next = -1;
    int16_t *out = c1 + base + tid;
    for (int y = L - 1; y >= 0; y--) {
        const int pv = prev[y * kCols + tid];
        if (pv == y) next = y;
        const int f = (pv >= 0 && (next < 0 || y - pv <= next - y)) ? pv : next;
        if (active) out[(int64_t)y * inner] = (int16_t)f;
    }
}

// Unstaged variant for long axis-0 lines: one thread per column, two sweeps
// through global memory with 8 loads in flight.
template <typename In>
__global__ void __launch_bounds__(128) edt_c0_kernel(const In *__restrict__ in, int16_t *__restrict__ c1,
                                                     CompactParams p) {
    const int64_t inner = p.numel_item / p.L0;
    const int64_t nlines = p.batch * inner;
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= nlines) return;
    const int64_t item = line / inner;
    const int64_t i = line - item * inner;
    const int64_t base = item * p.numel_item + i;
    const int L = p.L0;
    int last = -1;
    int q = 0;
    for (; q + 8 <= L; q += 8) {
        In v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = in[base + (int64_t)(q + k) * inner];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            if (v[k] == (In)0) last = q + k;
            c1[base + (int64_t)(q + k) * inner] = (int16_t)last;
        }
    }
    for (; q < L; q++) {
        if (in[base + (int64_t)q * inner] == (In)0) last = q;
        c1[base + (int64_t)q * inner] = (int16_t)last;
    }
    int next = -1;
    q = L - 1;
    for (; q - 8 >= -1; q -= 8) {
        int prev[8];
#pragma unroll
        for (int k = 0; k < 8; k++) prev[k] = c1[base + (int64_t)(q - k) * inner];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int z = q - k;
            if (prev[k] == z) next = z;
            const int f = (prev[k] >= 0 && (next < 0 || z - prev[k] <= next - z)) ? prev[k] : next;
            c1[base + (int64_t)z * inner] = (int16_t)f;
        }
    }
    for (; q >= 0; q--) {
        const int pv = c1[base + (int64_t)q * inner];
        if (pv == q) next = q;
        const int f = (pv >= 0 && (next < 0 || q - pv <= next - q)) ? pv : next;
        c1[base + (int64_t)q * inner] = (int16_t)f;
    }
}

// ------------------------------------------------------------------ pass 1
// 3-D only: lines along axis 1 at fixed (item, z, x).  A block owns the
// (L1 x 128) tile of one (item, z) plane; 4 threads share each line.
// Output per voxel: packed (f0 | f1 << 16); f0 = -1 when no site.
__device__ __forceinline__ int32_t g_of_f0(int f0, int z) {
    return f0 < 0 ? kBig : (z - f0) * (z - f0);
}

__global__ void __launch_bounds__(kCols *kSegs) edt_c1_kernel(const int16_t *__restrict__ c1,
                                                              int32_t *__restrict__ c2,
                                                              int16_t *__restrict__ gstack, CompactParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    int16_t *tile = reinterpret_cast<int16_t *>(smem_raw) + kNear1 * kCols;  // rows -kNear1 .. L1+kNear1-1
    int *colflag = reinterpret_cast<int *>(smem_raw + (size_t)(L1 + 2 * kNear1) * kCols * 2);
    const int xblocks = (W + kCols - 1) / kCols;
    const int64_t item_z = blockIdx.x / xblocks;
    const int xb = (int)(blockIdx.x - item_z * xblocks);
    const int64_t item = item_z / L0;
    const int z = (int)(item_z - item * L0);
    const int x0 = xb * kCols;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t plane = item * p.numel_item + (int64_t)z * L1 * W;
    // padding rows hold "no site"
    for (int i = tid; i < 2 * kNear1 * kCols; i += kCols * kSegs) {
        const int r = i / kCols, c = i % kCols;
        tile[(r < kNear1 ? r - kNear1 : L1 + r - kNear1) * kCols + c] = -1;
    }
    if (tid < kCols) colflag[tid] = 0;
    // stage rows: 16 warps, 4 int16 per lane, 4 rows in flight per warp
    const bool vec = (W % 4) == 0;
    for (int y0 = warp; y0 < L1; y0 += 16 * 4) {
        int16_t v[4][4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int y = y0 + 16 * r;
            const int64_t rb = plane + (int64_t)y * W + x0 + 4 * lane;
            if (y < L1 && vec && x0 + 4 * lane + 3 < W) {
                const short4 s4 = *reinterpret_cast<const short4 *>(c1 + rb);
                v[r][0] = s4.x;
                v[r][1] = s4.y;
                v[r][2] = s4.z;
                v[r][3] = s4.w;
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    v[r][k] = (y < L1 && x0 + 4 * lane + k < W) ? c1[rb + k] : (int16_t)-1;
            }
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int y = y0 + 16 * r;
            if (y < L1) {
                short4 s4;
                s4.x = v[r][0];
                s4.y = v[r][1];
                s4.z = v[r][2];
                s4.w = v[r][3];
                *reinterpret_cast<short4 *>(tile + y * kCols + 4 * lane) = s4;
            }
        }
    }
    __syncthreads();
    const int xl = tid % kCols, seg = tid / kCols;
    const int x = x0 + xl;
    const int16_t *col = tile + xl;  // element y at col[y * kCols], -2 <= y < L1 + 2
    int32_t *out = c2 + plane + x;
    auto G = [&](int pp) { return g_of_f0(col[pp * kCols], z); };
    bool fallback = false;
    if (x < W) {
        const int qa = seg * L1 / kSegs, qb = (seg + 1) * L1 / kSegs;
        constexpr int NW = 2 * kNear1 + 1;
        int32_t gw[NW];
        int fw[NW];
#pragma unroll
        for (int k = 0; k < NW - 1; k++) {
            fw[k] = col[(qa - kNear1 + k) * kCols];
            gw[k] = g_of_f0(fw[k], z);
        }
        for (int q = qa; q < qb; q++) {
            fw[NW - 1] = col[(q + kNear1) * kCols];
            gw[NW - 1] = g_of_f0(fw[NW - 1], z);
            int32_t best;
            int bi;
            best_window<kNear1>(gw, best, bi);
            int bp = q - kNear1 + bi;
            int bf = fw[0];
#pragma unroll
            for (int k = 1; k < NW; k++) bf = bi == k ? fw[k] : bf;
            if (best >= (kNear1 + 1) * (kNear1 + 1)) {
                if (!widen<kNear1>(q, L1, G, best, bp)) {
                    fallback = true;
                    break;
                }
                bf = col[bp * kCols];
            }
            out[(int64_t)q * W] = best >= kBig ? -1 : ((int32_t)(uint16_t)bf | (bp << 16));
#pragma unroll
            for (int k = 0; k < NW - 1; k++) {
                gw[k] = gw[k + 1];
                fw[k] = fw[k + 1];
            }
        }
    }
    if (fallback) colflag[xl] = 1;
    __syncthreads();
    if (seg != 0 || x >= W || !colflag[xl]) return;
    // exact lower envelope of the whole line; stack in the workspace
    const int64_t nlines = p.batch * (int64_t)L0 * W;
    const int64_t lid = (item * L0 + z) * (int64_t)W + x;
    int k = -1, top = 0, sec = 0;
    int32_t Gtop = 0, Gsec = 0;
    for (int q = 0; q < L1; q++) {
        const int32_t gq = G(q);
        if (gq >= kBig) continue;
        const int32_t Gq = gq + q * q;
        while (k >= 1) {
            const long long lhs = (long long)(Gq - Gtop) * (top - sec);
            const long long rhs = (long long)(Gtop - Gsec) * (q - top);
            if (lhs > rhs) break;
            k--;
            top = sec;
            Gtop = Gsec;
            if (k >= 1) {
                sec = gstack[(int64_t)(k - 1) * nlines + lid];
                Gsec = G(sec) + sec * sec;
            }
        }
        k++;
        gstack[(int64_t)k * nlines + lid] = (int16_t)q;
        sec = top;
        Gsec = Gtop;
        top = q;
        Gtop = Gq;
    }
    if (k < 0) {
        for (int q = 0; q < L1; q++) out[(int64_t)q * W] = -1;
        return;
    }
    int j = 0;
    int cur = gstack[lid];
    int32_t gcur = G(cur);
    int nxt = 0;
    int32_t gnxt = 0;
    if (k >= 1) {
        nxt = gstack[nlines + lid];
        gnxt = G(nxt);
    }
    for (int q = 0; q < L1; q++) {
        uint32_t fc = (uint32_t)((q - cur) * (q - cur)) + (uint32_t)gcur;
        while (j < k) {
            const uint32_t fn = (uint32_t)((q - nxt) * (q - nxt)) + (uint32_t)gnxt;
            if (!(fn < fc)) break;
            j++;
            cur = nxt;
            gcur = gnxt;
            fc = fn;
            if (j < k) {
                nxt = gstack[(int64_t)(j + 1) * nlines + lid];
                gnxt = G(nxt);
            }
        }
        out[(int64_t)q * W] = (int32_t)(uint16_t)col[cur * kCols] | (cur << 16);
    }
}

// ------------------------------------------------------------------ pass 2
// Final outputs of one voxel.
template <bool IN3D>
__device__ __forceinline__ void emit_c2(int64_t gi, int bp, int32_t best, int32_t f, float *dist,
                                        int32_t *indices, int32_t *sqdist, int64_t numel) {
    if (dist) dist[gi] = best < (1 << 24) ? __fsqrt_rn((float)best) : (float)sqrt((double)best);
    if (sqdist) sqdist[gi] = best;
    if (indices) {
        if (IN3D) {
            indices[gi] = (int16_t)(f & 0xffff);
            indices[numel + gi] = f >> 16;
            indices[2 * numel + gi] = bp;
        } else {
            indices[gi] = f;
            indices[numel + gi] = bp;
        }
    }
}

// Last axis, one warp per line.  IN3D: input is packed (f0, f1) per voxel;
// otherwise (2-D) it is f0.
template <bool IN3D>
__global__ void __launch_bounds__(kC2Warps * 32) edt_c2_kernel(const void *__restrict__ cin, float *__restrict__ dist,
                                                               int32_t *__restrict__ indices,
                                                               int32_t *__restrict__ sqdist, CompactParams p,
                                                               int warps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = IN3D ? p.L2 : p.L1;
    const int Lp = L + 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t *sg = reinterpret_cast<int32_t *>(smem_raw) + warp * Lp + 2;           // g, padded
    int32_t *sf = reinterpret_cast<int32_t *>(smem_raw) + (warps + warp) * Lp + 2;  // packed feature
    int16_t *st = reinterpret_cast<int16_t *>(reinterpret_cast<int32_t *>(smem_raw) + 2 * warps * Lp) + warp * L;
    const int64_t lines_per_item = IN3D ? (int64_t)p.L0 * p.L1 : (int64_t)p.L0;
    const int64_t nlines = p.batch * lines_per_item;
    const int64_t line = (int64_t)blockIdx.x * warps + warp;
    if (line >= nlines) return;
    const int64_t item = line / lines_per_item;
    const int64_t rem = line - item * lines_per_item;
    int z = 0, y;
    if (IN3D) {
        z = (int)(rem / p.L1);
        y = (int)(rem - (int64_t)z * p.L1);
    } else {
        y = (int)rem;
    }
    const int64_t base = line * L;
    if (lane < 4) {
        const int q = lane < 2 ? lane - 2 : L + lane - 2;
        sg[q] = kBig;
        sf[q] = -1;
    }
    // stage the line, 4 loads per lane in flight
    bool any = false;
    for (int q0 = lane; q0 < L; q0 += 128) {
        int32_t fv[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = q0 + 32 * k;
            if (IN3D)
                fv[k] = q < L ? reinterpret_cast<const int32_t *>(cin)[base + q] : -1;
            else
                fv[k] = q < L ? (int32_t)reinterpret_cast<const int16_t *>(cin)[base + q] : -1;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = q0 + 32 * k;
            if (q < L) {
                const int32_t f = fv[k];
                int32_t g;
                if (IN3D) {
                    const int f0 = (int16_t)(f & 0xffff), f1 = f >> 16;
                    g = f0 < 0 ? kBig : (z - f0) * (z - f0) + (y - f1) * (y - f1);
                } else {
                    g = f < 0 ? kBig : (y - f) * (y - f);
                }
                sg[q] = g;
                sf[q] = f;
                any |= g < kBig;
            }
        }
    }
    any = __any_sync(0xffffffffu, any);
    __syncwarp();
    const int64_t numel = p.numel;
    if (!any) {
        // no background anywhere in the item: virtual site (-1, 0, ...)
        for (int q = lane; q < L; q += 32) {
            const int64_t gi = base + q;
            const int32_t s2 = IN3D ? (z + 1) * (z + 1) + y * y + q * q : (y + 1) * (y + 1) + q * q;
            if (dist) dist[gi] = s2 < (1 << 24) ? __fsqrt_rn((float)s2) : (float)sqrt((double)s2);
            if (sqdist) sqdist[gi] = s2;
            if (indices) {
                indices[gi] = -1;
                indices[numel + gi] = 0;
                if (IN3D) indices[2 * numel + gi] = 0;
            }
        }
        return;
    }
    auto G = [&](int pp) { return sg[pp]; };
    bool fallback = false;
    for (int q = lane; q < L; q += 32) {
        int32_t gw[2 * kNear2 + 1];
#pragma unroll
        for (int k = 0; k <= 2 * kNear2; k++) gw[k] = sg[q - kNear2 + k];
        int32_t best;
        int bi;
        best_window<kNear2>(gw, best, bi);
        int bp = q - kNear2 + bi;
        if (best >= (kNear2 + 1) * (kNear2 + 1) && !widen<kNear2>(q, L, G, best, bp)) {
            fallback = true;
            break;
        }
        emit_c2<IN3D>(base + q, bp, best, sf[bp], dist, indices, sqdist, numel);
    }
    if (!__any_sync(0xffffffffu, fallback)) return;
    // exact lower envelope: lane 0 builds it into the shared stack, every
    // lane then locates its positions by binary search
    int ktop = 0;
    if (lane == 0) {
        int k = -1, top = 0, sec = 0;
        int32_t Gtop = 0, Gsec = 0;
        for (int q = 0; q < L; q++) {
            const int32_t gq = sg[q];
            if (gq >= kBig) continue;
            const int32_t Gq = gq + q * q;
            while (k >= 1) {
                const long long lhs = (long long)(Gq - Gtop) * (top - sec);
                const long long rhs = (long long)(Gtop - Gsec) * (q - top);
                if (lhs > rhs) break;
                k--;
                top = sec;
                Gtop = Gsec;
                if (k >= 1) {
                    sec = st[k - 1];
                    Gsec = sg[sec] + sec * sec;
                }
            }
            st[++k] = (int16_t)q;
            sec = top;
            Gsec = Gtop;
            top = q;
            Gtop = Gq;
        }
        ktop = k;
    }
    ktop = __shfl_sync(0xffffffffu, ktop, 0);
    __syncwarp();
    for (int q = lane; q < L; q += 32) {
        // largest k with f_{v[k]}(q) < f_{v[k-1]}(q): the envelope segment of q
        int lo = 0, hi = ktop;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            const int a = st[mid - 1], b = st[mid];
            const uint32_t fa = (uint32_t)((q - a) * (q - a)) + (uint32_t)sg[a];
            const uint32_t fb = (uint32_t)((q - b) * (q - b)) + (uint32_t)sg[b];
            if (fb < fa)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int bp = st[lo];
        const int32_t best = (q - bp) * (q - bp) + sg[bp];
        emit_c2<IN3D>(base + q, bp, best, sf[bp], dist, indices, sqdist, numel);
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

bool edt_compact_eligible(const Geometry &g, bool unit) {
    if (!unit || (g.ndim != 2 && g.ndim != 3)) return false;
    int64_t sum = 0;
    for (int d = 0; d < g.ndim; d++) {
        if (g.shape[d] > 32767) return false;
        sum += (g.shape[d] + 1) * (g.shape[d] + 1);
    }
    if (sum + 64 >= kBig) return false;  // every squared distance stays below kBig
    if (g.ndim == 3 && g.shape[1] > kMaxL1) return false;
    if (g.shape[g.ndim - 1] > kMaxL2) return false;
    if (g.numel >= ((int64_t)1 << 40)) return false;
    return true;
}

size_t edt_compact_workspace(const Geometry &g) {
    const size_t n = (size_t)g.numel;
    size_t s = align256(n * 2);                               // f0 per voxel
    if (g.ndim == 3) s += align256(n * 4) + align256(n * 2);  // (f0, f1) + pass-1 envelope stacks
    return s;
}

int edt_compact_run(const void *input, int in_dtype, const Geometry &g, float *dist, int32_t *indices,
                    int32_t *sqdist, unsigned char *ws, cudaStream_t stream) {
    CompactParams p;
    std::memset(&p, 0, sizeof(p));
    p.ndim = g.ndim;
    p.L0 = (int)g.shape[0];
    p.L1 = (int)g.shape[1];
    p.L2 = g.ndim == 3 ? (int)g.shape[2] : 1;
    p.batch = g.batch;
    p.numel = g.numel;
    p.numel_item = g.numel_item;
    const size_t n = (size_t)g.numel;
    int16_t *c1 = reinterpret_cast<int16_t *>(ws);
    int32_t *c2 = g.ndim == 3 ? reinterpret_cast<int32_t *>(ws + align256(n * 2)) : nullptr;
    int16_t *stack1 = g.ndim == 3 ? reinterpret_cast<int16_t *>(ws + align256(n * 2) + align256(n * 4)) : nullptr;
    // pass 0
    const int64_t inner0 = g.numel_item / g.shape[0];
    if (p.L0 <= kMaxL0Smem) {
        const int64_t blocks = g.batch * ceil_div(inner0, kCols);
        if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        const size_t smem = (size_t)p.L0 * kCols * 3;
        if (smem > 48 * 1024) {
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<float>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<uint8_t>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        }
        if (in_dtype == TM_F32)
            edt_c0_smem_kernel<float><<<(unsigned)blocks, kCols, smem, stream>>>(static_cast<const float *>(input), c1, p);
        else
            edt_c0_smem_kernel<uint8_t><<<(unsigned)blocks, kCols, smem, stream>>>(static_cast<const uint8_t *>(input),
                                                                                   c1, p);
        TM_LAUNCH_CHECK("edt_c0_smem_kernel");
    } else {
        const int64_t nlines0 = g.batch * inner0;
        const unsigned b0 = (unsigned)ceil_div(nlines0, 128);
        if (in_dtype == TM_F32)
            edt_c0_kernel<float><<<b0, 128, 0, stream>>>(static_cast<const float *>(input), c1, p);
        else
            edt_c0_kernel<uint8_t><<<b0, 128, 0, stream>>>(static_cast<const uint8_t *>(input), c1, p);
        TM_LAUNCH_CHECK("edt_c0_kernel");
    }
    // pass 1 (3-D)
    if (g.ndim == 3) {
        const int64_t blocks = g.batch * (int64_t)p.L0 * ceil_div(p.L2, kCols);
        if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        const size_t smem = (size_t)(p.L1 + 2 * kNear1) * kCols * sizeof(int16_t) + kCols * sizeof(int);
        if (smem > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        edt_c1_kernel<<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(c1, c2, stack1, p);
        TM_LAUNCH_CHECK("edt_c1_kernel");
    }
    // pass 2
    const int L = g.ndim == 3 ? p.L2 : p.L1;
    const size_t per_warp = (size_t)(L + 4) * 8 + (size_t)L * 2;
    int warps = kC2Warps;
    while (warps > 1 && per_warp * warps > 160 * 1024) warps >>= 1;
    const int64_t nlines2 = g.numel / L;
    const unsigned b2 = (unsigned)ceil_div(nlines2, warps);
    const size_t smem2 = per_warp * warps;
    if (g.ndim == 3) {
        if (smem2 > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c2_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem2));
        edt_c2_kernel<true><<<b2, warps * 32, smem2, stream>>>(c2, dist, indices, sqdist, p, warps);
    } else {
        if (smem2 > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c2_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem2));
        edt_c2_kernel<false><<<b2, warps * 32, smem2, stream>>>(c1, dist, indices, sqdist, p, warps);
    }
    TM_LAUNCH_CHECK("edt_c2_kernel");
    return TM_OK;
}

}  // namespace tmc
