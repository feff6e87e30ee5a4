// Exact EDT fast path for 2-D and 3-D items with unit spacing (GB300, sm_103a).
//
// Same result as the generic separable passes in edt.cu (scipy's feature
// tie rule), restructured around four facts of the workload:
//
//  * Compact features.  After pass 0 a voxel's nearest site so far is
//    (f0, own y, own x) and after pass 1 it is (f0, f1, own x), so the
//    intermediate state is one int16 (f0) or one packed int16x2 (f0, f1)
//    per voxel; squared distances are recomputed on chip instead of being
//    stored: 2 + 4 bytes of intermediates per voxel.
//
//  * Bounded windows.  d(q) = min_p (q-p)^2 + g(p) is at most the best
//    value among p = q-K .. q+K, and every minimiser -- ties included --
//    lies within |q-p| <= isqrt(d(q)).  So the (2K+1)-candidate window is
//    exact whenever its best value is below (K+1)^2 and is widened to the
//    exact radius otherwise (K = 4 in pass 1, 2 in pass 2).  Lines that
//    would need a radius above kFar run the Felzenszwalb-Huttenlocher lower
//    envelope instead, so sparse inputs keep O(L) work per line.
//
//  * Packed keys.  A candidate is the 32-bit key (value << 5) | k, k its
//    position in the window, so one unsigned min selects the smallest value
//    and, among equal values, the lowest position -- the separable tie
//    rule -- in two integer operations per candidate.
//
//  * Coalescing and occupancy.  Passes 0 and 1 run along non-contiguous axes:
//    a block stages 128 adjacent lines in shared memory with vectorised row
//    loads, adjacent threads own adjacent lines, and each line is split over
//    4 threads.  Pass 2 runs along the contiguous axis, one warp per line,
//    4 voxels per lane with 16-byte loads and stores.
#include <cmath>
#include <algorithm>
#include <array>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "edt_internal.cuh"

namespace tmc {
namespace {

constexpr uint32_t kBig = 1u << 26;  // "no site"; eligible shapes keep every real value below it
constexpr int kKeyShift = 5;         // key = value << 5 | window position
constexpr int kCols = 128;           // lines per block in passes 0 and 1
constexpr int kSegs = 4;             // threads per line in passes 0 and 1
constexpr int kC2Warps = 8;          // lines per block in pass 2
constexpr int kFar = 24;             // widest exact window before a line uses the envelope
constexpr int kNear1 = 4;            // first window of pass 1: q-4 .. q+4
constexpr int kNear2 = 2;            // first window of pass 2: q-2 .. q+2
constexpr int kQB = 8;               // pass 1 outputs per register window
constexpr int kPadTop = kNear1;      // pass 1 tile padding rows ("no site")
constexpr int kPadBot = kNear1 + kQB;
constexpr int kSqrtTab = 64;         // correctly rounded sqrt of 0..63 in shared memory
constexpr int kMaxL0Smem = 256;      // pass 0 stages lines up to this length
constexpr int kMaxL1 = 256;          // pass 1 tile: (L1 + 16) x 128 x 6 bytes
constexpr int kMaxL2 = 4096;         // pass 2 line: (L + 8) x 8 + L x 2 bytes per warp

struct CompactParams {
    int ndim;        // 2 or 3
    int L0, L1, L2;  // sizes (2-D: L0 = H, L1 = W, L2 = 1)
    int64_t batch;
    int64_t numel;   // batch * numel_item
    int64_t numel_item;
};

// floor(sqrt(u)) for 0 <= u < 2^31 (the float estimate is off by at most one).
__device__ __forceinline__ int isqrt_floor(uint32_t u) {
    long long r = (long long)sqrtf((float)u);
    while ((r + 1) * (r + 1) <= (long long)u) r++;
    while (r * r > (long long)u) r--;
    return (int)r;
}

// Smallest key of the window w[0..2K] (values already shifted by kKeyShift).
template <int K>
__device__ __forceinline__ uint32_t window_key(const uint32_t *w) {
    uint32_t key = w[0] + (uint32_t)((K * K) << kKeyShift);
#pragma unroll
    for (int k = 1; k <= 2 * K; k++) key = min(key, w[k] + (uint32_t)((((k - K) * (k - K)) << kKeyShift) | k));
    return key;
}

// Widen the search of position q from the first window |q-p| <= K to the
// exact radius isqrt(best).  G(p) reads the unshifted value for 0 <= p < L.
// Returns false when the radius exceeds `far`.
template <int K, typename GF>
__device__ __forceinline__ bool widen(int q, int L, GF G, uint32_t &best, int &bp, int far = kFar) {
    const int r = best >= kBig ? L : isqrt_floor(best);
    if (r > far) return false;
    const int lo = q - r < 0 ? 0 : q - r, hi = q + r >= L ? L - 1 : q + r;
    for (int pp = lo; pp < q - K; pp++) {
        const uint32_t v = (uint32_t)((q - pp) * (q - pp)) + G(pp);
        if (v < best || (v == best && pp < bp)) {
            best = v;
            bp = pp;
        }
    }
    for (int pp = q + K + 1; pp <= hi; pp++) {
        const uint32_t v = (uint32_t)((q - pp) * (q - pp)) + G(pp);
        if (v < best) {
            best = v;
            bp = pp;
        }
    }
    return true;
}

// ------------------------------------------------------------------ pass 0
// Nearest background along axis 0, written as its position f0 (-1: none).
// Staged variant: a block owns 128 adjacent columns of one item, 4 threads
// per column, each sweeping a quarter of the column; the quarters exchange
// their first/last background position through shared memory.
template <typename In>
__device__ __forceinline__ void edt_c0_smem_block(const int64_t blk, const In *__restrict__ in,
                                                  int16_t *__restrict__ c1, const CompactParams &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = p.L0;
    const int64_t inner = p.numel_item / L;
    uint8_t *fg = smem_raw;                                              // [L][kCols]
    int16_t *prev = reinterpret_cast<int16_t *>(smem_raw + L * kCols);   // [L][kCols]
    int16_t *seg_last = prev + L * kCols;                                // [kSegs][kCols]
    int16_t *seg_first = seg_last + kSegs * kCols;                       // [kSegs][kCols]
    const int64_t cblocks = (inner + kCols - 1) / kCols;
    const int64_t item = blk / cblocks;
    const int64_t c0 = (blk - item * cblocks) * kCols;
    const int64_t base = item * p.numel_item + c0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // stage: 16 warps take rows w, w+16, ...; lane covers columns 4*lane .. 4*lane+3
    for (int y0 = warp; y0 < L; y0 += 16 * 4) {
        In v[4][4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int y = y0 + 16 * r;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int64_t c = c0 + 4 * lane + k;
                v[r][k] = (y < L && c < inner) ? in[base + (int64_t)y * inner + 4 * lane + k] : (In)1;
            }
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int y = y0 + 16 * r;
            if (y < L) {
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < 4; k++) word |= (uint32_t)(v[r][k] != (In)0) << (8 * k);
                reinterpret_cast<uint32_t *>(fg + y * kCols)[lane] = word;
            }
        }
    }
    __syncthreads();
    const int col = tid % kCols, seg = tid / kCols;
    const int S = (L + kSegs - 1) / kSegs;
    const int ya = seg * S < L ? seg * S : L, yb = (seg + 1) * S < L ? (seg + 1) * S : L;
    int last = -1, first = -1;
    for (int y = ya; y < yb; y++) {
        if (fg[y * kCols + col] == 0) {
            last = y;
            first = first < 0 ? y : first;
        }
        prev[y * kCols + col] = (int16_t)last;
    }
    seg_last[seg * kCols + col] = (int16_t)last;
    seg_first[seg * kCols + col] = (int16_t)first;
    __syncthreads();
    int carry_prev = -1, next = -1;
    for (int s = seg - 1; s >= 0 && carry_prev < 0; s--) carry_prev = seg_last[s * kCols + col];
    for (int s = seg + 1; s < kSegs && next < 0; s++) next = seg_first[s * kCols + col];
    if (c0 + col >= inner) return;
    int16_t *out = c1 + base + col + (int64_t)(yb - 1) * inner;
    for (int y = yb - 1; y >= ya; y--, out -= inner) {
        int pv = prev[y * kCols + col];
        if (pv < 0) pv = carry_prev;
        if (pv == y) next = y;
        const int f = (pv >= 0 && (next < 0 || y - pv <= next - y)) ? pv : next;
        *out = (int16_t)f;
    }
}

// Grid-stride over column blocks (one resident wave when per-item flags are
// given, as for the fused passes).
template <typename In>
__global__ void __launch_bounds__(kCols *kSegs) edt_c0_smem_kernel(const In *__restrict__ in,
                                                                   int16_t *__restrict__ c1, CompactParams p,
                                                                   const int *__restrict__ todo) {
    pdl_wait();  // launched after the shell search: its flags are complete
    // the plane passes may be scheduled now: the flags they read are final
    pdl_trigger();
    const int64_t cblocks = (p.numel_item / p.L0 + kCols - 1) / kCols;
    const int64_t nblk = p.batch * cblocks;
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        if (todo && !todo[blk / cblocks]) continue;  // item finished by the shell pass
        edt_c0_smem_block<In>(blk, in, c1, p);
        __syncthreads();  // the next block reuses shared memory
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
        int prv[8];
#pragma unroll
        for (int k = 0; k < 8; k++) prv[k] = c1[base + (int64_t)(q - k) * inner];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int z = q - k;
            if (prv[k] == z) next = z;
            const int f = (prv[k] >= 0 && (next < 0 || z - prv[k] <= next - z)) ? prv[k] : next;
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
// (L1 x 128) tile of one (item, z) plane: shifted values gk = g << 5 and f0.
// Output per voxel: packed (f0 | f1 << 16); f0 = -1 when no site.
__global__ void __launch_bounds__(kCols *kSegs) edt_c1_kernel(const int16_t *__restrict__ c1,
                                                              int32_t *__restrict__ c2,
                                                              int16_t *__restrict__ gstack, CompactParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    const int rows = L1 + kPadTop + kPadBot;
    uint32_t *gk = reinterpret_cast<uint32_t *>(smem_raw) + kPadTop * kCols;  // rows -kPadTop .. L1+kPadBot-1
    int16_t *f0t = reinterpret_cast<int16_t *>(smem_raw + (size_t)rows * kCols * 4) + kPadTop * kCols;
    int *colflag = reinterpret_cast<int *>(smem_raw + (size_t)rows * kCols * 6);
    const int xblocks = (W + kCols - 1) / kCols;
    const int64_t item_z = blockIdx.x / xblocks;
    const int xb = (int)(blockIdx.x - item_z * xblocks);
    const int64_t item = item_z / L0;
    const int z = (int)(item_z - item * L0);
    const int x0 = xb * kCols;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t plane = item * p.numel_item + (int64_t)z * L1 * W;
    for (int i = tid; i < (kPadTop + kPadBot) * kCols; i += kCols * kSegs) {
        const int r = i / kCols, c = i % kCols;
        const int y = r < kPadTop ? r - kPadTop : L1 + r - kPadTop;
        gk[y * kCols + c] = kBig << kKeyShift;
        f0t[y * kCols + c] = -1;
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
                uint4 g4;
                uint32_t *gp = &g4.x;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int f = v[r][k];
                    gp[k] = (f < 0 ? kBig : (uint32_t)((z - f) * (z - f))) << kKeyShift;
                }
                *reinterpret_cast<uint4 *>(gk + y * kCols + 4 * lane) = g4;
                short4 s4;
                s4.x = v[r][0];
                s4.y = v[r][1];
                s4.z = v[r][2];
                s4.w = v[r][3];
                *reinterpret_cast<short4 *>(f0t + y * kCols + 4 * lane) = s4;
            }
        }
    }
    __syncthreads();
    const int xl = tid % kCols, seg = tid / kCols;
    const int x = x0 + xl;
    const uint32_t *gcol = gk + xl;  // element y at gcol[y * kCols]
    const int16_t *fcol = f0t + xl;
    int32_t *out = c2 + plane + x;
    auto G = [&](int pp) { return gcol[pp * kCols] >> kKeyShift; };
    bool fallback = false;
    if (x < W) {
        const int qa = seg * L1 / kSegs, qb = (seg + 1) * L1 / kSegs;
        constexpr int NW = kQB + 2 * kNear1;
        for (int q0 = qa; q0 < qb && !fallback; q0 += kQB) {
            uint32_t w[NW];
#pragma unroll
            for (int j = 0; j < NW; j++) w[j] = gcol[(q0 - kNear1 + j) * kCols];
#pragma unroll
            for (int i = 0; i < kQB; i++) {
                const int q = q0 + i;
                if (q < qb && !fallback) {
                    const uint32_t key = window_key<kNear1>(w + i);
                    uint32_t best = key >> kKeyShift;
                    int bp = q - kNear1 + (int)(key & 31u);
                    if (best >= (kNear1 + 1) * (kNear1 + 1) && !widen<kNear1>(q, L1, G, best, bp)) {
                        fallback = true;
                    } else {
                        const int bf = fcol[bp * kCols];
                        out[(int64_t)q * W] = best >= kBig ? -1 : ((int32_t)(uint16_t)bf | (bp << 16));
                    }
                }
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
        const uint32_t gq = G(q);
        if (gq >= kBig) continue;
        const int32_t Gq = (int32_t)gq + q * q;
        while (k >= 1) {
            const long long lhs = (long long)(Gq - Gtop) * (top - sec);
            const long long rhs = (long long)(Gtop - Gsec) * (q - top);
            if (lhs > rhs) break;
            k--;
            top = sec;
            Gtop = Gsec;
            if (k >= 1) {
                sec = gstack[(int64_t)(k - 1) * nlines + lid];
                Gsec = (int32_t)G(sec) + sec * sec;
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
    uint32_t gcur = G(cur);
    int nxt = 0;
    uint32_t gnxt = 0;
    if (k >= 1) {
        nxt = gstack[nlines + lid];
        gnxt = G(nxt);
    }
    for (int q = 0; q < L1; q++) {
        uint32_t fc = (uint32_t)((q - cur) * (q - cur)) + gcur;
        while (j < k) {
            const uint32_t fn = (uint32_t)((q - nxt) * (q - nxt)) + gnxt;
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
        out[(int64_t)q * W] = (int32_t)(uint16_t)fcol[cur * kCols] | (cur << 16);
    }
}

// ------------------------------------------------------------------ pass 2
__device__ __forceinline__ float dist_of(uint32_t best, const float *tab) {
    if (best < kSqrtTab) return tab[best];
    return best < (1u << 24) ? __fsqrt_rn((float)best) : (float)sqrt((double)best);
}

// Last axis, one warp per line.  IN3D: input is packed (f0, f1) per voxel;
// otherwise (2-D) it is f0.  VEC (lines a multiple of 128 long): each lane
// owns 4 consecutive voxels of every 128-voxel chunk, loads them with one
// vector load and writes each output plane with one 16-byte store.
template <bool IN3D, bool VEC>
__global__ void __launch_bounds__(kC2Warps * 32) edt_c2_kernel(const void *__restrict__ cin, float *__restrict__ dist,
                                                               int32_t *__restrict__ indices,
                                                               int32_t *__restrict__ sqdist, CompactParams p,
                                                               int warps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = IN3D ? p.L2 : p.L1;
    const int Lp = L + 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *tab = reinterpret_cast<float *>(smem_raw);                              // sqrt table
    uint32_t *base_u = reinterpret_cast<uint32_t *>(smem_raw) + kSqrtTab;
    uint32_t *sg = base_u + warp * Lp + 4;                                         // g << 5, padded by 4
    int32_t *sf = reinterpret_cast<int32_t *>(base_u) + (warps + warp) * Lp + 4;   // packed feature
    int16_t *st = reinterpret_cast<int16_t *>(base_u + 2 * warps * Lp) + warp * L;  // envelope stack
    for (int i = threadIdx.x; i < kSqrtTab; i += blockDim.x) tab[i] = __fsqrt_rn((float)i);
    __syncthreads();
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
    if (lane < 8) {
        const int q = lane < 4 ? lane - 4 : L + lane - 4;
        sg[q] = kBig << kKeyShift;
        sf[q] = -1;
    }
    auto gval = [&](int32_t f) -> uint32_t {
        if (IN3D) {
            const int f0 = (int16_t)(f & 0xffff), f1 = f >> 16;
            return f0 < 0 ? kBig : (uint32_t)((z - f0) * (z - f0) + (y - f1) * (y - f1));
        }
        return f < 0 ? kBig : (uint32_t)((y - f) * (y - f));
    };
    // stage the line
    bool any = false;
    if (VEC) {
        for (int c = 0; c < L; c += 128) {
            const int q0 = c + 4 * lane;
            int32_t f[4];
            if (IN3D) {
                const int4 v = *reinterpret_cast<const int4 *>(reinterpret_cast<const int32_t *>(cin) + base + q0);
                f[0] = v.x;
                f[1] = v.y;
                f[2] = v.z;
                f[3] = v.w;
            } else {
                const short4 v = *reinterpret_cast<const short4 *>(reinterpret_cast<const int16_t *>(cin) + base + q0);
                f[0] = v.x;
                f[1] = v.y;
                f[2] = v.z;
                f[3] = v.w;
            }
            uint4 g4;
            g4.x = gval(f[0]);
            g4.y = gval(f[1]);
            g4.z = gval(f[2]);
            g4.w = gval(f[3]);
            any |= (g4.x < kBig) | (g4.y < kBig) | (g4.z < kBig) | (g4.w < kBig);
            g4.x <<= kKeyShift;
            g4.y <<= kKeyShift;
            g4.z <<= kKeyShift;
            g4.w <<= kKeyShift;
            *reinterpret_cast<uint4 *>(sg + q0) = g4;
            *reinterpret_cast<int4 *>(sf + q0) = make_int4(f[0], f[1], f[2], f[3]);
        }
    } else {
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
                    const uint32_t g = gval(fv[k]);
                    sg[q] = g << kKeyShift;
                    sf[q] = fv[k];
                    any |= g < kBig;
                }
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
            const uint32_t s2 = IN3D ? (uint32_t)((z + 1) * (z + 1) + y * y + q * q)
                                     : (uint32_t)((y + 1) * (y + 1) + q * q);
            if (dist) dist[gi] = dist_of(s2, tab);
            if (sqdist) sqdist[gi] = (int32_t)s2;
            if (indices) {
                indices[gi] = -1;
                indices[numel + gi] = 0;
                if (IN3D) indices[2 * numel + gi] = 0;
            }
        }
        return;
    }
    auto G = [&](int pp) { return sg[pp] >> kKeyShift; };
    bool fallback = false;
    if (VEC) {
        for (int c = 0; c < L && !fallback; c += 128) {
            const int q0 = c + 4 * lane;
            uint32_t w[12];  // shifted g at q0-4 .. q0+7
            const uint4 a = *reinterpret_cast<const uint4 *>(sg + q0 - 4);
            const uint4 b = *reinterpret_cast<const uint4 *>(sg + q0);
            const uint4 d4 = *reinterpret_cast<const uint4 *>(sg + q0 + 4);
            w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
            w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
            w[8] = d4.x; w[9] = d4.y; w[10] = d4.z; w[11] = d4.w;
            float dv[4];
            int32_t i0[4], i1[4], i2[4], sq[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int q = q0 + i;
                const uint32_t key = window_key<kNear2>(w + i + 2);
                uint32_t best = key >> kKeyShift;
                int bp = q - kNear2 + (int)(key & 31u);
                if (best >= (kNear2 + 1) * (kNear2 + 1) && !widen<kNear2>(q, L, G, best, bp)) fallback = true;
                const int32_t f = sf[bp];
                dv[i] = dist_of(best, tab);
                sq[i] = (int32_t)best;
                if (IN3D) {
                    i0[i] = (int16_t)(f & 0xffff);
                    i1[i] = f >> 16;
                    i2[i] = bp;
                } else {
                    i0[i] = f;
                    i1[i] = bp;
                }
            }
            if (fallback) break;
            const int64_t gi = base + q0;
            if (dist) *reinterpret_cast<float4 *>(dist + gi) = make_float4(dv[0], dv[1], dv[2], dv[3]);
            if (sqdist) *reinterpret_cast<int4 *>(sqdist + gi) = make_int4(sq[0], sq[1], sq[2], sq[3]);
            if (indices) {
                *reinterpret_cast<int4 *>(indices + gi) = make_int4(i0[0], i0[1], i0[2], i0[3]);
                *reinterpret_cast<int4 *>(indices + numel + gi) = make_int4(i1[0], i1[1], i1[2], i1[3]);
                if (IN3D)
                    *reinterpret_cast<int4 *>(indices + 2 * numel + gi) = make_int4(i2[0], i2[1], i2[2], i2[3]);
            }
        }
    } else {
        for (int q = lane; q < L; q += 32) {
            uint32_t w[2 * kNear2 + 1];
#pragma unroll
            for (int k = 0; k <= 2 * kNear2; k++) w[k] = sg[q - kNear2 + k];
            const uint32_t key = window_key<kNear2>(w);
            uint32_t best = key >> kKeyShift;
            int bp = q - kNear2 + (int)(key & 31u);
            if (best >= (kNear2 + 1) * (kNear2 + 1) && !widen<kNear2>(q, L, G, best, bp)) {
                fallback = true;
                break;
            }
            const int64_t gi = base + q;
            const int32_t f = sf[bp];
            if (dist) dist[gi] = dist_of(best, tab);
            if (sqdist) sqdist[gi] = (int32_t)best;
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
    }
    if (!__any_sync(0xffffffffu, fallback)) return;
    // exact lower envelope: lane 0 builds it into the shared stack, every
    // lane then locates its positions by binary search
    int ktop = 0;
    if (lane == 0) {
        int k = -1, top = 0, sec = 0;
        int32_t Gtop = 0, Gsec = 0;
        for (int q = 0; q < L; q++) {
            const uint32_t gq = G(q);
            if (gq >= kBig) continue;
            const int32_t Gq = (int32_t)gq + q * q;
            while (k >= 1) {
                const long long lhs = (long long)(Gq - Gtop) * (top - sec);
                const long long rhs = (long long)(Gtop - Gsec) * (q - top);
                if (lhs > rhs) break;
                k--;
                top = sec;
                Gtop = Gsec;
                if (k >= 1) {
                    sec = st[k - 1];
                    Gsec = (int32_t)G(sec) + sec * sec;
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
            const uint32_t fa = (uint32_t)((q - a) * (q - a)) + G(a);
            const uint32_t fb = (uint32_t)((q - b) * (q - b)) + G(b);
            if (fb < fa)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int bp = st[lo];
        const uint32_t best = (uint32_t)((q - bp) * (q - bp)) + G(bp);
        const int64_t gi = base + q;
        const int32_t f = sf[bp];
        if (dist) dist[gi] = dist_of(best, tab);
        if (sqdist) sqdist[gi] = (int32_t)best;
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
}

// ------------------------------------------------------ passes 1 + 2 fused
// 3-D items with L0, L1 <= 255 and L2 a multiple of 4: one CTA per (item, z)
// plane runs pass 1 (axis 1) and pass 2 (axis 2) back to back on chip.  The
// plane's pass-0 features are staged as bytes (f0, 255 = none); pass 1
// writes packed (f0 | f1 << 8) uint16 features (0xFFFF = none) to a second
// shared-memory plane, which pass 2 reads row by row; only the final
// outputs go to global memory.  Same windows, widening, tie rules and
// envelope fallbacks as edt_c1_kernel / edt_c2_kernel.
constexpr int kC12Threads = 256;
constexpr int kC12Warps = kC12Threads / 32;
constexpr int kC12Cols = 128;  // pass-1 columns per group (2 threads per column)
constexpr int kC12PadTop = kNear1;
constexpr int kC12PadBot = kNear1 + kQB;
constexpr int kC12PadX = 4;
constexpr uint8_t kNoF0 = 255;
constexpr uint16_t kNoF01 = 0xFFFF;
// Widest window radius of the fused passes before a line takes its exact envelope:
// the items reaching these passes are mostly sparse, where wider windows cost
// O(radius) per voxel while the envelope costs O(1).
constexpr int kC12Far = 8;

struct C12Smem {
    int L1, L2, rowp;  // rowp: padded pass-2 row length (row rounded up to 4 voxels + both pads)
    size_t tab, f0s, p1, stk, flag, rflag, total;
};

// The envelope stacks of the fallbacks (sparse backgrounds) live in one
// shared region, used first by the pass-1 columns (L1 entries per column,
// interleaved over the 128 columns of a group) and then by the pass-2 rows
// (W entries per row, interleaved over the L1 rows).
__host__ __device__ inline C12Smem c12_smem(int L1, int L2) {
    C12Smem m;
    m.L1 = L1;
    m.L2 = L2;
    m.rowp = (L2 + 3) / 4 * 4 + 2 * kC12PadX;
    size_t off = 0;
    m.tab = off;
    off += kSqrtTab * 4;
    m.f0s = off;
    off += ((size_t)(L1 + kC12PadTop + kC12PadBot) * L2 + 15) / 16 * 16;
    m.p1 = off;
    off += ((size_t)L1 * m.rowp * 2 + 15) / 16 * 16;
    m.stk = off;
    const size_t col_stack = (size_t)L1 * kC12Cols * 2, row_stack = (size_t)L1 * L2 * 2;
    off += ((col_stack > row_stack ? col_stack : row_stack) + 15) / 16 * 16;
    m.flag = off;
    off += (size_t)kC12Cols * 4;
    m.rflag = off;
    off += ((size_t)L1 * 4 + 15) / 16 * 16;
    m.total = off;
    return m;
}

// One (L1 x W) plane of the fused passes 1 + 2: the plane's pass-0 features
// start at c1 + plane and its outputs at plane in each output (index planes
// `numel` apart); z is the plane's axis-0 coordinate.  VEC: W % 4 == 0 and
// 16-byte aligned planes (8-byte loads, 16-byte stores); otherwise every
// access is scalar, for items packed at any offset.
template <bool VEC>
__device__ __forceinline__ void edt_c12_plane(const int64_t plane, const int z, const int L1, const int W,
                                              const int64_t numel, const int16_t *__restrict__ c1,
                                              float *__restrict__ dist, int32_t *__restrict__ indices,
                                              int32_t *__restrict__ sqdist) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const C12Smem sm = c12_smem(L1, W);
    float *tab = reinterpret_cast<float *>(smem_raw + sm.tab);
    uint8_t *f0s = smem_raw + sm.f0s + kC12PadTop * W;  // row y at f0s + y * W, y in -4 .. L1+11
    uint16_t *p1 = reinterpret_cast<uint16_t *>(smem_raw + sm.p1);  // row y at p1 + y * rowp + kC12PadX
    int16_t *stk = reinterpret_cast<int16_t *>(smem_raw + sm.stk);
    int *colflag = reinterpret_cast<int *>(smem_raw + sm.flag);
    int *rowflag = reinterpret_cast<int *>(smem_raw + sm.rflag);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rowp = sm.rowp, padr = rowp - kC12PadX - W;  // right padding: kC12PadX + round-up
    for (int i = tid; i < kSqrtTab; i += kC12Threads) tab[i] = __fsqrt_rn((float)i);
    // padding: "no site" rows around the f0 plane and columns around each p1 row
    for (int i = tid; i < (kC12PadTop + kC12PadBot) * W; i += kC12Threads) {
        const int r = i / W, c = i % W;
        const int y = r < kC12PadTop ? r - kC12PadTop : L1 + r - kC12PadTop;
        f0s[y * W + c] = kNoF0;
    }
    for (int i = tid; i < L1 * (kC12PadX + padr); i += kC12Threads) {
        const int y = i / (kC12PadX + padr), k = i % (kC12PadX + padr);
        p1[y * rowp + (k < kC12PadX ? k : kC12PadX + W + (k - kC12PadX))] = kNoF01;
    }
    if (VEC) {  // stage the pass-0 features of the plane as bytes, 4 per lane per row
        for (int i = tid; i < L1 * (W / 4); i += kC12Threads) {
            const int y = i / (W / 4), c4 = i % (W / 4);
            const short4 v = *reinterpret_cast<const short4 *>(c1 + plane + (int64_t)y * W + 4 * c4);
            const uint32_t b0 = v.x < 0 ? kNoF0 : (uint32_t)v.x, b1 = v.y < 0 ? kNoF0 : (uint32_t)v.y;
            const uint32_t b2 = v.z < 0 ? kNoF0 : (uint32_t)v.z, b3 = v.w < 0 ? kNoF0 : (uint32_t)v.w;
            reinterpret_cast<uint32_t *>(f0s + y * W)[c4] = b0 | (b1 << 8) | (b2 << 16) | (b3 << 24);
        }
    } else {
        // (L2 loads: in the ragged launch other SMs wrote these features after
        // a grid barrier, so no L1 line may serve them)
        for (int i = tid; i < L1 * W; i += kC12Threads) {
            const int16_t v = __ldcg(c1 + plane + i);
            f0s[i] = v < 0 ? kNoF0 : (uint8_t)v;
        }
    }
    __syncthreads();

    // ---- pass 1: columns along axis 1, 2 threads per column
    for (int xg = 0; xg < W; xg += kC12Cols) {
        const int xl = tid % kC12Cols, seg = tid / kC12Cols;
        const int x = xg + xl;
        const uint8_t *fcol = f0s + x;
        auto G1 = [&](int pp) -> uint32_t {
            const int f = fcol[pp * W];
            return f == kNoF0 ? kBig : (uint32_t)((z - f) * (z - f));
        };
        bool fallback = false;
        if (tid < kC12Cols) colflag[tid] = 0;
        __syncthreads();
        if (x < W) {
            const int qa = seg * L1 / 2, qb = (seg + 1) * L1 / 2;
            constexpr int NW = kQB + 2 * kNear1;
            for (int q0 = qa; q0 < qb && !fallback; q0 += kQB) {
                uint32_t w[NW];
#pragma unroll
                for (int j = 0; j < NW; j++) {
                    const int f = fcol[(q0 - kNear1 + j) * W];
                    w[j] = (f == kNoF0 ? kBig : (uint32_t)((z - f) * (z - f))) << kKeyShift;
                }
#pragma unroll
                for (int i = 0; i < kQB; i++) {
                    const int q = q0 + i;
                    if (q < qb && !fallback) {
                        const uint32_t key = window_key<kNear1>(w + i);
                        uint32_t best = key >> kKeyShift;
                        int bp = q - kNear1 + (int)(key & 31u);
                        if (best >= (kNear1 + 1) * (kNear1 + 1) && !widen<kNear1>(q, L1, G1, best, bp, kC12Far)) {
                            fallback = true;
                        } else {
                            p1[q * rowp + kC12PadX + x] =
                                best >= kBig ? kNoF01 : (uint16_t)(fcol[bp * W] | (bp << 8));
                        }
                    }
                }
            }
        }
        if (fallback) colflag[xl] = 1;
        __syncthreads();
        if (seg == 0 && x < W && colflag[xl]) {
            // exact lower envelope of the column, stack in shared memory
            // (entry k of column xl at stk[k * kC12Cols + xl])
            int16_t *cst = stk + xl;
            int k = -1, top = 0, sec = 0;
            int32_t Gtop = 0, Gsec = 0;
            for (int q = 0; q < L1; q++) {
                const uint32_t gq = G1(q);
                if (gq >= kBig) continue;
                const int32_t Gq = (int32_t)gq + q * q;
                while (k >= 1) {
                    const long long lhs = (long long)(Gq - Gtop) * (top - sec);
                    const long long rhs = (long long)(Gtop - Gsec) * (q - top);
                    if (lhs > rhs) break;
                    k--;
                    top = sec;
                    Gtop = Gsec;
                    if (k >= 1) {
                        sec = cst[(k - 1) * kC12Cols];
                        Gsec = (int32_t)G1(sec) + sec * sec;
                    }
                }
                k++;
                cst[k * kC12Cols] = (int16_t)q;
                sec = top;
                Gsec = Gtop;
                top = q;
                Gtop = Gq;
            }
            if (k < 0) {
                for (int q = 0; q < L1; q++) p1[q * rowp + kC12PadX + x] = kNoF01;
            } else {
                int j = 0, cur = cst[0], nxt = 0;
                uint32_t gcur = G1(cur), gnxt = 0;
                if (k >= 1) {
                    nxt = cst[kC12Cols];
                    gnxt = G1(nxt);
                }
                for (int q = 0; q < L1; q++) {
                    uint32_t fc = (uint32_t)((q - cur) * (q - cur)) + gcur;
                    while (j < k) {
                        const uint32_t fn = (uint32_t)((q - nxt) * (q - nxt)) + gnxt;
                        if (!(fn < fc)) break;
                        j++;
                        cur = nxt;
                        gcur = gnxt;
                        fc = fn;
                        if (j < k) {
                            nxt = cst[(j + 1) * kC12Cols];
                            gnxt = G1(nxt);
                        }
                    }
                    p1[q * rowp + kC12PadX + x] = (uint16_t)(fcol[cur * W] | (cur << 8));
                }
            }
        }
        __syncthreads();
    }

    // ---- pass 2: rows along axis 2, one warp per row, 4 voxels per lane
    for (int i = tid; i < L1; i += kC12Threads) rowflag[i] = 0;
    __syncthreads();
    for (int y = warp; y < L1; y += kC12Warps) {
        const uint16_t *row = p1 + y * rowp + kC12PadX;
        auto dec = [&](uint32_t f) -> uint32_t {
            if (f == kNoF01) return kBig;
            const int f0 = (int)(f & 255u), f1 = (int)(f >> 8);
            return (uint32_t)((z - f0) * (z - f0) + (y - f1) * (y - f1));
        };
        auto G2 = [&](int pp) { return dec(row[pp]); };
        const int64_t base = plane + (int64_t)y * W;
        bool any = false;
        for (int q = lane; q < W; q += 32) any |= row[q] != kNoF01;
        any = __any_sync(0xffffffffu, any);
        if (!any) {
            // no background anywhere in the item: virtual site (-1, 0, 0)
            for (int q = lane; q < W; q += 32) {
                const int64_t gi = base + q;
                const uint32_t s2 = (uint32_t)((z + 1) * (z + 1) + y * y + q * q);
                if (dist) dist[gi] = dist_of(s2, tab);
                if (sqdist) sqdist[gi] = (int32_t)s2;
                if (indices) {
                    indices[gi] = -1;
                    indices[numel + gi] = 0;
                    indices[2 * numel + gi] = 0;
                }
            }
            continue;
        }
        bool fallback = false;
        for (int c = 0; c < W && !fallback; c += 128) {
            const int q0 = c + 4 * lane;
            if (q0 >= W) break;
            uint32_t w[12];  // shifted g at q0-4 .. q0+7
            uint32_t fv[12];
#pragma unroll
            for (int j = 0; j < 12; j++) {
                fv[j] = row[q0 - 4 + j];
                w[j] = dec(fv[j]) << kKeyShift;
            }
            float dv[4];
            int32_t i0[4], i1[4], i2[4], sq[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int q = q0 + i;
                const uint32_t key = window_key<kNear2>(w + i + 2);
                uint32_t best = key >> kKeyShift;
                int bp = q - kNear2 + (int)(key & 31u);
                // (VEC: q < W always; otherwise the round-up positions have no site
                // and are neither searched nor written)
                if (q < W && best >= (kNear2 + 1) * (kNear2 + 1) && !widen<kNear2>(q, W, G2, best, bp, kC12Far))
                    fallback = true;
                const uint32_t f = row[bp];
                dv[i] = dist_of(best, tab);
                sq[i] = (int32_t)best;
                i0[i] = (int32_t)(f & 255u);
                i1[i] = (int32_t)(f >> 8);
                i2[i] = bp;
            }
            if (fallback) break;
            const int64_t gi = base + q0;
            if (VEC) {
                if (dist) *reinterpret_cast<float4 *>(dist + gi) = make_float4(dv[0], dv[1], dv[2], dv[3]);
                if (sqdist) *reinterpret_cast<int4 *>(sqdist + gi) = make_int4(sq[0], sq[1], sq[2], sq[3]);
                if (indices) {
                    *reinterpret_cast<int4 *>(indices + gi) = make_int4(i0[0], i0[1], i0[2], i0[3]);
                    *reinterpret_cast<int4 *>(indices + numel + gi) = make_int4(i1[0], i1[1], i1[2], i1[3]);
                    *reinterpret_cast<int4 *>(indices + 2 * numel + gi) = make_int4(i2[0], i2[1], i2[2], i2[3]);
                }
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    if (q0 + i >= W) break;
                    if (dist) dist[gi + i] = dv[i];
                    if (sqdist) sqdist[gi + i] = sq[i];
                    if (indices) {
                        indices[gi + i] = i0[i];
                        indices[numel + gi + i] = i1[i];
                        indices[2 * numel + gi + i] = i2[i];
                    }
                }
            }
        }
        if (__any_sync(0xffffffffu, fallback) && lane == 0) rowflag[y] = 1;
    }
    __syncthreads();
    // rows the windows could not finish (sparse backgrounds): every thread builds
    // the exact lower envelope of one row (entry k of row y at stk[k * L1 + y]);
    // rowflag becomes 2 + the index of the top entry
    if (tid < L1 && rowflag[tid]) {
        const int y = tid;
        const uint16_t *row = p1 + y * rowp + kC12PadX;
        auto G2 = [&](int pp) -> uint32_t {
            const uint32_t f = row[pp];
            if (f == kNoF01) return kBig;
            const int f0 = (int)(f & 255u), f1 = (int)(f >> 8);
            return (uint32_t)((z - f0) * (z - f0) + (y - f1) * (y - f1));
        };
        int16_t *rst = stk + y;
        int k = -1, top = 0, sec = 0;
        int32_t Gtop = 0, Gsec = 0;
        for (int q = 0; q < W; q++) {
            const uint32_t gq = G2(q);
            if (gq >= kBig) continue;
            const int32_t Gq = (int32_t)gq + q * q;
            while (k >= 1) {
                const long long lhs = (long long)(Gq - Gtop) * (top - sec);
                const long long rhs = (long long)(Gtop - Gsec) * (q - top);
                if (lhs > rhs) break;
                k--;
                top = sec;
                Gtop = Gsec;
                if (k >= 1) {
                    sec = rst[(k - 1) * L1];
                    Gsec = (int32_t)G2(sec) + sec * sec;
                }
            }
            k++;
            rst[k * L1] = (int16_t)q;
            sec = top;
            Gsec = Gtop;
            top = q;
            Gtop = Gq;
        }
        rowflag[y] = 2 + k;  // flagged rows have a site: k >= 0
    }
    __syncthreads();
    // outputs of those rows: one warp per row, every lane searches the envelope
    for (int y = warp; y < L1; y += kC12Warps) {
        const int flag = rowflag[y];
        if (flag < 2) continue;
        const int ktop = flag - 2;
        const uint16_t *row = p1 + y * rowp + kC12PadX;
        auto G2 = [&](int pp) -> uint32_t {
            const uint32_t f = row[pp];
            if (f == kNoF01) return kBig;
            const int f0 = (int)(f & 255u), f1 = (int)(f >> 8);
            return (uint32_t)((z - f0) * (z - f0) + (y - f1) * (y - f1));
        };
        const int16_t *rst = stk + y;
        const int64_t base = plane + (int64_t)y * W;
        for (int q = lane; q < W; q += 32) {
            int lo = 0, hi = ktop;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                const int a = rst[(mid - 1) * L1], b = rst[mid * L1];
                const uint32_t fa = (uint32_t)((q - a) * (q - a)) + G2(a);
                const uint32_t fb = (uint32_t)((q - b) * (q - b)) + G2(b);
                if (fb < fa)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int bp = rst[lo * L1];
            const uint32_t best = (uint32_t)((q - bp) * (q - bp)) + G2(bp);
            const uint32_t f = row[bp];
            const int64_t gi = base + q;
            if (dist) dist[gi] = dist_of(best, tab);
            if (sqdist) sqdist[gi] = (int32_t)best;
            if (indices) {
                indices[gi] = (int32_t)(f & 255u);
                indices[numel + gi] = (int32_t)(f >> 8);
                indices[2 * numel + gi] = bp;
            }
        }
    }
}

// Grid-stride over planes: with per-item flags (after the shell search) the
// grid is one resident wave, so items the search finished cost one flag
// read per plane.
__global__ void __launch_bounds__(kC12Threads, 3) edt_c12_kernel(const int16_t *__restrict__ c1, float *__restrict__ dist,
                                                              int32_t *__restrict__ indices,
                                                              int32_t *__restrict__ sqdist, CompactParams p,
                                                              const int *__restrict__ todo) {
    // Launched behind pass 0, which lets this grid be scheduled once the shell
    // search has completed: the flags are final here (read through L2), and a
    // block waits for pass 0's features only when it has a plane to compute.
    const int64_t nblk = p.batch * (int64_t)p.L0;
    bool waited = false;
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const int64_t item = blk / p.L0;
        if (todo && !__ldcg(todo + item)) continue;  // item finished by the shell pass
        if (!waited) {
            pdl_wait();  // pass 0's features are complete
            waited = true;
        }
        const int z = (int)(blk - item * p.L0);
        edt_c12_plane<true>(item * p.numel_item + (int64_t)z * p.L1 * p.L2, z, p.L1, p.L2, p.numel, c1, dist, indices,
                            sqdist);
        __syncthreads();  // the next plane reuses shared memory
    }
}

// ------------------------------------------- ragged batches of 3-D items
// The fused plane passes over a ragged batch (items packed at any offset,
// every axis at most kRaggedC12MaxLine): one cooperative launch whose first
// phase runs pass 0 over the axis-0 columns of every item (one thread per
// column, adjacent threads on adjacent columns: coalesced), and whose second
// phase, after a bounded grid barrier, gives the planes of all items to the
// CTAs in turn (edt_c12_plane with scalar accesses).
constexpr int kRaggedC12MaxLine = 180;  // the plane code's shared memory stays below 170 KB

struct RaggedC12Args {
    const void *in;
    int in_f32;
    int nitems;
    const ReItem *items;
    int64_t cols, total;
    int16_t *c1;
    float *dist;
    int32_t *indices, *sqdist;
    GridControl *ctl;
    int *status;
    long long spin_limit;
};

__global__ void __launch_bounds__(kC12Threads, 2) ragged_edt3_kernel(RaggedC12Args A) {
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const ReItem *items = A.items;
    // pass 0: the nearest background along axis 0 as its position (int16, -1:
    // none), ties to the lower position; input loads 8 deep per thread
    for (int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; col < A.cols; col += nthreads) {
        int lo = 0, hi = A.nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].line_begin[0] <= col) lo = mid;
            else hi = mid - 1;
        }
        const ReItem &it = items[lo];
        const int D = it.shape[0];
        const int64_t stride = (int64_t)it.shape[1] * it.shape[2];
        const int64_t base = it.off + (col - it.line_begin[0]);
        int prev = -1;
        for (int q0 = 0; q0 < D; q0 += 8) {
            bool bg[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int64_t p = base + (int64_t)(q0 + u) * stride;
                bg[u] = q0 + u < D && (A.in_f32 ? static_cast<const float *>(A.in)[p] == 0.0f
                                                : static_cast<const uint8_t *>(A.in)[p] == 0);
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                if (q0 + u >= D) break;
                if (bg[u]) prev = q0 + u;
                A.c1[base + (int64_t)(q0 + u) * stride] = (int16_t)prev;
            }
        }
        // backward: the first background after q replaces the forward result only when
        // strictly nearer (this thread's own stores, read back in program order)
        int next = -1;
        for (int q0 = ((D - 1) / 8) * 8; q0 >= 0; q0 -= 8) {
            int v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = q0 + u < D ? A.c1[base + (int64_t)(q0 + u) * stride] : -1;
#pragma unroll
            for (int u = 7; u >= 0; u--) {
                const int q = q0 + u;
                if (q >= D) continue;
                if (v[u] == q) next = q;
                else if (next >= 0 && (v[u] < 0 || next - q < q - v[u]))
                    A.c1[base + (int64_t)q * stride] = (int16_t)next;
            }
        }
    }
    if (!grid_barrier_bounded(A.ctl, gridDim.x, A.status, A.spin_limit)) return;
    // passes 1 + 2: one plane of one item per CTA at a time
    const ReItem &last = items[A.nitems - 1];
    const int64_t nplanes = (int64_t)last.plane_begin + last.shape[0];
    for (int64_t k = blockIdx.x; k < nplanes; k += gridDim.x) {
        int lo = 0, hi = A.nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].plane_begin <= k) lo = mid;
            else hi = mid - 1;
        }
        const ReItem &it = items[lo];
        const int z = (int)(k - it.plane_begin), H = it.shape[1], W = it.shape[2];
        edt_c12_plane<false>(it.off + (int64_t)z * H * W, z, H, W, A.total, A.c1, A.dist, A.indices, A.sqdist);
        __syncthreads();  // the next plane reuses shared memory
    }
}

// -------------------------------------------------------- shell search
// 3-D items whose voxels all have a background voxel within squared distance
// kShellD2 (dense backgrounds, e.g. 10 %): the answer is the first background
// offset in the list of all offsets with |d|^2 <= kShellD2 sorted by
// (|d|^2, dx, dy, dz) -- nearest first, ties to the smallest last-axis, then
// middle-axis, then first-axis coordinate, which is the separable passes'
// (scipy's) tie rule.  Background is kept as bitmaps (bit b of word w of a
// row = voxel 32 w + b), so one funnel shift tests an offset for 32 voxels.
// Voxels without a background within the radius mark their item; those
// items then run the separable passes (which skip every other item).
constexpr int kShellR = 4;
constexpr int kShellD2 = 16;
constexpr int kShellN = 257;  // offsets with |d|^2 <= 16
constexpr int kShellRows = 32;  // rows (axis 1) per CTA
constexpr int kShellThreads = 128;
// The offset list, packed (dz+8) | (dy+8) << 4 | (dx+8) << 8 | d2 << 12, built at
// compile time in list order (|d|^2, then dx, dy, dz ascending), so no launch
// depends on a host-side upload.
struct ShellTable {
    uint32_t v[kShellN];
};
constexpr ShellTable make_shell_table() {
    ShellTable t{};
    int n = 0;
    for (int d2 = 0; d2 <= kShellD2; d2++)
        for (int dx = -kShellR; dx <= kShellR; dx++)
            for (int dy = -kShellR; dy <= kShellR; dy++)
                for (int dz = -kShellR; dz <= kShellR; dz++)
                    if (dx * dx + dy * dy + dz * dz == d2 && n < kShellN)
                        t.v[n++] = (uint32_t)(dz + 8) | ((uint32_t)(dy + 8) << 4) | ((uint32_t)(dx + 8) << 8) |
                                   ((uint32_t)d2 << 12);
    return t;
}
constexpr int shell_count() {
    int n = 0;
    for (int dx = -kShellR; dx <= kShellR; dx++)
        for (int dy = -kShellR; dy <= kShellR; dy++)
            for (int dz = -kShellR; dz <= kShellR; dz++) n += dx * dx + dy * dy + dz * dz <= kShellD2;
    return n;
}
static_assert(shell_count() == kShellN, "offset list size");
__constant__ ShellTable c_shell = make_shell_table();

// Background bitmap, ceil(L2 / 32) words per row, one word per thread.  When
// rows are a multiple of 32 voxels (and the input 16-byte aligned) a word is
// read with 16-byte loads and the bytes tested four at a time.
__device__ __forceinline__ uint32_t zero_bytes4(uint32_t v) {
    // bit k set when byte k of v is zero
    const uint32_t m = __vcmpeq4(v, 0u);
    return ((m >> 7) & 1u) | ((m >> 14) & 2u) | ((m >> 21) & 4u) | ((m >> 28) & 8u);
}

template <typename In, bool VEC>
__global__ void __launch_bounds__(256) edt_bitmap_kernel(const In *__restrict__ in, uint32_t *__restrict__ bm,
                                                         CompactParams p, int ww, int64_t nwords,
                                                         int *__restrict__ clear, int nclear) {
    // the shell pass's per-item flags and work counter start at zero
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < nclear; i += blockDim.x) clear[i] = 0;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = w / ww;
        const int wi = (int)(w - row * ww);
        const In *src = in + row * p.L2 + 32 * wi;
        uint32_t bits = 0;
        if (VEC) {
            if (sizeof(In) == 1) {
                const uint4 a = reinterpret_cast<const uint4 *>(src)[0], b = reinterpret_cast<const uint4 *>(src)[1];
                const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
                for (int k = 0; k < 8; k++) bits |= zero_bytes4(v[k]) << (4 * k);
            } else {
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    const float4 f = reinterpret_cast<const float4 *>(src)[k];
                    bits |= ((uint32_t)(f.x == 0.f) | ((uint32_t)(f.y == 0.f) << 1) | ((uint32_t)(f.z == 0.f) << 2) |
                             ((uint32_t)(f.w == 0.f) << 3))
                            << (4 * k);
                }
            }
        } else {
            const int nb = min(32, p.L2 - 32 * wi);
            for (int b = 0; b < nb; b++) bits |= (uint32_t)(src[b] == (In)0) << b;
        }
        bm[w] = bits;
    }
}

struct ShellSmem {
    int ww, pitch, planep;  // words per row, padded words per row, words per padded plane
    size_t bits, res, tab, tab2, total;
};

// Padded bitmap rows: a zero word, the row's words, a zero word.
constexpr int kShellPadW = 1;

__host__ __device__ inline ShellSmem shell_smem(int L2) {
    ShellSmem m;
    m.ww = (L2 + 31) / 32;
    m.pitch = m.ww + 2 * kShellPadW;
    m.planep = (kShellRows + 2 * kShellR) * m.pitch;
    size_t off = 0;
    m.bits = off;
    off += (size_t)(2 * kShellR + 1) * m.planep * 4;
    m.res = off;
    off += ((size_t)kShellRows * L2 * 2 + 15) / 16 * 16;
    m.tab = off;
    off += (size_t)kShellN * 8;
    m.tab2 = off;
    off += (size_t)kShellN * 4;
    m.total = off;
    return m;
}

// One CTA: rows y0 .. y0+31 of plane z of one item.  Stage the bitmaps of
// planes z-4 .. z+4, rows y0-4 .. y0+35 (zero outside the item), search each
// 32-voxel word through the sorted offsets until all its voxels are
// resolved, then write distances / indices 4 voxels per thread.
__global__ void __launch_bounds__(kShellThreads) edt_shell_kernel(const uint32_t *__restrict__ bm,
                                                                  float *__restrict__ dist,
                                                                  int32_t *__restrict__ indices,
                                                                  int32_t *__restrict__ sqdist, int *__restrict__ todo,
                                                                  CompactParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    const ShellSmem sm = shell_smem(W);
    uint32_t *bits = reinterpret_cast<uint32_t *>(smem_raw + sm.bits);
    uint16_t *res = reinterpret_cast<uint16_t *>(smem_raw + sm.res);
    int2 *tab = reinterpret_cast<int2 *>(smem_raw + sm.tab);  // (word delta, shift | d2 << 8)
    uint32_t *tab2 = reinterpret_cast<uint32_t *>(smem_raw + sm.tab2);  // packed offsets
    __shared__ int s_unresolved;
    const int ybl = (L1 + kShellRows - 1) / kShellRows;
    const int64_t item = blockIdx.x / ((int64_t)L0 * ybl);
    const int rem = (int)(blockIdx.x - item * L0 * ybl);
    const int z = rem / ybl, y0 = (rem % ybl) * kShellRows;
    const int nrows = min(kShellRows, L1 - y0);
    const int ww = sm.ww, pitch = sm.pitch, planep = sm.planep;
    const int tid = threadIdx.x;
    if (tid == 0) s_unresolved = 0;
    for (int t = tid; t < kShellN; t += kShellThreads) {
        const uint32_t e = c_shell.v[t];
        const int dz = (int)(e & 15u) - 8, dy = (int)((e >> 4) & 15u) - 8, dx = (int)((e >> 8) & 15u) - 8;
        const int d2 = (int)(e >> 12);
        tab[t] = make_int2(dz * planep + dy * pitch + (dx >= 0 ? 0 : -1), (dx >= 0 ? dx : 32 + dx) | (d2 << 8));
        tab2[t] = e;
    }
    // stage bitmaps: plane k = z-4+k, padded row r = y0-4+r; zero outside the item
    const uint32_t *ibm = bm + item * (int64_t)L0 * L1 * ww;
    constexpr int kRowsP = kShellRows + 2 * kShellR;
    for (int i = tid; i < (2 * kShellR + 1) * kRowsP; i += kShellThreads) {
        const int k = i / kRowsP, r = i - k * kRowsP;
        const int zz = z - kShellR + k, yy = y0 - kShellR + r;
        uint32_t *dst = bits + k * planep + r * pitch;
        const bool in_item = (unsigned)zz < (unsigned)L0 && (unsigned)yy < (unsigned)L1;
        const uint32_t *src = ibm + ((int64_t)zz * L1 + yy) * ww;
        dst[0] = 0u;
        dst[kShellPadW + ww] = 0u;
        if ((ww & 3) == 0) {  // 16-byte global loads (rows of the bitmap are 16-byte aligned)
            for (int c = 0; c < ww; c += 4) {
                const uint4 v = in_item ? *reinterpret_cast<const uint4 *>(src + c) : make_uint4(0, 0, 0, 0);
                dst[kShellPadW + c] = v.x;
                dst[kShellPadW + c + 1] = v.y;
                dst[kShellPadW + c + 2] = v.z;
                dst[kShellPadW + c + 3] = v.w;
            }
        } else {
            for (int c = 0; c < ww; c++) dst[kShellPadW + c] = in_item ? src[c] : 0u;
        }
    }
    __syncthreads();
    // search: one 32-voxel word per thread
    const uint32_t *center = bits + kShellR * planep + kShellR * pitch + kShellPadW;  // (z, y0, word 0)
    for (int e = tid; e < nrows * ww; e += kShellThreads) {
        const int r = e / ww, wi = e % ww;
        const int nb = min(32, W - 32 * wi);
        uint32_t U = nb == 32 ? 0xffffffffu : ((1u << nb) - 1u);
        const uint32_t *here = center + r * pitch + wi;
        uint16_t *out = res + r * W + 32 * wi;
        // four offsets per step: their loads are independent, the hits are
        // applied in list order so earlier offsets keep priority
        for (int t = 0; t < kShellN && U; t += 4) {
            uint32_t bg[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                bg[k] = 0;
                if (t + k < kShellN) {
                    const int2 tb = tab[t + k];
                    bg[k] = __funnelshift_r(here[tb.x], here[tb.x + 1], tb.y & 31);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                uint32_t hit = bg[k] & U;
                if (hit) {
                    U &= ~hit;
                    do {
                        const int b = __ffs(hit) - 1;
                        out[b] = (uint16_t)(t + k);
                        hit &= hit - 1;
                    } while (hit);
                }
            }
        }
        if (U) {
            s_unresolved = 1;
            do {
                const int b = __ffs(U) - 1;
                out[b] = 0xFFFF;
                U &= U - 1;
            } while (U);
        }
    }
    __syncthreads();
    if (s_unresolved) {  // the separable passes redo this item
        if (tid == 0) atomicExch(&todo[item], 1);
        return;
    }
    // outputs: a warp per row, 4 consecutive voxels per lane (16-byte stores)
    const int64_t numel = p.numel;
    const int64_t rowbase = item * p.numel_item + ((int64_t)z * L1 + y0) * W;
    const int warp = tid >> 5, lane = tid & 31;
    for (int r = warp; r < nrows; r += kShellThreads / 32) {
        const uint16_t *rres = res + r * W;
        for (int x = 4 * lane; x < W; x += 128) {
            float dv[4];
            int32_t i0[4], i1[4], i2[4], sq[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t c = tab2[rres[x + k]];
                const uint32_t d2 = c >> 12;
                dv[k] = __fsqrt_rn((float)d2);
                sq[k] = (int32_t)d2;
                i0[k] = z + (int)(c & 15u) - 8;
                i1[k] = y0 + r + (int)((c >> 4) & 15u) - 8;
                i2[k] = x + k + (int)((c >> 8) & 15u) - 8;
            }
            const int64_t gi = rowbase + (int64_t)r * W + x;
            if (dist) *reinterpret_cast<float4 *>(dist + gi) = make_float4(dv[0], dv[1], dv[2], dv[3]);
            if (sqdist) *reinterpret_cast<int4 *>(sqdist + gi) = make_int4(sq[0], sq[1], sq[2], sq[3]);
            if (indices) {
                *reinterpret_cast<int4 *>(indices + gi) = make_int4(i0[0], i0[1], i0[2], i0[3]);
                *reinterpret_cast<int4 *>(indices + numel + gi) = make_int4(i1[0], i1[1], i1[2], i1[3]);
                *reinterpret_cast<int4 *>(indices + 2 * numel + gi) = make_int4(i2[0], i2[1], i2[2], i2[3]);
            }
        }
    }
}

// Compile-time variant for rows of WW words: the offsets, word deltas and
// shifts are constants, so the search is straight-line code with immediate
// shared-memory offsets (no table reads, no address arithmetic).
struct ShellOff {
    int dz, dy, dx, d2;
};

struct ShellList {
    ShellOff o[kShellN];
};

__host__ __device__ constexpr ShellList make_shell_list() {
    ShellList l{};
    int n = 0;
    for (int d2 = 0; d2 <= kShellD2; d2++)
        for (int dx = -kShellR; dx <= kShellR; dx++)
            for (int dy = -kShellR; dy <= kShellR; dy++)
                for (int dz = -kShellR; dz <= kShellR; dz++)
                    if (dz * dz + dy * dy + dx * dx == d2) l.o[n++] = ShellOff{dz, dy, dx, d2};
    return l;
}

// Nearest background of voxel (z, y, x) of one item beyond the radius-4
// shell (none with |d|^2 <= 16; near the item's faces the shell is cut
// off).  All 32 lanes of the warp search the cube of Chebyshev radius R on
// the background bitmap, R = 6, 13, 27, ... until the best squared distance
// is below (R + 1)^2 (nothing outside the cube can be nearer or tie) or the
// cube covers the item.  Per row (dz, dy) only the nearest background bit on
// each side of x can be the row's best.  Among equal squared distances the
// smallest axis-2 coordinate wins, then axis 1, then axis 0 -- the order of
// the shell list (|d|^2, dx, dy, dz), which is the separable passes' tie
// rule (each pass keeps the lower coordinate).  Returns
// (d2 << 24) | (x' << 16) | (y' << 8) | z', or ~0 if the item has no background.
__device__ unsigned long long far_search(const uint32_t *__restrict__ ibm, int z, int y, int x, int L0, int L1, int W,
                                         int lane) {
    constexpr int WW = 4;
    unsigned long long best = ~0ull;
    for (int R = 6;; R = 2 * R + 1) {
        const int side = 2 * R + 1;
        const int xl = max(0, x - R), xr = min(W - 1, x + R);
        for (int k = lane; k < side * side; k += 32) {
            const int dz = k / side - R, dy = k % side - R;
            const int zz = z + dz, yy = y + dy;
            if ((unsigned)zz >= (unsigned)L0 || (unsigned)yy >= (unsigned)L1) continue;
            const unsigned rowd2 = (unsigned)(dz * dz + dy * dy);
            if (((unsigned long long)rowd2 << 24) >= best) continue;
            const uint32_t *row = ibm + ((int64_t)zz * L1 + yy) * WW;
            for (int w = x >> 5; w >= (xl >> 5); w--) {  // nearest background at x' <= x
                uint32_t m = row[w];
                if (w == (x >> 5)) m &= (x & 31) == 31 ? 0xffffffffu : ((2u << (x & 31)) - 1u);
                if (w == (xl >> 5)) m &= ~((1u << (xl & 31)) - 1u);
                if (m) {
                    const int xp = 32 * w + 31 - __clz(m);
                    const unsigned d2 = rowd2 + (unsigned)((x - xp) * (x - xp));
                    const unsigned long long key =
                        ((unsigned long long)d2 << 24) | ((unsigned)xp << 16) | ((unsigned)yy << 8) | (unsigned)zz;
                    best = key < best ? key : best;
                    break;
                }
            }
            if (x < xr)
                for (int w = (x + 1) >> 5; w <= (xr >> 5); w++) {  // nearest background at x' > x
                    uint32_t m = row[w];
                    if (w == ((x + 1) >> 5)) m &= ~((1u << ((x + 1) & 31)) - 1u);
                    if (w == (xr >> 5)) m &= (xr & 31) == 31 ? 0xffffffffu : ((2u << (xr & 31)) - 1u);
                    if (m) {
                        const int xp = 32 * w + __ffs(m) - 1;
                        const unsigned d2 = rowd2 + (unsigned)((xp - x) * (xp - x));
                        const unsigned long long key =
                            ((unsigned long long)d2 << 24) | ((unsigned)xp << 16) | ((unsigned)yy << 8) | (unsigned)zz;
                        best = key < best ? key : best;
                        break;
                    }
                }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(~0u, best, o);
            best = other < best ? other : best;
        }
        const bool covers =
            z - R <= 0 && z + R >= L0 - 1 && y - R <= 0 && y + R >= L1 - 1 && x - R <= 0 && x + R >= W - 1;
        if ((best >> 24) < (unsigned long long)(R + 1) * (R + 1) || covers) return best;
    }
}

// Shell search with the offset list unrolled at compile time, for rows of
// WW = 4 words (97..128 voxels).  Each warp works alone on units of 8 rows
// of one plane taken from a work queue: it stages the background words the
// offsets reach (9 planes x 16 rows), searches one word per lane, and writes
// the unit's outputs itself.  Warps synchronise only within themselves, so
// on one SM some warps write while others stage or search.
constexpr int kShellCtWarps = 4;
constexpr unsigned kFarPerUnit = 32;  // voxels beyond the shell searched per 8-row unit at most
constexpr int kShellCtThreads = 32 * kShellCtWarps;
constexpr int kShellWarpRows = 8;                        // rows per warp unit (8 rows x 4 words = 32 lanes)
constexpr int kSwRowsP = kShellWarpRows + 2 * kShellR;   // 16 staged rows per plane
constexpr int kSwStageRows = (2 * kShellR + 1) * kSwRowsP;  // 144
// Staged rows are the 4 words of the bitmap row with no padding: the 32 lanes
// of a warp (8 rows x 4 words) read 32 consecutive words -- conflict-free --
// and a lane masks the word left of word 0 and right of word 3 itself.
constexpr int kCwPlane = kSwRowsP * 4;                  // 64 words per staged plane
constexpr int kCwWords = (2 * kShellR + 1) * kCwPlane;  // 576

template <int WW>
__global__ void __launch_bounds__(kShellCtThreads) edt_shell_ct_kernel(const uint32_t *__restrict__ bm,
                                                                       float *__restrict__ dist,
                                                                       int32_t *__restrict__ indices,
                                                                       int32_t *__restrict__ sqdist,
                                                                       int *__restrict__ todo, CompactParams p) {
    static_assert(WW == 4, "rows of four words (97..128 voxels)");
    static_assert(kShellWarpRows * WW == 32, "one word per lane");
    constexpr ShellList kL = make_shell_list();
    constexpr int kStageIters = (kSwStageRows + 31) / 32;
    // 4 words before and after the staged planes: the masked neighbour reads of
    // the first and last rows stay inside the array
    __shared__ __align__(16) uint32_t bits_all[kShellCtWarps][kCwWords + 8];
    // per word: bit-planes 0..8 of the resolving offset number (12 words, 16-byte aligned)
    __shared__ __align__(16) uint32_t planes_all[kShellCtWarps][32 * 12];
    __shared__ int2 tab2[kShellN];  // (packed offset, distance as float bits)
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    const int ybl = (L1 + kShellWarpRows - 1) / kShellWarpRows;
    const int64_t nunits = p.batch * (int64_t)L0 * ybl;
    // 64-bit work counter after the per-item flags (8-byte aligned), zeroed with them
    unsigned long long *queue = reinterpret_cast<unsigned long long *>(todo + ((p.batch + 1) & ~(int64_t)1));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *bits = bits_all[warp] + 4;
    uint32_t *planes = planes_all[warp];
    pdl_trigger();  // the fallback passes may be scheduled as this grid's CTAs retire
    for (int t = threadIdx.x; t < kShellN; t += kShellCtThreads) {
        const uint32_t c = c_shell.v[t];
        tab2[t] = make_int2((int)c, __float_as_int(__fsqrt_rn((float)(c >> 12))));
    }
    if (lane < 4) bits[-4 + lane] = 0u;
    else if (lane < 8) bits[kCwWords + lane - 4] = 0u;
    __syncthreads();
    pdl_wait();  // the background bitmap and the zeroed flags / counter are complete
    const int64_t numel = p.numel;
    for (;;) {
        int64_t unit = 0;
        if (lane == 0) unit = (int64_t)atomicAdd(queue, 1ull);
        unit = __shfl_sync(~0u, unit, 0);
        if (unit >= nunits) break;
        const int64_t item = unit / ((int64_t)L0 * ybl);
        const int rem = (int)(unit - item * L0 * ybl);
        const int z = rem / ybl, y0 = (rem % ybl) * kShellWarpRows;
        const int nrows = min(kShellWarpRows, L1 - y0);
        const uint32_t *ibm = bm + item * (int64_t)L0 * L1 * WW;
        // stage: every load of the lane before any store
        uint4 v[kStageIters];
#pragma unroll
        for (int j = 0; j < kStageIters; j++) {
            const int i = lane + 32 * j;
            const int kk = i / kSwRowsP, r = i - kk * kSwRowsP;
            const int zz = z - kShellR + kk, yy = y0 - kShellR + r;
            const bool ok = i < kSwStageRows && (unsigned)zz < (unsigned)L0 && (unsigned)yy < (unsigned)L1;
            v[j] = ok ? *reinterpret_cast<const uint4 *>(ibm + ((int64_t)zz * L1 + yy) * WW) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int j = 0; j < kStageIters; j++) {
            const int i = lane + 32 * j;
            if (i < kSwStageRows) reinterpret_cast<uint4 *>(bits)[i] = v[j];  // row i = plane i / 16, row i % 16
        }
        __syncwarp();
        // search: lane = word (row lane / 4, word lane % 4).  The offset number
        // t = 8 * batch + i resolving each voxel is kept as bit-planes P[0..8]
        // of the word: per batch, f_i = the voxels whose first background
        // offset is the batch's i-th (earlier offsets keep priority), then
        // planes 0-2 take the bits of i and planes 3-8 the batch number.
        uint32_t U = 0u;
        {
            const int r = lane >> 2, wi = lane & 3;
            const int nb = min(32, W - 32 * wi);
            if (r < nrows) U = nb == 32 ? 0xffffffffu : ((1u << nb) - 1u);
            const volatile uint32_t *vhere = bits + kShellR * kCwPlane + (kShellR + r) * 4 + wi;
            // neighbour words are always inside the staged array (pads at both ends);
            // these masks zero the words left of word 0 and right of word 3
            const uint32_t ml = wi != 0 ? ~0u : 0u, mr = wi != WW - 1 ? ~0u : 0u;
            uint32_t P[9] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
            constexpr int kB = 8;
#pragma unroll
            for (int t0 = 0; t0 < kShellN; t0 += kB) {
                if (U == 0u) break;
                uint32_t bg[kB];
                uint32_t any = 0;
#pragma unroll
                for (int i = 0; i < kB; i++) {
                    const int t = t0 + i < kShellN ? t0 + i : kShellN - 1;
                    const int d = kL.o[t].dz * kCwPlane + kL.o[t].dy * 4, dx = kL.o[t].dx;
                    // volatile: each batch's loads stay behind its exit test
                    uint32_t b = 0u;
                    if (t0 + i < kShellN) {
                        if (dx == 0) b = vhere[d];
                        else if (dx > 0) b = __funnelshift_r(vhere[d], vhere[d + 1] & mr, dx);
                        else b = __funnelshift_r(vhere[d - 1] & ml, vhere[d], 32 + dx);
                    }
                    bg[i] = b;
                    any |= bg[i];
                }
                const uint32_t H = any & U;  // resolved in this batch
                U &= ~H;
                uint32_t rem = H, f[kB];
#pragma unroll
                for (int i = 0; i < kB; i++) {
                    f[i] = bg[i] & rem;
                    rem &= ~bg[i];
                }
                P[0] |= f[1] | f[3] | f[5] | f[7];
                P[1] |= f[2] | f[3] | f[6] | f[7];
                P[2] |= f[4] | f[5] | f[6] | f[7];
                const int bi = t0 / kB;  // a constant once the loop is unrolled
#pragma unroll
                for (int j = 0; j < 6; j++)
                    if ((bi >> j) & 1) P[3 + j] |= H;
            }
            uint4 *pw = reinterpret_cast<uint4 *>(planes + lane * 12);
            pw[0] = make_uint4(P[0], P[1], P[2], P[3]);
            pw[1] = make_uint4(P[4], P[5], P[6], P[7]);
            pw[2] = make_uint4(P[8], 0u, 0u, 0u);
        }
        const unsigned nfar = __reduce_add_sync(~0u, (unsigned)__popc(U));  // voxels beyond the shell
        if (nfar > kFarPerUnit) {  // many: the item takes the separable passes
            if (lane == 0) atomicExch(&todo[item], 1);
            continue;
        }
        __syncwarp();
        // write: lane = 4 consecutive voxels of a row
        const int64_t rowbase = item * p.numel_item + ((int64_t)z * L1 + y0) * W;
        const int x = 4 * lane;
        if (x < W) {
            const int b = x & 31;
            for (int r = 0; r < nrows; r++) {
                float dv[4];
                int32_t i0[4], i1[4], i2[4], sq[4];
                // offset numbers of voxels x..x+3 from the word's bit-planes:
                // a plane's nibble spread to one bit per byte, bytes = t & 255
                const uint4 *pw = reinterpret_cast<const uint4 *>(planes + (r * 4 + (x >> 5)) * 12);
                const uint4 qa = pw[0], qb = pw[1];
                const uint32_t p8 = planes[(r * 4 + (x >> 5)) * 12 + 8];
                const uint32_t pl[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
                uint32_t acc = 0u;
#pragma unroll
                for (int j = 0; j < 8; j++) acc += ((((pl[j] >> b) & 15u) * 0x00204081u) & 0x01010101u) << j;
                const uint32_t hi = (((p8 >> b) & 15u) * 0x00204081u) & 0x01010101u;
                int tt[4];
#pragma unroll
                for (int q = 0; q < 4; q++) tt[q] = (int)(((acc >> (8 * q)) & 255u) | (((hi >> (8 * q)) & 1u) << 8));
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int2 e = tab2[tt[q]];
                    const uint32_t c = (uint32_t)e.x;
                    dv[q] = __int_as_float(e.y);
                    sq[q] = (int32_t)(c >> 12);
                    i0[q] = z + (int)(c & 15u) - 8;
                    i1[q] = y0 + r + (int)((c >> 4) & 15u) - 8;
                    i2[q] = x + q + (int)((c >> 8) & 15u) - 8;
                }
                // streaming stores: the outputs are not read again by this call
                const int64_t gi = rowbase + (int64_t)r * W + x;
                if (dist) __stcs(reinterpret_cast<float4 *>(dist + gi), make_float4(dv[0], dv[1], dv[2], dv[3]));
                if (sqdist) __stcs(reinterpret_cast<int4 *>(sqdist + gi), make_int4(sq[0], sq[1], sq[2], sq[3]));
                if (indices) {
                    __stcs(reinterpret_cast<int4 *>(indices + gi), make_int4(i0[0], i0[1], i0[2], i0[3]));
                    __stcs(reinterpret_cast<int4 *>(indices + numel + gi), make_int4(i1[0], i1[1], i1[2], i1[3]));
                    __stcs(reinterpret_cast<int4 *>(indices + 2 * numel + gi), make_int4(i2[0], i2[1], i2[2], i2[3]));
                }
            }
        }
        if (nfar) {
            // the few voxels beyond the shell: searched by the whole warp, written
            // after the unit's stores above (ordered by the warp barrier)
            __syncwarp();
            for (unsigned has = __ballot_sync(~0u, U != 0u); has; has &= has - 1) {
                const int src = __ffs(has) - 1;
                for (uint32_t m = __shfl_sync(~0u, U, src); m; m &= m - 1) {
                    const int yv = y0 + (src >> 2), xv = 32 * (src & 3) + __ffs(m) - 1;
                    const unsigned long long best = far_search(ibm, z, yv, xv, L0, L1, W, lane);
                    if (lane != 0) continue;
                    if (best == ~0ull) {  // no background in the item
                        atomicExch(&todo[item], 1);
                        continue;
                    }
                    const unsigned d2 = (unsigned)(best >> 24);
                    const int64_t gi = rowbase + (int64_t)(yv - y0) * W + xv;
                    if (dist) dist[gi] = __fsqrt_rn((float)d2);
                    if (sqdist) sqdist[gi] = (int32_t)d2;
                    if (indices) {
                        indices[gi] = (int32_t)(best & 255u);
                        indices[numel + gi] = (int32_t)((best >> 8) & 255u);
                        indices[2 * numel + gi] = (int32_t)((best >> 16) & 255u);
                    }
                }
            }
        }
        __syncwarp();  // res and bits are free for the next unit
    }
}

// ------------------------------------------------- chamfer, distances only
// The chamfer distances of scipy's two-pass raster transform are the
// minimum over background voxels b of a norm of (voxel - b) (monotone
// paths stay inside the box): chessboard max|d|, taxicab sum|d|, 3-4-5
// 3a + b + c for |d| sorted a >= b >= c (in thirds).  For distances only,
// the offsets of the radius-4 cube with norm <= kCdtVmax(metric) are grouped
// by norm; per 32-voxel word the union of a class's shifted background
// masks resolves every voxel whose nearest background has that norm.  The
// few voxels left (nearest background beyond the class bound) are searched
// on the bitmap; a unit with many of them marks its item for the raster
// passes.
__host__ __device__ constexpr int cdt_norm(int metric, int dz, int dy, int dx) {
    int a = dz < 0 ? -dz : dz, b = dy < 0 ? -dy : dy, c = dx < 0 ? -dx : dx;
    if (metric == 0) return a > b ? (a > c ? a : c) : (b > c ? b : c);  // chessboard
    if (metric == 1) return a + b + c;                                   // taxicab
    // 3-4-5: sort descending
    if (a < b) { int t = a; a = b; b = t; }
    if (b < c) { int t = b; b = c; c = t; }
    if (a < b) { int t = a; a = b; b = t; }
    return 3 * a + b + c;
}

__host__ __device__ constexpr int cdt_vmax(int metric) { return metric == 2 ? 12 : 4; }

constexpr int kCdtShellMax = 729;

struct CdtShellList {
    int n;
    int nclass;
    int cls_value[64];
    int cls_begin[65];
    ShellOff o[kCdtShellMax];
};

__host__ __device__ constexpr CdtShellList make_cdt_list(int metric) {
    CdtShellList l{};
    const int vmax = cdt_vmax(metric);
    int n = 0, nc = 0;
    for (int v = 0; v <= vmax; v++) {
        bool any = false;
        for (int dz = -kShellR; dz <= kShellR; dz++)
            for (int dy = -kShellR; dy <= kShellR; dy++)
                for (int dx = -kShellR; dx <= kShellR; dx++)
                    if (cdt_norm(metric, dz, dy, dx) == v) {
                        if (!any) {
                            l.cls_value[nc] = v;
                            l.cls_begin[nc] = n;
                            nc++;
                            any = true;
                        }
                        l.o[n++] = ShellOff{dz, dy, dx, v};
                    }
    }
    l.n = n;
    l.nclass = nc;
    l.cls_begin[nc] = n;
    return l;
}

// Smallest chamfer norm from voxel (z, y, x) of one item to a background
// voxel beyond the shell, by the whole warp on the bitmap: cubes of
// Chebyshev radius R = 6, 13, 27, ... until the best norm is at most the
// smallest norm outside the cube (R + 1, or 3 (R + 1) for 3-4-5) or the cube
// covers the item.  Each norm grows with |dx| for fixed (dz, dy), so per row
// the nearest background bit on either side of x is the row's best.
// Returns -1 if the item has no background.
template <int MET>
__device__ int far_norm_search(const uint32_t *__restrict__ ibm, int z, int y, int x, int L0, int L1, int W,
                               int lane) {
    constexpr int WW = 4;
    int best = 0x7fffffff;
    for (int R = 6;; R = 2 * R + 1) {
        const int side = 2 * R + 1;
        const int xl = max(0, x - R), xr = min(W - 1, x + R);
        for (int k = lane; k < side * side; k += 32) {
            const int dz = k / side - R, dy = k % side - R;
            const int zz = z + dz, yy = y + dy;
            if ((unsigned)zz >= (unsigned)L0 || (unsigned)yy >= (unsigned)L1) continue;
            if (cdt_norm(MET, dz, dy, 0) >= best) continue;
            const uint32_t *row = ibm + ((int64_t)zz * L1 + yy) * WW;
            for (int w = x >> 5; w >= (xl >> 5); w--) {  // nearest background at x' <= x
                uint32_t m = row[w];
                if (w == (x >> 5)) m &= (x & 31) == 31 ? 0xffffffffu : ((2u << (x & 31)) - 1u);
                if (w == (xl >> 5)) m &= ~((1u << (xl & 31)) - 1u);
                if (m) {
                    best = min(best, cdt_norm(MET, dz, dy, x - (32 * w + 31 - __clz(m))));
                    break;
                }
            }
            if (x < xr)
                for (int w = (x + 1) >> 5; w <= (xr >> 5); w++) {  // nearest background at x' > x
                    uint32_t m = row[w];
                    if (w == ((x + 1) >> 5)) m &= ~((1u << ((x + 1) & 31)) - 1u);
                    if (w == (xr >> 5)) m &= (xr & 31) == 31 ? 0xffffffffu : ((2u << (xr & 31)) - 1u);
                    if (m) {
                        best = min(best, cdt_norm(MET, dz, dy, 32 * w + __ffs(m) - 1 - x));
                        break;
                    }
                }
        }
        best = __reduce_min_sync(~0u, best);
        const int outside = MET == 2 ? 3 * (R + 1) : R + 1;
        const bool covers =
            z - R <= 0 && z + R >= L0 - 1 && y - R <= 0 && y + R >= L1 - 1 && x - R <= 0 && x + R >= W - 1;
        if (best <= outside || covers) return best == 0x7fffffff ? -1 : best;
    }
}

constexpr int kCdtFarPerUnit = 64;  // voxels beyond the shell searched per 32-row unit at most

template <int WW, int MET>
__global__ void __launch_bounds__(kShellThreads) cdt_shell_kernel(const uint32_t *__restrict__ bm,
                                                                  float *__restrict__ dist, int *__restrict__ todo,
                                                                  CompactParams p, float divisor) {
    constexpr CdtShellList kL = make_cdt_list(MET);
    constexpr int kPitch = WW + 2 * kShellPadW;
    constexpr int kRowsP = kShellRows + 2 * kShellR;
    constexpr int kPlaneP = kRowsP * kPitch;
    __shared__ __align__(16) uint32_t bits[(2 * kShellR + 1) * kPlaneP];
    __shared__ __align__(16) uint8_t res[kShellRows * WW * 32];
    __shared__ int s_nfar;
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    const int ybl = (L1 + kShellRows - 1) / kShellRows;
    const int64_t item = blockIdx.x / ((int64_t)L0 * ybl);
    const int rem = (int)(blockIdx.x - item * L0 * ybl);
    const int z = rem / ybl, y0 = (rem % ybl) * kShellRows;
    const int nrows = min(kShellRows, L1 - y0);
    const int tid = threadIdx.x;
    pdl_trigger();  // the raster kernels may be scheduled as this grid's CTAs retire
    pdl_wait();     // the bitmap and the zeroed flags are complete
    if (tid == 0) s_nfar = 0;
    const uint32_t *ibm = bm + item * (int64_t)L0 * L1 * WW;
    for (int i = tid; i < (2 * kShellR + 1) * kRowsP; i += kShellThreads) {
        const int k = i / kRowsP, r = i - k * kRowsP;
        const int zz = z - kShellR + k, yy = y0 - kShellR + r;
        uint32_t *dst = bits + k * kPlaneP + r * kPitch;
        const bool in_item = (unsigned)zz < (unsigned)L0 && (unsigned)yy < (unsigned)L1;
        const uint32_t *src = ibm + ((int64_t)zz * L1 + yy) * WW;
        dst[0] = 0u;
        dst[kShellPadW + WW] = 0u;
#pragma unroll
        for (int c = 0; c < WW; c++) dst[kShellPadW + c] = in_item ? src[c] : 0u;
    }
    __syncthreads();
    static_assert(kShellRows * WW <= kShellThreads, "one word per thread");
    uint32_t Ufar = 0;  // voxels of this thread's word beyond the shell
    for (int e = tid; e < nrows * WW; e += kShellThreads) {
        const int r = e / WW, wi = e % WW;
        const int nb = min(32, W - 32 * wi);
        uint32_t U = nb == 32 ? 0xffffffffu : ((1u << nb) - 1u);
        const uint32_t *here = bits + kShellR * kPlaneP + (kShellR + r) * kPitch + kShellPadW + wi;
        uint8_t *out = res + r * W + 32 * wi;
        // one straight-line pass over the offsets (norm order); at the end of
        // each norm class the class's union resolves the voxels it covers
        uint32_t H = 0;
#pragma unroll
        for (int t = 0; t < kL.n; t++) {
            const int delta = kL.o[t].dz * kPlaneP + kL.o[t].dy * kPitch + (kL.o[t].dx >= 0 ? 0 : -1);
            const int sh = kL.o[t].dx >= 0 ? kL.o[t].dx : 32 + kL.o[t].dx;
            H |= __funnelshift_r(here[delta], here[delta + 1], sh);
            if (t + 1 == kL.n || kL.o[t + 1].d2 != kL.o[t].d2) {
                uint32_t hit = H & U;
                U &= ~hit;
                while (hit) {
                    const int b = __ffs(hit) - 1;
                    out[b] = (uint8_t)kL.o[t].d2;
                    hit &= hit - 1;
                }
                H = 0;
                if (U == 0u) break;
            }
        }
        if (U) atomicAdd(&s_nfar, __popc(U));
        Ufar = U;
    }
    __syncthreads();
    const int nfar = s_nfar;
    if (nfar > kCdtFarPerUnit) {  // many voxels beyond the shell: the item takes the raster passes
        if (tid == 0) {
            atomicExch(&todo[item], 1);
            atomicExch(&todo[p.batch], 1);  // some item is marked
        }
        return;
    }
    const int64_t rowbase = item * p.numel_item + ((int64_t)z * L1 + y0) * W;
    const int warp = tid >> 5, lane = tid & 31;
    for (int r = warp; r < nrows; r += kShellThreads / 32) {
        for (int x = 4 * lane; x < W; x += 128) {
            const uint32_t v4 = *reinterpret_cast<const uint32_t *>(res + r * W + x);
            float4 d;
            // divisor 3 (3-4-5): correctly rounded v / 3 as the raster path computes it
            d.x = divisor == 1.f ? (float)(v4 & 255u) : (float)(v4 & 255u) / divisor;
            d.y = divisor == 1.f ? (float)((v4 >> 8) & 255u) : (float)((v4 >> 8) & 255u) / divisor;
            d.z = divisor == 1.f ? (float)((v4 >> 16) & 255u) : (float)((v4 >> 16) & 255u) / divisor;
            d.w = divisor == 1.f ? (float)(v4 >> 24) : (float)(v4 >> 24) / divisor;
            __stcs(reinterpret_cast<float4 *>(dist + rowbase + (int64_t)r * W + x), d);
        }
    }
    if (nfar == 0) return;
    // the few voxels beyond the shell: each warp searches its own threads'
    // voxels and overwrites what was written for them above (block barrier)
    __syncthreads();
    for (unsigned has = __ballot_sync(~0u, Ufar != 0u); has; has &= has - 1) {
        const int src = __ffs(has) - 1;
        const int e = warp * 32 + src, r = e / WW, wi = e % WW;
        for (uint32_t m = __shfl_sync(~0u, Ufar, src); m; m &= m - 1) {
            const int xv = 32 * wi + __ffs(m) - 1;
            const int best = far_norm_search<MET>(ibm, z, y0 + r, xv, L0, L1, W, lane);
            if (lane != 0) continue;
            if (best < 0) {  // no background: the raster passes give -1
                atomicExch(&todo[item], 1);
                atomicExch(&todo[p.batch], 1);
            } else dist[rowbase + (int64_t)r * W + xv] = divisor == 1.f ? (float)best : (float)best / divisor;
        }
    }
}

// The offsets of the chamfer list grouped by row (dz, dy) within each norm
// class: the three staged words around a lane's word in that row (left
// neighbour, own, right neighbour) serve every dx of the class in the row.
struct CdtRow {
    int dz, dy;
    int mask;  // bit dx + 4 for each dx of the class in this row
    int val;   // the class's norm
    bool last; // last row of its class
};
constexpr int kCdtRowMax = 1024;
struct CdtRowList {
    int n;
    CdtRow r[kCdtRowMax];
};

__host__ __device__ constexpr CdtRowList make_cdt_rows(int metric) {
    CdtRowList l{};
    const CdtShellList o = make_cdt_list(metric);
    for (int c = 0; c < o.nclass; c++) {
        int mask[81] = {};
        for (int t = o.cls_begin[c]; t < o.cls_begin[c + 1]; t++)
            mask[(o.o[t].dz + kShellR) * 9 + (o.o[t].dy + kShellR)] |= 1 << (o.o[t].dx + kShellR);
        for (int k = 0; k < 81; k++)
            if (mask[k]) l.r[l.n++] = CdtRow{k / 9 - kShellR, k % 9 - kShellR, mask[k], o.cls_value[c], false};
        l.r[l.n - 1].last = true;
    }
    return l;
}

template <int MET>
constexpr CdtRowList kCdtRows = make_cdt_rows(MET);

struct CdtSearch {
    uint32_t U;               // voxels of the word not resolved yet
    uint32_t H;               // union of the current class's shifted backgrounds
    uint32_t P0, P1, P2, P3;  // bit-planes of the resolved voxels' norms
};

// One row of the row list (a compile-time constant): OR its dx shifts into H
// and, at the end of a class, resolve the class.  Returns false once every
// voxel of the word is resolved (the rest of the list is skipped).
template <int MET, int E>
__device__ __forceinline__ bool cdt_row_step(const volatile uint32_t *vh, uint32_t ml, uint32_t mr, CdtSearch &s) {
    constexpr CdtRow row = kCdtRows<MET>.r[E];
    constexpr int d = row.dz * kCwPlane + row.dy * 4;
    const uint32_t mw = vh[d];
    uint32_t lw = 0u, rw = 0u;
    // the neighbour words are always inside the staged array (pads at both ends);
    // the lane's masks zero the words left of word 0 and right of word 3
    if constexpr ((row.mask & 0x00f) != 0) lw = vh[d - 1] & ml;  // some dx < 0
    if constexpr ((row.mask & 0x1e0) != 0) rw = vh[d + 1] & mr;  // some dx > 0
#pragma unroll
    for (int dx = -kShellR; dx <= kShellR; dx++)
        if (row.mask & (1 << (dx + kShellR)))
            s.H |= dx == 0 ? mw : dx > 0 ? __funnelshift_r(mw, rw, dx) : __funnelshift_r(lw, mw, 32 + dx);
    if constexpr (row.last) {
        const uint32_t hit = s.H & s.U;
        s.U &= ~hit;
        if constexpr ((row.val & 1) != 0) s.P0 |= hit;
        if constexpr ((row.val & 2) != 0) s.P1 |= hit;
        if constexpr ((row.val & 4) != 0) s.P2 |= hit;
        if constexpr ((row.val & 8) != 0) s.P3 |= hit;
        s.H = 0u;
        return s.U != 0u;
    }
    return true;
}

template <int MET, int... Es>
__device__ __forceinline__ void cdt_rows_all(std::integer_sequence<int, Es...>, const volatile uint32_t *vh, uint32_t ml,
                                             uint32_t mr, CdtSearch &s) {
    (cdt_row_step<MET, Es>(vh, ml, mr, s) && ...);  // stops at the first false
}

// The same search on the EDT shell kernel's work-queue design: persistent
// warps take 8-row units (one 32-voxel word per lane), stage the 9 x 16
// bitmap rows they read, and keep each voxel's norm (<= 12) as 4 bit-planes
// of the word: per norm class, the voxels the class resolves OR into the
// planes of the class value's set bits, so nothing is stored per voxel until
// the writing lanes decode four voxels at once.  Staged rows are 4 words with
// no padding, so the 32 lanes (8 rows x 4 words) read 32 consecutive words --
// conflict-free -- and a lane masks the words left of word 0 and right of
// word 3 itself.  Flags: todo[item], todo[batch] as in cdt_shell_kernel; the
// 64-bit work counter follows them (8-byte aligned), zeroed with them.

template <int MET>
__global__ void __launch_bounds__(kShellCtThreads) cdt_shell_warp_kernel(const uint32_t *__restrict__ bm,
                                                                         float *__restrict__ dist,
                                                                         int *__restrict__ todo, CompactParams p,
                                                                         float divisor) {
    constexpr int WW = 4;
    constexpr int kStageIters = (kSwStageRows + 31) / 32;
    static_assert(kShellWarpRows * WW == 32, "one word per lane");
    static_assert(cdt_vmax(MET) < 16, "norms fit four bit-planes");
    // 4 words before and after the staged planes: the masked neighbour reads of
    // the first and last rows stay inside the array
    __shared__ __align__(16) uint32_t bits_all[kShellCtWarps][kCwWords + 8];
    __shared__ __align__(16) uint4 planes_all[kShellCtWarps][32];
    const int L0 = p.L0, L1 = p.L1, W = p.L2;
    const int ybl = (L1 + kShellWarpRows - 1) / kShellWarpRows;
    const int64_t nunits = p.batch * (int64_t)L0 * ybl;
    unsigned long long *queue = reinterpret_cast<unsigned long long *>(todo + ((p.batch + 2) & ~(int64_t)1));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *bits = bits_all[warp] + 4;
    uint4 *planes = planes_all[warp];
    pdl_trigger();  // the raster kernel may be scheduled as this grid's CTAs retire
    if (lane < 4) bits[-4 + lane] = 0u;
    else if (lane < 8) bits[kCwWords + lane - 4] = 0u;
    __syncwarp();
    pdl_wait();  // the background bitmap and the zeroed flags / counter are complete
    for (;;) {
        int64_t unit = 0;
        if (lane == 0) unit = (int64_t)atomicAdd(queue, 1ull);
        unit = __shfl_sync(~0u, unit, 0);
        if (unit >= nunits) break;
        const int64_t item = unit / ((int64_t)L0 * ybl);
        const int rem = (int)(unit - item * L0 * ybl);
        const int z = rem / ybl, y0 = (rem % ybl) * kShellWarpRows;
        const int nrows = min(kShellWarpRows, L1 - y0);
        const uint32_t *ibm = bm + item * (int64_t)L0 * L1 * WW;
        uint4 v[kStageIters];
#pragma unroll
        for (int j = 0; j < kStageIters; j++) {
            const int i = lane + 32 * j;
            const int kk = i / kSwRowsP, r = i - kk * kSwRowsP;
            const int zz = z - kShellR + kk, yy = y0 - kShellR + r;
            const bool ok = i < kSwStageRows && (unsigned)zz < (unsigned)L0 && (unsigned)yy < (unsigned)L1;
            v[j] = ok ? *reinterpret_cast<const uint4 *>(ibm + ((int64_t)zz * L1 + yy) * WW) : make_uint4(0, 0, 0, 0);
        }
#pragma unroll
        for (int j = 0; j < kStageIters; j++) {
            const int i = lane + 32 * j;
            if (i < kSwStageRows) reinterpret_cast<uint4 *>(bits)[i] = v[j];  // row i = plane i / 16, row i % 16
        }
        __syncwarp();
        uint32_t U = 0u;
        {
            const int r = lane >> 2, wi = lane & 3;
            const int nb = min(32, W - 32 * wi);
            if (r < nrows) U = nb == 32 ? 0xffffffffu : ((1u << nb) - 1u);
            const volatile uint32_t *vh = bits + kShellR * kCwPlane + (kShellR + r) * 4 + wi;
            const uint32_t ml = wi != 0 ? ~0u : 0u, mr = wi != WW - 1 ? ~0u : 0u;
            // one straight-line pass over the rows of each norm class in turn; at
            // the end of a class its union resolves the voxels it covers
            CdtSearch cs{U, 0u, 0u, 0u, 0u, 0u};
            cdt_rows_all<MET>(std::make_integer_sequence<int, kCdtRows<MET>.n>{}, vh, ml, mr, cs);
            U = cs.U;
            planes[lane] = make_uint4(cs.P0, cs.P1, cs.P2, cs.P3);
        }
        const unsigned nfar = __reduce_add_sync(~0u, (unsigned)__popc(U));
        if (nfar > kFarPerUnit) {  // many voxels beyond the shell: the item takes the raster passes
            if (lane == 0) {
                atomicExch(&todo[item], 1);
                atomicExch(&todo[p.batch], 1);
            }
            continue;
        }
        __syncwarp();
        const int64_t rowbase = item * p.numel_item + ((int64_t)z * L1 + y0) * W;
        const int x = 4 * lane;
        if (x < W) {
            const int b = x & 31;
            for (int r = 0; r < nrows; r++) {
                const uint4 q = planes[r * 4 + (x >> 5)];
                // the norms of voxels x..x+3, one per byte: each plane's nibble
                // spread to one bit per byte
                const uint32_t acc = ((((q.x >> b) & 15u) * 0x00204081u) & 0x01010101u) |
                                     (((((q.y >> b) & 15u) * 0x00204081u) & 0x01010101u) << 1) |
                                     (((((q.z >> b) & 15u) * 0x00204081u) & 0x01010101u) << 2) |
                                     (((((q.w >> b) & 15u) * 0x00204081u) & 0x01010101u) << 3);
                float4 d;
                // divisor 3 (3-4-5): correctly rounded v / 3 as the raster path computes it
                d.x = divisor == 1.f ? (float)(acc & 255u) : (float)(acc & 255u) / divisor;
                d.y = divisor == 1.f ? (float)((acc >> 8) & 255u) : (float)((acc >> 8) & 255u) / divisor;
                d.z = divisor == 1.f ? (float)((acc >> 16) & 255u) : (float)((acc >> 16) & 255u) / divisor;
                d.w = divisor == 1.f ? (float)(acc >> 24) : (float)(acc >> 24) / divisor;
                __stcs(reinterpret_cast<float4 *>(dist + rowbase + (int64_t)r * W + x), d);
            }
        }
        if (nfar) {
            __syncwarp();  // the unit's stores above come first
            for (unsigned has = __ballot_sync(~0u, U != 0u); has; has &= has - 1) {
                const int src = __ffs(has) - 1;
                for (uint32_t m = __shfl_sync(~0u, U, src); m; m &= m - 1) {
                    const int yv = y0 + (src >> 2), xv = 32 * (src & 3) + __ffs(m) - 1;
                    const int best = far_norm_search<MET>(ibm, z, yv, xv, L0, L1, W, lane);
                    if (lane != 0) continue;
                    if (best < 0) {  // no background: the raster passes give -1
                        atomicExch(&todo[item], 1);
                        atomicExch(&todo[p.batch], 1);
                    } else {
                        dist[rowbase + (int64_t)(yv - y0) * W + xv] =
                            divisor == 1.f ? (float)best : (float)best / divisor;
                    }
                }
            }
        }
        __syncwarp();  // bits and planes are free for the next unit
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
    if (sum + 64 >= (int64_t)kBig) return false;  // every squared distance stays below kBig
    if (g.ndim == 3 && g.shape[1] > kMaxL1) return false;
    if (g.shape[g.ndim - 1] > kMaxL2) return false;
    if (g.numel >= ((int64_t)1 << 40)) return false;
    return true;
}

// CTAs of one kernel resident at once on the device (one wave), at least one.
template <typename K>
int64_t wave_ctas(K kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return (int64_t)per_sm * sm_count();
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
    const bool fused = g.ndim == 3 && p.L0 <= 254 && p.L1 <= 254 && (p.L2 % 4) == 0 && ((uintptr_t)dist & 15) == 0 &&
                       ((uintptr_t)indices & 15) == 0 && ((uintptr_t)sqdist & 15) == 0 && (g.numel % 4) == 0 &&
                       c12_smem(p.L1, p.L2).total <= 200 * 1024;
    // dense backgrounds: shell search first; the separable passes then run only
    // for the items it could not finish (todo flags).  The (f0, f1) plane of
    // the unfused pass 1 is unused on this path and holds the bitmap + flags.
    int *todo = nullptr;
    // autotuned variant 1: the separable passes for every item (no shell search)
    const bool shell = tune_variant(kTuneEdt3D, tune_class(kTuneEdt3D, g.numel, 0)) != 1;
    if (fused && p.L2 <= 1024 && shell) {
        int st = TM_OK;
        const int ww = (p.L2 + 31) / 32;
        const int64_t nwords = g.batch * (int64_t)p.L0 * p.L1 * ww;
        uint32_t *bm = reinterpret_cast<uint32_t *>(c2);
        todo = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(c2) + align256((size_t)nwords * 4));
        // per-item flags, then (8-byte aligned) the shell kernel's 64-bit work
        // counter: zeroed by the bitmap kernel
        const int nclear = (int)((g.batch + 1) & ~(int64_t)1) + 2;
        if (g.batch > ((int64_t)1 << 30)) return fail(TM_ERR_TOO_LARGE, "batch too large");
        const unsigned bblocks = (unsigned)std::min<int64_t>(ceil_div(nwords, 256), (int64_t)sm_count() * 16);
        const bool vrow = (p.L2 % 32) == 0 && ((uintptr_t)input & 15) == 0;
        if (in_dtype == TM_F32) {
            const float *in = static_cast<const float *>(input);
            if (vrow) edt_bitmap_kernel<float, true><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
            else edt_bitmap_kernel<float, false><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
        } else {
            const uint8_t *in = static_cast<const uint8_t *>(input);
            if (vrow) edt_bitmap_kernel<uint8_t, true><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
            else edt_bitmap_kernel<uint8_t, false><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
        }
        TM_LAUNCH_CHECK("edt_bitmap_kernel");
        const ShellSmem sm = shell_smem(p.L2);
        const int64_t sblocks = g.batch * (int64_t)p.L0 * ceil_div(p.L1, kShellRows);
        if (sblocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        auto launch_ct = [&](auto kernel) -> int {
            static thread_local int cached_dev = -1, cached_ctas = 0;
            static thread_local const void *cached_fn = nullptr;
            int dev = 0;
            TM_CHECK_CUDA(cudaGetDevice(&dev));
            if (cached_dev != dev || cached_fn != (const void *)kernel) {
                int per_sm = 0;
                TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kShellCtThreads, 0));
                cached_ctas = (per_sm < 1 ? 1 : per_sm) * sm_count();
                cached_dev = dev;
                cached_fn = (const void *)kernel;
            }
            // persistent warps on a work queue of 8-row units
            const int64_t wunits = g.batch * (int64_t)p.L0 * ceil_div(p.L1, kShellWarpRows);
            const int64_t grid = std::min<int64_t>(cached_ctas, ceil_div(wunits, kShellCtWarps));
            TM_CHECK_CUDA(launch_pdl(kernel, dim3((unsigned)grid), dim3(kShellCtThreads), 0, stream, bm, dist,
                                     indices, sqdist, todo, p));
            return TM_OK;
        };
        if (ww == 4) {  // rows of 97..128 voxels: straight-line search
            if ((st = launch_ct(edt_shell_ct_kernel<4>)) != TM_OK) return st;
        } else {
            if (sm.total > 48 * 1024)
                TM_CHECK_CUDA(cudaFuncSetAttribute(edt_shell_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)sm.total));
            edt_shell_kernel<<<(unsigned)sblocks, kShellThreads, sm.total, stream>>>(bm, dist, indices, sqdist, todo,
                                                                                    p);
        }
        TM_LAUNCH_CHECK("edt_shell_kernel");
    }
    // pass 0
    const int64_t inner0 = g.numel_item / g.shape[0];
    if (p.L0 <= kMaxL0Smem) {
        const int64_t blocks = g.batch * ceil_div(inner0, kCols);
        if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        const size_t smem = (size_t)p.L0 * kCols * 3 + (size_t)kSegs * kCols * 4;
        if (smem > 48 * 1024) {
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<float>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<uint8_t>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        }
        // after the shell search: overlap this launch with its last CTAs, one
        // resident wave striding over the column blocks
        if (in_dtype == TM_F32) {
            const float *in = static_cast<const float *>(input);
            if (todo) {
                const int64_t grid = std::min<int64_t>(blocks, wave_ctas(edt_c0_smem_kernel<float>, kCols * kSegs, smem));
                TM_CHECK_CUDA(launch_pdl(edt_c0_smem_kernel<float>, dim3((unsigned)grid), dim3(kCols * kSegs), smem,
                                         stream, in, c1, p, (const int *)todo));
            } else {
                edt_c0_smem_kernel<float><<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(in, c1, p, todo);
            }
        } else {
            const uint8_t *in = static_cast<const uint8_t *>(input);
            if (todo) {
                const int64_t grid =
                    std::min<int64_t>(blocks, wave_ctas(edt_c0_smem_kernel<uint8_t>, kCols * kSegs, smem));
                TM_CHECK_CUDA(launch_pdl(edt_c0_smem_kernel<uint8_t>, dim3((unsigned)grid), dim3(kCols * kSegs),
                                         smem, stream, in, c1, p, (const int *)todo));
            } else {
                edt_c0_smem_kernel<uint8_t><<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(in, c1, p, todo);
            }
        }
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
    // passes 1 + 2 fused per plane when the plane fits on chip
    if (fused) {
        const size_t smem = c12_smem(p.L1, p.L2).total;
        const int64_t blocks = g.batch * (int64_t)p.L0;
        if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        if (smem > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c12_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
        // launched after pass 0 (whose kernel runs normally when there is no shell search)
        const int64_t grid = todo ? std::min<int64_t>(blocks, wave_ctas(edt_c12_kernel, kC12Threads, smem)) : blocks;
        TM_CHECK_CUDA(launch_pdl(edt_c12_kernel, dim3((unsigned)grid), dim3(kC12Threads), smem, stream,
                                 (const int16_t *)c1, dist, indices, sqdist, p, (const int *)todo));
        TM_LAUNCH_CHECK("edt_c12_kernel");
        return TM_OK;
    }
    // pass 1 (3-D)
    if (g.ndim == 3) {
        const int64_t blocks = g.batch * (int64_t)p.L0 * ceil_div(p.L2, kCols);
        if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
        const size_t smem = (size_t)(p.L1 + kPadTop + kPadBot) * kCols * 6 + kCols * sizeof(int);
        if (smem > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        edt_c1_kernel<<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(c1, c2, stack1, p);
        TM_LAUNCH_CHECK("edt_c1_kernel");
    }
    // pass 2
    const int L = g.ndim == 3 ? p.L2 : p.L1;
    const size_t per_warp = (size_t)(L + 8) * 8 + (size_t)L * 2;
    // 16-byte vector path: whole 128-voxel chunks and 16-byte aligned planes
    auto a16 = [](const void *ptr) { return ((uintptr_t)ptr & 15) == 0; };
    const bool vec = (L % 128) == 0 && (g.numel % 4) == 0 && a16(dist) && a16(indices) && a16(sqdist);
    int warps = kC2Warps;
    while (warps > 1 && per_warp * warps > 160 * 1024) warps >>= 1;
    const int64_t nlines2 = g.numel / L;
    const unsigned b2 = (unsigned)ceil_div(nlines2, warps);
    const size_t smem2 = per_warp * warps + kSqrtTab * sizeof(float);
    auto launch2 = [&](auto kernel, const void *cin) -> int {
        if (smem2 > 48 * 1024)
            TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
        kernel<<<b2, warps * 32, smem2, stream>>>(cin, dist, indices, sqdist, p, warps);
        return TM_OK;
    };
    int st;
    if (g.ndim == 3)
        st = vec ? launch2(edt_c2_kernel<true, true>, c2) : launch2(edt_c2_kernel<true, false>, c2);
    else
        st = vec ? launch2(edt_c2_kernel<false, true>, c1) : launch2(edt_c2_kernel<false, false>, c1);
    if (st != TM_OK) return st;
    TM_LAUNCH_CHECK("edt_c2_kernel");
    return TM_OK;
}


bool cdt_shell_eligible(const Geometry &g, const float *dist, const int32_t *indices) {
    if (g.ndim != 3 || indices || !dist) return false;
    const int64_t L0 = g.shape[0], L1 = g.shape[1], L2 = g.shape[2];
    const int ww = (int)((L2 + 31) / 32);
    return (L2 % 4) == 0 && ((uintptr_t)dist & 15) == 0 && ww == 4 && L0 < 32768 && L1 < 32768 &&
           g.numel_item < ((int64_t)1 << 31);
}

size_t cdt_shell_workspace(const Geometry &g) {
    const int ww = (int)((g.shape[2] + 31) / 32);
    // per-item flags, the "some item is marked" flag, then the 64-bit work counter
    return align256((size_t)g.batch * g.shape[0] * g.shape[1] * ww * 4) +
           align256((size_t)((g.batch + 2) & ~(int64_t)1) * 4 + 8);
}

int cdt_shell_run(const void *input, int in_dtype, const Geometry &g, int metric, float *dist, unsigned char *ws,
                  int **todo_out, cudaStream_t stream, bool block_kernel) {
    CompactParams p;
    std::memset(&p, 0, sizeof(p));
    p.ndim = 3;
    p.L0 = (int)g.shape[0];
    p.L1 = (int)g.shape[1];
    p.L2 = (int)g.shape[2];
    p.batch = g.batch;
    p.numel = g.numel;
    p.numel_item = g.numel_item;
    const int ww = (p.L2 + 31) / 32;
    const int64_t nwords = g.batch * (int64_t)p.L0 * p.L1 * ww;
    uint32_t *bm = reinterpret_cast<uint32_t *>(ws);
    int *todo = reinterpret_cast<int *>(ws + align256((size_t)nwords * 4));
    if (g.batch > ((int64_t)1 << 30)) return fail(TM_ERR_TOO_LARGE, "batch too large");
    // per-item flags, the "any item marked" flag and (8-byte aligned) the warp
    // kernel's work counter, zeroed by the bitmap kernel
    const int nclear = (int)((g.batch + 2) & ~(int64_t)1) + 2;
    const unsigned bblocks = (unsigned)std::min<int64_t>(ceil_div(nwords, 256), (int64_t)sm_count() * 16);
    const bool vrow = (p.L2 % 32) == 0 && ((uintptr_t)input & 15) == 0;
    if (in_dtype == TM_F32) {
        const float *in = static_cast<const float *>(input);
        if (vrow) edt_bitmap_kernel<float, true><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
        else edt_bitmap_kernel<float, false><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
    } else {
        const uint8_t *in = static_cast<const uint8_t *>(input);
        if (vrow) edt_bitmap_kernel<uint8_t, true><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
        else edt_bitmap_kernel<uint8_t, false><<<bblocks, 256, 0, stream>>>(in, bm, p, ww, nwords, todo, nclear);
    }
    TM_LAUNCH_CHECK("edt_bitmap_kernel");
    const int64_t blocks = g.batch * (int64_t)p.L0 * ceil_div(p.L1, kShellRows);
    if (blocks >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "too many blocks");
    const float div = metric == TM_CDT_CHAMFER345 ? 3.0f : 1.0f;
    if (block_kernel) {  // one CTA per 32-row block
        auto go = [&](auto kernel) {
            return launch_pdl(kernel, dim3((unsigned)blocks), dim3(kShellThreads), 0, stream, (const uint32_t *)bm,
                              dist, todo, p, div);
        };
        if (metric == TM_CDT_CHESSBOARD) TM_CHECK_CUDA(go(cdt_shell_kernel<4, 0>));
        else if (metric == TM_CDT_TAXICAB) TM_CHECK_CUDA(go(cdt_shell_kernel<4, 1>));
        else TM_CHECK_CUDA(go(cdt_shell_kernel<4, 2>));
        TM_LAUNCH_CHECK("cdt_shell_kernel");
    } else {  // persistent warps on a work queue of 8-row units
        auto go = [&](auto kernel) -> int {
            int per_sm = 0;
            TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kShellCtThreads, 0));
            const int64_t wunits = g.batch * (int64_t)p.L0 * ceil_div(p.L1, kShellWarpRows);
            const int64_t grid = std::min<int64_t>((int64_t)(per_sm < 1 ? 1 : per_sm) * sm_count(),
                                                   ceil_div(wunits, kShellCtWarps));
            TM_CHECK_CUDA(launch_pdl(kernel, dim3((unsigned)grid), dim3(kShellCtThreads), 0, stream,
                                     (const uint32_t *)bm, dist, todo, p, div));
            return TM_OK;
        };
        int st;
        if (metric == TM_CDT_CHESSBOARD) st = go(cdt_shell_warp_kernel<0>);
        else if (metric == TM_CDT_TAXICAB) st = go(cdt_shell_warp_kernel<1>);
        else st = go(cdt_shell_warp_kernel<2>);
        if (st != TM_OK) return st;
        TM_LAUNCH_CHECK("cdt_shell_warp_kernel");
    }
    *todo_out = todo;
    return TM_OK;
}

int ragged_edt3_max_line() { return kRaggedC12MaxLine; }

int ragged_edt3_run(const void *input, int in_f32, const ReItem *items, int nitems, int64_t cols, int64_t total,
                    int max_line, int16_t *c1, float *dist, int32_t *indices, int32_t *sqdist, GridControl *ctl,
                    cudaStream_t stream) {
    if (max_line < 1 || max_line > kRaggedC12MaxLine)
        return fail(TM_ERR_UNSUPPORTED, "ragged 3-D planes need axes of at most %d voxels", kRaggedC12MaxLine);
    RaggedC12Args A{};
    A.in = input;
    A.in_f32 = in_f32;
    A.nitems = nitems;
    A.items = items;
    A.cols = cols;
    A.total = total;
    A.c1 = c1;
    A.dist = dist;
    A.indices = indices;
    A.sqdist = sqdist;
    A.ctl = ctl;
    int st = device_status_word(&A.status);
    if (st != TM_OK) return st;
    A.spin_limit = grid_wait_budget();
    // every plane's regions fit the largest item's layout (each grows with L1 and W)
    const size_t smem = c12_smem(max_line, max_line).total;
    static thread_local int cached_dev = -1, cached_per_sm = 0;
    static thread_local size_t cached_smem = 0;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev != dev || cached_smem != smem) {
        TM_CHECK_CUDA(cudaFuncSetAttribute(ragged_edt3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)c12_smem(kRaggedC12MaxLine, kRaggedC12MaxLine).total));
        TM_CHECK_CUDA(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_per_sm, ragged_edt3_kernel, kC12Threads, smem));
        cached_dev = dev;
        cached_smem = smem;
    }
    if (cached_per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "ragged 3-D EDT kernel does not fit on an SM");
    const int64_t blocks = (int64_t)cached_per_sm * sm_count();  // one wave: both phases are grid-stride loops
    TM_CHECK_CUDA(cudaMemsetAsync(ctl, 0, sizeof(GridControl), stream));
    void *params[] = {&A};
    TM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void *)ragged_edt3_kernel, dim3((unsigned)blocks),
                                              dim3(kC12Threads), params, smem, stream));
    TM_LAUNCH_CHECK("ragged_edt3_kernel");
    return TM_OK;
}

}  // namespace tmc
