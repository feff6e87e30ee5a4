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
#include <cstring>

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
// Returns false when the radius exceeds kFar.
template <int K, typename GF>
__device__ __forceinline__ bool widen(int q, int L, GF G, uint32_t &best, int &bp) {
    const int r = best >= kBig ? L : isqrt_floor(best);
    if (r > kFar) return false;
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
__global__ void __launch_bounds__(kCols *kSegs) edt_c0_smem_kernel(const In *__restrict__ in,
                                                                   int16_t *__restrict__ c1, CompactParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int L = p.L0;
    const int64_t inner = p.numel_item / L;
    uint8_t *fg = smem_raw;                                              // [L][kCols]
    int16_t *prev = reinterpret_cast<int16_t *>(smem_raw + L * kCols);   // [L][kCols]
    int16_t *seg_last = prev + L * kCols;                                // [kSegs][kCols]
    int16_t *seg_first = seg_last + kSegs * kCols;                       // [kSegs][kCols]
    const int64_t cblocks = (inner + kCols - 1) / kCols;
    const int64_t item = blockIdx.x / cblocks;
    const int64_t c0 = (blockIdx.x - item * cblocks) * kCols;
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
        const size_t smem = (size_t)p.L0 * kCols * 3 + (size_t)kSegs * kCols * 4;
        if (smem > 48 * 1024) {
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<float>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            TM_CHECK_CUDA(cudaFuncSetAttribute(edt_c0_smem_kernel<uint8_t>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        }
        if (in_dtype == TM_F32)
            edt_c0_smem_kernel<float><<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(
                static_cast<const float *>(input), c1, p);
        else
            edt_c0_smem_kernel<uint8_t><<<(unsigned)blocks, kCols * kSegs, smem, stream>>>(
                static_cast<const uint8_t *>(input), c1, p);
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

}  // namespace tmc
