// Binary morphology of 1-D / 2-D items on bit-packed tiles (GB300, sm_103a):
// erosion, dilation, and the opening / closing fused into one pass.
//
// The reference runs one byte per voxel through a tap loop, and its opening /
// closing are two full launches with the intermediate image in HBM
// (torchmorph/morphology/binary.py:231-290, csrc/binary_kernel.cu:56-127).
// Here one CTA of 128 threads owns a 32 x 128 output tile (the ragged plan's
// tile, ragged.cu) and keeps its input region as 32-voxel words:
//  * staging: a warp reads 32 consecutive bytes of a row (one per lane,
//    coalesced) and __ballot_sync packs them into one word; positions outside
//    the item read border_value;
//  * one operator on words: out = AND (erosion) / OR (dilation) over the taps
//    of the 32-voxel row segment shifted by the tap -- one funnel shift and one
//    logic operation per tap for 32 voxels;
//  * fused opening / closing: the first operator over the tile grown by the
//    second one's halo, kept in shared memory, positions outside the item set
//    to border_value (the reference's intermediate image is read with
//    border_value outside the item), then the second operator;
//  * output: each lane writes one byte of a row segment (32 consecutive bytes
//    per warp store).
// Taps follow the reference's offsets (erosion reads x + d, dilation x - d,
// d = k - (size // 2 + origin)); erosion with no taps inside the item still
// ANDs border_value, exactly as the per-voxel loop does.  Limits: every tap
// within 16 rows and 32 columns of the output, at most 1024 taps per
// operator.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "bitmorph.cuh"
#include "tile_queue.cuh"

namespace tmc {
namespace {

constexpr int kBTileH = 32, kBTileW = 128, kBWords = kBTileW / 32;  // 4 words per tile row
constexpr int kBThreads = kBTileH * kBWords;                           // one output word per thread
constexpr int kBMaxTaps = 1024;
constexpr int kBMaxDy = 16, kBMaxDx = 32;

struct BitTaps {
    int n;
    int hy, hx;  // largest |dy| and |dx| of the read offsets
    int8_t dy[kBMaxTaps], dx[kBMaxTaps];
};

struct BitOps {
    BitTaps op[2];  // read offsets of the first and (fused) second operator
    int nops;       // 1 or 2
    int or1, or2;   // operator k is a dilation (OR) rather than an erosion (AND)
    int border;     // border_value, 0 or 1
};

struct BitItem {  // the layout of ragged.cu's plan descriptors
    int64_t off;
    int H, W;
    int tile_begin;
    int tiles_x;
    int pad[2];
};

struct BitPlanHeader {
    int queue;
    int ntiles;
    int nitems;
    int pad[61];
};

struct BitUniform {
    int64_t batch;
    int H, W;
    int tiles_x, tiles_item;
};

__host__ __device__ inline int floor32(int v) { return v >= 0 ? v / 32 : -((-v + 31) / 32); }

// Word ranges of a tile (word j of a row = columns x0 + 32 j .. + 31).  An
// operator with column reach hx that computes words clo .. chi reads words
// clo + floor32(-hx) .. chi + floor32(hx) + 1 (the + 1: the funnel shift's
// high word).
struct BitGeom {
    int HY, srows, sjlo, sld;  // staged input: rows y0 - HY .., words sjlo .. sjlo + sld - 1
    int irows, ijlo, ild;      // first operator's result (fused): rows y0 - hy2 .., words ijlo ..
};

__host__ __device__ inline BitGeom bit_geom(const BitOps &ops) {
    const bool fused = ops.nops == 2;
    const int hy1 = ops.op[0].hy, hx1 = ops.op[0].hx;
    const int hy2 = fused ? ops.op[1].hy : 0, hx2 = fused ? ops.op[1].hx : 0;
    int clo = 0, chi = kBWords - 1;  // words the first operator computes
    if (fused) {
        clo = floor32(-hx2);
        chi = kBWords - 1 + floor32(hx2) + 1;
    }
    BitGeom g;
    g.irows = kBTileH + 2 * hy2;
    g.ijlo = clo;
    g.ild = chi - clo + 1;
    g.HY = hy1 + hy2;
    g.srows = kBTileH + 2 * g.HY;
    g.sjlo = clo + floor32(-hx1);
    g.sld = chi + floor32(hx1) + 1 - g.sjlo + 1;
    return g;
}

// One operator over a word array: out word (r, w) for rows r < nrows, words
// wlo <= w <= whi of the output region; `src` holds rows with row offset
// `srow` (source row of output row r and tap dy: r + srow + dy) and words from
// `sjlo` (ld words per row).
__device__ __forceinline__ uint32_t bit_op(const uint32_t *src, int ld, int sjlo, int srow, int r, int w,
                                           const BitTaps &t, bool is_or) {
    uint32_t acc = is_or ? 0u : ~0u;
    for (int k = 0; k < t.n; k++) {
        const int dx = t.dx[k];
        const int q = floor32(dx), sh = dx - 32 * q;
        const uint32_t *row = src + (r + srow + t.dy[k]) * ld + (w - sjlo + q);
        const uint32_t v = sh ? __funnelshift_r(row[0], row[1], sh) : row[0];
        acc = is_or ? (acc | v) : (acc & v);
    }
    return acc;
}

__global__ void __launch_bounds__(kBThreads) bitmorph_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                             BitPlanHeader *hdr, const BitItem *__restrict__ items,
                                                             BitUniform u, const __grid_constant__ BitOps ops) {
    extern __shared__ __align__(16) uint32_t bsm[];
    __shared__ int s_slot[2];
    __shared__ int s_tb[kQueueCache];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    TileQueue<BitItem> q{hdr ? &hdr->queue : nullptr, hdr ? hdr->ntiles : 0, hdr ? hdr->nitems : 0, items, s_tb,
                         s_slot, 0};
    if (hdr) q.init();
    const BitTaps &t1 = ops.op[0];
    const BitTaps &t2 = ops.op[1];
    const bool fused = ops.nops == 2;
    const int hy2 = fused ? t2.hy : 0;
    const BitGeom g = bit_geom(ops);
    const int HY = g.HY, srows = g.srows, sjlo = g.sjlo, sld = g.sld;
    const int irows = g.irows, ijlo = g.ijlo, ild = g.ild;
    uint32_t *S = bsm;
    uint32_t *I = bsm + srows * sld;
    const uint32_t bvw = ops.border ? ~0u : 0u;
    const int64_t ntiles = hdr ? 0 : u.batch * (int64_t)u.tiles_item;
    for (int64_t k = blockIdx.x;; k += gridDim.x) {
        int lt, H, W, tiles_x;
        int64_t off;
        if (hdr) {
            __syncthreads();  // the previous tile's readers are done with s_slot and the buffers
            if (!q.take()) break;
            const BitItem &v = items[s_slot[1]];
            lt = s_slot[0] - v.tile_begin;
            off = v.off;
            H = v.H;
            W = v.W;
            tiles_x = v.tiles_x;
        } else {
            if (k >= ntiles) break;
            __syncthreads();
            const int64_t item = k / u.tiles_item;
            lt = (int)(k - item * u.tiles_item);
            H = u.H;
            W = u.W;
            off = item * (int64_t)H * W;
            tiles_x = u.tiles_x;
        }
        const int ty = lt / tiles_x, tx = lt - ty * tiles_x;
        const int y0 = ty * kBTileH, x0 = tx * kBTileW;
        const uint8_t *src = in + off;
        // ---- stage: every lane packs one 32-voxel word from the 8 (or 9, when the
        // row segment is not 4-byte aligned) aligned 4-byte words that hold its 32
        // bytes -- all its loads in flight at once.  Words reaching past the item's
        // columns are packed by the whole warp instead: one byte per lane and a ballot.
        const int nwords = srows * sld;
        for (int e0 = warp * 32; e0 < nwords; e0 += kBThreads) {
            const int e = e0 + lane;
            const int rw = e / sld, j = e - rw * sld;
            const int y = y0 - HY + rw, xs = x0 + 32 * (sjlo + j);
            const bool valid = e < nwords;
            const bool yin = valid && (unsigned)y < (unsigned)H;
            const bool full = yin && xs >= 0 && xs + 32 <= W;
            uint32_t word = bvw;
            if (full) {
                const uintptr_t a = reinterpret_cast<uintptr_t>(src + (int64_t)y * W + xs);
                const uint32_t *w4 = reinterpret_cast<const uint32_t *>(a & ~(uintptr_t)3);
                const int sh = (int)(a & 3) * 8;
                uint32_t v[9];
#pragma unroll
                for (int i = 0; i < 8; i++) v[i] = __ldg(w4 + i);
                v[8] = sh ? __ldg(w4 + 8) : 0u;  // holds byte 31 exactly when the segment is unaligned
                word = 0u;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const uint32_t q = sh ? __funnelshift_r(v[i], v[i + 1], sh) : v[i];  // bytes 4i .. 4i+3, 0 or 1
                    word |= ((q * 0x01020408u) >> 24) << (4 * i);
                }
            }
            // words partly outside the item's columns: the warp packs them one by one
            for (unsigned part = __ballot_sync(~0u, yin && !full); part; part &= part - 1) {
                const int src_lane = __ffs(part) - 1;
                const int py = __shfl_sync(~0u, y, src_lane), pxs = __shfl_sync(~0u, xs, src_lane);
                const int x = pxs + lane;
                const bool inside = (unsigned)x < (unsigned)W;
                const uint32_t bits = __ballot_sync(~0u, inside ? src[(int64_t)py * W + x] != 0 : ops.border != 0);
                if (lane == src_lane) word = bits;
            }
            if (valid) S[e] = word;
        }
        __syncthreads();
        uint32_t res = 0u;
        const int r = tid / kBWords, w = tid % kBWords;
        if (!fused) {
            res = bit_op(S, sld, sjlo, HY, r, w, t1, ops.or1);
        } else {
            // first operator over the intermediate region, outside the item = border_value
            for (int e = tid; e < irows * ild; e += kBThreads) {
                const int ir = e / ild, iw = ijlo + e % ild;
                const int y = y0 - hy2 + ir;
                uint32_t v = bit_op(S, sld, sjlo, t1.hy, ir, iw, t1, ops.or1);
                if ((unsigned)y >= (unsigned)H) {
                    v = bvw;
                } else {
                    const int xb = x0 + 32 * iw;  // column of bit 0
                    uint32_t inside = 0u;
                    if (xb >= 0 && xb + 32 <= W) inside = ~0u;
                    else if (xb + 32 > 0 && xb < W) {
                        const int lo = max(0, -xb), hi = min(32, W - xb);  // bits lo .. hi-1 inside
                        inside = (hi >= 32 ? ~0u : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
                    }
                    v = (v & inside) | (bvw & ~inside);
                }
                I[ir * ild + (iw - ijlo)] = v;
            }
            __syncthreads();
            res = bit_op(I, ild, ijlo, hy2, r, w, t2, ops.or2);
        }
        // ---- output: a warp writes its 8 rows one at a time; lane l writes columns
        // x0 + 4l .. x0 + 4l + 3, its nibble of the row's words spread to one byte
        // per bit by a multiply -- one 4-byte store when the row segment is 4-byte
        // aligned and inside the item, bytes otherwise
        uint8_t *dst = out + off;
        const int wr0 = warp * (32 / kBWords);  // first tile row of this warp
#pragma unroll
        for (int rr = 0; rr < 32 / kBWords; rr++) {
            const uint32_t word = __shfl_sync(~0u, res, rr * kBWords + (lane >> 3));
            const int y = y0 + wr0 + rr;
            if (y >= H) break;  // warp-uniform
            const uint32_t nib = (word >> (4 * (lane & 7))) & 15u;
            const uint32_t bytes = (nib * 0x00204081u) & 0x01010101u;
            const int x = x0 + 4 * lane;
            uint8_t *row = dst + (int64_t)y * W;
            if ((reinterpret_cast<uintptr_t>(row + x0) & 3) == 0 && x + 3 < W) {
                __stcs(reinterpret_cast<unsigned int *>(row + x), bytes);
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (x + k < W) row[x + k] = (uint8_t)((bytes >> (8 * k)) & 1u);
            }
        }
    }
}

// ---------------------------------------------------------------- walkers
// Uniform batches whose rows start on 16-byte boundaries (W % 16 == 0, aligned
// buffers) and whose structures reach at most HY rows and 32 columns: every
// warp streams down a strip of 32 words (1024 columns) of one item.  Lane l
// holds word s0 - HW + l of each row (two 16-byte loads, 4 bool bytes -> 4
// bits by one multiply); the words left and right of it come from the
// neighbouring lanes by shuffles, so an operator is, per output row, one
// funnel shift and one AND / OR per tap on registers.  The rows an operator
// reads stay in a register window; the fused opening / closing keeps a second
// window of the first operator's rows (border_value outside the item).  Lanes
// HW .. 31 - HW write their word as 32 bytes (two 16-byte stores).
constexpr int kWalkBRows = 32;   // output rows per task
constexpr int kWalkBChunk = 4;   // input rows whose loads are in flight together

struct BitRows {  // an operator's taps grouped by row offset dy = k - hy
    int n[5];
    int8_t dx[5][66];
};

struct BitWalk {
    BitRows op[2];
    int or1, or2;
    int border;
    int64_t batch;
    int H, W, nw;  // nw: words per row (W / 32 rounded up)
    int strips, rblocks;
};

// bits of words wi of row y (item rows; outside the item: border words)
__device__ __forceinline__ uint32_t walk_load(const uint8_t *item, int y, int wi, const BitWalk &a, uint32_t bvw) {
    if ((unsigned)y >= (unsigned)a.H || wi < 0 || wi >= a.nw) return bvw;
    const uint8_t *p = item + (int64_t)y * a.W + 32 * wi;
    const int valid = min(32, a.W - 32 * wi);  // a multiple of 16
    uint4 q0 = __ldg(reinterpret_cast<const uint4 *>(p));
    uint4 q1 = valid > 16 ? __ldg(reinterpret_cast<const uint4 *>(p + 16)) : make_uint4(0, 0, 0, 0);
    const uint32_t v[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
    uint32_t w = 0u;
#pragma unroll
    for (int i = 0; i < 8; i++) w |= ((v[i] * 0x01020408u) >> 24) << (4 * i);
    if (valid < 32) w = (w & ((1u << valid) - 1u)) | (bvw & ~((1u << valid) - 1u));
    return w;
}

template <bool OR, int HY>
__device__ __forceinline__ uint32_t walk_op(const uint32_t (&wl)[2 * HY + 1], const uint32_t (&wc)[2 * HY + 1],
                                            const uint32_t (&wr)[2 * HY + 1], const BitRows &t) {
    uint32_t acc = OR ? 0u : ~0u;
#pragma unroll
    for (int k = 0; k < 2 * HY + 1; k++) {
        for (int i = 0; i < t.n[k]; i++) {
            const int dx = t.dx[k][i];
            const uint32_t v = dx == 0 ? wc[k]
                               : dx > 0 ? (dx == 32 ? wr[k] : __funnelshift_r(wc[k], wr[k], dx))
                                        : (dx == -32 ? wl[k] : __funnelshift_r(wl[k], wc[k], 32 + dx));
            acc = OR ? (acc | v) : (acc & v);
        }
    }
    return acc;
}

template <int HY1, int HY2, bool FUSED>
__global__ void __launch_bounds__(256) bitwalk_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                      const __grid_constant__ BitWalk a) {
    constexpr int HW = FUSED ? 2 : 1;       // halo words per side
    constexpr int KY1 = 2 * HY1 + 1, KY2 = 2 * HY2 + 1;
    constexpr int HYT = HY1 + (FUSED ? HY2 : 0);  // input rows read above / below an output row
    const int lane = threadIdx.x & 31;
    const uint32_t bvw = a.border ? ~0u : 0u;
    const int64_t per_item = (int64_t)a.strips * a.rblocks;
    for (int64_t task = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); task < a.batch * per_item;
         task += (int64_t)gridDim.x * (blockDim.x / 32)) {
        const int64_t item = task / per_item;
        const int rem = (int)(task - item * per_item);
        const int sx = rem % a.strips, by = rem / a.strips;
        const int wi = sx * (32 - 2 * HW) - HW + lane;  // this lane's word
        const int ya = by * kWalkBRows, yb = min(ya + kWalkBRows, a.H);
        const uint8_t *src = in + item * (int64_t)a.H * a.W;
        uint8_t *dst = out + item * (int64_t)a.H * a.W;
        uint32_t l1[KY1], c1[KY1], r1[KY1];  // input rows of the first operator (word, left, right)
        uint32_t l2[KY2], c2[KY2], r2[KY2];  // first operator's rows (fused)
        // rows y - HYT .. : the first row the window needs
        const int y_first = ya - HYT;
        const int nrows = (yb - ya) + 2 * HYT;  // input rows streamed
#pragma unroll
        for (int k = 0; k < KY1; k++) l1[k] = c1[k] = r1[k] = bvw;
#pragma unroll
        for (int k = 0; k < KY2; k++) l2[k] = c2[k] = r2[k] = bvw;
        for (int t0 = 0; t0 < nrows; t0 += kWalkBChunk) {
          uint32_t wch[kWalkBChunk];
#pragma unroll
          for (int u = 0; u < kWalkBChunk; u++) wch[u] = walk_load(src, y_first + t0 + u, wi, a, bvw);
#pragma unroll
          for (int u = 0; u < kWalkBChunk; u++) {
            const int t = t0 + u;
            if (t >= nrows) continue;  // (not break: the loop stays fully unrolled)
            const int yin = y_first + t;
            const uint32_t w = wch[u];
            // shift the input window and append the new row with its neighbours
#pragma unroll
            for (int k = 0; k < KY1 - 1; k++) {
                l1[k] = l1[k + 1];
                c1[k] = c1[k + 1];
                r1[k] = r1[k + 1];
            }
            c1[KY1 - 1] = w;
            l1[KY1 - 1] = __shfl_up_sync(~0u, w, 1);
            r1[KY1 - 1] = __shfl_down_sync(~0u, w, 1);
            if (t < 2 * HY1) continue;  // window not full yet
            const int y1 = yin - HY1;   // row of the first operator's result
            uint32_t v = a.or1 ? walk_op<true, HY1>(l1, c1, r1, a.op[0]) : walk_op<false, HY1>(l1, c1, r1, a.op[0]);
            if (!FUSED) {
                if (lane >= HW && lane < 32 - HW && wi < a.nw) {
                    // 32 bytes of row y1 (only whole 16-byte groups inside the item)
                    uint8_t *p = dst + (int64_t)y1 * a.W + 32 * wi;
                    uint32_t b[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) b[i] = (((v >> (4 * i)) & 15u) * 0x00204081u) & 0x01010101u;
                    __stcs(reinterpret_cast<uint4 *>(p), make_uint4(b[0], b[1], b[2], b[3]));
                    if (a.W - 32 * wi > 16) __stcs(reinterpret_cast<uint4 *>(p + 16), make_uint4(b[4], b[5], b[6], b[7]));
                }
                continue;
            }
            // fused: the intermediate image outside the item is border_value
            if ((unsigned)y1 >= (unsigned)a.H || wi < 0 || wi >= a.nw) v = bvw;
            else if (a.W - 32 * wi < 32) {
                const int valid = a.W - 32 * wi;
                v = (v & ((1u << valid) - 1u)) | (bvw & ~((1u << valid) - 1u));
            }
#pragma unroll
            for (int k = 0; k < KY2 - 1; k++) {
                l2[k] = l2[k + 1];
                c2[k] = c2[k + 1];
                r2[k] = r2[k + 1];
            }
            c2[KY2 - 1] = v;
            l2[KY2 - 1] = __shfl_up_sync(~0u, v, 1);
            r2[KY2 - 1] = __shfl_down_sync(~0u, v, 1);
            if (t < 2 * HY1 + 2 * HY2) continue;
            const int y2 = y1 - HY2;  // output row
            const uint32_t o =
                a.or2 ? walk_op<true, HY2>(l2, c2, r2, a.op[1]) : walk_op<false, HY2>(l2, c2, r2, a.op[1]);
            if (lane >= HW && lane < 32 - HW && wi < a.nw) {
                uint8_t *p = dst + (int64_t)y2 * a.W + 32 * wi;
                uint32_t b[8];
#pragma unroll
                for (int i = 0; i < 8; i++) b[i] = (((o >> (4 * i)) & 15u) * 0x00204081u) & 0x01010101u;
                __stcs(reinterpret_cast<uint4 *>(p), make_uint4(b[0], b[1], b[2], b[3]));
                if (a.W - 32 * wi > 16) __stcs(reinterpret_cast<uint4 *>(p + 16), make_uint4(b[4], b[5], b[6], b[7]));
            }
          }
        }
    }
}

// Tap lists of an operator grouped by row for the walkers; false when a tap is
// beyond the walkers' reach (2 rows, 32 columns).
bool walk_rows(const BitTaps &t, int hy, BitRows *r) {
    std::memset(r, 0, sizeof(BitRows));
    if (t.hy > hy || t.hx > 32) return false;
    for (int i = 0; i < t.n; i++) {
        const int k = t.dy[i] + hy;
        r->dx[k][r->n[k]++] = t.dx[i];
    }
    return true;
}

template <int HY1, int HY2, bool FUSED>
int launch_walk(const uint8_t *in, uint8_t *out, const BitWalk &a, cudaStream_t s) {
    auto kernel = bitwalk_kernel<HY1, HY2, FUSED>;
    static thread_local int cached_dev = -1, cached_ctas = 0;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev != dev) {
        int per_sm = 0;
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
        cached_ctas = (per_sm < 1 ? 1 : per_sm) * sm_count();
        cached_dev = dev;
    }
    const int64_t tasks = a.batch * (int64_t)a.strips * a.rblocks;
    const int64_t blocks = std::min<int64_t>(cached_ctas, ceil_div(tasks, 8));
    kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, a);
    TM_LAUNCH_CHECK("bitwalk_kernel");
    return TM_OK;
}

// The walkers for a uniform batch, when they apply; *done = false otherwise.
int try_walk(const BitOps &ops, const uint8_t *in, uint8_t *out, int64_t batch, int64_t H, int64_t W, cudaStream_t s,
             bool *done) {
    *done = false;
    if (W % 16 != 0 || (reinterpret_cast<uintptr_t>(in) & 15) || (reinterpret_cast<uintptr_t>(out) & 15)) return TM_OK;
    const bool fused = ops.nops == 2;
    const int hy = ops.op[0].hy;
    if (hy > 2 || (fused && ops.op[1].hy != hy)) return TM_OK;
    BitWalk a;
    std::memset(&a, 0, sizeof(a));
    if (!walk_rows(ops.op[0], hy, &a.op[0])) return TM_OK;
    if (fused && !walk_rows(ops.op[1], hy, &a.op[1])) return TM_OK;
    a.or1 = ops.or1;
    a.or2 = ops.or2;
    a.border = ops.border;
    a.batch = batch;
    a.H = (int)H;
    a.W = (int)W;
    a.nw = (int)ceil_div(W, 32);
    const int sw = 32 - 2 * (fused ? 2 : 1);
    a.strips = (int)ceil_div(a.nw, sw);
    a.rblocks = (int)ceil_div(H, kWalkBRows);
    int st;
    if (!fused)
        st = hy == 0 ? launch_walk<0, 0, false>(in, out, a, s)
             : hy == 1 ? launch_walk<1, 0, false>(in, out, a, s) : launch_walk<2, 0, false>(in, out, a, s);
    else
        st = hy == 0 ? launch_walk<0, 0, true>(in, out, a, s)
             : hy == 1 ? launch_walk<1, 1, true>(in, out, a, s) : launch_walk<2, 2, true>(in, out, a, s);
    if (st == TM_OK) *done = true;
    return st;
}

size_t bitmorph_smem(const BitOps &ops) {
    const BitGeom g = bit_geom(ops);
    size_t words = (size_t)g.srows * g.sld;
    if (ops.nops == 2) words += (size_t)g.irows * g.ild;
    return words * 4;
}

// Read offsets of one operator on an (kh, kw) structure (1-D items: kh = 1).
int bit_taps(const uint8_t *structure, int kh, int kw, int oy, int ox, bool dilation, BitTaps *t) {
    std::memset(t, 0, sizeof(BitTaps));
    const int cy = kh / 2 + oy, cx = kw / 2 + ox;
    for (int a = 0; a < kh; a++)
        for (int b = 0; b < kw; b++) {
            if (!structure[a * kw + b]) continue;
            int dy = a - cy, dx = b - cx;
            if (dilation) {
                dy = -dy;
                dx = -dx;
            }
            if (dy < -kBMaxDy || dy > kBMaxDy || dx < -kBMaxDx || dx > kBMaxDx || t->n >= kBMaxTaps) return 0;
            t->dy[t->n] = (int8_t)dy;
            t->dx[t->n] = (int8_t)dx;
            t->hy = std::max(t->hy, std::abs(dy));
            t->hx = std::max(t->hx, std::abs(dx));
            t->n++;
        }
    return t->n > 0;
}

int bit_grid(size_t smem, int *grid) {
    struct Entry {
        size_t smem;
        int dev, ctas;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    for (const Entry &e : cache)
        if (e.smem == smem && e.dev == dev) {
            *grid = e.ctas;
            return TM_OK;
        }
    int per_sm = 0;
    TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bitmorph_kernel, kBThreads, smem));
    if (per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "bit tile does not fit on an SM");
    cache.push_back({smem, dev, per_sm * sm_count()});
    *grid = per_sm * sm_count();
    return TM_OK;
}

// kind: 0 erosion, 1 dilation, 2 opening, 3 closing.
int build_bitops(int kind, const uint8_t *structure, int kh, int kw, int oy, int ox, int border, BitOps *ops) {
    std::memset(ops, 0, sizeof(BitOps));
    const bool first_dil = kind == 1 || kind == 3;
    if (!bit_taps(structure, kh, kw, oy, ox, first_dil, &ops->op[0])) return 0;
    ops->or1 = first_dil;
    ops->nops = kind >= 2 ? 2 : 1;
    if (ops->nops == 2) {
        if (!bit_taps(structure, kh, kw, oy, ox, !first_dil, &ops->op[1])) return 0;
        ops->or2 = !first_dil;
    }
    ops->border = border ? 1 : 0;
    return 1;
}

}  // namespace

// 1-D / 2-D binary morphology on bit tiles.  Sets *done = false (launching
// nothing) when the structure is beyond the kernel's limits.
int bitmorph_uniform(int kind, const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                     const uint8_t *structure, const int64_t *sshape, const int64_t *origin, int border,
                     cudaStream_t s, bool *done) {
    *done = false;
    if (ndim != 1 && ndim != 2) return TM_OK;
    const int64_t H = ndim == 2 ? shape[0] : 1, W = shape[ndim - 1];
    if (H < 1 || W < 1 || H * W >= ((int64_t)1 << 31) || sshape[0] > 255 || sshape[ndim - 1] > 255) return TM_OK;
    const int kh = ndim == 2 ? (int)sshape[0] : 1, kw = (int)sshape[ndim - 1];
    const int oy = ndim == 2 ? (int)origin[0] : 0, ox = (int)origin[ndim - 1];
    BitOps ops;
    if (!build_bitops(kind, structure, kh, kw, oy, ox, border, &ops)) return TM_OK;
    int st = try_walk(ops, in, out, batch, H, W, s, done);
    if (st != TM_OK || *done) return st;
    BitUniform u;
    u.batch = batch;
    u.H = (int)H;
    u.W = (int)W;
    u.tiles_x = (int)ceil_div(W, kBTileW);
    const int64_t tiles_item = ceil_div(H, kBTileH) * (int64_t)u.tiles_x;
    if (tiles_item >= ((int64_t)1 << 31)) return TM_OK;
    u.tiles_item = (int)tiles_item;
    const size_t smem = bitmorph_smem(ops);
    int grid = 0;
    if ((st = bit_grid(smem, &grid)) != TM_OK) return st;
    const int64_t blocks = std::min<int64_t>((int64_t)grid, batch * tiles_item);
    if (blocks > 0)
        bitmorph_kernel<<<(unsigned)blocks, kBThreads, smem, s>>>(in, out, nullptr, nullptr, u, ops);
    TM_LAUNCH_CHECK("bitmorph_kernel");
    *done = true;
    return TM_OK;
}

// Ragged batches of 2-D images (the plan of tm_ragged_plan: 128 x 32 tiles).
int bitmorph_ragged(int kind, const uint8_t *in, uint8_t *out, const void *plan, const uint8_t *structure,
                    const int64_t *sshape, const int64_t *origin, int border, cudaStream_t s, bool *done) {
    *done = false;
    if (sshape[0] > 255 || sshape[1] > 255) return TM_OK;
    BitOps ops;
    if (!build_bitops(kind, structure, (int)sshape[0], (int)sshape[1], (int)origin[0], (int)origin[1], border, &ops))
        return TM_OK;
    const size_t smem = bitmorph_smem(ops);
    int grid = 0, st;
    if ((st = bit_grid(smem, &grid)) != TM_OK) return st;
    auto *hdr = static_cast<BitPlanHeader *>(const_cast<void *>(plan));
    auto *items = reinterpret_cast<const BitItem *>(static_cast<const unsigned char *>(plan) + sizeof(BitPlanHeader));
    TM_CHECK_CUDA(cudaMemsetAsync(&hdr->queue, 0, sizeof(int), s));
    BitUniform u{};
    bitmorph_kernel<<<(unsigned)grid, kBThreads, smem, s>>>(in, out, hdr, items, u, ops);
    TM_LAUNCH_CHECK("bitmorph_kernel");
    *done = true;
    return TM_OK;
}

}  // namespace tmc

namespace {

int check_binary_args(const uint8_t *in, const uint8_t *out, const uint8_t *structure, const int64_t *sshape,
                      const int64_t *origin, int nd) {
    using namespace tmc;
    if (!in || !out || !structure || !sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    for (int d = 0; d < nd; d++) {
        if (sshape[d] < 1 || sshape[d] > 255)
            return fail(TM_ERR_UNSUPPORTED, "structure sizes must be 1..255, got %lld", (long long)sshape[d]);
        if (origin[d] < -(sshape[d] / 2) || origin[d] > (sshape[d] - 1) / 2)
            return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
    }
    return TM_OK;
}

int uniform_open(int kind, const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                 const uint8_t *structure, const int64_t *sshape, const int64_t *origin, int border_value,
                 tm_stream_t stream) {
    using namespace tmc;
    if (ndim != 1 && ndim != 2) return fail(TM_ERR_UNSUPPORTED, "fused binary opening / closing: 1-D or 2-D items");
    if (batch < 1 || !shape) return fail(TM_ERR_INVALID_ARGUMENT, "empty batch or NULL shape");
    for (int d = 0; d < ndim; d++)
        if (shape[d] < 1) return fail(TM_ERR_INVALID_ARGUMENT, "empty item");
    int st = check_binary_args(in, out, structure, sshape, origin, ndim);
    if (st != TM_OK) return st;
    bool done = false;
    st = bitmorph_uniform(kind, in, out, batch, ndim, shape, structure, sshape, origin, border_value,
                          (cudaStream_t)stream, &done);
    if (st != TM_OK) return st;
    if (!done)
        return fail(TM_ERR_UNSUPPORTED, "structure beyond the fused kernel (taps within 16 rows / 32 columns)");
    return TM_OK;
}

int ragged_open(int kind, const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes, int64_t n_items,
                const uint8_t *structure, const int64_t *sshape, const int64_t *origin, int border_value,
                tm_stream_t stream) {
    using namespace tmc;
    if (!plan || n_items < 1) return fail(TM_ERR_INVALID_ARGUMENT, "NULL plan or empty batch");
    if (plan_bytes < sizeof(BitPlanHeader) + (size_t)n_items * sizeof(BitItem))
        return fail(TM_ERR_WORKSPACE, "ragged plan buffer too small for %lld images", (long long)n_items);
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    int st = check_binary_args(in, out, structure, sshape, origin, 2);
    if (st != TM_OK) return st;
    bool done = false;
    st = bitmorph_ragged(kind, in, out, plan, structure, sshape, origin, border_value, (cudaStream_t)stream, &done);
    if (st != TM_OK) return st;
    if (!done)
        return fail(TM_ERR_UNSUPPORTED, "structure beyond the fused kernel (taps within 16 rows / 32 columns)");
    return TM_OK;
}

}  // namespace

extern "C" int tm_binary_opening(const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                                 const uint8_t *structure, const int64_t *sshape, const int64_t *origin,
                                 int border_value, tm_stream_t stream) {
    return uniform_open(2, in, out, batch, ndim, shape, structure, sshape, origin, border_value, stream);
}

extern "C" int tm_binary_closing(const uint8_t *in, uint8_t *out, int64_t batch, int ndim, const int64_t *shape,
                                 const uint8_t *structure, const int64_t *sshape, const int64_t *origin,
                                 int border_value, tm_stream_t stream) {
    return uniform_open(3, in, out, batch, ndim, shape, structure, sshape, origin, border_value, stream);
}

extern "C" int tm_ragged_binary_opening(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                        int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                        const int64_t *origin, int border_value, tm_stream_t stream) {
    return ragged_open(2, in, out, plan, plan_bytes, n_items, structure, sshape, origin, border_value, stream);
}

extern "C" int tm_ragged_binary_closing(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                        int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                        const int64_t *origin, int border_value, tm_stream_t stream) {
    return ragged_open(3, in, out, plan, plan_bytes, n_items, structure, sshape, origin, border_value, stream);
}
