// 3-D morphology on shared-memory tiles (GB300, sm_103a): uniform batches of
// 3-D items and ragged batches of 3-D volumes of different shapes.
//
// Every output tile of 4 x 8 x 32 voxels (z, y, x) is computed by one CTA of
// 256 threads from a staged copy of its input region -- the tile grown by the
// footprint's extent on each axis, out-of-item coordinates mapped with the
// reference's border modes (torchmorph/csrc/grey_kernel.cu:63-97) -- so every
// input voxel is read from HBM once per tile instead of once per tap.  Flat
// boxes are reduced separably (x through shared memory, y and z in
// registers); other elements: each thread owns one (y, x) column of the tile
// and walks the taps over shared memory for its 4 voxels; the taps (offsets and values, up to 1024) sit in
// the launch parameters, their shared-memory offsets are computed once per
// CTA.  Erosion reads x + delta, dilation x - delta, delta = k - (size // 2 +
// origin), with min(v - s) / max(v + s) as in the reference's kernel
// (grey_kernel.cu:101-170, binary_kernel.cu:56-127): bit-identical results.
//
// Uniform batches: a grid of CTAs walks the tiles of all items in order.
// Ragged batches: a plan holds one descriptor per volume {offset, D, H, W,
// first tile, tiles per row and per plane}; persistent CTAs take tile numbers
// from an atomic counter in the plan and find the volume by binary search --
// ONE launch for all volumes, as for the ragged 2-D images (ragged.cu).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "morph_tile.cuh"
#include "tile_queue.cuh"

namespace tmc {
namespace {

using namespace morph;

constexpr int kT3Z = 4, kT3Y = 8, kT3X = 32;
constexpr int kT3Threads = kT3Y * kT3X;  // one (y, x) column of the tile per thread
constexpr int kMax3Taps = 1024;
constexpr size_t kMaxStencil3Smem = 200 * 1024;

struct Taps3 {
    int n;
    int lo[3];   // smallest offset per axis
    int ext[3];  // max - min offset per axis
    int8_t off[3][kMax3Taps];
    float val[kMax3Taps];
};

struct Vol3Item {
    int64_t off;  // first element of the volume in the packed input and output
    int D, H, W;
    int tile_begin;
    int tiles_x, tiles_xy;
    int pad[2];
};
static_assert(sizeof(Vol3Item) == 40, "descriptor layout");

struct Plan3Header {
    int queue;  // next tile to hand out (reset before every launch)
    int ntiles;
    int nitems;
    int pad[61];
};
static_assert(sizeof(Plan3Header) == 256, "plan header is 256 bytes");

struct Uniform3 {  // a uniform batch: `batch` items of D x H x W
    int64_t batch;
    int D, H, W;
    int tiles_x, tiles_xy, tiles_item;
};

// Stage the tile's input region: consecutive threads take consecutive
// elements of the region in raster order (coalesced along x).  Interior tiles
// read straight through; others map every coordinate with the border mode.
// (Measured on the ragged 3-D benchmark: faster than per-row staging with
// several rows' loads in flight per lane, whose lanes idle on rows narrower
// than 64 elements.)
template <typename T>
__device__ __forceinline__ void stage3d(const T *__restrict__ src, T *tile, int D, int H, int W, int gz0, int gy0,
                                        int gx0, int RZ, int RY, int RX, int mode, T cval) {
    const int ryx = RY * RX, total = RZ * ryx;
    const bool interior = gz0 >= 0 && gy0 >= 0 && gx0 >= 0 && gz0 + RZ <= D && gy0 + RY <= H && gx0 + RX <= W;
    if (interior) {
        for (int i = threadIdx.x; i < total; i += kT3Threads) {
            const int rz = i / ryx, r2 = i - rz * ryx, ry = r2 / RX, rx = r2 - ry * RX;
            tile[i] = src[((int64_t)(gz0 + rz) * H + (gy0 + ry)) * W + (gx0 + rx)];
        }
    } else {
        for (int i = threadIdx.x; i < total; i += kT3Threads) {
            const int rz = i / ryx, r2 = i - rz * ryx, ry = r2 / RX, rx = r2 - ry * RX;
            const int mz = map_coord(gz0 + rz, D, mode), my = map_coord(gy0 + ry, H, mode),
                      mx = map_coord(gx0 + rx, W, mode);
            tile[i] = (mz < 0 || my < 0 || mx < 0) ? cval : src[((int64_t)mz * H + my) * W + mx];
        }
    }
}

constexpr int kSepMaxZ = 9;  // flat boxes up to 9 deep take the separable path

// SEP: the element is a full box with one structure value s (flat), at most
// kSepMaxZ deep: the min / max is taken along x into a shared buffer, then
// each thread takes it along y for every staged z and along z in registers,
// and applies s once -- erosion min(v) - s, dilation max(v) + s, equal to the
// per-tap min(v - s) / max(v + s) because rounding is monotone (accumulators
// start at the identity, so NaN inputs are skipped exactly as the tap loop
// skips them).  Otherwise every thread loops over the taps.
template <typename T, bool MAX, bool SEP>
__global__ void __launch_bounds__(kT3Threads) stencil3d_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                               Plan3Header *hdr, const Vol3Item *__restrict__ items,
                                                               Uniform3 u, const __grid_constant__ Taps3 taps,
                                                               int mode, float cval_f) {
    using Op = MorphOp<T, MAX>;
    extern __shared__ __align__(16) unsigned char smem3[];
    const int rz_n = kT3Z + taps.ext[0], RY = kT3Y + taps.ext[1], RX = kT3X + taps.ext[2];
    const int ryx = RY * RX;
    const int n = taps.n;
    int *soff = reinterpret_cast<int *>(smem3);
    T *tile = reinterpret_cast<T *>(smem3 + (((size_t)n * 4 + 15) & ~(size_t)15));
    // SEP: x-reduced rows, (rz, ry) x kT3X
    T *xr = reinterpret_cast<T *>(smem3 + (((size_t)n * 4 + 15) & ~(size_t)15) +
                                  (((size_t)rz_n * ryx * sizeof(T) + 15) & ~(size_t)15));
    __shared__ int s_slot[2];
    __shared__ int s_tb[kQueueCache];
    const int tid = threadIdx.x;
    TileQueue<Vol3Item> q{hdr ? &hdr->queue : nullptr, hdr ? hdr->ntiles : 0, hdr ? hdr->nitems : 0, items, s_tb,
                          s_slot, 0};
    if (hdr) q.init();
    if (!SEP)
        for (int t = tid; t < n; t += kT3Threads)
            soff[t] = (taps.off[0][t] - taps.lo[0]) * ryx + (taps.off[1][t] - taps.lo[1]) * RX +
                      (taps.off[2][t] - taps.lo[2]);
    const T cval = (T)cval_f;
    const int y = tid / kT3X, x = tid % kT3X;
    const int64_t ntiles = hdr ? (int64_t)0 : u.batch * (int64_t)u.tiles_item;
    for (int64_t k = blockIdx.x;; k += gridDim.x) {
        int lt;
        int64_t off;
        int D, H, W, tiles_x, tiles_xy;
        if (hdr) {  // ragged: the next tile from the plan's queue
            __syncthreads();  // the previous tile's readers are done with s_slot and the tile
            if (!q.take()) break;
            const Vol3Item &v = items[s_slot[1]];
            lt = s_slot[0] - v.tile_begin;
            off = v.off;
            D = v.D;
            H = v.H;
            W = v.W;
            tiles_x = v.tiles_x;
            tiles_xy = v.tiles_xy;
        } else {
            if (k >= ntiles) break;
            __syncthreads();  // the previous tile's readers are done with the tile
            const int64_t item = k / u.tiles_item;
            lt = (int)(k - item * u.tiles_item);
            D = u.D;
            H = u.H;
            W = u.W;
            off = item * (int64_t)D * H * W;
            tiles_x = u.tiles_x;
            tiles_xy = u.tiles_xy;
        }
        const int tz = lt / tiles_xy, rem = lt - tz * tiles_xy;
        const int ty = rem / tiles_x, tx = rem - ty * tiles_x;
        const int z0 = tz * kT3Z, y0 = ty * kT3Y, x0 = tx * kT3X;
        stage3d(in + off, tile, D, H, W, z0 + taps.lo[0], y0 + taps.lo[1], x0 + taps.lo[2], rz_n, RY, RX, mode, cval);
        __syncthreads();
        const int zn = min(kT3Z, D - z0);
        if (SEP) {
            const int kx = taps.ext[2] + 1, ky = taps.ext[1] + 1, kz = taps.ext[0] + 1;
            for (int i = tid; i < rz_n * RY * kT3X; i += kT3Threads) {  // along x
                const int row = i / kT3X, c = i - row * kT3X;
                const T *t = tile + row * RX + c;
                T acc = Op::identity();
                for (int dx = 0; dx < kx; dx++) acc = Op::combine(acc, t[dx]);
                xr[i] = acc;
            }
            __syncthreads();
            if (y0 + y < H && x0 + x < W) {
                T a[kT3Z + kSepMaxZ - 1];
#pragma unroll
                for (int rz = 0; rz < kT3Z + kSepMaxZ - 1; rz++) {  // along y, every staged z
                    T acc = Op::identity();
                    if (rz < rz_n)
                        for (int dy = 0; dy < ky; dy++) acc = Op::combine(acc, xr[(rz * RY + y + dy) * kT3X + x]);
                    a[rz] = acc;
                }
                const float sval = taps.val[0];
#pragma unroll
                for (int z = 0; z < kT3Z; z++) {  // along z
                    if (z >= zn) break;
                    T acc = Op::identity();
#pragma unroll
                    for (int dz = 0; dz < kSepMaxZ; dz++)
                        if (dz < kz) acc = Op::combine(acc, a[z + dz]);
                    out[off + ((int64_t)(z0 + z) * H + (y0 + y)) * W + (x0 + x)] = Op::apply(acc, sval);
                }
            }
        } else if (y0 + y < H && x0 + x < W) {
            for (int z = 0; z < zn; z++) {
                const T *base = tile + z * ryx + y * RX + x;
                T acc = Op::identity();
                for (int t = 0; t < n; t++) acc = Op::combine(acc, Op::apply(base[soff[t]], taps.val[t]));
                out[off + ((int64_t)(z0 + z) * H + (y0 + y)) * W + (x0 + x)] = acc;
            }
        }
    }
}

// A full box with one structure value, at most kSepMaxZ deep.
bool taps3_separable(const Taps3 &taps) {
    const int kz = taps.ext[0] + 1, ky = taps.ext[1] + 1, kx = taps.ext[2] + 1;
    if (kz > kSepMaxZ || taps.n != kz * ky * kx) return false;
    for (int t = 1; t < taps.n; t++)
        if (taps.val[t] != taps.val[0]) return false;
    return true;
}

size_t stencil3d_smem(const Taps3 &taps, size_t elem) {
    const size_t rz = kT3Z + taps.ext[0], ry = kT3Y + taps.ext[1];
    const size_t tile = (rz * ry * (kT3X + taps.ext[2]) * elem + 15) & ~(size_t)15;
    return (((size_t)taps.n * 4 + 15) & ~(size_t)15) + tile + (taps3_separable(taps) ? rz * ry * kT3X * elem : 0);
}

// Taps of a 3-D element (torchmorph/csrc/grey_kernel.cu:271-291).
template <bool MAX>
int build_taps3(const float *structure, const uint8_t *footprint, const int64_t *sshape, const int64_t *origin,
                Taps3 *taps) {
    std::memset(taps, 0, sizeof(Taps3));
    for (int d = 0; d < 3; d++) {
        if (sshape[d] < 1 || sshape[d] > 255)
            return fail(TM_ERR_UNSUPPORTED, "3-D structure sizes must be 1..255, got %lld", (long long)sshape[d]);
        if (origin[d] < -(sshape[d] / 2) || origin[d] > (sshape[d] - 1) / 2)
            return fail(TM_ERR_INVALID_ARGUMENT, "invalid origin");
    }
    const int kz = (int)sshape[0], ky = (int)sshape[1], kx = (int)sshape[2];
    const int c[3] = {kz / 2 + (int)origin[0], ky / 2 + (int)origin[1], kx / 2 + (int)origin[2]};
    int n = 0;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int a = 0; a < kz; a++)
        for (int b = 0; b < ky; b++)
            for (int e = 0; e < kx; e++) {
                const int i = (a * ky + b) * kx + e;
                if (footprint && !footprint[i]) continue;
                if (n >= kMax3Taps)
                    return fail(TM_ERR_UNSUPPORTED, "3-D footprints are limited to %d active taps", kMax3Taps);
                const int k[3] = {a, b, e};
                for (int d = 0; d < 3; d++) {
                    const int delta = k[d] - c[d];
                    const int o = MAX ? -delta : delta;
                    taps->off[d][n] = (int8_t)o;
                    lo[d] = n == 0 ? o : std::min(lo[d], o);
                    hi[d] = n == 0 ? o : std::max(hi[d], o);
                }
                taps->val[n] = structure ? structure[i] : 0.0f;
                n++;
            }
    if (n == 0) return fail(TM_ERR_INVALID_ARGUMENT, "footprint must contain at least one active position");
    taps->n = n;
    for (int d = 0; d < 3; d++) {
        taps->lo[d] = lo[d];
        taps->ext[d] = hi[d] - lo[d];
    }
    return TM_OK;
}

// CTAs of one wave for a tile size (cached per device and size).  The
// dynamic shared-memory attribute is set to the largest tile this kernel
// takes, so a cached size never falls below a later launch's.
template <typename T, bool MAX, bool SEP>
int grid_for_kernel(size_t smem, int *grid) {
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
    auto kernel = stencil3d_kernel<T, MAX, SEP>;
    TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxStencil3Smem));
    int per_sm = 0;
    TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kT3Threads, smem));
    if (per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "3-D tile does not fit on an SM");
    cache.push_back({smem, dev, per_sm * sm_count()});
    *grid = per_sm * sm_count();
    return TM_OK;
}

// One launch of the tile kernel: `blocks` CTAs (at most one wave; -1: one
// wave), the separable variant for flat boxes.
template <typename T, bool MAX>
int launch3d(bool sep, int64_t blocks, size_t smem, const T *in, T *out, Plan3Header *hdr, const Vol3Item *items,
             const Uniform3 &u, const Taps3 &taps, int mode, float cval, cudaStream_t s) {
    int grid = 0, st;
    if (sep) st = grid_for_kernel<T, MAX, true>(smem, &grid);
    else st = grid_for_kernel<T, MAX, false>(smem, &grid);
    if (st != TM_OK) return st;
    const unsigned g = (unsigned)(blocks < 0 ? grid : std::min<int64_t>(blocks, grid));
    if (sep) stencil3d_kernel<T, MAX, true><<<g, kT3Threads, smem, s>>>(in, out, hdr, items, u, taps, mode, cval);
    else stencil3d_kernel<T, MAX, false><<<g, kT3Threads, smem, s>>>(in, out, hdr, items, u, taps, mode, cval);
    TM_LAUNCH_CHECK("stencil3d_kernel");
    return TM_OK;
}

template <typename T, bool MAX>
int run_ragged3d(const T *in, T *out, const void *plan, size_t plan_bytes, int64_t n_items, const float *structure,
                 const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
                 cudaStream_t s) {
    if (!in || !out || !plan) return fail(TM_ERR_INVALID_ARGUMENT, "NULL input, output or plan");
    if (in == out) return fail(TM_ERR_INVALID_ARGUMENT, "output must not alias the input");
    if (n_items < 1) return fail(TM_ERR_INVALID_ARGUMENT, "a ragged batch needs at least one volume");
    if (plan_bytes < sizeof(Plan3Header) + (size_t)n_items * sizeof(Vol3Item))
        return fail(TM_ERR_WORKSPACE, "ragged plan buffer too small for %lld volumes", (long long)n_items);
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    if (!sshape || !origin) return fail(TM_ERR_INVALID_ARGUMENT, "structure shape/origin is NULL");
    if (mode < 0 || mode > 4) return fail(TM_ERR_INVALID_ARGUMENT, "unknown border mode %d", mode);
    Taps3 taps;
    int st = build_taps3<MAX>(structure, footprint, sshape, origin, &taps);
    if (st != TM_OK) return st;
    const size_t smem = stencil3d_smem(taps, sizeof(T));
    if (smem > kMaxStencil3Smem) return fail(TM_ERR_UNSUPPORTED, "3-D structure too large for the shared-memory tile");
    auto *hdr = static_cast<Plan3Header *>(const_cast<void *>(plan));
    auto *items = reinterpret_cast<const Vol3Item *>(static_cast<const unsigned char *>(plan) + sizeof(Plan3Header));
    TM_CHECK_CUDA(cudaMemsetAsync(&hdr->queue, 0, sizeof(int), s));
    Uniform3 u{};
    return launch3d<T, MAX>(taps3_separable(taps), -1, smem, in, out, hdr, items, u, taps, mode, cval, s);
}

}  // namespace

// Uniform batches of 3-D items (morphology.cu).  *done = false (nothing
// launched) when the element does not fit the tile kernel; the caller then
// uses its tap-loop kernel.
template <typename T, bool MAX>
int stencil3d_uniform(const T *in, T *out, int64_t batch, const int64_t *shape, const float *structure,
                      const uint8_t *footprint, const int64_t *sshape, const int64_t *origin, int mode, float cval,
                      cudaStream_t s, bool *done) {
    *done = false;
    for (int d = 0; d < 3; d++)
        if (sshape[d] > 255 || shape[d] > (1 << 24)) return TM_OK;
    int64_t active = 0;
    const int64_t stotal = sshape[0] * sshape[1] * sshape[2];
    for (int64_t i = 0; i < stotal; i++) active += !footprint || footprint[i];
    if (active > kMax3Taps) return TM_OK;
    Taps3 taps;
    int st = build_taps3<MAX>(structure, footprint, sshape, origin, &taps);
    if (st != TM_OK) return st;
    const size_t smem = stencil3d_smem(taps, sizeof(T));
    if (smem > kMaxStencil3Smem) return TM_OK;
    Uniform3 u;
    u.batch = batch;
    u.D = (int)shape[0];
    u.H = (int)shape[1];
    u.W = (int)shape[2];
    u.tiles_x = (int)ceil_div(u.W, kT3X);
    u.tiles_xy = u.tiles_x * (int)ceil_div(u.H, kT3Y);
    const int64_t tiles_item = (int64_t)u.tiles_xy * ceil_div(u.D, kT3Z);
    if (tiles_item >= ((int64_t)1 << 31)) return TM_OK;
    u.tiles_item = (int)tiles_item;
    if ((st = launch3d<T, MAX>(taps3_separable(taps), batch * tiles_item, smem, in, out, nullptr, nullptr, u, taps,
                               mode, cval, s)) != TM_OK)
        return st;
    *done = true;
    return TM_OK;
}

template int stencil3d_uniform<float, false>(const float *, float *, int64_t, const int64_t *, const float *,
                                             const uint8_t *, const int64_t *, const int64_t *, int, float,
                                             cudaStream_t, bool *);
template int stencil3d_uniform<float, true>(const float *, float *, int64_t, const int64_t *, const float *,
                                            const uint8_t *, const int64_t *, const int64_t *, int, float,
                                            cudaStream_t, bool *);
template int stencil3d_uniform<uint8_t, false>(const uint8_t *, uint8_t *, int64_t, const int64_t *, const float *,
                                               const uint8_t *, const int64_t *, const int64_t *, int, float,
                                               cudaStream_t, bool *);
template int stencil3d_uniform<uint8_t, true>(const uint8_t *, uint8_t *, int64_t, const int64_t *, const float *,
                                              const uint8_t *, const int64_t *, const int64_t *, int, float,
                                              cudaStream_t, bool *);

}  // namespace tmc

extern "C" size_t tm_ragged3d_plan_size(int64_t n_items) {
    if (n_items < 1) return 0;
    return sizeof(tmc::Plan3Header) + (size_t)n_items * sizeof(tmc::Vol3Item);
}

extern "C" int tm_ragged3d_plan(int64_t n_items, const int64_t *depths, const int64_t *heights, const int64_t *widths,
                                const int64_t *offsets, void *plan, size_t plan_bytes, tm_stream_t stream) {
    using namespace tmc;
    if (n_items < 1 || n_items > (1 << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "n_items must be 1..2^30");
    if (!depths || !heights || !widths || !offsets || !plan) return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (plan_bytes < tm_ragged3d_plan_size(n_items))
        return fail(TM_ERR_WORKSPACE, "ragged plan needs %zu bytes", tm_ragged3d_plan_size(n_items));
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    std::vector<unsigned char> host(tm_ragged3d_plan_size(n_items), 0);
    auto *hdr = reinterpret_cast<Plan3Header *>(host.data());
    auto *items = reinterpret_cast<Vol3Item *>(host.data() + sizeof(Plan3Header));
    int64_t tiles = 0;
    for (int64_t i = 0; i < n_items; i++) {
        const int64_t D = depths[i], H = heights[i], W = widths[i];
        if (D < 1 || H < 1 || W < 1) return fail(TM_ERR_INVALID_ARGUMENT, "volume %lld is empty", (long long)i);
        if (D * H * W >= ((int64_t)1 << 31))
            return fail(TM_ERR_TOO_LARGE, "volume %lld has 2^31 or more voxels", (long long)i);
        if (offsets[i] < 0) return fail(TM_ERR_INVALID_ARGUMENT, "negative offset for volume %lld", (long long)i);
        items[i].off = offsets[i];
        items[i].D = (int)D;
        items[i].H = (int)H;
        items[i].W = (int)W;
        items[i].tiles_x = (int)ceil_div(W, kT3X);
        items[i].tiles_xy = items[i].tiles_x * (int)ceil_div(H, kT3Y);
        items[i].tile_begin = (int)tiles;
        tiles += (int64_t)items[i].tiles_xy * ceil_div(D, kT3Z);
        if (tiles >= ((int64_t)1 << 31) - 65536) return fail(TM_ERR_TOO_LARGE, "too many tiles in one ragged batch");
    }
    hdr->ntiles = (int)tiles;
    hdr->nitems = (int)n_items;
    // pageable source: the call returns once the bytes are staged
    TM_CHECK_CUDA(cudaMemcpyAsync(plan, host.data(), host.size(), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return TM_OK;
}

extern "C" int tm_ragged3d_grey_erosion(const float *in, float *out, const void *plan, size_t plan_bytes,
                                        int64_t n_items, const float *structure, const uint8_t *footprint,
                                        const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                        tm_stream_t stream) {
    return tmc::run_ragged3d<float, false>(in, out, plan, plan_bytes, n_items, structure, footprint, sshape, origin,
                                           mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_ragged3d_grey_dilation(const float *in, float *out, const void *plan, size_t plan_bytes,
                                         int64_t n_items, const float *structure, const uint8_t *footprint,
                                         const int64_t *sshape, const int64_t *origin, int mode, float cval,
                                         tm_stream_t stream) {
    return tmc::run_ragged3d<float, true>(in, out, plan, plan_bytes, n_items, structure, footprint, sshape, origin,
                                          mode, cval, (cudaStream_t)stream);
}

extern "C" int tm_ragged3d_binary_erosion(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                          int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                          const int64_t *origin, int border_value, tm_stream_t stream) {
    return tmc::run_ragged3d<uint8_t, false>(in, out, plan, plan_bytes, n_items, nullptr, structure, sshape, origin,
                                             TM_MODE_CONSTANT, border_value ? 1.0f : 0.0f, (cudaStream_t)stream);
}

extern "C" int tm_ragged3d_binary_dilation(const uint8_t *in, uint8_t *out, const void *plan, size_t plan_bytes,
                                           int64_t n_items, const uint8_t *structure, const int64_t *sshape,
                                           const int64_t *origin, int border_value, tm_stream_t stream) {
    return tmc::run_ragged3d<uint8_t, true>(in, out, plan, plan_bytes, n_items, nullptr, structure, sshape, origin,
                                            TM_MODE_CONSTANT, border_value ? 1.0f : 0.0f, (cudaStream_t)stream);
}
