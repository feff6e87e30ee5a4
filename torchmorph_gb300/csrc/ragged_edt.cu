// Exact EDT of a ragged batch (GB300, sm_103a): every item of a batch of 2-D
// images or 3-D volumes of different shapes in ONE cooperative persistent
// launch.
//
// The transform is the separable one of the uniform operator
// (torchmorph/distance_transform.py:72-102, edt_cuda): pass 0 gives, along
// axis 0, the nearest background voxel of the line; pass a > 0 takes, along
// axis a, the lower envelope of the parabolas (q - p)^2 + g(p) (Felzenszwalb
// and Huttenlocher), exact on int32 / int64 squared distances.  Every pass
// keeps the lowest position on a tie, which makes the feature the nearest
// background voxel with the smallest last-axis coordinate, then the previous
// axis -- scipy.ndimage's choice.  An item without background gets the
// virtual site (-1, 0, ...), as scipy and the reference do.
//
// One pass is one phase of the launch: the lines of ALL items along that
// axis are spread over the threads of the grid (item found by binary search
// over the per-axis line starts), with a bounded grid barrier between
// phases.  A thread walks its line once; adjacent threads own adjacent lines
// so loads along the non-contiguous axes are coalesced; envelope stacks of
// lines up to 256 voxels live in shared memory (interleaved per thread),
// longer ones in the workspace.  The per-item loop the reference runs on the
// host (three axis passes with transposes per item) becomes one launch.
//
// Batches of 3-D items whose axes are all at most ragged_edt3_max_line()
// voxels take the uniform operator's fused plane passes instead
// (edt_compact.cu, ragged_edt3_run): pass 0 as above, then passes 1 + 2 of
// each (item, z) plane on chip by one CTA, with coalesced row stores -- the
// same cooperative single launch, and the same results.
#include <algorithm>
#include <vector>

#include "edt_internal.cuh"

namespace tmc {
namespace {

constexpr int kReThreads = 128;
constexpr int kReSmemL = 256;  // longest line with its stack in shared memory
constexpr int32_t kReInf = 0x7fffffff;

struct RePlanHeader {
    int nitems, ndim;
    int64_t lines[3];
    int64_t total;
    int64_t max_line;
    int pad[52];
};
static_assert(sizeof(RePlanHeader) == 256, "plan header is 256 bytes");

struct ReArgs {
    const void *in;
    int in_f32;
    int ndim;
    int nitems;
    const ReItem *items;
    int64_t lines[3];
    int64_t total;
    int32_t *g[2];
    int32_t *f[2];
    int16_t *gstack;
    int smem_l;  // longest line whose stack fits the shared region (min(max_line, 256))
    float *dist;
    int32_t *indices;
    int32_t *sqdist;
    GridControl *ctl;
    int *status;
    long long spin_limit;
};

// Item of line `line` along `axis` (binary search over the per-axis line starts).
__device__ __forceinline__ int re_item(const ReArgs &A, int axis, int64_t line) {
    int lo = 0, hi = A.nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.items[mid].line_begin[axis] <= line) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Output of the voxel at packed position `pos` (item-local flat index
// `q_flat`) with feature `f` (item-local flat index, -1: the item has no
// background) and squared distance `s2`.
__device__ __forceinline__ void re_write(const ReArgs &A, const ReItem &it, int64_t pos, int64_t q_flat, int32_t f,
                                         int64_t s2) {
    const int nd = A.ndim;
    int fc[3] = {0, 0, 0}, qc[3] = {0, 0, 0};
    if (nd == 3) {
        const int H = it.shape[1], W = it.shape[2];
        qc[0] = (int)(q_flat / ((int64_t)H * W));
        qc[1] = (int)((q_flat / W) % H);
        qc[2] = (int)(q_flat % W);
        if (f >= 0) {
            fc[0] = f / (H * W);
            fc[1] = (f / W) % H;
            fc[2] = f % W;
        }
    } else {
        const int W = it.shape[1];
        qc[0] = (int)(q_flat / W);
        qc[1] = (int)(q_flat % W);
        if (f >= 0) {
            fc[0] = f / W;
            fc[1] = f % W;
        }
    }
    if (f < 0) {  // no background in the item: the virtual site (-1, 0, ...)
        fc[0] = -1;
        s2 = (int64_t)(qc[0] + 1) * (qc[0] + 1);
        for (int d = 1; d < nd; d++) s2 += (int64_t)qc[d] * qc[d];
    }
    if (A.dist) A.dist[pos] = __fsqrt_rn((float)s2);  // exact integer below 2^24: correctly rounded
    if (A.sqdist) A.sqdist[pos] = (int32_t)s2;
    if (A.indices)
        for (int d = 0; d < nd; d++) A.indices[(int64_t)d * A.total + pos] = fc[d];
}

__global__ void __launch_bounds__(kReThreads) ragged_edt_kernel(ReArgs A) {
    extern __shared__ int16_t re_stack[];  // [smem_l][kReThreads]
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int a = 0; a < A.ndim; a++) {
        const bool last = a == A.ndim - 1;
        const int32_t *gin = a == 0 ? nullptr : A.g[(a - 1) & 1];
        const int32_t *fin = a == 0 ? nullptr : A.f[(a - 1) & 1];
        int32_t *gout = last ? nullptr : A.g[a & 1];
        int32_t *fout = last ? nullptr : A.f[a & 1];
        for (int64_t line = gtid; line < A.lines[a]; line += nthreads) {
            const ReItem &it = A.items[re_item(A, a, line)];
            const int64_t local = line - it.line_begin[a];
            int64_t inner = 1;
            for (int d = a + 1; d < A.ndim; d++) inner *= it.shape[d];
            const int L = it.shape[a];
            const int64_t outer = local / inner, in_off = local - outer * inner;
            const int64_t lbase = outer * L * inner + in_off;  // item-local flat index of q = 0
            const int64_t base = it.off + lbase;
            if (a == 0) {  // items have 2 or 3 axes: pass 0 is never the last
                // nearest background along the line; ties to the lower position.
                // Forward sweep: the last background at or before q; the inputs of 8
                // voxels are loaded before any is used (8 loads in flight per thread).
                int prev = -1;
                for (int q0 = 0; q0 < L; q0 += 8) {
                    bool bg[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const int64_t p = base + (int64_t)(q0 + u) * inner;
                        bg[u] = q0 + u < L && (A.in_f32 ? static_cast<const float *>(A.in)[p] == 0.0f
                                                        : static_cast<const uint8_t *>(A.in)[p] == 0);
                    }
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const int q = q0 + u;
                        if (q >= L) break;
                        const int64_t p = base + (int64_t)q * inner;
                        if (bg[u]) prev = q;
                        gout[p] = prev < 0 ? kReInf : (q - prev) * (q - prev);
                        fout[p] = prev < 0 ? -1 : (int32_t)(lbase + (int64_t)prev * inner);
                    }
                }
                // backward sweep: the first background after q, taken only when strictly closer
                int next = -1;
                for (int q0 = ((L - 1) / 8) * 8; q0 >= 0; q0 -= 8) {
                    int32_t gv[8];
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        gv[u] = q0 + u < L ? gout[base + (int64_t)(q0 + u) * inner] : kReInf;
#pragma unroll
                    for (int u = 7; u >= 0; u--) {
                        const int q = q0 + u;
                        if (q >= L) continue;
                        if (gv[u] == 0) {
                            next = q;
                        } else if (next >= 0) {
                            const int32_t gn = (next - q) * (next - q);
                            if (gn < gv[u]) {
                                const int64_t p = base + (int64_t)q * inner;
                                gout[p] = gn;
                                fout[p] = (int32_t)(lbase + (int64_t)next * inner);
                            }
                        }
                    }
                }
                continue;
            }
            // lower envelope of the parabolas (q - p)^2 + g(p) over the finite g;
            // the two topmost entries (position, g + position^2) stay in registers
            const bool smem = L <= A.smem_l;
            auto push = [&](int k, int v) {
                if (smem) re_stack[k * kReThreads + threadIdx.x] = (int16_t)v;
                else A.gstack[base + (int64_t)k * inner] = (int16_t)v;
            };
            auto peek = [&](int k) -> int {
                return smem ? re_stack[k * kReThreads + threadIdx.x] : A.gstack[base + (int64_t)k * inner];
            };
            // the previous pass's planes were written by other SMs: L2 loads, never a stale L1 line
            auto G = [&](int q) -> int32_t { return __ldcg(gin + base + (int64_t)q * inner); };
            int k = -1, top = 0, sec = 0;
            int64_t Gtop = 0, Gsec = 0;
            for (int q0 = 0; q0 < L; q0 += 8) {
                int32_t gv[8];
#pragma unroll
                for (int u = 0; u < 8; u++) gv[u] = q0 + u < L ? G(q0 + u) : kReInf;
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int q = q0 + u;
                    if (gv[u] == kReInf) continue;  // also every q >= L
                    const int64_t Gq = (int64_t)gv[u] + (int64_t)q * q;
                    while (k >= 1) {
                        // pop top when the intersection with q is at or left of the one with sec
                        if ((Gq - Gtop) * (top - sec) > (Gtop - Gsec) * (q - top)) break;
                        k--;
                        top = sec;
                        Gtop = Gsec;
                        if (k >= 1) {
                            sec = peek(k - 1);
                            Gsec = (int64_t)G(sec) + (int64_t)sec * sec;
                        }
                    }
                    push(++k, q);
                    sec = top;
                    Gsec = Gtop;
                    top = q;
                    Gtop = Gq;
                }
            }
            // walk the envelope: cur and the next entry with their g in registers
            int j = 0, cur = 0, nxt = 0;
            int64_t gcur = 0, gnxt = 0;
            int32_t fcur = -1;
            if (k >= 0) {
                cur = peek(0);
                gcur = G(cur);
                fcur = __ldcg(fin + base + (int64_t)cur * inner);
                if (k >= 1) {
                    nxt = peek(1);
                    gnxt = G(nxt);
                }
            }
            for (int q = 0; q < L; q++) {
                const int64_t p = base + (int64_t)q * inner;
                int64_t s = kReInf;
                if (k >= 0) {
                    s = (int64_t)(q - cur) * (q - cur) + gcur;
                    while (j < k) {
                        const int64_t sn = (int64_t)(q - nxt) * (q - nxt) + gnxt;
                        if (!(sn < s)) break;  // ties keep the lower position
                        j++;
                        cur = nxt;
                        gcur = gnxt;
                        s = sn;
                        fcur = __ldcg(fin + base + (int64_t)cur * inner);
                        if (j < k) {
                            nxt = peek(j + 1);
                            gnxt = G(nxt);
                        }
                    }
                }
                if (!last) {
                    gout[p] = s >= kReInf ? kReInf : (int32_t)s;
                    fout[p] = k >= 0 ? fcur : -1;
                } else {
                    re_write(A, it, p, lbase + (int64_t)q * inner, k >= 0 ? fcur : -1, s);
                }
            }
        }
        if (!last && !grid_barrier_bounded(A.ctl, gridDim.x, A.status, A.spin_limit)) return;
    }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace tmc

extern "C" size_t tm_ragged_edt_plan_size(int64_t n_items) {
    if (n_items < 1) return 0;
    return sizeof(tmc::RePlanHeader) + (size_t)n_items * sizeof(tmc::ReItem);
}

extern "C" int tm_ragged_edt_plan(int64_t n_items, int ndim, const int64_t *shapes, const int64_t *offsets, void *plan,
                                  size_t plan_bytes, tm_stream_t stream) {
    using namespace tmc;
    if (n_items < 1 || n_items > (1 << 30)) return fail(TM_ERR_INVALID_ARGUMENT, "n_items must be 1..2^30");
    if (ndim != 2 && ndim != 3) return fail(TM_ERR_UNSUPPORTED, "ragged EDT items must be 2-D or 3-D");
    if (!shapes || !offsets || !plan) return fail(TM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (plan_bytes < tm_ragged_edt_plan_size(n_items))
        return fail(TM_ERR_WORKSPACE, "ragged EDT plan needs %zu bytes", tm_ragged_edt_plan_size(n_items));
    if (((uintptr_t)plan & 255) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "ragged plan must be 256-byte aligned");
    std::vector<unsigned char> host(tm_ragged_edt_plan_size(n_items), 0);
    auto *hdr = reinterpret_cast<RePlanHeader *>(host.data());
    auto *items = reinterpret_cast<ReItem *>(host.data() + sizeof(RePlanHeader));
    int64_t lines[3] = {0, 0, 0}, total = 0, max_line = 0, planes = 0;
    for (int64_t i = 0; i < n_items; i++) {
        int64_t n = 1, sq = 0;
        for (int d = 0; d < ndim; d++) {
            const int64_t v = shapes[i * ndim + d];
            if (v < 1) return fail(TM_ERR_INVALID_ARGUMENT, "item %lld is empty", (long long)i);
            if (v > 32767)
                return fail(TM_ERR_TOO_LARGE, "item %lld: axis length %lld above 32767", (long long)i, (long long)v);
            n *= v;
            sq += (v + 1) * (v + 1);
            max_line = std::max(max_line, v);
        }
        if (n >= ((int64_t)1 << 31) || sq >= kReInf)
            return fail(TM_ERR_TOO_LARGE, "item %lld is too large for 32-bit squared distances", (long long)i);
        if (offsets[i] < 0) return fail(TM_ERR_INVALID_ARGUMENT, "negative offset for item %lld", (long long)i);
        items[i].off = offsets[i];
        for (int d = 0; d < 3; d++) items[i].shape[d] = d < ndim ? (int)shapes[i * ndim + d] : 1;
        if (planes >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "more than 2^31 - 1 planes");
        items[i].plane_begin = (int)planes;
        planes += shapes[i * ndim];
        for (int d = 0; d < ndim; d++) {
            items[i].line_begin[d] = lines[d];
            lines[d] += n / shapes[i * ndim + d];
        }
        total = std::max(total, offsets[i] + n);
    }
    hdr->nitems = (int)n_items;
    hdr->ndim = ndim;
    for (int d = 0; d < 3; d++) hdr->lines[d] = lines[d];
    hdr->total = total;
    hdr->max_line = max_line;
    // pageable source: the call returns once the bytes are staged
    TM_CHECK_CUDA(cudaMemcpyAsync(plan, host.data(), host.size(), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return TM_OK;
}

// Workspace: ping-pong (g, f) int32 planes of `total` voxels, the envelope
// stacks of lines longer than 256 (int16), and the launch's control block.
extern "C" size_t tm_ragged_edt_workspace_size(int64_t total, int64_t max_line) {
    using namespace tmc;
    if (total < 1) return 0;
    const size_t n = (size_t)total;
    return 4 * align256(n * 4) + (max_line > kReSmemL ? align256(n * 2) : 0) + sizeof(GridControl);
}

extern "C" int tm_ragged_edt(const void *input, int in_dtype, const void *plan, size_t plan_bytes, int64_t n_items,
                             int ndim, int64_t total, int64_t max_line, const int64_t *lines, float *dist,
                             int32_t *indices, int32_t *sqdist, void *workspace, size_t workspace_bytes,
                             tm_stream_t stream) {
    using namespace tmc;
    if (!input || !plan || !lines) return fail(TM_ERR_INVALID_ARGUMENT, "NULL input, plan or line counts");
    if (in_dtype != TM_F32 && in_dtype != TM_U8) return fail(TM_ERR_INVALID_ARGUMENT, "unknown input dtype %d", in_dtype);
    if (ndim != 2 && ndim != 3) return fail(TM_ERR_UNSUPPORTED, "ragged EDT items must be 2-D or 3-D");
    if (!dist && !indices && !sqdist) return fail(TM_ERR_INVALID_ARGUMENT, "at least one output must be requested");
    if (n_items < 1 || plan_bytes < tm_ragged_edt_plan_size(n_items))
        return fail(TM_ERR_WORKSPACE, "ragged EDT plan too small for %lld items", (long long)n_items);
    if (total < 1 || max_line < 1) return fail(TM_ERR_INVALID_ARGUMENT, "empty ragged batch");
    const size_t need = tm_ragged_edt_workspace_size(total, max_line);
    if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255))
        return fail(TM_ERR_WORKSPACE, "workspace must be 256-byte aligned and hold %zu bytes", need);
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    const size_t n = (size_t)total;
    ReArgs A{};
    A.in = input;
    A.in_f32 = in_dtype == TM_F32;
    A.ndim = ndim;
    A.nitems = (int)n_items;
    A.items = reinterpret_cast<const ReItem *>(static_cast<const unsigned char *>(plan) + sizeof(RePlanHeader));
    int64_t max_lines = 0;
    for (int d = 0; d < 3; d++) {
        A.lines[d] = d < ndim ? lines[d] : 0;
        max_lines = std::max(max_lines, A.lines[d]);
    }
    A.total = total;
    for (int b = 0; b < 2; b++) {
        A.g[b] = reinterpret_cast<int32_t *>(ws + (2 * b) * align256(n * 4));
        A.f[b] = reinterpret_cast<int32_t *>(ws + (2 * b + 1) * align256(n * 4));
    }
    size_t off = 4 * align256(n * 4);
    A.gstack = max_line > kReSmemL ? reinterpret_cast<int16_t *>(ws + off) : nullptr;
    if (A.gstack) off += align256(n * 2);
    A.ctl = reinterpret_cast<GridControl *>(ws + off);
    A.dist = dist;
    A.indices = indices;
    A.sqdist = sqdist;
    int st = device_status_word(&A.status);
    if (st != TM_OK) return st;
    A.spin_limit = grid_wait_budget();
    // the shared stack region holds the longest line's stack (up to 256 entries),
    // so short lines leave room for more CTAs per SM
    if (ndim == 3 && max_line <= ragged_edt3_max_line())  // every plane fits on chip
        return ragged_edt3_run(input, A.in_f32, A.items, A.nitems, A.lines[0], total, (int)max_line,
                               reinterpret_cast<int16_t *>(A.g[0]), dist, indices, sqdist, A.ctl, s);
    A.smem_l = (int)std::min<int64_t>(max_line, kReSmemL);
    const size_t smem = (size_t)A.smem_l * kReThreads * sizeof(int16_t);
    static thread_local int cached_dev = -1, cached_per_sm = 0;
    static thread_local size_t cached_smem = 0;
    int dev = 0;
    TM_CHECK_CUDA(cudaGetDevice(&dev));
    if (cached_dev != dev || cached_smem != smem) {
        TM_CHECK_CUDA(cudaFuncSetAttribute(ragged_edt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)((size_t)kReSmemL * kReThreads * sizeof(int16_t))));
        TM_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_per_sm, ragged_edt_kernel, kReThreads,
                                                                    smem));
        cached_dev = dev;
        cached_smem = smem;
    }
    if (cached_per_sm < 1) return fail(TM_ERR_UNSUPPORTED, "ragged EDT kernel does not fit on an SM");
    const int64_t blocks =
        std::max<int64_t>(1, std::min<int64_t>((int64_t)cached_per_sm * sm_count(), ceil_div(max_lines, kReThreads)));
    TM_CHECK_CUDA(cudaMemsetAsync(A.ctl, 0, sizeof(GridControl), s));
    void *params[] = {&A};
    TM_CHECK_CUDA(cudaLaunchCooperativeKernel((const void *)ragged_edt_kernel, dim3((unsigned)blocks),
                                              dim3(kReThreads), params, smem, s));
    TM_LAUNCH_CHECK("ragged_edt_kernel");
    return TM_OK;
}
