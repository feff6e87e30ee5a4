// Exact Euclidean distance transform for GB300 (sm_103a).
//
// Replaces the reference's edt_cuda (torchmorph/csrc/edt_kernel.cu:904-958).
// The transform is separable: pass a (axis order 0..n-1) computes, for every
// voxel q of every line along axis a,
//     g_a(q) = min_p (q - p)^2 * s_a^2 + g_{a-1}(p),
// keeping the LOWEST p on a tie and carrying p's feature (a flat voxel index
// inside the item).  With this order and tie rule the final feature is the
// nearest background voxel with the smallest last-axis coordinate, then the
// smallest previous-axis coordinate, ... -- scipy.ndimage's result, which the
// reference's tests use as their oracle.
//
//   pass 0   edt_scan_kernel: axis 0 only sees the binary input, so the
//            minimum is the distance to the nearest background along the
//            line.  One thread per line walks the line once and resolves
//            each foreground run when its closing background arrives
//            (O(1) state, every element read and written once).
//   pass a>0 edt_envelope_kernel: Felzenszwalb-Huttenlocher lower envelope,
//            one thread per line.  Adjacent threads own adjacent lines, so
//            every load and store along a non-contiguous axis is coalesced.
//            The envelope stack holds only positions (int16 in shared
//            memory, interleaved across threads; int32 in the workspace for
//            lines too long for shared memory); the parabola values are
//            re-read from the line, and the two topmost entries live in
//            registers, so the intersection test needs no memory access
//            except after a pop.
//   Unit spacing runs on exact int32 squared distances: the intersection
//   test is cross-multiplied into 32x32->64-bit products, no division.
//   Sampled spacing runs the envelope in float (as the reference does) and
//   computes the output distance from the final feature in double, the
//   way scipy does.
//   The last pass writes the public outputs: float32 distance (correctly
//   rounded sqrt), int32 feature indices, and optionally int32 squared
//   distances.  An item without any background gets the reference/scipy
//   "virtual background" at (-1, 0, ..., 0)
//   (torchmorph/csrc/edt_kernel.cu:415-437).
#include <cmath>
#include <cstring>
#include <type_traits>

#include "edt_internal.cuh"

namespace tmc {
namespace {

constexpr int kEdtThreads = 128;
constexpr int kSmemStackMaxL = 768;  // longer lines keep their stack in the workspace
constexpr int32_t kInfI = 0x7fffffff;

struct EdtParams {
    int ndim;
    int axis;
    int L;               // line length (shape[axis])
    int64_t inner;       // product of the sizes after axis (element stride of the line)
    int64_t nlines;      // batch * numel_item / L
    int64_t numel;       // batch * numel_item
    int64_t numel_item;
    int64_t lines_per_item;
    FastDiv inner_div;   // divides a line index into (outer, inner)
    FastDiv stride_div[TM_MAX_NDIM];  // spatial strides, to unravel features
    int shape[TM_MAX_NDIM];
    float spacing;       // sampling[axis]
    float sampling[TM_MAX_NDIM];
    int sampled;         // 0: exact int32 path
    int in_f32;          // input dtype of pass 0
};

struct EdtOutputs {
    float *dist;
    int32_t *indices;
    int32_t *sqdist;
};

template <typename V>
struct Val;
template <>
struct Val<int32_t> {
    __device__ __forceinline__ static bool inf(int32_t v) { return v == kInfI; }
    __device__ __forceinline__ static int32_t infv() { return kInfI; }
};
template <>
struct Val<float> {
    __device__ __forceinline__ static bool inf(float v) { return isinf(v); }
    __device__ __forceinline__ static float infv() { return INFINITY; }
};

// Final outputs of one voxel.  gi: global element index; feat: flat feature
// inside the item or -1 for "no background in the item" (virtual site).
template <typename V>
__device__ __forceinline__ void emit_final(const EdtParams &p, const EdtOutputs &o, int64_t gi,
                                           int64_t item, int32_t feat, V d2) {
    const uint32_t vox = (uint32_t)(gi - item * p.numel_item);
    int fc[TM_MAX_NDIM];
    int xc[TM_MAX_NDIM];
    uint32_t rv = vox, rf = (uint32_t)feat;
#pragma unroll
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        if (d < p.ndim) {
            uint32_t qx = fdiv(rv, p.stride_div[d]);
            rv -= qx * p.stride_div[d].d;
            xc[d] = (int)qx;
            if (feat >= 0) {
                uint32_t qf = fdiv(rf, p.stride_div[d]);
                rf -= qf * p.stride_div[d].d;
                fc[d] = (int)qf;
            } else {
                fc[d] = d == 0 ? -1 : 0;
            }
        }
    }
    if (o.indices) {
#pragma unroll
        for (int d = 0; d < TM_MAX_NDIM; d++)
            if (d < p.ndim) o.indices[(int64_t)d * p.numel + gi] = fc[d];
    }
    if (!p.sampled) {
        int32_t s2;
        if (feat >= 0) {
            s2 = (int32_t)d2;
        } else {
            s2 = 0;
#pragma unroll
            for (int d = 0; d < TM_MAX_NDIM; d++)
                if (d < p.ndim) s2 += (xc[d] - fc[d]) * (xc[d] - fc[d]);
        }
        if (o.sqdist) o.sqdist[gi] = s2;
        if (o.dist) {
            // float(s2) is exact below 2^24, and a correctly rounded float
            // sqrt of an exact input equals float(sqrt_double(s2)).
            o.dist[gi] = s2 < (1 << 24) ? __fsqrt_rn((float)s2) : (float)sqrt((double)s2);
        }
    } else if (o.dist) {
        double acc = 0.0;
#pragma unroll
        for (int d = 0; d < TM_MAX_NDIM; d++) {
            if (d < p.ndim) {
                double t = (double)(xc[d] - fc[d]) * (double)p.sampling[d];
                acc += t * t;
            }
        }
        o.dist[gi] = (float)sqrt(acc);
    }
}

// ------------------------------------------------------------------ pass 0
template <typename V>
__device__ __forceinline__ V scan_d2(int dz, float s);
template <>
__device__ __forceinline__ int32_t scan_d2<int32_t>(int dz, float) { return dz * dz; }
template <>
__device__ __forceinline__ float scan_d2<float>(int dz, float s) {
    float t = (float)dz * s;
    return t * t;
}

template <typename In, typename V, bool FINAL>
__global__ void __launch_bounds__(kEdtThreads) edt_scan_kernel(const In *__restrict__ in, V *__restrict__ g_out,
                                                               int32_t *__restrict__ f_out, EdtParams p,
                                                               EdtOutputs o) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.nlines) return;
    // line -> (outer, inner); pass 0 has outer == item
    const int64_t outer = (int64_t)fdiv((uint32_t)line, p.inner_div);
    const int64_t inner = line - outer * p.inner;
    const int64_t base = outer * p.L * p.inner + inner;
    const int64_t item = outer;
    const int L = p.L;
    const float s = p.spacing;
    int last = -1;  // previous background position
    for (int q = 0; q < L; q++) {
        const int64_t gi = base + (int64_t)q * p.inner;
        if (in[gi] != (In)0) continue;
        // resolve the foreground run (last, q)
        for (int z = last + 1; z < q; z++) {
            int pz = (last >= 0 && z - last <= q - z) ? last : q;
            int dz = z - pz;
            const int64_t gz = base + (int64_t)z * p.inner;
            int32_t feat = (int32_t)((int64_t)pz * p.inner + inner);
            V d2 = scan_d2<V>(dz, s);
            if (FINAL)
                emit_final<V>(p, o, gz, item, feat, d2);
            else {
                g_out[gz] = d2;
                f_out[gz] = feat;
            }
        }
        int32_t featq = (int32_t)((int64_t)q * p.inner + inner);
        if (FINAL)
            emit_final<V>(p, o, gi, item, featq, (V)0);
        else {
            g_out[gi] = (V)0;
            f_out[gi] = featq;
        }
        last = q;
    }
    for (int z = last + 1; z < L; z++) {
        const int64_t gz = base + (int64_t)z * p.inner;
        if (last >= 0) {
            int dz = z - last;
            int32_t feat = (int32_t)((int64_t)last * p.inner + inner);
            V d2 = scan_d2<V>(dz, s);
            if (FINAL)
                emit_final<V>(p, o, gz, item, feat, d2);
            else {
                g_out[gz] = d2;
                f_out[gz] = feat;
            }
        } else {
            if (FINAL)
                emit_final<V>(p, o, gz, item, -1, (V)0);
            else {
                g_out[gz] = Val<V>::infv();
                f_out[gz] = -1;
            }
        }
    }
}

// ------------------------------------------------------- pass a > 0 (FH)
struct SmemStack {
    int16_t *base;
    int nthreads;
    int tid;
    __device__ __forceinline__ int get(int k) const { return base[k * nthreads + tid]; }
    __device__ __forceinline__ void set(int k, int v) { base[k * nthreads + tid] = (int16_t)v; }
};
struct GlobalStack {
    int32_t *base;
    int64_t nlines;
    int64_t line;
    __device__ __forceinline__ int get(int k) const { return base[(int64_t)k * nlines + line]; }
    __device__ __forceinline__ void set(int k, int v) { base[(int64_t)k * nlines + line] = v; }
};

// Squared-position term of a parabola focus; exact in the int path.
template <typename V>
__device__ __forceinline__ V pos2(int q, float s);
template <>
__device__ __forceinline__ int32_t pos2<int32_t>(int q, float) { return q * q; }
template <>
__device__ __forceinline__ float pos2<float>(int q, float s) {
    float P = (float)q * s;
    return P * P;
}

// Pop test: is the top parabola r (below it p) hidden once q is added, i.e.
// s(q, r) <= s(r, p)?  Cross-multiplied; denominators are positive.
__device__ __forceinline__ bool hides(int32_t Gq, int32_t Gr, int32_t Gp, int q, int r, int pp, float) {
    long long lhs = (long long)(Gq - Gr) * (long long)(r - pp);
    long long rhs = (long long)(Gr - Gp) * (long long)(q - r);
    return lhs <= rhs;
}
__device__ __forceinline__ bool hides(float Gq, float Gr, float Gp, int q, int r, int pp, float s) {
    return (Gq - Gr) * ((float)(r - pp) * s) <= (Gr - Gp) * ((float)(q - r) * s);
}

// Value of parabola (focus pos, offset g) at q, in a type wide enough.
__device__ __forceinline__ uint32_t pval(int q, int pos, int32_t g, float) {
    int d = q - pos;
    return (uint32_t)(d * d) + (uint32_t)g;
}
__device__ __forceinline__ float pval(int q, int pos, float g, float s) {
    float d = (float)(q - pos) * s;
    return d * d + g;
}

template <typename V, bool FINAL, typename Stack>
__device__ __forceinline__ void envelope_line(const V *__restrict__ g_in, const int32_t *__restrict__ f_in,
                                              V *__restrict__ g_out, int32_t *__restrict__ f_out,
                                              const EdtParams &p, const EdtOutputs &o, Stack st,
                                              int64_t base, int64_t item) {
    const int L = p.L;
    const int64_t step = p.inner;
    const float s = p.spacing;
    int k = -1;
    int top = 0, sec = 0;
    V Gtop = 0, Gsec = 0;
    for (int q = 0; q < L; q++) {
        const V gq = g_in[base + (int64_t)q * step];
        if (Val<V>::inf(gq)) continue;
        const V Gq = gq + pos2<V>(q, s);
        while (k >= 1 && hides(Gq, Gtop, Gsec, q, top, sec, s)) {
            k--;
            top = sec;
            Gtop = Gsec;
            if (k >= 1) {
                sec = st.get(k - 1);
                Gsec = g_in[base + (int64_t)sec * step] + pos2<V>(sec, s);
            }
        }
        k++;
        st.set(k, q);
        sec = top;
        Gsec = Gtop;
        top = q;
        Gtop = Gq;
    }
    if (k < 0) {
        for (int q = 0; q < L; q++) {
            const int64_t gi = base + (int64_t)q * step;
            if (FINAL)
                emit_final<V>(p, o, gi, item, -1, (V)0);
            else {
                g_out[gi] = Val<V>::infv();
                f_out[gi] = -1;
            }
        }
        return;
    }
    int j = 0;
    int cur = st.get(0);
    V gcur = g_in[base + (int64_t)cur * step];
    int nxt = 0;
    V gnxt = 0;
    if (k >= 1) {
        nxt = st.get(1);
        gnxt = g_in[base + (int64_t)nxt * step];
    }
    for (int q = 0; q < L; q++) {
        auto fcur = pval(q, cur, gcur, s);
        while (j < k) {
            auto fn = pval(q, nxt, gnxt, s);
            if (!(fn < fcur)) break;  // ties keep the lower position
            j++;
            cur = nxt;
            gcur = gnxt;
            fcur = fn;
            if (j < k) {
                nxt = st.get(j + 1);
                gnxt = g_in[base + (int64_t)nxt * step];
            }
        }
        const int64_t gi = base + (int64_t)q * step;
        const int32_t feat = f_in[base + (int64_t)cur * step];
        const V d2 = (V)fcur;
        if (FINAL)
            emit_final<V>(p, o, gi, item, feat, d2);
        else {
            g_out[gi] = d2;
            f_out[gi] = feat;
        }
    }
}

template <typename V, bool FINAL>
__global__ void __launch_bounds__(kEdtThreads) edt_envelope_smem_kernel(const V *__restrict__ g_in,
                                                                        const int32_t *__restrict__ f_in,
                                                                        V *__restrict__ g_out,
                                                                        int32_t *__restrict__ f_out, EdtParams p,
                                                                        EdtOutputs o) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.nlines) return;
    SmemStack st{reinterpret_cast<int16_t *>(smem_raw), (int)blockDim.x, (int)threadIdx.x};
    const int64_t outer = (int64_t)fdiv((uint32_t)line, p.inner_div);
    const int64_t inner = line - outer * p.inner;
    const int64_t base = outer * p.L * p.inner + inner;
    const int64_t item = line / p.lines_per_item;
    envelope_line<V, FINAL>(g_in, f_in, g_out, f_out, p, o, st, base, item);
}

template <typename V, bool FINAL>
__global__ void __launch_bounds__(kEdtThreads) edt_envelope_gmem_kernel(const V *__restrict__ g_in,
                                                                        const int32_t *__restrict__ f_in,
                                                                        V *__restrict__ g_out,
                                                                        int32_t *__restrict__ f_out,
                                                                        int32_t *__restrict__ stack, EdtParams p,
                                                                        EdtOutputs o) {
    const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.nlines) return;
    GlobalStack st{stack, p.nlines, line};
    const int64_t outer = (int64_t)fdiv((uint32_t)line, p.inner_div);
    const int64_t inner = line - outer * p.inner;
    const int64_t base = outer * p.L * p.inner + inner;
    const int64_t item = line / p.lines_per_item;
    envelope_line<V, FINAL>(g_in, f_in, g_out, f_out, p, o, st, base, item);
}

// ----------------------------------------------------------------- host
inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct EdtPlan {
    size_t g_bytes, f_bytes, stack_bytes, total;
    int nbuf;
    bool gstack;
};

EdtPlan plan_edt(const Geometry &g) {
    EdtPlan pl;
    const size_t n = (size_t)g.numel;
    pl.g_bytes = align256(n * 4);
    pl.f_bytes = align256(n * 4);
    pl.nbuf = g.ndim == 1 ? 0 : (g.ndim == 2 ? 1 : 2);
    pl.gstack = false;
    for (int a = 1; a < g.ndim; a++)
        if (g.shape[a] > kSmemStackMaxL) pl.gstack = true;
    pl.stack_bytes = pl.gstack ? align256(n * 4) : 0;
    pl.total = pl.nbuf * (pl.g_bytes + pl.f_bytes) + pl.stack_bytes;
    return pl;
}

template <typename In, typename V>
int launch_edt(const In *in, const Geometry &g, const float *sampling, EdtOutputs o, unsigned char *ws,
               const EdtPlan &pl, cudaStream_t stream) {
    EdtParams p;
    std::memset(&p, 0, sizeof(p));
    p.ndim = g.ndim;
    p.numel = g.numel;
    p.numel_item = g.numel_item;
    p.sampled = std::is_same<V, float>::value ? 1 : 0;
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        p.stride_div[d] = make_fastdiv(d < g.ndim ? (uint32_t)g.stride[d] : 1u);
        p.shape[d] = d < g.ndim ? (int)g.shape[d] : 1;
        p.sampling[d] = (d < g.ndim && sampling) ? sampling[d] : 1.0f;
    }
    V *gbuf[2] = {nullptr, nullptr};
    int32_t *fbuf[2] = {nullptr, nullptr};
    for (int b = 0; b < pl.nbuf; b++) {
        gbuf[b] = reinterpret_cast<V *>(ws + b * (pl.g_bytes + pl.f_bytes));
        fbuf[b] = reinterpret_cast<int32_t *>(ws + b * (pl.g_bytes + pl.f_bytes) + pl.g_bytes);
    }
    int32_t *gstack = pl.gstack ? reinterpret_cast<int32_t *>(ws + pl.nbuf * (pl.g_bytes + pl.f_bytes)) : nullptr;
    for (int a = 0; a < g.ndim; a++) {
        p.axis = a;
        p.L = (int)g.shape[a];
        p.inner = g.stride[a];
        p.nlines = g.numel / p.L;
        p.lines_per_item = g.numel_item / p.L;
        p.inner_div = make_fastdiv((uint32_t)p.inner);
        p.spacing = p.sampling[a];
        const bool final_pass = a == g.ndim - 1;
        const unsigned blocks = (unsigned)ceil_div(p.nlines, kEdtThreads);
        V *gout = final_pass ? nullptr : gbuf[a & 1];
        int32_t *fout = final_pass ? nullptr : fbuf[a & 1];
        const V *gin = a == 0 ? nullptr : gbuf[(a - 1) & 1];
        const int32_t *fin = a == 0 ? nullptr : fbuf[(a - 1) & 1];
        if (a == 0) {
            if (final_pass)
                edt_scan_kernel<In, V, true><<<blocks, kEdtThreads, 0, stream>>>(in, gout, fout, p, o);
            else
                edt_scan_kernel<In, V, false><<<blocks, kEdtThreads, 0, stream>>>(in, gout, fout, p, o);
            TM_LAUNCH_CHECK("edt_scan_kernel");
        } else if (p.L <= kSmemStackMaxL) {
            size_t smem = (size_t)kEdtThreads * p.L * sizeof(int16_t);
            if (final_pass) {
                if (smem > 48 * 1024)
                    TM_CHECK_CUDA(cudaFuncSetAttribute(edt_envelope_smem_kernel<V, true>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                edt_envelope_smem_kernel<V, true><<<blocks, kEdtThreads, smem, stream>>>(gin, fin, gout, fout, p, o);
            } else {
                if (smem > 48 * 1024)
                    TM_CHECK_CUDA(cudaFuncSetAttribute(edt_envelope_smem_kernel<V, false>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                edt_envelope_smem_kernel<V, false><<<blocks, kEdtThreads, smem, stream>>>(gin, fin, gout, fout, p, o);
            }
            TM_LAUNCH_CHECK("edt_envelope_smem_kernel");
        } else {
            if (final_pass)
                edt_envelope_gmem_kernel<V, true><<<blocks, kEdtThreads, 0, stream>>>(gin, fin, gout, fout, gstack, p, o);
            else
                edt_envelope_gmem_kernel<V, false><<<blocks, kEdtThreads, 0, stream>>>(gin, fin, gout, fout, gstack, p, o);
            TM_LAUNCH_CHECK("edt_envelope_gmem_kernel");
        }
    }
    return TM_OK;
}

int check_edt_args(const void *input, int in_dtype, const Geometry &g, const float *sampling, bool *unit) {
    if (!input) return fail(TM_ERR_INVALID_ARGUMENT, "input is NULL");
    if (in_dtype != TM_F32 && in_dtype != TM_U8) return fail(TM_ERR_INVALID_ARGUMENT, "unknown input dtype %d", in_dtype);
    if (g.numel_item >= ((int64_t)1 << 31)) return fail(TM_ERR_TOO_LARGE, "items of 2^31 or more voxels are not supported");
    for (int d = 0; d < g.ndim; d++)
        if (g.numel / g.shape[d] >= ((int64_t)1 << 32)) return fail(TM_ERR_TOO_LARGE, "too many lines");
    *unit = true;
    if (sampling) {
        for (int d = 0; d < g.ndim; d++) {
            if (!(std::isfinite(sampling[d]) && sampling[d] > 0.0f))
                return fail(TM_ERR_INVALID_ARGUMENT, "sampling values must be finite and greater than zero");
            if (sampling[d] != 1.0f) *unit = false;
        }
    }
    // exact path: every squared distance and every parabola value must fit
    int64_t sum = 0, mx = 0;
    for (int d = 0; d < g.ndim; d++) {
        sum += (g.shape[d] + 1) * (g.shape[d] + 1);
        mx = g.shape[d] > mx ? g.shape[d] : mx;
    }
    if (*unit && sum + mx * mx >= ((int64_t)1 << 31))
        return fail(TM_ERR_TOO_LARGE, "squared distances of this shape overflow int32");
    return TM_OK;
}

}  // namespace
}  // namespace tmc

static bool unit_sampling(int ndim, const float *sampling) {
    if (!sampling) return true;
    for (int d = 0; d < ndim; d++)
        if (sampling[d] != 1.0f) return false;
    return true;
}

extern "C" size_t tm_edt_workspace_size(int64_t batch, int ndim, const int64_t *shape, const float *sampling) {
    tmc::Geometry g;
    if (tmc::make_geometry(batch, ndim, shape, &g) != TM_OK) return 0;
    if (tmc::edt_compact_eligible(g, unit_sampling(ndim, sampling))) return tmc::edt_compact_workspace(g);
    return tmc::plan_edt(g).total;
}

extern "C" int tm_edt(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
                      const float *sampling, float *dist, int32_t *indices, int32_t *sqdist, void *workspace,
                      size_t workspace_bytes, tm_stream_t stream) {
    using namespace tmc;
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    bool unit = true;
    st = check_edt_args(input, in_dtype, g, sampling, &unit);
    if (st != TM_OK) return st;
    if (!dist && !indices && !sqdist) return fail(TM_ERR_INVALID_ARGUMENT, "at least one output must be requested");
    if (sqdist && !unit) return fail(TM_ERR_INVALID_ARGUMENT, "squared integer distances need unit sampling");
    unsigned char *ws = static_cast<unsigned char *>(workspace);
    cudaStream_t s = (cudaStream_t)stream;
    if (edt_compact_eligible(g, unit)) {
        const size_t need = edt_compact_workspace(g);
        if (!workspace || workspace_bytes < need)
            return fail(TM_ERR_WORKSPACE, "workspace of %zu bytes required, got %zu", need, workspace_bytes);
        return edt_compact_run(input, in_dtype, g, dist, indices, sqdist, ws, s);
    }
    EdtPlan pl = plan_edt(g);
    if (pl.total > 0 && (!workspace || workspace_bytes < pl.total))
        return fail(TM_ERR_WORKSPACE, "workspace of %zu bytes required, got %zu", pl.total, workspace_bytes);
    EdtOutputs o{dist, indices, sqdist};
    if (unit) {
        if (in_dtype == TM_F32) return launch_edt<float, int32_t>((const float *)input, g, nullptr, o, ws, pl, s);
        return launch_edt<uint8_t, int32_t>((const uint8_t *)input, g, nullptr, o, ws, pl, s);
    }
    if (in_dtype == TM_F32) return launch_edt<float, float>((const float *)input, g, sampling, o, ws, pl, s);
    return launch_edt<uint8_t, float>((const uint8_t *)input, g, sampling, o, ws, pl, s);
}
