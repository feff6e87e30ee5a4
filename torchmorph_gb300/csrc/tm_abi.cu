// Status strings, error reporting and geometry helpers of libtmcore.
#include <cudaTypedefs.h>

#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>

#include "tm_common.cuh"
#include "tm_tma.cuh"

namespace tmc {

static thread_local char g_last_error[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_check(cudaError_t err, const char *what) {
    if (err == cudaSuccess) return TM_OK;
    return fail(TM_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(err), cudaGetErrorName(err));
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

int make_geometry(int64_t batch, int ndim, const int64_t *shape, Geometry *g) {
    if (ndim < 1 || ndim > TM_MAX_NDIM)
        return fail(TM_ERR_INVALID_ARGUMENT, "spatial ndim must be in 1..%d, got %d", TM_MAX_NDIM, ndim);
    if (batch < 1) return fail(TM_ERR_INVALID_ARGUMENT, "batch must be >= 1, got %lld", (long long)batch);
    if (!shape) return fail(TM_ERR_INVALID_ARGUMENT, "shape is NULL");
    g->ndim = ndim;
    g->batch = batch;
    int64_t n = 1;
    for (int d = 0; d < TM_MAX_NDIM; d++) {
        g->shape[d] = d < ndim ? shape[d] : 1;
        g->stride[d] = 0;
    }
    for (int d = 0; d < ndim; d++) {
        if (shape[d] < 1)
            return fail(TM_ERR_INVALID_ARGUMENT, "spatial size %d is %lld; sizes must be >= 1", d,
                        (long long)shape[d]);
        if (n > ((int64_t)1 << 62) / shape[d]) return fail(TM_ERR_TOO_LARGE, "item size overflows int64");
        n *= shape[d];
    }
    g->stride[ndim - 1] = 1;
    for (int d = ndim - 2; d >= 0; d--) g->stride[d] = g->stride[d + 1] * shape[d + 1];
    g->numel_item = n;
    if (n > ((int64_t)1 << 62) / batch) return fail(TM_ERR_TOO_LARGE, "batch size overflows int64");
    g->numel = n * batch;
    return TM_OK;
}

// ----------------------------------------------------------------------------
// Device status word: kernels record device-side failures here (for example a
// bounded wait that gave up); tm_device_error() reads and optionally clears it.
static __device__ int g_device_status;
static std::mutex g_status_mutex;
static int *g_status_ptr[64] = {nullptr};

int device_status_word(int **out) {
    int dev = 0;
    int st = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (st != TM_OK) return st;
    if (dev < 0 || dev >= 64) return fail(TM_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_status_mutex);
    if (!g_status_ptr[dev]) {
        void *p = nullptr;
        st = cuda_check(cudaGetSymbolAddress(&p, g_device_status), "cudaGetSymbolAddress(status word)");
        if (st != TM_OK) return st;
        g_status_ptr[dev] = static_cast<int *>(p);
    }
    *out = g_status_ptr[dev];
    return TM_OK;
}

int encode_tensor_map(CUtensorMap *map, CUtensorMapDataType dtype, int rank, const void *gaddr,
                      const uint64_t *dims, const uint64_t *strides_bytes, const uint32_t *box,
                      CUtensorMapSwizzle swizzle) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    static cudaError_t once_err = cudaSuccess;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        once_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q);
        if (once_err == cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    if (!fn) return fail(TM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t gdim[5];
    cuuint64_t gstride[4];
    cuuint32_t bdim[5], estride[5];
    for (int i = 0; i < rank; i++) {
        gdim[i] = dims[i];
        bdim[i] = box[i];
        estride[i] = 1;
    }
    for (int i = 0; i < rank - 1; i++) gstride[i] = strides_bytes[i];
    CUresult r = fn(map, dtype, (cuuint32_t)rank, const_cast<void *>(gaddr), gdim, gstride, bdim, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(TM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return TM_OK;
}

// --------------------------------------------------------------- autotuning
// Variant table: (operator, work class) -> variant, -1 = built-in choice.
constexpr int kTuneClasses = 64;
static const int kTuneVariants[kTuneOps] = {4, 4, 2, 3};
static std::atomic<int> g_tune[kTuneOps][kTuneClasses];
static std::once_flag g_tune_once;

static void tune_init() {
    std::call_once(g_tune_once, [] {
        for (auto &row : g_tune)
            for (auto &v : row) v.store(-1);
    });
}

static int floor_log2(int64_t x) {
    int k = 0;
    while (x > 1) {
        x >>= 1;
        k++;
    }
    return k;
}

// Work class: log2 of the voxel count (morphology, distance transforms), or
// 8 * min(7, log2 n) + min(7, log2 d - 6) for n histogram pairs of d points.
int tune_class(int op, int64_t a, int64_t b) {
    if (op == kTuneSinkhornF32) {
        const int cn = std::min(7, floor_log2(std::max<int64_t>(a, 1)));
        const int cd = std::min(7, std::max(0, floor_log2(std::max<int64_t>(b, 1)) - 6));
        return 8 * cn + cd;
    }
    return std::min(kTuneClasses - 1, floor_log2(std::max<int64_t>(a, 1)));
}

int tune_variant(int op, int cls) {
    if (op < 0 || op >= kTuneOps || cls < 0 || cls >= kTuneClasses) return -1;
    tune_init();
    return g_tune[op][cls].load(std::memory_order_relaxed);
}

static std::atomic<long long> g_grid_wait_budget{kSpinLimit};

long long grid_wait_budget() { return g_grid_wait_budget.load(); }

}  // namespace tmc

extern "C" int tm_tune_variants(int op) {
    if (op < 0 || op >= tmc::kTuneOps) return tmc::fail(TM_ERR_INVALID_ARGUMENT, "unknown tuning operator %d", op), 0;
    return tmc::kTuneVariants[op];
}

extern "C" int tm_tune_class(int op, int64_t a, int64_t b) {
    if (op < 0 || op >= tmc::kTuneOps) return -1;
    return tmc::tune_class(op, a, b);
}

extern "C" int tm_tune_set(int op, int cls, int variant) {
    using namespace tmc;
    if (op < 0 || op >= kTuneOps) return fail(TM_ERR_INVALID_ARGUMENT, "unknown tuning operator %d", op);
    if (cls < 0 || cls >= kTuneClasses) return fail(TM_ERR_INVALID_ARGUMENT, "work class %d out of range", cls);
    if (variant < -1 || variant >= kTuneVariants[op])
        return fail(TM_ERR_INVALID_ARGUMENT, "operator %d has variants 0..%d (-1: built-in)", op, kTuneVariants[op] - 1);
    tune_init();
    g_tune[op][cls].store(variant);
    return TM_OK;
}

extern "C" int tm_tune_get(int op, int cls) { return tmc::tune_variant(op, cls); }

extern "C" void tm_set_grid_wait_budget(int64_t polls) {
    tmc::g_grid_wait_budget.store(polls < 0 ? tmc::kSpinLimit : (long long)polls);
}

extern "C" int tm_device_error(int reset) {
    int *word = nullptr;
    if (tmc::device_status_word(&word) != TM_OK) return -1;
    int v = 0;
    if (cudaMemcpy(&v, word, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    if (reset && v != 0) {
        const int zero = 0;
        if (cudaMemcpy(word, &zero, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) return -1;
    }
    return v;
}

extern "C" const char *tm_status_string(int status) {
    switch (status) {
    case TM_OK: return "ok";
    case TM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TM_ERR_UNSUPPORTED: return "unsupported";
    case TM_ERR_CUDA: return "CUDA error";
    case TM_ERR_TOO_LARGE: return "too large";
    case TM_ERR_WORKSPACE: return "workspace missing or too small";
    case TM_ERR_TIMEOUT: return "device-side wait timed out";
    default: return "unknown status";
    }
}

extern "C" const char *tm_last_error(void) { return tmc::g_last_error; }

extern "C" int tm_version(void) { return 100; }
