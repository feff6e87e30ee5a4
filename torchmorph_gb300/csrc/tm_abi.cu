// Status strings, error reporting and geometry helpers of libtmcore.
#include <cstring>

#include "tm_common.cuh"

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

}  // namespace tmc

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
