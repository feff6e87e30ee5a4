// Allocation-free variant of the exact EDT entry point.
//
// tm_edt needs a caller-provided device workspace.  Some callers cannot
// provide one: code that runs where device allocation is not allowed or not
// wanted (inside another library's allocation-free call path, in processes
// whose memory is fully reserved up front, or in C callers that have no
// allocator of their own at hand).  tm_edt_noalloc serves them by running the
// same 2-D/3-D unit-spacing kernels on a fixed scratch area that lives in
// this file as a device global: the driver reserves it on every GPU that
// loads the library, and it stays reserved until the process exits.  This
// function itself allocates nothing.
//
// The scratch is shared by every call on a device and keeps whatever the
// previous call left there; the kernels overwrite every scratch byte they
// read, so no clearing is needed.  Two calls whose GPU work overlaps (on
// different streams or from different host threads without ordering) race
// on the scratch and must be serialised by the caller.
#include <mutex>

#include "edt_internal.cuh"

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;  // 32 MiB per device

static __device__ __align__(256) unsigned char g_edt_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, resolved once
// per device (the host-side symbol is only a handle, not a device address).
int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    int st = tmc::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (st != TM_OK) return st;
    if (dev < 0 || dev >= kMaxDevices) return tmc::fail(TM_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        st = tmc::cuda_check(cudaGetSymbolAddress(&p, g_edt_scratch), "cudaGetSymbolAddress(edt scratch)");
        if (st != TM_OK) return st;
        g_scratch_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_scratch_ptr[dev]);
    return TM_OK;
}

}  // namespace

extern "C" int tm_edt_noalloc(const void *input, int in_dtype, int64_t batch, int ndim, const int64_t *shape,
                              float *dist, int32_t *indices, int32_t *sqdist, tm_stream_t stream) {
    using namespace tmc;
    Geometry g;
    int st = make_geometry(batch, ndim, shape, &g);
    if (st != TM_OK) return st;
    if (!input) return fail(TM_ERR_INVALID_ARGUMENT, "input is NULL");
    if (in_dtype != TM_F32 && in_dtype != TM_U8) return fail(TM_ERR_INVALID_ARGUMENT, "unknown input dtype %d", in_dtype);
    if (!dist && !indices && !sqdist) return fail(TM_ERR_INVALID_ARGUMENT, "at least one output must be requested");
    if (!edt_compact_eligible(g, true))
        return fail(TM_ERR_UNSUPPORTED,
                    "tm_edt_noalloc handles 2-D or 3-D items with unit spacing only (use tm_edt with a workspace)");
    const size_t need = edt_compact_workspace(g);
    if (need > kScratchBytes)
        return fail(TM_ERR_TOO_LARGE,
                    "tm_edt_noalloc: this batch needs %zu bytes of scratch, above its fixed %zu-byte area "
                    "(at most ~4M voxels for 3-D items, ~16M for 2-D); split the batch or use tm_edt",
                    need, kScratchBytes);
    unsigned char *scratch = nullptr;
    st = scratch_for_current_device(&scratch);
    if (st != TM_OK) return st;
    return edt_compact_run(input, in_dtype, g, dist, indices, sqdist, scratch, (cudaStream_t)stream);
}
