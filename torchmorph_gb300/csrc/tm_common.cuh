// Shared host/device helpers of libtmcore (GB300, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/torchmorph_gb300.h"

#define TM_MAX_NDIM 8

namespace tmc {

// Per-thread last-error message (reported through tm_last_error()).
void set_error(const char *fmt, ...);
int fail(int status, const char *fmt, ...);

// Checks a CUDA call made by the library; records the message on failure.
int cuda_check(cudaError_t err, const char *what);

// Launch check after every kernel launch.
inline int launch_check(const char *kernel) { return cuda_check(cudaGetLastError(), kernel); }

// Number of SMs of the current device (cached per device).
int sm_count();

// Implementation variants picked by the autotuner (tm_tune_set), per operator
// and work class; -1 = the library's built-in choice.  Every variant of an
// operator gives bit-identical results.
enum TuneOp { kTuneGreyFlat2D = 0, kTuneSinkhornF32 = 1, kTuneEdt3D = 2, kTuneCdt3D = 3, kTuneOps = 4 };
int tune_variant(int op, int cls);
int tune_class(int op, int64_t a, int64_t b);

// Host-side geometry of a batch of items.
struct Geometry {
    int ndim;
    int64_t batch;
    int64_t shape[TM_MAX_NDIM];
    int64_t stride[TM_MAX_NDIM];
    int64_t numel_item;
    int64_t numel;
};

int make_geometry(int64_t batch, int ndim, const int64_t *shape, Geometry *g);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Fast unsigned division by a runtime constant (Granlund-Montgomery magic
// numbers; valid for 32-bit dividends).  Used in kernels to unravel flat
// indices without hardware integer division.
struct FastDiv {
    uint32_t d;
    uint32_t mul;
    uint32_t shift;
};

inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    if (d <= 1) {
        f.mul = 0;
        f.shift = 0;
        return f;
    }
    uint32_t l = 0;
    while ((1ull << l) < d) l++;
    // mul = floor(2^32 * (2^l - d) / d) + 1, q = (hi(n*mul) + n) >> l
    uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    f.mul = (uint32_t)m;
    f.shift = l;
    return f;
}

__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
    if (f.d == 1) return n;
#ifdef __CUDA_ARCH__
    uint32_t hi = __umulhi(n, f.mul);
#else
    uint32_t hi = (uint32_t)(((uint64_t)n * f.mul) >> 32);
#endif
    return (hi + ((n - hi) >> 1)) >> (f.shift - 1);
}

// Programmatic dependent launch: the kernel may be scheduled while the
// previous kernel of the stream is still finishing.  A kernel launched this
// way calls pdl_wait() before it touches anything the previous kernel writes
// or reads; pdl_wait() then returns once that kernel has completed and its
// writes are visible (it is a no-op in a kernel launched normally).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel of the stream (if launched with launch_pdl) be scheduled now.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace tmc

#define TM_CHECK_CUDA(call)                                    \
    do {                                                       \
        int _st = tmc::cuda_check((call), #call);               \
        if (_st != TM_OK) return _st;                          \
    } while (0)

#define TM_LAUNCH_CHECK(name)                                  \
    do {                                                       \
        int _st = tmc::launch_check(name);                      \
        if (_st != TM_OK) return _st;                          \
    } while (0)
