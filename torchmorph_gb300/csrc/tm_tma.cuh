// Tensor Memory Accelerator (TMA) and mbarrier helpers for sm_103a kernels,
// written as inline PTX, plus the host-side tensor-map encoder.
//
// Every wait on an mbarrier is bounded: after kSpinLimit polls the waiting
// thread records TM_DEV_ERR_TIMEOUT in the library's device status word
// (read by tm_device_error()) and the wait returns false, so a kernel never
// hangs on a copy that does not arrive.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "tm_common.cuh"

namespace tmc {

enum DeviceError { TM_DEV_OK = 0, TM_DEV_ERR_TIMEOUT = 1 };

// Device address of the status word on the current device (resolved once).
int device_status_word(int **out);

// Encode a tiled tensor map (rank <= 5).  dims[0] is the innermost
// (contiguous) extent; strides_bytes has rank-1 entries (dims 1..rank-1).
int encode_tensor_map(CUtensorMap *map, CUtensorMapDataType dtype, int rank, const void *gaddr,
                      const uint64_t *dims, const uint64_t *strides_bytes, const uint32_t *box,
                      CUtensorMapSwizzle swizzle = CU_TENSOR_MAP_SWIZZLE_NONE);

constexpr long long kSpinLimit = 1LL << 26;

// Poll budget of the grid barriers of the cooperative persistent kernels
// (point-cloud and FP32 Sinkhorn solvers): kSpinLimit unless the host set
// another with tm_set_grid_wait_budget().  The waits that guard TMA copies and
// tensor-core work in flight always use kSpinLimit.
long long grid_wait_budget();

// Control block of a cooperative launch whose CTAs meet at grid barriers;
// zeroed before the launch.  Kernels with more launch-wide state keep their
// own 256-byte block with the same first three fields.
struct GridControl {
    unsigned barrier_count;  // CTAs arrived at the current barrier
    unsigned barrier_gen;    // barriers completed
    int abort;               // set by a CTA whose wait gave up: every CTA leaves
    int pad[61];
};
static_assert(sizeof(GridControl) == 256, "control block is 256 bytes");

// Barrier of the `nblocks` CTAs of a cooperative launch (all co-resident).
// The last CTA to arrive resets the count and advances the generation; the
// others poll the generation at most spin_limit times.  A wait that gives up
// (or sees another CTA's abort) sets the abort flag and TM_DEV_ERR_TIMEOUT in
// `status`; the barrier then returns false in every CTA that reaches it, and
// the caller returns.  Writes before the barrier are visible to loads after
// it that bypass L1 (__ldcg, or data this CTA has not cached).
// Ctl: a control block with barrier_count, barrier_gen and abort.
template <typename Ctl>
__device__ inline bool grid_barrier_bounded(Ctl *ctl, unsigned nblocks, int *status, long long spin_limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &ctl->barrier_gen;
        volatile int *abort = &ctl->abort;
        const unsigned g = *gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&ctl->barrier_count, 1u) == nblocks - 1) {
            ctl->barrier_count = 0;
            __threadfence();
            atomicAdd(&ctl->barrier_gen, 1u);
        } else {
            long long polls = 0;
            while (*gen == g) {
                if (*abort || ++polls > spin_limit) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        if (!ok) {
            atomicExch(&ctl->abort, 1);
            if (status) atomicExch(status, TM_DEV_ERR_TIMEOUT);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity` of an mbarrier; false (and the status word
// set) when it did not complete within kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status) {
    for (long long i = 0; i < kSpinLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    if (status) atomicExch(status, TM_DEV_ERR_TIMEOUT);
    return false;
}

// 3-D tiled load: box at coordinates (c0 innermost, c1, c2) into shared
// memory, completion counted on `bar` in bytes.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace tmc
