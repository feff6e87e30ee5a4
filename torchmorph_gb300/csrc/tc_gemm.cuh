// tcgen05 (5th-generation tensor core) building blocks for sm_103a, as
// inline PTX, and the error-compensated BF16 product kernel built on them.
//
// Operand layout used throughout: K-major tiles of 128 rows x 64 bf16
// (128 bytes per row) written by TMA with 128-byte swizzling; eight rows form
// one 1024-byte swizzle atom, atoms are stacked 1024 bytes apart.
//
// The product D[M x N] = A . B^T with A = A_hi + A_lo, B = B_hi + B_lo (each
// term bf16) is computed as A_hi B_hi + (A_lo B_hi + A_hi B_lo).  Splitting an
// fp32 operand into a bf16 value and a bf16 remainder keeps ~16 mantissa
// bits, so each product is accurate to ~4e-6 relative instead of bf16's 4e-3.
//
// Accumulation precision.  Measured on GB300, every tcgen05.mma that adds
// into an fp32 TMEM accumulator biases it by about -1 ulp of the accumulator
// (the sum is truncated, not rounded): over K = 4096 (256 MMAs) the relative
// error reaches -1.1e-5.  The kernel therefore
//   * accumulates A_hi B_hi for one k-block (4 MMAs) at a time in one of two
//     TMEM buffers, and four "accumulator" warps add each finished buffer
//     into fp32 registers (round-to-nearest) while the tensor core fills the
//     other buffer;
//   * accumulates the two cross terms, which are 2^-8 smaller, in a third
//     TMEM buffer for the whole K range (their truncation error is 2^-8 of
//     the result's).
// The truncation bias is then that of four MMAs per k-block partial sum,
// whatever K is.
//
// Roles (192 threads): warp 0 lane 0 issues the TMA loads of the four
// operand tiles of each 64-wide k-block into a STAGES-deep ring; warp 1 owns
// TMEM and lane 0 issues the MMAs; warps 2..5 drain the accumulators and run
// the epilogue (warp w reads TMEM lanes 32*(w%4) .. +31, the quarter its SM
// sub-partition can access).  Every mbarrier wait is bounded; on a timeout
// the CTA records it in the device status word, skips its epilogue, waits
// for its copies and MMAs in flight, frees TMEM and returns.
#pragma once

#include <stdint.h>

#include "tm_tma.cuh"

namespace tmc {
namespace tc {

constexpr int kBM = 128;  // MMA M (TMEM lanes)
constexpr int kBN = 128;  // MMA N (fp32 TMEM columns per accumulator)
constexpr int kBK = 64;   // K elements per stage (one 128-byte swizzle row)
constexpr int kUmmaK = 16;
constexpr int kGemmThreads = 192;
constexpr int kTmemCols = 512;  // main[2] at 0 / kBN, cross terms at 2*kBN

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (unused for swizzled K-major), stride byte offset 1024 (between
// 8-row atoms), descriptor version 1, 128-byte swizzle.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void *smem_ptr) {
    const uint32_t addr = smem_u32(smem_ptr);
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);  // bits 0-13
    d |= (uint64_t)(16 >> 4) << 16;           // bits 16-29: LBO (16 bytes)
    d |= (uint64_t)(1024 >> 4) << 32;         // bits 32-45: SBO
    d |= (uint64_t)1 << 46;                   // bits 46-47: version
    d |= (uint64_t)2 << 61;                   // bits 61-63: 128-byte swizzle
    return d;
}

// Instruction descriptor: D fp32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4)                      // D format: f32
           | (1u << 7)                    // A format: bf16
           | (1u << 10)                   // B format: bf16
           | ((uint32_t)(N >> 3) << 17)   // N >> 3
           | ((uint32_t)(M >> 4) << 24);  // M >> 4
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive (once) on `bar` when every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 16 consecutive fp32 columns: thread `lane` of the warp gets
// row (lane base + lane), columns col .. col+15.  Completes asynchronously;
// tmem_wait_ld() makes the registers valid.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

template <int STAGES>
struct Gemm3Smem {
    static constexpr int kTileA = kBM * kBK * 2;  // 16 KB
    static constexpr int kTileB = kBN * kBK * 2;  // 16 KB
    static constexpr int kStage = 2 * kTileA + 2 * kTileB;
    static constexpr int kBars = (2 * STAGES + 4) * 8;
    static constexpr int kBytes = STAGES * kStage + kBars + 16 + 1024;  // + alignment slack
    static_assert(STAGES * kStage >= 4 * kBN * 32 * 4, "the epilogue tile is staged in the operand ring");
};

// Epi: __device__ void operator()(const float *tile, int row, int n0) const,
// called once by all 32 lanes of each accumulator warp together; lane l
// owns output row `row` (32 consecutive rows per warp) and finds
// D[row][n0 + c] at tile[c * 32 + l] (shared memory), c < kBN.
// Epi::prefetch(row, n0) is called by the same threads when the mainloop
// starts, to pull the epilogue's other inputs towards L2 early.
template <int STAGES, typename Epi>
__global__ void __launch_bounds__(kGemmThreads, 1)
    gemm3_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                 const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo, int K, Epi epi,
                 int *status) {
    using L = Gemm3Smem<STAGES>;
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + STAGES * L::kStage);
    uint64_t *empty = full + STAGES;
    uint64_t *acc_full = empty + STAGES;  // [2]
    uint64_t *acc_empty = acc_full + 2;   // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(acc_empty + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int nk = K / kBK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            bool ok = true;
            int issued = 0;
            for (int kb = 0; kb < nk && ok; kb++) {
                const int s = kb % STAGES;
                if (kb >= STAGES) ok = mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1, status);
                if (!ok) break;
                unsigned char *st = smem + s * L::kStage;
                mbar_arrive_expect_tx(&full[s], L::kStage);
                tma_load_2d(st, &ta_hi, kb * kBK, m0, &full[s]);
                tma_load_2d(st + L::kTileA, &ta_lo, kb * kBK, m0, &full[s]);
                tma_load_2d(st + 2 * L::kTileA, &tb_hi, kb * kBK, n0, &full[s]);
                tma_load_2d(st + 2 * L::kTileA + L::kTileB, &tb_lo, kb * kBK, n0, &full[s]);
                issued = kb + 1;
            }
            // no copy may still be landing in shared memory when the CTA exits
            for (int kb = issued - STAGES > 0 ? issued - STAGES : 0; kb < issued; kb++)
                mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1, status);
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16_f32(kBM, kBN);
            const uint32_t t_cross = tmem + 2 * kBN;
            bool ok = true;
            int issued = 0;
            for (int kb = 0; kb < nk && ok; kb++) {
                const int s = kb % STAGES, buf = kb & 1;
                if (kb >= 2) ok = mbar_wait(&acc_empty[buf], ((kb >> 1) - 1) & 1, status);
                if (ok) ok = mbar_wait(&full[s], (kb / STAGES) & 1, status);
                if (!ok) break;
                fence_after_sync();
                const uint32_t t_main = tmem + buf * kBN;
                unsigned char *st = smem + s * L::kStage;
                const unsigned char *a_hi = st, *a_lo = st + L::kTileA;
                const unsigned char *b_hi = st + 2 * L::kTileA, *b_lo = st + 2 * L::kTileA + L::kTileB;
#pragma unroll
                for (int kk = 0; kk < kBK / kUmmaK; kk++) {
                    const int off = kk * kUmmaK * 2;  // bytes along the 128-byte swizzled row
                    const uint64_t dah = smem_desc_sw128(a_hi + off), dal = smem_desc_sw128(a_lo + off);
                    const uint64_t dbh = smem_desc_sw128(b_hi + off), dbl = smem_desc_sw128(b_lo + off);
                    mma_bf16(t_main, dah, dbh, idesc, kk != 0);
                    mma_bf16(t_cross, dal, dbh, idesc, (kb | kk) != 0);
                    mma_bf16(t_cross, dah, dbl, idesc, 1);
                }
                mma_commit(&empty[s]);
                mma_commit(&acc_full[buf]);
                issued = kb + 1;
            }
            // TMEM stays allocated until every issued MMA has finished
            if (issued > 0) mbar_wait(&acc_full[(issued - 1) & 1], ((issued - 1) >> 1) & 1, status);
        }
        __syncwarp();
    } else {
        const int q = warp & 3;
        const uint32_t t_lane = tmem + ((uint32_t)(q * 32) << 16);
        const int row = m0 + q * 32 + lane;
        epi.prefetch(row, n0);
        float acc[kBN];
#pragma unroll
        for (int i = 0; i < kBN; i++) acc[i] = 0.f;
        bool ok = true;
        for (int kb = 0; kb < nk; kb++) {
            const int buf = kb & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], (kb >> 1) & 1, status));
            if (!ok) break;
            fence_after_sync();
#pragma unroll
            for (int g = 0; g < kBN / 16; g += 2) {
                uint32_t r0[16], r1[16];
                tmem_ld16(t_lane + buf * kBN + g * 16, r0);
                tmem_ld16(t_lane + buf * kBN + g * 16 + 16, r1);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    acc[g * 16 + i] += __uint_as_float(r0[i]);
                    acc[g * 16 + 16 + i] += __uint_as_float(r1[i]);
                }
            }
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
        if (ok && nk > 0) {
            // Every TMA copy has landed and every MMA has finished (the last
            // acc_full phase covers them all), so the operand ring is idle:
            // stage this warp's 32 x kBN block there, column-major, and run
            // the epilogue from shared memory with compact code.
            float *tile = reinterpret_cast<float *>(smem) + q * (kBN * 32);
#pragma unroll
            for (int g = 0; g < kBN / 16; g++) {
                uint32_t r[16];
                tmem_ld16(t_lane + 2 * kBN + g * 16, r);
                tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; i++) tile[(g * 16 + i) * 32 + lane] = acc[g * 16 + i] + __uint_as_float(r[i]);
            }
            __syncwarp();
            epi(tile, row, n0);
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, kTmemCols);
}

// bf16 row-major [rows x K] operand as a 2-D tensor map with 64 x 128 boxes.
inline int make_operand_map(CUtensorMap *map, const void *ptr, int64_t rows, int64_t K) {
    const uint64_t dims[2] = {(uint64_t)K, (uint64_t)rows};
    const uint64_t strides[1] = {(uint64_t)K * 2};
    const uint32_t box[2] = {(uint32_t)kBK, 128u};
    return encode_tensor_map(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box,
                             CU_TENSOR_MAP_SWIZZLE_128B);
}

// D = (a_hi + a_lo)(b_hi + b_lo)^T delivered tile by tile to `epi`.
// M, N multiples of 128, K a multiple of 64 (checked by the callers).
template <int STAGES, typename Epi>
int launch_gemm3(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo, int64_t M, int64_t N,
                 int64_t K, const Epi &epi, cudaStream_t stream) {
    using L = Gemm3Smem<STAGES>;
    CUtensorMap ta_hi, ta_lo, tb_hi, tb_lo;
    int st = make_operand_map(&ta_hi, a_hi, M, K);
    if (st == TM_OK) st = make_operand_map(&ta_lo, a_lo, M, K);
    if (st == TM_OK) st = make_operand_map(&tb_hi, b_hi, N, K);
    if (st == TM_OK) st = make_operand_map(&tb_lo, b_lo, N, K);
    if (st != TM_OK) return st;
    int *status = nullptr;
    st = device_status_word(&status);
    if (st != TM_OK) return st;
    auto kernel = gemm3_kernel<STAGES, Epi>;
    TM_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, L::kBytes));
    dim3 grid((unsigned)(N / kBN), (unsigned)(M / kBM));
    kernel<<<grid, kGemmThreads, L::kBytes, stream>>>(ta_hi, ta_lo, tb_hi, tb_lo, (int)K, epi, status);
    TM_LAUNCH_CHECK("gemm3_kernel");
    return TM_OK;
}

}  // namespace tc
}  // namespace tmc
