// tm_gemm_bf16x3: the error-compensated BF16 tensor-core product on its own,
// D = (a_hi + a_lo)(b_hi + b_lo)^T stored as fp32.  The kernel lives in
// tc_gemm.cuh; the shared-cost Sinkhorn solver runs the same kernel with
// its own epilogues.
#include "tc_gemm.cuh"

namespace tmc {
namespace {

struct StoreEpilogue {
    float *d;
    int64_t ldd;
    __device__ __forceinline__ void prefetch(int, int) const {}
    __device__ __forceinline__ void operator()(const float *tile, int row, int n0) const {
        const int lane = threadIdx.x & 31;
        float4 *dst = reinterpret_cast<float4 *>(d + row * ldd + n0);
#pragma unroll 4
        for (int c = 0; c < tc::kBN; c += 4)
            dst[c / 4] = make_float4(tile[c * 32 + lane], tile[(c + 1) * 32 + lane], tile[(c + 2) * 32 + lane],
                                     tile[(c + 3) * 32 + lane]);
    }
};

}  // namespace
}  // namespace tmc

extern "C" int tm_gemm_bf16x3(const void *a_hi, const void *a_lo, const void *b_hi, const void *b_lo, float *d,
                              int64_t M, int64_t N, int64_t K, tm_stream_t stream) {
    using namespace tmc;
    if (!a_hi || !a_lo || !b_hi || !b_lo || !d) return fail(TM_ERR_INVALID_ARGUMENT, "NULL operand");
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 64)
        return fail(TM_ERR_INVALID_ARGUMENT, "tm_gemm_bf16x3 needs M, N multiples of 128 and K a multiple of 64");
    if (M > (1 << 30) || N > (1 << 30) || K > (1 << 30)) return fail(TM_ERR_TOO_LARGE, "dimension too large");
    const void *ptrs[] = {a_hi, a_lo, b_hi, b_lo, d};
    for (const void *p : ptrs)
        if (((uintptr_t)p & 15) != 0) return fail(TM_ERR_INVALID_ARGUMENT, "operands must be 16-byte aligned");
    return tc::launch_gemm3<3>(a_hi, a_lo, b_hi, b_lo, M, N, K, StoreEpilogue{d, N}, (cudaStream_t)stream);
}
