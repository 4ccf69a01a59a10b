// Tensor-core contraction path (digit-sliced BF16 tcgen05 GEMM).
#include "kvft_internal.h"

int kv_gemm_tc(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha, const KMat &A,
               const KMat &B, double beta, const KOut &C, int digits) {
    (void)M; (void)N; (void)K; (void)batch; (void)alpha; (void)A; (void)B; (void)beta;
    (void)C; (void)digits;
    return kv_fail(ctx, KVFT_EINVAL, "tensor-core contraction path is not built");
}
