// FP64 (DFMA) strided, batched GEMM for the CCSD contractions.
//
// C[b](m,n) = alpha * sum_k A[b](m,k) B[b](k,n) + beta * C[b](m,n), where every
// index is a composite of up to three tensor indices with their own strides
// (KIdx), so permuted views of the n^4 amplitude/integral tensors are read in
// place.  GB300 issues only ~2 FP64 FMAs per clock per SM, so the kernel keeps
// every SM busy (split-K with FP64 atomics when the tile count is small) and
// spends integer work freely on index decoding.
#include "kvft_internal.h"

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

__global__ void __launch_bounds__(NT)
gemm_f64_kernel(int M, int N, int K, int nsplit, int klen, double alpha,
                KMat A, KMat B, double beta, KOut C, int atomic) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int bz = blockIdx.z;
    const int batch = bz / nsplit;
    const int ks = bz - batch * nsplit;
    const int bm = blockIdx.y * BM;
    const int bn = blockIdx.x * BN;
    const int kbeg = ks * klen;
    const int kend = min(K, kbeg + klen);

    const double *Ap = A.p + (long long)batch * A.bst;
    const double *Bp = B.p + (long long)batch * B.bst;

    // load mapping: k fastest across threads when k is the contiguous index
    const bool a_kfast = (A.c.st[2] == 1);
    const bool b_kfast = (B.r.st[2] == 1);
    int am[4], ak[4], bk[4], bnn[4];
    long long aoff_m[4], boff_n[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (a_kfast) { ak[r] = tid % BK; am[r] = tid / BK + 16 * r; }
        else { am[r] = tid % BM; ak[r] = tid / BM + 4 * r; }
        if (b_kfast) { bk[r] = tid % BK; bnn[r] = tid / BK + 16 * r; }
        else { bnn[r] = tid % BN; bk[r] = tid / BN + 4 * r; }
        int m = bm + am[r];
        int n = bn + bnn[r];
        aoff_m[r] = (m < M) ? A.r.off(m) : -1;
        boff_n[r] = (n < N) ? B.c.off(n) : -1;
    }

    const int tx = tid % 16, ty = tid / 16;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            int k = k0 + ak[r];
            double v = 0.0;
            if (aoff_m[r] >= 0 && k < kend) v = Ap[aoff_m[r] + A.c.off(k)];
            As[ak[r]][am[r]] = v;
            k = k0 + bk[r];
            v = 0.0;
            if (boff_n[r] >= 0 && k < kend) v = Bp[boff_n[r] + B.r.off(k)];
            Bs[bk[r]][bnn[r]] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }

    double *Cp = C.p + (long long)batch * C.bst;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int m = bm + ty + 16 * i;
        if (m >= M) continue;
        long long ro = C.r.off(m);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int n = bn + tx + 16 * j;
            if (n >= N) continue;
            double *dst = Cp + ro + C.c.off(n);
            double v = alpha * acc[i][j];
            if (atomic) atomicAdd(dst, v);
            else *dst = (beta != 0.0) ? v + beta * (*dst) : v;
        }
    }
}

__global__ void scale_view_kernel(int M, int N, int batch, double beta, KOut C) {
    long long total = (long long)M * N * batch;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        int n = (int)(x % N);
        long long r = x / N;
        int m = (int)(r % M);
        int b = (int)(r / M);
        double *d = C.p + (long long)b * C.bst + C.r.off(m) + C.c.off(n);
        *d = (beta == 0.0) ? 0.0 : beta * (*d);
    }
}

}  // namespace

int kv_scale_view(kvft_ctx *ctx, int M, int N, int batch, double beta, const KOut &C) {
    if (beta == 1.0 || M <= 0 || N <= 0 || batch <= 0) return KVFT_OK;
    if (ctx->dry) {
        KvDryOp op;
        op.kind = 3;
        op.M = M, op.N = N, op.batch = batch, op.beta = beta, op.C = C;
        ctx->dry->push_back(op);
        return KVFT_OK;
    }
    scale_view_kernel<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(M, N, batch, beta, C);
    return kv_launch_check(ctx, "scale_view");
}

int kv_gemm_f64(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha,
                const KMat &A, const KMat &B, double beta, const KOut &C) {
    if (M <= 0 || N <= 0 || batch <= 0) return KVFT_OK;
    if (K <= 0) {
        if (beta == 1.0) return KVFT_OK;
        int blocks = ctx->sm_count * 4;
        scale_view_kernel<<<blocks, 256, 0, ctx->stream>>>(M, N, batch, beta, C);
        return kv_launch_check(ctx, "scale_view");
    }
    long long tiles = (long long)((M + BM - 1) / BM) * ((N + BN - 1) / BN) * batch;
    int nsplit = 1;
    long long want = 2LL * ctx->sm_count;
    if (tiles < want && K > 4 * BK) {
        long long s = (want + tiles - 1) / tiles;
        long long smax = (K + 4 * BK - 1) / (4 * BK);
        nsplit = (int)std::min(s, smax);
        while ((long long)batch * nsplit > 65535) nsplit--;
        if (nsplit < 1) nsplit = 1;
    }
    int klen = (K + nsplit - 1) / nsplit;
    klen = (klen + BK - 1) / BK * BK;
    nsplit = (K + klen - 1) / klen;
    int atomic = nsplit > 1;
    if (atomic && beta != 1.0) {
        int blocks = ctx->sm_count * 4;
        scale_view_kernel<<<blocks, 256, 0, ctx->stream>>>(M, N, batch, beta, C);
        KV_TRY(kv_launch_check(ctx, "scale_view"));
    }
    if ((long long)batch * nsplit > 65535)
        return kv_fail(ctx, KVFT_EINVAL, "gemm batch too large");
    KvProfScope prof(ctx, ctx->gemm_cat, ctx->gemm_work);
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch * nsplit);
    gemm_f64_kernel<<<grid, NT, 0, ctx->stream>>>(M, N, K, nsplit, klen, alpha, A, B,
                                                   beta, C, atomic);
    return kv_launch_check(ctx, "gemm_f64");
}

namespace {

// Moves K component p of both operands' K indices to the fastest position,
// keeping the order of the others (the contraction is the same sum).
void k_to_fast(KIdx &a, KIdx &b, int p) {
    KIdx na = a, nb = b;
    int q = 0;
    for (int d = 0; d < 3; d++)
        if (d != p) {
            na.size[q] = a.size[d];
            na.st[q] = a.st[d];
            nb.size[q] = b.size[d];
            nb.st[q] = b.st[d];
            q++;
        }
    na.size[2] = a.size[p];
    na.st[2] = a.st[p];
    nb.size[2] = b.size[p];
    nb.st[2] = b.st[p];
    a = na;
    b = nb;
}

// The order of the contraction index's components is free.  Operands are read
// in tiles coalesced along their row index or along K, whichever is contiguous
// in memory; when an operand's rows are not, the K component that is
// contiguous in it (if any) is made the fastest, for the larger operand first.
void order_k(int M, int N, int batch, KMat &A, KMat &B) {
    const long long sa = (long long)M * (A.bst ? batch : 1);
    const long long sb = (long long)N * (B.bst ? batch : 1);
    for (int pass = 0; pass < 2; pass++) {
        const bool a_turn = (pass == 0) == (sa >= sb);
        const KIdx &rows = a_turn ? A.r : B.c;      // rows of the packed form
        const KIdx &k = a_turn ? A.c : B.r;
        if (kidx_fast_stride(rows) == 1) continue;
        if (kidx_fast_stride(k) == 1) return;        // already contiguous along K
        for (int d = 0; d < 3; d++)
            if (k.size[d] > 1 && k.st[d] == 1) {
                k_to_fast(A.c, B.r, d);
                return;
            }
    }
}

}  // namespace

void kv_gemm_prof_set(kvft_ctx *ctx, int M, int N, int K, int batch, int nbA, int nbB,
                      double beta, bool tc) {
    // n^6-class: every GEMM dimension is a pair of orbital indices or more;
    // its work is counted in flops, the other contractions' in the bytes the
    // kernel must move (operands as read: BF16 digit planes on the tensor
    // cores, FP64 otherwise; C written, or read and written when added to)
    const long long mn = std::min(std::min(M, N), K), mx = std::max(std::max(M, N), K);
    ctx->gemm_cat = (mn * mn > mx) ? KV_CAT_GEMM6 : KV_CAT_GEMM;
    if (ctx->gemm_cat == KV_CAT_GEMM6) {
        ctx->gemm_work = 2.0 * M * N * (double)K * batch;
    } else {
        const double el = tc ? 2.0 * std::min(ctx->digits - 1, 6) : 8.0;
        ctx->gemm_work = el * K * ((double)M * nbA + (double)N * nbB) +
                         8.0 * M * (double)N * batch * (beta != 0.0 ? 2 : 1);
    }
}

int kv_gemm(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha,
            const KMat &A_in, const KMat &B_in, double beta, const KOut &C) {
    if (ctx->dry) {
        KvDryOp op;
        op.kind = 0;
        op.M = M, op.N = N, op.K = K, op.batch = batch;
        op.alpha = alpha, op.beta = beta;
        op.A = A_in, op.B = B_in, op.C = C;
        ctx->dry->push_back(op);
        return KVFT_OK;
    }
    KMat A = A_in, B = B_in;
    order_k(M, N, batch, A, B);
    // Tensor cores for everything but short sums and tiny products, which stay
    // on the FP64 pipe.  Skinny shapes (a few columns against a long K) go to
    // the tensor cores too: even with most of a 128-wide tile idle they beat
    // GB300's FP64 pipe by an order of magnitude.
    const bool tc = ctx->precision != KVFT_PREC_FP64 && K >= 16 &&
                    2.0 * M * N * (double)K * batch >= 2.0e6;
    kv_gemm_prof_set(ctx, M, N, K, batch, A.bst ? batch : 1, B.bst ? batch : 1, beta, tc);
    if (ctx->prof) {
        ctx->prof->shape[0] = M, ctx->prof->shape[1] = N;
        ctx->prof->shape[2] = K, ctx->prof->shape[3] = batch;
    }
    if (!tc) return kv_gemm_f64(ctx, M, N, K, batch, alpha, A, B, beta, C);
    return kv_gemm_tc(ctx, M, N, K, batch, alpha, A, B, beta, C, ctx->digits);
}
