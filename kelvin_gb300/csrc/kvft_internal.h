// Internal definitions shared by the libkvft translation units.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <stdint.h>
#include <string>
#include <vector>
#include <map>

#include "../../include/kvft.h"

// ---------------------------------------------------------------------------
// Strided views.  A contraction operand is a matrix whose row and column
// indices are each a composite of up to three tensor indices, every one with
// its own element stride, plus a stride between tau points (batch).  This is
// how index permutations of the n^4 tensors enter the GEMMs without copies.
// ---------------------------------------------------------------------------
struct KIdx {
    int size[3];        // slow -> fast; unused entries have size 1
    long long st[3];    // element strides
    __host__ __device__ int total() const { return size[0] * size[1] * size[2]; }
    __host__ __device__ long long off(int x) const {
        int i2 = x % size[2];
        int r = x / size[2];
        int i1 = r % size[1];
        int i0 = r / size[1];
        return (long long)i0 * st[0] + (long long)i1 * st[1] + (long long)i2 * st[2];
    }
};

struct KMat {
    const double *p;
    KIdx r, c;
    long long bst;      // stride between batch entries (0: shared operand)
    int stable = 0;     // contents fixed for the solver's lifetime (integral blocks)
};

struct KOut {
    double *p;
    KIdx r, c;
    long long bst;
};

inline KIdx kidx1(int s0, long long t0) { return KIdx{{1, 1, s0}, {0, 0, t0}}; }
inline KIdx kidx2(int s0, long long t0, int s1, long long t1) {
    return KIdx{{1, s0, s1}, {0, t0, t1}};
}
inline KIdx kidx3(int s0, long long t0, int s1, long long t1, int s2, long long t2) {
    return KIdx{{s0, s1, s2}, {t0, t1, t2}};
}
// Element stride of the fastest component of extent > 1 (0 for one element):
// consecutive index values are adjacent in memory when it is 1.
inline long long kidx_fast_stride(const KIdx &x) {
    for (int d = 2; d >= 0; d--)
        if (x.size[d] > 1) return x.st[d];
    return 0;
}

// Profile categories (kvft_profile_stats order): work in flops for
// KV_CAT_GEMM6, in bytes for the others.
enum KvCat { KV_CAT_GEMM6 = 0, KV_CAT_GEMM = 1, KV_CAT_QUAD = 2, KV_CAT_ENERGY = 3,
             KV_CAT_ELEM = 4, KV_CAT_PACK = 5, KV_NCAT = 6 };

// One recorded launch of a dry-run context (kvft_dryrun_create): the
// descriptors a kernel would have been launched with.
struct KvDryOp {
    int kind;                        // 0 contraction, 1 strided axpby, 2 tau integral,
                                     // 3 scale
    int M = 0, N = 0, K = 0, batch = 0;
    double alpha = 0.0, beta = 0.0;
    KMat A{}, B{};
    KOut C{};
    int dims[4] = {1, 1, 1, 1};
    long long ss[4] = {0, 0, 0, 0}, ds[4] = {0, 0, 0, 0}, sbst = 0, dbst = 0;
    const double *src = nullptr;
    double *dst = nullptr;
    // tau integral: ng, P, rank, full, nv, no and its operands
    int ng = 0, rank = 0, full = 0, nv = 0, no = 0;
    long long P = 0;
    const double *ti = nullptr, *G = nullptr, *ev = nullptr, *eo = nullptr;
    // sum of squares: src2 (second operand, may be null) and the result word
    const double *src2 = nullptr;
    double *res = nullptr;
};

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
struct kvft_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    int precision = KVFT_PREC_FP64;
    int digits = 7;                  // digit levels for the tensor-core GEMM
    std::string err;
    cudaEvent_t ev[64] = {};
    uint64_t launches = 0;
    void *l2buf = nullptr;
    // cached scratch buffers keyed by purpose
    std::map<std::string, std::pair<void *, size_t>> scratch;
    int *dflag = nullptr;            // device status word for bounded waits
    struct KvProf *prof = nullptr;
    // Digit planes of stable operands (the integral blocks), kept across the
    // residual evaluations of one solver: on only inside solver-driven
    // evaluations, emptied when a solver is destroyed.
    bool pack_cache_on = false;
    std::map<std::string, std::pair<void *, size_t>> pack_cache;
    // profile category and algorithmic work of the contraction being
    // launched (its kernel is timed alone, without the operand packing)
    int gemm_cat = KV_CAT_GEMM;
    double gemm_work = 0.0;
    // Spin blocks of the residual's operands: 0, or the size h of the alpha
    // half when every orbital index runs over [0, h) alpha then [h, 2h) beta
    // and the integrals and amplitudes vanish outside spin-conserving blocks
    // (set by a solver that has checked its integrals).
    int spin_half = 0;
    // Dry run: launches are recorded here instead of executed, and scratch
    // is host memory filled with NaN (a context without a device).
    std::vector<KvDryOp> *dry = nullptr;
    // Spin blocks of the Lambda path's operands (kvft_set_lambda_spin_blocks):
    // 0, or h when every index-string contraction may run over its nonzero
    // spin-block products only (nv = no = 2h, alpha half first).
    int lam_spin = 0;
    // cap on the bytes a solver's tau-chunk workspace may take on this
    // context (0: 60% of the free memory), so that several solvers fit
    size_t workspace_limit = 0;
    // bumped whenever a scratch or cached buffer is (re)allocated or freed:
    // a captured CUDA graph holds the addresses it saw
    uint64_t scratch_gen = 0;
    // Packed operands shared by the products of one spin-blocked contraction
    // (on inside KvTPackScope): key -> pool slot; the slots' buffers are
    // scratch kept for the next contraction.
    bool tpack_on = false;
    std::map<std::string, int> tpack;
    // Pinned, device-mapped host staging of the amplitude read-back (two
    // halves), kept for the context's lifetime.
    void *hstage = nullptr;
    size_t hstage_bytes = 0;
};
struct KvTPackScope {
    kvft_ctx *ctx;
    bool prev;
    explicit KvTPackScope(kvft_ctx *c) : ctx(c), prev(c->tpack_on) {
        c->tpack_on = true;
        if (!prev) c->tpack.clear();
    }
    ~KvTPackScope() {
        ctx->tpack_on = prev;
        if (!prev) ctx->tpack.clear();
    }
};
// FP64 <-> FP32 by integer operations on the bit patterns, for values that
// only steer the iteration (norms, the Anderson history): GB300's FP64 pipe
// runs conversions at its FP64 rate.  To FP32: mantissa truncated, below
// 2^-126 zero, above the FP32 range infinite (NaN stays NaN).  To FP64:
// exact (FP32 subnormals become zero).
__device__ __forceinline__ float kv_d2f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned sg = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FF) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sg);
    if (e >= 255) {
        const bool nan = (hi & 0x7FF00000u) == 0x7FF00000u && (((hi & 0xFFFFFu) | lo) != 0);
        return __uint_as_float(nan ? 0x7FC00000u : (sg | 0x7F800000u));
    }
    return __uint_as_float(sg | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}
__device__ __forceinline__ double kv_f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const int E = (int)((u >> 23) & 0xFF);
    if (E == 0) return __hiloint2double((int)(u & 0x80000000u), 0);
    if (E == 255) return __hiloint2double((int)((u & 0x80000000u) | 0x7FF00000u | ((u >> 3) & 0xFFFFFu)),
                                          (int)(u << 29));
    return __hiloint2double((int)((u & 0x80000000u) | ((unsigned)(E - 127 + 1023) << 20) |
                                  ((u >> 3) & 0xFFFFFu)),
                            (int)(u << 29));
}

// Fraction of a T2-shaped tensor (nv nv no no) that the spin-conserving
// blocks hold: 6 of the 16 spin blocks when nv = no = 2 sh, else all.  The
// profiled algorithmic bytes of a pass that touches only those elements are
// scaled by it.
inline double kv_spin_frac(int nv, int no, int sh) {
    return (sh > 0 && nv == no && nv == 2 * sh) ? 6.0 / 16.0 : 1.0;
}
struct KvSpinScope {
    kvft_ctx *ctx;
    int prev;
    KvSpinScope(kvft_ctx *c, int h) : ctx(c), prev(c->spin_half) { c->spin_half = h; }
    ~KvSpinScope() { ctx->spin_half = prev; }
};
void kv_pack_cache_clear(kvft_ctx *ctx);
// Turns the pack cache on for the lifetime of the guard.
struct KvPackCacheScope {
    kvft_ctx *ctx;
    bool prev;
    explicit KvPackCacheScope(kvft_ctx *c) : ctx(c), prev(c->pack_cache_on) {
        c->pack_cache_on = true;
    }
    ~KvPackCacheScope() { ctx->pack_cache_on = prev; }
};

// Live per-launch timing (enabled by kvft_profile_begin): event pairs around
// launches of each category, with the algorithmic work they carry.
struct KvProf {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    struct Rec { int cat; size_t e0, e1; double work; int shape[4]; };
    std::vector<Rec> recs;
    // GEMM shape (M, N, K, batch) of the contraction being launched: tagged
    // on its packing and kernel scopes
    int shape[4] = {0, 0, 0, 0};
};
int kv_prof_mark(kvft_ctx *ctx, size_t *slot);            // record one event
void kv_prof_add(kvft_ctx *ctx, int cat, size_t e0, size_t e1, double work);
struct KvProfScope {                                      // RAII helper
    kvft_ctx *ctx; int cat; double work; size_t e0; bool on;
    KvProfScope(kvft_ctx *c, int k, double w);
    ~KvProfScope();
};

// error helpers --------------------------------------------------------------
int kv_fail(kvft_ctx *ctx, int code, const std::string &msg);
int kv_cuda(kvft_ctx *ctx, cudaError_t e, const char *what);
#define KV_CHECK(ctx, call)                                   \
    do {                                                      \
        cudaError_t _e = (call);                              \
        if (_e != cudaSuccess) return kv_cuda(ctx, _e, #call); \
    } while (0)
#define KV_TRY(expr)                 \
    do {                             \
        int _s = (expr);             \
        if (_s != KVFT_OK) return _s; \
    } while (0)
int kv_launch_check(kvft_ctx *ctx, const char *what);

// scratch memory owned by the context (grows, never shrinks until destroy)
int kv_scratch(kvft_ctx *ctx, const char *key, size_t bytes, void **p);

// ---------------------------------------------------------------------------
// Kernel launchers (each returns a kvft_status)
// ---------------------------------------------------------------------------
// C = alpha * A * B + beta * C, batched over `batch` tau points.
int kv_gemm(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha,
            const KMat &A, const KMat &B, double beta, const KOut &C);
int kv_gemm_f64(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha,
                const KMat &A, const KMat &B, double beta, const KOut &C);
int kv_gemm_tc(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha,
               const KMat &A, const KMat &B, double beta, const KOut &C,
               int digits);
// Sets the profile category (n^6-class or not) and work (flops, or bytes
// for the other class) of the next contraction launch.
void kv_gemm_prof_set(kvft_ctx *ctx, int M, int N, int K, int batch, int nbA, int nbB,
                      double beta, bool tc);
// C = beta * C over a strided output view (beta == 0 writes zeros).
int kv_scale_view(kvft_ctx *ctx, int M, int N, int batch, double beta, const KOut &C);
// Reads (and clears) the device status word set by bounded waits; syncs.
int kv_device_status(kvft_ctx *ctx);

// 4-index strided axpby: dst = beta*dst + alpha*src over a [b][d0][d1][d2][d3]
// index space; each side gives element strides for the 4 indices + batch.
struct K4 {
    int d[4];
    long long s[4];
    long long bst;
};
int kv_axpby4(kvft_ctx *ctx, int batch, const int dims[4], double alpha,
              const double *src, const long long ss[4], long long sbst,
              double beta, double *dst, const long long ds[4], long long dbst);

// tau-type amplitudes: out = t2 + c * (t1[a,i] t1[b,j] - t1[b,i] t1[a,j])
// (spin_half > 0: the spin-conserving elements only)
int kv_make_tau(kvft_ctx *ctx, int batch, int nv, int no, const double *t1,
                const double *t2, double c, double *out, int spin_half = 0);
// tmp[b,j,n,f] = 0.5 t2[f,b,j,n] + t1[f,j] t1[b,n] (spin_half > 0: the
// spin-conserving elements only)
int kv_make_wmbej_tmp(kvft_ctx *ctx, int batch, int nv, int no,
                      const double *t1, const double *t2, double *out, int spin_half = 0);
// T2 += fac (1 - P(ab))(1 - P(ij)) (Z + L), L = the ladder sum stored over
// a < b, i < j (Lc, or nullptr), zero elsewhere.  With a seed (a
// tau-independent [a][b][i][j] block) T2 is written, not updated:
// T2 = -seed + fac (...).
int kv_assemble_t2(kvft_ctx *ctx, int batch, int nv, int no, double fac, const double *Z,
                   const double *Lc, double *T2, const double *seed = nullptr,
                   int spin_half = 0);
// Antisymmetric pair compression (pairs p < q, x = p(2n-p-1)/2 + q-p-1):
// tau_c[y][(e<f)][(i<j)] from t1, t2
// (spin_half > 0: spin-sorted pair order, only pairs of one spin type linked)
int kv_make_tau_pairs(kvft_ctx *ctx, int batch, int nv, int no, const double *t1,
                      const double *t2, double *out, int spin_half = 0);
// out[y][(p<q) over n1][(r<s) over n2] = ca A[p,q,r,s] + c1 B[y][p,q,r,s] + c2 B[y](sb2)
int kv_pair_gather(kvft_ctx *ctx, int batch, int n1, int n2, const double *A,
                   const long long sa[4], double ca, const double *B, const long long sb1[4],
                   double c1, const long long sb2[4], double c2, long long bst, double *out,
                   int spin_half = 0);
// broadcast a tau-independent block over the batch: dst[b] = src
int kv_bcast(kvft_ctx *ctx, int batch, size_t count, const double *src,
             double *dst);

// The tau integral out[y] = sum_x G[y,x] w(y,x) tbar[x] over P elements per
// tau point, w = exp((ti[x]-ti[y]) d) for x <= y and, for x > y, 1 (the
// reference's rule) or the same exponential (full); d from D or, when D is
// null, ev[p]-eo[q] (rank 1) / ev[a]+ev[b]-eo[i]-eo[j] (rank 2).  ti and G on
// the device, hti/hG their host copies.  mode 1 also damps and takes norms.
int kv_quad_launch(kvft_ctx *ctx, int mode, int ng, long long P, int rank, int nv, int no,
                   const double *tbar, const double *ti, const double *hti, const double *G,
                   const double *hG, const double *D, const double *ev, const double *eo,
                   int full, double alpha, double *out, double *res, int spin_half = 0);
int kv_int_tbar(kvft_ctx *ctx, int ng, size_t P, const double *tbar,
                const double *ti, const double *D, const double *eps_v,
                const double *eps_o, int nv, int no, int rank,
                const double *G, int full, double *out);

// spin_half > 0: the amplitudes vanish outside the spin-conserving blocks
// (alpha half first), whose zero tiles are skipped
int kv_energy(kvft_ctx *ctx, int ng, int nv, int no, const double *T1,
              const double *T2, const double *f, const double *eri,
              const double *g, double beta, int qterm, double *dres, int spin_half = 0);

// T1/T2 += fac * residual; with seed_t2, T2 = -seed_t2 + fac * residual
// (T2 need not be initialised).
int kv_stanton(kvft_ctx *ctx, int nb, int nv, int no,
               const double *const F[4], const double *const I[9],
               const double *t1, const double *t2, double fac, double *T1,
               double *T2, const double *seed_t2 = nullptr);
size_t kv_stanton_workspace(int nb, int nv, int no);

// ---- contractions named by index strings ------------------------------------
// A tensor laid out row-major over the letters of `ix` (last fastest); a..h
// run over the nv virtual orbitals, i..n over the no occupied ones.  bst is
// the stride between tau points (0: shared by the batch).
struct KvTen {
    const double *p;
    const char *ix;
    long long bst;
    int stable;                      // an integral block (fixed for a solver's lifetime)
    // spin rule over the axes of ix: '+'/'-' signs with sum sign * spin = 0 on
    // every nonzero element ("+-" for two axes, "++--" for four when null)
    const char *spin = nullptr;
};
// The strided-GEMM form of C[cix] = alpha sum A[A.ix] B[B.ix] + beta C: rows
// are the letters of A and C, columns those of B and C, the sum runs over the
// letters of A and B; each group keeps at most three strided components.
int kv_einsum_desc(int nv, int no, const char *aix, const char *bix, const char *cix,
                   int *M, int *N, int *K, KIdx *Ar, KIdx *Ac, KIdx *Br, KIdx *Bc,
                   KIdx *Cr, KIdx *Cc, std::string *err, int sub = 0);
int kv_einsum(kvft_ctx *ctx, int nv, int no, int batch, double alpha, const KvTen &A,
              const KvTen &B, double beta, double *C, const char *cix, long long cbst);
// dst[dix] = beta dst + alpha src[src.ix] over the same letters (a transpose
// or a copy; at most four letters)
int kv_add(kvft_ctx *ctx, int nv, int no, int batch, double alpha, const KvTen &src,
           double beta, double *dst, const char *dix, long long dbst);
// *out = sum (a x + b y)^2 over a [batch][d0][d1][d2][d3] index space with the
// given element strides (y may be null), in a fixed summation order
int kv_sumsq4(kvft_ctx *ctx, int batch, const int dims[4], double a, const double *x,
              const long long xs[4], long long xbst, double b, const double *y,
              const long long ys[4], long long ybst, double *out);

// Lambda terms of one tau batch: g = R'(t)^T m, the transpose of the
// residual's Jacobian applied to m (m1[i,a], m2[i,j,a,b] in Lambda layout;
// g1[a,i], g2[a,b,i,j] in amplitude layout, g2 antisymmetric), with
//   sum g1 dt1 + 1/4 sum g2 dt2 = sum m1 dR1 + 1/4 sum m2 dR2.
// With Fg[4] / Ig[9] (nb = 1) it also adds wt times the gradient of
// sum m1 R1 + 1/4 sum m2 R2 with respect to each integral block the residual
// reads (blocks laid out as F, I; F.vo and I.vvoo get nothing).
int kv_lambda_vjp(kvft_ctx *ctx, int nb, int nv, int no, const double *const F[4],
                  const double *const I[9], const double *t1, const double *t2,
                  const double *m1, const double *m2, double *g1, double *g2,
                  double *const *Fg = nullptr, double *const *Ig = nullptr, double wt = 1.0);
size_t kv_lambda_workspace(int nb, int nv, int no);
size_t kv_chunk_bytes_per_tau(kvft_ctx *ctx, int nv, int no);
