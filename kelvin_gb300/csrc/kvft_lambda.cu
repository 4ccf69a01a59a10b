// The Lambda terms of FT-CCSD on the device: R'(t)^T m, the transpose of the
// CCSD residual's Jacobian applied to a Lambda-shaped tensor.  Kelvin's Lambda
// iteration (kelvin/ft_cc_equations.py:385-409) hands these terms to
// cqcpy.cc_equations._Lambda_opt; Lambda is the adjoint of the amplitude
// iteration, so they are evaluated here as the reverse pass through the same
// Stanton-Gauss intermediates the residual builds (F_ae, F_mi, F_me, W_mnij,
// W_abef, W_mbej), term by term.
//
// Every contraction is written as an index-string contraction (kv_einsum),
// which lowers to one strided GEMM (kv_gemm: tensor cores or the FP64 pipe),
// and every permuted sum as a strided axpby (kv_add); no other kernel runs.
// The intermediates are kept in plain (not pair-compressed) form; the spin-
// block and pair-ladder savings of the forward residual are not applied here.
#include "kvft_internal.h"

#include <cmath>
#include <cstring>

namespace {

long long letter_extent(char c, int nv, int no) {
    if (c >= 'a' && c <= 'h') return nv;
    if (c >= 'i' && c <= 'n') return no;
    return -1;
}

struct Layout {
    std::string ix;
    std::vector<long long> ext, st;
    long long size = 1;
};

bool make_layout(const char *ix, int nv, int no, Layout *L, std::string *err) {
    L->ix = ix ? ix : "";
    const int n = (int)L->ix.size();
    if (n == 0 || n > 4) {
        *err = "einsum: a tensor needs one to four indices: " + L->ix;
        return false;
    }
    L->ext.assign(n, 0);
    L->st.assign(n, 0);
    long long s = 1;
    for (int k = n - 1; k >= 0; k--) {
        const long long e = letter_extent(L->ix[k], nv, no);
        if (e < 0) {
            *err = "einsum: index letters are a-h (virtual) or i-n (occupied): " + L->ix;
            return false;
        }
        if (L->ix.find(L->ix[k]) != (size_t)k) {
            *err = "einsum: repeated index in " + L->ix;
            return false;
        }
        L->ext[k] = e;
        L->st[k] = s;
        s *= e;
    }
    L->size = s;
    return true;
}

long long stride_of(const Layout &L, char c) {
    const size_t k = L.ix.find(c);
    return k == std::string::npos ? -1 : L.st[k];
}

// One composite index (at most three strided components) per tensor for the
// letters of group g, merging neighbours that are contiguous in every tensor.
bool group_index(const std::string &g, const Layout *const *ts, KIdx *const *out, int nt,
                 int nv, int no, std::string *err, int sub = 0) {
    struct Comp {
        long long ext;
        long long st[2];
    };
    std::vector<Comp> comps;
    for (char c : g) {
        Comp cp;
        cp.ext = sub > 0 ? sub : letter_extent(c, nv, no);
        for (int t = 0; t < nt; t++) cp.st[t] = stride_of(*ts[t], c);
        comps.push_back(cp);
    }
    while (comps.size() > 3) {
        bool merged = false;
        for (size_t k = 0; k + 1 < comps.size() && !merged; k++) {
            bool ok = true;
            for (int t = 0; t < nt; t++)
                if (comps[k].st[t] != comps[k + 1].st[t] * comps[k + 1].ext) ok = false;
            if (ok) {
                comps[k].ext *= comps[k + 1].ext;
                for (int t = 0; t < nt; t++) comps[k].st[t] = comps[k + 1].st[t];
                comps.erase(comps.begin() + k + 1);
                merged = true;
            }
        }
        if (!merged) {
            *err = "einsum: index group " + g + " needs more than three strided components";
            return false;
        }
    }
    const int off = 3 - (int)comps.size();
    for (int t = 0; t < nt; t++) {
        KIdx &x = *out[t];
        x = KIdx{{1, 1, 1}, {0, 0, 0}};
        for (size_t k = 0; k < comps.size(); k++) {
            x.size[off + k] = (int)comps[k].ext;
            x.st[off + k] = comps[k].st[t];
        }
    }
    return true;
}

}  // namespace

int kv_einsum_desc(int nv, int no, const char *aix, const char *bix, const char *cix, int *M,
                   int *N, int *K, KIdx *Ar, KIdx *Ac, KIdx *Br, KIdx *Bc, KIdx *Cr, KIdx *Cc,
                   std::string *err, int sub) {
    Layout A, B, C;
    if (!make_layout(aix, nv, no, &A, err) || !make_layout(bix, nv, no, &B, err) ||
        !make_layout(cix, nv, no, &C, err))
        return KVFT_EINVAL;
    const size_t npos = std::string::npos;
    std::string gm, gn, gk;
    for (char c : A.ix) {
        const bool inB = B.ix.find(c) != npos, inC = C.ix.find(c) != npos;
        if (inB == inC) {
            *err = std::string("einsum: index ") + c + " must be in exactly one of " + B.ix +
                   " and " + C.ix;
            return KVFT_EINVAL;
        }
        if (inB) gk += c;
    }
    for (char c : B.ix)
        if ((A.ix.find(c) != npos) == (C.ix.find(c) != npos)) {
            *err = std::string("einsum: index ") + c + " must be in exactly one of " + A.ix +
                   " and " + C.ix;
            return KVFT_EINVAL;
        }
    for (char c : C.ix) {
        const bool inA = A.ix.find(c) != npos, inB = B.ix.find(c) != npos;
        if (inA == inB) {
            *err = std::string("einsum: output index ") + c + " must come from one input";
            return KVFT_EINVAL;
        }
        (inA ? gm : gn) += c;
    }
    const Layout *mt[2] = {&A, &C}, *nt[2] = {&B, &C}, *kt[2] = {&A, &B};
    KIdx *mo[2] = {Ar, Cr}, *no_[2] = {Bc, Cc}, *ko[2] = {Ac, Br};
    if (!group_index(gm, mt, mo, 2, nv, no, err, sub) ||
        !group_index(gn, nt, no_, 2, nv, no, err, sub) ||
        !group_index(gk, kt, ko, 2, nv, no, err, sub))
        return KVFT_EINVAL;
    const long long m = (long long)Ar->size[0] * Ar->size[1] * Ar->size[2];
    const long long n = (long long)Bc->size[0] * Bc->size[1] * Bc->size[2];
    const long long k = (long long)Ac->size[0] * Ac->size[1] * Ac->size[2];
    if (m > 0x7fffffffLL || n > 0x7fffffffLL || k > 0x7fffffffLL) {
        *err = "einsum: a GEMM dimension exceeds 2^31";
        return KVFT_EINVAL;
    }
    *M = (int)m;
    *N = (int)n;
    *K = (int)k;
    return KVFT_OK;
}

namespace {

// One strided GEMM for a contraction already in GEMM form; a single row goes
// as the transposed product C^T = B^T A^T, so that the long free dimension
// is the GEMM's row dimension.
int gemm_piece(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha, const KvTen &A,
               const KvTen &B, const KIdx &ar, const KIdx &ac, const KIdx &br, const KIdx &bc,
               double beta, double *C, const KIdx &cr, const KIdx &cc, long long cbst) {
    if (M == 1 && N > 1) {
        KMat a{B.p, bc, br, B.bst, B.stable}, b{A.p, ac, ar, A.bst, A.stable};
        KOut c{C, cc, cr, cbst};
        return kv_gemm(ctx, N, M, K, batch, alpha, a, b, beta, c);
    }
    KMat a{A.p, ar, ac, A.bst, A.stable}, b{B.p, br, bc, B.bst, B.stable};
    KOut c{C, cr, cc, cbst};
    return kv_gemm(ctx, M, N, K, batch, alpha, a, b, beta, c);
}

// true when the spin assignment (bit of each letter in `spins`) satisfies
// the tensor's rule
bool spin_ok(const KvTen &T, const unsigned char *bit) {
    const size_t n = std::strlen(T.ix);
    const char *rule = T.spin ? T.spin : (n == 2 ? "+-" : "++--");
    if (std::strlen(rule) != n) return true;
    int sum = 0;
    for (size_t k = 0; k < n; k++)
        sum += (rule[k] == '+' ? 1 : -1) * bit[(unsigned char)T.ix[k]];
    return sum == 0;
}

long long spin_offset(const char *ix, const unsigned char *bit, int h, int nv, int no) {
    const size_t n = std::strlen(ix);
    long long st = 1, off = 0;
    for (size_t k = n; k-- > 0;) {
        off += (long long)bit[(unsigned char)ix[k]] * h * st;
        st *= letter_extent(ix[k], nv, no);
    }
    return off;
}

}  // namespace

int kv_einsum(kvft_ctx *ctx, int nv, int no, int batch, double alpha, const KvTen &A,
              const KvTen &B, double beta, double *C, const char *cix, long long cbst) {
    int M, N, K;
    KIdx ar, ac, br, bc, cr, cc;
    std::string err;
    if (kv_einsum_desc(nv, no, A.ix, B.ix, cix, &M, &N, &K, &ar, &ac, &br, &bc, &cr, &cc,
                       &err) != KVFT_OK)
        return kv_fail(ctx, KVFT_EINVAL, err);
    const int h = ctx->lam_spin;
    if (h <= 0 || nv != no || nv != 2 * h)
        return gemm_piece(ctx, M, N, K, batch, alpha, A, B, ar, ac, br, bc, beta, C, cr, cc,
                          cbst);
    // Spin blocks: every letter runs over an alpha half and a beta half, and
    // only the products whose operands satisfy their spin rules are nonzero.
    // C is scaled by beta first; the products then add into it.
    if (beta != 1.0) KV_TRY(kv_scale_view(ctx, M, N, batch, beta, KOut{C, cr, cc, cbst}));
    std::string letters;
    for (const char *p : {A.ix, B.ix})
        for (const char *q = p; *q; q++)
            if (letters.find(*q) == std::string::npos) letters += *q;
    int sM, sN, sK;
    KIdx sar, sac, sbr, sbc, scr, scc;
    if (kv_einsum_desc(nv, no, A.ix, B.ix, cix, &sM, &sN, &sK, &sar, &sac, &sbr, &sbc, &scr,
                       &scc, &err, h) != KVFT_OK)
        return kv_fail(ctx, KVFT_EINVAL, err);
    unsigned char bit[128] = {0};
    const int L = (int)letters.size();
    for (unsigned m = 0; m < (1u << L); m++) {
        for (int k = 0; k < L; k++) bit[(unsigned char)letters[k]] = (m >> k) & 1;
        if (!spin_ok(A, bit) || !spin_ok(B, bit)) continue;
        KvTen a = A, b = B;
        a.p += spin_offset(A.ix, bit, h, nv, no);
        b.p += spin_offset(B.ix, bit, h, nv, no);
        double *c = C + spin_offset(cix, bit, h, nv, no);
        KV_TRY(gemm_piece(ctx, sM, sN, sK, batch, alpha, a, b, sar, sac, sbr, sbc, 1.0, c, scr,
                          scc, cbst));
    }
    return KVFT_OK;
}

int kv_add(kvft_ctx *ctx, int nv, int no, int batch, double alpha, const KvTen &src,
           double beta, double *dst, const char *dix, long long dbst) {
    Layout S, D;
    std::string err;
    if (!make_layout(src.ix, nv, no, &S, &err) || !make_layout(dix, nv, no, &D, &err))
        return kv_fail(ctx, KVFT_EINVAL, err);
    if (S.ix.size() != D.ix.size())
        return kv_fail(ctx, KVFT_EINVAL, "add: " + S.ix + " and " + D.ix + " differ");
    int dims[4] = {1, 1, 1, 1};
    long long ss[4] = {0, 0, 0, 0}, ds[4] = {0, 0, 0, 0};
    const int off = 4 - (int)D.ix.size();
    for (size_t k = 0; k < D.ix.size(); k++) {
        const long long s = stride_of(S, D.ix[k]);
        if (s < 0) return kv_fail(ctx, KVFT_EINVAL, "add: " + S.ix + " and " + D.ix + " differ");
        dims[off + k] = (int)D.ext[k];
        ds[off + k] = D.st[k];
        ss[off + k] = s;
    }
    return kv_axpby4(ctx, batch, dims, alpha, src.p, ss, src.bst, beta, dst, ds, dbst);
}

// ---- sums of squares (the iteration's norms) ----------------------------------

namespace {

struct SQ {
    int d[4];
    long long xs[4], ys[4], xbst, ybst;
};

constexpr int SQ_T = 256;

// per-block partial sums of (a x + b y)^2 over a flat walk of the index space
__global__ void __launch_bounds__(SQ_T)
sumsq_kernel(long long total, SQ q, double a, const double *__restrict__ x, double b,
             const double *__restrict__ y, double *__restrict__ part) {
    double acc = 0.0;
    for (long long t = blockIdx.x * (long long)SQ_T + threadIdx.x; t < total;
         t += (long long)gridDim.x * SQ_T) {
        long long r = t;
        const int i3 = (int)(r % q.d[3]); r /= q.d[3];
        const int i2 = (int)(r % q.d[2]); r /= q.d[2];
        const int i1 = (int)(r % q.d[1]); r /= q.d[1];
        const int i0 = (int)(r % q.d[0]);
        const long long bt = r / q.d[0];
        double v = a * x[bt * q.xbst + i0 * q.xs[0] + i1 * q.xs[1] + i2 * q.xs[2] +
                         i3 * q.xs[3]];
        if (y)
            v = fma(b, y[bt * q.ybst + i0 * q.ys[0] + i1 * q.ys[1] + i2 * q.ys[2] +
                         i3 * q.ys[3]], v);
        acc = fma(v, v, acc);
    }
    __shared__ double red[SQ_T];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = SQ_T / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_parts_kernel(const double *__restrict__ part, int n, double *out) {
    __shared__ double red[SQ_T];
    double acc = 0.0;
    for (int k = threadIdx.x; k < n; k += SQ_T) acc += part[k];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = SQ_T / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

int kv_sumsq4(kvft_ctx *ctx, int batch, const int dims[4], double a, const double *x,
              const long long xs[4], long long xbst, double b, const double *y,
              const long long ys[4], long long ybst, double *out) {
    long long total = batch;
    for (int k = 0; k < 4; k++) total *= dims[k];
    if (ctx->dry) {
        KvDryOp op;
        op.kind = 4;
        op.batch = batch, op.alpha = a, op.beta = b;
        for (int k = 0; k < 4; k++) op.dims[k] = dims[k], op.ss[k] = xs[k], op.ds[k] = ys[k];
        op.sbst = xbst, op.dbst = ybst, op.src = x, op.src2 = y, op.res = out;
        ctx->dry->push_back(op);
        return KVFT_OK;
    }
    SQ q;
    for (int k = 0; k < 4; k++) q.d[k] = dims[k], q.xs[k] = xs[k], q.ys[k] = y ? ys[k] : 0;
    q.xbst = xbst;
    q.ybst = y ? ybst : 0;
    const int grid = (int)std::max(1LL, std::min((total + SQ_T - 1) / SQ_T,
                                                 (long long)ctx->sm_count * 8));
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "sumsq_part", sizeof(double) * grid, &part));
    KvProfScope prof(ctx, KV_CAT_ELEM, 8.0 * total * (y ? 2 : 1));
    sumsq_kernel<<<grid, SQ_T, 0, ctx->stream>>>(total, q, a, x, b, y, (double *)part);
    KV_TRY(kv_launch_check(ctx, "sumsq"));
    sum_parts_kernel<<<1, SQ_T, 0, ctx->stream>>>((const double *)part, grid, out);
    return kv_launch_check(ctx, "sum_parts");
}

// ---- the reverse pass ----------------------------------------------------------

namespace {

struct LWS {
    double *tau, *ttau, *tmp, *Wmbej, *Wabef, *Wmnij, *Fae, *Fmi, *Fme, *Xbe, *Xmj;
    double *xA, *xI, *xAI, *Y1, *Y2, *taub, *ttaub, *ttb, *t2b, *tmpb, *Wmbejb, *Wabefb,
        *Wmnijb, *xW4, *Faeb, *Fmib, *Fmeb, *Xbeb, *Xmjb;
};

// doubles per tau point, in carve order
void ws_sizes(long long v, long long o, long long *sz) {
    const long long v2o2 = v * v * o * o, v4 = v * v * v * v, o4 = o * o * o * o;
    const long long t[30] = {v2o2, v2o2, v2o2, v2o2, v4, o4, v * v, o * o, o * v, v * v,
                             o * o, v2o2, v2o2, v2o2, v * o * o * o, v * v * v * o, v2o2, v2o2,
                             v2o2, v2o2, v2o2, v2o2, v4, o4, std::max(v4, o4), v * v, o * o,
                             o * v, v * v, o * o};
    for (int k = 0; k < 30; k++) sz[k] = t[k];
}

long long per_tau(long long v, long long o) {
    long long sz[30], s = 0;
    ws_sizes(v, o, sz);
    for (int k = 0; k < 30; k++) s += (sz[k] + 1) / 2 * 2;      // 16-byte aligned slices
    return s;
}

LWS carve(double *p, int nb, long long v, long long o) {
    long long sz[30];
    ws_sizes(v, o, sz);
    double **slot[30];
    LWS w;
    double **q[30] = {&w.tau, &w.ttau, &w.tmp, &w.Wmbej, &w.Wabef, &w.Wmnij, &w.Fae, &w.Fmi,
                      &w.Fme, &w.Xbe, &w.Xmj, &w.xA, &w.xI, &w.xAI, &w.Y1, &w.Y2, &w.taub,
                      &w.ttaub, &w.ttb, &w.t2b, &w.tmpb, &w.Wmbejb, &w.Wabefb, &w.Wmnijb,
                      &w.xW4, &w.Faeb, &w.Fmib, &w.Fmeb, &w.Xbeb, &w.Xmjb};
    for (int k = 0; k < 30; k++) slot[k] = q[k];
    for (int k = 0; k < 30; k++) {
        *slot[k] = p;
        p += (long long)nb * ((sz[k] + 1) / 2 * 2);
    }
    return w;
}

}  // namespace

size_t kv_lambda_workspace(int nb, int nv, int no) {
    return sizeof(double) * (size_t)nb * (size_t)per_tau(nv, no);
}

int kv_lambda_vjp(kvft_ctx *ctx, int nb, int nv, int no, const double *const F[4],
                  const double *const I[9], const double *t1, const double *t2,
                  const double *m1, const double *m2, double *g1, double *g2,
                  double *const *Fg, double *const *Ig, double wt) {
    if (nb <= 0) return KVFT_OK;
    if ((Fg || Ig) && (!Fg || !Ig || nb != 1))
        return kv_fail(ctx, KVFT_EINVAL, "lambda: integral gradients take one tau point");
    const long long v = nv, o = no;
    const long long vo = v * o, v2o2 = v * v * o * o;
    const double *Foo = F[0], *Fov = F[1], *Fvv = F[3];
    const double *vvvv = I[0], *vvvo = I[1], *vovv = I[2], *vovo = I[4], *oovv = I[5],
                 *vooo = I[6], *ooov = I[7], *oooo = I[8];
    void *wsp = nullptr;
    KV_TRY(kv_scratch(ctx, "lambda", kv_lambda_workspace(nb, nv, no), &wsp));
    long long sz[30];
    ws_sizes(v, o, sz);
    const LWS w = carve((double *)wsp, nb, v, o);
    const int B = nb;
    // per-tau strides of the workspace slices (16-byte aligned sizes)
    auto bs = [&](int k) { return (sz[k] + 1) / 2 * 2; };
    const long long s_tau = bs(0), s_tmp = bs(2), s_wmbej = bs(3), s_w4v = bs(4),
                    s_w4o = bs(5), s_vv = bs(6), s_oo = bs(7), s_ov = bs(8), s_y1 = bs(14),
                    s_y2 = bs(15), s_x4 = bs(24);

    // tensors: an integral block (shared, stable), a per-tau operand
    auto IB = [](const double *p, const char *ix) { return KvTen{p, ix, 0, 1}; };
    auto TT = [](const double *p, const char *ix, long long bst) { return KvTen{p, ix, bst, 0}; };
    auto E = [&](double alpha, const KvTen &A, const KvTen &Bt, double beta, double *C,
                 const char *cix, long long cbst) {
        return kv_einsum(ctx, nv, no, B, alpha, A, Bt, beta, C, cix, cbst);
    };
    auto ADD = [&](double alpha, const KvTen &S, double beta, double *D, const char *dix,
                   long long dbst) { return kv_add(ctx, nv, no, B, alpha, S, beta, D, dix, dbst); };
    // integral gradients (one tau point, weight wt), accumulated when asked for
    auto GE = [&](double alpha, const KvTen &A, const KvTen &Bt, double *C, const char *cix) {
        return Fg ? kv_einsum(ctx, nv, no, 1, alpha * wt, A, Bt, 1.0, C, cix, 0) : KVFT_OK;
    };
    auto GA = [&](double alpha, const KvTen &S, double *D, const char *dix) {
        return Fg ? kv_add(ctx, nv, no, 1, alpha * wt, S, 1.0, D, dix, 0) : KVFT_OK;
    };

    // ---- forward intermediates (oracle cc_equations.intermediates) ----------
    // ttau = t2 + 1/2 P(ab) t1 t1, tau = t2 + P(ab) t1 t1
    KV_TRY(ADD(1.0, TT(t2, "abij", v2o2), 0.0, w.ttau, "abij", s_tau));
    KV_TRY(E(0.5, TT(t1, "ai", vo), TT(t1, "bj", vo), 1.0, w.ttau, "abij", s_tau));
    KV_TRY(E(-0.5, TT(t1, "bi", vo), TT(t1, "aj", vo), 1.0, w.ttau, "abij", s_tau));
    KV_TRY(ADD(1.0, TT(t2, "abij", v2o2), 0.0, w.tau, "abij", s_tau));
    KV_TRY(E(1.0, TT(t1, "ai", vo), TT(t1, "bj", vo), 1.0, w.tau, "abij", s_tau));
    KV_TRY(E(-1.0, TT(t1, "bi", vo), TT(t1, "aj", vo), 1.0, w.tau, "abij", s_tau));
    // F_ae = vv - 1/2 ov[m,e] t1[a,m] - t1[f,m] vovv[a,m,f,e] - 1/2 ttau[a,f,m,n] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, IB(Fvv, "ae"), 0.0, w.Fae, "ae", s_vv));
    KV_TRY(E(-0.5, IB(Fov, "me"), TT(t1, "am", vo), 1.0, w.Fae, "ae", s_vv));
    KV_TRY(E(-1.0, TT(t1, "fm", vo), IB(vovv, "amfe"), 1.0, w.Fae, "ae", s_vv));
    KV_TRY(E(-0.5, TT(w.ttau, "afmn", s_tau), IB(oovv, "mnef"), 1.0, w.Fae, "ae", s_vv));
    // F_mi = oo + 1/2 t1[e,i] ov[m,e] + t1[e,n] ooov[m,n,i,e] + 1/2 ttau[e,f,i,n] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, IB(Foo, "mi"), 0.0, w.Fmi, "mi", s_oo));
    KV_TRY(E(0.5, TT(t1, "ei", vo), IB(Fov, "me"), 1.0, w.Fmi, "mi", s_oo));
    KV_TRY(E(1.0, TT(t1, "en", vo), IB(ooov, "mnie"), 1.0, w.Fmi, "mi", s_oo));
    KV_TRY(E(0.5, TT(w.ttau, "efin", s_tau), IB(oovv, "mnef"), 1.0, w.Fmi, "mi", s_oo));
    // F_me = ov + t1[f,n] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, IB(Fov, "me"), 0.0, w.Fme, "me", s_ov));
    KV_TRY(E(1.0, TT(t1, "fn", vo), IB(oovv, "mnef"), 1.0, w.Fme, "me", s_ov));
    // W_mnij = oooo + P(ij) t1[e,j] ooov[m,n,i,e] + 1/4 tau[e,f,i,j] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, IB(oooo, "mnij"), 0.0, w.Wmnij, "mnij", s_w4o));
    KV_TRY(E(1.0, TT(t1, "ej", vo), IB(ooov, "mnie"), 1.0, w.Wmnij, "mnij", s_w4o));
    KV_TRY(E(-1.0, TT(t1, "ej", vo), IB(ooov, "mnie"), 1.0, w.Wmnij, "mnji", s_w4o));
    KV_TRY(E(0.25, TT(w.tau, "efij", s_tau), IB(oovv, "mnef"), 1.0, w.Wmnij, "mnij", s_w4o));
    // W_abef = vvvv - P(ab) t1[b,m] vovv[a,m,e,f] + 1/4 tau[a,b,m,n] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, IB(vvvv, "abef"), 0.0, w.Wabef, "abef", s_w4v));
    KV_TRY(E(-1.0, TT(t1, "bm", vo), IB(vovv, "amef"), 1.0, w.Wabef, "abef", s_w4v));
    KV_TRY(E(1.0, TT(t1, "bm", vo), IB(vovv, "amef"), 1.0, w.Wabef, "baef", s_w4v));
    KV_TRY(E(0.25, TT(w.tau, "abmn", s_tau), IB(oovv, "mnef"), 1.0, w.Wabef, "abef", s_w4v));
    // tmp = 1/2 t2[f,b,j,n] + t1[f,j] t1[b,n]
    KV_TRY(ADD(0.5, TT(t2, "fbjn", v2o2), 0.0, w.tmp, "fbjn", s_tmp));
    KV_TRY(E(1.0, TT(t1, "fj", vo), TT(t1, "bn", vo), 1.0, w.tmp, "fbjn", s_tmp));
    // W_mbej = -vovo[b,m,e,j] - t1[f,j] vovv[b,m,e,f] + t1[b,n] ooov[m,n,j,e]
    //          - tmp[f,b,j,n] oovv[m,n,e,f]
    KV_TRY(ADD(-1.0, IB(vovo, "bmej"), 0.0, w.Wmbej, "mbej", s_wmbej));
    KV_TRY(E(-1.0, TT(t1, "fj", vo), IB(vovv, "bmef"), 1.0, w.Wmbej, "mbej", s_wmbej));
    KV_TRY(E(1.0, TT(t1, "bn", vo), IB(ooov, "mnje"), 1.0, w.Wmbej, "mbej", s_wmbej));
    KV_TRY(E(-1.0, TT(w.tmp, "fbjn", s_tmp), IB(oovv, "mnef"), 1.0, w.Wmbej, "mbej", s_wmbej));

    // ---- R2 terms, with R2b = m2 / 4 ------------------------------------------
    // xA = P(ab) R2b, xI = P(ij) R2b, xAI = P(ab) P(ij) R2b (amplitude layout)
    KV_TRY(ADD(0.25, TT(m2, "ijab", v2o2), 0.0, w.xA, "abij", s_tau));
    KV_TRY(ADD(-0.25, TT(m2, "ijba", v2o2), 1.0, w.xA, "abij", s_tau));
    KV_TRY(ADD(0.25, TT(m2, "ijab", v2o2), 0.0, w.xI, "abij", s_tau));
    KV_TRY(ADD(-0.25, TT(m2, "jiab", v2o2), 1.0, w.xI, "abij", s_tau));
    KV_TRY(ADD(1.0, TT(w.xA, "abij", s_tau), 0.0, w.xAI, "abij", s_tau));
    KV_TRY(ADD(-1.0, TT(w.xA, "abji", s_tau), 1.0, w.xAI, "abij", s_tau));
    // x = t1[a,m] vooo[b,m,i,j]: t1b[a,m] = xA . vooo   (first write of g1)
    KV_TRY(E(1.0, TT(w.xA, "abij", s_tau), IB(vooo, "bmij"), 0.0, g1, "am", vo));
    KV_TRY(GE(1.0, TT(w.xA, "abij", s_tau), TT(t1, "am", vo), Fg ? Ig[6] : nullptr, "bmij"));
    // x = t1[e,i] vvvo[a,b,e,j]
    KV_TRY(E(1.0, TT(w.xI, "abij", s_tau), IB(vvvo, "abej"), 1.0, g1, "ei", vo));
    KV_TRY(GE(1.0, TT(w.xI, "abij", s_tau), TT(t1, "ei", vo), Fg ? Ig[1] : nullptr, "abej"));
    // ring: x = t2[a,e,i,m] W_mbej + t1[e,i] t1[a,m] vovo[b,m,e,j]   (first write of t2b)
    KV_TRY(E(1.0, TT(w.xAI, "abij", s_tau), TT(w.Wmbej, "mbej", s_wmbej), 0.0, w.t2b, "aeim",
             s_tau));
    KV_TRY(E(1.0, TT(w.xAI, "abij", s_tau), TT(t2, "aeim", v2o2), 0.0, w.Wmbejb, "mbej",
             s_wmbej));
    KV_TRY(E(1.0, TT(w.xAI, "abij", s_tau), TT(t1, "am", vo), 0.0, w.Y1, "bijm", s_y1));
    // Y1[b,i,j,m] conserves b + m = i + j
    KV_TRY(E(1.0, KvTen{w.Y1, "bijm", s_y1, 0, "+--+"}, IB(vovo, "bmej"), 1.0, g1, "ei", vo));
    KV_TRY(E(1.0, TT(w.xAI, "abij", s_tau), TT(t1, "ei", vo), 0.0, w.Y2, "abej", s_y2));
    KV_TRY(E(1.0, TT(w.Y2, "abej", s_y2), IB(vovo, "bmej"), 1.0, g1, "am", vo));
    KV_TRY(GE(1.0, TT(w.Y2, "abej", s_y2), TT(t1, "am", vo), Fg ? Ig[4] : nullptr, "bmej"));
    // R2 += 1/2 tau[e,f,i,j] W_abef and 1/2 tau[a,b,m,n] W_mnij (R2b = m2/4)
    KV_TRY(E(0.125, TT(m2, "ijab", v2o2), TT(w.Wabef, "abef", s_w4v), 0.0, w.taub, "efij",
             s_tau));
    KV_TRY(E(0.125, TT(m2, "ijab", v2o2), TT(w.tau, "efij", s_tau), 0.0, w.Wabefb, "abef",
             s_w4v));
    KV_TRY(E(0.125, TT(m2, "ijab", v2o2), TT(w.Wmnij, "mnij", s_w4o), 1.0, w.taub, "abmn",
             s_tau));
    KV_TRY(E(0.125, TT(m2, "ijab", v2o2), TT(w.tau, "abmn", s_tau), 0.0, w.Wmnijb, "mnij",
             s_w4o));
    // x = t2[a,b,i,m] X_mj, X_mj = F_mi + 1/2 t1[e,j] F_me;  R2 -= P(ij) x
    KV_TRY(ADD(1.0, TT(w.Fmi, "mj", s_oo), 0.0, w.Xmj, "mj", s_oo));
    KV_TRY(E(0.5, TT(t1, "ej", vo), TT(w.Fme, "me", s_ov), 1.0, w.Xmj, "mj", s_oo));
    KV_TRY(E(-1.0, TT(w.xI, "abij", s_tau), TT(w.Xmj, "mj", s_oo), 1.0, w.t2b, "abim", s_tau));
    KV_TRY(E(-1.0, TT(w.xI, "abij", s_tau), TT(t2, "abim", v2o2), 0.0, w.Xmjb, "mj", s_oo));
    // x = t2[a,e,i,j] X_be, X_be = F_ae - 1/2 t1[b,m] F_me;  R2 += P(ab) x
    KV_TRY(ADD(1.0, TT(w.Fae, "be", s_vv), 0.0, w.Xbe, "be", s_vv));
    KV_TRY(E(-0.5, TT(t1, "bm", vo), TT(w.Fme, "me", s_ov), 1.0, w.Xbe, "be", s_vv));
    KV_TRY(E(1.0, TT(w.xA, "abij", s_tau), TT(w.Xbe, "be", s_vv), 1.0, w.t2b, "aeij", s_tau));
    KV_TRY(E(1.0, TT(w.xA, "abij", s_tau), TT(t2, "aeij", v2o2), 0.0, w.Xbeb, "be", s_vv));
    // back through X_mj and X_be
    KV_TRY(ADD(1.0, TT(w.Xmjb, "mi", s_oo), 0.0, w.Fmib, "mi", s_oo));
    KV_TRY(E(0.5, TT(w.Xmjb, "mj", s_oo), TT(w.Fme, "me", s_ov), 1.0, g1, "ej", vo));
    KV_TRY(E(0.5, TT(w.Xmjb, "mj", s_oo), TT(t1, "ej", vo), 0.0, w.Fmeb, "me", s_ov));
    KV_TRY(ADD(1.0, TT(w.Xbeb, "ae", s_vv), 0.0, w.Faeb, "ae", s_vv));
    KV_TRY(E(-0.5, TT(w.Xbeb, "be", s_vv), TT(w.Fme, "me", s_ov), 1.0, g1, "bm", vo));
    KV_TRY(E(-0.5, TT(w.Xbeb, "be", s_vv), TT(t1, "bm", vo), 1.0, w.Fmeb, "me", s_ov));

    // ---- R1 terms, R1b = m1 ----------------------------------------------------
    const KvTen m1v = TT(m1, "ia", vo);
    KV_TRY(E(1.0, m1v, TT(t1, "ei", vo), 1.0, w.Faeb, "ae", s_vv));
    KV_TRY(E(1.0, m1v, TT(w.Fae, "ae", s_vv), 1.0, g1, "ei", vo));
    KV_TRY(E(-1.0, TT(m1, "ia", vo), TT(w.Fmi, "mi", s_oo), 1.0, g1, "am", vo));
    KV_TRY(E(-1.0, TT(m1, "ia", vo), TT(t1, "am", vo), 1.0, w.Fmib, "mi", s_oo));
    KV_TRY(E(1.0, m1v, TT(w.Fme, "me", s_ov), 1.0, w.t2b, "aeim", s_tau));
    KV_TRY(E(1.0, m1v, TT(t2, "aeim", v2o2), 1.0, w.Fmeb, "me", s_ov));
    KV_TRY(E(-1.0, m1v, IB(vovo, "anfi"), 1.0, g1, "fn", vo));
    KV_TRY(E(0.5, m1v, IB(vovv, "amef"), 1.0, w.t2b, "efim", s_tau));
    KV_TRY(E(0.5, m1v, IB(ooov, "nmie"), 1.0, w.t2b, "aemn", s_tau));
    if (Fg) {
        KV_TRY(GE(-1.0, m1v, TT(t1, "fn", vo), Ig[4], "anfi"));
        KV_TRY(GE(0.5, m1v, TT(t2, "efim", v2o2), Ig[2], "amef"));
        KV_TRY(GE(0.5, m1v, TT(t2, "aemn", v2o2), Ig[7], "nmie"));
    }

    // ---- back through the intermediates ----------------------------------------
    // W_abef: -P(ab) t1[b,m] vovv[a,m,e,f] and 1/4 tau[a,b,m,n] oovv[m,n,e,f]
    KV_TRY(ADD(-1.0, TT(w.Wabefb, "abef", s_w4v), 0.0, w.xW4, "abef", s_x4));
    KV_TRY(ADD(1.0, TT(w.Wabefb, "baef", s_w4v), 1.0, w.xW4, "abef", s_x4));
    KV_TRY(E(1.0, TT(w.xW4, "abef", s_x4), IB(vovv, "amef"), 1.0, g1, "bm", vo));
    if (Fg) {
        KV_TRY(GA(1.0, TT(w.Wabefb, "abef", s_w4v), Ig[0], "abef"));
        KV_TRY(GE(1.0, TT(w.xW4, "abef", s_x4), TT(t1, "bm", vo), Ig[2], "amef"));
        KV_TRY(GE(0.25, TT(w.Wabefb, "abef", s_w4v), TT(w.tau, "abmn", s_tau), Ig[5], "mnef"));
    }
    KV_TRY(E(0.25, TT(w.Wabefb, "abef", s_w4v), IB(oovv, "mnef"), 1.0, w.taub, "abmn", s_tau));
    // W_mnij: P(ij) t1[e,j] ooov[m,n,i,e] and 1/4 tau[e,f,i,j] oovv[m,n,e,f]
    KV_TRY(ADD(1.0, TT(w.Wmnijb, "mnij", s_w4o), 0.0, w.xW4, "mnij", s_x4));
    KV_TRY(ADD(-1.0, TT(w.Wmnijb, "mnji", s_w4o), 1.0, w.xW4, "mnij", s_x4));
    KV_TRY(E(1.0, TT(w.xW4, "mnij", s_x4), IB(ooov, "mnie"), 1.0, g1, "ej", vo));
    if (Fg) {
        KV_TRY(GA(1.0, TT(w.Wmnijb, "mnij", s_w4o), Ig[8], "mnij"));
        KV_TRY(GE(1.0, TT(w.xW4, "mnij", s_x4), TT(t1, "ej", vo), Ig[7], "mnie"));
        KV_TRY(GE(0.25, TT(w.Wmnijb, "mnij", s_w4o), TT(w.tau, "efij", s_tau), Ig[5], "mnef"));
    }
    KV_TRY(E(0.25, TT(w.Wmnijb, "mnij", s_w4o), IB(oovv, "mnef"), 1.0, w.taub, "efij", s_tau));
    // W_mbej
    KV_TRY(E(-1.0, TT(w.Wmbejb, "mbej", s_wmbej), IB(vovv, "bmef"), 1.0, g1, "fj", vo));
    KV_TRY(E(1.0, TT(w.Wmbejb, "mbej", s_wmbej), IB(ooov, "mnje"), 1.0, g1, "bn", vo));
    KV_TRY(E(-1.0, TT(w.Wmbejb, "mbej", s_wmbej), IB(oovv, "mnef"), 0.0, w.tmpb, "fbjn",
             s_tmp));
    if (Fg) {
        KV_TRY(GA(-1.0, TT(w.Wmbejb, "mbej", s_wmbej), Ig[4], "bmej"));
        KV_TRY(GE(-1.0, TT(w.Wmbejb, "mbej", s_wmbej), TT(t1, "fj", vo), Ig[2], "bmef"));
        KV_TRY(GE(1.0, TT(w.Wmbejb, "mbej", s_wmbej), TT(t1, "bn", vo), Ig[7], "mnje"));
        KV_TRY(GE(-1.0, TT(w.Wmbejb, "mbej", s_wmbej), TT(w.tmp, "fbjn", s_tmp), Ig[5], "mnef"));
    }
    KV_TRY(ADD(0.5, TT(w.tmpb, "fbjn", s_tmp), 1.0, w.t2b, "fbjn", s_tau));
    KV_TRY(E(1.0, TT(w.tmpb, "fbjn", s_tmp), TT(t1, "bn", vo), 1.0, g1, "fj", vo));
    KV_TRY(E(1.0, TT(w.tmpb, "fbjn", s_tmp), TT(t1, "fj", vo), 1.0, g1, "bn", vo));
    // F_me
    KV_TRY(E(1.0, TT(w.Fmeb, "me", s_ov), IB(oovv, "mnef"), 1.0, g1, "fn", vo));
    if (Fg) {
        KV_TRY(GA(1.0, TT(w.Fmeb, "me", s_ov), Fg[1], "me"));
        KV_TRY(GE(1.0, TT(w.Fmeb, "me", s_ov), TT(t1, "fn", vo), Ig[5], "mnef"));
    }
    // F_mi
    KV_TRY(E(0.5, TT(w.Fmib, "mi", s_oo), IB(Fov, "me"), 1.0, g1, "ei", vo));
    KV_TRY(E(1.0, TT(w.Fmib, "mi", s_oo), IB(ooov, "mnie"), 1.0, g1, "en", vo));
    KV_TRY(E(0.5, TT(w.Fmib, "mi", s_oo), IB(oovv, "mnef"), 0.0, w.ttaub, "efin", s_tau));
    if (Fg) {
        KV_TRY(GA(1.0, TT(w.Fmib, "mi", s_oo), Fg[0], "mi"));
        KV_TRY(GE(0.5, TT(w.Fmib, "mi", s_oo), TT(t1, "ei", vo), Fg[1], "me"));
        KV_TRY(GE(1.0, TT(w.Fmib, "mi", s_oo), TT(t1, "en", vo), Ig[7], "mnie"));
        KV_TRY(GE(0.5, TT(w.Fmib, "mi", s_oo), TT(w.ttau, "efin", s_tau), Ig[5], "mnef"));
    }
    // F_ae
    KV_TRY(E(-0.5, TT(w.Faeb, "ae", s_vv), IB(Fov, "me"), 1.0, g1, "am", vo));
    KV_TRY(E(-1.0, TT(w.Faeb, "ae", s_vv), IB(vovv, "amfe"), 1.0, g1, "fm", vo));
    KV_TRY(E(-0.5, TT(w.Faeb, "ae", s_vv), IB(oovv, "mnef"), 1.0, w.ttaub, "afmn", s_tau));
    if (Fg) {
        KV_TRY(GA(1.0, TT(w.Faeb, "ae", s_vv), Fg[3], "ae"));
        KV_TRY(GE(-0.5, TT(w.Faeb, "ae", s_vv), TT(t1, "am", vo), Fg[1], "me"));
        KV_TRY(GE(-1.0, TT(w.Faeb, "ae", s_vv), TT(t1, "fm", vo), Ig[2], "amfe"));
        KV_TRY(GE(-0.5, TT(w.Faeb, "ae", s_vv), TT(w.ttau, "afmn", s_tau), Ig[5], "mnef"));
    }
    // tau and tau-tilde
    KV_TRY(ADD(1.0, TT(w.taub, "abij", s_tau), 1.0, w.t2b, "abij", s_tau));
    KV_TRY(ADD(1.0, TT(w.ttaub, "abij", s_tau), 1.0, w.t2b, "abij", s_tau));
    KV_TRY(ADD(1.0, TT(w.taub, "abij", s_tau), 0.0, w.ttb, "abij", s_tau));
    KV_TRY(ADD(-1.0, TT(w.taub, "baij", s_tau), 1.0, w.ttb, "abij", s_tau));
    KV_TRY(ADD(0.5, TT(w.ttaub, "abij", s_tau), 1.0, w.ttb, "abij", s_tau));
    KV_TRY(ADD(-0.5, TT(w.ttaub, "baij", s_tau), 1.0, w.ttb, "abij", s_tau));
    KV_TRY(E(1.0, TT(w.ttb, "abij", s_tau), TT(t1, "bj", vo), 1.0, g1, "ai", vo));
    KV_TRY(E(1.0, TT(w.ttb, "abij", s_tau), TT(t1, "ai", vo), 1.0, g1, "bj", vo));
    // g2 = (1 - P(ab))(1 - P(ij)) t2b
    KV_TRY(ADD(1.0, TT(w.t2b, "abij", s_tau), 0.0, g2, "abij", v2o2));
    KV_TRY(ADD(-1.0, TT(w.t2b, "baij", s_tau), 1.0, g2, "abij", v2o2));
    KV_TRY(ADD(-1.0, TT(w.t2b, "abji", s_tau), 1.0, g2, "abij", v2o2));
    KV_TRY(ADD(1.0, TT(w.t2b, "baji", s_tau), 1.0, g2, "abij", v2o2));
    return KVFT_OK;
}

extern "C" int kvft_lambda_residual(kvft_ctx *ctx, int nb, int nv, int no,
                                    const double *const F[4], const double *const I[9],
                                    const double *t1, const double *t2, const double *m1,
                                    const double *m2, double *g1, double *g2) {
    if (!ctx || nb < 0 || nv <= 0 || no <= 0 || !F || !I || !t1 || !t2 || !m1 || !m2 || !g1 ||
        !g2)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_residual: bad argument");
    for (int k = 0; k < 4; k++)
        if (!F[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_residual: null F block");
    for (int k = 0; k < 9; k++)
        if (!I[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_residual: null I block");
    if (!ctx->dry) cudaSetDevice(ctx->device);
    return kv_lambda_vjp(ctx, nb, nv, no, F, I, t1, t2, m1, m2, g1, g2);
}

namespace {

int to_host(kvft_ctx *ctx, double *dst, const double *src, size_t n) {
    if (ctx->dry) {
        std::memcpy(dst, src, sizeof(double) * n);
        return KVFT_OK;
    }
    KV_CHECK(ctx, cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return KVFT_OK;
}

int to_device(kvft_ctx *ctx, double *dst, const double *src, size_t n) {
    if (ctx->dry) {
        std::memcpy(dst, src, sizeof(double) * n);
        return KVFT_OK;
    }
    KV_CHECK(ctx, cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice,
                                  ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return KVFT_OK;
}

// Lint = int_L(L) (quadrature.py:320-345): the tau integral run backwards,
// Lint[s] = sum_{y>=s} Gf[s,y] exp((t_y - t_s) d') L[y] with
// Gf[s,y] = g_y G[y,s] / g_s and d' the Lambda layout's denominator
// (e_i + e_j - e_a - e_b): the full-exponential forward integral with the
// roles of the orbital energies swapped.  Lint lives in scratch; hg (if not
// null) receives the host copy of g.
int lambda_int(kvft_ctx *ctx, int ng, int nv, int no, const double *L1, const double *L2,
               const double *ev, const double *eo, const double *ti, const double *g,
               const double *G, double **Lint1, double **Lint2, std::vector<double> *hgout) {
    const long long v = nv, o = no, vo = v * o, v2o2 = v * v * o * o;
    std::vector<double> hti(ng), hg(ng), hG((size_t)ng * ng), hGf((size_t)ng * ng, 0.0);
    KV_TRY(to_host(ctx, hti.data(), ti, ng));
    KV_TRY(to_host(ctx, hg.data(), g, ng));
    KV_TRY(to_host(ctx, hG.data(), G, (size_t)ng * ng));
    for (int s = 0; s < ng; s++)
        for (int y = s; y < ng; y++) hGf[(size_t)s * ng + y] = hg[y] * hG[(size_t)y * ng + s] / hg[s];
    void *gp = nullptr, *ip = nullptr;
    KV_TRY(kv_scratch(ctx, "lambda_grid", sizeof(double) * ng * ng, &gp));
    KV_TRY(to_device(ctx, (double *)gp, hGf.data(), (size_t)ng * ng));
    KV_TRY(kv_scratch(ctx, "lambda_int", sizeof(double) * ng * (vo + v2o2), &ip));
    *Lint1 = (double *)ip;
    *Lint2 = *Lint1 + ng * vo;
    const double *Gf = (const double *)gp;
    // Lambda layout [i][a] / [i][j][a][b]: occupied energies lead
    KV_TRY(kv_quad_launch(ctx, 0, ng, vo, 1, no, nv, L1, ti, hti.data(), Gf, hGf.data(),
                          nullptr, eo, ev, 1, 0.0, *Lint1, nullptr));
    KV_TRY(kv_quad_launch(ctx, 0, ng, v2o2, 2, no, nv, L2, ti, hti.data(), Gf, hGf.data(),
                          nullptr, eo, ev, 1, 0.0, *Lint2, nullptr));
    if (hgout) *hgout = hg;
    return KVFT_OK;
}

}  // namespace

// One Lambda update (kelvin/ft_cc_equations.py:385-409):
//   Lint = int_L(L_old)                      (quadrature.py:320-345)
//   L[y] = -(F.ov + I.oovv T1[y]) - R'(T[y])^T Lint[y],   L2[y] = -I.oovv - ...
// int_L is the tau integral run backwards: Lint[s] = sum_{y>=s} Gf[s,y]
// exp((t_y - t_s) d') L_old[y] with Gf[s,y] = g_y G[y,s] / g_s and d' the
// denominator of the Lambda layout (e_i + e_j - e_a - e_b), i.e. the full-
// exponential form of the forward integral with the roles of the orbital
// energies swapped.  L1/L2 may alias L1old/L2old.
extern "C" int kvft_ccsd_lambda(kvft_ctx *ctx, int ng, int nv, int no,
                                const double *const F[4], const double *const I[9],
                                const double *T1, const double *T2, const double *L1old,
                                const double *L2old, const double *ev, const double *eo,
                                const double *ti, const double *g, const double *G, double *L1,
                                double *L2) {
    if (!ctx || ng < 1 || ng > 64 || nv <= 0 || no <= 0 || !F || !I || !T1 || !T2 || !L1old ||
        !L2old || !ev || !eo || !ti || !g || !G || !L1 || !L2)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_ccsd_lambda: bad argument (ng must be 1..64)");
    for (int k = 0; k < 4; k++)
        if (!F[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_ccsd_lambda: null F block");
    for (int k = 0; k < 9; k++)
        if (!I[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_ccsd_lambda: null I block");
    if (!ctx->dry) cudaSetDevice(ctx->device);
    const long long v = nv, o = no, vo = v * o, v2o2 = v * v * o * o;
    double *Lint1 = nullptr, *Lint2 = nullptr;
    KV_TRY(lambda_int(ctx, ng, nv, no, L1old, L2old, ev, eo, ti, g, G, &Lint1, &Lint2, nullptr));
    // tau points per pass: the reverse pass keeps ~21 n^4 doubles per point
    int nb = ng;
    if (!ctx->dry) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) {
            const double per = (double)kv_lambda_workspace(1, nv, no) + 8.0 * (vo + v2o2);
            nb = (int)std::max(1.0, std::min((double)ng, 0.7 * (double)fr / per));
        }
    }
    void *gb = nullptr;
    KV_TRY(kv_scratch(ctx, "lambda_g", sizeof(double) * nb * (vo + v2o2), &gb));
    double *g1 = (double *)gb, *g2 = g1 + nb * vo;
    const double *Fov = F[1], *oovv = I[5];
    for (int y0 = 0; y0 < ng; y0 += nb) {
        const int b = std::min(nb, ng - y0);
        KV_TRY(kv_lambda_vjp(ctx, b, nv, no, F, I, T1 + y0 * vo, T2 + y0 * v2o2, Lint1 + y0 * vo,
                             Lint2 + y0 * v2o2, g1, g2));
        double *l1 = L1 + y0 * vo, *l2 = L2 + y0 * v2o2;
        KV_TRY(kv_add(ctx, nv, no, b, -1.0, KvTen{Fov, "ia", 0, 1}, 0.0, l1, "ia", vo));
        KV_TRY(kv_einsum(ctx, nv, no, b, -1.0, KvTen{oovv, "ijab", 0, 1},
                         KvTen{T1 + y0 * vo, "bj", vo, 0}, 1.0, l1, "ia", vo));
        KV_TRY(kv_add(ctx, nv, no, b, -1.0, KvTen{g1, "ai", vo, 0}, 1.0, l1, "ia", vo));
        KV_TRY(kv_add(ctx, nv, no, b, -1.0, KvTen{oovv, "ijab", 0, 1}, 0.0, l2, "ijab", v2o2));
        KV_TRY(kv_add(ctx, nv, no, b, -1.0, KvTen{g2, "abij", v2o2, 0}, 1.0, l2, "ijab", v2o2));
    }
    return KVFT_OK;
}

// The integral gradients of the Lagrangian (kelvin/ft_cc_equations.py:704-753
// assembles Kelvin's response densities from the same quantities):
//   Fg[b], Ig[b] = sum_y g_y d/d(block) [E(T_y) + <Lint_y, F.vo + I.vvoo + R(T_y)>]
// in the blocks' own layouts (F: oo ov vo vv, I: Kelvin's nine), Lint =
// int_L(L).  One tau point per reverse pass.
extern "C" int kvft_lambda_densities(kvft_ctx *ctx, int ng, int nv, int no,
                                     const double *const F[4], const double *const I[9],
                                     const double *T1, const double *T2, const double *L1,
                                     const double *L2, const double *ev, const double *eo,
                                     const double *ti, const double *g, const double *G,
                                     double *const Fg[4], double *const Ig[9]) {
    if (!ctx || ng < 1 || ng > 64 || nv <= 0 || no <= 0 || !F || !I || !T1 || !T2 || !L1 ||
        !L2 || !ev || !eo || !ti || !g || !G || !Fg || !Ig)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_densities: bad argument");
    for (int k = 0; k < 4; k++)
        if (!F[k] || !Fg[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_densities: null F");
    for (int k = 0; k < 9; k++)
        if (!I[k] || !Ig[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_densities: null I");
    if (!ctx->dry) cudaSetDevice(ctx->device);
    const long long v = nv, o = no, vo = v * o, v2o2 = v * v * o * o;
    double *Lint1 = nullptr, *Lint2 = nullptr;
    std::vector<double> hg;
    KV_TRY(lambda_int(ctx, ng, nv, no, L1, L2, ev, eo, ti, g, G, &Lint1, &Lint2, &hg));
    // zero the outputs
    const long long fsz[4] = {o * o, o * v, v * o, v * v};
    const long long isz[9] = {v * v * v * v, v * v * v * o, v * o * v * v, v2o2, v2o2, v2o2,
                              v * o * o * o, o * o * o * v, o * o * o * o};
    for (int k = 0; k < 13; k++) {
        const long long n = k < 4 ? fsz[k] : isz[k - 4];
        KOut c{k < 4 ? Fg[k] : Ig[k - 4], kidx1((int)n, 1), kidx1(1, 0), 0};
        KV_TRY(kv_scale_view(ctx, (int)n, 1, 1, 0.0, c));
    }
    void *gb = nullptr;
    KV_TRY(kv_scratch(ctx, "lambda_g", sizeof(double) * (vo + v2o2), &gb));
    double *g1 = (double *)gb, *g2 = g1 + vo;
    for (int y = 0; y < ng; y++) {
        const double w = hg[y];
        const double *t1 = T1 + y * vo, *t2 = T2 + y * v2o2;
        const double *l1 = Lint1 + y * vo, *l2 = Lint2 + y * v2o2;
        KV_TRY(kv_lambda_vjp(ctx, 1, nv, no, F, I, t1, t2, l1, l2, g1, g2, Fg, Ig, w));
        // the energy's own integrals (ft_cc_energy.py:7-32)
        KV_TRY(kv_add(ctx, nv, no, 1, w, KvTen{t1, "ai", 0, 0}, 1.0, Fg[1], "ia", 0));
        KV_TRY(kv_add(ctx, nv, no, 1, 0.25 * w, KvTen{t2, "abij", 0, 0}, 1.0, Ig[5], "ijab", 0));
        KV_TRY(kv_einsum(ctx, nv, no, 1, 0.5 * w, KvTen{t1, "ai", 0, 0}, KvTen{t1, "bj", 0, 0},
                         1.0, Ig[5], "ijab", 0));
        // the driving terms F.vo and I.vvoo meet Lint itself
        KV_TRY(kv_add(ctx, nv, no, 1, w, KvTen{l1, "ia", 0, 0}, 1.0, Fg[2], "ai", 0));
        KV_TRY(kv_add(ctx, nv, no, 1, 0.25 * w, KvTen{l2, "ijab", 0, 0}, 1.0, Ig[3], "abij", 0));
    }
    return KVFT_OK;
}

// Kelvin's damped Lambda iteration (kelvin/cc_utils.py:414-480) with every
// array resident: per iteration one Lambda update (kvft_ccsd_lambda), the
// norms of the change and of the damped Lambda on the device, and a read-back
// of a few doubles.  res = |L - L_old| / (|L_old| + 0.1) summed over L1, L2,
// or over the spin cases (alpha half h = spin_half first, the unrestricted
// driver's measure, cc_utils.py:482-560).  L1/L2 hold the guess on entry and
// the result on return; hist (may be null) receives res per iteration.  A
// dry-run context runs all max_iter iterations.
extern "C" int kvft_lambda_solve(kvft_ctx *ctx, int ng, int nv, int no,
                                 const double *const F[4], const double *const I[9],
                                 const double *T1, const double *T2, const double *ev,
                                 const double *eo, const double *ti, const double *g,
                                 const double *G, double damp, double tconv, int max_iter,
                                 int spin_half, double *L1, double *L2, double *hist,
                                 int *iters) {
    if (!ctx || ng < 1 || nv <= 0 || no <= 0 || !L1 || !L2 || max_iter < 0 || !iters ||
        (spin_half > 0 && (nv != no || nv != 2 * spin_half)))
        return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_solve: bad argument");
    const long long v = nv, o = no, vo = v * o, v2o2 = v * v * o * o;
    void *np = nullptr, *wp = nullptr;
    KV_TRY(kv_scratch(ctx, "lambda_new", sizeof(double) * ng * (vo + v2o2), &np));
    KV_TRY(kv_scratch(ctx, "lambda_norm", sizeof(double) * 32, &wp));
    double *N1 = (double *)np, *N2 = N1 + ng * vo, *nw = (double *)wp;
    // the blocks the measure runs over: (rank, element offset, dims, strides)
    struct Blk {
        int rank;
        long long off;
        int d[4];
        long long st[4];
    };
    std::vector<Blk> blks;
    const int h = spin_half;
    if (h > 0) {
        const long long n = nv, n2 = n * n, n3 = n2 * n;
        blks.push_back({1, 0, {1, 1, h, h}, {0, 0, n, 1}});
        blks.push_back({1, h * n + h, {1, 1, h, h}, {0, 0, n, 1}});
        blks.push_back({2, 0, {h, h, h, h}, {n3, n2, n, 1}});
        blks.push_back({2, h * n2 + h, {h, h, h, h}, {n3, n2, n, 1}});
        blks.push_back({2, h * (n3 + n2 + n + 1), {h, h, h, h}, {n3, n2, n, 1}});
    } else {
        blks.push_back({1, 0, {1, 1, no, nv}, {0, 0, nv, 1}});
        blks.push_back({2, 0, {no, no, nv, nv}, {o * v * v, v * v, v, 1}});
    }
    const int nb = (int)blks.size();
    // norms of a + b * x over the blocks into nw[base + k]
    auto norms = [&](const double *x1, const double *x2, double b, const double *y1,
                     const double *y2, int base) -> int {
        for (int k = 0; k < nb; k++) {
            const Blk &q = blks[k];
            const double *x = (q.rank == 1 ? x1 : x2) + q.off;
            const double *y = y1 ? (q.rank == 1 ? y1 : y2) + q.off : nullptr;
            const long long bst = q.rank == 1 ? vo : v2o2;
            KV_TRY(kv_sumsq4(ctx, ng, q.d, 1.0, x, q.st, bst, b, y, q.st, bst, nw + base + k));
        }
        return KVFT_OK;
    };
    double hw[32];
    auto read = [&](int count) -> int {
        if (ctx->dry) {
            std::memcpy(hw, nw, sizeof(double) * count);
            return KVFT_OK;
        }
        KV_CHECK(ctx, cudaMemcpyAsync(hw, nw, sizeof(double) * count, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
        return KVFT_OK;
    };
    // Kelvin's normalisers: singles and doubles, the ab case weighted 4
    auto normalisers = [&](const double *w, double *n1, double *n2) {
        *n1 = 0.1;
        *n2 = 0.1;
        for (int k = 0; k < nb; k++) {
            const double r = std::sqrt(w[k]);
            if (blks[k].rank == 1) *n1 += r;
            else *n2 += (h > 0 && k == 3) ? 4.0 * r : r;
        }
    };
    KV_TRY(norms(L1, L2, 0.0, nullptr, nullptr, 0));
    KV_TRY(read(nb));
    double nl1, nl2;
    normalisers(hw, &nl1, &nl2);
    int it = 0;
    for (; it < max_iter; it++) {
        KV_TRY(kvft_ccsd_lambda(ctx, ng, nv, no, F, I, T1, T2, L1, L2, ev, eo, ti, g, G, N1, N2));
        KV_TRY(norms(N1, N2, -1.0, L1, L2, 0));               // |L - L_old|
        KV_TRY(kv_add(ctx, nv, no, ng, 1.0 - damp, KvTen{N1, "ia", vo, 0}, damp, L1, "ia", vo));
        KV_TRY(kv_add(ctx, nv, no, ng, 1.0 - damp, KvTen{N2, "ijab", v2o2, 0}, damp, L2, "ijab",
                      v2o2));
        KV_TRY(norms(L1, L2, 0.0, nullptr, nullptr, nb));      // |L_old| after damping
        KV_TRY(read(2 * nb));
        double res = 0.0;
        for (int k = 0; k < nb; k++)
            res += std::sqrt(hw[k]) / (blks[k].rank == 1 ? nl1 : nl2);
        normalisers(hw + nb, &nl1, &nl2);
        if (hist) hist[it] = res;
        if (!ctx->dry && !std::isfinite(res)) {
            *iters = it + 1;
            return kv_fail(ctx, KVFT_EDIVERGE, "lambda iteration: non-finite residual");
        }
        if (!ctx->dry && res < tconv) {
            it++;
            break;
        }
    }
    *iters = it;
    // a tensor-core wait that expired during the iteration
    return ctx->dry ? KVFT_OK : kv_device_status(ctx);
}

// Kelvin's starting Lambda (ft_cc_equations.py:502-512; unrestricted:
// 515-526, whose I.oovv T1 term has no 1/beta): L1 = F.ov / beta +
// c I.oovv T1, L2 = I.oovv / beta at every tau point, c = 1/beta or 1.
extern "C" int kvft_lambda_guess(kvft_ctx *ctx, int ng, int nv, int no,
                                 const double *const F[4], const double *const I[9],
                                 const double *T1, double beta, int unrestricted, double *L1,
                                 double *L2) {
    if (!ctx || ng < 1 || nv <= 0 || no <= 0 || !F || !I || !F[1] || !I[5] || !T1 || !L1 ||
        !L2 || !(beta > 0.0))
        return kv_fail(ctx, KVFT_EINVAL, "kvft_lambda_guess: bad argument");
    if (!ctx->dry) cudaSetDevice(ctx->device);
    const long long vo = (long long)nv * no, v2o2 = vo * vo;
    const double c = unrestricted ? 1.0 : 1.0 / beta;
    KV_TRY(kv_add(ctx, nv, no, ng, 1.0 / beta, KvTen{F[1], "ia", 0, 1}, 0.0, L1, "ia", vo));
    KV_TRY(kv_einsum(ctx, nv, no, ng, c, KvTen{I[5], "ijab", 0, 1}, KvTen{T1, "bj", vo, 0}, 1.0,
                     L1, "ia", vo));
    return kv_add(ctx, nv, no, ng, 1.0 / beta, KvTen{I[5], "ijab", 0, 1}, 0.0, L2, "ijab", v2o2);
}

extern "C" int kvft_set_lambda_spin_blocks(kvft_ctx *ctx, int half) {
    if (!ctx || half < 0) return kv_fail(ctx, KVFT_EINVAL, "lambda spin blocks: bad argument");
    ctx->lam_spin = half;
    return KVFT_OK;
}

extern "C" int kvft_einsum_plan(int nv, int no, const char *aix, const char *bix,
                                const char *cix, int *mnk, int *sizes, long long *strides) {
    if (!aix || !bix || !cix || !mnk || !sizes || !strides) return KVFT_EINVAL;
    KIdx x[6];
    std::string err;
    int st = kv_einsum_desc(nv, no, aix, bix, cix, &mnk[0], &mnk[1], &mnk[2], &x[0], &x[1],
                            &x[2], &x[3], &x[4], &x[5], &err);
    if (st != KVFT_OK) return st;
    for (int k = 0; k < 6; k++)
        for (int d = 0; d < 3; d++) {
            sizes[3 * k + d] = x[k].size[d];
            strides[3 * k + d] = x[k].st[d];
        }
    return KVFT_OK;
}
