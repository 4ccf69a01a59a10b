// The spin-orbital CCSD residual with Stanton-Gauss intermediates, evaluated
// for a batch of tau points on the device (the arithmetic Kelvin delegates to
// cqcpy.cc_equations._Stanton at kelvin/ft_cc_equations.py:105-107).
//
// Every contraction is one strided GEMM (kv_gemm) whose operands are permuted
// views of the amplitude / integral tensors; tau-independent integrals are
// shared across the batch (batch stride 0) and, where the other operand is per
// tau point, the tau index is folded into the GEMM's N dimension so that one
// launch covers the whole batch.  The n^6 work per tau point is
//   X      = <mn||ef> tau_ef^ij                        (folded over tau)
//   T2    += 1/2 tau_ab^mn W'_mnij, W' = W_mnij + X/4   (the W_abef tau-tau
//            term is carried by X, saving the explicit 1/4 tau <mn||ef> GEMM)
//   T2    += 1/2 W'_abef tau_ef^ij, W'_abef = <ab||ef> - P(ab) t_m^b <am||ef>
//   W_mbej -= <mn||ef> (t_jn^fb / 2 + t_j^f t_n^b)     (folded over tau)
//   Z      = t_im^ae W_mbej, then T2 += P(ij)P(ab) Z (with the n^5 Zab and
//            Zij terms folded into the same array, see the assembly)
// where the first three run over antisymmetric index pairs p < q only
// (n^6/4 flops each instead of 2 n^6), so 4.75 n^6 flops per tau point remain
// besides about thirty n^5 terms.
#include "kvft_internal.h"

namespace {

struct Sizes {
    long long v, o;
    long long vo, oo, vv, v2o2, o4, v4, vo3;
};

inline KIdx X1(int s, long long t) { return kidx1(s, t); }
inline KIdx X2(int s0, long long t0, int s1, long long t1) { return kidx2(s0, t0, s1, t1); }
inline KIdx X3(int s0, long long t0, int s1, long long t1, int s2, long long t2) {
    return kidx3(s0, t0, s1, t1, s2, t2);
}
inline KMat MA(const double *p, KIdx r, KIdx c, long long bst) { return KMat{p, r, c, bst}; }
// an integral block: shared by the batch and fixed for the solver's lifetime
inline KMat MAI(const double *p, KIdx r, KIdx c) { return KMat{p, r, c, 0, 1}; }
inline KOut MO(double *p, KIdx r, KIdx c, long long bst) { return KOut{p, r, c, bst}; }

// ---- spin-blocked contractions ----------------------------------------------
// With spin blocks (ctx->spin_half = h > 0, nv = no = 2h) every orbital index
// splits into an alpha half [0, h) and a beta half [h, 2h), and the integrals
// and amplitudes vanish outside spin-conserving blocks (x_pqrs = 0 unless
// s_p + s_q = s_r + s_s).  An n^6 contraction over six orbital indices then
// has only 10 of its 64 spin-block products nonzero; each runs as a strided
// GEMM on sub-views (halved index extents, offset pointers).

// A view slot of an orbital index: operand (0 A, 1 B, 2 C), dimension (0
// rows, 1 columns) and component of that composite index.
struct Slot {
    int op, dim, comp;
};

void halve(KIdx &x, int comp, int h, int s, long long &off) {
    x.size[comp] = h;
    off += (long long)s * h * x.st[comp];
}

// C = alpha A B + beta C over the block products that keep(spins) allows
// (bit x of spins = spin of orbital index x, whose slots are idx[x]).  C
// blocks that no product writes are scaled by beta (zeroed when C is the
// whole contiguous buffer of `cwords` doubles and beta = 0), or left alone
// with cwords = -1 (an intermediate whose readers skip those blocks too).
template <class Keep>
int spin_gemm(kvft_ctx *ctx, int h, int batch, double alpha, const KMat &A, const KMat &B,
              double beta, const KOut &C, const std::vector<std::vector<Slot>> &idx, Keep keep,
              long long cwords = 0) {
    const int nx = (int)idx.size();
    unsigned cmask = 0;
    for (int x = 0; x < nx; x++)
        for (const Slot &s : idx[x])
            if (s.op == 2) cmask |= 1u << x;
    for (int x = 0; x < nx; x++)
        for (const Slot &s : idx[x]) {
            const KIdx &v = s.op == 0 ? (s.dim ? A.c : A.r)
                                      : s.op == 1 ? (s.dim ? B.c : B.r) : (s.dim ? C.c : C.r);
            if (v.size[s.comp] != 2 * h)
                return kv_fail(ctx, KVFT_EINVAL, "spin blocks: index extent is not 2h");
        }
    // products that share an operand sub-block share its digit planes
    KvTPackScope tpack(ctx);
    bool zeroed = false;
    if (beta == 0.0 && cwords > 0) {
        KV_CHECK(ctx, cudaMemsetAsync(C.p, 0, sizeof(double) * cwords, ctx->stream));
        zeroed = true;
    }
    std::vector<char> written(1u << nx, 0);
    for (unsigned m = 0; m < (1u << nx); m++) {
        if (!keep(m)) continue;
        KMat a = A, b = B;
        KOut c = C;
        long long oa = 0, ob = 0, oc = 0;
        for (int x = 0; x < nx; x++) {
            const int sp = (m >> x) & 1;
            for (const Slot &s : idx[x]) {
                if (s.op == 0) halve(s.dim ? a.c : a.r, s.comp, h, sp, oa);
                else if (s.op == 1) halve(s.dim ? b.c : b.r, s.comp, h, sp, ob);
                else halve(s.dim ? c.c : c.r, s.comp, h, sp, oc);
            }
        }
        a.p += oa;
        b.p += ob;
        c.p += oc;
        const unsigned key = m & cmask;
        const double be = written[key] ? 1.0 : beta;
        written[key] = 1;
        KV_TRY(kv_gemm(ctx, a.r.total(), b.c.total(), a.c.total(), batch, alpha, a, b, be, c));
    }
    if (beta == 1.0 || zeroed || cwords < 0) return KVFT_OK;
    for (unsigned m = 0; m < (1u << nx); m++) {
        if ((m & ~cmask) || written[m]) continue;
        KOut c = C;
        long long oc = 0;
        for (int x = 0; x < nx; x++)
            for (const Slot &s : idx[x])
                if (s.op == 2) halve(s.dim ? c.c : c.r, s.comp, h, (m >> x) & 1, oc);
        c.p += oc;
        KV_TRY(kv_scale_view(ctx, c.r.total(), c.c.total(), batch, beta, c));
    }
    return KVFT_OK;
}

inline int sp(unsigned m, int x) { return (m >> x) & 1; }

// workspace layout (per tau point, doubles)
struct WS {
    double *tau, *ttau, *Fae, *Fmi, *Fme, *Xbe, *Xmj, *Wmnij, *Wabef, *Wmbej,
        *tmp4, *Q, *Z, *Lc;
};

size_t ws_per_tau(long long v, long long o) {
    long long v2o2 = v * v * o * o, o4 = o * o * o * o, v4 = v * v * v * v;
    long long big = std::max(std::max(v4, o4), v2o2);
    // tau_c ttau Wmbej Z Lc (v2o2 each) + W'_mnij_c (o4) + W'_abef_c (v4)
    // + tmp4 (max) + Q (v o^3) + five small matrices
    return (size_t)(5 * v2o2 + o4 + v4 + big + v * o * o * o + 2 * v * v + 3 * o * o + 2 * o * v);
}

WS carve(double *base, int nb, long long v, long long o) {
    WS w;
    long long v2o2 = v * v * o * o, o4 = o * o * o * o, v4 = v * v * v * v;
    long long big = std::max(std::max(v4, o4), v2o2);
    double *p = base;
    auto take = [&](long long per) { double *q = p; p += per * nb; return q; };
    w.tau = take(v2o2);
    w.ttau = take(v2o2);
    w.Wmbej = take(v2o2);
    w.Z = take(v2o2);
    w.Lc = take(v2o2);
    w.Wmnij = take(o4);
    w.Wabef = take(v4);
    w.tmp4 = take(big);
    w.Q = take(v * o * o * o);
    w.Fae = take(v * v);
    w.Xbe = take(v * v);
    w.Fmi = take(o * o);
    w.Xmj = take(o * o);
    w.Fme = take(o * v);
    (void)take(o * v);
    (void)take(o * o);
    return w;
}

}  // namespace

size_t kv_stanton_workspace(int nb, int nv, int no) {
    return ws_per_tau(nv, no) * (size_t)nb * sizeof(double);
}

// Device bytes one tau point of a Stanton call needs: the workspace and, on
// the tensor-core path, BF16 digit planes of two n^4-sized operands.
size_t kv_chunk_bytes_per_tau(kvft_ctx *ctx, int nv, int no) {
    size_t per = kv_stanton_workspace(1, nv, no);
    if (ctx->precision != KVFT_PREC_FP64) {
        const size_t big = std::max(std::max((size_t)nv * nv * nv * nv, (size_t)no * no * no * no),
                                    (size_t)nv * nv * no * no);
        const size_t S = (size_t)std::min(ctx->digits - 1, 6);
        per += 2 * S * 2 * big / 8 * 9;       // plane rows are padded to 64 k values
    }
    return per;
}

int kv_stanton(kvft_ctx *ctx, int nb, int nv, int no, const double *const F[4],
               const double *const I[9], const double *t1, const double *t2,
               double fac, double *T1, double *T2, const double *seed_t2) {
    if (nb <= 0) return KVFT_OK;
    const long long v = nv, o = no;
    const long long vo = v * o, oo = o * o, vv = v * v;
    const long long v2o2 = vv * oo, o4 = oo * oo, v4 = vv * vv, vo2 = v * oo;
    const long long vo3 = v * o * oo;
    // F.vo and I.vvoo enter only through the caller's seed of T1/T2
    const double *Foo = F[0], *Fov = F[1], *Fvv = F[3];
    const double *vvvv = I[0], *vvvo = I[1], *vovv = I[2], *vovo = I[4],
                 *oovv = I[5], *vooo = I[6], *ooov = I[7], *oooo = I[8];

    void *wsp = nullptr;
    KV_TRY(kv_scratch(ctx, "stanton", kv_stanton_workspace(nb, nv, no), &wsp));
    WS w = carve((double *)wsp, nb, v, o);
    const int B = nb;
    const KIdx one = X1(1, 0);
    // spin blocks (nv = no = 2h): contractions whose operands all live on the
    // spin-conserving blocks run as their nonzero spin-block products
    const int sh = (ctx->spin_half > 0 && nv == no && nv == 2 * ctx->spin_half) ? ctx->spin_half
                                                                               : 0;
    typedef std::vector<std::vector<Slot>> Slots;
    auto sgemm = [&](int M, int N, int K, int batch, double alpha, const KMat &A,
                     const KMat &Bm, double beta, const KOut &C, const Slots &idx, auto keep,
                     long long cwords) -> int {
        if (sh) return spin_gemm(ctx, sh, batch, alpha, A, Bm, beta, C, idx, keep, cwords);
        return kv_gemm(ctx, M, N, K, batch, alpha, A, Bm, beta, C);
    };

    // ---- tau-tilde (tau itself is only needed pair-compressed) --------------
    // tau-tilde feeds only F_ae and F_mi, whose contractions read its
    // spin-conserving blocks alone
    KV_TRY(kv_make_tau(ctx, B, nv, no, t1, t2, 0.5, w.ttau, sh));

    // ---- F_ae ------------------------------------------------------------
    KV_TRY(kv_bcast(ctx, B, vv, Fvv, w.Fae));
    // -1/2 t1[a,m] Fov[m,e]
    KV_TRY(kv_gemm(ctx, nv, nv, no, B, -0.5, MA(t1, X1(nv, o), X1(no, 1), vo),
                   MA(Fov, X1(no, v), X1(nv, 1), 0), 1.0,
                   MO(w.Fae, X1(nv, v), X1(nv, 1), vv)));
    // - vovv[a,m,f,e] t1[f,m]    (M=(a,e), K=(m,f), N=tau)
    KV_TRY(kv_gemm(ctx, nv * nv, B, no * nv, 1, -1.0,
                   MAI(vovv, X2(nv, o * vv, nv, 1), X2(no, vv, nv, v)),
                   MA(t1, X2(no, 1, nv, o), X1(B, vo), 0), 1.0,
                   MO(w.Fae, X2(nv, v, nv, 1), X1(B, vv), 0)));
    // -1/2 ttau[a,f,m,n] oovv[m,n,e,f]; spins a f m n e
    KV_TRY(sgemm(nv, nv, nv * no * no, B, -0.5,
                 MA(w.ttau, X1(nv, vo2), X3(nv, oo, no, o, no, 1), v2o2),
                 MAI(oovv, X3(nv, 1, no, o * vv, no, vv), X1(nv, v)), 1.0,
                 MO(w.Fae, X1(nv, v), X1(nv, 1), vv),
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 0}, {1, 0, 0}}, {{0, 1, 1}, {1, 0, 1}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) &&
                            sp(m, 2) + sp(m, 3) == sp(m, 4) + sp(m, 1);
                 }, 0));

    // ---- F_mi ------------------------------------------------------------
    KV_TRY(kv_bcast(ctx, B, oo, Foo, w.Fmi));
    // +1/2 Fov[m,e] t1[e,i]
    KV_TRY(kv_gemm(ctx, no, no, nv, B, 0.5, MA(Fov, X1(no, v), X1(nv, 1), 0),
                   MA(t1, X1(nv, o), X1(no, 1), vo), 1.0,
                   MO(w.Fmi, X1(no, o), X1(no, 1), oo)));
    // + ooov[m,n,i,e] t1[e,n]    (M=(m,i), K=(n,e), N=tau)
    KV_TRY(kv_gemm(ctx, no * no, B, no * nv, 1, 1.0,
                   MAI(ooov, X2(no, oo * v, no, v), X2(no, vo, nv, 1)),
                   MA(t1, X2(no, 1, nv, o), X1(B, vo), 0), 1.0,
                   MO(w.Fmi, X2(no, o, no, 1), X1(B, oo), 0)));
    // +1/2 oovv[m,n,e,f] ttau[e,f,i,n]; spins m n e f i
    KV_TRY(sgemm(no, no, no * nv * nv, B, 0.5,
                 MAI(oovv, X1(no, o * vv), X3(no, vv, nv, v, nv, 1)),
                 MA(w.ttau, X3(no, 1, nv, vo2, nv, oo), X1(no, o), v2o2), 1.0,
                 MO(w.Fmi, X1(no, o), X1(no, 1), oo),
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 0}, {1, 0, 0}}, {{0, 1, 1}, {1, 0, 1}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) &&
                            sp(m, 2) + sp(m, 3) == sp(m, 4) + sp(m, 1);
                 }, 0));

    // ---- F_me ------------------------------------------------------------
    KV_TRY(kv_bcast(ctx, B, vo, Fov, w.Fme));
    // + oovv[m,n,e,f] t1[f,n]    (M=(m,e), K=(n,f), N=tau)
    KV_TRY(kv_gemm(ctx, no * nv, B, no * nv, 1, 1.0,
                   MAI(oovv, X2(no, o * vv, nv, v), X2(no, vv, nv, 1)),
                   MA(t1, X2(no, 1, nv, o), X1(B, vo), 0), 1.0,
                   MO(w.Fme, X2(no, v, nv, 1), X1(B, vo), 0)));

    // ---- R1 ----------------------------------------------------------------
    const KOut T1o = MO(T1, X1(nv, o), X1(no, 1), vo);
    KV_TRY(kv_gemm(ctx, nv, no, nv, B, fac, MA(w.Fae, X1(nv, v), X1(nv, 1), vv),
                   MA(t1, X1(nv, o), X1(no, 1), vo), 1.0, T1o));
    KV_TRY(kv_gemm(ctx, nv, no, no, B, -fac, MA(t1, X1(nv, o), X1(no, 1), vo),
                   MA(w.Fmi, X1(no, o), X1(no, 1), oo), 1.0, T1o));
    // t2[a,e,i,m] Fme[m,e]   (M=(a,i), K=(m,e), N=1); spins a i m e
    KV_TRY(sgemm(nv * no, 1, no * nv, B, fac,
                 MA(t2, X2(nv, vo2, no, o), X2(no, 1, nv, oo), v2o2),
                 MA(w.Fme, X2(no, v, nv, 1), one, vo), 1.0,
                 MO(T1, X2(nv, o, no, 1), one, vo),
                 Slots{{{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}}, {{0, 1, 1}, {1, 0, 1}},
                       {{0, 1, 2}, {1, 0, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 3) == sp(m, 1) + sp(m, 2) && sp(m, 2) == sp(m, 3);
                 }, 0));
    // - vovo[a,n,f,i] t1[f,n]   (M=(a,i), K=(n,f), N=tau)
    KV_TRY(kv_gemm(ctx, nv * no, B, no * nv, 1, -fac,
                   MAI(vovo, X2(nv, vo2, no, 1), X2(no, vo, nv, o)),
                   MA(t1, X2(no, 1, nv, o), X1(B, vo), 0), 1.0,
                   MO(T1, X2(nv, o, no, 1), X1(B, vo), 0)));
    // +1/2 vovv[a,m,e,f] t2[e,f,i,m]; spins a m e f i
    KV_TRY(sgemm(nv, no, no * nv * nv, B, 0.5 * fac,
                 MAI(vovv, X1(nv, o * vv), X3(no, vv, nv, v, nv, 1)),
                 MA(t2, X3(no, 1, nv, vo2, nv, oo), X1(no, o), v2o2), 1.0, T1o,
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 0}, {1, 0, 0}}, {{0, 1, 1}, {1, 0, 1}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) &&
                            sp(m, 2) + sp(m, 3) == sp(m, 4) + sp(m, 1);
                 }, 0));
    // +1/2 t2[a,e,m,n] ooov[n,m,i,e]; spins a e m n i
    KV_TRY(sgemm(nv, no, nv * no * no, B, 0.5 * fac,
                 MA(t2, X1(nv, vo2), X3(nv, oo, no, o, no, 1), v2o2),
                 MAI(ooov, X3(nv, 1, no, vo, no, oo * v), X1(no, v)), 1.0, T1o,
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 0}, {1, 0, 0}}, {{0, 1, 1}, {1, 0, 1}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) &&
                            sp(m, 3) + sp(m, 2) == sp(m, 4) + sp(m, 1);
                 }, 0));

    // ---- ladder terms over antisymmetric pairs ---------------------------------
    // tau, W'_mnij, W'_abef and <mn||ef> are antisymmetric in each index pair,
    // so the three ladder contractions run over p < q only (8x fewer flops):
    //   W'_c[mn,ij] = oooo + P(ij) ooov t1 + sum_{e<f} oovv[mn,ef] tau[ef,ij]
    //   Lc[ab,ij]   = sum_{m<n} tau[ab,mn] W'_c[mn,ij] + sum_{e<f} W'_c[ab,ef] tau[ef,ij]
    // (the 1/2 of each full-range sum cancels the factor 2 of the pair sum; the
    // X/4 of W_mnij plus the tau <mn||ef>/4 of W_abef make the X/2 in W'_mnij),
    // and T2 += fac Lc, expanded with signs, in the final assembly.
    const int pv = nv * (nv - 1) / 2, po = no * (no - 1) / 2;
    const long long pvo = (long long)pv * po, poo = (long long)po * po, pvv = (long long)pv * pv;
    const bool ladders = pv > 0 && po > 0;
    if (ladders) {
        // With spin blocks the pairs are in spin-sorted order and every pair
        // tensor links only pairs of one spin type (alpha-alpha, alpha-beta,
        // beta-beta), so each pair contraction runs as three block products
        // on the diagonal type blocks; the other blocks are neither written
        // nor read.  ntype = 1 with the whole range otherwise.
        const long long paa = (long long)sh * (sh - 1) / 2, hh = (long long)sh * sh;
        const int ntype = sh ? 3 : 1;
        // first index and count of the type-t pairs (virtual / occupied pairs;
        // the same ranges when spin-blocked, since then nv = no)
        auto rlo = [&](int t) -> long long { return sh ? (t == 0 ? 0 : t == 1 ? paa : paa + hh) : 0; };
        auto rnv = [&](int t) -> int { return sh ? (int)(t == 1 ? hh : paa) : pv; };
        auto rno = [&](int t) -> int { return sh ? (int)(t == 1 ? hh : paa) : po; };
        KV_TRY(kv_make_tau_pairs(ctx, B, nv, no, t1, t2, w.tau, sh));  // tau_c[y][ef][ij]
        void *oc = nullptr;
        KV_TRY(kv_scratch(ctx, "oovv_pairs", sizeof(double) * (size_t)po * pv, &oc));
        const long long sov[4] = {o * vv, vv, v, 1};
        KV_TRY(kv_pair_gather(ctx, 1, no, nv, oovv, sov, 1.0, nullptr, nullptr, 0.0, nullptr,
                              0.0, 0, (double *)oc, sh));
        // Z[m,n,i,j] = ooov[m,n,i,e] t1[e,j]; spins m n i e j (the gather below
        // reads its spin-conserving elements only)
        KV_TRY(sgemm(no * no * no, no, nv, B, 1.0,
                     MAI(ooov, X3(no, oo * v, no, vo, no, v), X1(nv, 1)),
                     MA(t1, X1(nv, o), X1(no, 1), vo), 0.0,
                     MO(w.tmp4, X3(no, o * oo, no, oo, no, o), X1(no, 1), o4),
                     Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                           {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                     [](unsigned m) {
                         return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) && sp(m, 3) == sp(m, 4);
                     }, -1));
        // W'_c = oooo + Z - Z^(ij)
        const long long s4o[4] = {o * oo, oo, o, 1}, s4t[4] = {o * oo, oo, 1, o};
        KV_TRY(kv_pair_gather(ctx, B, no, no, oooo, s4o, 1.0, w.tmp4, s4o, 1.0, s4t, -1.0, o4,
                              w.Wmnij, sh));
        for (int t = 0; t < ntype; t++) {
            const long long lo = rlo(t);          // lo applies to both pair kinds
            const int nvt = rnv(t), not_ = rno(t);
            // W'_c += oovv_c tau_c   (M = mn pairs, K = ef pairs, N = (tau, ij pairs))
            KV_TRY(kv_gemm(ctx, not_, B * not_, nvt, 1, 1.0,
                           MA((const double *)oc + lo * pv + lo, X1(not_, pv), X1(nvt, 1), 0),
                           MA(w.tau + lo * po + lo, X1(nvt, po), X2(B, pvo, not_, 1), 0), 1.0,
                           MO(w.Wmnij + lo * po + lo, X1(not_, po), X2(B, poo, not_, 1), 0)));
            // Lc = tau_c W'_c        (M = ab pairs, K = mn pairs, N = ij pairs)
            KV_TRY(kv_gemm(ctx, nvt, not_, not_, B, 1.0,
                           MA(w.tau + lo * po + lo, X1(nvt, po), X1(not_, 1), pvo),
                           MA(w.Wmnij + lo * po + lo, X1(not_, po), X1(not_, 1), poo), 0.0,
                           MO(w.Lc + lo * po + lo, X1(nvt, po), X1(not_, 1), pvo)));
        }
        // Y[a,b,e,f] = t1[b,m] vovv[a,m,e,f]   (M=b, K=m, N=(a,e,f)); spins b m a e f
        KV_TRY(sgemm(nv, nv * nv * nv, no, B, 1.0,
                     MA(t1, X1(nv, o), X1(no, 1), vo),
                     MAI(vovv, X1(no, vv), X3(nv, o * vv, nv, v, nv, 1)), 0.0,
                     MO(w.tmp4, X1(nv, vv), X3(nv, v * vv, nv, v, nv, 1), v4),
                     Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 0}, {2, 1, 0}},
                           {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}},
                     [](unsigned m) {
                         return sp(m, 0) == sp(m, 1) && sp(m, 2) + sp(m, 1) == sp(m, 3) + sp(m, 4);
                     }, -1));
        // W'_abef_c = vvvv - Y + Y^(ab)
        const long long s4v[4] = {v * vv, vv, v, 1}, s4s[4] = {vv, v * vv, v, 1};
        KV_TRY(kv_pair_gather(ctx, B, nv, nv, vvvv, s4v, 1.0, w.tmp4, s4v, -1.0, s4s, 1.0, v4,
                              w.Wabef, sh));
        // Lc += W'_abef_c tau_c   (M = ab pairs, K = ef pairs, N = ij pairs)
        for (int t = 0; t < ntype; t++) {
            const long long lo = rlo(t);
            const int nvt = rnv(t), not_ = rno(t);
            KV_TRY(kv_gemm(ctx, nvt, not_, nvt, B, 1.0,
                           MA(w.Wabef + lo * pv + lo, X1(nvt, pv), X1(nvt, 1), pvv),
                           MA(w.tau + lo * po + lo, X1(nvt, po), X1(not_, 1), pvo), 1.0,
                           MO(w.Lc + lo * po + lo, X1(nvt, po), X1(not_, 1), pvo)));
        }
    }

    // ---- W_mbej (layout [m][b][e][j]) ----------------------------------------
    const long long wm = vv * o, wb = vo, we = o;
    {
        int d[4] = {no, nv, nv, no};
        long long ss[4] = {vo, vo2, o, 1};          // vovo[b,m,e,j]
        long long ds[4] = {wm, wb, we, 1};
        if (sh) {
            // W_mbej is read only on its spin-conserving blocks (s_m + s_b =
            // s_e + s_j): six of the sixteen (m, b, e, j) spin blocks
            const int hd[4] = {sh, sh, sh, sh};
            for (int m = 0; m < 16; m++) {
                const int sm = m & 1, sb = (m >> 1) & 1, se = (m >> 2) & 1, sj = (m >> 3) & 1;
                if (sm + sb != se + sj) continue;
                const long long os = (long long)sh * (sm * ss[0] + sb * ss[1] + se * ss[2] + sj),
                                od = (long long)sh * (sm * ds[0] + sb * ds[1] + se * ds[2] + sj);
                KV_TRY(kv_axpby4(ctx, B, hd, -1.0, vovo + os, ss, 0, 0.0, w.Wmbej + od, ds,
                                 v2o2));
            }
        } else {
            KV_TRY(kv_axpby4(ctx, B, d, -1.0, vovo, ss, 0, 0.0, w.Wmbej, ds, v2o2));
        }
    }
    // - vovv[b,m,e,f] t1[f,j]    (M=(m,b,e), K=f, N=j); spins m b e f j
    KV_TRY(sgemm(no * nv * nv, no, nv, B, -1.0,
                 MAI(vovv, X3(no, vv, nv, o * vv, nv, v), X1(nv, 1)),
                 MA(t1, X1(nv, o), X1(no, 1), vo), 1.0,
                 MO(w.Wmbej, X3(no, wm, nv, wb, nv, we), X1(no, 1), v2o2),
                 Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 1) + sp(m, 0) == sp(m, 2) + sp(m, 3) && sp(m, 3) == sp(m, 4);
                 }, 0));
    // + t1[b,n] ooov[m,n,j,e]    (M=b, K=n, N=(m,e,j)); spins b n m e j
    KV_TRY(sgemm(nv, no * nv * no, no, B, 1.0,
                 MA(t1, X1(nv, o), X1(no, 1), vo),
                 MAI(ooov, X1(no, vo), X3(no, oo * v, nv, 1, no, v)), 1.0,
                 MO(w.Wmbej, X1(nv, wb), X3(no, wm, nv, we, no, 1), v2o2),
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 0}, {2, 1, 0}},
                       {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) == sp(m, 1) && sp(m, 2) + sp(m, 1) == sp(m, 4) + sp(m, 3);
                 }, 0));
    // - oovv[m,n,e,f] (t2[f,b,j,n]/2 + t1[f,j] t1[b,n])  (M=(m,e), K=(n,f), N=(tau,b,j))
    KV_TRY(kv_make_wmbej_tmp(ctx, B, nv, no, t1, t2, w.tmp4, sh));
    {
        // tmp4 holds [tau][b][j][n][f] with per-tau stride v2o2 (tmp4 is sized
        // for the largest block, so index it with the v2o2 layout directly);
        // the contraction index (n, f) is contiguous in both operands
        const KMat A = MAI(oovv, X2(no, o * vv, nv, v), X2(no, vv, nv, 1));
        const KMat Bm = MA(w.tmp4, X2(no, v, nv, 1), X3(B, v2o2, nv, vo2, no, vo), 0);
        const KOut C = MO(w.Wmbej, X2(no, wm, nv, we), X3(B, v2o2, nv, wb, no, 1), 0);
        if (sh) {
            // orbital indices m e n f b j; <mn||ef> and tmp[b,j,n,f] (t2[f,b,j,n])
            const std::vector<std::vector<Slot>> idx = {
                {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}}, {{0, 1, 1}, {1, 0, 1}},
                {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}};
            KV_TRY(spin_gemm(ctx, sh, 1, -1.0, A, Bm, 1.0, C, idx, [](unsigned m) {
                return sp(m, 0) + sp(m, 2) == sp(m, 1) + sp(m, 3) &&
                       sp(m, 3) + sp(m, 4) == sp(m, 5) + sp(m, 2);
            }));
        } else {
            KV_TRY(kv_gemm(ctx, no * nv, B * nv * no, no * nv, 1, -1.0, A, Bm, 1.0, C));
        }
    }
    // The three doubles terms share one array Z:
    //   T2 += P(ab) Zab + P(ij) Zij + P(ab)P(ij) Zabij
    //       = (1 - P(ab))(1 - P(ij)) (Zabij + Zab/2 + Zij/2)
    // because Zab is antisymmetric in (i,j) and Zij in (a,b) (as t2 and the
    // antisymmetrised integrals are), so the assembly reads one n^4 array.
    // Zabij[a,b,i,j] = t2[a,e,i,m] Wmbej[m,b,e,j]   (M=(a,i), K=(m,e), N=(b,j))
    {
        const KMat A = MA(t2, X2(nv, vo2, no, o), X2(no, 1, nv, oo), v2o2);
        const KMat Bm = MA(w.Wmbej, X2(no, wm, nv, we), X2(nv, wb, no, 1), v2o2);
        const KOut C = MO(w.Z, X2(nv, vo2, no, o), X2(nv, oo, no, 1), v2o2);
        if (sh) {
            // orbital indices a i m e b j; t2[a,e,i,m] and Wmbej[m,b,e,j]
            const std::vector<std::vector<Slot>> idx = {
                {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}}, {{0, 1, 1}, {1, 0, 1}},
                {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}};
            KV_TRY(spin_gemm(ctx, sh, B, 1.0, A, Bm, 0.0, C, idx, [](unsigned m) {
                return sp(m, 0) + sp(m, 3) == sp(m, 1) + sp(m, 2) &&
                       sp(m, 2) + sp(m, 4) == sp(m, 3) + sp(m, 5);
            }, (long long)B * v2o2));
        } else {
            KV_TRY(kv_gemm(ctx, nv * no, nv * no, no * nv, B, 1.0, A, Bm, 0.0, C));
        }
    }
    // Q[b,m,i,j] = vovo[b,m,e,j] t1[e,i]   (M=(b,m,j), K=e, N=i); spins b m j e i.
    // With spin blocks only Q's spin-conserving blocks are written, and they
    // are the only ones its reader below touches.
    KV_TRY(sgemm(nv * no * no, no, nv, B, 1.0,
                 MAI(vovo, X3(nv, vo2, no, vo, no, 1), X1(nv, o)),
                 MA(t1, X1(nv, o), X1(no, 1), vo), 0.0,
                 MO(w.Q, X3(nv, o * oo, no, oo, no, 1), X1(no, o), vo3),
                 Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 3) + sp(m, 2) && sp(m, 3) == sp(m, 4);
                 }, -1));
    // Zabij += t1[a,m] Q[b,m,i,j]   (M=a, K=m, N=(b,i,j)); spins a m b i j
    KV_TRY(sgemm(nv, nv * no * no, no, B, 1.0,
                 MA(t1, X1(nv, o), X1(no, 1), vo),
                 MA(w.Q, X1(no, oo), X3(nv, o * oo, no, o, no, 1), vo3), 1.0,
                 MO(w.Z, X1(nv, vo2), X3(nv, oo, no, o, no, 1), v2o2),
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 0}, {2, 1, 0}},
                       {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) == sp(m, 1) && sp(m, 2) + sp(m, 1) == sp(m, 3) + sp(m, 4);
                 }, 0));

    // ---- Z += Zab/2: t2 (F_be - 1/2 t1 F_me) and t1 vooo ----------------------
    KV_TRY(kv_bcast(ctx, 1, vv * B, w.Fae, w.Xbe));
    KV_TRY(kv_gemm(ctx, nv, nv, no, B, -0.5, MA(t1, X1(nv, o), X1(no, 1), vo),
                   MA(w.Fme, X1(no, v), X1(nv, 1), vo), 1.0,
                   MO(w.Xbe, X1(nv, v), X1(nv, 1), vv)));
    // Zab[a,b,i,j] = t2[a,e,i,j] Xbe[b,e]   (M=(a,i,j), K=e, N=b); spins a i j e b
    KV_TRY(sgemm(nv * no * no, nv, nv, B, 0.5,
                 MA(t2, X3(nv, vo2, no, o, no, 1), X1(nv, oo), v2o2),
                 MA(w.Xbe, X1(nv, 1), X1(nv, v), vv), 1.0,
                 MO(w.Z, X3(nv, vo2, no, o, no, 1), X1(nv, oo), v2o2),
                 Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 3) == sp(m, 1) + sp(m, 2) && sp(m, 4) == sp(m, 3);
                 }, 0));
    // Zab += t1[a,m] vooo[b,m,i,j]   (M=a, K=m, N=(b,i,j)); spins a m b i j
    KV_TRY(sgemm(nv, nv * no * no, no, B, 0.5,
                 MA(t1, X1(nv, o), X1(no, 1), vo),
                 MAI(vooo, X1(no, oo), X3(nv, o * oo, no, o, no, 1)), 1.0,
                 MO(w.Z, X1(nv, vo2), X3(nv, oo, no, o, no, 1), v2o2),
                 Slots{{{0, 0, 2}, {2, 0, 2}}, {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 0}, {2, 1, 0}},
                       {{1, 1, 1}, {2, 1, 1}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) == sp(m, 1) && sp(m, 2) + sp(m, 1) == sp(m, 3) + sp(m, 4);
                 }, 0));

    // ---- Z += Zij/2: -t2 (F_mj + 1/2 t1 F_me) and vvvo t1 -----------------------
    KV_TRY(kv_bcast(ctx, 1, oo * B, w.Fmi, w.Xmj));
    KV_TRY(kv_gemm(ctx, no, no, nv, B, 0.5, MA(w.Fme, X1(no, v), X1(nv, 1), vo),
                   MA(t1, X1(nv, o), X1(no, 1), vo), 1.0,
                   MO(w.Xmj, X1(no, o), X1(no, 1), oo)));
    // Zij[a,b,i,j] = - t2[a,b,i,m] Xmj[m,j]   (M=(a,b,i), K=m, N=j); spins a b i m j
    KV_TRY(sgemm(nv * nv * no, no, no, B, -0.5,
                 MA(t2, X3(nv, vo2, nv, oo, no, o), X1(no, 1), v2o2),
                 MA(w.Xmj, X1(no, o), X1(no, 1), oo), 1.0,
                 MO(w.Z, X3(nv, vo2, nv, oo, no, o), X1(no, 1), v2o2),
                 Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 2) + sp(m, 3) && sp(m, 3) == sp(m, 4);
                 }, 0));
    // Zij += vvvo[a,b,e,j] t1[e,i]   (M=(a,b,j), K=e, N=i); spins a b j e i
    KV_TRY(sgemm(nv * nv * no, no, nv, B, 0.5,
                 MAI(vvvo, X3(nv, vv * o, nv, vo, no, 1), X1(nv, o)),
                 MA(t1, X1(nv, o), X1(no, 1), vo), 1.0,
                 MO(w.Z, X3(nv, vo2, nv, oo, no, 1), X1(no, o), v2o2),
                 Slots{{{0, 0, 0}, {2, 0, 0}}, {{0, 0, 1}, {2, 0, 1}}, {{0, 0, 2}, {2, 0, 2}},
                       {{0, 1, 2}, {1, 0, 2}}, {{1, 1, 2}, {2, 1, 2}}},
                 [](unsigned m) {
                     return sp(m, 0) + sp(m, 1) == sp(m, 3) + sp(m, 2) && sp(m, 3) == sp(m, 4);
                 }, 0));

    // ---- T2 += fac (1 - P(ab))(1 - P(ij)) (Z + ladders) -------------------------
    return kv_assemble_t2(ctx, B, nv, no, fac, w.Z, ladders ? w.Lc : nullptr, T2, seed_t2, sh);
}

extern "C" int kvft_stanton_residual(kvft_ctx *ctx, int nb, int nv, int no,
                                     const double *const F[4], const double *const I[9],
                                     const double *t1, const double *t2, double fac,
                                     double *T1, double *T2) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_stanton_residual: not on a dry-run context");
    if (!ctx || nb < 0 || nv <= 0 || no <= 0 || !F || !I || !t1 || !t2 || !T1 || !T2)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_stanton_residual: bad argument");
    for (int k = 0; k < 4; k++)
        if (!F[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_stanton_residual: null F block");
    for (int k = 0; k < 9; k++)
        if (!I[k]) return kv_fail(ctx, KVFT_EINVAL, "kvft_stanton_residual: null I block");
    cudaSetDevice(ctx->device);
    return kv_stanton(ctx, nb, nv, no, F, I, t1, t2, fac, T1, T2);
}

extern "C" int kvft_set_residual_spin_blocks(kvft_ctx *ctx, int half) {
    if (!ctx || half < 0) return kv_fail(ctx, KVFT_EINVAL, "residual spin blocks: bad argument");
    ctx->spin_half = half;
    return KVFT_OK;
}
