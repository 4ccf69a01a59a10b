// Device-resident FT-CCSD solve: Fermi-scaled integrals (kelvin/cc_utils.py:
// 569-602), the damped amplitude iteration (kelvin/cc_utils.py:111-173) and
// the one-call CCSD update (kelvin/ft_cc_equations.py:96-113).
//
// HBM layout of a solver (nv virtual / no occupied indices, ng tau points;
// for a system built from orbital energies nv = no = n), all FP64:
//   F blocks oo/ov/vo/vv; nine I blocks; eps[n] or explicit D1/D2
//   T1[ng][nv][no], T2[ng][nv][nv][no][no]   damped amplitudes (Kelvin's T_old)
//   T1b, T2b (same shapes)                   tbar = -F.vo - R1, -I.vvoo - R2
//   Stanton workspace for a chunk of tau points (context scratch).
// The fused quadrature pass integrates tbar and damps T in place, so the
// undamped T never touches HBM.
#include "kvft_internal.h"

#include <cstring>

#include <cmath>
#include <cstdio>
#include <thread>
#include <vector>

int kv_quad_single(kvft_ctx *ctx, int ng, int ig, long long P, int rank, int nv, int no,
                   const double *tbar, const double *ti, const double *G, const double *D,
                   const double *ev, const double *eo, double *out);

namespace {

__device__ __forceinline__ void fermi_sqrt(double beta, double e, double mu, double *so,
                                           double *sv) {
    const double x = beta * (e - mu);
    const double ex = exp(-fabs(x));
    const double f = (x > 0) ? ex / (1.0 + ex) : 1.0 / (1.0 + ex);      // occupation
    const double fv = (x > 0) ? 1.0 / (1.0 + ex) : ex / (1.0 + ex);     // vacancy
    *so = sqrt(f);
    *sv = sqrt(fv);
}

__global__ void fermi_kernel(int n, double beta, double mu, const double *__restrict__ eps,
                             double *__restrict__ sfo, double *__restrict__ sfv) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        fermi_sqrt(beta, eps[p], mu, &sfo[p], &sfv[p]);
}

// F_xy[p,q] = (fock - diag eps)[p,q] s_x[p] s_y[q], s_o = sqrt(f), s_v = sqrt(1-f)
__global__ void scale_fock_kernel(int n, const double *__restrict__ fock,
                                  const double *__restrict__ eps,
                                  const double *__restrict__ sfo,
                                  const double *__restrict__ sfv, double *oo, double *ov,
                                  double *vo, double *vv) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n * n; k += gridDim.x * blockDim.x) {
        const int p = k / n, q = k % n;
        const double f = fock[k] - (p == q ? eps[p] : 0.0);
        oo[k] = f * sfo[p] * sfo[q];
        ov[k] = f * sfo[p] * sfv[q];
        vo[k] = f * sfv[p] * sfo[q];
        vv[k] = f * sfv[p] * sfv[q];
    }
}

struct Blk9 {
    double *p[9];
};

// I_wxyz[p,q,r,s] = eri[p,q,r,s] s_w[p] s_x[q] s_y[r] s_z[s]; one read of eri,
// nine writes, block order vvvv vvvo vovv vvoo vovo oovv vooo ooov oooo
__global__ void scale_eri_kernel(int n, const double *__restrict__ eri,
                                 const double *__restrict__ sfo,
                                 const double *__restrict__ sfv, Blk9 out) {
    const long long n4 = (long long)n * n * n * n;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n4;
         k += (long long)gridDim.x * blockDim.x) {
        long long r = k;
        const int s = (int)(r % n); r /= n;
        const int q2 = (int)(r % n); r /= n;
        const int q = (int)(r % n);
        const int p = (int)(r / n);
        const double e = eri[k];
        const double op = sfo[p], vp = sfv[p], oq = sfo[q], vq = sfv[q];
        const double orr = sfo[q2], vr = sfv[q2], os = sfo[s], vs = sfv[s];
        out.p[0][k] = e * vp * vq * vr * vs;
        out.p[1][k] = e * vp * vq * vr * os;
        out.p[2][k] = e * vp * oq * vr * vs;
        out.p[3][k] = e * vp * vq * orr * os;
        out.p[4][k] = e * vp * oq * vr * os;
        out.p[5][k] = e * op * oq * vr * vs;
        out.p[6][k] = e * vp * oq * orr * os;
        out.p[7][k] = e * op * oq * orr * vs;
        out.p[8][k] = e * op * oq * orr * os;
    }
}

__global__ void sumsq_kernel(long long n, const double *__restrict__ x, double *__restrict__ part) {
    __shared__ double red[256];
    double a = 0.0;
    for (long long k = blockIdx.x * 256LL + threadIdx.x; k < n; k += (long long)gridDim.x * 256)
        a = fma(x[k], x[k], a);
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sum_kernel(const double *__restrict__ part, int n, double *__restrict__ out) {
    __shared__ double red[256];
    double a = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) a += part[k];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int sumsq(kvft_ctx *ctx, long long n, const double *x, double *dout) {
    int grid = (int)std::max(1LL, std::min((long long)ctx->sm_count * 4, (n + 255) / 256));
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "sumsq_partial", sizeof(double) * grid, &part));
    sumsq_kernel<<<grid, 256, 0, ctx->stream>>>(n, x, (double *)part);
    KV_TRY(kv_launch_check(ctx, "sumsq"));
    sum_kernel<<<1, 256, 0, ctx->stream>>>((double *)part, grid, dout);
    return kv_launch_check(ctx, "sum");
}

// T = alpha T + (1 - alpha) u with a block partial of |u - T_old|^2
__global__ void damp_norm_kernel(long long n, double alpha, const double *__restrict__ u,
                                 double *__restrict__ T, double *__restrict__ part) {
    __shared__ double red[256];
    double a = 0.0;
    for (long long k = blockIdx.x * 256LL + threadIdx.x; k < n; k += (long long)gridDim.x * 256) {
        const double told = T[k];
        const double d = u[k] - told;
        a = fma(d, d, a);
        T[k] = alpha * told + (1.0 - alpha) * u[k];
    }
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

int damp_norm(kvft_ctx *ctx, long long n, double alpha, const double *u, double *T,
              double *dout) {
    const int grid = (int)std::max(1LL, std::min((long long)ctx->sm_count * 4, (n + 255) / 256));
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "damp_norm_partial", sizeof(double) * grid, &part));
    KvProfScope prof(ctx, KV_CAT_ELEM, 24.0 * n);
    damp_norm_kernel<<<grid, 256, 0, ctx->stream>>>(n, alpha, u, T, (double *)part);
    KV_TRY(kv_launch_check(ctx, "damp_norm"));
    sum_kernel<<<1, 256, 0, ctx->stream>>>((double *)part, grid, dout);
    return kv_launch_check(ctx, "sum");
}

// tbar seed: dst[b] = -blk for every tau point b
int seed_neg(kvft_ctx *ctx, int nb, long long count, const double *blk, double *dst) {
    int d[4] = {1, 1, 1, (int)count};
    long long ss[4] = {0, 0, 0, 1}, ds[4] = {0, 0, 0, 1};
    return kv_axpby4(ctx, nb, d, -1.0, blk, ss, 0, 0.0, dst, ds, count);
}

}  // namespace

struct kvft_solver {
    kvft_ctx *ctx = nullptr;
    int nv = 0, no = 0, ng = 0, chunk = 1;
    int chunk_prec = -1;        // precision/digits the chunk was sized for
    double beta = 0, mu = 0;
    double *eps = nullptr, *sfo = nullptr, *sfv = nullptr;   // orbital-energy form
    double *D1 = nullptr, *D2 = nullptr;                     // explicit-denominator form
    double *F[4] = {};
    double *I[9] = {};
    double *ti = nullptr, *g = nullptr, *G = nullptr;
    std::vector<double> hti, hg, hG;
    double *T1 = nullptr, *T2 = nullptr, *T1b = nullptr, *T2b = nullptr;
    double *dsc = nullptr;      // device scalars
    std::vector<void *> allocs;
    double nl1 = 0.1, nl2 = 0.1;
    bool norms_valid = false;
    // spin blocks: the half h when the integrals were found spin-blocked
    // (0: not), and whether the residual uses them (amplitudes set from
    // outside that break the structure turn them off)
    int spin_half = 0;
    bool spin_on = true;
    // tau-integral convention: 0 Kelvin's (exp factor for x < y only), 1 the
    // dense-G convention of Gauss-Legendre grids (exp factor for every x)
    int full = 0;
    // asynchronous steps: the step's scalars land in pinned host memory and
    // `done` marks their arrival (kvft_solver_step_begin / _end)
    double *hsc = nullptr;
    cudaEvent_t done = nullptr;
    bool pending = false;
    // Anderson acceleration of the damped update (depth aa_m, 0: Kelvin's
    // update): FP32 history of steps dX and residual changes dR in slots,
    // the last residual, the Gram matrix of the dR, steps since a restart
    int aa_m = 0;
    float *aa_dX[3] = {}, *aa_dR[3] = {}, *aa_rprev = nullptr;
    double aa_G[3][3] = {};
    long long aa_k = 0;
    int aa_prec = -1;
    double aa_rr = 0.0;
    // an accelerated step split at its host decision: the first half (update
    // map and statistics) is queued and its statistics land in hsc + 16;
    // aa_step_finish waits for them, solves for the mixing coefficients and
    // queues the second half
    bool aa_mid = false;
    int aa_h = -1;              // spin layout of the history (0: every element)
    cudaEvent_t aa_ev = nullptr;
    double aa_damp = 0.0;
    int aa_nvalid = 0, aa_grid[2] = {0, 0};
    double *aa_part = nullptr;
    // history slots: aa_ord the complete pairs, newest first; aa_pend the
    // slot whose step dX the last update wrote (its dR completes at the next
    // statistics pass; -1: none); aa_slots the pairs of the step in flight
    int aa_ord[3] = {0, 0, 0}, aa_nord = 0, aa_pend = -1, aa_slots[3] = {0, 0, 0};
    bool aa_has_new = false;
    // CUDA graph of the damped iteration: on when graph_on; gexec replays the
    // launches captured for gkey (damping, precision, spin blocks, grid
    // convention, scratch generation); gwarm: the key of the last eager step
    struct GKey {
        double damp = -1.0;
        int prec = -1, spin = -1, full = -1;
        uint64_t gen = 0;
        bool operator==(const GKey &o) const {
            return damp == o.damp && prec == o.prec && spin == o.spin && full == o.full &&
                   gen == o.gen;
        }
    };
    int graph_on = 0;
    int graph_state = 0;        // 0 eager, 2 replaying, -1 capture failed (eager from then)
    cudaGraphExec_t gexec = nullptr;
    GKey gkey, gwarm;
    uint64_t glaunches = 0;
    long long s1() const { return (long long)nv * no; }
    long long s2() const { return s1() * s1(); }
};

namespace {

int salloc(kvft_solver *s, size_t bytes, double **p) {
    void *q = nullptr;
    KV_CHECK(s->ctx, cudaMalloc(&q, bytes ? bytes : 16));
    s->allocs.push_back(q);
    *p = (double *)q;
    return KVFT_OK;
}

int alloc_common(kvft_solver *s) {
    const size_t n1 = s->s1(), n2 = s->s2();
    const size_t no = s->no, nv = s->nv;
    const size_t bsz[4] = {no * no, no * nv, nv * no, nv * nv};
    for (int k = 0; k < 4; k++) KV_TRY(salloc(s, sizeof(double) * bsz[k], &s->F[k]));
    // vvvv vvvo vovv vvoo vovo oovv vooo ooov oooo
    const size_t isz[9] = {nv * nv * nv * nv, nv * nv * nv * no, nv * no * nv * nv,
                           nv * nv * no * no, nv * no * nv * no, no * no * nv * nv,
                           nv * no * no * no, no * no * no * nv, no * no * no * no};
    for (int k = 0; k < 9; k++) KV_TRY(salloc(s, sizeof(double) * isz[k], &s->I[k]));
    KV_TRY(salloc(s, sizeof(double) * s->ng, &s->ti));
    KV_TRY(salloc(s, sizeof(double) * s->ng, &s->g));
    KV_TRY(salloc(s, sizeof(double) * s->ng * s->ng, &s->G));
    KV_TRY(salloc(s, sizeof(double) * s->ng * n1, &s->T1));
    KV_TRY(salloc(s, sizeof(double) * s->ng * n2, &s->T2));
    KV_TRY(salloc(s, sizeof(double) * s->ng * n1, &s->T1b));
    KV_TRY(salloc(s, sizeof(double) * s->ng * n2, &s->T2b));
    KV_TRY(salloc(s, sizeof(double) * 32, &s->dsc));
    return KVFT_OK;
}

int upload_grid(kvft_solver *s, const double *ti, const double *g, const double *G) {
    const int ng = s->ng;
    s->hti.assign(ti, ti + ng);
    s->hg.assign(g, g + ng);
    s->hG.assign(G, G + (size_t)ng * ng);
    cudaStream_t str = s->ctx->stream;
    KV_CHECK(s->ctx, cudaMemcpyAsync(s->ti, ti, sizeof(double) * ng, cudaMemcpyHostToDevice, str));
    KV_CHECK(s->ctx, cudaMemcpyAsync(s->g, g, sizeof(double) * ng, cudaMemcpyHostToDevice, str));
    KV_CHECK(s->ctx, cudaMemcpyAsync(s->G, G, sizeof(double) * ng * ng, cudaMemcpyHostToDevice,
                                     str));
    KV_CHECK(s->ctx, cudaMemsetAsync(s->T1, 0, sizeof(double) * ng * s->s1(), str));
    KV_CHECK(s->ctx, cudaMemsetAsync(s->T2, 0, sizeof(double) * ng * s->s2(), str));
    return KVFT_OK;
}

// tau points per Stanton call: workspace plus (tensor-core precisions) digit
// planes of two operands must fit in 60% of the memory not held by the solver
int pick_chunk(kvft_solver *s) {
    size_t fr = 0, tot = 0;
    KV_CHECK(s->ctx, cudaMemGetInfo(&fr, &tot));
    size_t held = 0;
    for (auto &kv : s->ctx->scratch) held += kv.second.second;
    size_t per = kv_chunk_bytes_per_tau(s->ctx, s->nv, s->no);
    size_t budget = (size_t)(0.6 * (double)(fr + held));
    if (s->ctx->workspace_limit > 0) budget = std::min(budget, s->ctx->workspace_limit);
    long long c = per ? (long long)(budget / per) : s->ng;
    s->chunk = (int)std::max(1LL, std::min((long long)s->ng, c));
    s->chunk_prec = s->ctx->precision * 16 + s->ctx->digits;
    return KVFT_OK;
}

// tbar = -F.vo - R1, -I.vvoo - R2 for all tau points
int form_tbar(kvft_solver *s) {
    kvft_ctx *ctx = s->ctx;
    if (s->chunk_prec != ctx->precision * 16 + ctx->digits) KV_TRY(pick_chunk(s));
    const long long n1 = s->s1(), n2 = s->s2();
    // the T2 seed -I.vvoo is written by the residual's final assembly
    KV_TRY(seed_neg(ctx, s->ng, n1, s->F[2], s->T1b));
    const double *Fc[4] = {s->F[0], s->F[1], s->F[2], s->F[3]};
    const double *Ic[9];
    for (int k = 0; k < 9; k++) Ic[k] = s->I[k];
    KvPackCacheScope cache(ctx);          // the integral blocks are the solver's own
    KvSpinScope spins(ctx, s->spin_on ? s->spin_half : 0);
    for (int y0 = 0; y0 < s->ng; y0 += s->chunk) {
        int nb = std::min(s->chunk, s->ng - y0);
        KV_TRY(kv_stanton(ctx, nb, s->nv, s->no, Fc, Ic, s->T1 + y0 * n1, s->T2 + y0 * n2, -1.0,
                          s->T1b + y0 * n1, s->T2b + y0 * n2, s->I[3]));
    }
    return KVFT_OK;
}

int integrate(kvft_solver *s, int mode, double damp, const double *t1b, const double *t2b,
              double *o1, double *o2, double *r1, double *r2) {
    KV_TRY(kv_quad_launch(s->ctx, mode, s->ng, s->s1(), 1, s->nv, s->no, t1b, s->ti,
                          s->hti.data(), s->G, s->hG.data(), s->D1, s->eps, s->eps, s->full,
                          damp, o1, r1));
    // the damped update skips the zero spin blocks of T2 (they stay zero)
    return kv_quad_launch(s->ctx, mode, s->ng, s->s2(), 2, s->nv, s->no, t2b, s->ti,
                          s->hti.data(), s->G, s->hG.data(), s->D2, s->eps, s->eps, s->full,
                          damp, o2, r2, s->spin_on ? s->spin_half : 0);
}

int read_scalars(kvft_solver *s, int count, double *h) {
    KV_CHECK(s->ctx, cudaMemcpyAsync(h, s->dsc, sizeof(double) * count, cudaMemcpyDeviceToHost,
                                     s->ctx->stream));
    KV_CHECK(s->ctx, cudaStreamSynchronize(s->ctx->stream));
    return KVFT_OK;
}

int refresh_norms(kvft_solver *s) {
    KV_TRY(sumsq(s->ctx, s->ng * s->s1(), s->T1, s->dsc + 8));
    KV_TRY(sumsq(s->ctx, s->ng * s->s2(), s->T2, s->dsc + 9));
    double h[10];
    KV_TRY(read_scalars(s, 10, h));
    s->nl1 = std::sqrt(h[8]) + 0.1;
    s->nl2 = std::sqrt(h[9]) + 0.1;
    s->norms_valid = true;
    return KVFT_OK;
}

// Spin-block check: 1 in *bad if any element of the [nb][n]^rank arrays
// outside the spin-conserving blocks is nonzero (rank 2: s_p = s_q; rank 4:
// s_p + s_q = s_r + s_s; s = index >= h).  Blocks over (batch, p, q), threads
// over the remaining (r, s) with 32-bit index arithmetic.
__global__ void spin_check_kernel(const double *__restrict__ x, int n, int h, int rank,
                                  long long rows, int *__restrict__ bad) {
    const int inner = rank == 4 ? n * n : n;
    for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
        int lead = 0;
        if (rank == 4) {
            const int pq = (int)(row % ((long long)n * n));
            lead = (pq / n >= h) + (pq % n >= h);
        } else {
            lead = ((int)(row % n) >= h) ? 1 : 0;
        }
        const double *r = x + row * inner;
        for (int e = threadIdx.x; e < inner; e += blockDim.x) {
            const int tail = rank == 4 ? (e / n >= h) + (e % n >= h) : (e >= h ? 1 : 0);
            if (tail != lead && r[e] != 0.0) *bad = 1;
        }
    }
}

// 1 when every listed array is spin-blocked with alpha half h
int spin_blocked(kvft_ctx *ctx, int n, int h, int count, const double *const *arr,
                 const int *rank, const long long *batch, int *yes) {
    void *flag = nullptr;
    KV_TRY(kv_scratch(ctx, "spin_check", sizeof(int), &flag));
    KV_CHECK(ctx, cudaMemsetAsync(flag, 0, sizeof(int), ctx->stream));
    for (int k = 0; k < count; k++) {
        const long long rows = batch[k] * (rank[k] == 4 ? (long long)n * n : n);
        const int grid = (int)std::min<long long>(rows, (long long)ctx->sm_count * 16);
        spin_check_kernel<<<grid, 256, 0, ctx->stream>>>(arr[k], n, h, rank[k], rows,
                                                         (int *)flag);
        KV_TRY(kv_launch_check(ctx, "spin_check"));
    }
    int h_bad = 0;
    KV_CHECK(ctx, cudaMemcpyAsync(&h_bad, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    *yes = h_bad ? 0 : 1;
    return KVFT_OK;
}

// Finds the spin blocks of the solver's integrals (general-spin ordering of
// the model systems: alpha half, then beta half).
int detect_spin_blocks(kvft_solver *s) {
    s->spin_half = 0;
    if (s->nv != s->no || s->nv % 2) return KVFT_OK;
    const int n = s->nv, h = n / 2;
    const double *arr[13];
    int rank[13];
    long long batch[13];
    for (int k = 0; k < 4; k++) arr[k] = s->F[k], rank[k] = 2, batch[k] = 1;
    for (int k = 0; k < 9; k++) arr[4 + k] = s->I[k], rank[4 + k] = 4, batch[4 + k] = 1;
    int yes = 0;
    KV_TRY(spin_blocked(s->ctx, n, h, 13, arr, rank, batch, &yes));
    s->spin_half = yes ? h : 0;
    return KVFT_OK;
}

int finish_create(kvft_solver *s, kvft_solver **out) {
    if (cudaStreamSynchronize(s->ctx->stream) != cudaSuccess)
        return kv_fail(s->ctx, KVFT_EDEVICE, "solver set-up kernels failed");
    KV_CHECK(s->ctx, cudaMallocHost(&s->hsc, 32 * sizeof(double)));
    KV_CHECK(s->ctx, cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
    KV_CHECK(s->ctx, cudaEventCreateWithFlags(&s->aa_ev, cudaEventDisableTiming));
    KV_TRY(detect_spin_blocks(s));
    KV_TRY(pick_chunk(s));
    *out = s;
    return KVFT_OK;
}

// ---------------------------------------------------------------------------
// Anderson acceleration (type II) of the fixed-point map Phi (the amplitude
// update ccsd_stanton) with mixing beta = 1 - damp:
//     r_k = Phi(x_k) - x_k,
//     x_{k+1} = x_k + beta r_k - sum_i gamma_i (dX_i + beta dR_i),
// gamma minimising |r_k - sum_i gamma_i dR_i| over the last m pairs
// dX_i = x_{i+1} - x_i, dR_i = r_{i+1} - r_i.  With no history the step is
// Kelvin's damped update.  The history is FP32: dX is stored as the step
// itself and dR from the FP64 residual minus the FP32 previous residual, so
// each keeps its precision relative to its own size.  Two fused passes per
// iteration over T1 and the spin-conserving elements of T2 (the rest stays
// zero), with fixed-order block reductions.
// ---------------------------------------------------------------------------
struct AaSeg {
    double *x;
    const double *phi;
    float *rprev;       // rprev and the history: the visit order (compact)
    float *dX[3], *dR[3];
    long long P;        // elements per tau point
    int ng;
    int h, n;           // h > 0: T2 spin runs (P = n^4), else every element
};
constexpr int AA_T = 256;
constexpr int AA_U = 4;     // elements per thread per batch (all loads before any store)
constexpr int AA_BLOCKS = 3; // resident blocks per SM (at most 85 registers a thread)

// The six spin patterns (sa, sb, si, sj) with sa + sb = si + sj (0 = alpha,
// 1 = beta), four bits each: sa | sb << 1 | si << 2 | sj << 3.
constexpr unsigned AA_PATTERNS = 0u | 15u << 4 | 10u << 8 | 6u << 12 | 9u << 16 | 5u << 20;

// Calls f(base, o, cb, cs, cnt) with batches of up to AA_U elements: the
// amplitude index base + o[u] and the compact index cb + u cs (the position
// in the visit order, which the FP32 history uses), u < cnt valid.  T2 with
// spin runs: one warp per (tau, spin pattern, a, b) quadrant of h x h
// elements (i, j in their halves), lanes along j; only the spin-conserving
// elements are visited and the compact order holds only them (6/16 of T2).
// Otherwise every element, the compact index the amplitude index.
template <class F>
__device__ __forceinline__ void aa_visit(const AaSeg &g, F f) {
    const int t = threadIdx.x, lane = t % 32;
    int o[AA_U];
    if (g.h > 0) {
        const int h = g.h, n = g.n, hh = h * h;
        const long long items = (long long)g.ng * 6 * hh;
        const long long nw = (long long)gridDim.x * (AA_T / 32);
        for (long long it = blockIdx.x * (long long)(AA_T / 32) + t / 32; it < items; it += nw) {
            const long long y = it / (6 * hh);
            const int rem = (int)(it - y * 6 * hh);
            const int pat = rem / hh, ab = rem - pat * hh;
            const int a1 = ab / h, b1 = ab - a1 * h;
            const unsigned c = AA_PATTERNS >> (4 * pat);
            const int a = a1 + (int)(c & 1u) * h, b = b1 + (int)((c >> 1) & 1u) * h;
            const long long base = y * g.P + (((long long)a * n + b) * n + (long long)((c >> 2) & 1u) * h) * n +
                                   (long long)((c >> 3) & 1u) * h;
            for (int k0 = 0; k0 < hh; k0 += 32 * AA_U) {
                int cnt = 0;
#pragma unroll
                for (int u = 0; u < AA_U; u++) {
                    const int k = k0 + u * 32 + lane;
                    const int i1 = k / h;
                    o[u] = i1 * n + (k - i1 * h);
                    if (k < hh) cnt = u + 1;
                }
                f(base, o, it * hh + k0 + lane, 32, cnt);
            }
        }
    } else {
        const long long tot = g.P * g.ng;
        const long long stride = (long long)gridDim.x * AA_T;
        for (long long e0 = blockIdx.x * (long long)AA_T + t; e0 < tot; e0 += stride * AA_U) {
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < AA_U; u++) {
                o[u] = (int)(u * stride);
                if (e0 + o[u] < tot) cnt = u + 1;
            }
            f(e0, o, e0, (int)stride, cnt);
        }
    }
}

template <int K>
__device__ __forceinline__ void aa_block_sum(double (&v)[K], double *part) {
    __shared__ double red[K][AA_T / 32];
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double a = v[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) red[k][w] = a;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double a = 0.0;
        for (int q = 0; q < AA_T / 32; q++) a += red[threadIdx.x][q];
        part[blockIdx.x * K + threadIdx.x] = a;
    }
}

// The history pointers of one pass, newest first (q = 0 .. NV-1), resolved
// on the host so that the kernels index nothing at run time.
struct AaHist {
    const float *dX[3];
    const float *dR[3];
    float *dRnew;        // pass A: the slot completed now (null: none)
    float *dXst;         // pass B: the slot the step goes to
};

// GB300 has ~64x more FP32 than FP64 throughput, so the passes keep FP64
// only where the iterate needs it (r = Phi - x and the update of x); the
// history, the dot products (which only steer the mixing coefficients) and
// the norms of Kelvin's residual measure run in FP32 per thread and are
// summed in FP64 per block; the conversions between the two are integer
// operations on the bit patterns (kv_d2f, kv_f2d), not FP64-pipe ones.

// pass A: r = Phi - x; dRnew = r - rprev; rprev = r; sums <dR_q, dRnew>,
// <dR_q, r> over the NV valid slots, and <r, r>
template <int NV>
__global__ void __launch_bounds__(AA_T, AA_BLOCKS)
aa_stats_kernel(AaSeg g, AaHist hs, double *part) {
    float v[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const bool has_new = hs.dRnew != nullptr;
    aa_visit(g, [&](long long base, const int (&o)[AA_U], long long cb, int cs, int cnt) {
        const double *phi = g.phi + base, *x = g.x + base;
        float *rprev = g.rprev + cb;
        double ph[AA_U], xx[AA_U];
        float rp[AA_U], dh[NV > 0 ? NV : 1][AA_U];
#pragma unroll
        for (int u = 0; u < AA_U; u++) {
            if (u >= cnt) break;
            ph[u] = phi[o[u]];
            xx[u] = x[o[u]];
            rp[u] = has_new ? rprev[u * cs] : 0.f;
#pragma unroll
            for (int q = 0; q < NV; q++)
                dh[q][u] = (q == 0 && has_new) ? 0.f : hs.dR[q][cb + u * cs];
        }
#pragma unroll
        for (int u = 0; u < AA_U; u++) {
            if (u >= cnt) break;
            const float r = kv_d2f(ph[u] - xx[u]);
            const float dn = has_new ? r - rp[u] : 0.f;
            if (has_new) hs.dRnew[cb + u * cs] = dn;
            rprev[u * cs] = r;
#pragma unroll
            for (int q = 0; q < NV; q++) {
                const float di = (q == 0 && has_new) ? dn : dh[q][u];
                v[q] = fmaf(di, dn, v[q]);
                v[3 + q] = fmaf(di, r, v[3 + q]);
            }
            v[6] = fmaf(r, r, v[6]);
        }
    });
    double w[7];
#pragma unroll
    for (int k = 0; k < 7; k++) w[k] = (double)v[k];
    aa_block_sum<7>(w, part);
}

// pass B: x += beta r - sum_q gamma_q (dX_q + beta dR_q); dXst = the step;
// sums |step|^2 and |x_new|^2
template <int NV>
__global__ void __launch_bounds__(AA_T, AA_BLOCKS)
aa_update_kernel(AaSeg g, AaHist hs, double beta, float g0, float g1, float g2,
                 double *part) {
    float v[2] = {0.f, 0.f};
    const float gam[3] = {g0, g1, g2};
    const float bf = (float)beta;
    aa_visit(g, [&](long long base, const int (&o)[AA_U], long long cb, int cs, int cnt) {
        const double *phi = g.phi + base;
        double *x = g.x + base;
        double ph[AA_U], xx[AA_U];
        float hsum[AA_U];
#pragma unroll
        for (int u = 0; u < AA_U; u++) {
            if (u >= cnt) break;
            ph[u] = phi[o[u]];
            xx[u] = x[o[u]];
            float a = 0.f;
#pragma unroll
            for (int q = 0; q < NV; q++)
                a = fmaf(gam[q], fmaf(bf, hs.dR[q][cb + u * cs], hs.dX[q][cb + u * cs]), a);
            hsum[u] = a;
        }
#pragma unroll
        for (int u = 0; u < AA_U; u++) {
            if (u >= cnt) break;
            const double d = fma(beta, ph[u] - xx[u], -kv_f2d(hsum[u]));
            const double xn = xx[u] + d;
            x[o[u]] = xn;
            const float df = kv_d2f(d), xf = kv_d2f(xn);
            hs.dXst[cb + u * cs] = df;
            v[0] = fmaf(df, df, v[0]);
            v[1] = fmaf(xf, xf, v[1]);
        }
    });
    double w[2] = {(double)v[0], (double)v[1]};
    aa_block_sum<2>(w, part);
}

// out[k] = sum over blocks of part[b K + k] (fixed order)
__global__ void aa_reduce_kernel(const double *__restrict__ part, int nb, int K,
                                 double *__restrict__ out) {
    __shared__ double red[256];
    for (int k = 0; k < K; k++) {
        double a = 0.0;
        for (int b = threadIdx.x; b < nb; b += 256) a += part[b * K + k];
        red[threadIdx.x] = a;
        __syncthreads();
        for (int s2 = 128; s2 > 0; s2 >>= 1) {
            if (threadIdx.x < s2) red[threadIdx.x] += red[threadIdx.x + s2];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[k] = red[0];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Amplitude read-back through pinned staging.  A chunk of T2 goes to one half
// of the context's pinned, device-mapped staging buffer (written by a gather
// kernel over the C2C / PCIe link), and host threads copy it on into the
// caller's array while the device fills the other half, so that the first
// touch of the destination pages is spread over the host cores.  With spin
// blocks and a destination known to be zero, only the spin-conserving
// elements travel, in the quadrant order of the Anderson passes (tau, spin
// pattern, a, b, then the h x h block of (i, j)).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ long long spin_item_base(long long it, long long P, int n,
                                                            int h) {
    const int hh = h * h;
    const long long y = it / (6 * hh);
    const int rem = (int)(it - y * 6 * hh);
    const int pat = rem / hh, ab = rem - pat * hh;
    const int a1 = ab / h, b1 = ab - a1 * h;
    const unsigned c = AA_PATTERNS >> (4 * pat);
    const long long a = a1 + (long long)(c & 1u) * h, b = b1 + (long long)((c >> 1) & 1u) * h;
    return y * P + ((a * n + b) * n + (long long)((c >> 2) & 1u) * h) * n +
           (long long)((c >> 3) & 1u) * h;
}

// out[t] = T2 at the t-th element of items [it0, it0 + nit)
__global__ void __launch_bounds__(256)
amp_gather_kernel(const double *__restrict__ T2, long long P, int n, int h, long long it0,
                  long long nit, double *__restrict__ out) {
    const int hh = h * h;
    const long long tot = nit * hh;
    for (long long t = blockIdx.x * 256LL + threadIdx.x; t < tot; t += (long long)gridDim.x * 256) {
        const long long it = t / hh;
        const int k = (int)(t - it * hh), i1 = k / h;
        out[t] = T2[spin_item_base(it0 + it, P, n, h) + (long long)i1 * n + (k - i1 * h)];
    }
}

// runs f(lo, hi) over [0, n) split across the host threads
template <class F>
void host_parallel(long long n, F f) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = (int)std::max(1LL, std::min<long long>(hw ? hw : 4, (n + 1023) / 1024));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; t++)
        th.emplace_back(f, n * t / nt, n * (t + 1) / nt);
    f(0, n / nt);
    for (auto &x : th) x.join();
}

void destroy(kvft_solver *s) {
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    for (void *p : s->allocs) cudaFree(p);
    if (s->hsc) cudaFreeHost(s->hsc);
    if (s->done) cudaEventDestroy(s->done);
    if (s->aa_ev) cudaEventDestroy(s->aa_ev);
    delete s;
}

}  // namespace

extern "C" {

size_t kvft_solver_footprint(int n, int ng, int precision) {
    (void)precision;
    size_t n2 = (size_t)n * n, n4 = n2 * n2;
    size_t fixed = sizeof(double) * (9 * n4 + 4 * n2 + 3 * n + 2 * (size_t)ng * (n2 + n4) + n4);
    return fixed + kv_stanton_workspace(1, n, n);
}

int kvft_solver_create(kvft_ctx *ctx, int n, int ng, const double *eps, const double *fock,
                       const double *eri, double beta, double mu, const double *ti,
                       const double *g, const double *G, kvft_solver **out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_solver_create: not on a dry-run context");
    if (!ctx || !out || n <= 0 || ng < 1 || ng > 64 || !eps || !fock || !eri || !ti || !g ||
        !G || !(beta > 0.0))
        return kv_fail(ctx, KVFT_EINVAL, "solver_create: bad argument");
    cudaSetDevice(ctx->device);
    *out = nullptr;
    kvft_solver *s = new kvft_solver();
    s->ctx = ctx;
    s->nv = s->no = n;
    s->ng = ng;
    s->beta = beta;
    s->mu = mu;
    const size_t n2 = (size_t)n * n, n4 = n2 * n2;
    double *dfock = nullptr, *deri = nullptr;
    int st = alloc_common(s);
    if (st == KVFT_OK) st = salloc(s, sizeof(double) * n, &s->eps);
    if (st == KVFT_OK) st = salloc(s, sizeof(double) * n, &s->sfo);
    if (st == KVFT_OK) st = salloc(s, sizeof(double) * n, &s->sfv);
    if (st == KVFT_OK) st = upload_grid(s, ti, g, G);
    if (st == KVFT_OK && (cudaMalloc(&dfock, sizeof(double) * n2) != cudaSuccess ||
                          cudaMalloc(&deri, sizeof(double) * n4) != cudaSuccess))
        st = kv_fail(ctx, KVFT_ENOMEM, "solver_create: no room for the raw integrals");
    if (st == KVFT_OK) {
        cudaStream_t str = ctx->stream;
        // host or device pointers (unified addressing picks the direction)
        if (cudaMemcpyAsync(s->eps, eps, sizeof(double) * n, cudaMemcpyDefault, str) ||
            cudaMemcpyAsync(dfock, fock, sizeof(double) * n2, cudaMemcpyDefault, str) ||
            cudaMemcpyAsync(deri, eri, sizeof(double) * n4, cudaMemcpyDefault, str))
            st = kv_fail(ctx, KVFT_EDEVICE, "solver_create: upload failed");
    }
    if (st == KVFT_OK) {
        cudaStream_t str = ctx->stream;
        fermi_kernel<<<1, 256, 0, str>>>(n, beta, mu, s->eps, s->sfo, s->sfv);
        st = kv_launch_check(ctx, "fermi");
        if (st == KVFT_OK) {
            int gb = (int)std::max<size_t>(1, std::min<size_t>((n2 + 255) / 256, 1024));
            scale_fock_kernel<<<gb, 256, 0, str>>>(n, dfock, s->eps, s->sfo, s->sfv, s->F[0],
                                                   s->F[1], s->F[2], s->F[3]);
            st = kv_launch_check(ctx, "scale_fock");
        }
        if (st == KVFT_OK) {
            Blk9 b;
            for (int k = 0; k < 9; k++) b.p[k] = s->I[k];
            scale_eri_kernel<<<ctx->sm_count * 8, 256, 0, str>>>(n, deri, s->sfo, s->sfv, b);
            st = kv_launch_check(ctx, "scale_eri");
        }
    }
    if (st == KVFT_OK) st = finish_create(s, out);
    cudaStreamSynchronize(ctx->stream);
    if (dfock) cudaFree(dfock);
    if (deri) cudaFree(deri);
    if (st != KVFT_OK) destroy(s);
    return st;
}

// Solver over given blocks (host pointers) and explicit denominators, for
// Kelvin's cc_utils.ft_cc_iter signature: F[4], I[9] in the kvft.h order,
// D1[nv][no], D2[nv][nv][no][no].
int kvft_solver_create_blocks(kvft_ctx *ctx, int nv, int no, int ng, const double *const F[4],
                              const double *const I[9], const double *D1, const double *D2,
                              double beta, const double *ti, const double *g, const double *G,
                              kvft_solver **out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_solver_create_blocks: not on a dry-run context");
    if (!ctx || !out || nv <= 0 || no <= 0 || ng < 1 || ng > 64 || !F || !I || !D1 || !D2 ||
        !ti || !g || !G || beta == 0.0)
        return kv_fail(ctx, KVFT_EINVAL, "solver_create_blocks: bad argument");
    cudaSetDevice(ctx->device);
    *out = nullptr;
    kvft_solver *s = new kvft_solver();
    s->ctx = ctx;
    s->nv = nv;
    s->no = no;
    s->ng = ng;
    s->beta = beta;
    const size_t n1 = s->s1(), n2 = s->s2();
    int st = alloc_common(s);
    if (st == KVFT_OK) st = salloc(s, sizeof(double) * n1, &s->D1);
    if (st == KVFT_OK) st = salloc(s, sizeof(double) * n2, &s->D2);
    if (st == KVFT_OK) st = upload_grid(s, ti, g, G);
    if (st == KVFT_OK) {
        const size_t sv = nv, so = no;
        const size_t bsz[4] = {so * so, so * sv, sv * so, sv * sv};
        const size_t isz[9] = {sv * sv * sv * sv, sv * sv * sv * so, sv * so * sv * sv,
                               sv * sv * so * so, sv * so * sv * so, so * so * sv * sv,
                               sv * so * so * so, so * so * so * sv, so * so * so * so};
        cudaStream_t str = ctx->stream;
        for (int k = 0; k < 4 && st == KVFT_OK; k++)
            if (!F[k] || cudaMemcpyAsync(s->F[k], F[k], sizeof(double) * bsz[k],
                                         cudaMemcpyHostToDevice, str))
                st = kv_fail(ctx, KVFT_EINVAL, "solver_create_blocks: F upload");
        for (int k = 0; k < 9 && st == KVFT_OK; k++)
            if (!I[k] || cudaMemcpyAsync(s->I[k], I[k], sizeof(double) * isz[k],
                                         cudaMemcpyHostToDevice, str))
                st = kv_fail(ctx, KVFT_EINVAL, "solver_create_blocks: I upload");
        if (st == KVFT_OK &&
            (cudaMemcpyAsync(s->D1, D1, sizeof(double) * n1, cudaMemcpyHostToDevice, str) ||
             cudaMemcpyAsync(s->D2, D2, sizeof(double) * n2, cudaMemcpyHostToDevice, str)))
            st = kv_fail(ctx, KVFT_EDEVICE, "solver_create_blocks: D upload");
    }
    if (st == KVFT_OK) st = finish_create(s, out);
    if (st != KVFT_OK) destroy(s);
    return st;
}

int kvft_solver_destroy(kvft_solver *s) {
    if (!s) return KVFT_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    // cached digit planes of this solver's integrals (their addresses may be
    // reused by later allocations)
    kv_pack_cache_clear(s->ctx);
    destroy(s);
    return KVFT_OK;
}

namespace {

// The step's five scalars and the device status word of the bounded waits
// (a tensor-core wait that expired) into pinned host memory, on the stream.
int queue_readback(kvft_solver *s) {
    kvft_ctx *ctx = s->ctx;
    KV_CHECK(ctx, cudaMemcpyAsync(s->hsc, s->dsc, 5 * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaMemcpyAsync(s->hsc + 15, ctx->dflag, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    return KVFT_OK;
}

// Solves (A + lambda I) g = t for the n <= 3 valid slots (Gaussian
// elimination with partial pivoting); false if it is singular or not finite.
bool aa_solve(int n, double A[3][3], double *t, double *g) {
    double tr = 0.0;
    for (int i = 0; i < n; i++) tr += A[i][i];
    const double lam = 1e-12 * (tr > 0.0 ? tr : 1.0) / (n > 0 ? n : 1);
    double M[3][4];
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) M[i][j] = A[i][j] + (i == j ? lam : 0.0);
        M[i][3] = t[i];
    }
    for (int c = 0; c < n; c++) {
        int pv = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(M[r][c]) > std::fabs(M[pv][c])) pv = r;
        if (!(std::fabs(M[pv][c]) > 0.0)) return false;
        if (pv != c)
            for (int j = 0; j < 4; j++) std::swap(M[c][j], M[pv][j]);
        for (int r = c + 1; r < n; r++) {
            const double f = M[r][c] / M[c][c];
            for (int j = c; j < 4; j++) M[r][j] -= f * M[c][j];
        }
    }
    for (int c = n - 1; c >= 0; c--) {
        double v = M[c][3];
        for (int j = c + 1; j < n; j++) v -= M[c][j] * g[j];
        g[c] = v / M[c][c];
        if (!std::isfinite(g[c])) return false;
    }
    return true;
}

// The T2 spin half the Anderson passes visit by (0: every element).
int aa_half(const kvft_solver *s) {
    return (s->spin_on && s->spin_half > 0 && s->nv == s->no) ? s->spin_half : 0;
}

// FP32 history of depth m in the visit order of the current spin layout:
// ng (nv no + 6 h^4) words per array with spin runs, ng (nv no + (nv no)^2)
// without; arrays of another layout are freed first.
int aa_alloc(kvft_solver *s, int m) {
    const int h = aa_half(s);
    float **arr[7] = {&s->aa_rprev, &s->aa_dX[0], &s->aa_dR[0], &s->aa_dX[1], &s->aa_dR[1],
                      &s->aa_dX[2], &s->aa_dR[2]};
    if (s->aa_h != h) {
        cudaStreamSynchronize(s->ctx->stream);
        for (float **p : arr) {
            if (!*p) continue;
            for (size_t i = 0; i < s->allocs.size(); i++)
                if (s->allocs[i] == (void *)*p) {
                    s->allocs.erase(s->allocs.begin() + i);
                    break;
                }
            cudaFree(*p);
            *p = nullptr;
        }
        s->aa_h = h;
        s->chunk_prec = -1;
    }
    if (m == 0) return KVFT_OK;
    const size_t words = (size_t)s->ng * (s->s1() + (h ? 6 * (size_t)h * h * h * h : s->s2()));
    for (int i = 0; i < 1 + 2 * m; i++) {
        if (*arr[i]) continue;
        void *q = nullptr;
        if (cudaMalloc(&q, sizeof(float) * words) != cudaSuccess) {
            cudaGetLastError();
            return kv_fail(s->ctx, KVFT_ENOMEM, "solver_set_acceleration: no room for the history");
        }
        s->allocs.push_back(q);
        *arr[i] = (float *)q;
        s->chunk_prec = -1;            // re-size the tau chunk for the memory left
    }
    return KVFT_OK;
}

void aa_segments(kvft_solver *s, AaSeg *g1, AaSeg *g2) {
    const long long n1 = s->s1(), n2 = s->s2(), ng = s->ng;
    *g1 = AaSeg{s->T1, s->T1b, s->aa_rprev, {}, {}, n1, s->ng, 0, 0};
    *g2 = AaSeg{s->T2, s->T2b, s->aa_rprev + ng * n1, {}, {}, n2, s->ng, aa_half(s), s->no};
    for (int i = 0; i < s->aa_m; i++) {
        g1->dX[i] = s->aa_dX[i];
        g1->dR[i] = s->aa_dR[i];
        g2->dX[i] = s->aa_dX[i] + ng * n1;
        g2->dR[i] = s->aa_dR[i] + ng * n1;
    }
}

// grid and partial-sum buffer of one Anderson pass over a segment
// (one wave: AA_BLOCKS resident blocks per SM, every block striding over
// the segment)
int aa_launch_grid(kvft_ctx *ctx, const AaSeg &g) {
    const long long wanted = g.h > 0 ? ((long long)g.ng * 6 * g.h * g.h + AA_T / 32 - 1) / (AA_T / 32)
                                     : (g.P * g.ng + AA_T * AA_U - 1) / (AA_T * AA_U);
    return (int)std::max(1LL, std::min((long long)ctx->sm_count * AA_BLOCKS, wanted));
}

// elements one pass visits (the spin-conserving sixth-of-16 of T2 with
// spin runs)
double aa_visited(const AaSeg &g) {
    return g.h > 0 ? (double)g.ng * 6.0 * g.h * g.h * g.h * g.h : (double)g.P * g.ng;
}

// The accelerated iteration up to the queued scalars (as the damped one
// leaves them for kvft_solver_step_end: |dT1|^2, |T1|^2, |dT2|^2, |T2|^2,
// Omega_cc).  One host wait, for the least-squares coefficients.
int aa_step_begin(kvft_solver *s, double damp) {
    kvft_ctx *ctx = s->ctx;
    if (aa_half(s) != s->aa_h) {       // the spin layout changed: a new history
        KV_TRY(aa_alloc(s, s->aa_m));
        s->aa_k = 0;
    }
    if (!s->norms_valid) KV_TRY(refresh_norms(s));
    KV_TRY(form_tbar(s));
    // Phi(x) in place of tbar (spin-conserving elements only: the passes
    // below read no other)
    KV_TRY(integrate(s, 0, 0.0, s->T1b, s->T2b, s->T1b, s->T2b, nullptr, nullptr));
    const int prec = ctx->precision * 16 + ctx->digits;
    // a new precision is a new map: restart (keeping the earlier map's pairs
    // doubled the FP64-accurate sweeps of the 114-spin-orbital mixed solve)
    if (prec != s->aa_prec) {
        s->aa_k = 0;
        s->aa_prec = prec;
    }
    if (s->aa_k == 0) {
        s->aa_nord = 0;
        s->aa_pend = -1;
    }
    const int m = s->aa_m;
    AaSeg g[2];
    aa_segments(s, &g[0], &g[1]);
    // the pairs of this step, newest first: the pending one (completed by
    // this pass) and the complete ones
    const bool has_new = s->aa_pend >= 0;
    int slots[3], nvalid = 0;
    if (has_new) slots[nvalid++] = s->aa_pend;
    for (int i = 0; i < s->aa_nord && nvalid < m; i++) slots[nvalid++] = s->aa_ord[i];
    const int gridA[2] = {aa_launch_grid(ctx, g[0]), aa_launch_grid(ctx, g[1])};
    void *pp = nullptr;
    KV_TRY(kv_scratch(ctx, "aa_partial",
                      sizeof(double) * 7 * (size_t)(gridA[0] + gridA[1]), &pp));
    double *part = (double *)pp;
    {
        KvProfScope prof(ctx, KV_CAT_ELEM,
                         (aa_visited(g[0]) + aa_visited(g[1])) *
                             (28.0 + 4.0 * (nvalid - (has_new ? 1 : 0))));
        for (int q = 0; q < 2; q++) {
            AaHist hs{};
            for (int t = 0; t < nvalid; t++) {
                hs.dX[t] = g[q].dX[slots[t]];
                hs.dR[t] = g[q].dR[slots[t]];
            }
            hs.dRnew = has_new ? g[q].dR[slots[0]] : nullptr;
            double *pq = part + (q ? 7 * gridA[0] : 0);
            switch (nvalid) {
            case 0: aa_stats_kernel<0><<<gridA[q], AA_T, 0, ctx->stream>>>(g[q], hs, pq); break;
            case 1: aa_stats_kernel<1><<<gridA[q], AA_T, 0, ctx->stream>>>(g[q], hs, pq); break;
            case 2: aa_stats_kernel<2><<<gridA[q], AA_T, 0, ctx->stream>>>(g[q], hs, pq); break;
            default: aa_stats_kernel<3><<<gridA[q], AA_T, 0, ctx->stream>>>(g[q], hs, pq); break;
            }
            KV_TRY(kv_launch_check(ctx, "aa_stats"));
            aa_reduce_kernel<<<1, 256, 0, ctx->stream>>>(part + (q ? 7 * gridA[0] : 0),
                                                         gridA[q], 7, s->dsc + 8 + 7 * q);
            KV_TRY(kv_launch_check(ctx, "aa_reduce"));
        }
    }
    KV_CHECK(ctx, cudaMemcpyAsync(s->hsc + 16, s->dsc + 8, 14 * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK(ctx, cudaEventRecord(s->aa_ev, ctx->stream));
    s->aa_mid = true;
    s->aa_damp = damp;
    s->aa_nvalid = nvalid;
    s->aa_has_new = has_new;
    for (int t = 0; t < nvalid; t++) s->aa_slots[t] = slots[t];
    s->aa_grid[0] = gridA[0];
    s->aa_grid[1] = gridA[1];
    s->aa_part = part;
    s->pending = true;
    return KVFT_OK;
}

// The second half of an accelerated step: the host's least-squares solve on
// the statistics of the first, then the update pass, the energy and the
// step's scalars (as the damped step leaves them).
int aa_step_finish(kvft_solver *s) {
    kvft_ctx *ctx = s->ctx;
    s->aa_mid = false;
    KV_CHECK(ctx, cudaEventSynchronize(s->aa_ev));
    const double *st = s->hsc + 16;
    const int m = s->aa_m;
    AaSeg g[2];
    aa_segments(s, &g[0], &g[1]);
    const long long k = s->aa_k;
    const bool has_new = s->aa_has_new;
    int nvalid = s->aa_nvalid;
    int slot[3];
    for (int t = 0; t < nvalid; t++) slot[t] = s->aa_slots[t];
    const int gridA[2] = {s->aa_grid[0], s->aa_grid[1]};
    double *part = s->aa_part;
    const double damp = s->aa_damp;
    const double rr = st[6] + st[13];
    if (!std::isfinite(rr)) return kv_fail(ctx, KVFT_EDIVERGE, "non-finite residual");
    double gam[3] = {0.0, 0.0, 0.0};
    if (nvalid > 0 && rr > 100.0 * s->aa_rr) nvalid = 0;     // blew up: plain step, restart
    if (nvalid > 0) {
        if (has_new)                   // the completed pair against every pair
            for (int q = 0; q < nvalid; q++)
                s->aa_G[slot[0]][slot[q]] = s->aa_G[slot[q]][slot[0]] = st[q] + st[7 + q];
        double A[3][3], t[3];
        for (int q = 0; q < nvalid; q++) {
            t[q] = st[3 + q] + st[10 + q];
            for (int p2 = 0; p2 < nvalid; p2++) A[q][p2] = s->aa_G[slot[q]][slot[p2]];
        }
        if (!aa_solve(nvalid, A, t, gam)) nvalid = 0;
    }
    // complete pairs after this step (none: the history restarts here), and
    // the slot this step's dX goes to: a free one, else the oldest pair's
    // (read by this update before each element is overwritten)
    s->aa_nord = nvalid;
    for (int t = 0; t < nvalid; t++) s->aa_ord[t] = slot[t];
    bool used[3] = {false, false, false};
    for (int t = 0; t < s->aa_nord; t++) used[s->aa_ord[t]] = true;
    int jst = -1;
    for (int j = 0; j < m && jst < 0; j++)
        if (!used[j]) jst = j;
    if (jst < 0) jst = s->aa_ord[--s->aa_nord];
    s->aa_pend = jst;
    const double beta = 1.0 - damp;
    const float gf[3] = {(float)gam[0], (float)gam[1], (float)gam[2]};
    const int gridB[2] = {gridA[0], gridA[1]};
    {
        KvProfScope prof(ctx, KV_CAT_ELEM,
                         (aa_visited(g[0]) + aa_visited(g[1])) * (28.0 + 8.0 * nvalid));
        for (int q = 0; q < 2; q++) {
            AaHist hs{};
            for (int t = 0; t < nvalid; t++) {
                hs.dX[t] = g[q].dX[slot[t]];
                hs.dR[t] = g[q].dR[slot[t]];
            }
            hs.dXst = g[q].dX[jst];
            double *pq = part + (q ? 2 * gridB[0] : 0);
            switch (nvalid) {
            case 0:
                aa_update_kernel<0><<<gridB[q], AA_T, 0, ctx->stream>>>(g[q], hs, beta, gf[0],
                                                                       gf[1], gf[2], pq);
                break;
            case 1:
                aa_update_kernel<1><<<gridB[q], AA_T, 0, ctx->stream>>>(g[q], hs, beta, gf[0],
                                                                       gf[1], gf[2], pq);
                break;
            case 2:
                aa_update_kernel<2><<<gridB[q], AA_T, 0, ctx->stream>>>(g[q], hs, beta, gf[0],
                                                                       gf[1], gf[2], pq);
                break;
            default:
                aa_update_kernel<3><<<gridB[q], AA_T, 0, ctx->stream>>>(g[q], hs, beta, gf[0],
                                                                       gf[1], gf[2], pq);
                break;
            }
            KV_TRY(kv_launch_check(ctx, "aa_update"));
            aa_reduce_kernel<<<1, 256, 0, ctx->stream>>>(part + (q ? 2 * gridB[0] : 0),
                                                         gridB[q], 2, s->dsc + 2 * q);
            KV_TRY(kv_launch_check(ctx, "aa_reduce"));
        }
    }
    s->aa_k = k + 1;
    s->aa_rr = rr;
    KV_TRY(kv_energy(ctx, s->ng, s->nv, s->no, s->T1, s->T2, s->F[1], s->I[5], s->g, s->beta, 1,
                     s->dsc + 4, s->spin_on ? s->spin_half : 0));
    KV_TRY(queue_readback(s));
    KV_CHECK(ctx, cudaEventRecord(s->done, ctx->stream));
    return KVFT_OK;
}

}  // namespace

namespace {

// The damped iteration's launches on the context's stream: update,
// integration + damping + norms, energy, read-back of the scalars.
int enqueue_damped(kvft_solver *s, double damp) {
    kvft_ctx *ctx = s->ctx;
    KV_TRY(form_tbar(s));
    // integrate + damp in place: T <- damp T + (1-damp) int(tbar)
    KV_TRY(integrate(s, 1, damp, s->T1b, s->T2b, s->T1, s->T2, s->dsc + 0, s->dsc + 2));
    KV_TRY(kv_energy(ctx, s->ng, s->nv, s->no, s->T1, s->T2, s->F[1], s->I[5], s->g, s->beta, 1,
                     s->dsc + 4, s->spin_on ? s->spin_half : 0));
    return queue_readback(s);
}

kvft_solver::GKey graph_key(kvft_solver *s, double damp) {
    kvft_solver::GKey k;
    k.damp = damp;
    k.prec = s->ctx->precision * 16 + s->ctx->digits;
    k.spin = s->spin_on ? s->spin_half : 0;
    k.full = s->full;
    k.gen = s->ctx->scratch_gen;
    return k;
}

// The damped iteration through a CUDA graph: an eager step with these
// settings first (it sizes every scratch buffer and fills the packed-integral
// cache), then one step captured and launched, then replays.  A capture
// that fails (or that would allocate) leaves the solver eager.
int graph_step(kvft_solver *s, double damp) {
    kvft_ctx *ctx = s->ctx;
    const kvft_solver::GKey k = graph_key(s, damp);
    if (s->gexec && !(k == s->gkey)) {
        cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
    }
    if (s->gexec) {
        KV_CHECK(ctx, cudaGraphLaunch(s->gexec, ctx->stream));
        ctx->launches += s->glaunches;
        return KVFT_OK;
    }
    if (!(k == s->gwarm)) {
        KV_TRY(enqueue_damped(s, damp));
        s->gwarm = graph_key(s, damp);
        return KVFT_OK;
    }
    const uint64_t l0 = ctx->launches, gen0 = ctx->scratch_gen;
    bool ok = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    int st = ok ? enqueue_damped(s, damp) : KVFT_OK;
    cudaGraph_t g = nullptr;
    if (ok) ok = cudaStreamEndCapture(ctx->stream, &g) == cudaSuccess && g != nullptr;
    ok = ok && st == KVFT_OK && ctx->scratch_gen == gen0;
    if (ok) ok = cudaGraphInstantiate(&s->gexec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    const uint64_t captured = ctx->launches - l0;
    ctx->launches = l0;                // nothing ran during the capture
    if (!ok) {
        cudaGetLastError();
        if (s->gexec) cudaGraphExecDestroy(s->gexec);
        s->gexec = nullptr;
        s->graph_state = -1;
        s->graph_on = 0;
        ctx->err.clear();
        return enqueue_damped(s, damp);
    }
    s->gkey = k;
    s->glaunches = captured;
    s->graph_state = 2;
    KV_CHECK(ctx, cudaGraphLaunch(s->gexec, ctx->stream));
    ctx->launches += captured;
    return KVFT_OK;
}

}  // namespace

// One amplitude iteration queued on the context's stream without waiting:
// update, integration + damping + norms, energy, and the copy of the five
// scalars to pinned host memory.  kvft_solver_step_end waits for them.
int kvft_solver_step_begin(kvft_solver *s, double damp) {
    if (!s) return KVFT_EINVAL;
    kvft_ctx *ctx = s->ctx;
    if (s->pending) return kv_fail(ctx, KVFT_EINVAL, "solver_step_begin: a step is pending");
    cudaSetDevice(ctx->device);
    if (s->aa_m > 0) return aa_step_begin(s, damp);
    if (!s->norms_valid) KV_TRY(refresh_norms(s));
    if (s->graph_on && !(ctx->prof && ctx->prof->on))
        KV_TRY(graph_step(s, damp));
    else
        KV_TRY(enqueue_damped(s, damp));
    KV_CHECK(ctx, cudaEventRecord(s->done, ctx->stream));
    s->pending = true;
    return KVFT_OK;
}

// Waits for the step queued by kvft_solver_step_begin; Kelvin's residual
// measure and the energy, as kvft_solver_step returns them.
int kvft_solver_step_end(kvft_solver *s, double *energy, double *res) {
    if (!s) return KVFT_EINVAL;
    kvft_ctx *ctx = s->ctx;
    if (!s->pending) return kv_fail(ctx, KVFT_EINVAL, "solver_step_end: no step is pending");
    s->pending = false;
    if (s->aa_mid) KV_TRY(aa_step_finish(s));
    KV_CHECK(ctx, cudaEventSynchronize(s->done));
    const double *h = s->hsc;
    int flag = 0;
    std::memcpy(&flag, h + 15, sizeof(int));
    if (flag != 0) {
        KV_CHECK(ctx, cudaMemsetAsync(ctx->dflag, 0, sizeof(int), ctx->stream));
        return kv_fail(ctx, KVFT_ETIMEOUT, "solver step: a bounded device wait expired (code " +
                                               std::to_string(flag) + ")");
    }
    const double res1 = std::sqrt(h[0]) / s->nl1;
    const double res2 = std::sqrt(h[2]) / s->nl2;
    s->nl1 = std::sqrt(h[1]) + 0.1;
    s->nl2 = std::sqrt(h[3]) + 0.1;
    if (energy) *energy = h[4];
    if (res) *res = res1 + res2;
    if (!std::isfinite(h[4]) || !std::isfinite(res1 + res2))
        return kv_fail(ctx, KVFT_EDIVERGE, "non-finite energy or residual");
    return KVFT_OK;
}

int kvft_solver_step(kvft_solver *s, double damp, double *energy, double *res) {
    KV_TRY(kvft_solver_step_begin(s, damp));
    return kvft_solver_step_end(s, energy, res);
}

int kvft_solver_run(kvft_solver *s, const kvft_solve_opts *o, kvft_result *r) {
    if (!s || !o || !r) return KVFT_EINVAL;
    kvft_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    if (o->full != 0 && o->full != 1) return kv_fail(ctx, KVFT_EINVAL, "solver: full must be 0 or 1");
    // the convention holds for this run and the steps that follow it
    s->full = o->full;
    if (o->guess != 2) s->aa_k = 0;
    if (o->guess == 0) {
        KV_CHECK(ctx, cudaMemsetAsync(s->T1, 0, sizeof(double) * s->ng * s->s1(), ctx->stream));
        KV_CHECK(ctx, cudaMemsetAsync(s->T2, 0, sizeof(double) * s->ng * s->s2(), ctx->stream));
    } else if (o->guess == 1) {
        KV_TRY(seed_neg(ctx, s->ng, s->s1(), s->F[2], s->T1b));
        KV_TRY(seed_neg(ctx, s->ng, s->s2(), s->I[3], s->T2b));
        KV_TRY(integrate(s, 0, 0.0, s->T1b, s->T2b, s->T1, s->T2, nullptr, nullptr));
    }
    KV_TRY(kv_energy(ctx, s->ng, s->nv, s->no, s->T1, s->T2, s->F[1], s->I[5], s->g, s->beta, 0,
                     s->dsc + 6, s->spin_on ? s->spin_half : 0));
    double h[7];
    KV_TRY(read_scalars(s, 7, h));
    r->e_guess = h[6];
    KV_TRY(refresh_norms(s));
    double Eold = 888888888.888888888;
    r->converged = 0;
    r->iterations = 0;
    r->res = 0.0;
    int i = 0;
    while (i < o->max_iter && !r->converged) {
        double E = 0.0, res = 0.0;
        KV_TRY(kvft_solver_step(s, o->damp, &E, &res));
        if (o->verbose) fprintf(stderr, " %2d  %.10f   %.4E\n", i + 1, E, res);
        i++;
        r->res = res;
        if (std::fabs(E - Eold) < o->econv && res < o->tconv) r->converged = 1;
        Eold = E;
    }
    r->iterations = i;
    r->omega_cc = Eold;
    return r->converged ? KVFT_OK : KVFT_ENOTCONV;
}

// Kelvin's tau-pointwise schedule (cc_utils.py:176-242, rt_iter = "point"):
// grid point by grid point, start from the linear extrapolation of the two
// previous points and iterate the single-point update (ft_cc_equations.py:
// 116-127) to res1 + res2 < tconv; the integrals of later points see the
// converged tbar of the earlier ones.  Omega = ft_cc_energy of the result.
int kvft_solver_run_point(kvft_solver *s, const kvft_solve_opts *o, kvft_result *r) {
    if (!s || !o || !r) return KVFT_EINVAL;
    kvft_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    // Kelvin's pointwise schedule integrates up to each point only, which is
    // the lower-triangular convention
    if (o->full) return kv_fail(ctx, KVFT_EINVAL, "solver_run_point: dense-G grids are not pointwise");
    const long long n1 = s->s1(), n2 = s->s2();
    const int ng = s->ng;
    if (s->chunk_prec != ctx->precision * 16 + ctx->digits) KV_TRY(pick_chunk(s));
    KV_CHECK(ctx, cudaMemsetAsync(s->T1, 0, sizeof(double) * ng * n1, ctx->stream));
    KV_CHECK(ctx, cudaMemsetAsync(s->T2, 0, sizeof(double) * ng * n2, ctx->stream));
    KV_CHECK(ctx, cudaMemsetAsync(s->T1b, 0, sizeof(double) * ng * n1, ctx->stream));
    KV_CHECK(ctx, cudaMemsetAsync(s->T2b, 0, sizeof(double) * ng * n2, ctx->stream));
    void *tmp = nullptr;
    KV_TRY(kv_scratch(ctx, "point_tmp", sizeof(double) * (n1 + n2), &tmp));
    double *u1 = (double *)tmp, *u2 = u1 + n1;
    const double *Fc[4] = {s->F[0], s->F[1], s->F[2], s->F[3]};
    const double *Ic[9];
    for (int k = 0; k < 9; k++) Ic[k] = s->I[k];
    const double nl1 = std::sqrt((double)n1), nl2 = std::sqrt((double)n2);
    int total = 0, all_conv = 1;
    double res = 0.0;
    for (int ig = 0; ig < ng; ig++) {
        double *t1b = s->T1b + ig * n1, *t2b = s->T2b + ig * n2;
        double *T1g = s->T1 + ig * n1, *T2g = s->T2 + ig * n2;
        KV_TRY(seed_neg(ctx, 1, n1, s->F[2], t1b));
        KV_TRY(seed_neg(ctx, 1, n2, s->I[3], t2b));
        if (ig == 0) continue;
        if (ig == 1) {
            KV_TRY(kv_quad_single(ctx, ng, ig, n1, 1, s->nv, s->no, s->T1b, s->ti, s->G, s->D1,
                                  s->eps, s->eps, T1g));
            KV_TRY(kv_quad_single(ctx, ng, ig, n2, 2, s->nv, s->no, s->T2b, s->ti, s->G, s->D2,
                                  s->eps, s->eps, T2g));
        } else {
            // linear extrapolation from the two previous grid points
            const double c = (s->hti[ig] - s->hti[ig - 1]) / (s->hti[ig - 2] - s->hti[ig - 1]);
            int d1[4] = {1, 1, 1, (int)n1}, d2[4] = {1, 1, 1, (int)n2};
            long long one[4] = {0, 0, 0, 1};
            KV_TRY(kv_axpby4(ctx, 1, d1, 1.0 - c, T1g - n1, one, 0, 0.0, T1g, one, 0));
            KV_TRY(kv_axpby4(ctx, 1, d1, c, T1g - 2 * n1, one, 0, 1.0, T1g, one, 0));
            KV_TRY(kv_axpby4(ctx, 1, d2, 1.0 - c, T2g - n2, one, 0, 0.0, T2g, one, 0));
            KV_TRY(kv_axpby4(ctx, 1, d2, c, T2g - 2 * n2, one, 0, 1.0, T2g, one, 0));
        }
        bool conv = false;
        int i = 0;
        while (i < o->max_iter && !conv) {
            KV_TRY(seed_neg(ctx, 1, n1, s->F[2], t1b));
            {
                KvPackCacheScope cache(ctx);
                KvSpinScope spins(ctx, s->spin_on ? s->spin_half : 0);
                KV_TRY(kv_stanton(ctx, 1, s->nv, s->no, Fc, Ic, T1g, T2g, -1.0, t1b, t2b,
                                  s->I[3]));
            }
            KV_TRY(kv_quad_single(ctx, ng, ig, n1, 1, s->nv, s->no, s->T1b, s->ti, s->G, s->D1,
                                  s->eps, s->eps, u1));
            KV_TRY(kv_quad_single(ctx, ng, ig, n2, 2, s->nv, s->no, s->T2b, s->ti, s->G, s->D2,
                                  s->eps, s->eps, u2));
            KV_TRY(damp_norm(ctx, n1, o->damp, u1, T1g, s->dsc + 0));
            KV_TRY(damp_norm(ctx, n2, o->damp, u2, T2g, s->dsc + 1));
            double h[2];
            KV_TRY(read_scalars(s, 2, h));
            res = std::sqrt(h[0]) / nl1 + std::sqrt(h[1]) / nl2;
            if (!std::isfinite(res)) return kv_fail(ctx, KVFT_EDIVERGE, "non-finite residual");
            if (o->verbose) fprintf(stderr, " point %d  %2d  %.4E\n", ig, i + 1, res);
            i++;
            conv = res < o->tconv;
        }
        total += i;
        if (!conv) all_conv = 0;
    }
    KV_TRY(kv_energy(ctx, s->ng, s->nv, s->no, s->T1, s->T2, s->F[1], s->I[5], s->g, s->beta, 1,
                     s->dsc + 4, s->spin_on ? s->spin_half : 0));
    double h[5];
    KV_TRY(read_scalars(s, 5, h));
    r->omega_cc = h[4];
    r->e_guess = 0.0;
    r->res = res;
    r->iterations = total;
    r->converged = all_conv;
    s->norms_valid = false;
    KV_TRY(kv_device_status(ctx));     // a tensor-core wait that expired
    return all_conv ? KVFT_OK : KVFT_ENOTCONV;
}

int kvft_solver_get_amplitudes(kvft_solver *s, double *T1h, double *T2h) {
    if (!s) return KVFT_EINVAL;
    if (T1h)
        KV_CHECK(s->ctx, cudaMemcpyAsync(T1h, s->T1, sizeof(double) * s->ng * s->s1(),
                                         cudaMemcpyDeviceToHost, s->ctx->stream));
    if (T2h)
        KV_CHECK(s->ctx, cudaMemcpyAsync(T2h, s->T2, sizeof(double) * s->ng * s->s2(),
                                         cudaMemcpyDeviceToHost, s->ctx->stream));
    KV_CHECK(s->ctx, cudaStreamSynchronize(s->ctx->stream));
    return KVFT_OK;
}

int kvft_solver_read_amplitudes(kvft_solver *s, double *T1h, double *T2h, int dst_zeroed) {
    if (!s || !T1h || !T2h) return KVFT_EINVAL;
    kvft_ctx *ctx = s->ctx;
    cudaSetDevice(ctx->device);
    KV_CHECK(ctx, cudaMemcpyAsync(T1h, s->T1, sizeof(double) * s->ng * s->s1(),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    constexpr size_t HALF = (size_t)32 << 20;          // doubles per staging half
    if (ctx->hstage_bytes < 2 * HALF * sizeof(double)) {
        if (ctx->hstage) cudaFreeHost(ctx->hstage);
        ctx->hstage = nullptr;
        ctx->hstage_bytes = 0;
        KV_CHECK(ctx, cudaHostAlloc(&ctx->hstage, 2 * HALF * sizeof(double),
                                    cudaHostAllocMapped));
        ctx->hstage_bytes = 2 * HALF * sizeof(double);
    }
    double *hs = (double *)ctx->hstage;
    double *ds = nullptr;
    KV_CHECK(ctx, cudaHostGetDevicePointer((void **)&ds, ctx->hstage, 0));
    const int h = (s->spin_on && s->spin_half > 0 && s->nv == s->no) ? s->spin_half : 0;
    const bool sparse = dst_zeroed && h > 0;
    const long long P = s->s2(), n = s->no, hh = (long long)h * h;
    // chunks: whole items of the spin order, or plain ranges of T2
    const long long per = sparse ? (long long)(HALF / hh) : (long long)HALF;
    const long long total = sparse ? (long long)s->ng * 6 * hh : (long long)s->ng * P;
    const long long nch = (total + per - 1) / per;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int st = KVFT_OK;
    for (int q = 0; q < 2 && st == KVFT_OK; q++)
        if (cudaEventCreateWithFlags(&ev[q], cudaEventDisableTiming) != cudaSuccess)
            st = kv_fail(ctx, KVFT_EDEVICE, "read_amplitudes: event");
    auto fill = [&](long long k) -> int {
        const long long c0 = k * per, cnt = std::min(per, total - c0);
        double *dst = ds + (k % 2) * HALF;
        if (sparse) {
            const long long el = cnt * hh;
            const int grid = (int)std::min<long long>((el + 255) / 256, (long long)ctx->sm_count * 8);
            amp_gather_kernel<<<grid, 256, 0, ctx->stream>>>(s->T2, P, (int)n, h, c0, cnt, dst);
            KV_TRY(kv_launch_check(ctx, "amp_gather"));
        } else {
            KV_CHECK(ctx, cudaMemcpyAsync(dst, s->T2 + c0, sizeof(double) * cnt,
                                          cudaMemcpyDeviceToHost, ctx->stream));
        }
        KV_CHECK(ctx, cudaEventRecord(ev[k % 2], ctx->stream));
        return KVFT_OK;
    };
    if (st == KVFT_OK && nch > 0) st = fill(0);
    for (long long k = 0; k < nch && st == KVFT_OK; k++) {
        if (k + 1 < nch) st = fill(k + 1);     // the other half was drained at k - 1
        if (st != KVFT_OK) break;
        if (cudaEventSynchronize(ev[k % 2]) != cudaSuccess) {
            st = kv_fail(ctx, KVFT_EDEVICE, "read_amplitudes: device copy failed");
            break;
        }
        const double *src = hs + (k % 2) * HALF;
        const long long c0 = k * per, cnt = std::min(per, total - c0);
        if (sparse) {
            host_parallel(cnt, [&](long long lo, long long hi) {
                for (long long it = lo; it < hi; it++) {
                    double *d = T2h + spin_item_base(c0 + it, P, (int)n, h);
                    const double *q = src + it * hh;
                    for (int i1 = 0; i1 < h; i1++)
                        std::memcpy(d + (long long)i1 * n, q + (long long)i1 * h,
                                    sizeof(double) * h);
                }
            });
        } else {
            host_parallel(cnt, [&](long long lo, long long hi) {
                std::memcpy(T2h + c0 + lo, src + lo, sizeof(double) * (hi - lo));
            });
        }
    }
    if (st == KVFT_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        st = kv_fail(ctx, KVFT_EDEVICE, "read_amplitudes: T1 copy failed");
    for (int q = 0; q < 2; q++)
        if (ev[q]) cudaEventDestroy(ev[q]);
    return st;
}

int kvft_solver_set_amplitudes(kvft_solver *s, const double *T1h, const double *T2h) {
    if (!s || !T1h || !T2h) return KVFT_EINVAL;
    KV_CHECK(s->ctx, cudaMemcpyAsync(s->T1, T1h, sizeof(double) * s->ng * s->s1(),
                                     cudaMemcpyHostToDevice, s->ctx->stream));
    KV_CHECK(s->ctx, cudaMemcpyAsync(s->T2, T2h, sizeof(double) * s->ng * s->s2(),
                                     cudaMemcpyHostToDevice, s->ctx->stream));
    s->norms_valid = false;
    s->aa_k = 0;
    if (s->spin_half && s->spin_on) {
        // amplitudes from outside keep the spin blocks only if they conserve spin
        const double *arr[2] = {s->T1, s->T2};
        const int rank[2] = {2, 4};
        const long long batch[2] = {s->ng, s->ng};
        int yes = 0;
        KV_TRY(spin_blocked(s->ctx, s->nv, s->spin_half, 2, arr, rank, batch, &yes));
        if (!yes) s->spin_on = false;
    }
    return KVFT_OK;
}

// Lambda on the solver's resident integrals and amplitudes: the guess
// (guess 1: Kelvin's, 2: its unrestricted driver's; 0: L1/L2 already hold
// one), then the resident damped iteration; L1/L2 are device buffers.  The
// orbital energies are the solver's or, for the explicit-denominator form,
// read off D1 (ev[a] = D1[a,0], eo[i] = D1[0,0] - D1[0,i]).
namespace {

int solver_energies(kvft_solver *s, const double **ev, const double **eo) {
    if (s->eps) {
        *ev = *eo = s->eps;
        return KVFT_OK;
    }
    const int nv = s->nv, no = s->no;
    std::vector<double> d1((size_t)nv * no), h((size_t)nv + no);
    KV_CHECK(s->ctx, cudaMemcpy(d1.data(), s->D1, sizeof(double) * d1.size(),
                                cudaMemcpyDeviceToHost));
    for (int a = 0; a < nv; a++) h[a] = d1[(size_t)a * no];
    for (int i = 0; i < no; i++) h[nv + i] = d1[0] - d1[i];
    // the backward integral needs D1 of that form (a block-diagonal D1 with
    // zeros between spin cases is not).  The rebuilt h[a] - h[nv+i] carries
    // rounding of the size of the largest |D1|, so the bar is relative to
    // that maximum, not to the element (the test of energies_from_d1)
    double dmax = 0.0;
    for (double d : d1) dmax = std::max(dmax, std::fabs(d));
    for (int a = 0; a < nv; a++)
        for (int i = 0; i < no; i++) {
            const double d = d1[(size_t)a * no + i], r = h[a] - h[nv + i];
            if (std::fabs(d - r) > 1e-12 * (1.0 + dmax))
                return kv_fail(s->ctx, KVFT_EINVAL,
                               "solver_lambda: D1 is not a difference of orbital energies");
        }
    void *p = nullptr;
    KV_TRY(kv_scratch(s->ctx, "solver_energies", sizeof(double) * h.size(), &p));
    KV_CHECK(s->ctx, cudaMemcpy(p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    *ev = (const double *)p;
    *eo = (const double *)p + nv;
    return KVFT_OK;
}

struct LamSpinScope {
    kvft_ctx *ctx;
    int prev;
    LamSpinScope(kvft_ctx *c, int h) : ctx(c), prev(c->lam_spin) { c->lam_spin = h; }
    ~LamSpinScope() { ctx->lam_spin = prev; }
};

}  // namespace

int kvft_solver_lambda(kvft_solver *s, int guess, double damp, double tconv, int max_iter,
                       int measure_half, double *L1, double *L2, double *hist, int *iters) {
    if (!s || !L1 || !L2 || !iters || guess < 0 || guess > 2)
        return kv_fail(s ? s->ctx : nullptr, KVFT_EINVAL, "solver_lambda: bad argument");
    // the backward integral is the adjoint of Kelvin's lower-triangular one
    if (s->full) return kv_fail(s->ctx, KVFT_EINVAL, "solver_lambda: not on a dense-G grid");
    cudaSetDevice(s->ctx->device);
    const double *ev = nullptr, *eo = nullptr;
    KV_TRY(solver_energies(s, &ev, &eo));
    LamSpinScope spin(s->ctx, (s->spin_half > 0 && s->spin_on) ? s->spin_half : 0);
    const double *F[4] = {s->F[0], s->F[1], s->F[2], s->F[3]};
    const double *I[9];
    for (int k = 0; k < 9; k++) I[k] = s->I[k];
    if (guess)
        KV_TRY(kvft_lambda_guess(s->ctx, s->ng, s->nv, s->no, F, I, s->T1, s->beta, guess == 2,
                                 L1, L2));
    return kvft_lambda_solve(s->ctx, s->ng, s->nv, s->no, F, I, s->T1, s->T2, ev, eo, s->ti,
                             s->g, s->G, damp, tconv, max_iter, measure_half, L1, L2, hist,
                             iters);
}

int kvft_solver_lambda_densities(kvft_solver *s, const double *L1, const double *L2,
                                 double *const Fg[4], double *const Ig[9]) {
    if (!s || !L1 || !L2 || !Fg || !Ig)
        return kv_fail(s ? s->ctx : nullptr, KVFT_EINVAL, "solver_lambda_densities: bad argument");
    if (s->full) return kv_fail(s->ctx, KVFT_EINVAL, "solver_lambda_densities: not on a dense-G grid");
    cudaSetDevice(s->ctx->device);
    const double *ev = nullptr, *eo = nullptr;
    KV_TRY(solver_energies(s, &ev, &eo));
    LamSpinScope spin(s->ctx, (s->spin_half > 0 && s->spin_on) ? s->spin_half : 0);
    const double *F[4] = {s->F[0], s->F[1], s->F[2], s->F[3]};
    const double *I[9];
    for (int k = 0; k < 9; k++) I[k] = s->I[k];
    return kvft_lambda_densities(s->ctx, s->ng, s->nv, s->no, F, I, s->T1, s->T2, L1, L2, ev,
                                 eo, s->ti, s->g, s->G, Fg, Ig);
}

// Anderson depth m (0: Kelvin's damped update).  The FP32 history (2m + 1
// arrays of the amplitudes' size) is allocated here, and the tau chunk is
// sized again for the memory that is left.
int kvft_solver_set_acceleration(kvft_solver *s, int m) {
    if (!s || m < 0 || m > 3) return kv_fail(s ? s->ctx : nullptr, KVFT_EINVAL,
                                             "solver_set_acceleration: depth must be 0..3");
    if (s->pending) return kv_fail(s->ctx, KVFT_EINVAL, "solver_set_acceleration: a step is pending");
    cudaSetDevice(s->ctx->device);
    KV_TRY(aa_alloc(s, m));
    s->aa_m = m;
    s->aa_k = 0;
    return KVFT_OK;
}

// CUDA graphs for the damped iteration: on = 1 / 0, -1 leaves it; *state
// (may be NULL): 2 when a captured graph is being replayed, -1 when a capture
// failed (the solver then runs eagerly), 0 otherwise.
int kvft_solver_set_graph(kvft_solver *s, int on, int *state) {
    if (!s || on < -1 || on > 1) return kv_fail(s ? s->ctx : nullptr, KVFT_EINVAL,
                                                "solver_set_graph: bad argument");
    if (on >= 0) {
        s->graph_on = on;
        if (!on && s->gexec) {
            cudaSetDevice(s->ctx->device);
            cudaStreamSynchronize(s->ctx->stream);
            cudaGraphExecDestroy(s->gexec);
            s->gexec = nullptr;
        }
        if (on && s->graph_state < 0) s->graph_state = 0;
    }
    if (state) *state = s->gexec ? 2 : s->graph_state < 0 ? -1 : 0;
    return KVFT_OK;
}

int kvft_solver_set_spin_blocks(kvft_solver *s, int on, int *half) {
    if (!s) return KVFT_EINVAL;
    if (on >= 0) s->spin_on = on != 0;
    if (half) *half = s->spin_on ? s->spin_half : 0;
    return KVFT_OK;
}

int kvft_solver_device_amplitudes(kvft_solver *s, double **T1, double **T2) {
    if (!s) return KVFT_EINVAL;
    if (T1) *T1 = s->T1;
    if (T2) *T2 = s->T2;
    return KVFT_OK;
}

// Fermi-scaled blocks from device eps[n], fock[n][n], eri[n]^4 into device
// F[4] (n x n each) and I[9] (n^4 each): kelvin/cc_utils.py:569-602.
int kvft_ft_integrals(kvft_ctx *ctx, int n, const double *eps, const double *fock,
                      const double *eri, double beta, double mu, double *const F[4],
                      double *const I[9]) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_ft_integrals: not on a dry-run context");
    if (!ctx || n <= 0 || !eps || !fock || !eri || !F || !I || !(beta > 0.0))
        return kv_fail(ctx, KVFT_EINVAL, "ft_integrals: bad argument");
    cudaSetDevice(ctx->device);
    void *sf = nullptr;
    KV_TRY(kv_scratch(ctx, "fermi_sqrt", sizeof(double) * 2 * n, &sf));
    double *sfo = (double *)sf, *sfv = sfo + n;
    fermi_kernel<<<1, 256, 0, ctx->stream>>>(n, beta, mu, eps, sfo, sfv);
    KV_TRY(kv_launch_check(ctx, "fermi"));
    const size_t n2 = (size_t)n * n;
    int gb = (int)std::max<size_t>(1, std::min<size_t>((n2 + 255) / 256, 1024));
    scale_fock_kernel<<<gb, 256, 0, ctx->stream>>>(n, fock, eps, sfo, sfv, F[0], F[1], F[2],
                                                   F[3]);
    KV_TRY(kv_launch_check(ctx, "scale_fock"));
    Blk9 b;
    for (int k = 0; k < 9; k++) b.p[k] = I[k];
    scale_eri_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(n, eri, sfo, sfv, b);
    return kv_launch_check(ctx, "scale_eri");
}

// One CCSD update for all tau points (ft_cc_equations.ccsd_stanton).
int kvft_ccsd_stanton(kvft_ctx *ctx, int ng, int nv, int no, const double *const F[4],
                      const double *const I[9], const double *T1old, const double *T2old,
                      const double *D1, const double *D2, const double *ti, const double *G,
                      int full, double *T1new, double *T2new) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_ccsd_stanton: not on a dry-run context");
    if (!ctx || ng < 1 || ng > 64 || nv <= 0 || no <= 0 || !F || !I || !T1old || !T2old ||
        !D1 || !D2 || !ti || !G || !T1new || !T2new)
        return kv_fail(ctx, KVFT_EINVAL, "ccsd_stanton: bad argument");
    cudaSetDevice(ctx->device);
    const long long s1 = (long long)nv * no, s2 = s1 * s1;
    void *tb = nullptr;
    KV_TRY(kv_scratch(ctx, "stanton_tbar", sizeof(double) * ng * (s1 + s2), &tb));
    double *T1b = (double *)tb, *T2b = T1b + ng * s1;
    // spin blocks: used when the integrals and the amplitudes given are all
    // spin-blocked (alpha half first); tbar's zero blocks are then cleared
    // here, since the residual does not write them and the integration reads
    // every element
    int sh = 0;
    if (nv == no && nv % 2 == 0) {
        const double *arr[15];
        int rank[15];
        long long bat[15];
        for (int k = 0; k < 4; k++) arr[k] = F[k], rank[k] = 2, bat[k] = 1;
        for (int k = 0; k < 9; k++) arr[4 + k] = I[k], rank[4 + k] = 4, bat[4 + k] = 1;
        arr[13] = T1old, rank[13] = 2, bat[13] = ng;
        arr[14] = T2old, rank[14] = 4, bat[14] = ng;
        int yes = 0;
        KV_TRY(spin_blocked(ctx, nv, nv / 2, 15, arr, rank, bat, &yes));
        if (yes) sh = nv / 2;
    }
    if (sh) KV_CHECK(ctx, cudaMemsetAsync(T2b, 0, sizeof(double) * ng * s2, ctx->stream));
    KvSpinScope spins(ctx, sh);
    KV_TRY(seed_neg(ctx, ng, s1, F[2], T1b));
    size_t fr = 0, tot = 0;
    KV_CHECK(ctx, cudaMemGetInfo(&fr, &tot));
    size_t held = 0;
    for (auto &kv : ctx->scratch) held += kv.second.second;
    size_t per = kv_chunk_bytes_per_tau(ctx, nv, no);
    int chunk = (int)std::max<long long>(
        1, std::min<long long>(ng, (long long)(0.6 * (double)(fr + held) / per)));
    for (int y0 = 0; y0 < ng; y0 += chunk) {
        int nb = std::min(chunk, ng - y0);
        KV_TRY(kv_stanton(ctx, nb, nv, no, F, I, T1old + y0 * s1, T2old + y0 * s2, -1.0,
                          T1b + y0 * s1, T2b + y0 * s2, I[3]));
    }
    KV_TRY(kvft_int_tbar1(ctx, ng, nv, no, T1b, ti, D1, G, full, T1new));
    return kvft_int_tbar2(ctx, ng, nv, no, T2b, ti, D2, G, full, T2new);
}

}  // extern "C"
