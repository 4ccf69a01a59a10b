/*
 * kvft -- GB300-native finite-temperature CCSD amplitude iteration.
 *
 * C ABI of libkvft.so.  Plain pointers and sizes only.  Unless a name ends in
 * "_host", array arguments are DEVICE pointers (allocate them with kvft_alloc
 * or any CUDA allocator on the context's device); "_host" variants take host
 * pointers and copy in/out on the context's stream.  All arrays are C-ordered
 * float64 with Kelvin's index order:
 *     T1[ng][nv][no]          (t_i^a at tau point y is T1[y][a][i])
 *     T2[ng][nv][nv][no][no]  (t_ij^ab)
 *     F blocks oo[no][no], ov[no][nv], vo[nv][no], vv[nv][nv]
 *     I blocks <pq||rs> with the block's o/v letters, e.g. oovv[i][j][a][b]
 *
 * Every call returns a kvft_status.  Errors never abort the process; the
 * message of the last failure on a context is kvft_last_error(ctx).
 * A context owns one CUDA stream; calls on one context are not thread-safe,
 * calls on different contexts are.
 */
#ifndef KVFT_H
#define KVFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    KVFT_OK = 0,
    KVFT_EINVAL = 1,    /* bad argument (Kelvin raises Exception here) */
    KVFT_ENOMEM = 2,    /* device allocation failed */
    KVFT_EDIVERGE = 3,  /* non-finite energy or residual */
    KVFT_ETIMEOUT = 4,  /* a bounded device wait gave up */
    KVFT_EDEVICE = 5,   /* CUDA runtime error */
    KVFT_ENOTCONV = 6   /* iteration limit reached (Kelvin logs a warning) */
} kvft_status;

/* Arithmetic used for the n^6/n^5 contractions.  Quadrature, energy,
 * damping and norms are FP64 in every mode. */
typedef enum {
    KVFT_PREC_FP64 = 0,      /* FP64 FMA (SIMT) contractions */
    KVFT_PREC_FP64_TC = 1,   /* FP64-accurate: digit-sliced BF16 tcgen05 GEMM */
    KVFT_PREC_MIXED = 2      /* few-digit BF16 tcgen05 GEMM, FP32-level */
} kvft_precision;

typedef struct kvft_ctx kvft_ctx;
typedef struct kvft_solver kvft_solver;

/* ---- context, memory, timing ------------------------------------------ */
int kvft_ctx_create(int device, void *stream, kvft_ctx **out);
int kvft_ctx_destroy(kvft_ctx *ctx);
const char *kvft_last_error(const kvft_ctx *ctx);
const char *kvft_status_string(int status);
int kvft_set_precision(kvft_ctx *ctx, int precision, int digits);
int kvft_alloc(kvft_ctx *ctx, size_t bytes, void **dptr);
int kvft_free(kvft_ctx *ctx, void *dptr);
int kvft_h2d(kvft_ctx *ctx, void *dst, const void *src, size_t bytes);
int kvft_d2h(kvft_ctx *ctx, void *dst, const void *src, size_t bytes);
int kvft_memset(kvft_ctx *ctx, void *dptr, int value, size_t bytes);
int kvft_sync(kvft_ctx *ctx);
int kvft_event_record(kvft_ctx *ctx, int slot);            /* slot < 64 */
int kvft_event_elapsed_ms(kvft_ctx *ctx, int s0, int s1, float *ms);
int kvft_launch_count(kvft_ctx *ctx, uint64_t *count);     /* own kernels */
int kvft_flush_l2(kvft_ctx *ctx);                          /* writes 256 MB */
/* Free and total device memory of the context's device (cudaMemGetInfo). */
int kvft_mem_info(kvft_ctx *ctx, size_t *free_bytes, size_t *total_bytes);
/* Cap on the tau-chunk workspace of solvers on this context (bytes; 0: the
 * default, 60% of the free device memory), so that several resident solvers
 * share one device. */
int kvft_set_workspace_limit(kvft_ctx *ctx, size_t bytes);

/* Live launch timing: between begin and end every library launch of the
 * categories below is bracketed by CUDA events on the context's stream.
 * work = algorithmic flops (GEMM categories) or bytes (the others). */
enum {
    KVFT_CAT_GEMM6 = 0,   /* n^6-class contractions (M, N, K all >= n^2) */
    KVFT_CAT_GEMM = 1,    /* the other contractions */
    KVFT_CAT_QUAD = 2,    /* tau integration (+ fused damping) */
    KVFT_CAT_ENERGY = 3,
    KVFT_CAT_ELEM = 4,    /* element-wise tensor passes */
    KVFT_CAT_PACK = 5     /* tensor-core operand packing */
};
/* Per category: launches, device milliseconds and algorithmic work --
 * flops for KVFT_CAT_GEMM6, bytes moved for every other category. */
typedef struct {
    uint64_t launches[6];
    double ms[6];
    double work[6];
} kvft_profile_stats;
int kvft_profile_begin(kvft_ctx *ctx);
int kvft_profile_end(kvft_ctx *ctx, kvft_profile_stats *out);
/* The timed scopes of the current profile one by one, in completion order
 * (a packing pass ends before the contraction that uses it): category,
 * device milliseconds and algorithmic work.  *count receives the number of
 * scopes; up to `max` are written.  Call before kvft_profile_end, which
 * discards them. */
int kvft_profile_records(kvft_ctx *ctx, int max, int *count, int *cat, float *ms,
                         double *work);
/* The GEMM shape (M, N, K, batch) behind each record of the current profile
 * (four ints per record; zeros for scopes that are not a contraction or its
 * operand packing).  Call before kvft_profile_end. */
int kvft_profile_shapes(kvft_ctx *ctx, int max, int *count, int *shapes);

/* ---- quadrature: replaces kelvin/quadrature.py:292-317 ------------------
 * out[y] = sum_x G[y][x] exp(dt D) tbar[x], dt = ti[x]-ti[y] for x < y and 0
 * otherwise (full != 0: for every x).  D has the shape of one tau slice
 * (D1[nv][no] / D2[nv][nv][no][no]); ti[ng], G[ng][ng]. */
int kvft_int_tbar1(kvft_ctx *ctx, int ng, int nv, int no, const double *t1bar,
                   const double *ti, const double *D1, const double *G,
                   int full, double *t1out);
int kvft_int_tbar2(kvft_ctx *ctx, int ng, int nv, int no, const double *t2bar,
                   const double *ti, const double *D2, const double *G,
                   int full, double *t2out);
/* single grid point ig: replaces quadrature.py:348-369 */
int kvft_int_tbar1_single(kvft_ctx *ctx, int ng, int ig, int nv, int no,
                          const double *t1bar, const double *ti,
                          const double *D1, const double *G, double *t1out);
int kvft_int_tbar2_single(kvft_ctx *ctx, int ng, int ig, int nv, int no,
                          const double *t2bar, const double *ti,
                          const double *D2, const double *G, double *t2out);

/* ---- energy: replaces kelvin/ft_cc_energy.py:7-32 -----------------------
 * omega_host receives (1/beta)[sum t1n.f + sum t2n.eri]; f = F.ov[no][nv],
 * eri = I.oovv[no][no][nv][nv], g[ng]. */
int kvft_ft_cc_energy(kvft_ctx *ctx, int ng, int nv, int no, const double *T1,
                      const double *T2, const double *f, const double *eri,
                      const double *g, double beta, int qterm,
                      double *omega_host);

/* ---- allocation-free energy (no counterpart in the reference) ------------
 * For callers that must not let a library allocate device memory (a host
 * whose memory pool owns the device, a latency-bound serving loop that cannot
 * absorb cudaMalloc's synchronisation, a plugin host that forbids foreign
 * allocations): the same value as kvft_ft_cc_energy, written to the DEVICE
 * double *omega_dev on `stream` (NULL: the legacy default stream; any stream
 * of the current device), with no context and no allocation.  Scratch is a
 * fixed 256 KiB static device array held by every GPU that loads the library
 * until exit.  The first call on a device looks up that array's address (do it
 * before any stream capture) and keeps it for the life of the process: after a
 * cudaDeviceReset that address is stale, so do not call this entry point on a
 * device that has been reset.  Calls share the array: calls that overlap on
 * the GPU race.  Limit: ceil(no*no/32) * ceil(nv*nv/32) <= 32767 tiles (up
 * to nv = no = 76); larger problems return KVFT_EINVAL without launching. */
int kvft_ft_cc_energy_noalloc(void *stream, int ng, int nv, int no,
                              const double *T1, const double *T2,
                              const double *f, const double *eri,
                              const double *g, double beta, int qterm,
                              double *omega_dev);

/* ---- CCSD update: replaces kelvin/ft_cc_equations.py:96-113 -------------
 * F[4] = {oo, ov, vo, vv}; I[9] = {vvvv, vvvo, vovv, vvoo, vovo, oovv, vooo,
 * ooov, oooo}.  T1new/T2new receive the integrated amplitudes. */
int kvft_ccsd_stanton(kvft_ctx *ctx, int ng, int nv, int no,
                      const double *const F[4], const double *const I[9],
                      const double *T1old, const double *T2old,
                      const double *D1, const double *D2, const double *ti,
                      const double *G, int full, double *T1new, double *T2new);
/* The tau-point residual alone (cqcpy _Stanton with fac, called at
 * ft_cc_equations.py:106-107): T1 += fac R1(t1,t2), T2 += fac R2, batched
 * over nb tau points. */
int kvft_stanton_residual(kvft_ctx *ctx, int nb, int nv, int no,
                          const double *const F[4], const double *const I[9],
                          const double *t1, const double *t2, double fac,
                          double *T1, double *T2);
/* Spin blocks of kvft_stanton_residual and kvft_ccsd_stanton (the blocking a
 * solver finds and uses by itself, kvft_solver_set_spin_blocks): half = h > 0
 * asserts that the integrals and amplitudes vanish outside the
 * spin-conserving blocks of an alpha-first layout with nv = no = 2h, so that
 * the residual's contractions run over their nonzero spin-block products
 * only; 0 turns it off (the default).  Calls whose nv, no are not 2h ignore
 * it. */
int kvft_set_residual_spin_blocks(kvft_ctx *ctx, int half);
/* Lambda terms (cqcpy _Lambda_opt, called at ft_cc_equations.py:400-401):
 * g = R'(t)^T m, the transpose of the residual's Jacobian at (t1, t2) applied
 * to m, batched over nb tau points, so that
 *   sum g1 dt1 + 1/4 sum g2 dt2 = sum m1 dR1 + 1/4 sum m2 dR2
 * for every dt1 and antisymmetric dt2.  m1[i][a], m2[i][j][a][b] are in
 * Lambda layout, g1[a][i], g2[a][b][i][j] in amplitude layout (device
 * pointers; F, I as for kvft_stanton_residual). */
int kvft_lambda_residual(kvft_ctx *ctx, int nb, int nv, int no,
                         const double *const F[4], const double *const I[9],
                         const double *t1, const double *t2, const double *m1,
                         const double *m2, double *g1, double *g2);
/* One Lambda update (kelvin/ft_cc_equations.py:385-409 ccsd_lambda_opt):
 * Lint = int_L(L_old) (quadrature.py:320-345), then per tau point
 *   L1 = -F.ov - I.oovv T1 - R1'^T Lint,  L2 = -I.oovv - R2'^T Lint
 * (the terms of kvft_lambda_residual, transposed to Lambda layout).
 * L1[ng][no][nv], L2[ng][no][no][nv][nv]; ev/eo are the orbital energies of
 * the virtual / occupied indices (D1 = ev - eo); ti, g, G the grid.  Device
 * pointers; L1/L2 may alias L1old/L2old. */
int kvft_ccsd_lambda(kvft_ctx *ctx, int ng, int nv, int no,
                     const double *const F[4], const double *const I[9],
                     const double *T1, const double *T2, const double *L1old,
                     const double *L2old, const double *ev, const double *eo,
                     const double *ti, const double *g, const double *G, double *L1,
                     double *L2);
/* Integral gradients of the Lagrangian at converged T and Lambda (the
 * ingredients of Kelvin's response densities, ft_cc_equations.py:704-753):
 *   Fg[b], Ig[b] = sum_y g_y d/d(block) [E(T_y) + <int_L(L)_y, F.vo + I.vvoo
 *                  + R(T_y)>]
 * in each block's own layout (F: oo ov vo vv, I as for kvft_ccsd_lambda).
 * Inputs as for kvft_ccsd_lambda; device pointers. */
int kvft_lambda_densities(kvft_ctx *ctx, int ng, int nv, int no,
                          const double *const F[4], const double *const I[9],
                          const double *T1, const double *T2, const double *L1,
                          const double *L2, const double *ev, const double *eo,
                          const double *ti, const double *g, const double *G,
                          double *const Fg[4], double *const Ig[9]);
/* Kelvin's damped Lambda iteration (cc_utils.py:414-480) resident on the
 * device: L1/L2 hold the guess on entry and the result on return; each
 * iteration is one kvft_ccsd_lambda update, damping and Kelvin's residual
 * (over the spin cases of an alpha-first layout when spin_half > 0, as its
 * unrestricted driver measures, cc_utils.py:482-560).  Stops when the
 * residual drops below tconv or after max_iter; hist (host, may be NULL)
 * receives the residual of each iteration, *iters their count. */
int kvft_lambda_solve(kvft_ctx *ctx, int ng, int nv, int no,
                      const double *const F[4], const double *const I[9],
                      const double *T1, const double *T2, const double *ev,
                      const double *eo, const double *ti, const double *g,
                      const double *G, double damp, double tconv, int max_iter,
                      int spin_half, double *L1, double *L2, double *hist, int *iters);
/* Kelvin's starting Lambda (ft_cc_equations.py:502-512): L1 = F.ov/beta +
 * I.oovv T1/beta, L2 = I.oovv/beta at every tau point; unrestricted != 0
 * drops the 1/beta of the T1 term as Kelvin's unrestricted guess does
 * (:515-526).  Device pointers. */
int kvft_lambda_guess(kvft_ctx *ctx, int ng, int nv, int no,
                      const double *const F[4], const double *const I[9],
                      const double *T1, double beta, int unrestricted, double *L1,
                      double *L2);
/* Spin blocks of the Lambda path (kvft_lambda_residual, kvft_ccsd_lambda,
 * kvft_lambda_solve, kvft_lambda_densities): half = h > 0 asserts that every
 * operand vanishes outside the spin-conserving blocks of an alpha-first
 * layout with nv = no = 2h, so that each contraction runs over its nonzero
 * spin-block products only; 0 turns it off (the default). */
int kvft_set_lambda_spin_blocks(kvft_ctx *ctx, int half);
/* The strided-GEMM form of an index-string contraction C[cix] = A[aix] B[bix]
 * (letters a-h virtual, i-n occupied; every letter in exactly two of the
 * three): mnk = {M, N, K}; sizes/strides hold the composite indices (three
 * components each, slow to fast) of A rows, A columns, B rows, B columns, C
 * rows, C columns.  Host arithmetic only. */
int kvft_einsum_plan(int nv, int no, const char *aix, const char *bix,
                     const char *cix, int *mnk, int *sizes, long long *strides);

/* ---- dry run ---------------------------------------------------------------
 * A context without a device whose calls record their launches (the
 * descriptors each kernel would receive) instead of running them; pointers
 * passed to it are host memory and its scratch is host memory filled with
 * NaN.  Lets the index arithmetic of a call be replayed and checked on a
 * CPU.  kvft_lambda_residual, kvft_ccsd_lambda, kvft_lambda_solve,
 * kvft_lambda_guess and kvft_lambda_densities accept it; every other call
 * that would touch the device returns KVFT_EINVAL.  Destroy it with
 * kvft_ctx_destroy. */
int kvft_dryrun_create(int precision, int digits, kvft_ctx **ctx);
int kvft_dryrun_count(const kvft_ctx *ctx, int *count);
/* op i: ints[32], longs[32], dbls[2], ptrs[11]; kind 0 contraction (M N K
 * batch, alpha, beta, A B C views), 1 strided axpby (dims, strides, src,
 * dst), 2 tau integral (ng, P, rank, full, nv, no; tbar, out, ti, G, eps
 * pair), 3 scale of a view, 4 sum of squares (dims, strides of the two
 * operands, a and b, result word).  Layout in kvft_ctx.cu. */
int kvft_dryrun_op(const kvft_ctx *ctx, int i, int *ints, long long *longs,
                   double *dbls, const void **ptrs);
/* scratch buffer i of a dry-run context (KVFT_EINVAL past the last one) */
int kvft_dryrun_scratch(const kvft_ctx *ctx, int i, const void **ptr, size_t *bytes);

/* ---- contraction engine: the GEMM under every einsum of the path --------
 * (Kelvin's pyscf.lib.einsum -> BLAS dgemm).  C[b] = A[b] B[b] for `batch`
 * consecutive row-major matrices A[M][K], B[K][N], C[M][N] (device).
 * precision KVFT_PREC_FP64 uses FP64 FMAs; the tensor-core precisions use
 * `digits` BF16 digit levels (7: FP64-accurate, 3..5: mixed). */
int kvft_gemm(kvft_ctx *ctx, int M, int N, int K, int batch, int precision,
              int digits, const double *A, const double *B, double *C);

/* ---- Fermi-scaled integrals: replaces kelvin/cc_utils.py:569-602 ---------
 * eps[n], fock[n][n] (System.g_fock_tot), eri[n]^4 (System.g_aint_tot) and
 * the outputs F[4] (n x n), I[9] (n^4) are device pointers. */
int kvft_ft_integrals(kvft_ctx *ctx, int n, const double *eps,
                      const double *fock, const double *eri, double beta,
                      double mu, double *const F[4], double *const I[9]);

/* ---- model-system integrals on the device: replace the n^4 loops of
 * kelvin/ueg_utils.py:83-138 (UEG) and kelvin/hubbard_system.py (1D Hubbard
 * ring in the momentum basis) behind System.g_aint_tot -------------------
 * Write the antisymmetrised spin-orbital <pq||rs> (general-spin order: nb
 * alpha orbitals, then nb beta) into the device array eri[n][n][n][n],
 * n = 2 nb.
 * kvft_ueg_eri: nvec[nb][3] (host) integer plane-wave vectors, c = 4 pi / L^3
 *   * (2 pi / L)^-2; <pq|rs> = c / |n_p - n_r|^2 for equal spins p,r and q,s,
 *   n_p + n_q = n_r + n_s, n_p != n_r.  nb <= 512.
 * kvft_hubbard_eri: `sites` momenta, u = U / sites; <pq|rs> = u for opposite
 *   spins (p,r alpha and q,s beta or the reverse) and k_p + k_q = k_r + k_s
 *   (mod sites). */
int kvft_ueg_eri(kvft_ctx *ctx, int nb, const int *nvec, double c, double *eri);
int kvft_hubbard_eri(kvft_ctx *ctx, int sites, double u, double *eri);

/* ---- device-resident solver: replaces kelvin/ccsd.py:595-712 with
 * cc_utils.ft_integrals (569-602) and cc_utils.ft_cc_iter (111-173) -------
 * eps[n] orbital energies, fock[n][n] (System.g_fock_tot), eri[n][n][n][n]
 * (System.g_aint_tot): host or device pointers (unified addressing; a device
 * eri from kvft_ueg_eri / kvft_hubbard_eri skips the upload); grid ti/g/G
 * host pointers. */
typedef struct {
    double econv;     /* |dE| threshold */
    double tconv;     /* res1+res2 threshold */
    double damp;      /* alpha in T_old = alpha T_old + (1-alpha) T */
    int max_iter;
    int full;         /* dense-G exponential convention */
    int guess;        /* 0: zero amplitudes, 1: Kelvin's first-order guess,
                         2: the amplitudes currently held (warm start) */
    int verbose;
} kvft_solve_opts;

typedef struct {
    double omega_cc;  /* Gcc */
    double e_guess;   /* energy of the initial amplitudes, Qterm = false */
    double res;       /* last res1 + res2 */
    int iterations;
    int converged;
} kvft_result;

int kvft_solver_create(kvft_ctx *ctx, int n, int ng, const double *eps,
                       const double *fock, const double *eri, double beta,
                       double mu, const double *ti, const double *g,
                       const double *G, kvft_solver **out);
/* Solver over given Fermi-scaled blocks and explicit denominators (host
 * pointers), the inputs of kelvin/cc_utils.py:111 ft_cc_iter. */
int kvft_solver_create_blocks(kvft_ctx *ctx, int nv, int no, int ng,
                              const double *const F[4],
                              const double *const I[9], const double *D1,
                              const double *D2, double beta, const double *ti,
                              const double *g, const double *G,
                              kvft_solver **out);
int kvft_solver_destroy(kvft_solver *s);
int kvft_solver_run(kvft_solver *s, const kvft_solve_opts *opts,
                    kvft_result *res);
/* Kelvin's tau-pointwise schedule (rt_iter = "point"; cc_utils.py:176-242):
 * converge grid point by grid point from a linear extrapolation, then
 * res->omega_cc = ft_cc_energy of the result.  Uses opts damp, tconv,
 * max_iter (per point). */
int kvft_solver_run_point(kvft_solver *s, const kvft_solve_opts *opts,
                          kvft_result *res);
/* one amplitude iteration (update + damping + norms + energy) */
int kvft_solver_step(kvft_solver *s, double damp, double *energy,
                     double *res);
/* The same iteration split in two: _begin queues it on the context's stream
 * and returns at once; _end waits for it and returns the energy and residual.
 * Solvers on different contexts (streams) overlap on the device between the
 * two calls; one step may be pending per solver. */
int kvft_solver_step_begin(kvft_solver *s, double damp);
int kvft_solver_step_end(kvft_solver *s, double *energy, double *res);
int kvft_solver_get_amplitudes(kvft_solver *s, double *T1_host,
                               double *T2_host);
/* The same read-back through the context's pinned staging buffer (2 x 256
 * MiB, allocated on first use and kept), with the host-side copy spread over
 * the host's threads.  dst_zeroed = 1 promises that T2_host holds zeros (a
 * fresh calloc): with spin blocks only the spin-conserving elements are
 * copied and the pages of the rest are never touched.  Replaces the host
 * arrays Kelvin's solve leaves in ccsd.T1 / ccsd.T2 (kelvin/ccsd.py:704-712). */
int kvft_solver_read_amplitudes(kvft_solver *s, double *T1_host, double *T2_host,
                                int dst_zeroed);
int kvft_solver_set_amplitudes(kvft_solver *s, const double *T1_host,
                               const double *T2_host);
/* Device pointers of the solver's resident amplitudes (T1, T2). */
int kvft_solver_device_amplitudes(kvft_solver *s, double **T1, double **T2);
/* Spin blocks.  When n is even and every integral block vanishes outside the
 * spin-conserving blocks with the alpha spin orbitals first (the general-spin
 * ordering of the UEG and Hubbard systems), the solver finds this at creation
 * and runs the n^6 contractions over the 10 nonzero spin-block products of
 * 64.  on = 0 turns that off, 1 back on, -1 leaves it; *half (may be NULL)
 * receives the alpha-half size in use (0: off).  Amplitudes given through
 * kvft_solver_set_amplitudes that do not conserve spin turn it off; writes
 * through kvft_solver_device_amplitudes are the caller's to keep
 * spin-conserving. */
int kvft_solver_set_spin_blocks(kvft_solver *s, int on, int *half);
/* Acceleration of the amplitude iteration (no counterpart in Kelvin, whose
 * loop is the damped update of cc_utils.py:131-173): m = 1..3 replaces the
 * damped update x <- x + (1 - damp)(Phi(x) - x) by Anderson mixing of depth m
 * with the same mixing factor, over an FP32 history of 2m + 1
 * amplitude-sized arrays allocated here (the tau chunk is re-sized for the
 * memory left); m = 0 restores Kelvin's update (the default).  Kelvin's
 * residual measure and convergence test apply to the accelerated iterates;
 * the fixed point is the same.  The history restarts when the contraction
 * precision changes, after a guess or new amplitudes, and when the residual
 * grows a hundredfold in one step. */
int kvft_solver_set_acceleration(kvft_solver *s, int m);
/* CUDA graphs for the damped iteration (no counterpart in Kelvin): on = 1
 * runs one eager step with the current settings, captures the next step's
 * launches into a graph and replays it from then on (launch overhead of the
 * several hundred launches of an iteration goes away, which matters for
 * small systems); a change of damping, precision, spin blocks, grid
 * convention or of any scratch buffer starts over.  A capture that fails
 * leaves the solver eager.  Profiling (kvft_profile_begin) and Anderson
 * acceleration run eagerly.  on = 0 turns it off, -1 leaves it; *state (may
 * be NULL): 2 replaying, -1 a capture failed, 0 otherwise. */
int kvft_solver_set_graph(kvft_solver *s, int on, int *state);
/* Lambda on the solver's resident integrals and amplitudes (the converged T
 * of its last solve): guess 1 forms Kelvin's starting Lambda in L1/L2, 2 its
 * unrestricted driver's, 0 keeps the one given; then kvft_lambda_solve
 * (damp, tconv, max_iter, measure_half as there).  L1[ng][no][nv],
 * L2[ng][no][no][nv][nv] are device buffers; the solver's spin blocks carry
 * over to the Lambda contractions. */
int kvft_solver_lambda(kvft_solver *s, int guess, double damp, double tconv, int max_iter,
                       int measure_half, double *L1, double *L2, double *hist, int *iters);
/* kvft_lambda_densities on the solver's integrals and amplitudes. */
int kvft_solver_lambda_densities(kvft_solver *s, const double *L1, const double *L2,
                                 double *const Fg[4], double *const Ig[9]);
size_t kvft_solver_footprint(int n, int ng, int precision);

#ifdef __cplusplus
}
#endif
#endif /* KVFT_H */
