// FP64-accurate contractions on the 5th-generation tensor cores.
//
// GB300 issues ~2 FP64 FMAs per clock per SM but ~3600 BF16 MACs, so an FP64
// GEMM is rebuilt from exact BF16 digit products (an Ozaki-style error-free
// splitting):
//
//   * packing: every row r of A (and every column of B) is scaled by 2^-e_r
//     so that |y| < 1/2, then y = 2^-7 sum_{s=1..S} P_s with balanced base-128
//     digits P_s = d_s 2^-7(s-1), d_s in [-64, 64] -- exact in BF16.  The
//     digits are extracted with integer arithmetic from the FP64 bit pattern.
//   * products: A B = 2^(e_m + e_n - 14) sum_{s,t} P_s^A P_t^B.  Pair (s,t)
//     carries the weight 2^-7(s+t-2); pairs with s + t <= D are kept.  Each
//     digit product is an integer below 2^12 (times a power of two), so an
//     FP32 accumulator over K <= 2048 terms and two pairs is exact.
//     tcgen05.mma accumulates level 2 (pair 1,1), level 3 (pairs 1,2 2,1) and
//     level 4 in separate TMEM accumulators and levels >= 5 in a fourth one:
//     the tensor core's FP32 adds truncate, and keeping every merged term
//     2^-21 below the leading level holds their error under ~1e-13.
//   * epilogue: the accumulators are read from TMEM (tcgen05.ld),
//     combined in FP64, scaled by 2^(e_m + e_n - 14) alpha and added to the
//     FP64 output view.  K > 2048 is split into sequential launches.
// With D = 7 (21 pair products, six digits) the norm-wise relative error is
// ~1e-11, far inside the 1e-8 amplitude / 1e-10 Ha parity bounds; D = 3..5 is
// the mixed-precision form.
//
// Kernel: one CTA per 128x128 output tile and K chunk; warp 0 = TMA producer,
// warp 1 = MMA issuer (and TMEM owner), warps 2..5 = epilogue.  Operands are
// staged by TMA (64-byte swizzle, 32-element k-blocks, every digit plane of a
// k-block per pipeline stage).  Every mbarrier wait is bounded by
// %globaltimer; on expiry the kernel records an error word and unwinds.
#include "kvft_internal.h"

#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <mutex>

namespace {

constexpr int TM = 128, TN = 128, KB = 32;
constexpr int PLANE_BYTES = TM * KB * 2;      // one digit plane of a k-block: 8 KB
constexpr int MAXS = 6;
constexpr int KCHUNK = 2048;                  // exactness bound of the level-3 sum
constexpr int NTHREADS = 192;
constexpr unsigned long long WAIT_NS = 2000000000ull;   // 2 s per wait

struct TcParams {
    int M, N;             // output extent of this launch
    int kb_base;          // first k-block of this launch
    int chunk_kb;         // k-blocks per K chunk (exactness bound)
    int nkb_total;        // k-blocks of the padded K extent
    int nsplit;           // K chunks run side by side (grid z = batch * nsplit)
    int atomic;           // 1: chunks add into C with FP64 atomics
    int S, D, NS;         // digit planes, levels, pipeline stages
    int Mp, Np;           // rows per digit plane of A / B
    int a_batch_rows, b_batch_rows;   // row offset between batch entries (0: shared)
    const int *ea, *eb;   // row exponents of A / column exponents of B
    int ea_bst, eb_bst;
    double alpha, beta;
    int alpha_pow2;       // alpha = +-2^alpha_exp: folded into the exponent field
    int alpha_exp;
    unsigned long long alpha_sign;   // sign bit of alpha (FP64 position)
    KOut C;
    int *err;
};

// Knuth's error-free sum: s + e == a + b exactly (round-to-nearest FP32)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// FP64 value of x 2^k with sign flipped by `sgn`, built from the FP32 bit
// pattern (exact; FP32 subnormals, below 2^-126 of the accumulator, give 0)
__device__ __forceinline__ double f32_scaled(float x, int k, unsigned long long sgn) {
    const uint32_t u = __float_as_uint(x);
    const int E = (int)((u >> 23) & 0xFF);
    const int e64 = E - 127 + 1023 + k;
    if (E == 0 || e64 <= 0) return 0.0;
    const unsigned long long bits = (((unsigned long long)(u >> 31) << 63) ^ sgn) |
                                    ((unsigned long long)e64 << 52) |
                                    ((unsigned long long)(u & 0x7FFFFFu) << 29);
    return __longlong_as_double(bits);
}

// Raw row exponents are reduced with atomicMax into an array preset to
// 0x80808080 (below any binary exponent); exp_of turns a raw maximum into the
// packing exponent e_r = max + 2 (|x| 2^-e_r < 1/2), or 0 for an all-zero row.
constexpr int EXP_RAW_FLOOR = -1100;
__host__ __device__ __forceinline__ int exp_of(int raw) {
    return raw < EXP_RAW_FLOOR ? 0 : raw + 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false after WAIT_NS of wall time
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity) {
    if (mbar_try(a, parity)) return true;
    const unsigned long long t0 = gtime();
    while (true) {
        if (mbar_try(a, parity)) return true;
        if (gtime() - t0 > WAIT_NS) return false;
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

// UMMA shared-memory descriptor: K-major, 64-byte swizzle, 8-row groups 512 B apart
__device__ __forceinline__ uint64_t desc_sw64(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;              // leading byte offset (unused, K-major swizzled)
    d |= (uint64_t)(512 >> 4) << 32;     // stride byte offset
    d |= (uint64_t)1 << 46;              // descriptor version
    d |= (uint64_t)4 << 61;              // SWIZZLE_64B
    return d;
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, K-major A and B
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
        : "memory");
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

#define TMEM_LD32(taddr, r)                                                                   \
    asm volatile(                                                                             \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"   \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),              \
          "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),           \
          "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),       \
          "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),       \
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),       \
          "=r"(r[30]), "=r"(r[31])                                                          \
        : "r"(taddr))

#define TMEM_LD16(taddr, r)                                                                   \
    asm volatile(                                                                             \
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
        "%14,%15}, [%16];"                                                                    \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),              \
          "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),           \
          "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])                                  \
        : "r"(taddr))

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMEM accumulator of digit level l: levels 2, 3, 4 each have their own
// (exact sums); levels >= 5 share the fourth, 2^-21 below the leading level,
// so the truncating FP32 adds of the tensor core stay below 2^-45 relative.
__device__ __forceinline__ int level_acc(int l) { return l >= 5 ? 3 : l - 2; }
__host__ __device__ __forceinline__ int n_acc(int D) { return D >= 5 ? 4 : D - 1; }

__global__ void __launch_bounds__(NTHREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               TcParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.S, NS = p.NS;
    uint8_t *sA = smem;
    uint8_t *sB = smem + (size_t)NS * S * PLANE_BYTES;
    uint64_t *bars = (uint64_t *)(sB + (size_t)NS * S * PLANE_BYTES);
    uint64_t *full = bars, *empty = bars + NS, *accf = bars + 2 * NS;
    uint32_t *tmem_slot = (uint32_t *)(accf + 1);
    __shared__ int s_fail;
    __shared__ long long s_coff[4][16];   // epilogue: per-warp column offsets
    __shared__ int s_cexp[4][16];         // and column exponents

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int b = blockIdx.z / p.nsplit, split = blockIdx.z % p.nsplit;
    const int kb_begin = p.kb_base + split * p.chunk_kb;
    const int nkb = min(p.chunk_kb, p.nkb_total - kb_begin);
    // TMEM columns: one 128-column FP32 accumulator per level group, power of two
    const int nacc_used = n_acc(p.D);
    const uint32_t tcols = nacc_used == 1 ? 128u : (nacc_used == 2 ? 256u : 512u);

    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int i = 0; i < NS; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(accf), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(tcols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            const uint32_t bytes = 2u * S * PLANE_BYTES;
            const int ya = b * p.a_batch_rows, yb = b * p.b_batch_rows;
            int issued = 0;
            for (int kb = 0; kb < nkb; kb++) {
                const int st = kb % NS;
                const uint32_t ph = (kb / NS) & 1;
                if (!mbar_wait(smem_u32(&empty[st]), ph ^ 1)) {
                    atomicExch(p.err, 1);
                    s_fail = 1;
                    break;
                }
                if (s_fail) break;
                const uint32_t fb = smem_u32(&full[st]);
                mbar_expect_tx(fb, bytes);
                const int x = (kb_begin + kb) * KB;
                for (int s = 0; s < S; s++) {
                    tma_load_2d(smem_u32(sA + ((size_t)st * S + s) * PLANE_BYTES), &tmA, x,
                                ya + s * p.Mp + m0, fb);
                    tma_load_2d(smem_u32(sB + ((size_t)st * S + s) * PLANE_BYTES), &tmB, x,
                                yb + s * p.Np + n0, fb);
                }
                issued = kb + 1;
            }
            // drain: every issued stage must have landed before the CTA exits
            for (int kb = (issued > NS ? issued - NS : 0); kb < issued; kb++) {
                const int st = kb % NS;
                if (!mbar_wait(smem_u32(&full[st]), (kb / NS) & 1)) atomicExch(p.err, 2);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            bool started[4] = {false, false, false, false};
            bool ok = true;
            for (int kb = 0; kb < nkb; kb++) {
                const int st = kb % NS;
                if (!mbar_wait(smem_u32(&full[st]), (kb / NS) & 1)) {
                    atomicExch(p.err, 3);
                    s_fail = 1;
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t a0 = smem_u32(sA + (size_t)st * S * PLANE_BYTES);
                const uint32_t b0 = smem_u32(sB + (size_t)st * S * PLANE_BYTES);
                for (int l = 2; l <= p.D; l++) {
                    const int acc = level_acc(l);
                    for (int s = 1; s < l; s++) {
                        const int t = l - s;
                        if (s > S || t > S) continue;
                        for (int kk = 0; kk < KB / 16; kk++) {
                            const uint64_t da = desc_sw64(a0 + (s - 1) * PLANE_BYTES + kk * 32);
                            const uint64_t db = desc_sw64(b0 + (t - 1) * PLANE_BYTES + kk * 32);
                            umma(tmem + acc * TN, da, db, started[acc] ? 1u : 0u);
                            started[acc] = true;
                        }
                    }
                }
                umma_commit(smem_u32(&empty[st]));
            }
            if (ok) umma_commit(smem_u32(accf));
        }
    } else {
        // ---- epilogue: warps 2..5, TMEM lane quadrant = warp % 4 ----
        const int q = warp % 4;
        const int row = q * 32 + lane;
        const bool okw = __all_sync(0xffffffffu, mbar_wait(smem_u32(accf), 0));
        if (!okw && lane == 0) atomicExch(p.err, 4);
        fence_after();
        __syncwarp();
        if (okw && !s_fail) {
            // GB300's FP64 pipe is ~1/1500 of its BF16 tensor rate, so the
            // levels are combined with error-free FP32 two-sums and the FP64
            // result is assembled from bit patterns, the scale
            // 2^(e_m + e_n - 14) (and a power-of-two alpha) going straight into
            // the exponent field: at most two FP64 operations per element.
            const int m = m0 + row;
            const int nacc = n_acc(p.D);
            const int ew = warp - 2;
            const int em = (m < p.M) ? exp_of(p.ea[(long long)b * p.ea_bst + m]) : 0;
            const int krow = em - 14 + p.alpha_exp;
            double *Cb = p.C.p + (long long)b * p.C.bst;
            const long long roff = (m < p.M) ? p.C.r.off(m) : 0;
            for (int c = 0; c < TN / 16; c++) {
                if (lane < 16) {
                    const int n = n0 + c * 16 + lane;
                    s_coff[ew][lane] = (n < p.N) ? p.C.c.off(n) : 0;
                    s_cexp[ew][lane] = (n < p.N) ? exp_of(p.eb[(long long)b * p.eb_bst + n]) : 0;
                }
                uint32_t r0[16], r1[16], r2[16], r3[16];
                const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + c * 16;
                TMEM_LD16(tbase, r0);
                if (nacc > 1) TMEM_LD16(tbase + TN, r1);
                if (nacc > 2) TMEM_LD16(tbase + 2 * TN, r2);
                if (nacc > 3) TMEM_LD16(tbase + 3 * TN, r3);
                tmem_wait_ld();
                __syncwarp();
                if (m < p.M) {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const int n = n0 + c * 16 + j;
                        if (n >= p.N) continue;
                        float hi = __uint_as_float(r0[j]), lo = 0.f, e = 0.f;
                        if (nacc > 1) two_sum(hi, __uint_as_float(r1[j]), hi, lo);
                        if (nacc > 2) {
                            two_sum(hi, __uint_as_float(r2[j]), hi, e);
                            lo += e;
                        }
                        if (nacc > 3) lo += __uint_as_float(r3[j]);
                        const int k = krow + s_cexp[ew][j];
                        double v = f32_scaled(hi, k, p.alpha_sign) + f32_scaled(lo, k, p.alpha_sign);
                        if (!p.alpha_pow2) v *= p.alpha;
                        double *dst = Cb + roff + s_coff[ew][j];
                        if (p.atomic) atomicAdd(dst, v);
                        else if (p.beta == 0.0) *dst = v;
                        else if (p.beta == 1.0) *dst += v;
                        else *dst = fma(p.beta, *dst, v);
                    }
                }
                __syncwarp();
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Digit packing: FP64 strided view (rows x K) -> S BF16 planes [b][s][Rp][Kp]
// and row exponents [b][Rp].
// ---------------------------------------------------------------------------
struct PackView {
    const double *p;
    KIdx r, c;
    long long bst;
};

// Operand tiles of 32 rows x 64 k go through shared memory so that global
// reads are coalesced along whichever operand index is contiguous in memory
// (the row index for some permuted views, k for others) and plane writes are
// coalesced along k.
constexpr int PT_R = 32, PT_K = 64;

__device__ __forceinline__ void load_tile(const PackView &v, int b, int r0, int k0, int R, int K,
                                          bool rows_fast,
                                          unsigned long long (*tile)[PT_K + 1]) {
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const double *base = v.p + (long long)b * v.bst;
    if (rows_fast) {
        const int row = r0 + tx;
        const long long ro = (row < R) ? v.r.off(row) : 0;
        for (int kk = ty; kk < PT_K; kk += 8) {
            const int k = k0 + kk;
            tile[tx][kk] =
                (row < R && k < K) ? (unsigned long long)__double_as_longlong(base[ro + v.c.off(k)])
                                   : 0ull;
        }
    } else {
        for (int rr = ty; rr < PT_R; rr += 8) {
            const int row = r0 + rr;
            const long long ro = (row < R) ? v.r.off(row) : 0;
            for (int h = 0; h < 2; h++) {
                const int k = k0 + tx + 32 * h;
                tile[rr][tx + 32 * h] =
                    (row < R && k < K)
                        ? (unsigned long long)__double_as_longlong(base[ro + v.c.off(k)])
                        : 0ull;
            }
        }
    }
}

// raw row exponents: max binary exponent over each tile row, atomicMax'ed
__global__ void __launch_bounds__(256)
pack_exp_kernel(PackView v, int R, int K, int rows_fast, int *__restrict__ ex) {
    __shared__ unsigned long long tile[PT_R][PT_K + 1];
    const int b = blockIdx.z, r0 = blockIdx.y * PT_R, k0 = blockIdx.x * PT_K;
    load_tile(v, b, r0, k0, R, K, rows_fast, tile);
    __syncthreads();
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    for (int rr = w; rr < PT_R; rr += 8) {
        int emax = -2000;
        for (int h = 0; h < 2; h++) {
            const unsigned long long bits = tile[rr][lane + 32 * h];
            if ((bits & 0x7FFFFFFFFFFFFFFFull) != 0)
                emax = max(emax, (int)((bits >> 52) & 0x7FF) - 1023);
        }
        for (int o = 16; o > 0; o >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        const int row = r0 + rr;
        if (lane == 0 && emax > -2000 && row < R) atomicMax(&ex[(long long)b * R + row], emax);
    }
}

// Balanced base-128 digits of x 2^-e (|x 2^-e| < 1/2), most significant
// first, from the FP64 bit pattern with integer arithmetic only.
__device__ __forceinline__ void digits_of(unsigned long long bits, int e, int S, int *d) {
    for (int s = 0; s < MAXS; s++) d[s] = 0;
    const int be = (int)((bits >> 52) & 0x7FF);
    if (be == 0) return;                        // zero / subnormal (< 2^-1022): zero
    const long long mant = (long long)((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52));
    // |x| 2^-e 2^(7S) = mant 2^(be - 1023 - 52 - e + 7S), rounded to an integer
    const int sh = be - 1023 - 52 - e + 7 * S;
    long long Y;
    if (sh >= 0) Y = mant << sh;
    else if (sh > -63) Y = (mant + (1ll << (-sh - 1))) >> (-sh);
    else Y = 0;
    // digits in [-64, 63], least significant first; the top one takes the
    // remainder, which is in [0, 64]
    for (int s = S - 1; s >= 1; s--) {
        int dd = (int)(Y & 127);
        if (dd >= 64) dd -= 128;
        d[s] = dd;
        Y = (Y - dd) >> 7;
    }
    d[0] = (int)Y;
    if (bits >> 63)
        for (int s = 0; s < S; s++) d[s] = -d[s];
}

// planes[b][s][row][k] (row stride ld) = d_s 2^-7s; each thread packs two k
template <int S>
__global__ void __launch_bounds__(256)
pack_digits_kernel(PackView v, int R, int K, int ld, int rows_fast, const int *__restrict__ ex,
                   __nv_bfloat16 *__restrict__ out) {
    __shared__ unsigned long long tile[PT_R][PT_K + 1];
    const int b = blockIdx.z, r0 = blockIdx.y * PT_R, k0 = blockIdx.x * PT_K;
    load_tile(v, b, r0, k0, R, K, rows_fast, tile);
    __syncthreads();
    const size_t plane = (size_t)R * ld;
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int k = k0 + 2 * tx;
    if (k >= K) return;
    for (int rr = ty; rr < PT_R; rr += 8) {
        const int row = r0 + rr;
        if (row >= R) break;
        const int e = exp_of(ex[(long long)b * R + row]);
        int d0[MAXS], d1[MAXS];
        digits_of(tile[rr][2 * tx], e, S, d0);
        digits_of(tile[rr][2 * tx + 1], e, S, d1);    // zero beyond K (tile fill)
        __nv_bfloat16 *ob = out + (size_t)b * S * plane + (size_t)row * ld + k;
#pragma unroll
        for (int s = 0; s < S; s++) {
            __nv_bfloat162 w2;
            w2.x = __float2bfloat16_rn(ldexpf((float)d0[s], -7 * s));
            w2.y = __float2bfloat16_rn(ldexpf((float)d1[s], -7 * s));
            *reinterpret_cast<__nv_bfloat162 *>(ob + (size_t)s * plane) = w2;
        }
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

int make_map(kvft_ctx *ctx, CUtensorMap *map, void *base, int K, int ld, long long rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return kv_fail(ctx, KVFT_EDEVICE, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {KB, TM};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return kv_fail(ctx, KVFT_EDEVICE, "cuTensorMapEncodeTiled failed");
    return KVFT_OK;
}

struct Packed {
    __nv_bfloat16 *planes;
    int *ex;
    int R, ld, K, nb;
};

// Digit planes [nb][S][R][ld] (ld = K rounded up to 8 for the 16-byte TMA row
// stride) and exponents [nb][R].  No row or K padding is written: the tensor
// map's extent is (K, nb S R) and TMA fills out-of-range boxes with zeros;
// rows past R inside a 128-row box belong to the next plane and only reach
// output rows/columns that the epilogue discards.
int pack(kvft_ctx *ctx, const char *key, const PackView &v, int R, int K, int nb, int S,
         Packed *out) {
    const int ld = (K + 7) / 8 * 8;
    const size_t plane_bytes = (size_t)R * ld * 2;
    const size_t pbytes = ((size_t)nb * S * plane_bytes + 1023) / 1024 * 1024;
    const size_t bytes = pbytes + (size_t)nb * R * sizeof(int);
    void *buf = nullptr;
    KV_TRY(kv_scratch(ctx, key, bytes, &buf));
    out->planes = (__nv_bfloat16 *)buf;
    out->ex = (int *)((uint8_t *)buf + pbytes);
    out->R = R;
    out->ld = ld;
    out->K = K;
    out->nb = nb;
    if (nb > 65535) return kv_fail(ctx, KVFT_EINVAL, "pack: batch too large");
    KvProfScope prof(ctx, KV_CAT_PACK, 8.0 * nb * (double)R * K + (double)nb * S * plane_bytes);
    KV_CHECK(ctx, cudaMemsetAsync(out->ex, 0x80, (size_t)nb * R * sizeof(int), ctx->stream));
    // coalesce global reads along the contiguous index
    const int rows_fast = (v.r.st[2] == 1 && v.c.st[2] != 1) ? 1 : 0;
    const long long rtiles = (R + PT_R - 1) / PT_R;
    if (rtiles > 65535) return kv_fail(ctx, KVFT_EINVAL, "pack: too many rows");
    const dim3 g((K + PT_K - 1) / PT_K, (unsigned)rtiles, nb);
    pack_exp_kernel<<<g, 256, 0, ctx->stream>>>(v, R, K, rows_fast, out->ex);
    KV_TRY(kv_launch_check(ctx, "pack_exp"));
    switch (S) {
#define KV_PACK_CASE(s_)                                                                    \
    case s_:                                                                                \
        pack_digits_kernel<s_><<<g, 256, 0, ctx->stream>>>(v, R, K, ld, rows_fast, out->ex, \
                                                           out->planes);                    \
        break;
        KV_PACK_CASE(1) KV_PACK_CASE(2) KV_PACK_CASE(3) KV_PACK_CASE(4) KV_PACK_CASE(5)
        KV_PACK_CASE(6)
#undef KV_PACK_CASE
    default: return kv_fail(ctx, KVFT_EINVAL, "pack: digit count out of range");
    }
    KV_TRY(kv_launch_check(ctx, "pack_digits"));
    return KVFT_OK;
}

size_t tc_smem(int S, int NS) { return 1024 + (size_t)2 * NS * S * PLANE_BYTES + 8 * (2 * NS + 2) + 64; }

}  // namespace

int kv_gemm_tc(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha, const KMat &A,
               const KMat &B, double beta, const KOut &C, int digits) {
    const int D = digits;
    const int S = std::min(D - 1, MAXS);
    if (D < 2 || D > MAXS + 1) return kv_fail(ctx, KVFT_EINVAL, "tensor-core digits out of range");
    if (M <= 0 || N <= 0 || batch <= 0) return KVFT_OK;
    if (K <= 0) return kv_gemm_f64(ctx, M, N, K, batch, alpha, A, B, beta, C);
    if (M < N) {
        // C^T = B^T A^T: the larger extent goes to the 128 TMEM lanes, which are
        // the epilogue's rows (a small M would leave most epilogue warps idle)
        const KMat At{B.p, B.c, B.r, B.bst};
        const KMat Bt{A.p, A.c, A.r, A.bst};
        const KOut Ct{C.p, C.c, C.r, C.bst};
        return kv_gemm_tc(ctx, N, M, K, batch, alpha, At, Bt, beta, Ct, digits);
    }
    const int nbA = A.bst ? batch : 1, nbB = B.bst ? batch : 1;
    Packed pa, pb;
    KV_TRY(pack(ctx, "tc_pack_a", PackView{A.p, A.r, A.c, A.bst}, M, K, nbA, S, &pa));
    // B is K x N; its K-major form has rows = N (B's column index), cols = K
    KV_TRY(pack(ctx, "tc_pack_b", PackView{B.p, B.c, B.r, B.bst}, N, K, nbB, S, &pb));
    CUtensorMap ma, mb;
    KV_TRY(make_map(ctx, &ma, pa.planes, pa.K, pa.ld, (long long)nbA * S * pa.R));
    KV_TRY(make_map(ctx, &mb, pb.planes, pb.K, pb.ld, (long long)nbB * S * pb.R));
    int NS = 2;
    while (NS < 6 && tc_smem(S, NS + 1) <= 225 * 1024) NS++;
    const size_t smem = tc_smem(S, NS);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             225 * 1024);
        attr = true;
    }
    if (batch > 65535) return kv_fail(ctx, KVFT_EINVAL, "tensor-core gemm: batch too large");
    const int mt = (M + TM - 1) / TM, nt = (N + TN - 1) / TN;
    const int nkb_total = (K + KB - 1) / KB;
    const int nchunks = (nkb_total + KCHUNK / KB - 1) / (KCHUNK / KB);
    const int chunk_kb = (nkb_total + nchunks - 1) / nchunks;     // balanced chunks
    const long long tiles = (long long)mt * nt * batch;
    // few output tiles and several K chunks: run the chunks side by side and
    // add them into C with FP64 atomics (C pre-scaled by beta)
    const bool par = nchunks > 1 && tiles < 2LL * ctx->sm_count &&
                     (long long)batch * nchunks <= 65535;
    if (par && beta != 1.0) KV_TRY(kv_scale_view(ctx, M, N, batch, beta, C));
    TcParams p;
    p.M = M;
    p.N = N;
    p.chunk_kb = chunk_kb;
    p.nkb_total = nkb_total;
    p.S = S;
    p.D = D;
    p.NS = NS;
    p.Mp = pa.R;
    p.Np = pb.R;
    p.a_batch_rows = (nbA > 1) ? S * pa.R : 0;
    p.b_batch_rows = (nbB > 1) ? S * pb.R : 0;
    p.ea = pa.ex;
    p.eb = pb.ex;
    p.ea_bst = (nbA > 1) ? pa.R : 0;
    p.eb_bst = (nbB > 1) ? pb.R : 0;
    p.alpha = alpha;
    {
        int ex2 = 0;
        const double fr = std::frexp(alpha, &ex2);
        p.alpha_pow2 = (std::fabs(fr) == 0.5) ? 1 : 0;
        p.alpha_exp = p.alpha_pow2 ? ex2 - 1 : 0;
        p.alpha_sign = (p.alpha_pow2 && alpha < 0) ? (1ull << 63) : 0ull;
    }
    p.C = C;
    p.err = ctx->dflag;
    if (par) {
        p.kb_base = 0;
        p.nsplit = nchunks;
        p.atomic = 1;
        p.beta = 1.0;
        dim3 grid(nt, mt, batch * nchunks);
        tc_gemm_kernel<<<grid, NTHREADS, smem, ctx->stream>>>(ma, mb, p);
        return kv_launch_check(ctx, "tc_gemm");
    }
    p.nsplit = 1;
    p.atomic = 0;
    dim3 grid(nt, mt, batch);
    for (int c = 0; c < nchunks; c++) {
        p.kb_base = c * chunk_kb;
        p.beta = (c == 0) ? beta : 1.0;
        tc_gemm_kernel<<<grid, NTHREADS, smem, ctx->stream>>>(ma, mb, p);
        KV_TRY(kv_launch_check(ctx, "tc_gemm"));
    }
    return KVFT_OK;
}

// Device status word written by bounded waits (0 = fine).
int kv_device_status(kvft_ctx *ctx) {
    int h = 0;
    KV_CHECK(ctx, cudaMemcpyAsync(&h, ctx->dflag, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h != 0) {
        cudaMemsetAsync(ctx->dflag, 0, sizeof(int), ctx->stream);
        return kv_fail(ctx, KVFT_ETIMEOUT,
                       "tensor-core GEMM: a bounded device wait expired (code " +
                           std::to_string(h) + ")");
    }
    return KVFT_OK;
}

// Plain row-major GEMM through the selected engine (test and measurement hook):
// C[M][N] = A[M][K] B[K][N] for `batch` consecutive matrices, device pointers.
extern "C" int kvft_gemm(kvft_ctx *ctx, int M, int N, int K, int batch, int precision,
                         int digits, const double *A, const double *B, double *C) {
    if (!ctx || M <= 0 || N <= 0 || K <= 0 || batch <= 0 || !A || !B || !C)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_gemm: bad argument");
    cudaSetDevice(ctx->device);
    KMat a{A, kidx1(M, K), kidx1(K, 1), (long long)M * K};
    KMat b{B, kidx1(K, N), kidx1(N, 1), (long long)K * N};
    KOut c{C, kidx1(M, N), kidx1(N, 1), (long long)M * N};
    int st;
    if (precision == KVFT_PREC_FP64)
        st = kv_gemm_f64(ctx, M, N, K, batch, 1.0, a, b, 0.0, c);
    else
        st = kv_gemm_tc(ctx, M, N, K, batch, 1.0, a, b, 0.0, c, digits);
    if (st != KVFT_OK) return st;
    return kv_device_status(ctx);
}
