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
//     Every level l = s + t has its own TMEM accumulator, at column
//     (l - 2) TN of the set, and the digit planes of a B tile lie one after
//     another in shared memory, so a single tcgen05.mma of A plane s against
//     B planes t0..t0+k-1 (N = k TN <= 256) adds each product into its own
//     level: 8 MMAs per 16-deep k-step for D = 7 instead of 21 pair MMAs,
//     which keeps the tensor core's shared-memory reads of A below the SM's
//     shared-memory bandwidth.
//   * epilogue: the accumulators are read from TMEM (tcgen05.ld), the K
//     chunks (K > 2048) are summed in registers, and the tile is scaled by
//     2^(e_m + e_n - 14) alpha and written to the FP64 output view once.
// With D = 7 (21 pair products, six digits) the norm-wise relative error is
// ~1e-11, far inside the 1e-8 amplitude / 1e-10 Ha parity bounds; D = 3..5 is
// the mixed-precision form.
//
// Kernel: persistent, one CTA per SM walking output tiles; warp 0 = TMA
// producer, warp 1 = MMA issuer (and TMEM owner), warps 2..9 = epilogue; the
// epilogue of one tile overlaps the MMAs of the next.  Operands are staged by
// TMA (64-byte swizzle, 32-element k-blocks, every digit plane of a k-block
// per pipeline stage).  Every mbarrier wait is bounded by %globaltimer; on
// expiry the kernel records an error word and unwinds.
#include "kvft_internal.h"

#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace {

constexpr int TM = 128;
constexpr int MAXS = 6;
constexpr int KCHUNK = 2048;                  // exactness bound of the level-3 sum
constexpr int NEPI = 8;                       // epilogue warps: two per TMEM lane quadrant
constexpr int NTHREADS = 64 + 32 * NEPI;      // + TMA producer warp + MMA warp
constexpr int TMEM_COLS = 512;               // all of an SM's TMEM (one CTA per SM)
constexpr int GROUP_M = 8;                    // m-tiles per raster group (L2 reuse)
constexpr unsigned long long WAIT_NS = 2000000000ull;   // 2 s per wait

// x / d for 0 <= x < 2^31 by a multiply and a shift (Granlund-Montgomery:
// m = ceil(2^(31+l) / d) with 2^l >= d), in place of the ~20 instructions of
// an integer division by a run-time divisor in the per-tile index arithmetic.
struct FastDiv {
    unsigned long long m;
    int s;
    __device__ __forceinline__ int div(int x) const {
        return (int)(((unsigned long long)(unsigned)x * m) >> s);
    }
};
inline FastDiv fastdiv(int d) {
    int l = 0;
    while ((1LL << l) < d) l++;
    FastDiv f;
    f.s = 31 + l;
    f.m = ((1ULL << f.s) + (unsigned long long)d - 1) / (unsigned long long)d;
    return f;
}

struct TcParams {
    int M, N;             // output extent
    int mt, nt;           // output tiles along M and N
    int units;            // work units: mt * nt * batch * nsplit
    int nsplit;           // >1: each K chunk is its own unit, added into C by FP64 atomics
    int chunk_kb;         // k-blocks per K chunk (exactness bound)
    int nkb_total;        // k-blocks of the padded K extent
    int S, D, NS;         // digit planes, levels, pipeline stages
    int Mp, Np;           // rows per digit plane of A / B
    int a_batch_rows, b_batch_rows;   // row offset between batch entries (0: shared)
    const int *ea, *eb;   // row exponents of A / column exponents of B
    int ea_bst, eb_bst;
    double alpha, beta;
    int alpha_pow2;       // alpha = +-2^alpha_exp: folded into the exponent field
    int alpha_exp;
    unsigned alpha_sign;  // sign bit of alpha (bit 31 of the FP64 high word)
    KOut C;
    int *err;
    FastDiv dv_split, dv_perb, dv_gsz;    // nsplit, mt nt, GROUP_M nt
    FastDiv dv_cr2, dv_cr1;               // C's row index: sizes of its fast components
};

// A work unit: one output tile of one batch entry over a k-block range.
struct Unit {
    int b, m0, n0, kb0, kb1;
};

// Units are numbered split-fastest, then in raster groups of GROUP_M m-tiles
// (n-tiles walk inside a group), then by batch entry, so the CTAs that run
// at the same time share a few A row panels and sweep B once per group.
__device__ __forceinline__ Unit unit_of(const TcParams &p, int u, int tn) {
    static_assert(GROUP_M == 8, "raster groups of 8 m-tiles (shift and mask below)");
    Unit w;
    const int t = p.dv_split.div(u);
    const int split = u - t * p.nsplit;
    const int per_b = p.mt * p.nt;
    w.b = p.dv_perb.div(t);
    const int r = t - w.b * per_b;
    const int gsz = GROUP_M * p.nt;
    const int g = p.dv_gsz.div(r);
    const int first = g * GROUP_M;
    const int gm = min(GROUP_M, p.mt - first);
    const int rr = r - g * gsz;
    if (gm == GROUP_M) {
        w.m0 = (first + (rr & 7)) * TM;
        w.n0 = (rr >> 3) * tn;
    } else {                              // the last, short group
        w.m0 = (first + rr % gm) * TM;
        w.n0 = (rr / gm) * tn;
    }
    if (p.nsplit > 1) {
        w.kb0 = split * p.chunk_kb;
        w.kb1 = min(w.kb0 + p.chunk_kb, p.nkb_total);
    } else {
        w.kb0 = 0;
        w.kb1 = p.nkb_total;
    }
    return w;
}

// Knuth's error-free sum: s + e == a + b exactly (round-to-nearest FP32)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// FP64 value of x 2^k with sign flipped by `sgn` (0 or 0x80000000), built
// from the FP32 bit pattern in 32-bit halves: high word = sign | exponent
// E - 127 + 1023 + k | top 20 mantissa bits, low word = the other 3 mantissa
// bits at the top (exact; FP32 subnormals, below 2^-126 of the accumulator,
// give 0)
__device__ __forceinline__ double f32_scaled(float x, int k, unsigned sgn) {
    const uint32_t u = __float_as_uint(x);
    const int E = (int)((u >> 23) & 0xFF);
    const int e64 = E + (1023 - 127) + k;
    if (E == 0 || e64 <= 0) return 0.0;
    const uint32_t hi = ((u & 0x80000000u) ^ sgn) | ((uint32_t)e64 << 20) | ((u >> 3) & 0xFFFFFu);
    return __hiloint2double((int)hi, (int)(u << 29));
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

// UMMA shared-memory descriptor of a K-major operand tile whose rows are one
// k-block of KBT BF16 values: KBT = 32 -> 64-byte swizzle (8-row groups 512 B
// apart), KBT = 64 -> 128-byte swizzle (8-row groups 1024 B apart)
template <int KBT>
__device__ __forceinline__ uint64_t desc_of(uint32_t saddr) {
    static_assert(KBT == 32 || KBT == 64, "k-block of 32 or 64");
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;                         // leading byte offset (unused)
    d |= (uint64_t)((8 * KBT * 2) >> 4) << 32;      // stride byte offset
    d |= (uint64_t)1 << 46;                         // descriptor version
    d |= (uint64_t)(KBT == 32 ? 4 : 2) << 61;       // SWIZZLE_64B / SWIZZLE_128B
    return d;
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, K-major A and B,
// M = 128, N = tn
__host__ __device__ constexpr uint32_t idesc_of(int tn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(tn >> 3) << 17) |
           ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
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

#define TMEM_LD16(taddr, r)                                                                   \
    asm volatile(                                                                             \
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13," \
        "%14,%15}, [%16];"                                                                    \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),              \
          "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),           \
          "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])                                  \
        : "r"(taddr))

#define TMEM_LD8(taddr, r)                                                                    \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"     \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),     \
                   "=r"(r[6]), "=r"(r[7])                                                     \
                 : "r"(taddr))

#define TMEM_LD4(taddr, r)                                                                    \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"                 \
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])                             \
                 : "r"(taddr))

// 32 lanes x LW consecutive columns of TMEM
template <int LW>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t *r) {
    static_assert(LW == 16 || LW == 8 || LW == 4, "TMEM load width");
    if constexpr (LW == 16) {
        TMEM_LD16(taddr, r);
    } else if constexpr (LW == 8) {
        TMEM_LD8(taddr, r);
    } else {
        TMEM_LD4(taddr, r);
    }
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory bytes of the kernel: 1 KB alignment slack, NS pipeline stages
// (S digit planes of A and of B per stage), the barriers, the epilogue's
// per-warp column tables and two words (TMEM base, failure flag).
__host__ __device__ constexpr size_t tc_smem(int S, int NS, int tn, int kb) {
    return 1024 + (size_t)NS * S * (TM + tn) * kb * 2 + 8 * (2 * NS + 5) +
           (size_t)NEPI * (tn / 2) * 12 + 16;
}

// Persistent kernel: each CTA walks the units blockIdx.x, blockIdx.x +
// gridDim.x, ...; the stage ring and the TMEM accumulator sets run on across
// units, so TMA, tensor core and epilogue of different units overlap.
//
//   warp 0      TMA producer: all S digit planes of A and B of one k-block per
//               stage.
//   warp 1      TMEM owner and MMA issuer: the level products of K chunk c
//               (at most KCHUNK deep, so each level sum is exact in FP32) go
//               to accumulator set c % NSET; a commit marks the set full.
//   warps 2-9   epilogue: warp w reads TMEM lanes 32 (w % 4).. of column half
//               (w - 2) / 4, frees the set, and carries the sum over the
//               unit's K chunks in registers -- one FP32 value per element
//               when D <= 3 (the few-digit form), an unevaluated FP32 pair
//               (error-free two-sums) otherwise.  After the last chunk the
//               tile goes to C once: FP64 built from bit patterns with the
//               scale 2^(e_m + e_n - 14) (and a power-of-two alpha) in the
//               exponent field, old values of C loaded 8 at a time.
//
// D <= 3: TN = 128, two levels (256 columns) per set, two sets, so the MMAs
// of one chunk run while the epilogue drains the other.  D >= 4: TN = 64, up
// to six levels (384 columns), one set; the epilogue frees it as soon as the
// levels are in registers (a few percent of a chunk's MMA time), and writes
// the tile while the next chunk accumulates.
//
// DL (the digit levels D) is a template parameter: the MMA issue loop is then
// straight-line code whose descriptors are per-stage bases plus constant
// offsets, so the single issuing thread keeps up with the tensor core.
template <int TN, bool FF, int KBT, int DL>
__global__ void __launch_bounds__(NTHREADS, 1)
tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               TcParams p) {
    constexpr int SD = DL - 1 < MAXS ? DL - 1 : MAXS;   // digit planes
    constexpr int PLANE_BYTES = TM * KBT * 2;    // one digit plane of an A k-block
    constexpr int BPLANE = TN * KBT * 2;         // one digit plane of a B k-block
    constexpr int WCOLS = TN / 2;            // columns per epilogue warp
    constexpr int LW = FF ? 4 : 16;          // columns per TMEM load (<= 32 registers in flight)
    constexpr int NG = WCOLS / LW;           // TMEM loads per level
    constexpr int WG = 8;                    // columns per store group
    constexpr int MAXL = FF ? 6 : 2;         // levels per set
    constexpr int NSET = FF ? 1 : 2;         // accumulator sets
    constexpr int SET_COLS = MAXL * TN;      // 384 or 256 TMEM columns
    constexpr int PMAX = 256 / TN;           // B planes per MMA (N <= 256)
    static_assert(NSET * SET_COLS <= TMEM_COLS, "accumulator sets exceed TMEM");
    constexpr uint32_t IDESC = idesc_of(TN);
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int S = SD;
    const int NS = p.NS;
    constexpr uint32_t stage_a = S * PLANE_BYTES, stage_b = S * BPLANE;
    uint8_t *sA = smem;
    uint8_t *sB = smem + NS * stage_a;
    uint64_t *bars = (uint64_t *)(sB + NS * stage_b);
    uint64_t *full = bars, *empty = bars + NS;
    uint64_t *accf = bars + 2 * NS, *acce = accf + 2, *done = acce + 2;
    long long *s_coff = (long long *)(done + 1);            // [NEPI][WCOLS]
    int *s_cexp = (int *)(s_coff + NEPI * WCOLS);           // [NEPI][WCOLS]
    uint32_t *tmem_slot = (uint32_t *)(s_cexp + NEPI * WCOLS);
    volatile int *s_fail = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    if (threadIdx.x == 0) {
        *s_fail = 0;
        for (int i = 0; i < NS; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        for (int i = 0; i < NSET; i++) {
            mbar_init(smem_u32(&accf[i]), 1);
            mbar_init(smem_u32(&acce[i]), NEPI);
        }
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
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
            const uint32_t bytes = (uint32_t)(stage_a + stage_b);
            int st = 0, issued = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int u = blockIdx.x; u < p.units && ok; u += gridDim.x) {
                const Unit w = unit_of(p, u, TN);
                const int ya = w.b * p.a_batch_rows + w.m0, yb = w.b * p.b_batch_rows + w.n0;
                for (int kb = w.kb0; kb < w.kb1; kb++) {
                    if (!mbar_wait(smem_u32(&empty[st]), ph ^ 1) || *s_fail) {
                        atomicExch(p.err, 1);
                        *s_fail = 1;
                        ok = false;
                        break;
                    }
                    const uint32_t fb = smem_u32(&full[st]);
                    mbar_expect_tx(fb, bytes);
                    const int x = kb * KBT;
                    for (int s = 0; s < S; s++) {
                        tma_load_2d(smem_u32(sA + st * stage_a + s * PLANE_BYTES), &tmA, x,
                                    ya + s * p.Mp, fb);
                        tma_load_2d(smem_u32(sB + st * stage_b + s * BPLANE), &tmB, x,
                                    yb + s * p.Np, fb);
                    }
                    issued++;
                    if (++st == NS) {
                        st = 0;
                        ph ^= 1;
                    }
                }
            }
            // drain: every issued stage must have landed before the CTA exits
            for (int i = 0; i < min(issued, NS); i++) {
                if (st == 0) {
                    st = NS - 1;
                    ph ^= 1;
                } else {
                    st--;
                }
                if (!mbar_wait(smem_u32(&full[st]), ph)) atomicExch(p.err, 2);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            // descriptors of stage 0's first planes; a stage or plane offset
            // adds (offset >> 4) to the address field (all of shared memory
            // fits its 14 bits)
            const uint64_t dA0 = desc_of<KBT>(smem_u32(sA)), dB0 = desc_of<KBT>(smem_u32(sB));
            int st = 0, gc = 0;
            uint32_t ph = 0;
            bool ok = true;
            for (int u = blockIdx.x; u < p.units && ok; u += gridDim.x) {
                const Unit w = unit_of(p, u, TN);
                for (int c0 = w.kb0; c0 < w.kb1 && ok; c0 += p.chunk_kb) {
                    const int c1 = min(c0 + p.chunk_kb, w.kb1);
                    const int set = gc % NSET;
                    if (!mbar_wait(smem_u32(&acce[set]), ((gc / NSET) & 1) ^ 1) || *s_fail) {
                        atomicExch(p.err, 3);
                        *s_fail = 1;
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t tacc = tmem + set * SET_COLS;
                    for (int kb = c0; kb < c1; kb++) {
                        if (!mbar_wait(smem_u32(&full[st]), ph) || *s_fail) {
                            atomicExch(p.err, 4);
                            *s_fail = 1;
                            ok = false;
                            break;
                        }
                        fence_after();
                        // A plane s against B planes t0.. (adjacent in shared
                        // memory) into levels s + t0.. (adjacent in TMEM); the
                        // first k-step of a chunk starts every level (s = 1
                        // reaches all of them) and later ones accumulate
                        const uint64_t dA = dA0 + ((st * stage_a) >> 4);
                        const uint64_t dB = dB0 + ((st * stage_b) >> 4);
                        const uint32_t later = (kb > c0) ? 1u : 0u;
#pragma unroll
                        for (int kk = 0; kk < KBT / 16; kk++) {
#pragma unroll
                            for (int s = 1; s <= S; s++) {
                                if (s >= DL) continue;
                                const int tmax = min(S, DL - s);
                                const uint32_t acc = (kk > 0 || s > 1) ? 1u : later;
                                const uint64_t da = dA + (((s - 1) * PLANE_BYTES + kk * 32) >> 4);
#pragma unroll
                                for (int t0 = 1; t0 <= tmax; t0 += PMAX) {
                                    const int np = min(PMAX, tmax - t0 + 1);
                                    const uint64_t db =
                                        dB + (((t0 - 1) * BPLANE + kk * 32) >> 4);
                                    umma(tacc + (s + t0 - 2) * TN, da, db, idesc_of(np * TN),
                                         acc);
                                }
                            }
                        }
                        umma_commit(smem_u32(&empty[st]));
                        if (++st == NS) {
                            st = 0;
                            ph ^= 1;
                        }
                    }
                    if (!ok) break;
                    umma_commit(smem_u32(&accf[set]));
                    gc++;
                }
            }
            // every MMA issued by this thread completes before TMEM is freed
            umma_commit(smem_u32(done));
            if (!mbar_wait(smem_u32(done), 0)) atomicExch(p.err, 5);
        }
    } else {
        // ---- epilogue ----
        const int ew = warp - 2, q = warp & 3, h = ew >> 2;
        const int row = q * 32 + lane;
        constexpr int nl = DL - 1;                  // levels 2..D
        long long *coff = s_coff + ew * WCOLS;
        int *cexp = s_cexp + ew * WCOLS;
        float rhi[WCOLS];
        float rlo[FF ? WCOLS : 1];
        int gc = 0;
        bool ok = true;
        int cached_n = -1, cached_b = -1;   // the columns coff / cexp hold (warp-uniform)
        for (int u = blockIdx.x; u < p.units && ok; u += gridDim.x) {
            const Unit w = unit_of(p, u, TN);
            if (w.kb0 >= w.kb1) continue;
            // C addresses of this unit; for the read-modify-write of a
            // general beta the old values are prefetched into L2 now, while
            // the MMAs run, so that it is not bound by the few loads a warp
            // keeps in flight (the L2 reductions of beta = 1 fetch their lines
            // at L2 themselves: prefetching them too cost 6 of 82 ms per
            // 114-spin-orbital iteration in issue slots)
            const int nw = w.n0 + h * WCOLS;          // first column of this warp
            // column offsets and exponents: the same for every tile of this
            // column range (and batch entry, when B is per batch)
            const int bkey = p.eb_bst ? w.b : 0;
            if (nw != cached_n || bkey != cached_b) {
                __syncwarp();                            // the last tile's reads are done
                for (int i = lane; i < WCOLS; i += 32) {
                    const int n = nw + i;
                    coff[i] = (n < p.N) ? p.C.c.off(n) : 0;
                    cexp[i] = (n < p.N) ? exp_of(p.eb[(long long)bkey * p.eb_bst + n]) : 0;
                }
                cached_n = nw;
                cached_b = bkey;
            }
            __syncwarp();
            const int m = w.m0 + row;
            const int nlim = p.N - nw;
            long long roff = 0;
            if (m < p.M) {                               // p.C.r.off(m), fast divisions
                const int r1 = p.dv_cr2.div(m), i2 = m - r1 * p.C.r.size[2];
                const int i0 = p.dv_cr1.div(r1), i1 = r1 - i0 * p.C.r.size[1];
                roff = (long long)i0 * p.C.r.st[0] + (long long)i1 * p.C.r.st[1] +
                       (long long)i2 * p.C.r.st[2];
            }
            double *Cr = p.C.p + (long long)w.b * p.C.bst + roff;
            const int krow =
                (m < p.M) ? exp_of(p.ea[(long long)w.b * p.ea_bst + m]) - 14 + p.alpha_exp : 0;
            if (m < p.M && p.nsplit == 1 && p.beta != 0.0 && p.beta != 1.0) {
                for (int i = 0; i < min(WCOLS, nlim); i++)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(Cr + coff[i]));
            }
            for (int c0 = w.kb0; c0 < w.kb1; c0 += p.chunk_kb) {
                const int set = gc % NSET;
                const bool got = mbar_wait(smem_u32(&accf[set]), (gc / NSET) & 1);
                // one verdict per warp: tcgen05.ld below needs every lane
                if (__any_sync(0xffffffffu, !got || *s_fail)) {
                    if (lane == 0) {
                        atomicExch(p.err, 6);
                        *s_fail = 1;
                    }
                    ok = false;
                    break;
                }
                fence_after();
                const bool first = (c0 == w.kb0);
                const uint32_t tb =
                    tmem + ((uint32_t)(q * 32) << 16) + set * SET_COLS + h * WCOLS;
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    uint32_t r[MAXL][LW];
#pragma unroll
                    for (int l = 0; l < MAXL; l++)
                        if (l < nl) tmem_ld<LW>(tb + l * TN + g * LW, r[l]);
                    tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < LW; j++) {
                        const int i = g * LW + j;
                        float hi = __uint_as_float(r[0][j]);
                        if constexpr (!FF) {
                            if (nl > 1) hi += __uint_as_float(r[1][j]);
                            rhi[i] = first ? hi : rhi[i] + hi;
                        } else {
                            // exact level sums, leading first: an FP32 pair
                            float lo = 0.f, e;
#pragma unroll
                            for (int l = 1; l < MAXL; l++) {
                                if (l < nl) {
                                    two_sum(hi, __uint_as_float(r[l][j]), hi, e);
                                    lo += e;
                                }
                            }
                            if (first) {
                                rhi[i] = hi;
                                rlo[i] = lo;
                            } else {
                                float sm;
                                two_sum(rhi[i], hi, sm, e);
                                rlo[i] += lo + e;
                                rhi[i] = sm;
                            }
                        }
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&acce[set]));
                gc++;
            }
            if (!ok) break;
            // ---- the tile to C ----
            if (m < p.M) {
                // value of column i of this thread's row
                auto value = [&](int i) -> double {
                    const int k = krow + cexp[i];
                    double v = f32_scaled(rhi[i], k, p.alpha_sign);
                    if constexpr (FF) v += f32_scaled(rlo[i], k, p.alpha_sign);
                    if (!p.alpha_pow2) v *= p.alpha;
                    return v;
                };
                if (p.nsplit > 1 || p.beta == 1.0) {
                    // C += value: each element gets exactly one addition in
                    // this launch unless K chunks run as separate units, so a
                    // fire-and-forget reduction at L2 gives old + value
                    // rounded once, like a load-add-store, without the
                    // thread waiting for the old value (measured on the
                    // 114-spin-orbital n^5 class: 82 ms per iteration
                    // against 120 ms for the load-add-store ring below)
                    if constexpr (FF) {
                        if (p.alpha_pow2) {
                            // the FP32 pair as two reductions at L2: no FP64
                            // add on the SM (GB300's FP64 pipe bounded this
                            // write); C gets old + hi + lo in two roundings
#pragma unroll
                            for (int i = 0; i < WCOLS; i++) {
                                if (i < nlim) {
                                    const int k = krow + cexp[i];
                                    atomicAdd(Cr + coff[i], f32_scaled(rhi[i], k, p.alpha_sign));
                                    atomicAdd(Cr + coff[i], f32_scaled(rlo[i], k, p.alpha_sign));
                                }
                            }
                        } else {
#pragma unroll
                            for (int i = 0; i < WCOLS; i++)
                                if (i < nlim) atomicAdd(Cr + coff[i], value(i));
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < WCOLS; i++)
                            if (i < nlim) atomicAdd(Cr + coff[i], value(i));
                    }
                } else if (p.beta == 0.0) {
                    if (FF && p.alpha_pow2) {
                        // hi stored, lo added at L2: hi + lo rounded once,
                        // as the FP64 add gave, without it on the SM
#pragma unroll
                        for (int i = 0; i < WCOLS; i++) {
                            if (i < nlim) {
                                const int k = krow + cexp[i];
                                Cr[coff[i]] = f32_scaled(rhi[i], k, p.alpha_sign);
                                if constexpr (FF)
                                    atomicAdd(Cr + coff[i], f32_scaled(rlo[i], k, p.alpha_sign));
                            }
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < WCOLS; i++)
                            if (i < nlim) Cr[coff[i]] = value(i);
                    }
                } else {
                    // read-modify-write: the old values of the next RING
                    // groups of WG columns are in flight while one group is
                    // combined and stored
                    constexpr int NGW = WCOLS / WG, RING = FF ? 3 : 2;
                    double old[RING][WG];
#pragma unroll
                    for (int q = 0; q < RING; q++)
#pragma unroll
                        for (int j = 0; j < WG; j++)
                            old[q][j] = (q < NGW && q * WG + j < nlim) ? Cr[coff[q * WG + j]] : 0.0;
#pragma unroll
                    for (int g = 0; g < NGW; g++) {
                        const int q = g % RING;
#pragma unroll
                        for (int j = 0; j < WG; j++) {
                            const int i = g * WG + j;
                            const double v = (p.beta == 1.0) ? old[q][j] + value(i)
                                                             : fma(p.beta, old[q][j], value(i));
                            if (i < nlim) Cr[coff[i]] = v;
                        }
                        if (g + RING < NGW) {
#pragma unroll
                            for (int j = 0; j < WG; j++) {
                                const int i = (g + RING) * WG + j;
                                old[q][j] = (i < nlim) ? Cr[coff[i]] : 0.0;
                            }
                        }
                    }
                }
            }
            __syncwarp();
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS)
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
    int stable;         // contents fixed while the pack cache is on
};

// Operand tiles of 32 rows x 64 k go through shared memory so that global
// reads are coalesced along whichever operand index is contiguous in memory
// (the row index for some permuted views, k for others) and plane writes are
// coalesced along k.  The composite-index offsets of the tile's rows and k
// columns are computed once per tile (96 divisions instead of one per
// element) and kept in shared memory; -1 marks a row or column outside the
// view.
constexpr int PT_R = 32, PT_K = 64;

// The tile walk: offsets of tile rows r0.. and k columns k0.. in a shared
// table (threads 0-95), then each thread's 8 values -- row lane at k = w + 8 i
// (rows_fast), else rows w + 8 i at k = lane, lane + 32 -- loaded into
// registers, so a block can have the next tile's loads in flight while it
// works on the current one.
__device__ __forceinline__ void tile_offsets(const PackView &v, int r0, int k0, int R, int K,
                                             long long *off) {
    const int tid = threadIdx.x;
    if (tid < PT_R) {
        off[tid] = (r0 + tid < R) ? v.r.off(r0 + tid) : -1;
    } else if (tid < PT_R + PT_K) {
        const int k = k0 + tid - PT_R;
        off[tid] = (k < K) ? v.c.off(k) : -1;
    }
}

__device__ __forceinline__ void tile_fetch(const double *base, const long long *off,
                                           int rows_fast, unsigned long long (&pre)[8]) {
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    if (rows_fast) {
        const long long ro = off[lane];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const long long ko = off[PT_R + w + 8 * i];
            pre[i] = (ro >= 0 && ko >= 0)
                         ? (unsigned long long)__double_as_longlong(__ldg(base + ro + ko))
                         : 0ull;
        }
    } else {
        const long long ko0 = off[PT_R + lane], ko1 = off[PT_R + lane + 32];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const long long ro = off[w + 8 * i];
            pre[2 * i] = (ro >= 0 && ko0 >= 0)
                             ? (unsigned long long)__double_as_longlong(__ldg(base + ro + ko0))
                             : 0ull;
            pre[2 * i + 1] = (ro >= 0 && ko1 >= 0)
                                 ? (unsigned long long)__double_as_longlong(__ldg(base + ro + ko1))
                                 : 0ull;
        }
    }
}

__device__ __forceinline__ int raw_exp(unsigned long long bits) {
    return (bits & 0x7FFFFFFFFFFFFFFFull) ? (int)((bits >> 52) & 0x7FF) - 1023 : -2000;
}

// raw row exponents: max binary exponent over each row of `ktiles`
// consecutive 64-wide k tiles, one atomicMax per row and block.  The maxima
// are taken in registers from each thread's 8 values, and the next tile's
// loads are issued before the current tile's values are used.
__global__ void __launch_bounds__(256)
pack_exp_kernel(PackView v, int R, int K, int rows_fast, int ktiles, int *__restrict__ ex) {
    __shared__ long long off[PT_R + PT_K];
    __shared__ int rmax[8][PT_R];
    const int b = blockIdx.z, r0 = blockIdx.y * PT_R;
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const double *base = v.p + (long long)b * v.bst;
    const int kt0 = blockIdx.x * ktiles;
    const int nkt = min(ktiles, (K + PT_K - 1) / PT_K - kt0);
    // rows_fast: one row per thread (lane); otherwise four rows (w + 8 i)
    int em[4] = {-2000, -2000, -2000, -2000};
    unsigned long long pre[8];
    tile_offsets(v, r0, kt0 * PT_K, R, K, off);
    __syncthreads();
    tile_fetch(base, off, rows_fast, pre);
    for (int t = 0; t < nkt; t++) {
        unsigned long long cur[8];
#pragma unroll
        for (int i = 0; i < 8; i++) cur[i] = pre[i];
        if (t + 1 < nkt) {
            __syncthreads();                    // every thread has read the offsets
            tile_offsets(v, r0, (kt0 + t + 1) * PT_K, R, K, off);
            __syncthreads();
            tile_fetch(base, off, rows_fast, pre);
        }
        if (rows_fast) {
#pragma unroll
            for (int i = 0; i < 8; i++) em[0] = max(em[0], raw_exp(cur[i]));
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++)
                em[i] = max(em[i], max(raw_exp(cur[2 * i]), raw_exp(cur[2 * i + 1])));
        }
    }
    if (rows_fast) {
        // row lane: combine the eight warps' maxima
        rmax[w][lane] = em[0];
        __syncthreads();
        if (w == 0) {
            int e = rmax[0][lane];
#pragma unroll
            for (int q = 1; q < 8; q++) e = max(e, rmax[q][lane]);
            if (e > -2000 && r0 + lane < R) atomicMax(&ex[(long long)b * R + r0 + lane], e);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int e = em[i];
            for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
            const int row = r0 + w + 8 * i;
            if (lane == 0 && e > -2000 && row < R) atomicMax(&ex[(long long)b * R + row], e);
        }
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

// Up to three planes take at most 21 bits of |x| 2^-e 2^(7S): the shift
// right is at least 33, so those bits and the rounding bit all lie in the
// high word of the significand, and 32-bit arithmetic on it gives the digits
// of the 64-bit form above exactly (adding the rounding bit 2^(n+31) cannot
// carry out of bits the low word decides).
template <int S>
__device__ __forceinline__ void digits_of_s(unsigned long long bits, int e, int *d) {
    if (S > 3) {
        digits_of(bits, e, S, d);
        return;
    }
#pragma unroll
    for (int s = 0; s < S; s++) d[s] = 0;
    const unsigned hi = (unsigned)(bits >> 32);
    const int be = (int)((hi >> 20) & 0x7FF);
    if (be == 0) return;
    const int n = 52 + e - (be - 1023) - 7 * S - 32;      // >= 1 since e >= be - 1021
    unsigned Y = n < 22 ? (((hi & 0xFFFFFu) | 0x100000u) + (1u << (n - 1))) >> n : 0u;
#pragma unroll
    for (int s = S - 1; s >= 1; s--) {
        int dd = (int)(Y & 127u);
        if (dd >= 64) dd -= 128;
        d[s] = dd;
        Y = (unsigned)((int)Y - dd) >> 7;
    }
    d[0] = (int)Y;
    if (hi >> 31)
#pragma unroll
        for (int s = 0; s < S; s++) d[s] = -d[s];
}

// bf16 pair (d0 2^-7s, d1 2^-7s), |d| <= 64: the float 1.5 2^23 + d is formed
// by an integer add on its bit pattern and the offset is removed, with the
// scaling, by one exact FMA; one conversion then packs both values.
template <int s>
__device__ __forceinline__ __nv_bfloat162 digit_pair(int d0, int d1) {
    constexpr float sc = 1.0f / (float)(1ull << (7 * s));     // 2^-7s, exact
    const float f0 = fmaf(__int_as_float(0x4B400000 + d0), sc, -12582912.0f * sc);
    const float f1 = fmaf(__int_as_float(0x4B400000 + d1), sc, -12582912.0f * sc);
    return __floats2bfloat162_rn(f0, f1);
}

template <int S>
__device__ __forceinline__ void store_digits(__nv_bfloat16 *ob, size_t plane,
                                             unsigned long long x0, unsigned long long x1,
                                             int e) {
    int d0[MAXS], d1[MAXS];
    digits_of_s<S>(x0, e, d0);
    digits_of_s<S>(x1, e, d1);
    *reinterpret_cast<__nv_bfloat162 *>(ob) = digit_pair<0>(d0[0], d1[0]);
    if (S > 1) *reinterpret_cast<__nv_bfloat162 *>(ob + plane) = digit_pair<1>(d0[1], d1[1]);
    if (S > 2) *reinterpret_cast<__nv_bfloat162 *>(ob + 2 * plane) = digit_pair<2>(d0[2], d1[2]);
    if (S > 3) *reinterpret_cast<__nv_bfloat162 *>(ob + 3 * plane) = digit_pair<3>(d0[3], d1[3]);
    if (S > 4) *reinterpret_cast<__nv_bfloat162 *>(ob + 4 * plane) = digit_pair<4>(d0[4], d1[4]);
    if (S > 5) *reinterpret_cast<__nv_bfloat162 *>(ob + 5 * plane) = digit_pair<5>(d0[5], d1[5]);
}

// planes[b][s][row][k] (row stride ld) = d_s 2^-7s; each thread packs two k.
// Persistent blocks walk the 32 x 64 tiles t = blockIdx.x, + gridDim.x, ...
// (k tile fastest, then row tile, then batch); the next tile's loads are in
// flight in registers while the current one is converted.
template <int S>
__global__ void __launch_bounds__(256)
pack_digits_kernel(PackView v, int R, int K, int ld, int rows_fast, int ktn, int rtn,
                   int ntiles, const int *__restrict__ ex, __nv_bfloat16 *__restrict__ out) {
    __shared__ unsigned long long val[PT_R][PT_K + 1];
    __shared__ long long off[PT_R + PT_K];
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const size_t plane = (size_t)R * ld;
    auto decode = [&](int t, int &b, int &r0, int &k0) {
        b = t / (rtn * ktn);
        const int rem = t - b * rtn * ktn;
        r0 = (rem / ktn) * PT_R;
        k0 = (rem % ktn) * PT_K;
    };
    unsigned long long pre[8];
    int t = blockIdx.x;
    if (t < ntiles) {
        int b, r0, k0;
        decode(t, b, r0, k0);
        tile_offsets(v, r0, k0, R, K, off);
        __syncthreads();
        tile_fetch(v.p + (long long)b * v.bst, off, rows_fast, pre);
    }
    for (; t < ntiles; t += gridDim.x) {
        const long long tn = (long long)t + gridDim.x;
        int b, r0, k0;
        decode(t, b, r0, k0);
        __syncthreads();              // val and the offsets are free again
        if (rows_fast) {
#pragma unroll
            for (int i = 0; i < 8; i++) val[lane][w + 8 * i] = pre[i];
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                val[w + 8 * i][lane] = pre[2 * i];
                val[w + 8 * i][lane + 32] = pre[2 * i + 1];
            }
        }
        int bn = 0, rn = 0, kn = 0;
        if (tn < ntiles) {
            decode((int)tn, bn, rn, kn);
            tile_offsets(v, rn, kn, R, K, off);
        }
        __syncthreads();
        if (tn < ntiles) tile_fetch(v.p + (long long)bn * v.bst, off, rows_fast, pre);
        const int k = k0 + 2 * lane;
        if (k < K) {
            for (int rr = w; rr < PT_R; rr += 8) {
                const int row = r0 + rr;
                if (row >= R) break;
                const int e = exp_of(ex[(long long)b * R + row]);
                // the second value is zero beyond K (tile fill)
                store_digits<S>(out + (size_t)b * S * plane + (size_t)row * ld + k, plane,
                                val[rr][2 * lane], val[rr][2 * lane + 1], e);
            }
        }
    }
}

// Short rows (K <= 64 KT): one pass.  A block holds 32 whole rows in shared
// memory, takes each row's exponent from there and writes its digits, so the
// operand is read once and no atomics are needed.  The raw exponents it
// stores are those of the two-pass path (0x80808080 for an all-zero row).
// Blocks are persistent: they walk the row tiles t = blockIdx.x, + gridDim.x,
// ... (batch-major), and while one tile is converted from shared memory the
// global loads of the block's next tile are already in flight into
// registers.
constexpr int PR_KMAX = 256;

__host__ __device__ constexpr size_t pack_rows_smem(int kt) {
    return (size_t)PT_R * (kt * PT_K + 1) * 8 + (size_t)(kt * PT_K) * 8;
}

template <int S, int KT>
__global__ void __launch_bounds__(256, 2)
pack_rows_kernel(PackView v, int R, int K, int ld, int rows_fast, int rtiles, int ntiles,
                 int *__restrict__ ex, __nv_bfloat16 *__restrict__ out) {
    constexpr int NK = KT * PT_K, LDV = NK + 1, PER = NK / 8;   // values per thread
    extern __shared__ unsigned long long prs[];
    unsigned long long *val = prs;                                      // [PT_R][LDV]
    long long *koff = reinterpret_cast<long long *>(prs + PT_R * LDV);  // [NK]
    __shared__ int rexp[PT_R];
    const int tid = threadIdx.x, lane = tid % 32, w = tid / 32;
    for (int x = tid; x < NK; x += 256) koff[x] = (x < K) ? v.c.off(x) : -1;
    __syncthreads();
    // rows_fast: thread (lane, w) reads row lane at k = w + 8 i; otherwise rows
    // w + 8 i at k = lane + 32 j.  Both cover 32 x NK values, PER per thread.
    unsigned long long pre[PER];
    auto fetch = [&](int t) {
        const int b = t / rtiles, r0 = (t - b * rtiles) * PT_R;
        const double *base = v.p + (long long)b * v.bst;
        if (rows_fast) {
            const long long ro = (r0 + lane < R) ? v.r.off(r0 + lane) : -1;
#pragma unroll
            for (int i = 0; i < PER; i++) {
                const long long ko = koff[w + 8 * i];
                pre[i] = (ro >= 0 && ko >= 0)
                             ? (unsigned long long)__double_as_longlong(__ldg(base + ro + ko))
                             : 0ull;
            }
        } else {
#pragma unroll
            for (int i = 0; i < PT_R / 8; i++) {
                const int row = r0 + w + 8 * i;
                const long long ro = (row < R) ? v.r.off(row) : -1;
#pragma unroll
                for (int j = 0; j < 2 * KT; j++) {
                    const long long ko = koff[lane + 32 * j];
                    pre[i * 2 * KT + j] =
                        (ro >= 0 && ko >= 0)
                            ? (unsigned long long)__double_as_longlong(__ldg(base + ro + ko))
                            : 0ull;
                }
            }
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x);
    const size_t plane = (size_t)R * ld;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        __syncthreads();                      // the previous tile's values are used up
        if (rows_fast) {
#pragma unroll
            for (int i = 0; i < PER; i++) val[lane * LDV + w + 8 * i] = pre[i];
        } else {
#pragma unroll
            for (int i = 0; i < PT_R / 8; i++)
#pragma unroll
                for (int j = 0; j < 2 * KT; j++)
                    val[(w + 8 * i) * LDV + lane + 32 * j] = pre[i * 2 * KT + j];
        }
        __syncthreads();
        if ((long long)t + gridDim.x < ntiles) fetch(t + gridDim.x);
        const int b = t / rtiles, r0 = (t - b * rtiles) * PT_R;
        // raw exponent of each row: warp w takes rows w, w + 8, ...
#pragma unroll
        for (int i = 0; i < PT_R / 8; i++) {
            const int rr = w + 8 * i;
            int e = -2000;
#pragma unroll
            for (int j = 0; j < KT * 2; j++) {
                const unsigned long long bits = val[rr * LDV + lane + 32 * j];
                if ((bits & 0x7FFFFFFFFFFFFFFFull) != 0)
                    e = max(e, (int)((bits >> 52) & 0x7FF) - 1023);
            }
            for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
            if (lane == 0) {
                const int raw = (e > -2000) ? e : (int)0x80808080u;
                rexp[rr] = raw;
                if (r0 + rr < R) ex[(long long)b * R + r0 + rr] = raw;
            }
        }
        __syncthreads();
        for (int rr = w; rr < PT_R; rr += 8) {
            const int row = r0 + rr;
            if (row >= R) break;
            const int e = exp_of(rexp[rr]);
            __nv_bfloat16 *ob = out + (size_t)b * S * plane + (size_t)row * ld;
#pragma unroll
            for (int j = 0; j < KT; j++) {
                const int k = 2 * lane + 64 * j;
                if (k >= K) break;
                // the second value is zero beyond K
                store_digits<S>(ob + k, plane, val[rr * LDV + k], val[rr * LDV + k + 1], e);
            }
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

// 2D map over digit planes (K x rows, row stride ld elements); one box is a
// k-block of kb values (swizzled by its 2 kb bytes) by box_rows rows
int make_map(kvft_ctx *ctx, CUtensorMap *map, void *base, int K, int ld, long long rows, int kb,
             int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return kv_fail(ctx, KVFT_EDEVICE, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)kb, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    kb == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return kv_fail(ctx, KVFT_EDEVICE, "cuTensorMapEncodeTiled failed");
    return KVFT_OK;
}

struct Packed {
    __nv_bfloat16 *planes;
    int *ex;
    int R, ld, K, nb;
};

// Digit planes [nb][S][R][ld] and exponents [nb][R].  ld = K rounded up to 64
// elements, so that every row starts on a 128-byte line and a TMA box row
// (one k-block of one row) touches one line, not two.  No row or K padding is
// written: the tensor map's extent is (K, nb S R) and TMA fills out-of-range
// boxes with zeros; rows past R inside a 128-row box belong to the next plane
// and only reach output rows/columns that the epilogue discards.
// Identity of a packed operand: address, view, extents and digit count.
std::string pack_key(const PackView &v, int R, int K, int nb, int S) {
    char b[320];
    snprintf(b, sizeof b, "%p|%d,%d,%d:%lld,%lld,%lld|%d,%d,%d:%lld,%lld,%lld|%lld|%d,%d,%d,%d",
             (const void *)v.p, v.r.size[0], v.r.size[1], v.r.size[2], v.r.st[0], v.r.st[1],
             v.r.st[2], v.c.size[0], v.c.size[1], v.c.size[2], v.c.st[0], v.c.st[1], v.c.st[2],
             v.bst, R, K, nb, S);
    return b;
}

// persistent digit pass: as many blocks as fit on the SMs at once
template <int S>
int launch_pack_digits(kvft_ctx *ctx, const PackView &v, int R, int K, int ld, int rows_fast,
                       int ktn, int rtn, long long tiles, Packed *out) {
    static int per_sm = 0;
    if (!per_sm) {
        KV_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, pack_digits_kernel<S>, 256, 0));
        per_sm = std::max(per_sm, 1);
    }
    const int grid = (int)std::min(tiles, (long long)per_sm * ctx->sm_count);
    pack_digits_kernel<S><<<grid, 256, 0, ctx->stream>>>(v, R, K, ld, rows_fast, ktn, rtn,
                                                        (int)tiles, out->ex, out->planes);
    return KVFT_OK;
}

template <int S, int KT>
int launch_pack_rows(kvft_ctx *ctx, const PackView &v, int R, int K, int ld, int nb,
                     int rows_fast, int rtiles, Packed *out) {
    constexpr size_t smem = pack_rows_smem(KT);
    static int per_sm = 0;
    if (!per_sm) {
        KV_CHECK(ctx, cudaFuncSetAttribute(pack_rows_kernel<S, KT>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        KV_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, pack_rows_kernel<S, KT>, 256, smem));
        per_sm = std::max(per_sm, 1);
    }
    const long long ntiles = (long long)rtiles * nb;
    if (ntiles > 0x7FFFFFFFLL) return kv_fail(ctx, KVFT_EINVAL, "pack: too many row tiles");
    const int grid = (int)std::min(ntiles, (long long)per_sm * ctx->sm_count);
    pack_rows_kernel<S, KT><<<grid, 256, smem, ctx->stream>>>(
        v, R, K, ld, rows_fast, rtiles, (int)ntiles, out->ex, out->planes);
    return kv_launch_check(ctx, "pack_rows");
}

template <int S>
int pack_rows_s(kvft_ctx *ctx, const PackView &v, int R, int K, int ld, int nb, int rows_fast,
                int rtiles, Packed *out) {
    if (K <= PT_K) return launch_pack_rows<S, 1>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    if (K <= 2 * PT_K)
        return launch_pack_rows<S, 2>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    return launch_pack_rows<S, 4>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
}

int pack_rows(kvft_ctx *ctx, const PackView &v, int R, int K, int ld, int nb, int S,
              int rows_fast, int rtiles, Packed *out) {
    switch (S) {
    case 1: return pack_rows_s<1>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    case 2: return pack_rows_s<2>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    case 3: return pack_rows_s<3>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    case 4: return pack_rows_s<4>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    case 5: return pack_rows_s<5>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    case 6: return pack_rows_s<6>(ctx, v, R, K, ld, nb, rows_fast, rtiles, out);
    default: return kv_fail(ctx, KVFT_EINVAL, "pack: digit count out of range");
    }
}

int pack(kvft_ctx *ctx, const char *key, const PackView &v, int R, int K, int nb, int S,
         Packed *out) {
    const int ld = (K + 63) / 64 * 64;
    const size_t plane_bytes = (size_t)R * ld * 2;
    const size_t pbytes = ((size_t)nb * S * plane_bytes + 1023) / 1024 * 1024;
    const size_t bytes = pbytes + (size_t)nb * R * sizeof(int);
    out->R = R;
    out->ld = ld;
    out->K = K;
    out->nb = nb;
    if (nb > 65535) return kv_fail(ctx, KVFT_EINVAL, "pack: batch too large");
    void *buf = nullptr;
    std::string ckey;
    if (v.stable && ctx->pack_cache_on) {
        // an integral block packed during an earlier residual evaluation
        ckey = pack_key(v, R, K, nb, S);
        auto it = ctx->pack_cache.find(ckey);
        if (it != ctx->pack_cache.end()) {
            out->planes = (__nv_bfloat16 *)it->second.first;
            out->ex = (int *)((uint8_t *)it->second.first + pbytes);
            return KVFT_OK;
        }
        // keep it only while a tenth of the device stays free
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && fr > bytes + tot / 10 &&
            cudaMalloc(&buf, bytes) == cudaSuccess) {
            ctx->pack_cache[ckey] = {buf, bytes};
            ctx->scratch_gen++;
        } else {
            cudaGetLastError();
            buf = nullptr;
        }
    }
    if (!buf && !v.stable && ctx->tpack_on) {
        // an operand sub-block already packed for an earlier product of the
        // same spin-blocked contraction
        ckey = pack_key(v, R, K, nb, S);
        auto it = ctx->tpack.find(ckey);
        const int slot = (it != ctx->tpack.end()) ? it->second : (int)ctx->tpack.size();
        char sk[32];
        snprintf(sk, sizeof sk, "tpack%d", slot);
        KV_TRY(kv_scratch(ctx, sk, bytes, &buf));
        out->planes = (__nv_bfloat16 *)buf;
        out->ex = (int *)((uint8_t *)buf + pbytes);
        if (it != ctx->tpack.end()) return KVFT_OK;
        ctx->tpack[ckey] = slot;
    }
    if (!buf) KV_TRY(kv_scratch(ctx, key, bytes, &buf));
    out->planes = (__nv_bfloat16 *)buf;
    out->ex = (int *)((uint8_t *)buf + pbytes);
    KvProfScope prof(ctx, KV_CAT_PACK, 8.0 * nb * (double)R * K + (double)nb * S * plane_bytes);
    // coalesce global reads along the contiguous index
    const int rows_fast = (kidx_fast_stride(v.r) == 1 && kidx_fast_stride(v.c) != 1) ? 1 : 0;
    const long long rtiles = (R + PT_R - 1) / PT_R;
    if (rtiles > 65535) return kv_fail(ctx, KVFT_EINVAL, "pack: too many rows");
    if (K <= PR_KMAX) return pack_rows(ctx, v, R, K, ld, nb, S, rows_fast, (int)rtiles, out);
    KV_CHECK(ctx, cudaMemsetAsync(out->ex, 0x80, (size_t)nb * R * sizeof(int), ctx->stream));
    const dim3 g((K + PT_K - 1) / PT_K, (unsigned)rtiles, nb);
    // long rows: each exponent block walks up to 16 k tiles, so that about
    // 32 blocks per SM remain and the atomics per row drop accordingly
    const long long tiles = (long long)g.x * g.y * g.z;
    const int ktiles = (int)std::max(1LL, std::min(16LL, tiles / (32LL * ctx->sm_count)));
    const dim3 ge((g.x + ktiles - 1) / ktiles, g.y, g.z);
    pack_exp_kernel<<<ge, 256, 0, ctx->stream>>>(v, R, K, rows_fast, ktiles, out->ex);
    KV_TRY(kv_launch_check(ctx, "pack_exp"));
    if (tiles > 0x7FFFFFFFLL) return kv_fail(ctx, KVFT_EINVAL, "pack: too many tiles");
    switch (S) {
#define KV_PACK_CASE(s_)                                                                   \
    case s_:                                                                               \
        KV_TRY(launch_pack_digits<s_>(ctx, v, R, K, ld, rows_fast, g.x, g.y, tiles, out)); \
        break;
        KV_PACK_CASE(1) KV_PACK_CASE(2) KV_PACK_CASE(3) KV_PACK_CASE(4) KV_PACK_CASE(5)
        KV_PACK_CASE(6)
#undef KV_PACK_CASE
    default: return kv_fail(ctx, KVFT_EINVAL, "pack: digit count out of range");
    }
    KV_TRY(kv_launch_check(ctx, "pack_digits"));
    return KVFT_OK;
}

// The stride-1 index of a view: its fastest dimension of extent > 1 has
// element stride 1 (or the index has a single value).
bool unit_stride(const KIdx &x) {
    const long long f = kidx_fast_stride(x);
    return f == 1 || f == 0;
}

constexpr size_t SMEM_CAP = 225 * 1024;
// Below half of an SM's shared memory two CTAs could share an SM and the
// second one's 512-column TMEM allocation would block: always take more.
constexpr size_t SMEM_FLOOR = 120 * 1024;

// Launches the persistent kernel, one CTA per SM.
template <int TN, bool FF, int KBT, int DL>
int launch_tc(kvft_ctx *ctx, const CUtensorMap &ma, const CUtensorMap &mb, TcParams &p) {
    auto kern = tc_gemm_kernel<TN, FF, KBT, DL>;
    int NS = 2;
    while (NS < 8 && tc_smem(p.S, NS + 1, TN, KBT) <= SMEM_CAP) NS++;
    if (tc_smem(p.S, NS, TN, KBT) > SMEM_CAP)
        return kv_fail(ctx, KVFT_EINVAL, "tensor-core gemm: stages exceed shared memory");
    p.NS = NS;
    const size_t smem = std::max(tc_smem(p.S, NS, TN, KBT), SMEM_FLOOR);
    static bool attr = false;
    if (!attr) {
        KV_CHECK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)SMEM_CAP));
        attr = true;
    }
    const int grid = std::min(p.units, ctx->sm_count);
    KvProfScope prof(ctx, ctx->gemm_cat, ctx->gemm_work);
    kern<<<grid, NTHREADS, smem, ctx->stream>>>(ma, mb, p);
    return kv_launch_check(ctx, "tc_gemm");
}

int gemm_tc_run(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha, const KMat &A,
                const KMat &B, double beta, const KOut &C, int D) {
    const int S = std::min(D - 1, MAXS);
    // D >= 4: three to six levels, FP32 pairs, TN = 64, and 32-deep k-blocks
    // (six digit planes per stage); D <= 3: 64-deep k-blocks, so that every
    // TMA box row is a full 128-byte line, and TN = 128 unless C has at most
    // 64 columns (then 64-wide tiles keep all eight epilogue warps busy)
    const bool ff = D >= 4;
    const int tn = (ff || N <= 64) ? 64 : 128;
    const int kb = ff ? 32 : 64;
    const int nbA = A.bst ? batch : 1, nbB = B.bst ? batch : 1;
    Packed pa, pb;
    KV_TRY(pack(ctx, "tc_pack_a", PackView{A.p, A.r, A.c, A.bst, A.stable}, M, K, nbA, S, &pa));
    // B is K x N; its K-major form has rows = N (B's column index), cols = K
    KV_TRY(pack(ctx, "tc_pack_b", PackView{B.p, B.c, B.r, B.bst, B.stable}, N, K, nbB, S, &pb));
    CUtensorMap ma, mb;
    KV_TRY(make_map(ctx, &ma, pa.planes, pa.K, pa.ld, (long long)nbA * S * pa.R, kb, TM));
    KV_TRY(make_map(ctx, &mb, pb.planes, pb.K, pb.ld, (long long)nbB * S * pb.R, kb, tn));
    const int mt = (M + TM - 1) / TM, nt = (N + tn - 1) / tn;
    const int nkb_total = (K + kb - 1) / kb;
    const int nchunks = (nkb_total + KCHUNK / kb - 1) / (KCHUNK / kb);
    const int chunk_kb = (nkb_total + nchunks - 1) / nchunks;     // balanced chunks
    const long long tiles = (long long)mt * nt * batch;
    // fewer output tiles than two waves of SMs and several K chunks: every
    // chunk becomes a unit of its own and adds into C with FP64 atomics
    // (C pre-scaled by beta)
    const bool par = nchunks > 1 && tiles < 2LL * ctx->sm_count;
    const long long units = tiles * (par ? nchunks : 1);
    if (units > 0x7FFFFFFFLL) return kv_fail(ctx, KVFT_EINVAL, "tensor-core gemm: too many tiles");
    if (par && beta != 1.0) KV_TRY(kv_scale_view(ctx, M, N, batch, beta, C));
    TcParams p;
    p.M = M;
    p.N = N;
    p.mt = mt;
    p.nt = nt;
    p.units = (int)units;
    p.nsplit = par ? nchunks : 1;
    p.chunk_kb = chunk_kb;
    p.nkb_total = nkb_total;
    p.S = S;
    p.D = D;
    p.NS = 0;
    p.Mp = pa.R;
    p.Np = pb.R;
    p.a_batch_rows = (nbA > 1) ? S * pa.R : 0;
    p.b_batch_rows = (nbB > 1) ? S * pb.R : 0;
    p.ea = pa.ex;
    p.eb = pb.ex;
    p.ea_bst = (nbA > 1) ? pa.R : 0;
    p.eb_bst = (nbB > 1) ? pb.R : 0;
    p.alpha = alpha;
    p.beta = par ? 1.0 : beta;
    {
        int ex2 = 0;
        const double fr = std::frexp(alpha, &ex2);
        p.alpha_pow2 = (std::fabs(fr) == 0.5) ? 1 : 0;
        p.alpha_exp = p.alpha_pow2 ? ex2 - 1 : 0;
        p.alpha_sign = (p.alpha_pow2 && alpha < 0) ? 0x80000000u : 0u;
    }
    p.C = C;
    p.err = ctx->dflag;
    p.dv_split = fastdiv(p.nsplit);
    p.dv_perb = fastdiv(p.mt * p.nt);
    p.dv_gsz = fastdiv(GROUP_M * p.nt);
    p.dv_cr2 = fastdiv(C.r.size[2]);
    p.dv_cr1 = fastdiv(C.r.size[1]);
    switch (D) {
    case 2:
        return tn == 64 ? launch_tc<64, false, 64, 2>(ctx, ma, mb, p)
                        : launch_tc<128, false, 64, 2>(ctx, ma, mb, p);
    case 3:
        return tn == 64 ? launch_tc<64, false, 64, 3>(ctx, ma, mb, p)
                        : launch_tc<128, false, 64, 3>(ctx, ma, mb, p);
    case 4: return launch_tc<64, true, 32, 4>(ctx, ma, mb, p);
    case 5: return launch_tc<64, true, 32, 5>(ctx, ma, mb, p);
    case 6: return launch_tc<64, true, 32, 6>(ctx, ma, mb, p);
    default: return launch_tc<64, true, 32, 7>(ctx, ma, mb, p);
    }
}

}  // namespace

int kv_gemm_tc(kvft_ctx *ctx, int M, int N, int K, int batch, double alpha, const KMat &A,
               const KMat &B, double beta, const KOut &C, int digits) {
    const int D = digits;
    if (D < 2 || D > MAXS + 1) return kv_fail(ctx, KVFT_EINVAL, "tensor-core digits out of range");
    if (M <= 0 || N <= 0 || batch <= 0) return KVFT_OK;
    if (K <= 0) return kv_gemm_f64(ctx, M, N, K, batch, alpha, A, B, beta, C);
    // C^T = B^T A^T costs nothing but the operand roles.  The epilogue's lanes
    // are the tile rows, so the stride-1 index of C goes to the rows (each
    // store then covers 32 consecutive doubles) unless that extent is short
    // and K long (the unused TMEM lanes would cost MMA time); otherwise the
    // larger extent goes to the rows.
    bool swap = M < N;
    const bool rc = unit_stride(C.r), cc = unit_stride(C.c);
    if (rc != cc) {
        const int ext = cc ? N : M;
        if (ext >= 64 || K <= 512) swap = cc;
    }
    if (swap) {
        const KMat At{B.p, B.c, B.r, B.bst, B.stable};
        const KMat Bt{A.p, A.c, A.r, A.bst, A.stable};
        const KOut Ct{C.p, C.c, C.r, C.bst};
        return gemm_tc_run(ctx, N, M, K, batch, alpha, At, Bt, beta, Ct, D);
    }
    return gemm_tc_run(ctx, M, N, K, batch, alpha, A, B, beta, C, D);
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
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_gemm: not on a dry-run context");
    if (!ctx || M <= 0 || N <= 0 || K <= 0 || batch <= 0 || !A || !B || !C)
        return kv_fail(ctx, KVFT_EINVAL, "kvft_gemm: bad argument");
    cudaSetDevice(ctx->device);
    KMat a{A, kidx1(M, K), kidx1(K, 1), (long long)M * K};
    KMat b{B, kidx1(K, N), kidx1(N, 1), (long long)K * N};
    KOut c{C, kidx1(M, N), kidx1(N, 1), (long long)M * N};
    kv_gemm_prof_set(ctx, M, N, K, batch, batch, batch, 0.0, precision != KVFT_PREC_FP64);
    int st;
    if (precision == KVFT_PREC_FP64)
        st = kv_gemm_f64(ctx, M, N, K, batch, 1.0, a, b, 0.0, c);
    else
        st = kv_gemm_tc(ctx, M, N, K, batch, 1.0, a, b, 0.0, c, digits);
    if (st != KVFT_OK) return st;
    return kv_device_status(ctx);
}
