// Element-wise kernels of the CCSD update: permuted axpby, tau amplitudes,
// W_mbej helper, the antisymmetrised T2 assembly and batch broadcast.  All are
// HBM-bound grid-stride loops over a tau batch of n^4 tensors.
#include "kvft_internal.h"

namespace {

inline int grid_for(kvft_ctx *ctx, long long total, int threads) {
    long long b = (total + threads - 1) / threads;
    long long cap = (long long)ctx->sm_count * 8;
    return (int)std::max(1LL, std::min(b, cap));
}

struct Dims4 {
    int d[4];
    long long ss[4], ds[4];
    long long sbst, dbst;
};

// ---- antisymmetric pair compression ------------------------------------------
// A tensor antisymmetric in an index pair is stored over p < q only; pair
// index x = p (2n - p - 1) / 2 + (q - p - 1).
__device__ __forceinline__ int pair_start(int p, int n) { return p * (2 * n - p - 1) / 2; }

__device__ __forceinline__ void pair_of(int x, int n, int &p, int &q) {
    const float b = 2.0f * n - 1.0f;
    p = (int)((b - sqrtf(b * b - 8.0f * x)) * 0.5f);
    p = max(0, min(p, n - 2));
    while (p > 0 && pair_start(p, n) > x) p--;
    while (p < n - 2 && pair_start(p + 1, n) <= x) p++;
    q = x - pair_start(p, n) + p + 1;
}

// Order of the pairs p < q over n orbitals.  h = 0: row-major triangle
// (x = pair_start(p, n) + q - p - 1).  h > 0 (spin blocks, n = 2h): the
// alpha-alpha pairs (triangle over [0, h)), then the alpha-beta pairs
// (p * h + q - h), then the beta-beta pairs (triangle over [h, 2h)), so each
// pair spin type is one contiguous range and a ladder contraction, nonzero
// only between pairs of one type, splits into three block products.
struct PairOrder {
    int n, h;
    __device__ __forceinline__ int index(int p, int q) const {
        if (!h) return pair_start(p, n) + q - p - 1;
        const int paa = h * (h - 1) / 2;
        if (q < h) return pair_start(p, h) + q - p - 1;
        if (p < h) return paa + p * h + (q - h);
        return paa + h * h + pair_start(p - h, h) + q - p - 1;
    }
    __device__ __forceinline__ void decode(int x, int &p, int &q) const {
        if (!h) {
            pair_of(x, n, p, q);
            return;
        }
        const int paa = h * (h - 1) / 2;
        if (x < paa) {
            pair_of(x, h, p, q);
            return;
        }
        x -= paa;
        if (x < h * h) {
            p = x / h;
            q = h + x % h;
            return;
        }
        pair_of(x - h * h, h, p, q);
        p += h;
        q += h;
    }
    // index range [lo, hi) of the pairs of spin type t = s_p + s_q
    __device__ __forceinline__ void range(int t, int &lo, int &hi) const {
        if (!h) {
            lo = 0;
            hi = n * (n - 1) / 2;
            return;
        }
        const int paa = h * (h - 1) / 2;
        lo = t == 0 ? 0 : (t == 1 ? paa : paa + h * h);
        hi = t == 0 ? paa : (t == 1 ? paa + h * h : 2 * paa + h * h);
    }
};

// One block per (batch, i0, i1, chunk of AX_CHUNK (i2, i3) positions); its
// threads walk (i2, i3), the innermost index fastest, so only a 32-bit
// division per element remains.  GB300 issues about two FP64 operations per
// clock per SM, so the common cases get their own instances: KIND 0 copies
// with alpha = +-1 (no FP64 operation), KIND 1 scales (beta = 0: dst is not
// read), KIND 2 is the general dst = beta dst + alpha src.
constexpr int AX_CHUNK = 2048;

template <int KIND>
__global__ void __launch_bounds__(256)
axpby4_kernel(long long nblk, Dims4 g, double alpha, const double *__restrict__ src,
              double beta, double *__restrict__ dst) {
    const long long n23 = (long long)g.d[2] * g.d[3];
    const long long nch = (n23 + AX_CHUNK - 1) / AX_CHUNK;
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const long long row = blk / nch;
        const long long e0 = (blk - row * nch) * AX_CHUNK;
        const long long b = row / ((long long)g.d[0] * g.d[1]);
        const int r = (int)(row - b * g.d[0] * g.d[1]);
        const int i0 = r / g.d[1], i1 = r % g.d[1];
        const double *s = src + b * g.sbst + i0 * g.ss[0] + i1 * g.ss[1];
        double *d = dst + b * g.dbst + i0 * g.ds[0] + i1 * g.ds[1];
        const int cnt = (int)min((long long)AX_CHUNK, n23 - e0);
        const long long i2s = e0 / g.d[3];
        const int i3s = (int)(e0 - i2s * g.d[3]);
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            const int t = i3s + k;               // < d3 + AX_CHUNK: 32-bit
            const long long i2 = i2s + t / g.d[3];
            const int i3 = t % g.d[3];
            const double x = s[i2 * g.ss[2] + i3 * g.ss[3]];
            double *o = d + i2 * g.ds[2] + i3 * g.ds[3];
            if (KIND == 0) *o = alpha < 0.0 ? -x : x;
            else if (KIND == 1) *o = alpha * x;
            else *o = fma(beta, *o, alpha * x);
        }
    }
}

// out[y,a,b,i,j] = t2 + c (t1[a,i] t1[b,j] - t1[b,i] t1[a,j]); one block per
// (y, a, b), threads over (i, j).  The rows c t1[a,:] and c t1[b,:] are formed
// once per block in shared memory, so each element costs two FP64 FMAs.
__global__ void __launch_bounds__(256)
make_tau_kernel(long long nblk, int nv, int no, int sh, const double *__restrict__ t1,
                const double *__restrict__ t2, double c, double *__restrict__ out) {
    extern __shared__ double cab[];                  // [2][no]: c t1[a,:], c t1[b,:]
    const int oo = no * no;
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const long long y = blk / ((long long)nv * nv);
        const int ab = (int)(blk - y * nv * nv);
        const int a = ab / nv, b = ab % nv;
        const double *u = t1 + y * nv * no;
        const double *ua = u + a * no, *ub = u + b * no;
        __syncthreads();
        for (int x = threadIdx.x; x < no; x += blockDim.x) {
            cab[x] = c * ua[x];
            cab[no + x] = c * ub[x];
        }
        __syncthreads();
        const long long base = blk * oo;
        if (sh) {
            // spin blocks (nv = no = 2 sh): only the spin-conserving (i, j) are
            // read later -- the quadrant(s) with s_i + s_j = s_a + s_b, walked
            // directly (j fastest)
            const int sab = (a >= sh) + (b >= sh), hh = sh * sh;
            const int nq = sab == 1 ? 2 : 1;
            for (int x = threadIdx.x; x < nq * hh; x += blockDim.x) {
                const int qq = x / hh, r = x - qq * hh;
                const int i1 = r / sh, j1 = r - i1 * sh;
                const int si = sab == 1 ? qq : sab / 2, sj = sab == 1 ? 1 - qq : sab / 2;
                const int i = si * sh + i1, j = sj * sh + j1, e = i * no + j;
                out[base + e] = fma(cab[i], ub[j], fma(-cab[no + i], ua[j], t2[base + e]));
            }
        } else {
            for (int e = threadIdx.x; e < oo; e += blockDim.x) {
                const int i = e / no, j = e % no;
                out[base + e] = fma(cab[i], ub[j], fma(-cab[no + i], ua[j], t2[base + e]));
            }
        }
    }
}

// out[y][b][j][n][f] = 0.5 t2[y][f][b][j][n] + t1[y][f][j] t1[y][b][n]: the
// contraction index (n, f) ends up contiguous, matching <mn||ef> of the W_mbej
// product.  32 x 32 (f, n) tiles go through shared memory so the reads are
// coalesced along n and the writes along f.  (Spin blocks: the kernel below.)
__global__ void __launch_bounds__(256)
wmbej_tmp_kernel(int nv, int no, const double *__restrict__ t1,
                 const double *__restrict__ t2, double *__restrict__ out) {
    __shared__ double tile[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int ntn = (no + 31) / 32;
    const int f0 = (blockIdx.x / ntn) * 32, n0 = (blockIdx.x % ntn) * 32;
    const long long y = blockIdx.z;
    const long long oo = (long long)no * no;
    const double *u = t1 + y * nv * no;
    for (int bj = blockIdx.y; bj < nv * no; bj += gridDim.y) {
        const int b = bj / no, j = bj % no;
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int f = f0 + ty + 8 * i, n = n0 + tx;
            if (f < nv && n < no)
                tile[ty + 8 * i][tx] = t2[((y * nv + f) * nv + b) * oo + (long long)j * no + n];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int n = n0 + ty + 8 * i, f = f0 + tx;
            if (f < nv && n < no)
                out[(((y * nv + b) * no + j) * no + n) * nv + f] =
                    0.5 * tile[tx][ty + 8 * i] + u[f * no + j] * u[b * no + n];
        }
    }
}

// T2[y,a,b,i,j] += fac (1 - P(ab))(1 - P(ij)) (Z + L)[y,a,b,i,j], L = the
// ladder sum stored over a < b, i < j and zero elsewhere.  One block per
// (a < b) pair and pair of 32 x 32 (i, j) tiles (a tile and its mirror):
// Q = Z[a,b] - Z[b,a] of both tiles goes through shared memory, so every Z
// element is read once, coalesced, and R = Q - Q^T + (L - L^T) is added to
// T2[a,b] and subtracted from T2[b,a].  The a = b blocks of T2 get nothing.
// Every other element of T2 receives exactly one addition, issued as a
// fire-and-forget reduction at L2 (one rounding, like load-add-store); the
// additions then cost the SM's scarce FP64 pipe nothing.
// FS: fac is +1 (1), -1 (2) or anything else (0); the signs cost no FP64
// operation.  SEED: T2 = -seed + R is stored (every a != b element once), no
// reduction and no pre-seeded T2.
template <int FS, bool SEED>
__global__ void __launch_bounds__(256, 3)
assemble_t2_kernel(int nv, int no, int sh, double fac, const double *__restrict__ Z,
                   const double *__restrict__ Lc, const double *__restrict__ seed,
                   double *__restrict__ T2) {
    const PairOrder ov{nv, sh}, oo_{no, sh};
    __shared__ double qa[32][33], qb[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int nt = (no + 31) / 32;
    int it = 0, rem = blockIdx.x;           // tile pair (it <= jt)
    while (rem >= nt - it) {
        rem -= nt - it;
        it++;
    }
    const int jt = it + rem;
    const int i0 = it * 32, j0 = jt * 32;
    const long long y = blockIdx.z;
    const int pv = nv * (nv - 1) / 2, po = no * (no - 1) / 2;
    const long long oo = (long long)no * no, s4 = (long long)nv * nv * oo;
    for (int pab = blockIdx.y; pab < pv; pab += gridDim.y) {
        int a, b;
        ov.decode(pab, a, b);
        const int tab = (a >= sh) + (b >= sh);
        const long long oab = y * s4 + ((long long)a * nv + b) * oo;
        const long long oba = y * s4 + ((long long)b * nv + a) * oo;
        const double *L = Lc ? Lc + (y * pv + pab) * (long long)po : nullptr;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = ty + 8 * k;
            int i = i0 + r, j = j0 + tx;
            qa[r][tx] = (i < no && j < no) ? Z[oab + i * no + j] - Z[oba + i * no + j] : 0.0;
            i = j0 + r;
            j = i0 + tx;
            qb[r][tx] = (i < no && j < no) ? Z[oab + i * no + j] - Z[oba + i * no + j] : 0.0;
        }
        __syncthreads();
        // L over (i < j); with spin blocks it vanishes between pair types
        auto ladder = [&](int i, int j) -> double {
            if (!L || i == j) return 0.0;
            if (sh && (i >= sh) + (j >= sh) != tab) return 0.0;
            return i < j ? L[oo_.index(i, j)] : -L[oo_.index(j, i)];
        };
        const long long sab = ((long long)a * nv + b) * oo, sba = ((long long)b * nv + a) * oo;
        auto put = [&](int x, double R) {
            if (SEED) {
                T2[oab + x] = R - seed[sab + x];
                T2[oba + x] = -R - seed[sba + x];
            } else {
                atomicAdd(T2 + oab + x, R);
                atomicAdd(T2 + oba + x, -R);
            }
        };
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = ty + 8 * k;
            int i = i0 + r, j = j0 + tx;
            if (i < no && j < no) {
                const double R0 = qa[r][tx] - qb[tx][r] + ladder(i, j);
                const double R = FS == 0 ? fac * R0 : (FS == 1 ? R0 : -R0);
                put(i * no + j, R);
            }
            i = j0 + r;
            j = i0 + tx;
            if (it != jt && i < no && j < no) {
                const double R0 = qb[r][tx] - qa[tx][r] + ladder(i, j);
                const double R = FS == 0 ? fac * R0 : (FS == 1 ? R0 : -R0);
                put(i * no + j, R);
            }
        }
    }
}

// The same with spin blocks (nv = no = n = 2h): for each (b, j) only the
// (f, n) with s_f - s_n = s_j - s_b are written -- the alpha-alpha and
// beta-beta quadrants, or the one mixed quadrant -- in 32 x 32 tiles laid out
// from each quadrant's origin (no tile straddles the spin boundary; block x
// = quadrant and tile).
__global__ void __launch_bounds__(256)
wmbej_tmp_spin_kernel(int n, int h, const double *__restrict__ t1,
                      const double *__restrict__ t2, double *__restrict__ out) {
    __shared__ double tile[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int nth = (h + 31) / 32, nt2 = nth * nth;
    const int q = blockIdx.x / nt2, tt = blockIdx.x % nt2;
    const long long y = blockIdx.z;
    const long long oo = (long long)n * n;
    const double *u = t1 + y * oo;
    for (int bj = blockIdx.y; bj < n * n; bj += gridDim.y) {
        const int b = bj / n, j = bj % n;
        const int d = (j >= h) - (b >= h);          // s_f - s_n
        if (d != 0 && q) continue;                  // block-uniform
        const int sf = d == 0 ? q : (d > 0), sn = d == 0 ? q : (d < 0);
        const int f0 = sf * h + 32 * (tt / nth), n0 = sn * h + 32 * (tt % nth);
        const int fhi = sf * h + h, nhi = sn * h + h;
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int f = f0 + ty + 8 * i, m = n0 + tx;
            if (f < fhi && m < nhi)
                tile[ty + 8 * i][tx] = t2[((y * n + f) * n + b) * oo + (long long)j * n + m];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int m = n0 + ty + 8 * i, f = f0 + tx;
            if (f < fhi && m < nhi)
                out[(((y * n + b) * n + j) * n + m) * n + f] =
                    0.5 * tile[tx][ty + 8 * i] + u[f * n + j] * u[b * n + m];
        }
    }
}

// The seeded assembly with spin blocks (nv = no = n = 2h): for the pair
// (a < b) of spin sum t = s_a + s_b only the (i, j) with s_i + s_j = t are
// written -- the alpha-alpha quadrant (t = 0), the beta-beta one (t = 2), or
// the alpha-beta quadrant with its mirror beta-alpha (t = 1).  Tiles are laid
// out from each quadrant's origin, so no tile straddles the spin boundary:
// tile pairs (it <= jt) of a diagonal quadrant, every (it, jt) of the
// alpha-beta one with its mirror tile in the beta-alpha one.  The other
// elements of T2 are left as they are (zero: nothing writes or reads them).
template <int FS>
__global__ void __launch_bounds__(256, 3)
assemble_t2_spin_kernel(int n, int h, double fac, const double *__restrict__ Z,
                        const double *__restrict__ Lc, const double *__restrict__ seed,
                        double *__restrict__ T2) {
    const PairOrder ov{n, h};
    __shared__ double qa[32][33], qb[32][33];
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    const int nth = (h + 31) / 32;
    const long long y = blockIdx.z;
    const int pv = n * (n - 1) / 2;
    const long long oo = (long long)n * n, s4 = oo * oo;
    for (int pab = blockIdx.y; pab < pv; pab += gridDim.y) {
        int a, b;
        ov.decode(pab, a, b);
        const int tab = (a >= h) + (b >= h);
        int it, jt;
        if (tab == 1) {
            if ((int)blockIdx.x >= nth * nth) continue;              // block-uniform
            it = blockIdx.x / nth;
            jt = blockIdx.x % nth;
        } else {
            if ((int)blockIdx.x >= nth * (nth + 1) / 2) continue;
            it = 0;
            int rem = blockIdx.x;
            while (rem >= nth - it) {
                rem -= nth - it;
                it++;
            }
            jt = it + rem;
        }
        const int ilo = tab == 2 ? h : 0, jlo = tab == 0 ? 0 : h;   // quadrant origins
        const int ihi = ilo + h, jhi = jlo + h;
        const int i0 = ilo + 32 * it, j0 = jlo + 32 * jt;
        const bool mirror = tab == 1 || it != jt;
        const long long oab = y * s4 + ((long long)a * n + b) * oo;
        const long long oba = y * s4 + ((long long)b * n + a) * oo;
        const double *L = Lc ? Lc + (y * pv + pab) * (long long)pv : nullptr;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = ty + 8 * k;
            int i = i0 + r, j = j0 + tx;
            qa[r][tx] = (i < ihi && j < jhi) ? Z[oab + i * n + j] - Z[oba + i * n + j] : 0.0;
            i = j0 + r;
            j = i0 + tx;
            qb[r][tx] = (i < jhi && j < ihi) ? Z[oab + i * n + j] - Z[oba + i * n + j] : 0.0;
        }
        __syncthreads();
        // L over (i < j); both indices of a written element have the pair's type
        auto ladder = [&](int i, int j) -> double {
            if (!L || i == j) return 0.0;
            return i < j ? L[ov.index(i, j)] : -L[ov.index(j, i)];
        };
        const long long sab = ((long long)a * n + b) * oo, sba = ((long long)b * n + a) * oo;
        auto put = [&](int x, double R) {
            T2[oab + x] = R - seed[sab + x];
            T2[oba + x] = -R - seed[sba + x];
        };
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = ty + 8 * k;
            int i = i0 + r, j = j0 + tx;
            if (i < ihi && j < jhi) {
                const double R0 = qa[r][tx] - qb[tx][r] + ladder(i, j);
                put(i * n + j, FS == 0 ? fac * R0 : (FS == 1 ? R0 : -R0));
            }
            i = j0 + r;
            j = i0 + tx;
            if (mirror && i < jhi && j < ihi) {
                const double R0 = qb[r][tx] - qa[tx][r] + ladder(i, j);
                put(i * n + j, FS == 0 ? fac * R0 : (FS == 1 ? R0 : -R0));
            }
        }
    }
}

__global__ void bcast_kernel(long long total, long long count,
                             const double *__restrict__ src,
                             double *__restrict__ dst) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x)
        dst[x] = src[x % count];
}

// tau_c[y][(e<f)][(i<j)] = t2[y,e,f,i,j] + t1[y,e,i] t1[y,f,j] - t1[y,f,i] t1[y,e,j];
// one block per (y, e<f), threads over the (i<j) pairs
__global__ void __launch_bounds__(256)
make_tau_pairs_kernel(long long nblk, int nv, int no, int pv, int po, int sh,
                      const double *__restrict__ t1, const double *__restrict__ t2,
                      double *__restrict__ out) {
    const long long s4 = (long long)nv * nv * no * no;
    const PairOrder ov{nv, sh}, oo_{no, sh};
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const long long y = blk / pv;
        int e, f;
        ov.decode((int)(blk - y * pv), e, f);
        const double *u = t1 + y * nv * no;
        const double *src = t2 + y * s4 + ((long long)e * nv + f) * no * no;
        double *dst = out + blk * po;
        // with spin blocks only the (i < j) of the same pair type are read
        int lo = 0, hi = po;
        if (sh) oo_.range((e >= sh) + (f >= sh), lo, hi);
        for (int x = lo + threadIdx.x; x < hi; x += blockDim.x) {
            int i, j;
            oo_.decode(x, i, j);
            dst[x] = src[i * no + j] + u[e * no + i] * u[f * no + j] - u[f * no + i] * u[e * no + j];
        }
    }
}

struct PairGather {
    int n1, n2, P1, P2;          // pair ranges: (p<q) over n1 rows, (r<s) over n2 columns
    const double *A;             // shared term, ca * A[p,q,r,s]
    long long sa[4];
    double ca;
    const double *B;             // per-batch terms c1 B[p,q,r,s] + c2 B[with strides sb2]
    long long sb1[4], sb2[4], bst;
    double c1, c2;
    int sh;                      // spin-sorted pair order; only same-type pairs written
};

// one block per (batch, p<q), threads over the (a<b) pairs
__global__ void __launch_bounds__(256)
pair_gather_kernel(long long nblk, PairGather g, double *__restrict__ out) {
    for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
        const long long y = blk / g.P1;
        int p, q;
        const PairOrder o1{g.n1, g.sh}, o2{g.n2, g.sh};
        o1.decode((int)(blk - y * g.P1), p, q);
        const double *Ar = g.A ? g.A + p * g.sa[0] + q * g.sa[1] : nullptr;
        const double *Bb = g.B ? g.B + y * g.bst : nullptr;
        const double *B1 = Bb ? Bb + p * g.sb1[0] + q * g.sb1[1] : nullptr;
        const double *B2 = Bb ? Bb + p * g.sb2[0] + q * g.sb2[1] : nullptr;
        double *o = out + blk * g.P2;
        int lo = 0, hi = g.P2;
        if (g.sh) o2.range((p >= g.sh) + (q >= g.sh), lo, hi);
        for (int x = lo + threadIdx.x; x < hi; x += blockDim.x) {
            int a, b;
            o2.decode(x, a, b);
            double v = 0.0;
            if (Ar) v = g.ca * Ar[a * g.sa[2] + b * g.sa[3]];
            if (Bb) {
                v += g.c1 * B1[a * g.sb1[2] + b * g.sb1[3]];
                if (g.c2 != 0.0) v += g.c2 * B2[a * g.sb2[2] + b * g.sb2[3]];
            }
            o[x] = v;
        }
    }
}

}  // namespace

int kv_axpby4(kvft_ctx *ctx, int batch, const int dims[4], double alpha,
              const double *src, const long long ss[4], long long sbst,
              double beta, double *dst, const long long ds[4], long long dbst) {
    Dims4 g;
    long long total = batch;
    for (int k = 0; k < 4; k++) {
        g.d[k] = dims[k];
        g.ss[k] = ss[k];
        g.ds[k] = ds[k];
        total *= dims[k];
    }
    g.sbst = sbst;
    g.dbst = dbst;
    if (total == 0) return KVFT_OK;
    if (ctx->dry) {
        KvDryOp op;
        op.kind = 1;
        op.batch = batch, op.alpha = alpha, op.beta = beta;
        for (int k = 0; k < 4; k++) op.dims[k] = dims[k], op.ss[k] = ss[k], op.ds[k] = ds[k];
        op.sbst = sbst, op.dbst = dbst, op.src = src, op.dst = dst;
        ctx->dry->push_back(op);
        return KVFT_OK;
    }
    KvProfScope prof(ctx, KV_CAT_ELEM, 8.0 * total * (beta != 0.0 ? 3 : 2));
    const long long nblk = (long long)batch * dims[0] * dims[1] *
                           (((long long)dims[2] * dims[3] + AX_CHUNK - 1) / AX_CHUNK);
    const unsigned grid = (unsigned)std::min(nblk, (long long)ctx->sm_count * 16);
    if (beta == 0.0 && (alpha == 1.0 || alpha == -1.0))
        axpby4_kernel<0><<<grid, 256, 0, ctx->stream>>>(nblk, g, alpha, src, beta, dst);
    else if (beta == 0.0)
        axpby4_kernel<1><<<grid, 256, 0, ctx->stream>>>(nblk, g, alpha, src, beta, dst);
    else
        axpby4_kernel<2><<<grid, 256, 0, ctx->stream>>>(nblk, g, alpha, src, beta, dst);
    return kv_launch_check(ctx, "axpby4");
}

int kv_make_tau(kvft_ctx *ctx, int batch, int nv, int no, const double *t1,
                const double *t2, double c, double *out, int spin_half) {
    long long total = (long long)batch * nv * nv * no * no;
    if (total == 0) return KVFT_OK;
    KvProfScope prof(ctx, KV_CAT_ELEM, 16.0 * total * kv_spin_frac(nv, no, spin_half));
    const long long nblk = (long long)batch * nv * nv;
    if (no > 3072) return kv_fail(ctx, KVFT_EINVAL, "make_tau: more than 3072 occupied orbitals");
    const int sh = (nv == no && nv == 2 * spin_half) ? spin_half : 0;
    make_tau_kernel<<<(unsigned)std::min(nblk, (long long)ctx->sm_count * 16), 256,
                      2 * no * sizeof(double), ctx->stream>>>(nblk, nv, no, sh, t1, t2, c, out);
    return kv_launch_check(ctx, "make_tau");
}

int kv_make_wmbej_tmp(kvft_ctx *ctx, int batch, int nv, int no,
                      const double *t1, const double *t2, double *out, int spin_half) {
    long long total = (long long)batch * nv * nv * no * no;
    if (total == 0) return KVFT_OK;
    if (batch > 65535) return kv_fail(ctx, KVFT_EINVAL, "wmbej_tmp: batch too large");
    KvProfScope prof(ctx, KV_CAT_ELEM, 16.0 * total * kv_spin_frac(nv, no, spin_half));
    if (spin_half > 0 && nv == no && nv == 2 * spin_half) {
        const int nth = (spin_half + 31) / 32;
        const dim3 gs(2 * nth * nth, std::min(nv * no, 2048), batch);
        wmbej_tmp_spin_kernel<<<gs, 256, 0, ctx->stream>>>(nv, spin_half, t1, t2, out);
        return kv_launch_check(ctx, "wmbej_tmp_spin");
    }
    // each block walks several (b, j): short-lived blocks would leave the SMs
    // waiting for new ones
    const dim3 grid(((nv + 31) / 32) * ((no + 31) / 32), std::min(nv * no, 2048), batch);
    wmbej_tmp_kernel<<<grid, 256, 0, ctx->stream>>>(nv, no, t1, t2, out);
    return kv_launch_check(ctx, "wmbej_tmp");
}

int kv_assemble_t2(kvft_ctx *ctx, int batch, int nv, int no, double fac, const double *Z,
                   const double *Lc, double *T2, const double *seed, int spin_half) {
    const long long oo = (long long)no * no, total = (long long)batch * nv * nv * oo;
    if (total == 0) return KVFT_OK;
    if (seed) {
        // the a = b blocks get the seed alone: T2[y][a][a] = -seed[a][a]
        const int d[4] = {nv, no, no, 1};
        const long long sd[4] = {(nv + 1) * oo, no, 1, 0};
        KV_TRY(kv_axpby4(ctx, batch, d, -1.0, seed, sd, 0, 0.0, T2, sd, nv * nv * oo));
    }
    if (nv < 2) return KVFT_OK;
    if (batch > 65535) return kv_fail(ctx, KVFT_EINVAL, "assemble_t2: batch too large");
    const int sh = (nv == no && nv == 2 * spin_half) ? spin_half : 0;
    KvProfScope prof(ctx, KV_CAT_ELEM,
                     8.0 * total * (Lc ? 3.25 : 3.0) * kv_spin_frac(nv, no, sh));
    const int nt = (no + 31) / 32;
    const int pv = nv * (nv - 1) / 2;
    const dim3 grid(nt * (nt + 1) / 2, std::min(pv, 65535), batch);
#define KV_ASM(fs_, seed_)                                                                  \
    assemble_t2_kernel<fs_, seed_><<<grid, 256, 0, ctx->stream>>>(nv, no, sh, fac, Z, Lc, seed, \
                                                                  T2)
    const int fs = fac == 1.0 ? 1 : (fac == -1.0 ? 2 : 0);
    if (seed && sh) {
        const int nth = (sh + 31) / 32;
        const dim3 gs(nth * nth, std::min(pv, 65535), batch);
        if (fs == 1)
            assemble_t2_spin_kernel<1><<<gs, 256, 0, ctx->stream>>>(nv, sh, fac, Z, Lc, seed, T2);
        else if (fs == 2)
            assemble_t2_spin_kernel<2><<<gs, 256, 0, ctx->stream>>>(nv, sh, fac, Z, Lc, seed, T2);
        else
            assemble_t2_spin_kernel<0><<<gs, 256, 0, ctx->stream>>>(nv, sh, fac, Z, Lc, seed, T2);
        return kv_launch_check(ctx, "assemble_t2_spin");
    }
    if (seed) {
        if (fs == 1) KV_ASM(1, true);
        else if (fs == 2) KV_ASM(2, true);
        else KV_ASM(0, true);
    } else {
        if (fs == 1) KV_ASM(1, false);
        else if (fs == 2) KV_ASM(2, false);
        else KV_ASM(0, false);
    }
#undef KV_ASM
    return kv_launch_check(ctx, "assemble_t2");
}

int kv_make_tau_pairs(kvft_ctx *ctx, int batch, int nv, int no, const double *t1,
                      const double *t2, double *out, int spin_half) {
    const int sh = (nv == no && nv == 2 * spin_half) ? spin_half : 0;
    const int pv = nv * (nv - 1) / 2, po = no * (no - 1) / 2;
    long long total = (long long)batch * pv * po;
    if (total == 0) return KVFT_OK;
    KvProfScope prof(ctx, KV_CAT_ELEM, 16.0 * total * kv_spin_frac(nv, no, sh));
    const long long nblk = (long long)batch * pv;
    make_tau_pairs_kernel<<<(unsigned)std::min(nblk, (long long)ctx->sm_count * 16), 256, 0,
                            ctx->stream>>>(nblk, nv, no, pv, po, sh, t1, t2, out);
    return kv_launch_check(ctx, "make_tau_pairs");
}

int kv_pair_gather(kvft_ctx *ctx, int batch, int n1, int n2, const double *A,
                   const long long sa[4], double ca, const double *B, const long long sb1[4],
                   double c1, const long long sb2[4], double c2, long long bst, double *out,
                   int spin_half) {
    PairGather g;
    g.sh = (n1 == n2 && n1 == 2 * spin_half) ? spin_half : 0;
    g.n1 = n1;
    g.n2 = n2;
    g.P1 = n1 * (n1 - 1) / 2;
    g.P2 = n2 * (n2 - 1) / 2;
    g.A = A;
    g.ca = ca;
    g.B = B;
    g.c1 = c1;
    g.c2 = c2;
    g.bst = bst;
    for (int k = 0; k < 4; k++) {
        g.sa[k] = sa ? sa[k] : 0;
        g.sb1[k] = sb1 ? sb1[k] : 0;
        g.sb2[k] = sb2 ? sb2[k] : 0;
    }
    long long total = (long long)batch * g.P1 * g.P2;
    if (total == 0) return KVFT_OK;
    KvProfScope prof(ctx, KV_CAT_ELEM,
                     8.0 * total * (B ? 3 : 2) * kv_spin_frac(n1, n2, g.sh));
    const long long nblk = (long long)batch * g.P1;
    pair_gather_kernel<<<(unsigned)std::min(nblk, (long long)ctx->sm_count * 16), 256, 0,
                         ctx->stream>>>(nblk, g, out);
    return kv_launch_check(ctx, "pair_gather");
}

int kv_bcast(kvft_ctx *ctx, int batch, size_t count, const double *src,
             double *dst) {
    long long total = (long long)batch * count;
    if (total == 0) return KVFT_OK;
    KvProfScope prof(ctx, KV_CAT_ELEM, 8.0 * total);
    bcast_kernel<<<grid_for(ctx, total, 256), 256, 0, ctx->stream>>>(total, (long long)count,
                                                                     src, dst);
    return kv_launch_check(ctx, "bcast");
}
