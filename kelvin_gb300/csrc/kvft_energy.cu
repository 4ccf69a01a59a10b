// FT-CC grand potential (kelvin/ft_cc_energy.py:7-32):
//   Omega = (1/beta) [ sum_ai t1n[a,i] f[i,a] + sum_abij t2n[a,b,i,j] eri[i,j,a,b] ]
//   t1n = sum_y g_y T1_y,  t2n = sum_y g_y (T2_y/4 + [Qterm] T1_y[a,i] T1_y[b,j]/2)
// One pass over T2 (HBM-bound apart from GB300's slow FP64 FMAs); eri is read
// through a shared-memory transpose so both streams stay coalesced.  Partial
// sums are reduced in a fixed order, so the result is deterministic.
#include "kvft_internal.h"

namespace {

constexpr int TILE = 32;

// One block per 32 x 32 tile of (a,b) x (i,j); thread (tx, ty) takes i,j =
// ij0 + tx and the four (a,b) rows ty + 8k.  Per element and tau point two
// FP64 FMAs: s1 += g_y T2_y and s2 += (g_y T1_y[a,i]) T1_y[b,j], the first
// factor of the second from a shared table over the few (a, i) values of the
// tile, filled for a chunk of tau points at a time; the element's weight is
// then s1/4 + s2/2.
constexpr int WTAB = 1024;                  // doubles of the (y, a, i) table

__global__ void __launch_bounds__(256, 2)
energy2_kernel(int ng, int nv, int no, const double *__restrict__ T1,
               const double *__restrict__ T2, const double *__restrict__ eri,
               const double *__restrict__ g, int qterm, int sh, double *__restrict__ partial) {
    __shared__ double E[TILE][TILE + 1];     // [ij][ab]
    __shared__ double red[256];
    __shared__ double gs[WTAB / 4];          // g_y of the chunk
    __shared__ double wt[WTAB];              // [y][a - a_lo][i - i_lo]: g_y T1_y[a,i]
    const long long V2 = (long long)nv * nv, O2 = (long long)no * no;
    const long long ab0 = (long long)blockIdx.y * TILE, ij0 = (long long)blockIdx.x * TILE;
    const int t = threadIdx.x, tx = t % TILE, ty = t / TILE;   // ty in [0, 8)
    if (sh > 0) {
        // spin blocks: a tile whose (a,b) spin sums and (i,j) spin sums never
        // meet holds only zero amplitudes and adds nothing
        __shared__ int live;
        if (t < 32) {
            const long long ab = ab0 + t, ij = ij0 + t;
            unsigned sab = 0, sij = 0;
            if (ab < V2) sab = 1u << ((int)(ab / nv >= sh) + (int)(ab % nv >= sh));
            if (ij < O2) sij = 1u << ((int)(ij / no >= sh) + (int)(ij % no >= sh));
            sab = __reduce_or_sync(0xffffffffu, sab);
            sij = __reduce_or_sync(0xffffffffu, sij);
            if (t == 0) live = (sab & sij) != 0;
        }
        __syncthreads();
        if (!live) {
            if (t == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = 0.0;
            return;
        }
    }
    for (int r = ty; r < TILE; r += 8) {
        long long ij = ij0 + r, ab = ab0 + tx;
        E[r][tx] = (ij < O2 && ab < V2) ? eri[ij * V2 + ab] : 0.0;
    }
    const long long ab_hi = min(ab0 + TILE, V2) - 1, ij_hi = min(ij0 + TILE, O2) - 1;
    const int a_lo = (int)(ab0 / nv), na = (int)(ab_hi / nv) - a_lo + 1;
    const int i_lo = (int)(ij0 / no), ni = (int)(ij_hi / no) - i_lo + 1;
    const int yc = qterm ? max(1, min(WTAB / 4, WTAB / (na * ni))) : WTAB / 4;
    const long long ij = ij0 + tx;
    const bool live = ij < O2;
    const int i = live ? (int)(ij / no) : 0, j = live ? (int)(ij % no) : 0;
    int ka[4], kb[4];
    long long kab[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const long long ab = min(ab0 + ty + 8 * k, ab_hi);
        kab[k] = ab;
        ka[k] = (int)(ab / nv);
        kb[k] = (int)(ab % nv);
    }
    double s1[4] = {0.0, 0.0, 0.0, 0.0}, s2[4] = {0.0, 0.0, 0.0, 0.0};
    const long long sy = (long long)nv * no;
    for (int y0 = 0; y0 < ng; y0 += yc) {
        const int ny = min(yc, ng - y0);
        __syncthreads();
        for (int x = t; x < ny; x += 256) gs[x] = g[y0 + x];
        if (qterm)
            for (int x = t; x < ny * na * ni; x += 256) {
                const int yy = x / (na * ni), r = x % (na * ni);
                const int a = a_lo + r / ni, ii = i_lo + r % ni;
                wt[x] = g[y0 + yy] * T1[(y0 + yy) * sy + (long long)a * no + ii];
            }
        __syncthreads();
        if (!live) continue;
        const double *t2 = T2 + (long long)y0 * V2 * O2 + ij;
        for (int yy = 0; yy < ny; yy++) {
            const double gy = gs[yy];
#pragma unroll
            for (int k = 0; k < 4; k++) s1[k] = fma(gy, t2[kab[k] * O2], s1[k]);
            t2 += V2 * O2;
        }
        if (qterm) {
            const double *u = T1 + (long long)y0 * sy + j;
            const double *w = wt + (i - i_lo);
            for (int yy = 0; yy < ny; yy++) {
#pragma unroll
                for (int k = 0; k < 4; k++)
                    s2[k] = fma(w[(ka[k] - a_lo) * ni], u[(long long)kb[k] * no], s2[k]);
                u += sy;
                w += na * ni;
            }
        }
    }
    double acc = 0.0;
    if (live)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = ty + 8 * k;
            if (ab0 + r < V2) acc = fma(fma(0.25, s1[k], 0.5 * s2[k]), E[tx][r], acc);
        }
    red[t] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (t < s) red[t] += red[t + s];
        __syncthreads();
    }
    if (t == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// Spin blocks (nv = no = 2h): only the spin-conserving (a, b, i, j) carry
// amplitudes and integrals.  Item (a, i, q) is one h x h block of (b, j): with
// s_a = s_i the blocks s_b = s_j = q (q = 0, 1), otherwise the one block
// s_b = s_i, s_j = s_a (q = 0; q = 1 is empty).  The block's integrals
// eri[i][j][a][b] are read along b into shared memory and its amplitudes
// T2_y[a][b][i][j] along j, so both streams are coalesced and no element
// outside the conserving blocks is read.  The T1 T1 term vanishes unless s_b
// = s_j (T1 is spin-diagonal), i.e. on the s_a = s_i items.  One partial sum
// per item, reduced in a fixed order.
constexpr int ESP_HMAX = 96;                 // h x (h + 1) doubles of shared memory

__global__ void __launch_bounds__(256)
energy2_spin_kernel(int ng, int n, int h, const double *__restrict__ T1,
                    const double *__restrict__ T2, const double *__restrict__ eri,
                    const double *__restrict__ g, int qterm, long long items,
                    double *__restrict__ partial) {
    extern __shared__ double E[];            // [h][h + 1]: E[j1][b1]
    __shared__ double red[256];
    __shared__ double gs[64], w[64];         // g_y and g_y T1_y[a][i]
    const int t = threadIdx.x, hh = h * h, ld = h + 1;
    const long long n2 = (long long)n * n, P = n2 * n2;
    for (long long it = blockIdx.x; it < items; it += gridDim.x) {
        const int q = (int)(it & 1);
        const long long ai = it >> 1;
        const int a = (int)(ai / n), i = (int)(ai - (long long)a * n);
        const int sa = a >= h, si = i >= h;
        double acc = 0.0;
        if (sa == si || q == 0) {            // block-uniform
            const int sb = sa == si ? q : si, sj = sa == si ? q : sa;
            const bool tt = qterm && sa == si;
            __syncthreads();                 // E, gs, w of the last item are used up
            for (int x = t; x < ng; x += 256) {
                gs[x] = g[x];
                w[x] = tt ? g[x] * T1[(long long)x * n2 + (long long)a * n + i] : 0.0;
            }
            for (int x = t; x < hh; x += 256) {
                const int j1 = x / h, b1 = x - j1 * h;
                E[j1 * ld + b1] = eri[(((long long)i * n + sj * h + j1) * n + a) * n + sb * h + b1];
            }
            __syncthreads();
            const long long base = ((long long)a * n + sb * h) * n2 + (long long)i * n + sj * h;
            for (int x = t; x < hh; x += 256) {
                const int b1 = x / h, j1 = x - b1 * h;
                const double *t2 = T2 + base + (long long)b1 * n2 + j1;
                double s1 = 0.0, s2 = 0.0;
                for (int y = 0; y < ng; y++) s1 = fma(gs[y], t2[(long long)y * P], s1);
                if (tt) {
                    const double *u = T1 + (long long)(sb * h + b1) * n + sj * h + j1;
                    for (int y = 0; y < ng; y++) s2 = fma(w[y], u[(long long)y * n2], s2);
                }
                acc = fma(fma(0.25, s1, 0.5 * s2), E[j1 * ld + b1], acc);
            }
        }
        red[t] = acc;
        __syncthreads();
        for (int st = 128; st > 0; st >>= 1) {
            if (t < st) red[t] += red[t + st];
            __syncthreads();
        }
        if (t == 0) partial[it] = red[0];
    }
}

__global__ void energy1_kernel(int ng, int nv, int no, const double *__restrict__ T1,
                               const double *__restrict__ f, const double *__restrict__ g,
                               double *__restrict__ out) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int k = threadIdx.x; k < nv * no; k += 256) {
        const int a = k / no, i = k % no;
        double s = 0.0;
        for (int y = 0; y < ng; y++) s = fma(g[y], T1[(long long)y * nv * no + k], s);
        acc = fma(s, f[i * nv + a], acc);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

__global__ void energy_final_kernel(const double *__restrict__ partial, int n,
                                    const double *__restrict__ e1, double inv_beta,
                                    double *__restrict__ res) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) acc += partial[k];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *res = (e1[0] + red[0]) * inv_beta;
}

}  // namespace

// Writes Omega to dres[0] (device).  Uses context scratch.
int kv_energy(kvft_ctx *ctx, int ng, int nv, int no, const double *T1, const double *T2,
              const double *f, const double *eri, const double *g, double beta, int qterm,
              double *dres, int spin_half) {
    const long long V2 = (long long)nv * nv, O2 = (long long)no * no;
    dim3 grid((unsigned)((O2 + TILE - 1) / TILE), (unsigned)((V2 + TILE - 1) / TILE));
    const int sh = (nv == no && nv == 2 * spin_half) ? spin_half : 0;
    const bool spin = sh > 0 && sh <= ESP_HMAX && ng <= 64;
    // spin items (a, i, q), or the 32 x 32 tiles of the dense kernel
    const long long nblk = spin ? 2LL * nv * nv : (long long)grid.x * grid.y;
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "energy_partial", sizeof(double) * (nblk + 1), &part));
    double *pp = (double *)part;
    // algorithmic bytes: T2 (all tau points) + eri + T1; with spin blocks the
    // spin-conserving elements of T2 and eri
    KvProfScope prof(ctx, KV_CAT_ENERGY,
                     8.0 * (((double)ng * V2 * O2 + (double)V2 * O2) * kv_spin_frac(nv, no, sh) +
                            (double)ng * nv * no));
    if (spin) {
        const size_t smem = sizeof(double) * (size_t)sh * (sh + 1);
        static bool attr = false;
        if (!attr) {
            KV_CHECK(ctx, cudaFuncSetAttribute(energy2_spin_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)(sizeof(double) * ESP_HMAX * (ESP_HMAX + 1))));
            attr = true;
        }
        const int gb = (int)std::min<long long>(nblk, (long long)ctx->sm_count * 8);
        energy2_spin_kernel<<<gb, 256, smem, ctx->stream>>>(ng, nv, sh, T1, T2, eri, g, qterm,
                                                           nblk, pp);
        KV_TRY(kv_launch_check(ctx, "energy2_spin"));
    } else {
        energy2_kernel<<<grid, 256, 0, ctx->stream>>>(ng, nv, no, T1, T2, eri, g, qterm, sh, pp);
        KV_TRY(kv_launch_check(ctx, "energy2"));
    }
    energy1_kernel<<<1, 256, 0, ctx->stream>>>(ng, nv, no, T1, f, g, pp + nblk);
    KV_TRY(kv_launch_check(ctx, "energy1"));
    energy_final_kernel<<<1, 256, 0, ctx->stream>>>(pp, (int)nblk, pp + nblk, 1.0 / beta, dres);
    return kv_launch_check(ctx, "energy_final");
}

extern "C" int kvft_ft_cc_energy(kvft_ctx *ctx, int ng, int nv, int no, const double *T1,
                                 const double *T2, const double *f, const double *eri,
                                 const double *g, double beta, int qterm,
                                 double *omega_host) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_ft_cc_energy: not on a dry-run context");
    if (!ctx || ng < 1 || nv <= 0 || no <= 0 || !T1 || !T2 || !f || !eri || !g || !omega_host ||
        beta == 0.0)
        return kv_fail(ctx, KVFT_EINVAL, "ft_cc_energy: bad argument");
    cudaSetDevice(ctx->device);
    void *res = nullptr;
    KV_TRY(kv_scratch(ctx, "energy_result", sizeof(double), &res));
    KV_TRY(kv_energy(ctx, ng, nv, no, T1, T2, f, eri, g, beta, qterm, (double *)res));
    KV_CHECK(ctx, cudaMemcpyAsync(omega_host, res, sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return KVFT_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free energy reduction.
//
// Some callers cannot let a library call cudaMalloc: a host process that has
// handed (nearly) all device memory to its own pool, a serving loop whose
// latency budget has no room for the device-wide synchronisation cudaMalloc
// and cudaFree can imply, or a plugin host that forbids allocations outside
// its allocator.  kvft_ft_cc_energy_noalloc computes the same grand
// potential as kvft_ft_cc_energy without any allocation: the per-tile
// partial sums live in the file-scope array below, which every GPU that loads
// libkvft holds (256 KiB) until the process exits.  Its device address is
// looked up with cudaGetSymbolAddress once per device, on that device's first
// call, so that first call should come before any stream capture.  All calls
// on a device share the array and every call overwrites the slots it reads,
// so nothing has to be cleared between calls; two calls that overlap on the
// GPU (different streams, no ordering) race on it.
// ---------------------------------------------------------------------------
#include <mutex>

namespace {
constexpr int NOALLOC_MAX_TILES = 32767;   // 32 x 32 tiles of (a,b) x (i,j)
__device__ __align__(256) double g_energy_scratch[NOALLOC_MAX_TILES + 1];
std::mutex g_energy_scratch_mu;
double *g_energy_scratch_ptr[64] = {};     // device address of the array, per device
}  // namespace

extern "C" int kvft_ft_cc_energy_noalloc(void *stream, int ng, int nv, int no,
                                         const double *T1, const double *T2,
                                         const double *f, const double *eri,
                                         const double *g, double beta, int qterm,
                                         double *omega_dev) {
    if (ng < 1 || nv <= 0 || no <= 0 || !T1 || !T2 || !f || !eri || !g || !omega_dev ||
        beta == 0.0)
        return KVFT_EINVAL;
    const long long V2 = (long long)nv * nv, O2 = (long long)no * no;
    const long long gx = (O2 + TILE - 1) / TILE, gy = (V2 + TILE - 1) / TILE;
    if (gx * gy > NOALLOC_MAX_TILES) return KVFT_EINVAL;   // beyond the static scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return KVFT_EDEVICE;
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_energy_scratch_mu);
        if (!g_energy_scratch_ptr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_energy_scratch) != cudaSuccess || !p)
                return KVFT_EDEVICE;
            g_energy_scratch_ptr[dev] = (double *)p;
        }
        scratch = g_energy_scratch_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int nblk = (int)(gx * gy);
    // each launch's own status (cudaLaunchKernel reports that launch), so
    // that an earlier unrelated error left on the thread is not returned as
    // this call's
    int sh = 0;
    double *part1 = scratch + nblk;
    double inv_beta = 1.0 / beta;
    void *a2[] = {&ng, &nv, &no, (void *)&T1, (void *)&T2, (void *)&eri, (void *)&g, &qterm,
                  &sh, &scratch};
    void *a1[] = {&ng, &nv, &no, (void *)&T1, (void *)&f, (void *)&g, &part1};
    int nb = nblk;
    void *af[] = {&scratch, &nb, &part1, &inv_beta, &omega_dev};
    if (cudaLaunchKernel((const void *)energy2_kernel, dim3((unsigned)gx, (unsigned)gy),
                         dim3(256), a2, 0, st) != cudaSuccess ||
        cudaLaunchKernel((const void *)energy1_kernel, dim3(1), dim3(256), a1, 0, st) !=
            cudaSuccess ||
        cudaLaunchKernel((const void *)energy_final_kernel, dim3(1), dim3(256), af, 0, st) !=
            cudaSuccess)
        return KVFT_EDEVICE;
    return KVFT_OK;
}
