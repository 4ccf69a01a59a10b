// On-device builders of the model systems' antisymmetrised spin-orbital
// integrals <pq||rs> (the systems of kelvin/ueg_system.py + ueg_utils.py:83-138
// and kelvin/hubbard_system.py in their general-spin 'g' ordering: the alpha
// block of nb spatial orbitals, then the beta block).  Kelvin builds these
// n^4 tensors with Python loops; here one pass writes them at HBM speed.
//
// Both tensors follow the host formulas of kelvin_gb300/systems.py operation
// for operation, so the results are bit-identical to them:
//   UEG:     <pq|rs> = c / |n_p - n_r|^2  if s_p = s_r, s_q = s_s,
//                      n_p + n_q = n_r + n_s and n_p != n_r  (c = 4 pi / L^3
//                      * (2 pi / L)^-2, from the host), else 0;
//   Hubbard: <pq|rs> = u (= U / L)  if (s_p, s_q, s_r, s_s) is (a, b, a, b) or
//                      (b, a, b, a) and k_p + k_q - k_r - k_s = 0 mod L;
//   <pq||rs> = <pq|rs> - <pq|sr>.
#include "kvft_internal.h"

namespace {

constexpr int MAXNB = 512;          // plane waves (6 KB of kernel parameters)

struct PlaneWaves {
    int nb;
    int v[3 * MAXNB];        // integer wave vectors n_p
};

__device__ __forceinline__ double ueg_direct(const PlaneWaves &w, double c, int p, int q, int r,
                                             int s) {
    const int nb = w.nb;
    if ((p >= nb) != (r >= nb) || (q >= nb) != (s >= nb)) return 0.0;
    const int *np = w.v + 3 * (p % nb), *nq = w.v + 3 * (q % nb);
    const int *nr = w.v + 3 * (r % nb), *ns = w.v + 3 * (s % nb);
    int q2 = 0;
    for (int d = 0; d < 3; d++) {
        if (np[d] + nq[d] != nr[d] + ns[d]) return 0.0;
        const int dd = np[d] - nr[d];
        q2 += dd * dd;
    }
    return q2 > 0 ? c / (double)q2 : 0.0;
}

// one block per (p, q); its threads walk (r, s)
__global__ void __launch_bounds__(256)
ueg_eri_kernel(PlaneWaves w, double c, double *__restrict__ eri) {
    const int n = 2 * w.nb, n2 = n * n;
    for (int pq = blockIdx.x; pq < n2; pq += gridDim.x) {
        const int p = pq / n, q = pq % n;
        double *row = eri + (long long)pq * n2;
        for (int e = threadIdx.x; e < n2; e += blockDim.x) {
            const int r = e / n, s = e % n;
            row[e] = ueg_direct(w, c, p, q, r, s) - ueg_direct(w, c, p, q, s, r);
        }
    }
}

__device__ __forceinline__ double hub_direct(int L, double u, int p, int q, int r, int s) {
    const int sp = p / L, sq = q / L, sr = r / L, ss = s / L;
    if (!(sp == sr && sq == ss && sp != sq)) return 0.0;
    return ((p % L) + (q % L) - (r % L) - (s % L)) % L == 0 ? u : 0.0;
}

__global__ void __launch_bounds__(256)
hubbard_eri_kernel(int L, double u, double *__restrict__ eri) {
    const int n = 2 * L, n2 = n * n;
    for (int pq = blockIdx.x; pq < n2; pq += gridDim.x) {
        const int p = pq / n, q = pq % n;
        double *row = eri + (long long)pq * n2;
        for (int e = threadIdx.x; e < n2; e += blockDim.x) {
            const int r = e / n, s = e % n;
            row[e] = hub_direct(L, u, p, q, r, s) - hub_direct(L, u, p, q, s, r);
        }
    }
}

}  // namespace

extern "C" int kvft_ueg_eri(kvft_ctx *ctx, int nb, const int *nvec, double c, double *eri) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_ueg_eri: not on a dry-run context");
    if (!ctx || nb <= 0 || nb > MAXNB || !nvec || !eri)
        return kv_fail(ctx, KVFT_EINVAL, "ueg_eri: bad argument (1 <= nb <= 512)");
    cudaSetDevice(ctx->device);
    PlaneWaves w;
    w.nb = nb;
    for (int k = 0; k < 3 * nb; k++) w.v[k] = nvec[k];
    const int n = 2 * nb;
    KvProfScope prof(ctx, KV_CAT_ELEM, 8.0 * (double)n * n * n * n);
    ueg_eri_kernel<<<std::min(n * n, ctx->sm_count * 16), 256, 0, ctx->stream>>>(w, c, eri);
    return kv_launch_check(ctx, "ueg_eri");
}

extern "C" int kvft_hubbard_eri(kvft_ctx *ctx, int sites, double u, double *eri) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_hubbard_eri: not on a dry-run context");
    if (!ctx || sites <= 0 || sites > 4096 || !eri)
        return kv_fail(ctx, KVFT_EINVAL, "hubbard_eri: bad argument");
    cudaSetDevice(ctx->device);
    const int n = 2 * sites;
    KvProfScope prof(ctx, KV_CAT_ELEM, 8.0 * (double)n * n * n * n);
    hubbard_eri_kernel<<<std::min(n * n, ctx->sm_count * 16), 256, 0, ctx->stream>>>(sites, u,
                                                                                   eri);
    return kv_launch_check(ctx, "hubbard_eri");
}
