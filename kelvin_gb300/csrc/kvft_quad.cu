// Exp-weighted cumulative tau integrals (kelvin/quadrature.py:292-317,
// 348-369) and the fused "integrate + damp + norms" pass of the solver.
//
// For every amplitude element p with denominator d:
//     T_y = sum_x G[y,x] w(y,x) tbar_x,
//     w(y,x) = exp((ti[x]-ti[y]) d) for x < y (all x if `full`), else 1.
// GB300 issues about two FP64 FMAs per clock per SM, so exp evaluations are
// the cost to cut, not HBM bytes:
//   * w(y,x) is built as a running product of step factors
//     r_k = exp((ti[k]-ti[k+1]) d), one exp per grid step -- and a single exp
//     when the grid is uniform (Kelvin's default 'lin' rule);
//   * when G has the structure of Kelvin's Simpson/midpoint/left rules
//     (G[y,x] == G[y-s,x] for x < y-s, zero above the diagonal), rows are
//     chained: T_y = w(y,y-s) (T_{y-s} - G[y-s,y-s] tbar_{y-s})
//                    + sum_{x=y-s}^{y} G[y,x] w(y,x) tbar_x,
//     which is O(ng) per element instead of O(ng^2).
// The product of <= ng correctly rounded factors differs from a direct exp
// by at most ~ng ulp (relative), far inside the 1e-10 parity tolerance.
#include "kvft_internal.h"

#include <cmath>

namespace {

constexpr int QT = 128;      // threads per block
constexpr int MAXNG = 64;

struct QuadParams {
    int ng;
    long long P;             // elements per tau slice
    int rank;                // 1: [nv][no], 2: [nv][nv][no][no]
    int nv, no;
    int step;                // recurrence step (0: general path)
    int uniform;             // all ti[k+1]-ti[k] equal
    int full;
    int symmetric;           // ti[x] + ti[ng-1-x] the same for every x
    double alpha;            // damping (fused update only)
    int spin_half;           // fused update over the spin-conserving elements only (0: all)
};

__device__ __forceinline__ double denom(const QuadParams &q, long long p,
                                        const double *D, const double *ev,
                                        const double *eo) {
    if (D) return D[p];
    if (q.rank == 1) {
        int i = (int)(p % q.no);
        int a = (int)(p / q.no);
        return ev[a] - eo[i];
    }
    long long r = p;
    int j = (int)(r % q.no); r /= q.no;
    int i = (int)(r % q.no); r /= q.no;
    int b = (int)(r % q.nv);
    int a = (int)(r / q.nv);
    return ev[a] + ev[b] - eo[i] - eo[j];
}

// Shared memory: ti[ng], G[ng*ng], the chained-row coefficients cs[ng]
// (G[y,y-s] - G[y-s,y-s]), g1[ng] (G[y,y-1]) and gd[ng] (G[y,y]), then the
// per-thread columns r[ng][QT] (non-uniform grids) and tb[ng][QT] (general
// path).
// |x| as a float (mantissa truncated), from the FP64 bit pattern with
// integer operations: GB300's FP64 pipe, not its integer or FP32 pipes, is
// the scarce unit of this kernel.  Below 2^-126 the result is 0; above the
// float range it is infinity (NaN stays NaN).
__device__ __forceinline__ float abs_to_f32(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7FF) - 1023 + 127;
    if (e <= 0) return 0.f;
    if (e >= 255) {
        const bool nan = (hi & 0x7FF00000u) == 0x7FF00000u && (((hi & 0xFFFFFu) | lo) != 0);
        return __int_as_float(nan ? 0x7FC00000 : 0x7F800000);
    }
    return __int_as_float((e << 23) | (int)((hi & 0xFFFFFu) << 3) | (int)(lo >> 29));
}

// MODE 0: out = T.  MODE 1 (fused solver update): Told = alpha Told + (1-alpha) T,
// with block partial sums of |T - Told|^2 and |Told_new|^2.  Those two norms
// only steer convergence: each element's sum over tau points is taken in
// FP32 (relative error ~1e-7) and added to FP64 block sums.  UNI: uniform
// grid, one step factor for every step.
template <int MODE, bool UNI>
__global__ void __launch_bounds__(QT)
quad_kernel(QuadParams q, const double *__restrict__ tbar, const double *__restrict__ ti_g,
            const double *__restrict__ G_g, const double *__restrict__ D,
            const double *__restrict__ ev, const double *__restrict__ eo,
            double *out, double *__restrict__ partial) {
    extern __shared__ double sm[];
    const int ng = q.ng;
    double *ti = sm;
    double *G = ti + ng;
    double *cs = G + ng * ng, *g1 = cs + ng, *gd = g1 + ng;
    double *rk = gd + ng;                                  // [ng][QT]
    double *tb = rk + (q.uniform ? 0 : ng * QT);           // [ng][QT]
    for (int k = threadIdx.x; k < ng; k += QT) ti[k] = ti_g[k];
    for (int k = threadIdx.x; k < ng * ng; k += QT) G[k] = G_g[k];
    for (int y = threadIdx.x; y < ng; y += QT) {
        const int sy = q.step > 0 ? q.step : 1;
        cs[y] = (y >= sy) ? G_g[y * ng + y - sy] - G_g[(y - sy) * ng + y - sy] : 0.0;
        g1[y] = (y >= 1) ? G_g[y * ng + y - 1] : 0.0;
        gd[y] = G_g[y * ng + y];
    }
    __syncthreads();
    const double oma = 1.0 - q.alpha;

    double s_diff = 0.0, s_norm = 0.0;
    const int t = threadIdx.x;
    auto element = [&](long long p) {
        const double d = denom(q, p, D, ev, eo);
        // step factors r_k = exp((ti[k]-ti[k+1]) d)
        double r0 = 1.0;
        if (UNI) {
            r0 = (ng > 1) ? exp((ti[0] - ti[1]) * d) : 1.0;
        } else {
            for (int k = 0; k + 1 < ng; k++) rk[k * QT + t] = exp((ti[k] - ti[k + 1]) * d);
        }
        const double r02 = r0 * r0;
        float f_diff = 0.f, f_norm = 0.f;
#define RK(k) (UNI ? r0 : rk[(k) * QT + t])
        if (q.step > 0) {
            // chained rows; keep the last `step` outputs and inputs in registers
            double Tm1 = 0.0, Tm2 = 0.0, tbm1 = 0.0, tbm2 = 0.0;
            for (int y = 0; y < ng; y++) {
                const double tby = tbar[(long long)y * q.P + p];
                double Ty;
                if (y < q.step) {
                    // direct: x in [0, y]
                    Ty = G[y * ng + y] * tby;
                    double w = 1.0;
                    for (int x = y - 1; x >= 0; x--) {
                        w *= RK(x);
                        const double v = (x == y - 1) ? tbm1 : tbm2;
                        Ty = fma(G[y * ng + x] * w, v, Ty);
                    }
                } else if (q.step == 1) {
                    // T_y = w (T_{y-1} - G[y-1,y-1] tb_{y-1}) + G[y,y-1] w tb_{y-1}
                    //       + G[y,y] tb_y
                    Ty = fma(gd[y], tby, RK(y - 1) * fma(cs[y], tbm1, Tm1));
                } else {  // step 2
                    const double w1 = RK(y - 1);
                    const double w2 = UNI ? r02 : w1 * RK(y - 2);
                    Ty = fma(gd[y], tby, fma(g1[y] * w1, tbm1, w2 * fma(cs[y], tbm2, Tm2)));
                }
                if (MODE == 0) {
                    out[(long long)y * q.P + p] = Ty;
                } else {
                    // damped update Told + (1 - alpha)(T - Told) and the norms
                    double *o = out + (long long)y * q.P + p;
                    const double told = *o;
                    const double df = Ty - told;
                    const double nt = fma(oma, df, told);
                    const float fd = abs_to_f32(df), fn = abs_to_f32(nt);
                    f_diff = fmaf(fd, fd, f_diff);
                    f_norm = fmaf(fn, fn, f_norm);
                    *o = nt;
                }
                Tm2 = Tm1; Tm1 = Ty;
                tbm2 = tbm1; tbm1 = tby;
            }
        } else {
            for (int x = 0; x < ng; x++) tb[x * QT + t] = tbar[(long long)x * q.P + p];
            for (int y = 0; y < ng; y++) {
                double Ty = 0.0;
                // x <= y: running product downward from x = y
                double w = 1.0;
                for (int x = y; x >= 0; x--) {
                    if (x < y) w *= RK(x);
                    const double gyx = G[y * ng + x];
                    if (gyx != 0.0) Ty = fma(gyx * w, tb[x * QT + t], Ty);
                }
                // x > y: factor 1 (the reference's rule; dense grids with
                // the exponential for every pair run quad_dense_kernel)
                for (int x = y + 1; x < ng; x++) {
                    const double gyx = G[y * ng + x];
                    if (gyx != 0.0) Ty = fma(gyx, tb[x * QT + t], Ty);
                }
                if (MODE == 0) {
                    out[(long long)y * q.P + p] = Ty;
                } else {
                    double *o = out + (long long)y * q.P + p;
                    const double told = *o;
                    const double df = Ty - told;
                    const double nt = fma(oma, df, told);
                    const float fd = abs_to_f32(df), fn = abs_to_f32(nt);
                    f_diff = fmaf(fd, fd, f_diff);
                    f_norm = fmaf(fn, fn, f_norm);
                    *o = nt;
                }
            }
        }
#undef RK
        if (MODE == 1) {
            s_diff += (double)f_diff;
            s_norm += (double)f_norm;
        }
    };
    if (q.spin_half > 0) {
        // spin blocks: only the spin-conserving elements move (the others
        // are zero and stay zero); each (a, b, i) row holds them as one run
        // of h consecutive j or none, and one warp takes one run
        const int h = q.spin_half, n = q.no;
        const long long rows = q.P / n;
        const int lane = t % 32;
        const long long tw = (long long)gridDim.x * (QT / 32);
        for (long long u = blockIdx.x * (long long)(QT / 32) + t / 32; u < 2 * rows; u += tw) {
            const long long r = u >> 1;
            const int jh = (int)(u & 1);
            const int i = (int)(r % n);
            const long long ab = r / n;
            const int b = (int)(ab % n), a = (int)(ab / n);
            if ((a >= h) + (b >= h) != (i >= h) + jh) continue;
            for (int jj = lane; jj < h; jj += 32) element(r * n + (long long)jh * h + jj);
        }
    } else {
        for (long long p = blockIdx.x * (long long)QT + t; p < q.P;
             p += (long long)gridDim.x * QT)
            element(p);
    }
    if (MODE == 1) {
        // block reduction of the two sums (fixed order: deterministic)
        __shared__ double red[2][QT];
        red[0][t] = s_diff;
        red[1][t] = s_norm;
        __syncthreads();
        for (int s = QT / 2; s > 0; s >>= 1) {
            if (t < s) {
                red[0][t] += red[0][t + s];
                red[1][t] += red[1][t + s];
            }
            __syncthreads();
        }
        if (t == 0) {
            partial[2 * blockIdx.x] = red[0][0];
            partial[2 * blockIdx.x + 1] = red[1][0];
        }
    }
}

// ---------------------------------------------------------------------------
// Dense G (Gauss-Legendre grids; the backward Lambda integral):
//     T_y = sum_x G[y,x] exp((ti[x]-ti[y]) d) tbar_x   for every x.
// Factorised about the grid's centre tc, exp((ti[x]-ti[y]) d) = E_x / E_y with
// E_x = exp((ti[x]-tc) d), so T_y = (1/E_y) sum_x G[y,x] u_x, u_x = E_x tbar_x.
// GB300 has ~64x more FP32 than FP64 throughput, so:
//   * no exponentials per element: d = e_a + e_b - e_i - e_j, and E_x, 1/E_y
//     are products of a pair table of the virtual indices and one of the
//     occupied indices (quad_tables_kernel, exps of the orbital energies);
//   * the ng^2 sum runs in compensated FP32: u (scaled by a power of two to
//     order one) and G split into FP32 high and low parts; the high products
//     are summed with error-free two-sums and their rounding errors, the
//     cross terms and the sum's errors go to a second FP32 accumulator
//     (relative error ~1e-14 of sum |G u|, far inside the parity bounds).
// An element whose factors leave the safe range (non-finite u, or a bound on
// |T_y| near the FP64 limit), and every element when D is given explicitly,
// takes the FP64 path: exps, E_{ng-1-x} = 1/E_x on a grid symmetric about tc,
// and FP64 FMAs.
// ---------------------------------------------------------------------------
struct DenseTabs {
    const double *v, *vi, *o, *oi;   // [ng][NL] / [ng][NR]: E and 1/E factors
    long long NL, NR;                // p = l NR + r
};

// tables: v[x][l] = exp((ti[x]-tc)(e_a (+ e_b))), vi = its inverse,
// o[x][r] = exp(-(ti[x]-tc)(e_i (+ e_j))), oi = its inverse; l = a (rank 1)
// or a nv + b (rank 2), r = i or i no + j
__global__ void quad_tables_kernel(int ng, int rank, int nv, int no, double tc,
                                   const double *__restrict__ ti, const double *__restrict__ ev,
                                   const double *__restrict__ eo, long long NL, long long NR,
                                   double *__restrict__ tab) {
    const long long per = NL + NR;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < ng * per;
         k += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(k / per);
        const long long c = k - x * per;
        const double dt = ti[x] - tc;
        double e;
        if (c < NL)
            e = (rank == 2) ? ev[c / nv] + ev[c % nv] : ev[c];
        else
            e = (rank == 2) ? -(eo[(c - NL) / no] + eo[(c - NL) % no]) : -eo[c - NL];
        const double f = exp(dt * e), fi = exp(-dt * e);
        if (c < NL) {
            tab[x * NL + c] = f;
            tab[ng * NL + x * NL + c] = fi;
        } else {
            tab[2 * ng * NL + x * NR + (c - NL)] = f;
            tab[2 * ng * NL + ng * NR + x * NR + (c - NL)] = fi;
        }
    }
}

// s + e == a + b exactly (FP32 round to nearest)
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Biased exponent field of x (0: zero or subnormal, 0x7FF: inf or NaN).
__device__ __forceinline__ int dexp(double x) {
    return (__double2hiint(x) >> 20) & 0x7FF;
}

// x 2^-k as an FP32 pair hi + lo, from the bit pattern with integer
// operations (hi: the sign, exponent and top 23 mantissa bits; lo: the
// remaining 29 bits, rounded to 24), |x 2^-k - hi - lo| <= 2^-47 |x 2^-k|.
// For |x 2^-k| < 2: parts below 2^-126 are dropped (absolute error below
// 2^-126 of the scale 1).
__device__ __forceinline__ float2 dsplit_scaled(double x, int k) {
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const int e = (int)((hw >> 20) & 0x7FF) - 1023 - k;      // unbiased exponent of x 2^-k
    if (((hw >> 20) & 0x7FF) == 0 || e < -126) return make_float2(0.f, 0.f);
    const unsigned sg = hw & 0x80000000u;
    const float hi = __uint_as_float(sg | ((unsigned)(e + 127) << 23) | ((hw & 0xFFFFFu) << 3) |
                                     (lw >> 29));
    const unsigned rem = lw & 0x1FFFFFFFu;                   // 29 low mantissa bits
    float lo = 0.f;
    if (rem != 0 && e - 52 >= -126)
        lo = __uint_as_float(sg | __float_as_uint(__uint2float_rn(rem) *
                                                  __uint_as_float((unsigned)(e - 52 + 127) << 23)));
    return make_float2(hi, lo);
}

// (double) f 2^k for a finite float f, by integer operations on the bit
// pattern: 0 stays 0, a result below 2^-1022 is 0 (an absolute error far
// below anything the integral resolves), one above the FP64 range infinite.
__device__ __forceinline__ double f32_to_f64_scaled(float f, int k) {
    const unsigned u = __float_as_uint(f);
    const int E = (int)((u >> 23) & 0xFF);
    const int eb = E - 127 + 1023 + k;                       // biased FP64 exponent
    if (E == 0 || eb <= 0) return 0.0;                       // zero, float subnormals, underflow
    const unsigned sg = u & 0x80000000u;
    if (eb >= 0x7FF) return __hiloint2double((int)(sg | 0x7FF00000u), 0);
    const unsigned hw = sg | ((unsigned)eb << 20) | ((u >> 3) & 0xFFFFFu);
    return __hiloint2double((int)hw, (int)(u << 29));
}

template <int MODE>
__global__ void __launch_bounds__(QT)
quad_dense_kernel(QuadParams q, DenseTabs tb_, const double *__restrict__ tbar,
                  const double *__restrict__ ti_g, const double *__restrict__ G_g,
                  const double *__restrict__ D, const double *__restrict__ ev,
                  const double *__restrict__ eo, double *out, double *__restrict__ partial) {
    extern __shared__ double sm[];
    const int ng = q.ng;
    double *ti = sm;
    double *G = ti + ng;                                   // [ng][ng] FP64
    float *Gh = reinterpret_cast<float *>(G + ng * ng);    // [ng][ng] FP32 high part
    float *Gl = Gh + ng * ng;                              //          low part
    double *c0 = G + ng * ng + ng * ng;                    // [ng][QT]: u (FP64 or FP32 pair)
    double *c1 = c0 + ng * QT;                             // [ng][QT]: E (FP64 path)
    for (int k = threadIdx.x; k < ng; k += QT) ti[k] = ti_g[k];
    for (int k = threadIdx.x; k < ng * ng; k += QT) {
        const double g = G_g[k];
        G[k] = g;
        const float h = (float)g;
        Gh[k] = h;
        Gl[k] = (float)(g - (double)h);
    }
    __syncthreads();
    const double oma = 1.0 - q.alpha;
    const double tc = 0.5 * (ti[0] + ti[ng - 1]);
    double s_diff = 0.0, s_norm = 0.0;
    const int t = threadIdx.x;
    float2 *uf = reinterpret_cast<float2 *>(c0);

    auto emit = [&](long long p, int y, double Ty, float &f_diff, float &f_norm) {
        if (MODE == 0) {
            out[(long long)y * q.P + p] = Ty;
        } else {
            double *o = out + (long long)y * q.P + p;
            const double told = *o;
            const double df = Ty - told;
            const double nt = fma(oma, df, told);
            const float fd = abs_to_f32(df), fn = abs_to_f32(nt);
            f_diff = fmaf(fd, fd, f_diff);
            f_norm = fmaf(fn, fn, f_norm);
            *o = nt;
        }
    };

    auto element = [&](long long p) {
        float f_diff = 0.f, f_norm = 0.f;
        bool table = tb_.v != nullptr;
        if (table) {
            const long long l = p / tb_.NR;
            const long long r = p - l * tb_.NR;
            // u_x = E_x tbar_x and the largest binary exponent among them.
            // Range tests and the scale are integer operations on exponent
            // fields: the FP64 pipe, GB300's scarce unit here, only takes the
            // products
            int umax_e = 0, eimax_e = 0;
            for (int x = 0; x < ng; x++) {
                const double E = __ldg(tb_.v + x * tb_.NL + l) * __ldg(tb_.o + x * tb_.NR + r);
                const double u = E * tbar[(long long)x * q.P + p];
                c0[x * QT + t] = u;
                umax_e = max(umax_e, dexp(u));        // inf / NaN: 0x7FF, refused below
            }
            for (int y = 0; y < ng; y++) {
                const double Ei = __ldg(tb_.vi + y * tb_.NL + l) * __ldg(tb_.oi + y * tb_.NR + r);
                c1[y * QT + t] = Ei;
                eimax_e = max(eimax_e, dexp(Ei));
            }
            // |u|, 1/E < 2^996 (< 1e300), and |T_y| <= ng max|G| max|u| max(1/E)
            // < 2^(umax_e + eimax_e - 2044 + 8) kept below 2^956 (~1e288):
            // well inside FP64
            if (umax_e > 1023 + 995 || eimax_e > 1023 + 995 ||
                umax_e + eimax_e - 2044 + 8 > 956)
                table = false;
            if (table) {
                if (umax_e == 0) {          // all u zero (or below 2^-1022)
                    for (int y = 0; y < ng; y++) emit(p, y, 0.0, f_diff, f_norm);
                } else {
                    const int k = umax_e - 1023;     // |u 2^-k| < 2
                    for (int x = 0; x < ng; x++) uf[x * QT + t] = dsplit_scaled(c0[x * QT + t], k);
                    for (int y = 0; y < ng; y++) {
                        float s = 0.f, c = 0.f;
                        const float *gh = Gh + y * ng, *gl = Gl + y * ng;
                        for (int x = 0; x < ng; x++) {
                            const float2 u = uf[x * QT + t];
                            const float pr = gh[x] * u.x;
                            const float pe = fmaf(gh[x], u.x, -pr);      // exact
                            float s2, e2;
                            two_sum_f(s, pr, s2, e2);
                            s = s2;
                            c += e2 + pe;
                            c = fmaf(gh[x], u.y, c);
                            c = fmaf(gl[x], u.x, c);
                        }
                        const double acc = f32_to_f64_scaled(s, k) + f32_to_f64_scaled(c, k);
                        emit(p, y, acc * c1[y * QT + t], f_diff, f_norm);
                    }
                }
            }
        }
        if (!table) {
            // FP64 path
            const double d = denom(q, p, D, ev, eo);
            const int nx = q.symmetric ? (ng + 1) / 2 : ng;
            for (int x = 0; x < nx; x++) {
                const double E = exp((ti[x] - tc) * d);
                c1[x * QT + t] = E;
                c0[x * QT + t] = E * tbar[(long long)x * q.P + p];
                const int xm = ng - 1 - x;
                if (q.symmetric && xm != x) {
                    const double Ei = 1.0 / E;
                    c1[xm * QT + t] = Ei;
                    c0[xm * QT + t] = Ei * tbar[(long long)xm * q.P + p];
                }
            }
            for (int y = 0; y < ng; y++) {
                double acc = 0.0;
                for (int x = 0; x < ng; x++) acc = fma(G[y * ng + x], c0[x * QT + t], acc);
                const double Ty = q.symmetric ? acc * c1[(ng - 1 - y) * QT + t]
                                              : acc / c1[y * QT + t];
                emit(p, y, Ty, f_diff, f_norm);
            }
        }
        if (MODE == 1) {
            s_diff += (double)f_diff;
            s_norm += (double)f_norm;
        }
    };
    if (q.spin_half > 0) {
        const int h = q.spin_half, n = q.no;
        const long long rows = q.P / n;
        const int lane = t % 32;
        const long long tw = (long long)gridDim.x * (QT / 32);
        for (long long u = blockIdx.x * (long long)(QT / 32) + t / 32; u < 2 * rows; u += tw) {
            const long long rr = u >> 1;
            const int jh = (int)(u & 1);
            const int i = (int)(rr % n);
            const long long ab = rr / n;
            const int b = (int)(ab % n), a = (int)(ab / n);
            if ((a >= h) + (b >= h) != (i >= h) + jh) continue;
            for (int jj = lane; jj < h; jj += 32) element(rr * n + (long long)jh * h + jj);
        }
    } else {
        for (long long p = blockIdx.x * (long long)QT + t; p < q.P;
             p += (long long)gridDim.x * QT)
            element(p);
    }
    if (MODE == 1) {
        __shared__ double red[2][QT];
        red[0][t] = s_diff;
        red[1][t] = s_norm;
        __syncthreads();
        for (int st = QT / 2; st > 0; st >>= 1) {
            if (t < st) {
                red[0][t] += red[0][t + st];
                red[1][t] += red[1][t + st];
            }
            __syncthreads();
        }
        if (t == 0) {
            partial[2 * blockIdx.x] = red[0][0];
            partial[2 * blockIdx.x + 1] = red[1][0];
        }
    }
}

// one grid point: out = sum_x G[ig,x] w(ig,x) tbar_x (quadrature.py:348-369)
__global__ void quad_single_kernel(QuadParams q, int ig, const double *__restrict__ tbar,
                                   const double *__restrict__ ti,
                                   const double *__restrict__ G,
                                   const double *__restrict__ D,
                                   const double *__restrict__ ev,
                                   const double *__restrict__ eo,
                                   double *__restrict__ out) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < q.P;
         p += (long long)gridDim.x * blockDim.x) {
        const double d = denom(q, p, D, ev, eo);
        double acc = 0.0;
        for (int x = 0; x < q.ng; x++) {
            const double g = G[ig * q.ng + x];
            if (g == 0.0) continue;
            const double dt = (x < ig) ? (ti[x] - ti[ig]) : 0.0;
            acc = fma(g * exp(dt * d), tbar[(long long)x * q.P + p], acc);
        }
        out[p] = acc;
    }
}

__global__ void reduce_pairs_kernel(const double *__restrict__ partial, int n,
                                    double *__restrict__ res) {
    __shared__ double red[2][256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) {
        a += partial[2 * k];
        b += partial[2 * k + 1];
    }
    red[0][threadIdx.x] = a;
    red[1][threadIdx.x] = b;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[0][threadIdx.x] += red[0][threadIdx.x + s];
            red[1][threadIdx.x] += red[1][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        res[0] = red[0][0];
        res[1] = red[1][0];
    }
}

// Host-side analysis of the grid: recurrence step and uniform spacing.
void analyse_grid(int ng, const double *ti, const double *G, int full, int *step,
                  int *uniform) {
    *uniform = 1;
    for (int k = 1; k + 1 < ng; k++) {
        double d0 = ti[1] - ti[0], dk = ti[k + 1] - ti[k];
        if (std::fabs(dk - d0) > 1e-14 * std::max(std::fabs(d0), 1e-300)) *uniform = 0;
    }
    *step = 0;
    if (full) return;
    for (int y = 0; y < ng; y++)
        for (int x = y + 1; x < ng; x++)
            if (G[y * ng + x] != 0.0) return;   // not lower-triangular
    for (int s = 1; s <= 2; s++) {
        bool ok = true;
        for (int y = s; y < ng && ok; y++)
            for (int x = 0; x < y - s && ok; x++)
                if (G[y * ng + x] != G[(y - s) * ng + x]) ok = false;
        if (ok) { *step = s; return; }
    }
}

// ti, G, cs, g1, gd; then the per-thread columns: step factors (general
// lower-triangular path on a non-uniform grid), inputs (general and dense
// paths), and the dense path's scale factors
size_t quad_smem(int ng, int uniform, int step, int full) {
    return sizeof(double) * (4 * ng + ng * ng + ((uniform || full) ? 0 : ng * QT) +
                             (step > 0 ? 0 : ng * QT) + (full ? ng * QT : 0));
}

// ti[x] + ti[ng-1-x] equal for every x (to rounding)
int grid_symmetric(int ng, const double *ti) {
    const double c = ti[0] + ti[ng - 1];
    const double tol = 1e-13 * std::max(std::fabs(ti[ng - 1] - ti[0]), 1e-300);
    for (int x = 0; x < ng; x++)
        if (std::fabs(ti[x] + ti[ng - 1 - x] - c) > tol) return 0;
    return 1;
}

}  // namespace

namespace {

size_t dense_smem(int ng) {
    return sizeof(double) * ((size_t)ng + 2 * (size_t)ng * ng + 2 * (size_t)ng * QT);
}

// The dense-G integral: pair tables of the orbital energies (when given),
// then quad_dense_kernel; mode 1 also damps and reduces the two norms.
int quad_dense_launch(kvft_ctx *ctx, int mode, QuadParams &q, const double *tbar,
                      const double *ti, const double *hti, const double *G, const double *D,
                      const double *ev, const double *eo, double *out, double *res) {
    const int ng = q.ng;
    DenseTabs tabs{nullptr, nullptr, nullptr, nullptr, 1, 1};
    if (!D && ev && eo) {
        const long long NL = q.rank == 2 ? (long long)q.nv * q.nv : q.nv;
        const long long NR = q.rank == 2 ? (long long)q.no * q.no : q.no;
        if (NL * NR == q.P) {
            void *tp = nullptr;
            KV_TRY(kv_scratch(ctx, "quad_tables", sizeof(double) * 2 * ng * (NL + NR), &tp));
            double *tab = (double *)tp;
            const double tc = 0.5 * (hti[0] + hti[ng - 1]);
            const long long work = ng * (NL + NR);
            const int gb = (int)std::max(1LL, std::min((work + 255) / 256, 4096LL));
            quad_tables_kernel<<<gb, 256, 0, ctx->stream>>>(ng, q.rank, q.nv, q.no, tc, ti, ev,
                                                            eo, NL, NR, tab);
            KV_TRY(kv_launch_check(ctx, "quad_tables"));
            tabs = DenseTabs{tab, tab + ng * NL, tab + 2 * ng * NL, tab + 2 * ng * NL + ng * NR,
                             NL, NR};
        }
    }
    const size_t smem = dense_smem(ng);
    static bool attr_done = false;
    if (!attr_done) {
        const int mx = (int)dense_smem(MAXNG);
        cudaFuncSetAttribute(quad_dense_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(quad_dense_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        attr_done = true;
    }
    int per_sm = 1;
    KV_CHECK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                      &per_sm, mode == 0 ? (const void *)quad_dense_kernel<0>
                                         : (const void *)quad_dense_kernel<1>,
                      QT, smem));
    const long long blocks = (q.P + QT - 1) / QT;
    const int grid = (int)std::max(1LL, std::min(blocks, (long long)std::max(per_sm, 1) *
                                                             ctx->sm_count));
    KvProfScope prof(ctx, KV_CAT_QUAD, 8.0 * ng * (double)q.P * (mode == 0 ? 2 : 3) *
                                           kv_spin_frac(q.nv, q.no, q.spin_half));
    if (mode == 0) {
        quad_dense_kernel<0><<<grid, QT, smem, ctx->stream>>>(q, tabs, tbar, ti, G, D, ev, eo,
                                                              out, nullptr);
        return kv_launch_check(ctx, "quad_dense_kernel");
    }
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "quad_partial", sizeof(double) * 2 * grid, &part));
    quad_dense_kernel<1><<<grid, QT, smem, ctx->stream>>>(q, tabs, tbar, ti, G, D, ev, eo, out,
                                                          (double *)part);
    KV_TRY(kv_launch_check(ctx, "quad_dense_update_kernel"));
    reduce_pairs_kernel<<<1, 256, 0, ctx->stream>>>((const double *)part, grid, res);
    return kv_launch_check(ctx, "reduce_pairs");
}

}  // namespace

// Shared launcher.  ti/G are DEVICE pointers; hti/hG are host copies used for
// the grid analysis.  MODE 1 requires `partial` (2 doubles per block) and
// `res` (2 doubles) device buffers.
int kv_quad_launch(kvft_ctx *ctx, int mode, int ng, long long P, int rank, int nv,
                   int no, const double *tbar, const double *ti, const double *hti,
                   const double *G, const double *hG, const double *D,
                   const double *ev, const double *eo, int full, double alpha,
                   double *out, double *res, int spin_half) {
    if (ng < 1 || ng > MAXNG) return kv_fail(ctx, KVFT_EINVAL, "ng must be in [1, 64]");
    if (P == 0) return KVFT_OK;
    if (ctx->dry) {
        if (mode != 0 || D) return kv_fail(ctx, KVFT_EINVAL, "dry run: tau integral mode");
        KvDryOp op;
        op.kind = 2;
        op.ng = ng, op.P = P, op.rank = rank, op.full = full, op.nv = nv, op.no = no;
        op.src = tbar, op.dst = out, op.ti = ti, op.G = G, op.ev = ev, op.eo = eo;
        ctx->dry->push_back(op);
        return KVFT_OK;
    }
    QuadParams q;
    q.ng = ng;
    q.P = P;
    q.rank = rank;
    q.nv = nv;
    q.no = no;
    q.full = full;
    q.alpha = alpha;
    // spin blocks: only the spin-conserving elements are integrated (the
    // solver's passes, which read no other; callers pass 0 otherwise)
    q.spin_half = (rank == 2 && nv == no && nv == 2 * spin_half) ? spin_half : 0;
    analyse_grid(ng, hti, hG, full, &q.step, &q.uniform);
    q.symmetric = grid_symmetric(ng, hti);
    if (full) return quad_dense_launch(ctx, mode, q, tbar, ti, hti, G, D, ev, eo, out, res);
    size_t smem = quad_smem(ng, q.uniform, q.step, q.full);
    long long blocks = (P + QT - 1) / QT;
    long long cap = (long long)ctx->sm_count * 16;
    int grid = (int)std::min(blocks, cap);
    static bool attr_done = false;
    if (!attr_done) {
        const int mx = (int)quad_smem(MAXNG, 0, 0, 1);
        cudaFuncSetAttribute(quad_kernel<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(quad_kernel<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(quad_kernel<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(quad_kernel<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        attr_done = true;
    }
    // algorithmic bytes: tbar in, T out (mode 0); tbar + T_old in, T_old out
    // (mode 1); with spin blocks, of the spin-conserving elements
    KvProfScope prof(ctx, KV_CAT_QUAD, 8.0 * ng * (double)P * (mode == 0 ? 2 : 3) *
                                           kv_spin_frac(nv, no, q.spin_half));
    if (mode == 0) {
        if (q.uniform)
            quad_kernel<0, true><<<grid, QT, smem, ctx->stream>>>(q, tbar, ti, G, D, ev, eo, out,
                                                                  nullptr);
        else
            quad_kernel<0, false><<<grid, QT, smem, ctx->stream>>>(q, tbar, ti, G, D, ev, eo,
                                                                   out, nullptr);
        return kv_launch_check(ctx, "quad_kernel");
    }
    void *part = nullptr;
    KV_TRY(kv_scratch(ctx, "quad_partial", sizeof(double) * 2 * grid, &part));
    if (q.uniform)
        quad_kernel<1, true><<<grid, QT, smem, ctx->stream>>>(q, tbar, ti, G, D, ev, eo, out,
                                                              (double *)part);
    else
        quad_kernel<1, false><<<grid, QT, smem, ctx->stream>>>(q, tbar, ti, G, D, ev, eo, out,
                                                               (double *)part);
    KV_TRY(kv_launch_check(ctx, "quad_update_kernel"));
    reduce_pairs_kernel<<<1, 256, 0, ctx->stream>>>((const double *)part, grid, res);
    return kv_launch_check(ctx, "reduce_pairs");
}

namespace {

int int_tbar_entry(kvft_ctx *ctx, int rank, int ng, int nv, int no, const double *tbar,
                   const double *ti, const double *D, const double *G, int full,
                   double *out) {
    if (!ctx || ng < 1 || ng > MAXNG || nv <= 0 || no <= 0 || !tbar || !ti || !D || !G || !out)
        return kv_fail(ctx, KVFT_EINVAL, "int_tbar: bad argument (ng must be 1..64)");
    if (tbar == out) return kv_fail(ctx, KVFT_EINVAL, "int_tbar: output must not alias input");
    cudaSetDevice(ctx->device);
    std::vector<double> hti(ng), hG((size_t)ng * ng);
    KV_CHECK(ctx, cudaMemcpyAsync(hti.data(), ti, sizeof(double) * ng, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaMemcpyAsync(hG.data(), G, sizeof(double) * ng * ng,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    long long P = (long long)nv * no * (rank == 2 ? (long long)nv * no : 1LL);
    return kv_quad_launch(ctx, 0, ng, P, rank, nv, no, tbar, ti, hti.data(), G, hG.data(), D,
                          nullptr, nullptr, full, 0.0, out, nullptr, 0);
}

int int_tbar_single_entry(kvft_ctx *ctx, int rank, int ng, int ig, int nv, int no,
                          const double *tbar, const double *ti, const double *D,
                          const double *G, double *out) {
    if (!ctx || ng < 1 || ig < 0 || ig >= ng || nv <= 0 || no <= 0 || !tbar || !ti || !D ||
        !G || !out)
        return kv_fail(ctx, KVFT_EINVAL, "int_tbar_single: bad argument");
    cudaSetDevice(ctx->device);
    QuadParams q{};
    q.ng = ng;
    q.P = (long long)nv * no * (rank == 2 ? (long long)nv * no : 1LL);
    long long blocks = (q.P + 255) / 256;
    int grid = (int)std::min(blocks, (long long)ctx->sm_count * 8);
    quad_single_kernel<<<grid, 256, 0, ctx->stream>>>(q, ig, tbar, ti, G, D, nullptr, nullptr,
                                                      out);
    return kv_launch_check(ctx, "quad_single");
}

}  // namespace

// one grid point ig of the tau integral for the solver (D or eps form)
int kv_quad_single(kvft_ctx *ctx, int ng, int ig, long long P, int rank, int nv, int no,
                   const double *tbar, const double *ti, const double *G, const double *D,
                   const double *ev, const double *eo, double *out) {
    QuadParams q{};
    q.ng = ng;
    q.P = P;
    q.rank = rank;
    q.nv = nv;
    q.no = no;
    const int grid = (int)std::min((P + 255) / 256, (long long)ctx->sm_count * 8);
    KvProfScope prof(ctx, KV_CAT_QUAD, 8.0 * (double)P * (ng + 1));
    quad_single_kernel<<<grid, 256, 0, ctx->stream>>>(q, ig, tbar, ti, G, D, ev, eo, out);
    return kv_launch_check(ctx, "quad_single");
}

int kv_int_tbar(kvft_ctx *ctx, int ng, size_t P, const double *tbar, const double *ti,
                const double *D, const double *eps_v, const double *eps_o, int nv, int no,
                int rank, const double *G, int full, double *out) {
    std::vector<double> hti(ng), hG((size_t)ng * ng);
    KV_CHECK(ctx, cudaMemcpyAsync(hti.data(), ti, sizeof(double) * ng, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    KV_CHECK(ctx, cudaMemcpyAsync(hG.data(), G, sizeof(double) * ng * ng,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    KV_CHECK(ctx, cudaStreamSynchronize(ctx->stream));
    return kv_quad_launch(ctx, 0, ng, (long long)P, rank, nv, no, tbar, ti, hti.data(), G,
                          hG.data(), D, eps_v, eps_o, full, 0.0, out, nullptr, 0);
}

extern "C" {

int kvft_int_tbar1(kvft_ctx *ctx, int ng, int nv, int no, const double *t1bar,
                   const double *ti, const double *D1, const double *G, int full,
                   double *t1out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_int_tbar1: not on a dry-run context");
    return int_tbar_entry(ctx, 1, ng, nv, no, t1bar, ti, D1, G, full, t1out);
}

int kvft_int_tbar2(kvft_ctx *ctx, int ng, int nv, int no, const double *t2bar,
                   const double *ti, const double *D2, const double *G, int full,
                   double *t2out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_int_tbar2: not on a dry-run context");
    return int_tbar_entry(ctx, 2, ng, nv, no, t2bar, ti, D2, G, full, t2out);
}

int kvft_int_tbar1_single(kvft_ctx *ctx, int ng, int ig, int nv, int no,
                          const double *t1bar, const double *ti, const double *D1,
                          const double *G, double *t1out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_int_tbar1_single: not on a dry-run context");
    return int_tbar_single_entry(ctx, 1, ng, ig, nv, no, t1bar, ti, D1, G, t1out);
}

int kvft_int_tbar2_single(kvft_ctx *ctx, int ng, int ig, int nv, int no,
                          const double *t2bar, const double *ti, const double *D2,
                          const double *G, double *t2out) {
    if (ctx && ctx->dry) return kv_fail(ctx, KVFT_EINVAL, "kvft_int_tbar2_single: not on a dry-run context");
    return int_tbar_single_entry(ctx, 2, ng, ig, nv, no, t2bar, ti, D2, G, t2out);
}

}  // extern "C"
