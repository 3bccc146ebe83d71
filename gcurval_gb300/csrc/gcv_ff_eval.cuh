// Float-float evaluators of the mixed-precision path: curve speeds in
// float-float arithmetic (gcv_ff.cuh), an own float-float sin(pi x) for
// ellipses, and the 15-node Kronrod panel built from them.
#pragma once

#include "gcv_ff.cuh"
#include "gcv_table.cuh"

namespace gcv {

// float-float constants from double literals (split at compile time)
struct ffc {
    float hi, lo;
};
__host__ __device__ constexpr ffc split_const(double x)
{
    return ffc{(float)x, (float)(x - (double)(float)x)};
}
__device__ __forceinline__ ff to_ff(ffc c) { return ff{c.hi, c.lo}; }

// ------------------------------------------------------- sin(pi x), |x| <= 1
// Reduce x to r in [-1/4, 1/4] with sin(pi x) = +-sin(pi r) or +-cos(pi r),
// then Taylor series of sin(t), cos(t) in t = pi r (|t| <= pi/4: the 17th /
// 16th order terms are below 2e-14, far under float-float rounding).
__device__ __forceinline__ ff ff_sin_taylor(ff t)
{
    const ff t2 = ff_mul(t, t);
    // t * (1 - t^2/3! + t^4/5! - ... + t^16/17!)
    ff p = to_ff(split_const(1.0 / 355687428096000.0));  // 1/17!
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 1307674368000.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 6227020800.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 39916800.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 362880.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 5040.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 120.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 6.0))));
    p = ff_fma(p, t2, ff{1.0f, 0.0f});
    return ff_mul(p, t);
}
__device__ __forceinline__ ff ff_cos_taylor(ff t)
{
    const ff t2 = ff_mul(t, t);
    ff p = to_ff(split_const(1.0 / 20922789888000.0));  // 1/16!
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 87178291200.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 479001600.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 3628800.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 40320.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(1.0 / 720.0))));
    p = ff_fma(p, t2, to_ff(split_const(1.0 / 24.0)));
    p = ff_fma(p, t2, ff_neg(to_ff(split_const(0.5))));
    return ff_fma(p, t2, ff{1.0f, 0.0f});
}

// sin(pi x)^2 for x in [-1, 1]
__device__ __forceinline__ ff ff_sinpi_sq(ff x)
{
    // sin^2(pi x) has period 1 and is even: fold to y in [0, 1/2]
    float ax = fabsf(x.hi);
    ff y = x.hi < 0.0f ? ff_neg(x) : x;
    if (ax > 0.5f) y = ff_add_f(ff_neg(y), 1.0f);  // 1 - |x|
    (void)ax;
    // y in [0, 1/2]: sin(pi y) = cos(pi (1/2 - y)); use sin for y <= 1/4
    const ff pi = to_ff(split_const(3.141592653589793238462643383279502884));
    ff s;
    if (y.hi <= 0.25f) {
        s = ff_sin_taylor(ff_mul(pi, y));
    } else {
        s = ff_cos_taylor(ff_mul(pi, ff_add_f(ff_neg(y), 0.5f)));
    }
    return ff_mul(s, s);
}

// ------------------------------------------------------------- evaluators
template <int CODE>
struct EvalFF {
    static constexpr int P = code_degree(CODE);
    static constexpr int D = code_dim(CODE);
    // A, B, w0 (ellipse piece) or the derivative polynomial
    // b[k][d] = (k + 1) a[k + 1][d] of the stored float-float position polynomial a
    __device__ __forceinline__ static void load(const float2* __restrict__ seg, ff* r)
    {
        if constexpr (CODE == 0) {
            r[0] = ff{seg[0].x, seg[0].y};
            r[1] = ff{seg[1].x, seg[1].y};
            r[2] = ff{seg[2].x, seg[2].y};  // w0 = (2 j + 1) / ELLIPSE_PIECES - 1: exact in FP32
        } else {
#pragma unroll
            for (int k = 0; k < P; ++k)
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    const float2 c = seg[(k + 1) * D + d];
                    r[k * D + d] = k == 0 ? ff{c.x, c.y} : ff_mul_f(ff{c.x, c.y}, float(k + 1));
                }
        }
    }
    __device__ __forceinline__ static ff speed(const ff* r, ff v)
    {
        if constexpr (CODE == 0) {
            // sqrt(B + A sin^2(pi w)), w = w0 + v / ELLIPSE_PIECES in [-1, 1]
            const ff w = ff_add_f(ff_scale(v, (float)ELLIPSE_PIECE_SCALE), r[2].hi);
            const ff s2 = ff_sinpi_sq(w);
            return ff_sqrt(ff_fma(r[0], s2, r[1]));
        } else {
            ff s{0.0f, 0.0f};
#pragma unroll
            for (int d = 0; d < D; ++d) {
                ff acc = r[(P - 1) * D + d];
#pragma unroll
                for (int k = P - 2; k >= 0; --k) acc = ff_fma(acc, v, r[k * D + d]);
                s = d == 0 ? ff_mul(acc, acc) : ff_fma(acc, acc, s);
            }
            return ff_sqrt(s);
        }
    }
    // speed and q = f * df/dv (q only to FP32 accuracy: it shapes the initial guess
    // and the stopping test, never the result)
    __device__ __forceinline__ static ff speed_slope(const ff* r, ff v, float& q)
    {
        if constexpr (CODE == 0) {
            float sn, cs;
            sincospif(fmaf(v.hi, (float)ELLIPSE_PIECE_SCALE, r[2].hi), &sn, &cs);
            q = (float)(PI * ELLIPSE_PIECE_SCALE) * r[0].hi * sn * cs;
            return speed(r, v);
        } else {
            ff s{0.0f, 0.0f};
            float t = 0.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                ff acc = r[(P - 1) * D + d];
                float dacc = 0.0f;
#pragma unroll
                for (int k = P - 2; k >= 0; --k) {
                    dacc = fmaf(dacc, v.hi, acc.hi);
                    acc = ff_fma(acc, v, r[k * D + d]);
                }
                s = d == 0 ? ff_mul(acc, acc) : ff_fma(acc, acc, s);
                t = fmaf(acc.hi, dacc, t);
            }
            q = t;
            return ff_sqrt(s);
        }
    }
    // speed rounded to FP32 and q at a float-float point: the components in
    // float-float (Horner at the full point), their norm in FP32 (the
    // sampler's Newton steps use f to FP32 accuracy only)
    __device__ __forceinline__ static float speed_slope_f(const ff* r, ff v, float& q)
    {
        if constexpr (CODE == 0) {
            return speed_slope(r, v, q).hi;
        } else {
            float s = 0.0f, t = 0.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                ff acc = r[(P - 1) * D + d];
                float dacc = 0.0f;
#pragma unroll
                for (int k = P - 2; k >= 0; --k) {
                    dacc = fmaf(dacc, v.hi, acc.hi);
                    acc = ff_fma(acc, v, r[k * D + d]);
                }
                const float a = acc.hi + acc.lo;
                s = fmaf(a, a, s);
                t = fmaf(a, dacc, t);
            }
            q = t;
            return sqrtf(s);
        }
    }
    // speed and q in plain FP32 from the coefficients' leading parts: for the
    // leaf table's f and q, which only shape the sampler's initial guess
    __device__ __forceinline__ static float speed_slope32(const ff* r, float v, float& q)
    {
        if constexpr (CODE == 0) {
            float sn, cs;
            sincospif(fmaf(v, (float)ELLIPSE_PIECE_SCALE, r[2].hi), &sn, &cs);
            q = (float)(PI * ELLIPSE_PIECE_SCALE) * r[0].hi * sn * cs;
            return sqrtf(fmaf(r[0].hi, sn * sn, r[1].hi));
        } else {
            float s = 0.0f, t = 0.0f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
                float acc = r[(P - 1) * D + d].hi, dacc = 0.0f;
#pragma unroll
                for (int k = P - 2; k >= 0; --k) {
                    dacc = fmaf(dacc, v, acc);
                    acc = fmaf(acc, v, r[k * D + d].hi);
                }
                s = fmaf(acc, acc, s);
                t = fmaf(acc, dacc, t);
            }
            q = t;
            return sqrtf(s);
        }
    }
};

// ------------------------------------------- symbolic de Boor set-up (FF)
// bspline_setup (gcv_device.cuh) in float-float arithmetic, for tables built
// for the mixed path: the same polynomial recursion in v on the FP32 pipes.
// FP64 is used only to centre the data: knots relative to the span midpoint
// m and control points relative to the first one of the span (differences
// that carry the cancellation), each converted once to float-float.
template <int P, int D>
__device__ void bspline_setup_ff(const double* __restrict__ kv, const double* __restrict__ cp, int span, float2* out)
{
    const double ka = kv[span], kb = kv[span + 1];
    const double m = 0.5 * (ka + kb);
    const ff w = ff_from_double(0.5 * (kb - ka));
    // knots span-P+1 .. span+P relative to m
    ff dk[2 * P];
#pragma unroll
    for (int i = 0; i < 2 * P; ++i) dk[i] = ff_from_double(kv[span - P + 1 + i] - m);
    // N[r][k]: basis polynomial r, coefficient of v^k
    ff N[P + 1][P + 1];
    N[0][0] = ff{1.0f, 0.0f};
#pragma unroll
    for (int j = 1; j <= P; ++j) {
        ff saved[P + 1];
#pragma unroll
        for (int r = 0; r < j; ++r) {
            const ff ra = dk[r + P];                // k[span + r + 1] - m
            const ff la = ff_neg(dk[r + P - j]);    // m - k[span + 1 - j + r]
            const ff inv = ff_recip(ff_add(ra, la));
            ff temp[P + 1];
#pragma unroll
            for (int k = 0; k < j; ++k) temp[k] = ff_mul(N[r][k], inv);
#pragma unroll
            for (int k = j; k >= 0; --k) {
                const ff a = r == 0 ? ff{0.0f, 0.0f} : saved[k];
                if (k == j) {
                    const ff wt = ff_mul(w, temp[k - 1]);
                    N[r][k] = r == 0 ? ff_neg(wt) : ff_add(a, ff_neg(wt));
                    saved[k] = wt;
                } else if (k == 0) {
                    const ff rt = ff_mul(ra, temp[0]);
                    N[r][k] = r == 0 ? rt : ff_add(a, rt);
                    saved[k] = ff_mul(la, temp[0]);
                } else {
                    const ff wt = ff_mul(w, temp[k - 1]);
                    const ff rt = ff_fma(ra, temp[k], ff_neg(wt));
                    N[r][k] = r == 0 ? rt : ff_add(a, rt);
                    saved[k] = ff_fma(la, temp[k], wt);
                }
            }
        }
#pragma unroll
        for (int k = 0; k <= j; ++k) N[j][k] = saved[k];
    }
    // C(v) = P_0 + sum_{i >= 1} (P_i - P_0) N_i(v)  (the basis sums to one)
    const double* c0 = cp + (size_t)(span - P) * D;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const double q = c0[d];
        ff dp[P];
#pragma unroll
        for (int i = 1; i <= P; ++i) dp[i - 1] = ff_from_double(c0[i * D + d] - q);
#pragma unroll
        for (int k = 0; k <= P; ++k) {
            ff acc{0.0f, 0.0f};
#pragma unroll
            for (int i = 1; i <= P; ++i) acc = i == 1 ? ff_mul(dp[0], N[1][k]) : ff_fma(dp[i - 1], N[i][k], acc);
            if (k == 0) acc = ff_from_double(q + ff_to_double(acc));
            out[k * D + d] = make_float2(acc.hi, acc.lo);
        }
    }
}

// float-float panel: K15, G7, right-end speed and slope of [vlo, vlo + 2 hw]
// with vlo = -1 + k 2^(1-depth) built exactly from the integer k.
// Kronrod nodes x0..x6, weights wk0..wk7 and Gauss weights wg0..wg7 (0 for
// the Kronrod-only nodes) as float-float pairs, for the rolled panel loop
#define GCV_FFC2(x) {split_const(x).hi, split_const(x).lo}
static __constant__ float2 c_gk_ff[23] = {
    GCV_FFC2(gk_x(0)),  GCV_FFC2(gk_x(1)),  GCV_FFC2(gk_x(2)),  GCV_FFC2(gk_x(3)),  GCV_FFC2(gk_x(4)),
    GCV_FFC2(gk_x(5)),  GCV_FFC2(gk_x(6)),  GCV_FFC2(gk_wk(0)), GCV_FFC2(gk_wk(1)), GCV_FFC2(gk_wk(2)),
    GCV_FFC2(gk_wk(3)), GCV_FFC2(gk_wk(4)), GCV_FFC2(gk_wk(5)), GCV_FFC2(gk_wk(6)), GCV_FFC2(gk_wk(7)),
    GCV_FFC2(gk_wg(0)), GCV_FFC2(gk_wg(1)), GCV_FFC2(gk_wg(2)), GCV_FFC2(gk_wg(3)), GCV_FFC2(gk_wg(4)),
    GCV_FFC2(gk_wg(5)), GCV_FFC2(gk_wg(6)), GCV_FFC2(gk_wg(7))};
#undef GCV_FFC2

// Large integrands (high degree x dimension, and the float-float ellipse with
// its two Taylor series) keep the node loop rolled: fourteen inlined copies
// overflow the instruction cache.
template <int CODE>
constexpr bool panel_rolled()
{
    return CODE == 0 || code_degree(CODE) * code_dim(CODE) >= 8;
}

template <int CODE>
__device__ __forceinline__ void panel_k15_ff(const ff* r, unsigned long long k, int depth, ff& K, ff& G)
{
    const float hw = __int_as_float((127 - depth) << 23);  // 2^-depth, exact
    const float kh = (float)(unsigned)(k >> 24), kl = (float)(unsigned)(k & 0xFFFFFFull);
    const float sh = __int_as_float((127 + 25 - depth) << 23), sl = 2.0f * hw;  // 2^(25-depth), 2^(1-depth)
    const ff vlo = ff_add_f(two_sum(-1.0f, kh * sh), kl * sl);
    const ff mid = ff_add_f(vlo, hw);
    const ff fc = EvalFF<CODE>::speed(r, mid);
    ff kk = ff_mul(to_ff(split_const(gk_wk(7))), fc);
    ff gg = ff_mul(to_ff(split_const(gk_wg(7))), fc);
    if constexpr (panel_rolled<CODE>()) {
#pragma unroll 1
        for (int i = 0; i < 7; ++i) {
            const ff dx = ff_scale(ff{c_gk_ff[i].x, c_gk_ff[i].y}, hw);
            const ff s = ff_add(EvalFF<CODE>::speed(r, ff_add(mid, ff_neg(dx))), EvalFF<CODE>::speed(r, ff_add(mid, dx)));
            kk = ff_fma(ff{c_gk_ff[7 + i].x, c_gk_ff[7 + i].y}, s, kk);
            if (i & 1) gg = ff_fma(ff{c_gk_ff[15 + i].x, c_gk_ff[15 + i].y}, s, gg);  // the Gauss nodes
        }
    } else {
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            const ff dx = ff_scale(to_ff(split_const(gk_x(i))), hw);
            const ff s = ff_add(EvalFF<CODE>::speed(r, ff_add(mid, ff_neg(dx))), EvalFF<CODE>::speed(r, ff_add(mid, dx)));
            kk = ff_fma(to_ff(split_const(gk_wk(i))), s, kk);
            if (i & 1) gg = ff_fma(to_ff(split_const(gk_wg(i))), s, gg);
        }
    }
    K = ff_scale(kk, hw);
    G = ff_scale(gg, hw);
}

// B-spline panels by node pairs.  The speed polynomials p_d (degree P - 1 in
// v) are shifted to the panel's midpoint m and scaled to its half width h:
// b_j = h^j p_d^(j)(m) / j!, so p_d(m + h x) = sum_j b_j x^j on x in [-1, 1]
// (Horner-form Taylor shift, (P - 1) P / 2 float-float FMAs per dimension,
// then exact power-of-two scaling; on deep panels the high terms may
// underflow, where they are below any float-float rounding of b_0).  The
// symmetric nodes m -+ h x_i then share one evaluation of the even part
// E = b_0 + b_2 x^2 + ... and the odd part O = x (b_1 + b_3 x^2 + ...):
// p(m -+ h x) = E -+ O.  Per pair of nodes this replaces two Horner passes
// in v (2 (P - 1) float-float FMAs per dimension) and the two node
// positions by about half the work; K15 and G7 are formed as in
// panel_k15_ff.
#define GCV_FFC2(x) {split_const(x).hi, split_const(x).lo}
static __constant__ float2 c_gk_x2_ff[7] = {
    GCV_FFC2(gk_x(0) * gk_x(0)), GCV_FFC2(gk_x(1) * gk_x(1)), GCV_FFC2(gk_x(2) * gk_x(2)),
    GCV_FFC2(gk_x(3) * gk_x(3)), GCV_FFC2(gk_x(4) * gk_x(4)), GCV_FFC2(gk_x(5) * gk_x(5)),
    GCV_FFC2(gk_x(6) * gk_x(6))};
#undef GCV_FFC2

template <int P, int D>
__device__ __forceinline__ void ff_node_pair(const ff* b, ff x, ff x2, ff& fm, ff& fp)
{
    constexpr int N = P - 1;                       // polynomial degree
    constexpr int JE = (N % 2 == 0) ? N : N - 1;   // highest even power
    constexpr int JO = (N % 2 == 1) ? N : N - 1;   // highest odd power (-1: none)
    ff sm{0.0f, 0.0f}, sp{0.0f, 0.0f};
#pragma unroll
    for (int d = 0; d < D; ++d) {
        ff e = b[JE * D + d];
#pragma unroll
        for (int j = JE - 2; j >= 0; j -= 2) e = ff_fma(e, x2, b[j * D + d]);
        ff lo_ = e, hi_ = e;
        if constexpr (JO >= 1) {
            ff o = b[JO * D + d];
#pragma unroll
            for (int j = JO - 2; j >= 1; j -= 2) o = ff_fma(o, x2, b[j * D + d]);
            o = ff_mul(o, x);
            lo_ = ff_add(e, ff_neg(o));
            hi_ = ff_add(e, o);
        }
        sm = d == 0 ? ff_mul(lo_, lo_) : ff_fma(lo_, lo_, sm);
        sp = d == 0 ? ff_mul(hi_, hi_) : ff_fma(hi_, hi_, sp);
    }
    fm = ff_sqrt(sm);
    fp = ff_sqrt(sp);
}

// b: the interval's speed coefficients on entry, shifted in place
template <int CODE>
__device__ __forceinline__ void panel_k15_ff_pairs(ff* b, unsigned long long k, int depth, ff& K, ff& G)
{
    constexpr int P = code_degree(CODE), D = code_dim(CODE);
    const float hw = __int_as_float((127 - depth) << 23);  // 2^-depth, exact
    const float kh = (float)(unsigned)(k >> 24), kl = (float)(unsigned)(k & 0xFFFFFFull);
    const float sh = __int_as_float((127 + 25 - depth) << 23), sl = 2.0f * hw;  // 2^(25-depth), 2^(1-depth)
    const ff vlo = ff_add_f(two_sum(-1.0f, kh * sh), kl * sl);
    const ff mid = ff_add_f(vlo, hw);
    // Taylor shift to mid: after pass i, b[i] holds p^(i)(mid) / i!
#pragma unroll
    for (int i = 0; i < P - 1; ++i)
#pragma unroll
        for (int j = P - 2; j >= i; --j)
#pragma unroll
            for (int d = 0; d < D; ++d) b[j * D + d] = ff_fma(b[(j + 1) * D + d], mid, b[j * D + d]);
    float sc = hw;
#pragma unroll
    for (int j = 1; j < P; ++j) {
#pragma unroll
        for (int d = 0; d < D; ++d) b[j * D + d] = ff_scale(b[j * D + d], sc);
        sc *= hw;
    }
    ff s0{0.0f, 0.0f};
#pragma unroll
    for (int d = 0; d < D; ++d) s0 = d == 0 ? ff_mul(b[d], b[d]) : ff_fma(b[d], b[d], s0);
    const ff fc = ff_sqrt(s0);
    ff kk = ff_mul(to_ff(split_const(gk_wk(7))), fc);
    ff gg = ff_mul(to_ff(split_const(gk_wg(7))), fc);
    if constexpr (panel_rolled<CODE>()) {
#pragma unroll 1
        for (int i = 0; i < 7; ++i) {
            ff fm, fp;
            ff_node_pair<P, D>(b, ff{c_gk_ff[i].x, c_gk_ff[i].y}, ff{c_gk_x2_ff[i].x, c_gk_x2_ff[i].y}, fm, fp);
            const ff sum = ff_add(fm, fp);
            kk = ff_fma(ff{c_gk_ff[7 + i].x, c_gk_ff[7 + i].y}, sum, kk);
            if (i & 1) gg = ff_fma(ff{c_gk_ff[15 + i].x, c_gk_ff[15 + i].y}, sum, gg);  // the Gauss nodes
        }
    } else {
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            ff fm, fp;
            ff_node_pair<P, D>(b, to_ff(split_const(gk_x(i))), to_ff(split_const(gk_x(i) * gk_x(i))), fm, fp);
            const ff sum = ff_add(fm, fp);
            kk = ff_fma(to_ff(split_const(gk_wk(i))), sum, kk);
            if (i & 1) gg = ff_fma(to_ff(split_const(gk_wg(i))), sum, gg);
        }
    }
    K = ff_scale(kk, hw);
    G = ff_scale(gg, hw);
}

// the float-float panel of a curve code: node pairs for B-splines, node by
// node for the ellipse's sin(pi x) integrand; r (the interval's speed
// coefficients) is scratch: the B-spline panel shifts it in place
template <int CODE>
__device__ __forceinline__ void panel_ff(ff* r, unsigned long long k, int depth, ff& K, ff& G)
{
    if constexpr (CODE == 0)
        panel_k15_ff<CODE>(r, k, depth, K, G);
    else
        panel_k15_ff_pairs<CODE>(r, k, depth, K, G);
}

__device__ __forceinline__ void load_ff_dyn(int code, const float2* __restrict__ seg, ff* r)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: EvalFF<C>::load(seg, r); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: break;
    }
}

__device__ __forceinline__ void panel_ff_dyn(int code, ff* r, unsigned long long k, int depth, ff& K, ff& G)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: panel_ff<C>(r, k, depth, K, G); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: K = G = ff{0.0f, 0.0f}; break;
    }
}

template <int CODE>
__device__ __forceinline__ float speed_slope32_of(int code, const ff* r, float v, float& q)
{
    if constexpr (CODE >= 0) {
        return EvalFF<CODE>::speed_slope32(r, v, q);
    } else {
        switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: return EvalFF<C>::speed_slope32(r, v, q);
            GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
        default: q = 0.0f; return 0.0f;
        }
    }
}

template <int CODE>
__device__ __forceinline__ ff speed_ff_of(int code, const ff* r, ff v)
{
    if constexpr (CODE >= 0) {
        return EvalFF<CODE>::speed(r, v);
    } else {
        switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: return EvalFF<C>::speed(r, v);
            GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
        default: return ff{0.0f, 0.0f};
        }
    }
}

template <int CODE>
__device__ __forceinline__ ff speed_slope_ff_of(int code, const ff* r, ff v, float& q)
{
    if constexpr (CODE >= 0) {
        return EvalFF<CODE>::speed_slope(r, v, q);
    } else {
        switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: return EvalFF<C>::speed_slope(r, v, q);
            GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
        default: q = 0.0f; return ff{0.0f, 0.0f};
        }
    }
}

}  // namespace gcv
