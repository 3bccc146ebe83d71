// Float-float evaluators of the mixed-precision path: curve speeds in
// float-float arithmetic (gcv_ff.cuh), an own float-float sin(pi x) for
// ellipses, and the 15-node Kronrod panel built from them.
#pragma once

#include "gcv_ff.cuh"
#include "gcv_ff2.cuh"
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

// ------------------------------------------------- sin^2(pi x), |x| <= 1
// sin^2(pi x) has period 1 and is even: fold x to y in [0, 1/2]; then
// sin^2(pi y) = S(y) for y <= 1/4 and 1 - S(1/2 - y) above, with S the
// even series S(u) = sin^2(pi u) = sum_{k >= 1} c_k u^(2k),
// c_k = (-1)^(k+1) 2^(2k-1) pi^(2k) / (2k)!, for |u| <= 1/4.  Eleven terms:
// the twelfth is below 1e-19 there, far under float-float rounding.  One
// series without a branch per node, so that two nodes share one packed
// evaluation (ff2_sinpi_sq).
constexpr int SIN2_TERMS = 11;
__host__ __device__ constexpr double sin2pi_coef(int k)
{
    double c = 0.5;  // (2 pi)^(2k) / (2k)! / 2
    for (int i = 1; i <= 2 * k; ++i) c *= 2.0 * PI / i;
    return (k % 2 == 1) ? c : -c;
}

// x in [-1, 1] -> u in [0, 1/4] and whether the result is 1 - S(u)
__device__ __forceinline__ ff sinpi_sq_fold(ff x, bool& upper)
{
    ff y = x.hi < 0.0f ? ff_neg(x) : x;
    if (y.hi > 0.5f) y = ff_add_f(ff_neg(y), 1.0f);  // 1 - |x|
    upper = y.hi > 0.25f;
    return upper ? ff_add_f(ff_neg(y), 0.5f) : y;
}

// S(u) = sin^2(pi u), two lanes
__device__ __forceinline__ ff2 ff2_sin2pi_series(ff2 u)
{
    const ff2 U = ff2_mul(u, u);
    ff2 p = splat(to_ff(split_const(sin2pi_coef(SIN2_TERMS))));
#pragma unroll
    for (int k = SIN2_TERMS - 1; k >= 1; --k) p = ff2_fma(p, U, splat(to_ff(split_const(sin2pi_coef(k)))));
    return ff2_mul(p, U);
}

// sin^2(pi x) for x in [-1, 1], two lanes
__device__ __forceinline__ ff2 ff2_sinpi_sq(ff2 x)
{
    bool up0, up1;
    const ff u0 = sinpi_sq_fold(lane0(x), up0), u1 = sinpi_sq_fold(lane1(x), up1);
    const ff2 S = ff2_sin2pi_series(pack(u0, u1));
    const ff2 C = ff2_add(splat(ff{1.0f, 0.0f}), ff2_neg(S));
    return pack(up0 ? lane0(C) : lane0(S), up1 ? lane1(C) : lane1(S));
}

// sin^2(pi x) for x in [-1, 1]
__device__ __forceinline__ ff ff_sinpi_sq(ff x)
{
    bool up;
    const ff u = sinpi_sq_fold(x, up);
    const ff U = ff_mul(u, u);
    ff p = to_ff(split_const(sin2pi_coef(SIN2_TERMS)));
#pragma unroll
    for (int k = SIN2_TERMS - 1; k >= 1; --k) p = ff_fma(p, U, to_ff(split_const(sin2pi_coef(k))));
    const ff S = ff_mul(p, U);
    return up ? ff_add_f(ff_neg(S), 1.0f) : S;
}

// ------------------------------------------------------------- evaluators
template <int CODE>
struct EvalFF {
    static constexpr int P = code_degree(CODE);
    static constexpr int D = code_dim(CODE);
    // A, B, w0 (ellipse piece) or the derivative polynomial
    // b[k][d] = (k + 1) a[k + 1][d], stored after the midpoint position a[0]
    // (bspline_setup_ff)
    __device__ __forceinline__ static void load(const float2* __restrict__ seg, ff* r)
    {
        if constexpr (CODE == 0) {
            r[0] = ff{seg[0].x, seg[0].y};
            r[1] = ff{seg[1].x, seg[1].y};
            r[2] = ff{seg[2].x, seg[2].y};  // w0 = (2 j + 1) / ELLIPSE_PIECES - 1: exact in FP32
        } else {
#pragma unroll
            for (int k = 0; k < P * D; ++k) {
                const float2 c = seg[D + k];
                r[k] = ff{c.x, c.y};
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
    // the speeds at two points at once (packed lanes): the arithmetic of
    // speed() lane by lane, each coefficient splat into both lanes
    __device__ __forceinline__ static ff2 speed2(const ff* r, ff2 v)
    {
        if constexpr (CODE == 0) {
            const ff2 w = ff2_add(ff2_scale(v, (float)ELLIPSE_PIECE_SCALE), splat(ff{r[2].hi, 0.0f}));
            return ff2_sqrt(ff2_fma(splat(r[0]), ff2_sinpi_sq(w), splat(r[1])));
        }
        ff2 s{};
#pragma unroll
        for (int d = 0; d < D; ++d) {
            ff2 acc = splat(r[(P - 1) * D + d]);
#pragma unroll
            for (int k = P - 2; k >= 0; --k) acc = ff2_fma(acc, v, splat(r[k * D + d]));
            s = d == 0 ? ff2_mul(acc, acc) : ff2_fma(acc, acc, s);
        }
        return ff2_sqrt(s);
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
// that carry the cancellation), each converted once to float-float.  The
// constant term (the position at the midpoint) is formed in float-float.
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
            // the position at the midpoint, P_0 + acc, in float-float (it
            // only enters points, never the speed); the higher terms are
            // stored as the derivative's coefficients k a_k, which the walk
            // and the sampler read without rescaling
            if (k == 0)
                acc = ff_add(ff_from_double(q), acc);
            else if (k > 1)
                acc = ff_mul_f(acc, float(k));
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
    // the two nodes of a pair in packed lanes
#pragma unroll 1
    for (int i = 0; i < 7; ++i) {
        const ff dx = ff_scale(ff{c_gk_ff[i].x, c_gk_ff[i].y}, hw);
        const ff2 f = EvalFF<CODE>::speed2(r, pack(ff_add(mid, ff_neg(dx)), ff_add(mid, dx)));
        const ff s = ff_add(lane0(f), lane1(f));
        kk = ff_fma(ff{c_gk_ff[7 + i].x, c_gk_ff[7 + i].y}, s, kk);
        if (i & 1) gg = ff_fma(ff{c_gk_ff[15 + i].x, c_gk_ff[15 + i].y}, s, gg);  // the Gauss nodes
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

// ff_node_pair for two node pairs at once, in the lanes of packed FP32 pairs
// (FFMA2 / FADD2 / FMUL2): x and x2 hold the two pairs' offsets, the
// coefficients b are shared (each is splat into both lanes where it is
// used).  Half the float-float instructions of two ff_node_pair calls, the
// same roundings lane by lane.
template <int P, int D>
__device__ __forceinline__ void ff_node_pair2(const ff* b, ff2 x, ff2 x2, ff2& fm, ff2& fp)
{
    constexpr int N = P - 1;
    constexpr int JE = (N % 2 == 0) ? N : N - 1;
    constexpr int JO = (N % 2 == 1) ? N : N - 1;
    ff2 sm{}, sp{};
#pragma unroll
    for (int d = 0; d < D; ++d) {
        ff2 e = splat(b[JE * D + d]);
#pragma unroll
        for (int j = JE - 2; j >= 0; j -= 2) e = ff2_fma(e, x2, splat(b[j * D + d]));
        ff2 lo_ = e, hi_ = e;
        if constexpr (JO >= 1) {
            ff2 o = splat(b[JO * D + d]);
#pragma unroll
            for (int j = JO - 2; j >= 1; j -= 2) o = ff2_fma(o, x2, splat(b[j * D + d]));
            o = ff2_mul(o, x);
            lo_ = ff2_add(e, ff2_neg(o));
            hi_ = ff2_add(e, o);
        }
        sm = d == 0 ? ff2_mul(lo_, lo_) : ff2_fma(lo_, lo_, sm);
        sp = d == 0 ? ff2_mul(hi_, hi_) : ff2_fma(hi_, hi_, sp);
    }
    fm = ff2_sqrt(sm);
    fp = ff2_sqrt(sp);
}

// The seven Kronrod node pairs and the centre as four packed steps: step j
// holds pairs 2j and 2j + 1, and the eighth lane is the centre node (x = 0:
// both of its "nodes" are the centre, so it carries half the centre
// weights).  Per step: x, x^2, the Kronrod weights and the Gauss weights
// (zero on the Kronrod-only pairs), each as the hi / lo float pairs of both
// lanes.
struct GkStep2 {
    float2 xh, xl, x2h, x2l, wkh, wkl, wgh, wgl;
};
__host__ __device__ constexpr double gk_pair_x(int i) { return i < 7 ? gk_x(i) : 0.0; }
__host__ __device__ constexpr double gk_pair_wk(int i) { return i < 7 ? gk_wk(i) : 0.5 * gk_wk(7); }
__host__ __device__ constexpr double gk_pair_wg(int i) { return i < 7 ? gk_wg(i) : 0.5 * gk_wg(7); }
#define GCV_GK_STEP2(j)                                                                                          \
    {{split_const(gk_pair_x(2 * j)).hi, split_const(gk_pair_x(2 * j + 1)).hi},                                  \
     {split_const(gk_pair_x(2 * j)).lo, split_const(gk_pair_x(2 * j + 1)).lo},                                  \
     {split_const(gk_pair_x(2 * j) * gk_pair_x(2 * j)).hi, split_const(gk_pair_x(2 * j + 1) * gk_pair_x(2 * j + 1)).hi}, \
     {split_const(gk_pair_x(2 * j) * gk_pair_x(2 * j)).lo, split_const(gk_pair_x(2 * j + 1) * gk_pair_x(2 * j + 1)).lo}, \
     {split_const(gk_pair_wk(2 * j)).hi, split_const(gk_pair_wk(2 * j + 1)).hi},                                \
     {split_const(gk_pair_wk(2 * j)).lo, split_const(gk_pair_wk(2 * j + 1)).lo},                                \
     {split_const(gk_pair_wg(2 * j)).hi, split_const(gk_pair_wg(2 * j + 1)).hi},                                \
     {split_const(gk_pair_wg(2 * j)).lo, split_const(gk_pair_wg(2 * j + 1)).lo}}
static __constant__ GkStep2 c_gk_step2[4] = {GCV_GK_STEP2(0), GCV_GK_STEP2(1), GCV_GK_STEP2(2), GCV_GK_STEP2(3)};
#undef GCV_GK_STEP2

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
    // the node pairs two at a time in packed lanes (the centre in the last
    // step's second lane); the two lanes' sums are added at the end
    ff2 kk2{}, gg2{};
    if constexpr (panel_rolled<CODE>()) {
#pragma unroll 1
        for (int j = 0; j < 4; ++j) {
            const GkStep2 c = c_gk_step2[j];
            ff2 fm, fp;
            ff_node_pair2<P, D>(b, ff2{c.xh, c.xl}, ff2{c.x2h, c.x2l}, fm, fp);
            const ff2 sum = ff2_add(fm, fp);
            kk2 = ff2_fma(ff2{c.wkh, c.wkl}, sum, kk2);
            gg2 = ff2_fma(ff2{c.wgh, c.wgl}, sum, gg2);  // zero weights on the Kronrod-only pairs
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const ff2 x = pack(to_ff(split_const(gk_pair_x(2 * j))), to_ff(split_const(gk_pair_x(2 * j + 1))));
            const ff2 x2 = pack(to_ff(split_const(gk_pair_x(2 * j) * gk_pair_x(2 * j))),
                                to_ff(split_const(gk_pair_x(2 * j + 1) * gk_pair_x(2 * j + 1))));
            ff2 fm, fp;
            ff_node_pair2<P, D>(b, x, x2, fm, fp);
            const ff2 sum = ff2_add(fm, fp);
            kk2 = ff2_fma(pack(to_ff(split_const(gk_pair_wk(2 * j))), to_ff(split_const(gk_pair_wk(2 * j + 1)))), sum, kk2);
            // the Gauss nodes: pairs 1, 3, 5 and the centre (lane 1)
            gg2 = ff2_fma(pack(to_ff(split_const(gk_pair_wg(2 * j))), to_ff(split_const(gk_pair_wg(2 * j + 1)))), sum,
                          gg2);
        }
    }
    const ff kk = ff_add(lane0(kk2), lane1(kk2));
    const ff gg = ff_add(lane0(gg2), lane1(gg2));
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
