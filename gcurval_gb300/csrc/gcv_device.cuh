// Device-side building blocks of the arc-length library: quadrature
// constants, curve evaluators on per-knot-interval polynomials, the symbolic
// de Boor set-up of those polynomials, and warp helpers.
//
// Every knot interval ("segment") is mapped to a local variable v in [-1, 1]:
//   B-spline  t = t0 + (v + 1) * hw,  hw = (k[span+1] - k[span]) / 2
//   ellipse   piece j of ELLIPSE_PIECES equal parameter pieces of [0, 2 pi]:
//             theta = pi * (2 j + 1 + v) / ELLIPSE_PIECES
// and the integrand is f(v) = |dC/dv| = |C'(t)| * hw, so that the segment
// length is the integral of f over [-1, 1].
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gcv {

// ---------------------------------------------------------------- constants
// 15-point Kronrod rule with its embedded 7-point Gauss rule (the published
// Gauss-Kronrod G7-K15 nodes and weights), nodes descending from the right end.
__host__ __device__ constexpr double gk_x(int i)
{
    return i == 0 ? 0.991455371120812639206854697526329
         : i == 1 ? 0.949107912342758524526189684047851
         : i == 2 ? 0.864864423359769072789712788640926
         : i == 3 ? 0.741531185599394439863864773280788
         : i == 4 ? 0.586087235467691130294144845693013
         : i == 5 ? 0.405845151377397166906606412076961
         : i == 6 ? 0.207784955007898467600689403773245
                  : 0.0;
}
__host__ __device__ constexpr double gk_wk(int i)
{
    return i == 0 ? 0.022935322010529224963732008058970
         : i == 1 ? 0.063092092629978553290700663189204
         : i == 2 ? 0.104790010322250183839876322541518
         : i == 3 ? 0.140653259715525918745189590510238
         : i == 4 ? 0.169004726639267902826583426598550
         : i == 5 ? 0.190350578064785409913256402421014
         : i == 6 ? 0.204432940075298892414161999234649
                  : 0.209482141084727828012999174891714;
}
// Gauss weights of the odd Kronrod indices 1, 3, 5 and of the centre (7)
__host__ __device__ constexpr double gk_wg(int i)
{
    return i == 1 ? 0.129484966168869693270611432679082
         : i == 3 ? 0.279705391489276667901467771423780
         : i == 5 ? 0.381830050505118944950369775488975
         : i == 7 ? 0.417959183673469387755102040816327
                  : 0.0;
}

// 8-point Gauss-Legendre nodes / weights (positive half; symmetric)
__host__ __device__ constexpr double gl8_x(int i)
{
    return i == 0 ? 0.183434642495649804939476142360184
         : i == 1 ? 0.525532409916328985817739049189254
         : i == 2 ? 0.796666477413626739591553936475830
                  : 0.960289856497536231683560868569473;
}
__host__ __device__ constexpr double gl8_w(int i)
{
    return i == 0 ? 0.362683783378361982965150449277196
         : i == 1 ? 0.313706645877887287337962201986601
         : i == 2 ? 0.222381034453374470544355994426241
                  : 0.101228536290376259152531354309962;
}

constexpr double PI = 3.141592653589793238462643383279502884;

// Node of half-warp lane `hl` (0..15): lanes 0..6 take -x_k, lane 7 the
// centre, lanes 8..14 +x_{14-hl}; lane 15 the panel's right end (weights 0).
__host__ __device__ inline void gk_lane(int hl, double& x, double& wk, double& wg)
{
    if (hl < 7) {
        x = -gk_x(hl);
        wk = gk_wk(hl);
        wg = gk_wg(hl);
    } else if (hl == 7) {
        x = 0.0;
        wk = gk_wk(7);
        wg = gk_wg(7);
    } else if (hl < 15) {
        x = gk_x(14 - hl);
        wk = gk_wk(14 - hl);
        wg = gk_wg(14 - hl);
    } else {
        x = 1.0;
        wk = 0.0;
        wg = 0.0;
    }
}

// ------------------------------------------------------------ curve codes
// 0 = ellipse; B-splines 16 + 4 p + D for degree p in 1..5 and D in {2, 3}.
constexpr int CODE_ELLIPSE = 0;
__host__ __device__ constexpr int bs_code(int p, int d) { return 16 + 4 * p + d; }
__host__ __device__ constexpr int code_degree(int code) { return code == 0 ? 0 : (code - 16) / 4; }
__host__ __device__ constexpr int code_dim(int code) { return code == 0 ? 2 : (code - 16) % 4; }
// values of coefficient data per segment: the position polynomial of a
// B-spline piece ((p + 1) D), the 9 ellipse terms
__host__ __device__ constexpr int code_stride(int code)
{
    return code == 0 ? 9 : (code_degree(code) + 1) * code_dim(code);
}
// An ellipse is integrated as this many equal parameter pieces (a power of
// two, so that v / ELLIPSE_PIECES is exact): more lanes per curve and a few
// leaves per piece instead of one long chain of panels.
constexpr int ELLIPSE_PIECES = 8;
constexpr double ELLIPSE_PIECE_SCALE = 1.0 / ELLIPSE_PIECES;
constexpr int MAX_DEGREE = 5;
constexpr int MAX_COEF = 18;  // (5 + 1) * 3

// Exact 2^-k for 0 <= k <= 1000 built from the exponent bits (no FP64 op).
__device__ __forceinline__ double pow2_neg(int k)
{
    return __longlong_as_double((long long)(1023 - k) << 52);
}

// ------------------------------------------------------------- evaluators
// Ellipse piece data (9 doubles): A = (a^2 - b^2) h^2, B = b^2 h^2 with
// h = pi / ELLIPSE_PIECES, w0 = (2 j + 1) / ELLIPSE_PIECES - 1, then a, b,
// cos(rot), sin(rot), cx, cy.  With w = w0 + v / ELLIPSE_PIECES in [-1, 1]
// (theta = pi (w + 1)): f(v) = sqrt(B + A sin^2(pi w)), because
// |C'(theta)|^2 = a^2 sin^2 + b^2 cos^2 and sin^2(pi (w + 1)) = sin^2(pi w).
__device__ __forceinline__ double ellipse_speed(double A, double B, double w0, double v)
{
    const double s = sinpi(fma(v, ELLIPSE_PIECE_SCALE, w0));
    return sqrt(fma(A * s, s, B));
}

// B-spline segment data: position polynomial a[k][d] (k = 0..P), then the
// derivative polynomial b[k][d] = (k + 1) a[k + 1][d] (k = 0..P-1), both in v.
template <int P, int D>
__device__ __forceinline__ double bs_speed(const double* b, double v)
{
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double acc = b[(P - 1) * D + d];
#pragma unroll
        for (int k = P - 2; k >= 0; --k) acc = fma(acc, v, b[k * D + d]);
        s = d == 0 ? acc * acc : fma(acc, acc, s);
    }
    return sqrt(s);
}

// f = |g(v)| and q = g(v) . g'(v) (so df/dv = q / f): Horner for the value
// and its derivative in one pass.
template <int P, int D>
__device__ __forceinline__ double bs_speed_slope(const double* b, double v, double& q)
{
    double s = 0.0, t = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double acc = b[(P - 1) * D + d], dacc = 0.0;
#pragma unroll
        for (int k = P - 2; k >= 0; --k) {
            dacc = fma(dacc, v, acc);
            acc = fma(acc, v, b[k * D + d]);
        }
        s = d == 0 ? acc * acc : fma(acc, acc, s);
        t = d == 0 ? acc * dacc : fma(acc, dacc, t);
    }
    q = t;
    return sqrt(s);
}

// ellipse: f^2 = B + A sin^2(pi w), dw/dv = 1 / ELLIPSE_PIECES, so
// q = f f' = A sin cos pi / ELLIPSE_PIECES
__device__ __forceinline__ double ellipse_speed_slope(double A, double B, double w0, double v, double& q)
{
    double s, c;
    sincospi(fma(v, ELLIPSE_PIECE_SCALE, w0), &s, &c);
    q = (PI * ELLIPSE_PIECE_SCALE) * A * s * c;
    return sqrt(fma(A * s, s, B));
}

template <int P, int D>
__device__ __forceinline__ void bs_point(const double* a, double v, double* out)
{
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double acc = a[P * D + d];
#pragma unroll
        for (int k = P - 1; k >= 0; --k) acc = fma(acc, v, a[k * D + d]);
        out[d] = acc;
    }
}

// Register copy of one segment's evaluation data.
struct SegRegs {
    double c[MAX_COEF];
};

template <int CODE>
struct Eval {
    static constexpr int P = code_degree(CODE);
    static constexpr int D = code_dim(CODE);
    static constexpr int NL = CODE == 0 ? 3 : P * D;  // doubles the speed needs
    // loads what speed() needs: ellipse A, B, w0, or the derivative polynomial
    // b[k][d] = (k + 1) a[k + 1][d] of the stored position polynomial a
    __device__ __forceinline__ static void load_speed(const double* __restrict__ seg, double* r)
    {
        if constexpr (CODE == 0) {
            r[0] = seg[0];
            r[1] = seg[1];
            r[2] = seg[2];
        } else {
#pragma unroll
            for (int k = 0; k < P; ++k)
#pragma unroll
                for (int d = 0; d < D; ++d) r[k * D + d] = double(k + 1) * seg[(k + 1) * D + d];
        }
    }
    __device__ __forceinline__ static double speed(const double* r, double v)
    {
        if constexpr (CODE == 0)
            return ellipse_speed(r[0], r[1], r[2], v);
        else
            return bs_speed<P, D>(r, v);
    }
    // speed and q = f * df/dv
    __device__ __forceinline__ static double speed_slope(const double* r, double v, double& q)
    {
        if constexpr (CODE == 0)
            return ellipse_speed_slope(r[0], r[1], r[2], v, q);
        else
            return bs_speed_slope<P, D>(r, v, q);
    }
    // point at local v (writes D doubles; ellipses apply rotation and centre)
    __device__ __forceinline__ static void point(const double* __restrict__ seg, double v, double* out)
    {
        if constexpr (CODE == 0) {
            // theta / pi = (2 j + 1 + v) / ELLIPSE_PIECES = (w0 + 1) + v / ELLIPSE_PIECES
            double s, c;
            sincospi(fma(v, ELLIPSE_PIECE_SCALE, seg[2] + 1.0), &s, &c);
            const double x = seg[3] * c, y = seg[4] * s;
            out[0] = seg[5] * x - seg[6] * y + seg[7];
            out[1] = seg[6] * x + seg[5] * y + seg[8];
        } else {
            double a[(P + 1) * D];
#pragma unroll
            for (int i = 0; i < (P + 1) * D; ++i) a[i] = seg[i];
            bs_point<P, D>(a, v, out);
        }
    }
};

// Runtime dispatch over every built-in code, for batches that mix curve kinds.
#define GCV_FOR_EACH_CODE(X)                                                                       \
    X(0) X(bs_code(1, 2)) X(bs_code(2, 2)) X(bs_code(3, 2)) X(bs_code(4, 2)) X(bs_code(5, 2))      \
        X(bs_code(1, 3)) X(bs_code(2, 3)) X(bs_code(3, 3)) X(bs_code(4, 3)) X(bs_code(5, 3))

__device__ __forceinline__ void load_speed_dyn(int code, const double* __restrict__ seg, double* r)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: Eval<C>::load_speed(seg, r); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: break;
    }
}

__device__ __forceinline__ double speed_dyn(int code, const double* r, double v)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: return Eval<C>::speed(r, v);
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: return 0.0;
    }
}

__device__ __forceinline__ double speed_slope_dyn(int code, const double* r, double v, double& q)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: return Eval<C>::speed_slope(r, v, q);
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: q = 0.0; return 0.0;
    }
}

__device__ __forceinline__ void point_dyn(int code, const double* __restrict__ seg, double v, double* out)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: Eval<C>::point(seg, v, out); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: break;
    }
}

// ------------------------------------------------- symbolic de Boor set-up
// Power-basis coefficients in v of the B-spline piece on knot span `span`
// (k[span] < k[span+1]): the reference's basis recursion
// (samples/sample2_bspline/BSpline.h:26-96, b_spline_func_value /
// b_spline_derv_o1 / to_point) run on polynomials in v instead of numbers,
// with u = m + w v, m the span midpoint and w its half width.  The
// denominators right[r+1] + left[j-r] are knot differences and do not depend
// on u.  Output: the position polynomial a[k][d], k = 0..P; the derivative
// dC/dv is b[k][d] = (k + 1) a[k + 1][d] (see Eval::load_speed).
template <int P, int D>
__device__ void bspline_setup(const double* __restrict__ kv, const double* __restrict__ cp, int span,
                              double* out)
{
    const double ka = kv[span], kb = kv[span + 1];
    const double m = 0.5 * (ka + kb), w = 0.5 * (kb - ka);
    // N[r][k]: basis polynomial r, coefficient of v^k (degree <= P)
    double N[P + 1][P + 1];
#pragma unroll
    for (int r = 0; r <= P; ++r)
#pragma unroll
        for (int k = 0; k <= P; ++k) N[r][k] = 0.0;
    N[0][0] = 1.0;
    // at step j the basis polynomials N[0..j-1] have degree j - 1 and the
    // new ones degree j: the loops run over those coefficients only
#pragma unroll
    for (int j = 1; j <= P; ++j) {
        double saved[P + 1];
#pragma unroll
        for (int k = 0; k <= j; ++k) saved[k] = 0.0;
#pragma unroll
        for (int r = 0; r < j; ++r) {
            const double kr = kv[span + r + 1];      // right[r+1] = kr - u
            const double kl = kv[span + 1 - j + r];  // left[j-r]  = u - kl
            const double inv = 1.0 / (kr - kl);
            double temp[P + 1];
#pragma unroll
            for (int k = 0; k < j; ++k) temp[k] = N[r][k] * inv;
            const double ra = kr - m, la = m - kl;  // right = ra - w v, left = la + w v
#pragma unroll
            for (int k = j; k >= 0; --k) {
                if (k == j) {  // only the v * temp[j-1] terms reach degree j
                    N[r][k] = saved[k] - w * temp[k - 1];
                    saved[k] = w * temp[k - 1];
                } else if (k == 0) {
                    N[r][k] = saved[k] + ra * temp[k];
                    saved[k] = la * temp[k];
                } else {
                    N[r][k] = saved[k] + (ra * temp[k] - w * temp[k - 1]);
                    saved[k] = la * temp[k] + w * temp[k - 1];
                }
            }
        }
#pragma unroll
        for (int k = 0; k <= j; ++k) N[j][k] = saved[k];
    }
    // position: C(v) = sum_i P_{span-P+i} N_i(v).  The basis sums to one, so
    // combining differences P_i - P_0 and adding P_0 back to the constant
    // term keeps the higher coefficients free of cancellation against |P|.
    const double* c0 = cp + (size_t)(span - P) * D;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const double q = c0[d];
#pragma unroll
        for (int k = 0; k <= P; ++k) {
            double acc = 0.0;
#pragma unroll
            for (int i = 1; i <= P; ++i) acc = fma(c0[i * D + d] - q, N[i][k], acc);
            out[k * D + d] = k == 0 ? acc + q : acc;
        }
    }
}

// ------------------------------------------------------------ warp helpers
__device__ __forceinline__ double half_sum(double x, unsigned mask)
{
    // xor butterfly inside a 16-lane half: partners add a+b and b+a, so every
    // lane ends with the bitwise-same total
    x += __shfl_xor_sync(mask, x, 8);
    x += __shfl_xor_sync(mask, x, 4);
    x += __shfl_xor_sync(mask, x, 2);
    x += __shfl_xor_sync(mask, x, 1);
    return x;
}

// Non-negative doubles order like their bit patterns: binary searches on
// cumulative lengths compare 64-bit integers instead of using the FP64 pipe.
__device__ __forceinline__ long long dkey(double x) { return __double_as_longlong(x); }

// first index in [lo, hi) with a[i] >= key (a non-decreasing, non-negative)
__device__ __forceinline__ int64_t lower_bound_key(const double* __restrict__ a, int64_t lo, int64_t hi,
                                                   long long key)
{
    int64_t n = hi - lo;
    while (n > 0) {
        const int64_t h = n >> 1;
        if (dkey(__ldg(a + lo + h)) < key) {
            lo += h + 1;
            n -= h + 1;
        } else {
            n = h;
        }
    }
    return lo;
}

// last index i in [0, n) with off[i] <= x (off non-decreasing, off[0] <= x)
__device__ __forceinline__ int upper_bound_i64(const int64_t* __restrict__ off, int n, int64_t x)
{
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int h = cnt >> 1;
        if (__ldg(off + lo + h) <= x) {
            lo += h + 1;
            cnt -= h + 1;
        } else {
            cnt = h;
        }
    }
    return lo - 1;
}

}  // namespace gcv
