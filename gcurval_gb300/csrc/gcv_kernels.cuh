// Kernels of the FP64 arc-length path (set-up, adaptive length, scan,
// sampling) and their parameter blocks.  Included by gcv_kernels.cu, which
// instantiates them, and by the header-only plugin path.
#pragma once

#include "gcv_table.cuh"

namespace gcv {

// ---------------------------------------------------------------- set-up
// One thread per segment: segment -> curve map consumer; writes the
// evaluation data of the segment (B-spline polynomials or ellipse terms).
// stores a segment's coefficients: FP64, or float-float (hi, lo) pairs when
// the table is built for the mixed path
template <int N>
__device__ __forceinline__ void store_coef(const Table& t, int64_t at, const double* cf)
{
    if (t.coef_ff) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float h = __double2float_rn(cf[i]);
            t.coef_ff[at + i] = make_float2(h, __double2float_rn(cf[i] - (double)h));
        }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) t.coef[at + i] = cf[i];
    }
}

template <int P, int D>
__device__ void setup_bspline_seg(const Batch& b, const Table& t, int64_t s, int64_t c)
{
    constexpr int N = code_stride(bs_code(P, D));
    const int64_t j = s - b.seg_off[c];
    const double* kv = b.knots + b.knot_off[c];
    const double* cp = b.ctrl + b.ctrl_off[c];
    const int span = int(j) + P;
    const int64_t at = b.coef_off[c] + j * N;
    const double ka = kv[span], kb = kv[span + 1];
    if (!(kb >= ka)) raise_err(t, ERR_BAD_KNOTS);
    double cf[N];
    if (kb > ka) {
        bspline_setup<P, D>(kv, cp, span, cf);
        t.seg_t0[s] = ka;
        t.seg_t1[s] = kb;
        double r[P * D], q0;
        Eval<bs_code(P, D)>::load_speed(cf, r);
        t.seg_f0[s] = Eval<bs_code(P, D)>::speed_slope(r, -1.0, q0);
        t.seg_q0[s] = q0;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) cf[i] = 0.0;
        t.seg_t0[s] = ka;
        t.seg_t1[s] = ka;
        t.seg_f0[s] = 0.0;
        t.seg_q0[s] = 0.0;
    }
    store_coef<N>(t, at, cf);
}

__device__ inline void setup_ellipse_seg(const Batch& b, const Table& t, int64_t s, int64_t c)
{
    const int j = int(s - b.seg_off[c]);  // piece 0 .. ELLIPSE_PIECES - 1
    const double* e = b.ctrl + b.ctrl_off[c];
    const double a = e[0], bb = e[1];
    double sr, cr;
    sincos(e[2], &sr, &cr);
    constexpr double h = PI * ELLIPSE_PIECE_SCALE;
    const double w0 = (2 * j + 1) * ELLIPSE_PIECE_SCALE - 1.0;
    const double out[9] = {(a * a - bb * bb) * (h * h), bb * bb * (h * h), w0, a, bb, cr, sr, e[3], e[4]};
    store_coef<9>(t, b.coef_off[c] + (int64_t)j * 9, out);
    t.seg_t0[s] = (2.0 * PI * ELLIPSE_PIECE_SCALE) * j;
    t.seg_t1[s] = j + 1 == ELLIPSE_PIECES ? 2.0 * PI : (2.0 * PI * ELLIPSE_PIECE_SCALE) * (j + 1);
    double q0;
    t.seg_f0[s] = ellipse_speed_slope(out[0], out[1], w0, -1.0, q0);
    t.seg_q0[s] = q0;
}

// ------------------------------------------------------------- sampling
// One thread per sample: curve by binary search of the sample offsets,
// segment by binary search of the cumulative segment table, leaf panel by
// binary search of the segment's leaves, then Newton on
//   F(v) = S(v_a) + GL8(v_a, v) - r
// from a cubic-Hermite guess of the inverse map, safeguarded by bisection.
struct SampleParams {
    Batch b;
    Table t;
    const int64_t* sample_off;  // [n_curve + 1]
    const double* pos;
    int is_relative;
    int what;  // 2 = parameters, 3 = points
    int pdim;
    double* out;
    int64_t n_samples;
    int collect;
    double rtol;  // the table's tolerance: samples are placed to SAMPLE_EPS_FRAC of rtol * L
    float eps_frac;  // SAMPLE_EPS_FRAC * rtol (the mixed sampler's stopping threshold over L)
    // Batches that mix curve codes run one launch per code over the curves
    // curve_list[cb .. ce) (grouped by code); list_off is the prefix of their
    // sample counts in that order.  curve_list NULL: all samples, curve order.
    const int* curve_list;
    const int64_t* list_off;
    int64_t cb, ce;
    int64_t s_begin, s_end;  // sample range of the launch when curve_list is NULL
    const int64_t* s_end_dev;  // when set: the end of that range, read on the device
};

// Sample range of a launch and, for launch-local sample i, its curve and its
// index gi in the caller's position / output arrays.
__device__ __forceinline__ void sample_range(const SampleParams& P, int64_t& i0, int64_t& i1)
{
    i0 = P.curve_list ? P.list_off[P.cb] : P.s_begin;
    i1 = P.curve_list ? P.list_off[P.ce] : (P.s_end_dev ? *P.s_end_dev : P.s_end);
}
__device__ __forceinline__ int sample_curve(const SampleParams& P, int64_t i, int64_t& gi)
{
    if (P.curve_list) {
        const int64_t j = P.cb + upper_bound_i64(P.list_off + P.cb, int(P.ce - P.cb) + 1, i);
        const int c = P.curve_list[j];
        gi = P.sample_off[c] + (i - P.list_off[j]);
        return c;
    }
    gi = i;
    return upper_bound_i64(P.sample_off, int(P.b.n_curve) + 1, i);
}

// The curve of sample i with a per-thread memory of the last curve found:
// a thread that meets the same curve again skips the binary search (the
// mixed sampler hands each warp runs of consecutive samples).
struct CurveHint {
    int64_t lo = 0, hi = 0;  // sample range (list order) of the remembered curve
    int64_t shift = 0;       // its global sample index minus the list-order one
    int c = 0;
};
__device__ __forceinline__ int sample_curve_hint(const SampleParams& P, int64_t i, int64_t& gi, CurveHint& h)
{
    if (i >= h.lo && i < h.hi) {
        gi = i + h.shift;
        return h.c;
    }
    if (P.curve_list) {
        const int64_t j = P.cb + upper_bound_i64(P.list_off + P.cb, int(P.ce - P.cb) + 1, i);
        h.c = P.curve_list[j];
        h.lo = P.list_off[j];
        h.hi = P.list_off[j + 1];
        h.shift = P.sample_off[h.c] - h.lo;
    } else {
        h.c = upper_bound_i64(P.sample_off, int(P.b.n_curve) + 1, i);
        h.lo = P.sample_off[h.c];
        h.hi = P.sample_off[h.c + 1];
        h.shift = 0;
    }
    gi = i + h.shift;
    return h.c;
}
// samples per warp and turn in the mixed sampler (8 per lane, 32 apart)
constexpr int SAMPLE_RUN = 256;

// Newton stops once the estimated residual of its last step is below
// SAMPLE_EPS_FRAC * rtol * L.  The table itself is good to rtol * L (the
// length walk's per-interval tolerance, summed), so a tenth of that keeps a
// sample's total error within 1.1 rtol * L.
constexpr double SAMPLE_EPS_FRAC = 0.1;

constexpr int SAMPLE_THREADS = 256;      // default block size
constexpr int SAMPLE_THREADS_MAX = 512;  // largest block size the autotuner tries
constexpr int NEWTON_MAXIT = 16;

template <int CODE>
__device__ __forceinline__ double speed_of(int code, const double* r, double v)
{
    if constexpr (CODE >= 0)
        return Eval<CODE>::speed(r, v);
    else
        return speed_dyn(code, r, v);
}

template <int CODE>
__device__ __forceinline__ double speed_slope_of(int code, const double* r, double v, double& q)
{
    if constexpr (CODE >= 0)
        return Eval<CODE>::speed_slope(r, v, q);
    else
        return speed_slope_dyn(code, r, v, q);
}

// Newton on one leaf [va, vb] (cumulative lengths base, cb) for the target rr,
// from the guess vg: F(v) = S(v) - rr with S(v) = S(va) + GL8(va, v) or
// S(vb) - GL8(v, vb), whichever side of v is shorter (at most half a leaf,
// where GL8 is far more accurate than the leaf's own G7 error estimate);
// bracketed by bisection.
// Each iteration takes a second-order step: with f0 = f(v) and f1 = f(v - dn)
// at the Newton point (dn = F / f0), the trapezoid rule d (f0 + f1) / 2
// gives the arc length of a step d, so d = 2 F / (f0 + f1).  It stops when
// that step's residual is below eps_s: the trapezoid error |d|^3 |f''| / 12
// with f'' from the two slopes, taken 4-fold (dn^2 |f'(v - dn) - f'(v)| / 3),
// plus |f'|^2 |dn|^3 / (4 f) for using f at v - dn rather than at v - d.
// A first-order test from the slope at v alone (|f'(v)| dn^2 / 2) accepts
// large steps wherever v sits at an extremum of the speed (f'(v) ~ 0), and
// misplaced such samples by 1e-8 of the curve's length; this test sees the
// slope change across the step.
// 8-point Gauss nodes (-x0..-x3, x0..x3) and weights w0..w3 for rolled loops
static __constant__ double c_gl8[12] = {-gl8_x(0), -gl8_x(1), -gl8_x(2), -gl8_x(3), gl8_x(0), gl8_x(1),
                                        gl8_x(2),  gl8_x(3),  gl8_w(0),  gl8_w(1),  gl8_w(2), gl8_w(3)};

// UNROLL: fixed-code kernels unroll the Gauss loop; the runtime-dispatch
// kernel keeps it rolled so that eleven specialised bodies fit the
// instruction cache.
template <int C, bool UNROLL = true>
__device__ __forceinline__ double leaf_newton(const double* __restrict__ seg, double va, double vb, double base,
                                              double cb, double rr, double vg, double eps_s,
                                              unsigned long long& newton)
{
    double r[MAX_COEF];
    Eval<C>::load_speed(seg, r);
    double blo = va, bhi = vb, v = vg;
    for (int it = 0; it < NEWTON_MAXIT; ++it) {
        ++newton;
        const bool from_left = (v - va) <= (vb - v);
        const double a0 = from_left ? va : v, a1 = from_left ? v : vb;
        const double h2 = 0.5 * (a1 - a0);
        const double m2 = a0 + h2;
        double I = 0.0;
        if constexpr (UNROLL) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const double xk = h2 * gl8_x(k);
                I = fma(gl8_w(k), Eval<C>::speed(r, m2 - xk) + Eval<C>::speed(r, m2 + xk), I);
            }
        } else {
#pragma unroll 1
            for (int k = 0; k < 8; ++k) I = fma(c_gl8[8 + (k & 3)], Eval<C>::speed(r, fma(h2, c_gl8[k], m2)), I);
        }
        const double F = (from_left ? base + I * h2 : cb - I * h2) - rr;
        if (F == 0.0) break;
        if (F < 0.0)
            blo = v;
        else
            bhi = v;
        double q0;
        const double f0 = Eval<C>::speed_slope(r, v, q0);
        const double dn = F / f0;
        double vn = v - dn;
        // the second-order step only from a Newton point inside the closed
        // bracket (a step below one ulp of v leaves vn == v, which must still
        // converge); a Newton point outside it would take f1 from the
        // polynomial extrapolated past the leaf
        if (vn >= blo && vn <= bhi) {
            double q1;
            const double f1 = Eval<C>::speed_slope(r, vn, q1);
            const double d = 2.0 * F / (f0 + f1);
            const double s0 = q0 / f0, s1 = q1 / f1;  // f'(v), f'(v - dn)
            const double res = dn * dn * (fabs(s1 - s0) * (1.0 / 3.0) + s1 * s1 * fabs(dn) / (4.0 * f1));
            vn = v - d;
            if (res <= eps_s && vn >= va && vn <= vb) {  // converged with this step
                v = vn;
                break;
            }
        }
        if (!(vn > blo && vn < bhi)) vn = 0.5 * (blo + bhi);  // safeguard (also NaN)
        v = vn;
    }
    return v;
}

template <int CODE>
__global__ void __launch_bounds__(SAMPLE_THREADS_MAX) k_sample(SampleParams P)
{
    const Batch& b = P.b;
    const Table& t = P.t;
    unsigned long long newton = 0;
    int64_t i0, i1;
    sample_range(P, i0, i1);
    for (int64_t ii = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ii < i1;
         ii += (int64_t)gridDim.x * blockDim.x) {
        int64_t i;
        const int c = sample_curve(P, ii, i);
        const int code = CODE >= 0 ? CODE : curve_code(b, c);
        const int64_t s0 = b.seg_off[c], s1 = b.seg_off[c + 1];
        int64_t s;
        double v;
        if (s1 == s0) {  // curve without knot intervals: its start
            s = -1;
            v = -1.0;
        } else {
            const double L = t.curve_len[c];
            const double pos = P.pos[i];
            const double target = P.is_relative ? pos * L : pos;
            if (!(target > 0.0)) {
                s = s0;
                v = -1.0;
            } else if (target >= L) {
                s = s1 - 1;
                v = 1.0;
            } else {
                s = lower_bound_key(t.seg_cum, s0, s1, dkey(target));
                if (s == s1) s = s1 - 1;
                const double prev = s > s0 ? t.seg_cum[s - 1] : 0.0;
                const double rr = target - prev;
                const int64_t lo = t.leaf_off[s];
                const int cnt = t.leaf_cnt[s];
                int64_t j = lower_bound_key(t.leaf_cum, lo, lo + cnt, dkey(rr)) - lo;
                if (j >= cnt) j = cnt - 1;
                const double base = j ? t.leaf_cum[lo + j - 1] : 0.0;
                const double va = j ? t.leaf_v[lo + j - 1] : -1.0;
                const double fa = j ? t.leaf_f[lo + j - 1] : t.seg_f0[s];
                const double qa = j ? t.leaf_q[lo + j - 1] : t.seg_q0[s];
                const double vb = t.leaf_v[lo + j];
                const double cb = t.leaf_cum[lo + j];
                const double fb = t.leaf_f[lo + j];
                const double qb = t.leaf_q[lo + j];
                const double dS = cb - base, dv = vb - va;
                // initial guess: quintic Hermite of the inverse map v(S) on the
                // leaf, from v' = 1/f and v'' = -f'/f^3 = -q/f^4 at both ends
                double sig = dS > 0.0 ? (rr - base) / dS : 0.0;
                sig = fmin(fmax(sig, 0.0), 1.0);
                double vg = va + sig * dv;
                const double fm = dS / dv;
                if (fa > 0.1 * fm && fb > 0.1 * fm) {
                    const double s2 = sig * sig, s3 = s2 * sig, s4 = s3 * sig, s5 = s4 * sig;
                    const double h5 = 10.0 * s3 - 15.0 * s4 + 6.0 * s5;
                    const double h1 = sig - 6.0 * s3 + 8.0 * s4 - 3.0 * s5;
                    const double h4 = -4.0 * s3 + 7.0 * s4 - 3.0 * s5;
                    const double h2 = 0.5 * (s2 - 3.0 * s3 + 3.0 * s4 - s5);
                    const double h3 = 0.5 * (s3 - 2.0 * s4 + s5);
                    const double ia = 1.0 / fa, ib = 1.0 / fb;
                    const double ka = -qa * (ia * ia) * (ia * ia), kb = -qb * (ib * ib) * (ib * ib);
                    vg = va + h5 * dv + dS * (h1 * ia + h4 * ib) + dS * dS * (h2 * ka + h3 * kb);
                    vg = fmin(fmax(vg, va), vb);
                }
                const double* seg = t.coef + b.coef_off[c] + (s - s0) * code_stride(code);
                // stop when the residual of the last step is below
                // SAMPLE_EPS_FRAC * rtol * L
                const double eps_s = SAMPLE_EPS_FRAC * P.rtol * L;
                if constexpr (CODE >= 0) {
                    v = leaf_newton<(CODE >= 0 ? CODE : 0)>(seg, va, vb, base, cb, rr, vg, eps_s, newton);
                } else {
                    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: v = leaf_newton<C, false>(seg, va, vb, base, cb, rr, vg, eps_s, newton); break;
                        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
                    default: v = vg; break;
                    }
                }
            }
        }
        if (P.what == 2) {
            double u;
            if (s < 0) {
                u = b.kind[c] == 0 ? 0.0 : b.knots[b.knot_off[c] + b.degree[c]];
            } else {
                // exact at both ends of the knot interval
                const double t0 = t.seg_t0[s], t1 = t.seg_t1[s], hw = 0.5 * (t1 - t0);
                u = v <= 0.0 ? fma(v + 1.0, hw, t0) : fma(v - 1.0, hw, t1);
            }
            P.out[i] = u;
        } else {
            double p3[3] = {0.0, 0.0, 0.0};
            if (s >= 0) {
                const double* seg = t.coef + b.coef_off[c] + (s - s0) * code_stride(code);
                if constexpr (CODE >= 0)
                    Eval<(CODE >= 0 ? CODE : 0)>::point(seg, v, p3);
                else
                    point_dyn(code, seg, v, p3);
            }
            for (int k = 0; k < P.pdim; ++k) P.out[i * P.pdim + k] = p3[k];
        }
    }
    if (P.collect) {
        for (int o = 16; o > 0; o >>= 1) newton += __shfl_xor_sync(0xffffffffu, newton, o);
        if ((threadIdx.x & 31) == 0 && newton) atomicAdd(t.ctr + C_NEWTON, newton);
    }
}

// ------------------------------------------------------------ FMA probe
// Register-only throughput probe: 8 independent FMA chains per thread.
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T seed)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + T(threadIdx.x + k);
    const T m = T(0.999999), c = T(1e-7);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == T(-1.2345)) out[0] = s;  // never true; keeps the chains live
}

}  // namespace gcv
