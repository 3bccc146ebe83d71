// Mixed-precision path (GCV_MIXED): the integrand and the panel sums run on
// the FP32 pipes in float-float arithmetic (gcv_ff.cuh, ~48-bit significand);
// FP64 is kept for the three steps whose stability needs it:
//   * the compensated prefix sum of interval lengths (k_scan, shared with the
//     FP64 path),
//   * the panel error test when the FP32 test lands near the tolerance,
//   * the final Newton update of every sample's parameter.
// Plain FP32 integrands (rounding ~3e-8 per evaluation, plus the systematic
// rounding of each interval's polynomial coefficients) cannot hold a 1e-8
// relative length on curves of one or a few knot intervals; float-float can,
// at a fraction of the FP64 cost on GB300 (FP32:FP64 throughput ~75:1).
//
// Ellipse integrands (sin^2(pi v)) are evaluated with an own float-float
// series for sin^2(pi u), |u| <= 1/4, after folding (gcv_ff_eval.cuh).
#pragma once

#include "gcv_ff_eval.cuh"
#include "gcv_kernels.cuh"

namespace gcv {

// ------------------------------------------------------------- sampling
// Newton on one leaf in float-float, in the local offset w = v - va in
// [0, dv]: F(w) = S(va + w) - S(va) - rl with the partial integral taken by
// 8-point Gauss over the shorter side of the leaf, bracketed by bisection.
// Second-order steps and the stopping test of leaf_newton (gcv_kernels.cuh):
// d = 2 F / (f0 + f1) with f1 the speed at the Newton point, stop when
// dn^2 (|f'(w - dn) - f'(w)| / 3 + |f'|^2 |dn| / (4 f)) <= eps_s.
// Returns the final offset, whose last update is done in FP64.
// 8-point Gauss nodes (-x0..-x3, x0..x3) then weights w0..w3, float-float
#define GCV_FFC(x) {split_const(x).hi, split_const(x).lo}
static __constant__ float2 c_gl8_ff[12] = {
    GCV_FFC(-gl8_x(0)), GCV_FFC(-gl8_x(1)), GCV_FFC(-gl8_x(2)), GCV_FFC(-gl8_x(3)),
    GCV_FFC(gl8_x(0)),  GCV_FFC(gl8_x(1)),  GCV_FFC(gl8_x(2)),  GCV_FFC(gl8_x(3)),
    GCV_FFC(gl8_w(0)),  GCV_FFC(gl8_w(1)),  GCV_FFC(gl8_w(2)),  GCV_FFC(gl8_w(3))};
#undef GCV_FFC

// Whether the sampler of curve code C takes its Gauss sums by node pairs
// (gl8_pairs) rather than by evaluating each node: the B-spline codes of
// degree x dimension below 8.  The larger codes hold more coefficients than
// their register cap leaves room for beside the pairs' temporaries (100-236
// bytes of spills at 80-88 registers, and fewer resident warps at 96-104);
// sampling of the uneven 1M batch took 153.4 ms node by node, 149.2 with
// pairs for the small codes, 153.1 and 154.6 with pairs for every code at
// the two register budgets.
__host__ __device__ constexpr bool sample_node_pairs(int code)
{
    return code > 0 && code_degree(code) * code_dim(code) < 8;
}

// The 8-point Gauss sum over [m - h, m + h] of a B-spline code by symmetric
// node pairs, as the length walk's panels take theirs: b, the interval's
// speed coefficients, is shifted in place to m (b[j] = p^(j)(m) / j!), then
// pair k evaluates the even and odd parts at X = h x_k and returns
// w_k (f(m - X) + f(m + X)) into the sum (the caller scales it by h).  For
// degree 5 in 3D that is 30 float-float multiply-adds of shift plus 4 pairs
// instead of 8 Horner evaluations of 12.
template <int C, bool UNROLL>
__device__ __forceinline__ ff gl8_pairs(ff* b, ff m, ff h)
{
    constexpr int P = code_degree(C), D = code_dim(C);
#pragma unroll
    for (int i = 0; i < P - 1; ++i)
#pragma unroll
        for (int j = P - 2; j >= i; --j)
#pragma unroll
            for (int d = 0; d < D; ++d) b[j * D + d] = ff_fma(b[(j + 1) * D + d], m, b[j * D + d]);
    // pairs (0, 1) and (2, 3) in packed lanes
    const ff2 h2 = splat(h);
    ff2 I2{};
#pragma unroll
    for (int k = 0; k < 4; k += 2) {
        const ff2 X = ff2_mul(h2, pack(to_ff(split_const(gl8_x(k))), to_ff(split_const(gl8_x(k + 1)))));
        ff2 fm, fp;
        ff_node_pair2<P, D>(b, X, ff2_mul(X, X), fm, fp);
        I2 = ff2_fma(pack(to_ff(split_const(gl8_w(k))), to_ff(split_const(gl8_w(k + 1)))), ff2_add(fm, fp), I2);
    }
    return ff_add(lane0(I2), lane1(I2));
}

// UNROLL: small integrands unroll the Gauss loop; large ones (panel_rolled)
// and the runtime-dispatch kernel keep it rolled, so that the body fits the
// instruction cache.
template <int C, bool UNROLL>
__device__ __forceinline__ double ff_leaf_newton(const float2* __restrict__ seg, ff vaf, float dv, ff rl, ff dS,
                                                 float dvg, float eps_s, unsigned long long& newton)
{
    constexpr bool PAIRS = sample_node_pairs(C);
    float blo = 0.0f, bhi = dv;
    ff w{dvg, 0.0f};
    float last = 0.0f;  // the converged Newton step, applied in FP64 at the end
    for (int it = 0; it < NEWTON_MAXIT; ++it) {
        ++newton;
        ff r[MAX_COEF];
        EvalFF<C>::load(seg, r);  // every iteration: the node-pair Gauss sum shifts r
        const bool from_left = w.hi <= 0.5f * dv;
        // [a0, a1] in local offsets: [0, w] or [w, dv]
        const ff a0 = from_left ? ff{0.0f, 0.0f} : w;
        const ff a1 = from_left ? w : ff{dv, 0.0f};
        const ff h2 = ff_scale(ff_add(a1, ff_neg(a0)), 0.5f);
        const ff m2 = ff_add(ff_add(vaf, a0), h2);
        ff I{0.0f, 0.0f};
        if constexpr (PAIRS) {
            I = gl8_pairs<C, UNROLL>(r, m2, h2);  // r now holds the coefficients about m2
        } else {
            // nodes -x_k and +x_k in packed lanes
#pragma unroll 1
            for (int k = 0; k < 4; ++k) {
                const ff xk = ff_mul(h2, ff{c_gl8_ff[4 + k].x, c_gl8_ff[4 + k].y});
                const ff2 f = EvalFF<C>::speed2(r, pack(ff_add(m2, ff_neg(xk)), ff_add(m2, xk)));
                I = ff_fma(ff{c_gl8_ff[8 + k].x, c_gl8_ff[8 + k].y}, ff_add(lane0(f), lane1(f)), I);
            }
        }
        I = ff_mul(I, h2);
        // F = S(v) - target inside the leaf
        const ff F = from_left ? ff_add(I, ff_neg(rl)) : ff_add(ff_add(dS, ff_neg(I)), ff_neg(rl));
        const float Fh = F.hi + F.lo;
        if (Fh == 0.0f) break;
        if (Fh < 0.0f)
            blo = w.hi;
        else
            bhi = w.hi;
        // speed at w: after the node-pair sum from the coefficients about m2,
        // at the end +-h2 of the summed side that is w
        float q0, f0;
        if constexpr (PAIRS)
            f0 = EvalFF<C>::speed_slope_f(r, from_left ? h2 : ff_neg(h2), q0);
        else
            f0 = EvalFF<C>::speed_slope_f(r, ff_add(vaf, w), q0);
        const float dn = Fh / f0;
        float step = dn;
        // the second-order step only from a Newton point inside the closed
        // bracket (a step below one FP32 ulp of w leaves w.hi - dn == w.hi,
        // which must still converge); a Newton point outside it would take
        // f1 from the polynomial extrapolated past the leaf
        const float wn = w.hi - dn;
        if (wn >= blo && wn <= bhi) {
            float q1;
            // after the node-pair sum from the coefficients about m2, at the
            // offset (w - dn) - (a0 + h2) from it; else at va + w - dn
            float f1;
            if constexpr (PAIRS)
                f1 = EvalFF<C>::speed_slope_f(r, ff_add(ff_add_f(w, -dn), ff_neg(ff_add(a0, h2))), q1);
            else
                f1 = EvalFF<C>::speed_slope_f(r, ff_add(vaf, ff_add_f(w, -dn)), q1);
            const float d = 2.0f * Fh / (f0 + f1);
            const float s0 = q0 / f0, s1 = q1 / f1;  // f'(w), f'(w - dn)
            const float res = dn * dn * (fabsf(s1 - s0) * (1.0f / 3.0f) + s1 * s1 * fabsf(dn) / (4.0f * f1));
            const float wd = w.hi - d;
            if (res <= eps_s && wd >= 0.0f && wd <= dv) {
                last = d;  // converged: the step is applied in FP64
                break;
            }
            step = d;
        }
        const float ws = w.hi - step;
        if (ws > blo && ws < bhi)
            w = ff_add_f(w, -step);
        else
            w = ff{0.5f * (blo + bhi), 0.0f};  // safeguard (also NaN)
    }
    // the final update in FP64
    return ((double)w.hi + (double)w.lo) - (double)last;
}

// Mixed-precision sampling: table lookups and the target in FP64, the
// quintic-Hermite guess in FP32, Newton on the leaf in float-float
// (G8 partial integral on the shorter side, local to the leaf), and the
// final update of v in FP64.
// Registers per thread are capped (blocks of up to SAMPLE_THREADS_MAX threads
// still fit): left to itself the compiler gave the degree-4/5 codes 95-117
// registers, and the occupancy lost cost more than a cap costs.  80 (6
// blocks of 128 threads per SM), 88 for degree-5 3D: with the packed Gauss
// sums several codes spill 12-88 bytes there, yet sampling of the uneven 1M
// batch took 139.9 ms, against 143.7 ms with a spill-free 96 (5 blocks).
__host__ __device__ constexpr int sample_ff_regs(int code) { return code == bs_code(5, 3) ? 88 : 80; }
static_assert(88 * SAMPLE_THREADS_MAX <= 65536, "a block of SAMPLE_THREADS_MAX must fit one SM");
template <int CODE>
__global__ void __maxnreg__(sample_ff_regs(CODE)) k_sample_ff(SampleParams P, const float2* __restrict__ coef_ff)
{
    const Batch& b = P.b;
    const Table& t = P.t;
    unsigned long long newton = 0;
    int64_t i0, i1;
    sample_range(P, i0, i1);
    // each warp takes runs of SAMPLE_RUN consecutive samples, 32 at a time:
    // a lane's samples then mostly share their curve (see CurveHint)
    CurveHint hint;
    const int lane = threadIdx.x & 31;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t run = i0 + wid * SAMPLE_RUN; run < i1; run += n_warps * SAMPLE_RUN)
    for (int64_t ii = run + lane; ii < run + SAMPLE_RUN && ii < i1; ii += 32) {
        int64_t i;
        const int c = sample_curve_hint(P, ii, i, hint);
        const int code = CODE >= 0 ? CODE : curve_code(b, c);
        const int64_t s0 = b.seg_off[c], s1 = b.seg_off[c + 1];
        int64_t s;
        double v;
        if (s1 == s0) {
            s = -1;
            v = -1.0;
        } else {
            const double L = t.curve_len[c];
            const double pos = P.pos[i];
            const double target = P.is_relative ? pos * L : pos;
            // target <= 0 / target >= L on the bit patterns (L >= 0; a negative
            // target has a negative pattern): integer compares, off the FP64 pipe
            const long long tb = __double_as_longlong(target), lb = __double_as_longlong(L);
            if (tb <= 0) {
                s = s0;
                v = -1.0;
            } else if (tb >= lb) {
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
                double base = 0.0, va = -1.0;
                float fa, qa;
                if (j) {
                    base = t.leaf_cum[lo + j - 1];
                    va = t.leaf_v[lo + j - 1];
                    fa = t.leaf_f[lo + j - 1];
                    qa = t.leaf_q[lo + j - 1];
                } else {  // the interval's start: its FP64 end values, converted once
                    fa = (float)t.seg_f0[s];
                    qa = (float)t.seg_q0[s];
                }
                const double vb = t.leaf_v[lo + j];
                const double cb = t.leaf_cum[lo + j];
                const float fb = (float)t.leaf_f[lo + j];
                const float qb = (float)t.leaf_q[lo + j];
                const ff rl = ff_from_double(rr - base);   // target inside the leaf
                const ff dS = ff_from_double(cb - base);   // leaf length
                const double dvd = vb - va;                 // leaf width (exact dyadic)
                const float dv = (float)dvd;
                const ff vaf = ff_from_double(va);
                // quintic Hermite guess of v(S) on the leaf (FP32)
                float sig = dS.hi > 0.0f ? rl.hi / dS.hi : 0.0f;
                sig = fminf(fmaxf(sig, 0.0f), 1.0f);
                float dvg = sig * dv;
                const float fm = dS.hi / dv;
                if (fa > 0.1f * fm && fb > 0.1f * fm) {
                    const float s2 = sig * sig, s3 = s2 * sig, s4 = s3 * sig, s5 = s4 * sig;
                    const float h5 = 10.0f * s3 - 15.0f * s4 + 6.0f * s5;
                    const float h1 = sig - 6.0f * s3 + 8.0f * s4 - 3.0f * s5;
                    const float h4 = -4.0f * s3 + 7.0f * s4 - 3.0f * s5;
                    const float h2 = 0.5f * (s2 - 3.0f * s3 + 3.0f * s4 - s5);
                    const float h3 = 0.5f * (s3 - 2.0f * s4 + s5);
                    const float ia = 1.0f / fa, ib = 1.0f / fb;
                    const float ka = -qa * (ia * ia) * (ia * ia), kb = -qb * (ib * ib) * (ib * ib);
                    dvg = h5 * dv + dS.hi * (h1 * ia + h4 * ib) + dS.hi * dS.hi * (h2 * ka + h3 * kb);
                    dvg = fminf(fmaxf(dvg, 0.0f), dv);
                }
                const float2* seg = coef_ff + b.coef_off[c] + (s - s0) * code_stride(code);
                const float eps_s = P.eps_frac * f32_of_f64_trunc(L);
                double wfinal;
                if constexpr (CODE >= 0) {
                    wfinal = ff_leaf_newton<(CODE >= 0 ? CODE : 0), !panel_rolled<(CODE >= 0 ? CODE : 0)>()>(
                        seg, vaf, dv, rl, dS, dvg, eps_s, newton);
                } else {
                    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: wfinal = ff_leaf_newton<C, false>(seg, vaf, dv, rl, dS, dvg, eps_s, newton); break;
                        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
                    default: wfinal = dvg; break;
                    }
                }
                // the offset clamped to [0, dv] on the bit patterns (both
                // non-negative there; a negative offset or NaN has its sign
                // bit set or the largest pattern): integer compares, off the
                // FP64 pipe, as fmin / fmax would clamp it
                const long long wb = __double_as_longlong(wfinal);
                if (wb < 0) wfinal = 0.0;
                else if (wb > __double_as_longlong(dvd)) wfinal = dvd;
                v = va + wfinal;
            }
        }
        if (P.what == 2) {
            double u;
            if (s < 0) {
                u = b.kind[c] == 0 ? 0.0 : b.knots[b.knot_off[c] + b.degree[c]];
            } else {
                const double t0 = t.seg_t0[s], t1 = t.seg_t1[s], hw = 0.5 * (t1 - t0);
                // v <= 0 on the bit pattern (-0 and negatives have the sign bit)
                u = __double_as_longlong(v) <= 0 ? fma(v + 1.0, hw, t0) : fma(v - 1.0, hw, t1);
            }
            P.out[i] = u;
        } else {
            double p3[3] = {0.0, 0.0, 0.0};
            if (s >= 0) {
                // points from the float-float coefficients, evaluated in FP64
                // (a B-spline stores a[0] and then b[k - 1] = k a[k])
                const float2* seg = coef_ff + b.coef_off[c] + (s - s0) * code_stride(code);
                double cd[MAX_COEF];
                const int n = code_stride(code), dim = code_dim(code);
                for (int k = 0; k < n; ++k) {
                    cd[k] = (double)seg[k].x + (double)seg[k].y;
                    if (code != 0 && k >= 2 * dim) cd[k] *= 1.0 / (double)(k / dim);
                }
                if constexpr (CODE >= 0)
                    Eval<(CODE >= 0 ? CODE : 0)>::point(cd, v, p3);
                else
                    point_dyn(code, cd, v, p3);
            }
            for (int k = 0; k < P.pdim; ++k) P.out[i * P.pdim + k] = p3[k];
        }
    }
    if (P.collect) {
        for (int o = 16; o > 0; o >>= 1) newton += __shfl_xor_sync(0xffffffffu, newton, o);
        if ((threadIdx.x & 31) == 0 && newton) atomicAdd(t.ctr + C_NEWTON, newton);
    }
}

}  // namespace gcv
