// Header-only plugin path of gcurval_gb300: arc-length tables and arc-length
// sampling of user-defined curve families, through the reference's
// header-level API (gcurval/arclength_calculate.h:10-18,
// gcurval/detail/cuda/arclength_calculate.h:141-237).
//
// A user describes a curve family the way the reference asks for it:
//   Curve          device-side batch (CurvesBase<Dt, PointType> + device pointers),
//   CurveTraits    DataType, PointType, ParaPack, ParaPackParser, CurveLocator,
//                  GetPoint, GetDerivative, SharedMemAllocator
//                  (gcurval/base/traits.inl.h:11-29),
// then subclasses ArclengthCalculateGpu<Curve, CurveTraits> and fills the
// protected d_curve with device pointers (samples/sample1_ellipse/ellipse.h:107-136).
// The same calls as the reference follow: createArclengthTable,
// getAllCurveArclengths (new[] host array), getArclength, arclengthReverse,
// clearArclength.
//
// The kernels are instantiated on the user's functors, so this path is
// header-only (compile with nvcc for sm_103a); the built-in ellipse and
// B-spline families run through the compiled library (gcurval_gb300.h) with
// their specialised float-float and FP64 kernels.  Here every knot interval
// is integrated by the adaptive 7/15-point Gauss-Kronrod walk (depth-first,
// stackless, one thread per interval) on |GetDerivative|, lengths are summed
// per curve in double-double arithmetic by one warp per curve, and samples are
// placed by safeguarded Newton steps on the leaf panels (8-point Gauss partial
// integrals), as in the compiled library.  When CurveTraits::CalculateFunction
// names one of the reference's point-based rules (Polyline, Simpson,
// Vincent-Forsey), the same walk refines with that rule on GetPoint instead,
// and samples invert the rule on their leaf by bisection; GetDerivative is
// then not needed.
//
// Differences from the reference, by design: the tolerance is relative
// (rtol * interval length, default 1e-10 for double, 1e-5 for float) instead of
// the fixed absolute per-level epsilon (gcurval/base/constants.inl.h:8-70);
// n_subdivided sets the depth limit (max_recursive_depth + log2 n_subdivided
// levels below the interval, the reference's finest resolution); the Gauss-
// Kronrod walk starts at the whole interval, the point-based rules at
// n_subdivided equal pieces as the reference's table does; CUDA errors
// throw std::runtime_error instead of printing and exiting
// (gcurval/detail/cuda/util.h:14-34).  Internal sums run in double for either
// DataType.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#ifndef GCURVAL_HD_FUNC
#define GCURVAL_HD_FUNC __host__ __device__
#endif

namespace gcurval_gb300 {

// ------------------------------------------------------------ base types
// gcurval/base/util.h:71-77
enum GcurvalEnum { gcurvalDevice, gcurvalHost, gcurvalReverseReturnUs, gcurvalReverseReturnPoints };

// gcurval/config.h:36-43
template <typename Dt>
struct MaxRecursiveDepth;
template <>
struct MaxRecursiveDepth<float> {
    static constexpr int value = 14;
};
template <>
struct MaxRecursiveDepth<double> {
    static constexpr int value = 23;
};

// gcurval/base/structs.inl.h:26-88
template <typename Dt, typename Pt>
struct CurvesBase {
    using DataType = Dt;
    using PointType = Pt;
    int n_curve = 0;
    GCURVAL_HD_FUNC CurvesBase(int n_curve = 0) : n_curve(n_curve) {}
};

template <typename Dt>
struct ParaPackBase {
    Dt begin;
    Dt end;
    int cid;
    int sid;
};

struct CurveIntervalPos {
    int begin;
    int end;
};

struct NoSharedMemAllocator {
    static constexpr int size(int) { return 0; }
};

template <typename DataType, typename PointType>
struct ArclengthReverseResult {
    int n_points = 0;
    GcurvalEnum store_where;
    GcurvalEnum store_what;
    union {
        DataType* us = nullptr;
        PointType* points;
    };
};

// gcurval/base/functors.inl.h:9-19: the default parser (one interval per curve)
template <typename Dt, typename PointType, typename Rt = ParaPackBase<Dt>>
struct ParaPackParserBase {
    using result_type = Rt;
    GCURVAL_HD_FUNC Rt operator()(const CurvesBase<Dt, PointType>&, int cid, int sid, bool = false) const
    {
        return Rt{Dt(0), Dt(0), cid, sid};
    }
};

// gcurval/base/functors.inl.h:262-269: curve cid owns interval cid
template <typename Curve>
struct CurveLocatorBase {
    GCURVAL_HD_FUNC constexpr CurveIntervalPos operator()(const Curve&, int cid) const
    {
        return CurveIntervalPos{cid, cid + 1};
    }
};

// gcurval/base/traits.inl.h:11-29 (the forward / backward space types of the
// reference's breadth-first pass have no counterpart here)
template <typename Curve>
struct CurveTraitsBase {
    using DataType = typename Curve::DataType;
    using PointType = typename Curve::PointType;
    using ParaPackParser = ParaPackParserBase<DataType, PointType>;
    using ParaPack = ParaPackBase<DataType>;
    using SharedMemAllocator = NoSharedMemAllocator;
    using CurveLocator = CurveLocatorBase<Curve>;
    using GetPoint = void;
    using GetDerivative = void;
    using CalculateFunction = void;
};

// ------------------------------------------------------- length rules
// The reference's point-based rules (gcurval/base/functors.inl.h:145-238):
// the length of [begin, end] from the curve points a = C(begin),
// m = C((begin + end) / 2) and b = C(end).  PointType must support
// a + b, a - b, scalar * a and .norm(), as Eigen vectors do.
enum LengthRule { RULE_GAUSS = 0, RULE_POLYLINE = 1, RULE_SIMPSON = 2, RULE_VINCENT_FORSEY = 3 };

template <int RULE, typename Pt>
GCURVAL_HD_FUNC double rule_from_points(const Pt& a, const Pt& m, const Pt& b)
{
    if constexpr (RULE == RULE_POLYLINE) {
        (void)m;
        return (double)(b - a).norm();  // the chord
    } else if constexpr (RULE == RULE_SIMPSON) {
        // Simpson's rule on |C'| with C' at begin, middle and end taken from
        // the quadratic through the three points
        return (1.0 / 6.0) * ((double)(-3.0 * a + 4.0 * m - b).norm() + 4.0 * (double)(b - a).norm() +
                              (double)(a - 4.0 * m + 3.0 * b).norm());
    } else {
        // Vincent-Forsey: (4 (|a m| + |m b|) - |a b|) / 3
        return 4.0 / 3.0 * ((double)(a - m).norm() + (double)(b - m).norm()) - 1.0 / 3.0 * (double)(b - a).norm();
    }
}

namespace plugin_detail {
template <int RULE, typename Dt>
struct PointRule {
    template <typename GetPoint, typename ParaPack>
    GCURVAL_HD_FUNC Dt operator()(Dt begin, Dt end, const GetPoint& gp, const ParaPack& pack) const
    {
        const Dt mid = (begin + end) / Dt(2.0);
        return (Dt)rule_from_points<RULE>(gp(begin, pack), gp(mid, pack), gp(end, pack));
    }
    template <typename GetPoint, typename ParaPack, typename SharedMem>
    GCURVAL_HD_FUNC Dt operator()(Dt begin, Dt end, const GetPoint& gp, const ParaPack& pack, SharedMem& buf) const
    {
        const Dt mid = (begin + end) / Dt(2.0);
        return (Dt)rule_from_points<RULE>(gp(begin, pack, buf), gp(mid, pack, buf), gp(end, pack, buf));
    }
};
}  // namespace plugin_detail

template <typename Dt>
struct PolylineMethod : plugin_detail::PointRule<RULE_POLYLINE, Dt> {};
template <typename Dt>
struct SimpsonMethod : plugin_detail::PointRule<RULE_SIMPSON, Dt> {};
template <typename Dt>
struct VincentForseyRule : plugin_detail::PointRule<RULE_VINCENT_FORSEY, Dt> {};

// CalculateFunction choices of CurveTraits (gcurval/base/functors.inl.h:
// 318-339), named as in the reference.  GetP is the GetPoint functor for the
// point-based rules.  GaussLegendreQuadrature (or no choice, void) integrates
// |GetDerivative| by the adaptive Gauss-Kronrod walk; a point-based rule
// refines each interval by halving where |L + R - P| (the two halves' rule
// values against the whole's) exceeds the tolerance, as the reference's
// arclengthRecursive does (gcurval/detail/cpu/arclength_calculate.h:242-279),
// and accepts L + R.
template <typename Dt, typename ParaPack, typename GetD>
struct CalculateFunctionGaussLegendreQuadratureImpl {};

#define GCURVAL_GB300_POINT_RULE(NAME, RULE)                                                           \
    template <typename Dt, typename ParaPack, typename GetP>                                           \
    struct CalculateFunction##NAME##Impl {                                                              \
        static constexpr int rule = RULE;                                                               \
        GCURVAL_HD_FUNC Dt operator()(Dt begin, Dt end, const ParaPack& pack) const                    \
        {                                                                                               \
            return NAME<Dt>{}(begin, end, GetP{}, pack);                                                \
        }                                                                                               \
        template <typename SharedMem>                                                                   \
        GCURVAL_HD_FUNC Dt operator()(Dt begin, Dt end, const ParaPack& pack, SharedMem& buffer) const \
        {                                                                                               \
            return NAME<Dt>{}(begin, end, GetP{}, pack, buffer);                                        \
        }                                                                                               \
    };
GCURVAL_GB300_POINT_RULE(PolylineMethod, RULE_POLYLINE)
GCURVAL_GB300_POINT_RULE(SimpsonMethod, RULE_SIMPSON)
GCURVAL_GB300_POINT_RULE(VincentForseyRule, RULE_VINCENT_FORSEY)
#undef GCURVAL_GB300_POINT_RULE

namespace plugin_detail {

// the rule a CurveTraits::CalculateFunction selects
template <typename CF, typename = void>
struct RuleOf {
    static constexpr int value = RULE_GAUSS;
};
template <typename CF>
struct RuleOf<CF, std::void_t<decltype(CF::rule)>> {
    static constexpr int value = CF::rule;
};

// 15-point Kronrod nodes / weights with the embedded 7-point Gauss weights
// (the published G7-K15 pair), nodes descending from the right end.
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
__host__ __device__ constexpr double gk_wg(int i)
{
    return i == 1 ? 0.129484966168869693270611432679082
         : i == 3 ? 0.279705391489276667901467771423780
         : i == 5 ? 0.381830050505118944950369775488975
         : i == 7 ? 0.417959183673469387755102040816327
                  : 0.0;
}
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

inline void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("gcurval_gb300: ") + what + ": " + cudaGetErrorString(e));
}

// |v| of GetDerivative's result: .norm() of a vector, or the scalar itself
// (gcurval/base/functors.inl.h:91-140)
template <typename Dt, typename Rt>
__device__ __forceinline__ double norm_of(const Rt& v)
{
    if constexpr (std::is_arithmetic<Rt>::value)
        return (double)v;
    else
        return (double)v.norm();
}

// GetDerivative / GetPoint with or without the traits' shared-memory view
// (gcurval/base/functors.inl.h:271-316)
template <typename Traits>
struct Calls {
    using Dt = typename Traits::DataType;
    using Alloc = typename Traits::SharedMemAllocator;
    static constexpr bool kSmem = !std::is_same<Alloc, NoSharedMemAllocator>::value;

    template <typename Pack>
    __device__ __forceinline__ static double speed(Dt u, const Pack& pk, uint8_t* smem)
    {
        if constexpr (kSmem) {
            auto buf = Alloc{}(smem);
            return norm_of<Dt>(typename Traits::GetDerivative{}(u, pk, buf));
        } else {
            (void)smem;
            return norm_of<Dt>(typename Traits::GetDerivative{}(u, pk));
        }
    }
    template <typename Pack>
    __device__ __forceinline__ static typename Traits::PointType point(Dt u, const Pack& pk, uint8_t* smem)
    {
        if constexpr (kSmem) {
            auto buf = Alloc{}(smem);
            return typename Traits::GetPoint{}(u, pk, buf);
        } else {
            (void)smem;
            return typename Traits::GetPoint{}(u, pk);
        }
    }
};

// One knot interval [t0, t1] in the local variable v in [-1, 1]:
// f(v) = |C'(t0 + (v + 1) hw)| hw.
template <typename Traits, typename Pack>
struct Interval {
    using Dt = typename Traits::DataType;
    const Pack& pk;
    double t0, t1, hw;
    uint8_t* smem;
    __device__ __forceinline__ double u_of(double v) const
    {
        return v <= 0.0 ? fma(v + 1.0, hw, t0) : fma(v - 1.0, hw, t1);
    }
    __device__ __forceinline__ double f(double v) const { return Calls<Traits>::speed((Dt)u_of(v), pk, smem) * hw; }
    __device__ __forceinline__ typename Traits::PointType p(double v) const
    {
        return Calls<Traits>::point((Dt)u_of(v), pk, smem);
    }
};

constexpr long long PANEL_BUDGET = 1ll << 22;

// Adaptive walk over the dyadic panels of one interval: panel (k, depth)
// spans [-1 + k 2^(1-depth), -1 + (k+1) 2^(1-depth)]; split -> (2k, depth+1);
// accept -> k + 1 with its trailing zero bits climbed out.  Accepted panels
// ("leaves") are counted, and written (right end v, cumulative length, f at
// the right end) when WRITE.  Returns the number of leaves; *len the length.
template <bool WRITE, typename Iv>
__device__ int walk(const Iv& iv, double rtol, int max_depth, double* len, double* lv, double* lc, float* lf)
{
    unsigned long long k = 0;
    int depth = 0, n = 0;
    long long panels = 0;
    double cum = 0.0, tol = 0.0;
    for (;;) {
        const double hwp = ldexp(1.0, -depth);
        const double vlo = fma((double)k, 2.0 * hwp, -1.0), mid = vlo + hwp;
        const double fc = iv.f(mid);
        double K = gk_wk(7) * fc, G = gk_wg(7) * fc;
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            const double dx = hwp * gk_x(i);
            const double s = iv.f(mid - dx) + iv.f(mid + dx);
            K = fma(gk_wk(i), s, K);
            if (i & 1) G = fma(gk_wg(i), s, G);
        }
        K *= hwp;
        G *= hwp;
        if (depth == 0) tol = rtol * fabs(K);
        ++panels;
        const bool ok = fabs(K - G) <= fmax(tol * hwp, 1.1102230246251565e-14 * fabs(K));
        if (ok || depth >= max_depth || panels >= PANEL_BUDGET || !isfinite(K)) {
            cum += K;
            if (WRITE) {
                const double vr = vlo + 2.0 * hwp;
                lv[n] = vr;
                lc[n] = cum;
                lf[n] = (float)iv.f(vr);
            }
            ++n;
            ++k;
            const int tz = __ffsll((long long)k) - 1;
            k >>= tz;
            depth -= tz;
            if (depth <= 0) break;
        } else {
            k <<= 1;
            ++depth;
        }
    }
    *len = cum;
    return n;
}

// Point-based rule of the sub-panel [v0, v1] of an interval, with its
// end points already evaluated.
template <int RULE, typename Iv, typename Pt>
__device__ __forceinline__ double rule_between(const Iv& iv, double v0, double v1, const Pt& p0, const Pt& p1)
{
    if constexpr (RULE == RULE_POLYLINE) {
        return rule_from_points<RULE>(p0, p0, p1);
    } else {
        return rule_from_points<RULE>(p0, iv.p(0.5 * (v0 + v1)), p1);
    }
}

// The adaptive walk of a point-based rule: panel (k, depth) as in walk();
// P = rule(panel), L and R = rule(halves); accepted when |L + R - P| is
// within the tolerance (rtol times the interval's first estimate, halved per
// level) or within the rounding noise of the chords, then contributes L + R.
// Panels above min_depth are always split: the walk starts from 2^min_depth
// equal pieces, as the reference's table starts from n_subdivided pieces per
// interval (gcurval/detail/cuda/kernel/generic.inl.cuh:10-48), because three
// or five points of a whole interval can agree by accident (an S-shaped
// interval whose quarter points line up).
template <bool WRITE, int RULE, typename Iv>
__device__ int walk_points(const Iv& iv, double rtol, int min_depth, int max_depth, double* len, double* lv, double* lc,
                           float* lf)
{
    unsigned long long k = 0;
    int depth = 0, n = 0;
    long long panels = 0;
    double cum = 0.0, tol = 0.0;
    for (;;) {
        const double hwp = ldexp(1.0, -depth);
        const double vlo = fma((double)k, 2.0 * hwp, -1.0), vm = vlo + hwp, vhi = vlo + 2.0 * hwp;
        const auto pa = iv.p(vlo);
        const auto pm = iv.p(vm);
        const auto pb = iv.p(vhi);
        const double P = rule_between<RULE>(iv, vlo, vhi, pa, pb);
        const double L = rule_between<RULE>(iv, vlo, vm, pa, pm);
        const double R = rule_between<RULE>(iv, vm, vhi, pm, pb);
        const double S = L + R;
        if (depth == 0) tol = rtol * fabs(S);
        ++panels;
        const double noise = 64.0 * 2.220446049250313e-16 * (fabs(S) + (double)pa.norm() + (double)pb.norm());
        const bool ok = depth >= min_depth && fabs(S - P) <= fmax(tol * hwp, noise);
        if (ok || depth >= max_depth || panels >= PANEL_BUDGET || !isfinite(S)) {
            cum += S;
            if (WRITE) {
                lv[n] = vhi;
                lc[n] = cum;
                lf[n] = 0.0f;
            }
            ++n;
            ++k;
            const int tz = __ffsll((long long)k) - 1;
            k >>= tz;
            depth -= tz;
            if (depth <= 0) break;
        } else {
            k <<= 1;
            ++depth;
        }
    }
    *len = cum;
    return n;
}

// Local variable of the point at arc length r (0 <= r <= rule(v0, v1))
// from v0 inside [v0, v1], by bisection of the rule's value over [v0, v],
// to the resolution of v.
template <int RULE, typename Iv>
__device__ double invert_rule(const Iv& iv, double v0, double v1, double r)
{
    const auto p0 = iv.p(v0);
    double lo = v0, hi = v1;
    for (int it = 0; it < 64; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (!(mid > lo && mid < hi)) break;
        if (rule_between<RULE>(iv, v0, mid, p0, iv.p(mid)) < r)
            lo = mid;
        else
            hi = mid;
    }
    return 0.5 * (lo + hi);
}

struct Params {
    double rtol;
    int max_depth;
    int min_depth;  // point-based rules: log2(n_subdivided)
};

// curve -> its interval range (CurveLocator), interval -> (curve, local id)
template <typename Curve, typename Traits>
__global__ void k_locate(Curve curve, int n_curve, int* seg_curve, int* seg_sid, int* curve_b, int* curve_e)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_curve; c += gridDim.x * blockDim.x) {
        const CurveIntervalPos r = typename Traits::CurveLocator{}(curve, c);
        curve_b[c] = r.begin;
        curve_e[c] = r.end;
        for (int s = r.begin; s < r.end; ++s) {
            seg_curve[s] = c;
            seg_sid[s] = s - r.begin;
        }
    }
}

// WRITE false: leaf counts and lengths; WRITE true: the leaves at leaf_off
template <bool WRITE, typename Curve, typename Traits>
__global__ void k_intervals(Curve curve, int n_seg, const int* seg_curve, const int* seg_sid, Params P,
                            int* leaf_cnt, double* seg_len, double* seg_t0, double* seg_t1,
                            const long long* leaf_off, double* lv, double* lc, float* lf)
{
    extern __shared__ __align__(16) uint8_t smem[];
    using Pack = typename Traits::ParaPack;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += gridDim.x * blockDim.x) {
        const Pack pk = typename Traits::ParaPackParser{}(curve, seg_curve[s], seg_sid[s], true);
        const double t0 = (double)pk.begin, t1 = (double)pk.end;
        double len = 0.0;
        if (t1 > t0) {
            const Interval<Traits, Pack> iv{pk, t0, t1, 0.5 * (t1 - t0), smem};
            const long long o = WRITE ? leaf_off[s] : 0;
            constexpr int rule = RuleOf<typename Traits::CalculateFunction>::value;
            int n;
            if constexpr (rule == RULE_GAUSS)
                n = walk<WRITE>(iv, P.rtol, P.max_depth, &len, lv + o, lc + o, lf + o);
            else
                n = walk_points<WRITE, rule>(iv, P.rtol, P.min_depth, P.max_depth, &len, lv + o, lc + o, lf + o);
            if (!WRITE) leaf_cnt[s] = n;
        } else if (WRITE) {  // empty interval: one leaf of length 0
            const long long o = leaf_off[s];
            lv[o] = 1.0;
            lc[o] = 0.0;
            lf[o] = 0.0f;
        } else {
            leaf_cnt[s] = 1;
        }
        if (!WRITE) {
            seg_len[s] = len;
            seg_t0[s] = t0;
            seg_t1[s] = t1 > t0 ? t1 : t0;
        }
    }
}

// exclusive prefix of n counts (two levels of 1024-item blocks and a serial
// top level over the block totals: sizes here are up to a few million blocks)
__global__ void k_block_sums(const int* cnt, long long n, long long* blk)
{
    __shared__ long long w[32];
    const long long base = (long long)blockIdx.x * 1024;
    long long x = 0;
    for (int i = threadIdx.x; i < 1024; i += blockDim.x)
        if (base + i < n) x += cnt[base + i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
        blk[blockIdx.x] = t;
    }
}
__global__ void k_scan_blocks(long long* blk, long long nb)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        long long run = 0;
        for (long long i = 0; i < nb; ++i) {
            const long long v = blk[i];
            blk[i] = run;
            run += v;
        }
        blk[nb] = run;
    }
}
__global__ void k_block_scan(const int* cnt, long long n, const long long* blk, long long* off)
{
    // 1024 items per block, 1024 threads: one item each
    __shared__ long long w[32];
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const long long x = i < n ? cnt[i] : 0;
    long long v = x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
    }
    if (lane == 31) w[wid] = v;
    __syncthreads();
    if (wid == 0) {
        long long t = w[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        w[lane] = t;
    }
    __syncthreads();
    const long long before = (wid ? w[wid - 1] : 0) + v - x;
    if (i < n) off[i] = blk[blockIdx.x] + before;
}

// double-double two-sum addition
struct DD {
    double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b)
{
    const double s = a.hi + b.hi, bb = s - a.hi;
    double e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const double h = s + e;
    return DD{h, e - (h - s)};
}

// one warp per curve: cumulative interval lengths within the curve
__global__ void k_curve_cum(int n_curve, const int* curve_b, const int* curve_e, const double* seg_len, double* seg_cum,
                            double* curve_len)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n_curve; c += warps) {
        const int b = curve_b[c], e = curve_e[c];
        DD carry{0.0, 0.0};
        for (int s0 = b; s0 < e; s0 += 32) {
            const int s = s0 + lane;
            DD v{s < e ? seg_len[s] : 0.0, 0.0};
            for (int d = 1; d < 32; d <<= 1) {
                DD y;
                y.hi = __shfl_up_sync(0xffffffffu, v.hi, d);
                y.lo = __shfl_up_sync(0xffffffffu, v.lo, d);
                if (lane >= d) v = dd_add(y, v);
            }
            const DD tot = dd_add(carry, v);
            if (s < e) seg_cum[s] = tot.hi + tot.lo;
            DD last;
            last.hi = __shfl_sync(0xffffffffu, tot.hi, 31);
            last.lo = __shfl_sync(0xffffffffu, tot.lo, 31);
            carry = last;
        }
        if (lane == 0) curve_len[c] = e > b ? carry.hi + carry.lo : 0.0;
    }
}

// first index in [lo, hi) with a[i] >= x
__device__ __forceinline__ long long lower_bound_d(const double* a, long long lo, long long hi, double x)
{
    long long n = hi - lo;
    while (n > 0) {
        const long long h = n >> 1;
        if (a[lo + h] < x) {
            lo += h + 1;
            n -= h + 1;
        } else {
            n = h;
        }
    }
    return lo;
}
__device__ __forceinline__ int upper_bound_ll(const long long* a, int n, long long x)
{
    int lo = 0, cnt = n;
    while (cnt > 0) {
        const int h = cnt >> 1;
        if (a[lo + h] <= x) {
            lo += h + 1;
            cnt -= h + 1;
        } else {
            cnt = h;
        }
    }
    return lo - 1;
}

struct SampleArgs {
    const long long* sample_off;  // [n_curve + 1]
    const double* pos;
    int n_curve;
    long long n_samples;
    int is_relative;
    double rtol;
    const int* curve_b;
    const double* seg_cum;
    const double* seg_len;
    const double* seg_t0;
    const double* seg_t1;
    const long long* leaf_off;
    const int* leaf_cnt;
    const double* lv;
    const double* lc;
    const float* lf;
    const double* curve_len;
    const int* curve_e;
};

// one thread per sample: interval by binary search of the cumulative table,
// leaf by binary search of the interval's leaves, then Newton on
// F(v) = S(v) - target with S from 8-point Gauss over the shorter side of the
// leaf, from a cubic Hermite guess of v(S), bracketed by bisection
template <bool POINTS, typename Curve, typename Traits>
__global__ void k_sample(Curve curve, SampleArgs A, typename Traits::DataType* us, typename Traits::PointType* pts)
{
    extern __shared__ __align__(16) uint8_t smem[];
    using Dt = typename Traits::DataType;
    using Pack = typename Traits::ParaPack;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < A.n_samples;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = upper_bound_ll(A.sample_off, A.n_curve + 1, i);
        const int b = A.curve_b[c], e = A.curve_e[c];
        double u = 0.0;
        int s = b;
        if (e > b) {
            const double L = A.curve_len[c];
            const double target = A.is_relative ? A.pos[i] * L : A.pos[i];
            double v;
            if (!(target > 0.0)) {
                s = b;
                v = -1.0;
            } else if (target >= L) {
                s = e - 1;
                v = 1.0;
            } else {
                s = (int)lower_bound_d(A.seg_cum, b, e, target);
                if (s >= e) s = e - 1;
                const double rr = target - (s > b ? A.seg_cum[s - 1] : 0.0);
                const long long lo = A.leaf_off[s];
                const int cnt = A.leaf_cnt[s];
                long long j = lower_bound_d(A.lc, lo, lo + cnt, rr) - lo;
                if (j >= cnt) j = cnt - 1;
                const double base = j ? A.lc[lo + j - 1] : 0.0, cb = A.lc[lo + j];
                const double va = j ? A.lv[lo + j - 1] : -1.0, vb = A.lv[lo + j];
                const Pack pk = typename Traits::ParaPackParser{}(curve, c, s - b, true);
                const double t0 = A.seg_t0[s], t1 = A.seg_t1[s];
                const Interval<Traits, Pack> iv{pk, t0, t1, 0.5 * (t1 - t0), smem};
                constexpr int rule = RuleOf<typename Traits::CalculateFunction>::value;
                if constexpr (rule != RULE_GAUSS) {
                    // the leaf's value is L + R of its halves: find the half,
                    // then invert the rule on it
                    const double vm = 0.5 * (va + vb), r = fmin(fmax(rr - base, 0.0), cb - base);
                    const double Lh = rule_between<rule>(iv, va, vm, iv.p(va), iv.p(vm));
                    v = r <= Lh ? invert_rule<rule>(iv, va, vm, r) : invert_rule<rule>(iv, vm, vb, r - Lh);
                } else {
                    const double fa = j ? (double)A.lf[lo + j - 1] : iv.f(-1.0), fb = (double)A.lf[lo + j];
                    const double dS = cb - base, dv = vb - va;
                    double sig = dS > 0.0 ? fmin(fmax((rr - base) / dS, 0.0), 1.0) : 0.0;
                    v = va + sig * dv;
                    if (fa > 0.1 * dS / dv && fb > 0.1 * dS / dv) {  // cubic Hermite of v(S): v' = 1/f
                        const double s2 = sig * sig, s3 = s2 * sig;
                        const double h00 = 2.0 * s3 - 3.0 * s2 + 1.0, h10 = s3 - 2.0 * s2 + sig;
                        const double h01 = -2.0 * s3 + 3.0 * s2, h11 = s3 - s2;
                        v = fmin(fmax(h00 * va + h01 * vb + dS * (h10 / fa + h11 / fb), va), vb);
                    }
                    const double eps = 0.01 * A.rtol * L;
                    double blo = va, bhi = vb;
                    for (int it = 0; it < 16; ++it) {
                        const bool left = (v - va) <= (vb - v);
                        const double a0 = left ? va : v, a1 = left ? v : vb;
                        const double h2 = 0.5 * (a1 - a0), m2 = a0 + h2;
                        double I = 0.0;
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const double xq = h2 * gl8_x(q);
                            I = fma(gl8_w(q), iv.f(m2 - xq) + iv.f(m2 + xq), I);
                        }
                        const double F = (left ? base + I * h2 : cb - I * h2) - rr;
                        if (fabs(F) <= eps) break;
                        if (F < 0.0)
                            blo = v;
                        else
                            bhi = v;
                        const double fv = iv.f(v);
                        double vn = fv > 0.0 ? v - F / fv : 0.5 * (blo + bhi);
                        if (!(vn > blo && vn < bhi)) vn = 0.5 * (blo + bhi);
                        v = vn;
                    }
                }
            }
            const double t0 = A.seg_t0[s], t1 = A.seg_t1[s], hw = 0.5 * (t1 - t0);
            u = v <= 0.0 ? fma(v + 1.0, hw, t0) : fma(v - 1.0, hw, t1);
        }
        if constexpr (POINTS) {
            const Pack pk = typename Traits::ParaPackParser{}(curve, c, e > b ? s - b : 0, true);
            pts[i] = Calls<Traits>::point((Dt)u, pk, smem);
        } else {
            us[i] = (Dt)u;
        }
    }
}

template <typename T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    void reserve(size_t count)
    {
        if (count <= n && p) return;
        release();
        check(cudaMalloc(&p, (count ? count : 1) * sizeof(T)), "cudaMalloc");
        n = count;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevArray() { release(); }
};

}  // namespace plugin_detail

// gcurval/detail/cuda/arclength_calculate.h:116-237
template <typename Curve, typename CurveTraits,
          int max_recursive_depth = MaxRecursiveDepth<typename CurveTraits::DataType>::value,
          int n_subdivided = 64>
class ArclengthCalculateCuda {
public:
    using Dt = typename CurveTraits::DataType;
    using PointType = typename CurveTraits::PointType;

    explicit ArclengthCalculateCuda(int n_curve, int n_seg) : n_seg(n_seg) { d_curve.n_curve = n_curve; }
    explicit ArclengthCalculateCuda(int n_curve) : n_seg(n_curve) { d_curve.n_curve = n_curve; }
    virtual ~ArclengthCalculateCuda() { delete[] h_arclength; }

    ArclengthCalculateCuda(const ArclengthCalculateCuda&) = delete;
    ArclengthCalculateCuda& operator=(const ArclengthCalculateCuda&) = delete;

    // relative tolerance of every interval's length (default 1e-10 for
    // double, 1e-5 for float); stream of every launch (default: legacy stream)
    void setTolerance(double rtol) { this->rtol = rtol; }
    void setStream(cudaStream_t s) { stream = s; }

    void createArclengthTable()
    {
        using namespace plugin_detail;
        const int n_curve = d_curve.n_curve;
        seg_curve.reserve(n_seg);
        seg_sid.reserve(n_seg);
        curve_b.reserve(n_curve);
        curve_e.reserve(n_curve);
        leaf_cnt.reserve(n_seg);
        seg_len.reserve(n_seg);
        seg_cum.reserve(n_seg);
        seg_t0.reserve(n_seg);
        seg_t1.reserve(n_seg);
        leaf_off.reserve((size_t)n_seg + 1);
        curve_len.reserve(n_curve);
        const int smem = Alloc::size(kThreads);
        if (n_curve > 0) {
            k_locate<Curve, CurveTraits><<<grid(n_curve), kThreads, 0, stream>>>(d_curve, n_curve, seg_curve.p, seg_sid.p,
                                                                               curve_b.p, curve_e.p);
            check(cudaGetLastError(), "k_locate");
        }
        Params P{rtol, max_recursive_depth + ilog2(n_subdivided), ilog2(n_subdivided)};
        if (n_seg > 0) {
            k_intervals<false, Curve, CurveTraits><<<grid(n_seg), kThreads, smem, stream>>>(
                d_curve, n_seg, seg_curve.p, seg_sid.p, P, leaf_cnt.p, seg_len.p, seg_t0.p, seg_t1.p, nullptr, nullptr,
                nullptr, nullptr);
            check(cudaGetLastError(), "k_intervals (count)");
            const long long nb = ((long long)n_seg + 1023) / 1024;
            blk.reserve((size_t)nb + 1);
            k_block_sums<<<(unsigned)nb, 1024, 0, stream>>>(leaf_cnt.p, n_seg, blk.p);
            k_scan_blocks<<<1, 32, 0, stream>>>(blk.p, nb);
            k_block_scan<<<(unsigned)nb, 1024, 0, stream>>>(leaf_cnt.p, n_seg, blk.p, leaf_off.p);
            check(cudaGetLastError(), "leaf offsets");
            long long total = 0;
            check(cudaMemcpyAsync(&total, blk.p + nb, sizeof(total), cudaMemcpyDeviceToHost, stream), "leaf total");
            check(cudaStreamSynchronize(stream), "leaf total");
            lv.reserve((size_t)total);
            lc.reserve((size_t)total);
            lf.reserve((size_t)total);
            k_intervals<true, Curve, CurveTraits><<<grid(n_seg), kThreads, smem, stream>>>(
                d_curve, n_seg, seg_curve.p, seg_sid.p, P, leaf_cnt.p, seg_len.p, seg_t0.p, seg_t1.p, leaf_off.p, lv.p,
                lc.p, lf.p);
            check(cudaGetLastError(), "k_intervals (write)");
        }
        if (n_curve > 0) {
            k_curve_cum<<<grid((long long)n_curve * 32), kThreads, 0, stream>>>(n_curve, curve_b.p, curve_e.p, seg_len.p,
                                                                               seg_cum.p, curve_len.p);
            check(cudaGetLastError(), "k_curve_cum");
        }
        check(cudaStreamSynchronize(stream), "createArclengthTable");
        table = true;
    }

    // a new[] host array of n_curve lengths, owned by the caller
    Dt* getAllCurveArclengths()
    {
        fetch_lengths();
        Dt* out = new Dt[d_curve.n_curve];
        for (int i = 0; i < d_curve.n_curve; ++i) out[i] = h_arclength[i];
        return out;
    }

    Dt getArclength(int cid)
    {
        fetch_lengths();
        if (cid < 0 || cid >= d_curve.n_curve) throw std::out_of_range("gcurval_gb300: curve id out of range");
        return h_arclength[cid];
    }

    // n_ptrs_for_curves (host, n_curve counts) and sample_position (host,
    // their sum) as in the reference; the result is allocated in `where`
    // memory (cudaMalloc / new[]) and owned by the caller
    ArclengthReverseResult<Dt, PointType> arclengthReverse(int* n_ptrs_for_curves, Dt* sample_position, bool is_relative,
                                                           GcurvalEnum where = gcurvalDevice,
                                                           GcurvalEnum what = gcurvalReverseReturnUs)
    {
        using namespace plugin_detail;
        if (!table) throw std::logic_error("gcurval_gb300: createArclengthTable has not run");
        const int n_curve = d_curve.n_curve;
        std::vector<long long> off((size_t)n_curve + 1, 0);
        for (int i = 0; i < n_curve; ++i) {
            if (n_ptrs_for_curves[i] < 0) throw std::invalid_argument("gcurval_gb300: negative sample count");
            off[(size_t)i + 1] = off[(size_t)i] + n_ptrs_for_curves[i];
        }
        const long long total = off[(size_t)n_curve];
        ArclengthReverseResult<Dt, PointType> res;
        res.n_points = (int)total;
        res.store_where = where;
        res.store_what = what;
        const size_t width = what == gcurvalReverseReturnPoints ? sizeof(PointType) : sizeof(Dt);
        DevArray<long long> d_off;
        DevArray<double> d_pos;
        DevArray<uint8_t> d_res;
        d_off.reserve(off.size());
        check(cudaMemcpyAsync(d_off.p, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, stream),
              "sample offsets");
        d_pos.reserve((size_t)total);
        if (total) {
            std::vector<double> pos_d((size_t)total);
            for (long long i = 0; i < total; ++i) pos_d[(size_t)i] = (double)sample_position[i];
            check(cudaMemcpyAsync(d_pos.p, pos_d.data(), (size_t)total * sizeof(double), cudaMemcpyHostToDevice, stream),
                  "sample positions");
            check(cudaStreamSynchronize(stream), "sample positions");
        }
        uint8_t* dst = nullptr;
        if (where == gcurvalDevice) {
            check(cudaMalloc(&dst, (size_t)(total ? total : 1) * width), "result");
        } else {
            d_res.reserve((size_t)(total ? total : 1) * width);
            dst = d_res.p;
        }
        SampleArgs A{d_off.p, d_pos.p, n_curve, total, is_relative ? 1 : 0, rtol, curve_b.p, seg_cum.p, seg_len.p,
                     seg_t0.p, seg_t1.p, leaf_off.p, leaf_cnt.p, lv.p, lc.p, lf.p, curve_len.p, curve_e.p};
        const int smem = Alloc::size(kThreads);
        if (total) {
            if (what == gcurvalReverseReturnPoints)
                k_sample<true, Curve, CurveTraits><<<grid(total), kThreads, smem, stream>>>(d_curve, A, nullptr,
                                                                                          (PointType*)dst);
            else
                k_sample<false, Curve, CurveTraits><<<grid(total), kThreads, smem, stream>>>(d_curve, A, (Dt*)dst,
                                                                                           nullptr);
            check(cudaGetLastError(), "k_sample");
        }
        if (where == gcurvalHost) {
            uint8_t* host = what == gcurvalReverseReturnPoints ? (uint8_t*)new PointType[total ? total : 1]
                                                               : (uint8_t*)new Dt[total ? total : 1];
            if (total) check(cudaMemcpyAsync(host, dst, (size_t)total * width, cudaMemcpyDeviceToHost, stream), "result");
            dst = host;
        }
        check(cudaStreamSynchronize(stream), "arclengthReverse");
        if (what == gcurvalReverseReturnPoints)
            res.points = (PointType*)dst;
        else
            res.us = (Dt*)dst;
        return res;
    }

    void clearArclength()
    {
        delete[] h_arclength;
        h_arclength = nullptr;
    }

protected:
    Curve d_curve;
    int n_seg;

private:
    using Alloc = typename CurveTraits::SharedMemAllocator;
    static constexpr int kThreads = 128;
    static constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x / 2); }
    static unsigned grid(long long work)
    {
        const long long g = (work + kThreads - 1) / kThreads;
        return (unsigned)(g < 1 ? 1 : (g > 152LL * 64 ? 152LL * 64 : g));
    }
    void fetch_lengths()
    {
        if (!table) throw std::logic_error("gcurval_gb300: createArclengthTable has not run");
        if (h_arclength) return;
        std::vector<double> tmp((size_t)d_curve.n_curve);
        if (!tmp.empty())
            plugin_detail::check(cudaMemcpy(tmp.data(), curve_len.p, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost),
                                 "lengths");
        h_arclength = new Dt[d_curve.n_curve];
        for (int i = 0; i < d_curve.n_curve; ++i) h_arclength[i] = (Dt)tmp[(size_t)i];
    }

    double rtol = std::is_same<Dt, float>::value ? 1e-5 : 1e-10;
    cudaStream_t stream = nullptr;
    bool table = false;
    Dt* h_arclength = nullptr;
    plugin_detail::DevArray<int> seg_curve, seg_sid, curve_b, curve_e, leaf_cnt;
    plugin_detail::DevArray<double> seg_len, seg_cum, seg_t0, seg_t1, curve_len, lv, lc;
    plugin_detail::DevArray<float> lf;
    plugin_detail::DevArray<long long> leaf_off, blk;
};

// gcurval/arclength_calculate.h:10-18
template <typename Curve, typename CurveTraits,
          int max_recursive_depth = MaxRecursiveDepth<typename CurveTraits::DataType>::value,
          int n_subdivided = 64>
using ArclengthCalculateGpu = ArclengthCalculateCuda<Curve, CurveTraits, max_recursive_depth, n_subdivided>;

}  // namespace gcurval_gb300
