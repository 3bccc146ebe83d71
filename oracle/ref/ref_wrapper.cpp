// C entry points around the reference's OWN CPU arc-length driver
// (gcurval::ArclengthCalculateCpu, gcurval/detail/cpu/arclength_calculate.h),
// compiled unmodified from the reference tree by oracle/Makefile.
//
// TEST INFRASTRUCTURE ONLY (the oracle).  Nothing in the product path links
// or loads this library; tests, golden-vector generation and bench.py's
// CPU-baseline leg do.
//
// The curve plugins below restate the reference samples' plugins so that
// they compile with g++ (the sample headers rely on MSVC extensions):
//   * ellipse:  samples/sample1_ellipse/ellipse.h:5-97
//   * B-spline: samples/sample2_bspline/structs.h:6-185 and
//               samples/sample2_bspline/arclength_calculate.h:8-24
// The B-spline basis and derivative are the reference's own functions from
// samples/sample2_bspline/BSpline.h (included from the reference tree).
// One deliberate difference: the reference sample calls
// b_spline_derv_o1/b_spline_func_value without the degree template argument
// (structs.h:343,354), so they always run the cubic recursion; here the
// degree is passed, which is identical for degree 3 and correct otherwise.

#include <gcurval/gcurval.h>
#include <samples/sample2_bspline/BSpline.h>
#include <samples/sample2_bspline/dataset_loader.h>

#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

namespace
{

// ------------------------------ ellipse -----------------------------------

template <typename Dt>
struct RefEllipses : gcurval::CurvesBase<Dt, gcurval::Vector2X<Dt>>
{
    using PointType = gcurval::Vector2X<Dt>;
    Dt* a = nullptr;
    Dt* b = nullptr;
};

template <typename Dt>
struct RefEllipsePack : gcurval::ParaPackBase<Dt>
{
    Dt a;
    Dt b;
    RefEllipsePack() = default;
    RefEllipsePack(Dt begin, Dt end, int cid, int sid, Dt a_, Dt b_)
        : gcurval::ParaPackBase<Dt>{begin, end, cid, sid}, a(a_), b(b_)
    {
    }
};

template <typename Dt>
struct RefEllipseParser
{
    RefEllipsePack<Dt> operator()(const RefEllipses<Dt>& c, int cid, int, bool = false) const
    {
        return RefEllipsePack<Dt>(Dt(0), Dt(2 * EIGEN_PI), cid, 0, c.a[cid], c.b[cid]);
    }
};

template <typename Dt>
struct RefEllipsePoint
{
    gcurval::Vector2X<Dt> operator()(Dt u, const RefEllipsePack<Dt>& p) const
    {
        return gcurval::Vector2X<Dt>(p.a * std::cos(u), p.b * std::sin(u));
    }
};

template <typename Dt>
struct RefEllipseDerivative
{
    gcurval::Vector2X<Dt> operator()(Dt u, const RefEllipsePack<Dt>& p) const
    {
        return gcurval::Vector2X<Dt>(-1.0 * p.a * std::sin(u), p.b * std::cos(u));
    }
};

template <typename Dt>
struct RefEllipseTraits : gcurval::CurveTraitsBase<RefEllipses<Dt>>
{
    using ParaPackParser = RefEllipseParser<Dt>;
    using ParaPack = RefEllipsePack<Dt>;
    using GetPoint = RefEllipsePoint<Dt>;
    using GetDerivative = RefEllipseDerivative<Dt>;
    using CalculateFunction =
        gcurval::CalculateFunctionGaussLegendreQuadratureImpl<Dt, ParaPack, GetDerivative>;
};

// ------------------------------ B-spline ----------------------------------

template <typename Dt, typename Pt, int P>
struct RefBSplines : gcurval::CurvesBase<Dt, Pt>
{
    using PointType = Pt;
    int* knots_offset = nullptr;
    Dt* knot_vector = nullptr;
    Pt* ctrl_ptrs = nullptr;
};

template <typename Dt, typename Pt>
struct RefBSplinePack : gcurval::ParaPackBase<Dt>
{
    int span;
    Dt* knot_vector;
    Pt* ctrl_ptrs;
    RefBSplinePack() = default;
    RefBSplinePack(Dt begin, Dt end, int cid, int sid, int span_, Dt* kv, Pt* cp)
        : gcurval::ParaPackBase<Dt>{begin, end, cid, sid}, span(span_), knot_vector(kv), ctrl_ptrs(cp)
    {
    }
};

template <typename Dt, typename Pt, int P>
struct RefBSplineParser
{
    RefBSplinePack<Dt, Pt> operator()(const RefBSplines<Dt, Pt, P>& c, int cid, int segid,
                                      bool need_interval = false) const
    {
        int ko = c.knots_offset[cid];
        int kseg = ko + segid + P;
        Dt b = need_interval ? c.knot_vector[kseg] : Dt(0);
        Dt e = need_interval ? c.knot_vector[kseg + 1] : Dt(0);
        return RefBSplinePack<Dt, Pt>(b, e, cid, segid, segid + P, c.knot_vector + ko,
                                      c.ctrl_ptrs + ko - (P + 1) * cid);
    }
};

template <typename Dt, typename Pt, int P>
struct RefBSplineLocator
{
    gcurval::CurveIntervalPos operator()(const RefBSplines<Dt, Pt, P>& c, int cid) const
    {
        return gcurval::CurveIntervalPos{c.knots_offset[cid] - (2 * P + 1) * cid,
                                         c.knots_offset[cid + 1] - (2 * P + 1) * (cid + 1)};
    }
};

template <typename Dt>
struct RefScratch
{
    Dt* func;
    Dt* left;
    Dt* right;
};

template <typename Dt, int P>
struct RefScratchAllocator
{
    // host: one thread, the view starts at offset 0 (structs.h:55-60)
    const RefScratch<Dt> operator()(uint8_t* buffer) const
    {
        Dt* b = reinterpret_cast<Dt*>(buffer);
        return RefScratch<Dt>{b, b + (P + 1), b + 2 * (P + 1)};
    }
    static int size(int block = 1) { return block * (P + 1) * 3 * int(sizeof(Dt)); }
};

template <typename Dt, typename Pt, int P>
struct RefBSplinePoint
{
    Pt operator()(Dt u, const RefBSplinePack<Dt, Pt>& pk, const RefScratch<Dt>& s) const
    {
        b_spline_func_value<P, Dt>(u, pk.span, pk.knot_vector, s.func, s.left, s.right);
        return to_point<Dt, Pt, P>(pk.span, pk.ctrl_ptrs, s.func);
    }
};

template <typename Dt, typename Pt, int P>
struct RefBSplineDerivative
{
    Pt operator()(Dt u, const RefBSplinePack<Dt, Pt>& pk, const RefScratch<Dt>& s) const
    {
        b_spline_derv_o1<P, Dt>(u, pk.span, pk.knot_vector, s.func, s.left, s.right);
        return to_point<Dt, Pt, P>(pk.span, pk.ctrl_ptrs, s.func);
    }
};

template <typename Dt, typename Pt, int P>
struct RefBSplineTraits : gcurval::CurveTraitsBase<RefBSplines<Dt, Pt, P>>
{
    using ParaPack = RefBSplinePack<Dt, Pt>;
    using ParaPackParser = RefBSplineParser<Dt, Pt, P>;
    using SharedMemAllocator = RefScratchAllocator<Dt, P>;
    using CurveLocator = RefBSplineLocator<Dt, Pt, P>;
    using GetPoint = RefBSplinePoint<Dt, Pt, P>;
    using GetDerivative = RefBSplineDerivative<Dt, Pt, P>;
    using CalculateFunction =
        gcurval::CalculateFunctionGaussLegendreQuadratureImpl<Dt, ParaPack, GetDerivative>;
};

// ------------------------- calculators (fill curve) -----------------------

template <typename Dt>
class EllipseCalc : public gcurval::ArclengthCalculateCpu<RefEllipses<Dt>, RefEllipseTraits<Dt>>
{
    using Base = gcurval::ArclengthCalculateCpu<RefEllipses<Dt>, RefEllipseTraits<Dt>>;

public:
    EllipseCalc(int n, const Dt* a, const Dt* b) : Base(n, n)
    {
        this->curve.a = const_cast<Dt*>(a);
        this->curve.b = const_cast<Dt*>(b);
    }
    long long entries() const
    {
        long long s = 0;
        for (int i = 0; i < this->curve.n_curve; ++i) s += this->table_length[i];
        return s;
    }
};

template <typename Dt, int P, int D>
using PtOf = gcurval::VectorX<Dt, D>;

template <typename Dt, int P, int D>
class BSplineCalc
    : public gcurval::ArclengthCalculateCpu<RefBSplines<Dt, PtOf<Dt, P, D>, P>,
                                            RefBSplineTraits<Dt, PtOf<Dt, P, D>, P>>
{
    using Pt = PtOf<Dt, P, D>;
    using Base = gcurval::ArclengthCalculateCpu<RefBSplines<Dt, Pt, P>, RefBSplineTraits<Dt, Pt, P>>;

public:
    // knots_offset: local (rebased to 0) offsets of this shard
    BSplineCalc(int n, int* knots_offset, const Dt* knots, const Dt* ctrl)
        : Base(n, knots_offset[n] - (2 * P + 1) * n)
    {
        this->curve.knots_offset = knots_offset;
        this->curve.knot_vector = const_cast<Dt*>(knots);
        // PointType is a plain array of D Dt values, so packed xyz data can be viewed directly
        static_assert(sizeof(Pt) == D * sizeof(Dt), "packed point layout");
        this->curve.ctrl_ptrs = reinterpret_cast<Pt*>(const_cast<Dt*>(ctrl));
    }
    long long entries() const
    {
        long long s = 0;
        for (int i = 0; i < this->curve.n_curve; ++i) s += this->table_length[i];
        return s;
    }
};

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Run fn(lo, hi) over [0, n) on nthreads threads, in chunks taken from a
// shared counter (dynamic scheduling: per-curve costs are heavy-tailed, so
// static ranges leave most threads idle behind the largest curves).  Each
// chunk builds its own calculator, as a harness sharding curves over
// std::threads with one calculator per shard does.
template <typename F>
void run_sharded(int n, int nthreads, F fn)
{
    if (nthreads <= 1 || n < 2)
    {
        fn(0, n);
        return;
    }
    if (nthreads > n) nthreads = n;
    const int chunk = std::max(1, n / (nthreads * 16));
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
    {
        th.emplace_back([&]() {
            for (;;)
            {
                const int lo = next.fetch_add(chunk);
                if (lo >= n) break;
                fn(lo, std::min(n, lo + chunk));
            }
        });
    }
    for (auto& x : th) x.join();
}

template <typename Calc, typename Make>
void reverse_shard(Make make, int lo, int hi, const int* n_per_curve, const long long* sample_off,
                   const double* pos, int is_relative, int what, int dim, double* out,
                   double* lengths)
{
    Calc* calc = make(lo, hi);
    calc->createArclengthTable();
    if (lengths)
    {
        double* l = calc->getAllCurveArclengths();
        std::memcpy(lengths + lo, l, sizeof(double) * (hi - lo));
        delete[] l;
    }
    if (n_per_curve)
    {
        auto res = calc->arclengthReverse(const_cast<int*>(n_per_curve + lo),
                                          const_cast<double*>(pos + sample_off[lo]), is_relative != 0,
                                          gcurval::gcurvalHost,
                                          what ? gcurval::gcurvalReverseReturnPoints
                                               : gcurval::gcurvalReverseReturnUs);
        long long nsamp = sample_off[hi] - sample_off[lo];
        if (what)
        {
            std::memcpy(out + sample_off[lo] * dim, reinterpret_cast<double*>(res.points),
                        sizeof(double) * nsamp * dim);
            delete[] res.points;
        }
        else
        {
            std::memcpy(out + sample_off[lo], res.us, sizeof(double) * nsamp);
            delete[] res.us;
        }
    }
    delete calc;
}

std::vector<long long> prefix(int n, const int* cnt)
{
    std::vector<long long> off(n + 1, 0);
    if (cnt)
        for (int i = 0; i < n; ++i) off[i + 1] = off[i] + cnt[i];
    return off;
}

template <int P, int D>
int bspline_run(int n, const int* knots_offset, const double* knots, const double* ctrl,
                const int* n_per_curve, const double* pos, int is_relative, int what, double* out,
                double* lengths, int nthreads)
{
    auto off = prefix(n, n_per_curve);
    run_sharded(n, nthreads, [&](int lo, int hi) {
        // rebase this shard's knot offsets to 0
        std::vector<int> ko(hi - lo + 1);
        for (int i = lo; i <= hi; ++i) ko[i - lo] = knots_offset[i] - knots_offset[lo];
        const double* kv = knots + knots_offset[lo];
        const double* cp = ctrl + (long long)(knots_offset[lo] - (P + 1) * lo) * D;
        auto make = [&](int l, int h) { return new BSplineCalc<double, P, D>(h - l, ko.data(), kv, cp); };
        reverse_shard<BSplineCalc<double, P, D>>(make, lo, hi, n_per_curve, off.data(), pos,
                                                  is_relative, what, D, out, lengths);
    });
    return 0;
}

// The reference's point-based length rules (gcurval/base/functors.inl.h:
// PolylineMethod :145-165, SimpsonMethod :167-206, VincentForseyRule
// :208-238) on [begin[i], end[i]] of one curve, through the curve plugins'
// GetPoint: rule 0 polyline, 1 Simpson, 2 Vincent-Forsey.
template <typename Rule, typename GetPoint, typename Pack>
void rule_values(int n, const double* begin, const double* end, const Pack& pk, double* out)
{
    for (int i = 0; i < n; ++i) out[i] = Rule()(begin[i], end[i], GetPoint(), pk);
}

template <typename Rule, typename GetPoint, typename Pack, typename Scratch>
void rule_values(int n, const double* begin, const double* end, const Pack& pk, Scratch& sc, double* out)
{
    for (int i = 0; i < n; ++i) out[i] = Rule()(begin[i], end[i], GetPoint(), pk, sc);
}

} // namespace

extern "C" {

// Lengths (and optionally samples) of n ellipses x = a cos t, y = b sin t,
// t in [0, 2 pi], through the reference CPU driver.  n_per_curve == NULL
// skips sampling.  what: 0 = parameters u, 1 = points (x, y).
int gcvref_ellipse_run(int n, const double* a, const double* b, const int* n_per_curve,
                       const double* pos, int is_relative, int what, double* out, double* lengths,
                       int nthreads)
{
    auto off = prefix(n, n_per_curve);
    run_sharded(n, nthreads, [&](int lo, int hi) {
        auto make = [&](int l, int h) { return new EllipseCalc<double>(h - l, a + l, b + l); };
        reverse_shard<EllipseCalc<double>>(make, lo, hi, n_per_curve, off.data(), pos, is_relative,
                                           what, 2, out, lengths);
    });
    return 0;
}

// Same for B-splines of one degree (1..5) and dimension (2, 3) in the
// reference's packed layout: knots_offset[n + 1], knot vectors back to back,
// control points back to back (D doubles each).
int gcvref_bspline_run(int n, int degree, int dim, const int* knots_offset, const double* knots,
                       const double* ctrl, const int* n_per_curve, const double* pos,
                       int is_relative, int what, double* out, double* lengths, int nthreads)
{
#define GCVREF_CASE(P, D)                                                                          \
    if (degree == P && dim == D)                                                                   \
        return bspline_run<P, D>(n, knots_offset, knots, ctrl, n_per_curve, pos, is_relative, what, \
                                 out, lengths, nthreads);
    GCVREF_CASE(1, 2) GCVREF_CASE(2, 2) GCVREF_CASE(3, 2) GCVREF_CASE(4, 2) GCVREF_CASE(5, 2)
    GCVREF_CASE(1, 3) GCVREF_CASE(2, 3) GCVREF_CASE(3, 3) GCVREF_CASE(4, 3) GCVREF_CASE(5, 3)
#undef GCVREF_CASE
    return -1;
}

// Number of adaptive table entries the reference CPU driver builds (a proxy
// for the work it does): ellipses.
long long gcvref_ellipse_table_entries(int n, const double* a, const double* b)
{
    EllipseCalc<double> c(n, a, b);
    c.createArclengthTable();
    return c.entries();
}

// The reference's dataset loader (load_dataset / read_a_curve,
// samples/sample2_bspline/dataset_loader.h:40-126) on one Bundle file: the
// first n_curve (<= 1000) curves as 2D points, centred and scaled as that
// loader does.  Copies knots_offset[n_curve + 1], the knots and the control
// points (x, y pairs) out; returns the number of knots, or -1 when they do
// not fit the caller's capacities (knots_cap doubles, ctrl_cap points).
// The loader itself holds 50 knots and 50 points per curve on average.
int gcvref_load_bundle(const char* path, int n_curve, int* knots_offset, double* knots, int knots_cap,
                       double* ctrl, int ctrl_cap)
{
    using Pt = gcurval::Vector2X<double>;
    if (n_curve < 1 || n_curve > 1000) return -1;
    const char* names[1] = {path};
    CurveSet<double, Pt>* cs = load_dataset<double, Pt>(n_curve, names, 1);
    const int nk = cs->knots_offset[n_curve];
    const int np = nk - (cs->degree + 1) * n_curve;
    int rc = nk;
    if (nk > knots_cap || np > ctrl_cap)
    {
        rc = -1;
    }
    else
    {
        std::memcpy(knots_offset, cs->knots_offset, sizeof(int) * (n_curve + 1));
        std::memcpy(knots, cs->knot_vector, sizeof(double) * nk);
        for (int i = 0; i < np; ++i)
        {
            ctrl[2 * i] = cs->ctrl_ptrs[i][0];
            ctrl[2 * i + 1] = cs->ctrl_ptrs[i][1];
        }
    }
    delete cs;
    return rc;
}

int gcvref_ellipse_rule(int rule, double a, double b, int n, const double* begin, const double* end, double* out)
{
    RefEllipsePack<double> pk(0.0, 2 * EIGEN_PI, 0, 0, a, b);
    using GP = RefEllipsePoint<double>;
    if (rule == 0) rule_values<gcurval::PolylineMethod<double>, GP>(n, begin, end, pk, out);
    else if (rule == 1) rule_values<gcurval::SimpsonMethod<double>, GP>(n, begin, end, pk, out);
    else if (rule == 2) rule_values<gcurval::VincentForseyRule<double>, GP>(n, begin, end, pk, out);
    else return -1;
    return 0;
}

// one cubic 2D B-spline (n_ctrl points, n_ctrl + 4 knots) on knot interval
// segid (span segid + 3), parameters inside that interval
int gcvref_bspline_rule(int rule, int n_ctrl, const double* knots, const double* ctrl, int segid, int n,
                        const double* begin, const double* end, double* out)
{
    using Pt = gcurval::Vector2X<double>;
    constexpr int P = 3;
    if (segid < 0 || segid >= n_ctrl - P) return -1;
    RefBSplinePack<double, Pt> pk(0.0, 0.0, 0, segid, segid + P, const_cast<double*>(knots),
                                  reinterpret_cast<Pt*>(const_cast<double*>(ctrl)));
    std::vector<uint8_t> buf(RefScratchAllocator<double, P>::size());
    const RefScratch<double> sc = RefScratchAllocator<double, P>()(buf.data());
    using GP = RefBSplinePoint<double, Pt, P>;
    if (rule == 0) rule_values<gcurval::PolylineMethod<double>, GP>(n, begin, end, pk, sc, out);
    else if (rule == 1) rule_values<gcurval::SimpsonMethod<double>, GP>(n, begin, end, pk, sc, out);
    else if (rule == 2) rule_values<gcurval::VincentForseyRule<double>, GP>(n, begin, end, pk, sc, out);
    else return -1;
    return 0;
}

double gcvref_max_error(void) { return double(gcurval::MAX_ERROR_DOUBLE); }
int gcvref_max_depth(void) { return gcurval::MaxRecursiveDepth<double>::value; }

} // extern "C"
