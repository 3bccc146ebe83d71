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

// Shard [0, n) into nthreads contiguous ranges and run fn(lo, hi) on each.
template <typename F>
void run_sharded(int n, int nthreads, F fn)
{
    if (nthreads <= 1 || n < 2)
    {
        fn(0, n);
        return;
    }
    if (nthreads > n) nthreads = n;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
    {
        int lo = int((long long)n * t / nthreads);
        int hi = int((long long)n * (t + 1) / nthreads);
        th.emplace_back([=]() { fn(lo, hi); });
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

double gcvref_max_error(void) { return double(gcurval::MAX_ERROR_DOUBLE); }
int gcvref_max_depth(void) { return gcurval::MaxRecursiveDepth<double>::value; }

} // extern "C"
