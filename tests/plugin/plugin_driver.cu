// Test driver of the header-only plugin path (include/gcurval_gb300/gcurval.cuh):
// two user-defined curve families written the way a reference user writes
// them (samples/sample1_ellipse/ellipse.h, samples/sample2_bspline/structs.h),
// one of them through the shared-memory auxiliary-space hook, each with the
// default length rule (Gauss-Kronrod on GetDerivative) and with the
// reference's point-based rules (CalculateFunction = Polyline, Simpson or
// Vincent-Forsey on GetPoint, no GetDerivative).
//
//   plugin_driver ellipse[_polyline|_simpson|_vf] <in.bin> <out.bin> [rtol]
//   plugin_driver bspline[_polyline|_simpson|_vf] <in.bin> <out.bin> [rtol]
//
// in.bin:  int32 n_curve, int32 what (0 parameters, 1 points), then
//          ellipse: a[n], b[n] (double);  bspline (cubic, 2D): knots_offset[n+1]
//          (int32), knots (double), control points (x, y doubles);
//          then int32 counts[n], double positions[sum]
// out.bin: double lengths[n], then double us[sum] or (x, y)[sum]
#include <gcurval_gb300/gcurval.cuh>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace g = gcurval_gb300;

struct Vec2 {
    double x, y;
    __host__ __device__ double norm() const { return sqrt(x * x + y * y); }
};
__host__ __device__ inline Vec2 operator+(Vec2 a, Vec2 b) { return Vec2{a.x + b.x, a.y + b.y}; }
__host__ __device__ inline Vec2 operator-(Vec2 a, Vec2 b) { return Vec2{a.x - b.x, a.y - b.y}; }
__host__ __device__ inline Vec2 operator*(double s, Vec2 a) { return Vec2{s * a.x, s * a.y}; }

// ------------------------------------------------------------- ellipses
struct CurvesEllipse : g::CurvesBase<double, Vec2> {
    double* a = nullptr;
    double* b = nullptr;
};
struct PackEllipse : g::ParaPackBase<double> {
    double a, b;
};
struct ParserEllipse {
    __host__ __device__ PackEllipse operator()(const CurvesEllipse& c, int cid, int sid, bool = false) const
    {
        PackEllipse p;
        p.begin = 0.0;
        p.end = 2.0 * 3.14159265358979323846;
        p.cid = cid;
        p.sid = sid;
        p.a = c.a[cid];
        p.b = c.b[cid];
        return p;
    }
};
struct PointEllipse {
    __host__ __device__ Vec2 operator()(double u, const PackEllipse& p) const { return Vec2{p.a * cos(u), p.b * sin(u)}; }
};
struct DerivEllipse {
    __host__ __device__ Vec2 operator()(double u, const PackEllipse& p) const { return Vec2{-p.a * sin(u), p.b * cos(u)}; }
};
struct TraitsEllipse : g::CurveTraitsBase<CurvesEllipse> {
    using ParaPack = PackEllipse;
    using ParaPackParser = ParserEllipse;
    using GetPoint = PointEllipse;
    using GetDerivative = DerivEllipse;
};
// a point-based rule on GetPoint alone
template <typename Rule>
struct TraitsEllipseRule : g::CurveTraitsBase<CurvesEllipse> {
    using ParaPack = PackEllipse;
    using ParaPackParser = ParserEllipse;
    using GetPoint = PointEllipse;
    using CalculateFunction = Rule;
};
template <typename Traits>
class CalcEllipse : public g::ArclengthCalculateGpu<CurvesEllipse, Traits> {
public:
    CalcEllipse(int n, const double* a, const double* b) : g::ArclengthCalculateGpu<CurvesEllipse, Traits>(n, n)
    {
        cudaMalloc(&this->d_curve.a, sizeof(double) * (n ? n : 1));
        cudaMalloc(&this->d_curve.b, sizeof(double) * (n ? n : 1));
        cudaMemcpy(this->d_curve.a, a, sizeof(double) * n, cudaMemcpyHostToDevice);
        cudaMemcpy(this->d_curve.b, b, sizeof(double) * n, cudaMemcpyHostToDevice);
    }
    ~CalcEllipse() override
    {
        cudaFree(this->d_curve.a);
        cudaFree(this->d_curve.b);
    }
};

// ------------------------------------------------- cubic planar B-splines
constexpr int P = 3;
struct CurvesBSpline : g::CurvesBase<double, Vec2> {
    int* knots_offset = nullptr;
    double* knot_vector = nullptr;
    Vec2* ctrl_ptrs = nullptr;
};
// per-thread scratch in dynamic shared memory: basis values and the two
// knot-difference rows of the de Boor-Cox recursion
struct Scratch {
    double* N;
    double* left;
    double* right;
};
struct ScratchAllocator {
    __host__ __device__ Scratch operator()(uint8_t* buffer) const
    {
#ifdef __CUDA_ARCH__
        double* base = (double*)buffer + 3 * (P + 1) * threadIdx.x;
#else
        double* base = (double*)buffer;
#endif
        return Scratch{base, base + (P + 1), base + 2 * (P + 1)};
    }
    static int size(int block) { return block * 3 * (P + 1) * (int)sizeof(double); }
};
struct PackBSpline : g::ParaPackBase<double> {
    int span;
    const double* kv;
    const Vec2* cp;
};
struct ParserBSpline {
    __host__ __device__ PackBSpline operator()(const CurvesBSpline& c, int cid, int sid, bool need_interval = false) const
    {
        const int ko = c.knots_offset[cid];
        PackBSpline p;
        p.cid = cid;
        p.sid = sid;
        p.span = sid + P;
        p.kv = c.knot_vector + ko;
        p.cp = c.ctrl_ptrs + (ko - (P + 1) * cid);
        p.begin = need_interval ? p.kv[p.span] : 0.0;
        p.end = need_interval ? p.kv[p.span + 1] : 0.0;
        return p;
    }
};
struct LocatorBSpline {
    __host__ __device__ g::CurveIntervalPos operator()(const CurvesBSpline& c, int cid) const
    {
        return g::CurveIntervalPos{c.knots_offset[cid] - (2 * P + 1) * cid, c.knots_offset[cid + 1] - (2 * P + 1) * (cid + 1)};
    }
};
// basis functions of degree q on span at u into s.N[0..q] (de Boor-Cox)
__host__ __device__ inline void basis(int q, double u, int span, const double* kv, Scratch& s)
{
    s.N[0] = 1.0;
    for (int j = 1; j <= q; ++j) {
        s.left[j] = u - kv[span + 1 - j];
        s.right[j] = kv[span + j] - u;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            const double t = s.N[r] / (s.right[r + 1] + s.left[j - r]);
            s.N[r] = saved + s.right[r + 1] * t;
            saved = s.left[j - r] * t;
        }
        s.N[j] = saved;
    }
}
struct PointBSpline {
    __host__ __device__ Vec2 operator()(double u, const PackBSpline& p, Scratch& s) const
    {
        basis(P, u, p.span, p.kv, s);
        Vec2 r{0.0, 0.0};
        for (int i = 0; i <= P; ++i) {
            r.x += s.N[i] * p.cp[p.span - P + i].x;
            r.y += s.N[i] * p.cp[p.span - P + i].y;
        }
        return r;
    }
};
struct DerivBSpline {
    // C'(u) = sum_i p (P_{i+1} - P_i) / (k_{i+p+1} - k_{i+1}) N_{i+1, p-1}(u)
    __host__ __device__ Vec2 operator()(double u, const PackBSpline& p, Scratch& s) const
    {
        basis(P - 1, u, p.span, p.kv, s);
        Vec2 r{0.0, 0.0};
        for (int i = 0; i < P; ++i) {
            const int k = p.span - P + 1 + i;  // control point index of N_{k, p-1}
            const double w = P / (p.kv[k + P] - p.kv[k]);
            r.x += s.N[i] * w * (p.cp[k].x - p.cp[k - 1].x);
            r.y += s.N[i] * w * (p.cp[k].y - p.cp[k - 1].y);
        }
        return r;
    }
};
struct TraitsBSpline : g::CurveTraitsBase<CurvesBSpline> {
    using ParaPack = PackBSpline;
    using ParaPackParser = ParserBSpline;
    using SharedMemAllocator = ScratchAllocator;
    using CurveLocator = LocatorBSpline;
    using GetPoint = PointBSpline;
    using GetDerivative = DerivBSpline;
};
template <typename Rule>
struct TraitsBSplineRule : g::CurveTraitsBase<CurvesBSpline> {
    using ParaPack = PackBSpline;
    using ParaPackParser = ParserBSpline;
    using SharedMemAllocator = ScratchAllocator;
    using CurveLocator = LocatorBSpline;
    using GetPoint = PointBSpline;
    using CalculateFunction = Rule;
};
template <typename Traits>
class CalcBSpline : public g::ArclengthCalculateGpu<CurvesBSpline, Traits> {
public:
    CalcBSpline(int n, const int* ko, const double* kv, const Vec2* cp)
        : g::ArclengthCalculateGpu<CurvesBSpline, Traits>(n, ko[n] - (2 * P + 1) * n)
    {
        const int nk = ko[n], np = ko[n] - (P + 1) * n;
        cudaMalloc(&this->d_curve.knots_offset, sizeof(int) * (n + 1));
        cudaMalloc(&this->d_curve.knot_vector, sizeof(double) * (nk ? nk : 1));
        cudaMalloc(&this->d_curve.ctrl_ptrs, sizeof(Vec2) * (np ? np : 1));
        cudaMemcpy(this->d_curve.knots_offset, ko, sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
        cudaMemcpy(this->d_curve.knot_vector, kv, sizeof(double) * nk, cudaMemcpyHostToDevice);
        cudaMemcpy(this->d_curve.ctrl_ptrs, cp, sizeof(Vec2) * np, cudaMemcpyHostToDevice);
    }
    ~CalcBSpline() override
    {
        cudaFree(this->d_curve.knots_offset);
        cudaFree(this->d_curve.knot_vector);
        cudaFree(this->d_curve.ctrl_ptrs);
    }
};

// ---------------------------------------------------------------- driver
template <typename T>
static std::vector<T> rd(FILE* f, size_t n)
{
    std::vector<T> v(n);
    if (n && fread(v.data(), sizeof(T), n, f) != n) {
        fprintf(stderr, "short input\n");
        exit(2);
    }
    return v;
}

template <typename Calc>
static void run(Calc& calc, int n, FILE* in, FILE* out, int what, double rtol)
{
    if (rtol > 0.0) calc.setTolerance(rtol);
    calc.createArclengthTable();
    double* L = calc.getAllCurveArclengths();
    fwrite(L, sizeof(double), n, out);
    delete[] L;
    std::vector<int> cnt = rd<int>(in, (size_t)n);
    long long total = 0;
    for (int c : cnt) total += c;
    std::vector<double> pos = rd<double>(in, (size_t)total);
    if (what == 0) {
        auto r = calc.arclengthReverse(cnt.data(), pos.data(), true, g::gcurvalHost, g::gcurvalReverseReturnUs);
        fwrite(r.us, sizeof(double), (size_t)total, out);
        delete[] r.us;
    } else {
        auto r = calc.arclengthReverse(cnt.data(), pos.data(), true, g::gcurvalDevice, g::gcurvalReverseReturnPoints);
        std::vector<Vec2> h((size_t)total);
        cudaMemcpy(h.data(), r.points, sizeof(Vec2) * total, cudaMemcpyDeviceToHost);
        cudaFree(r.points);
        fwrite(h.data(), sizeof(Vec2), (size_t)total, out);
    }
}

template <typename Traits>
static void run_ellipse(int n, FILE* in, FILE* out, int what, double rtol)
{
    std::vector<double> a = rd<double>(in, (size_t)n), b = rd<double>(in, (size_t)n);
    CalcEllipse<Traits> calc(n, a.data(), b.data());
    run(calc, n, in, out, what, rtol);
}

template <typename Traits>
static void run_bspline(int n, FILE* in, FILE* out, int what, double rtol)
{
    std::vector<int> ko = rd<int>(in, (size_t)n + 1);
    std::vector<double> kv = rd<double>(in, (size_t)ko[n]);
    std::vector<double> cp = rd<double>(in, (size_t)(ko[n] - (P + 1) * n) * 2);
    CalcBSpline<Traits> calc(n, ko.data(), kv.data(), (const Vec2*)cp.data());
    run(calc, n, in, out, what, rtol);
}

int main(int argc, char** argv)
{
    if (argc != 4 && argc != 5) {
        fprintf(stderr, "usage: plugin_driver ellipse|bspline[_polyline|_simpson|_vf] in.bin out.bin [rtol]\n");
        return 2;
    }
    FILE* in = fopen(argv[2], "rb");
    FILE* out = fopen(argv[3], "wb");
    if (!in || !out) return 2;
    const double rtol = argc == 5 ? atof(argv[4]) : 0.0;
    const int n = rd<int>(in, 1)[0];
    const int what = rd<int>(in, 1)[0];
    const std::string fam = argv[1];
    using EP = PackEllipse;
    using BP = PackBSpline;
    try {
        if (fam == "ellipse")
            run_ellipse<TraitsEllipse>(n, in, out, what, rtol);
        else if (fam == "ellipse_polyline")
            run_ellipse<TraitsEllipseRule<g::CalculateFunctionPolylineMethodImpl<double, EP, PointEllipse>>>(
                n, in, out, what, rtol);
        else if (fam == "ellipse_simpson")
            run_ellipse<TraitsEllipseRule<g::CalculateFunctionSimpsonMethodImpl<double, EP, PointEllipse>>>(
                n, in, out, what, rtol);
        else if (fam == "ellipse_vf")
            run_ellipse<TraitsEllipseRule<g::CalculateFunctionVincentForseyRuleImpl<double, EP, PointEllipse>>>(
                n, in, out, what, rtol);
        else if (fam == "bspline")
            run_bspline<TraitsBSpline>(n, in, out, what, rtol);
        else if (fam == "bspline_polyline")
            run_bspline<TraitsBSplineRule<g::CalculateFunctionPolylineMethodImpl<double, BP, PointBSpline>>>(
                n, in, out, what, rtol);
        else if (fam == "bspline_simpson")
            run_bspline<TraitsBSplineRule<g::CalculateFunctionSimpsonMethodImpl<double, BP, PointBSpline>>>(
                n, in, out, what, rtol);
        else if (fam == "bspline_vf")
            run_bspline<TraitsBSplineRule<g::CalculateFunctionVincentForseyRuleImpl<double, BP, PointBSpline>>>(
                n, in, out, what, rtol);
        else {
            fprintf(stderr, "unknown family %s\n", argv[1]);
            return 2;
        }
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    fclose(in);
    fclose(out);
    return 0;
}
