// Allocation-free total lengths of a B-spline batch (gcv_bspline_lengths_noalloc).
//
// Some callers cannot call cudaMalloc: services that reserve a fixed device
// memory budget at start-up and forbid allocation afterwards, and code that
// runs inside another library's allocator or memory-pool hooks, where a
// nested cudaMalloc would recurse or fail.  This entry point computes what
// gcv_create_arclength_table + gcv_get_all_curve_arclengths give for a batch
// in the reference B-spline layout, with every byte of working memory in one
// file-scope device array instead of allocations:
//
//   * kernel 0: one thread per curve checks knots_offset (it starts at 0 and
//     every curve has at least 2 degree + 1 knots) and records the first bad
//     curve; the kernels after it return at once when it found one, so
//     malformed offsets never steer a read outside the caller's arrays;
//   * kernel 1, a lengths-only variant of the interval-length kernel: one
//     thread per knot interval builds the interval's polynomial in registers
//     and runs the same adaptive G7-K15 depth-first refinement, writing the
//     interval's length to the scratch array (no leaf table);
//   * kernel 2: one thread per curve sums its intervals' lengths with
//     double-double compensation into the caller's output.
//
// The scratch array (g_noalloc_scratch) holds GCV_NOALLOC_MAX_INTERVALS
// interval lengths plus a 256-byte header, about 8 MiB; every GPU that loads
// the library keeps it until the process exits.  Its device address is looked
// up once per device, with that device current, on the first call made on
// that device, and kept for the life of the process; make that first call
// before any stream capture begins, and make no call on a device after
// cudaDeviceReset (the module, and with it the array, may move).  Every call
// waits for its stream before returning (it reads knots_offset[n_curve] and
// the header back to the host).  Every call shares the array and the last
// call's contents stay in it (the header is cleared at the start of each
// call; every interval slot a call reads it has written first), so calls
// whose GPU work overlaps (different streams, or different host threads on
// one device) race on it and must be serialised by the caller.
#include "gcurval_gb300.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gcv_kernels.cuh"
#include "gcv_length_impl.cuh"

extern "C" gcv_status gcv_internal_fail(gcv_status s, const char* msg);

namespace {

using namespace gcv;

constexpr int64_t NOALLOC_MAX_INTERVALS = GCV_NOALLOC_MAX_INTERVALS;
// header words (64-bit): [0] error bits, [1] capped panels, [2] n_curve minus
// the first curve whose offsets are bad (0: none); the rest is unused
constexpr int HEADER_DOUBLES = 32;
// beside the table's ERR_* bits: knots_offset[0] != 0, a curve with fewer
// than 2 degree + 1 knots (decreasing offsets included)
constexpr unsigned long long NA_ERR_START = 1ull << 8, NA_ERR_OFFSETS = 1ull << 9;
constexpr int64_t SCRATCH_DOUBLES = HEADER_DOUBLES + NOALLOC_MAX_INTERVALS;

static __device__ __align__(256) double g_noalloc_scratch[SCRATCH_DOUBLES];

constexpr int MAX_DEVICES = 64;
std::mutex g_addr_mutex;
double* g_addr[MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device (host code may
// not use the symbol itself as a pointer).
gcv_status scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gcv_internal_fail(GCV_ERR_NO_DEVICE, "no current CUDA device");
    }
    if (dev < 0 || dev >= MAX_DEVICES) return gcv_internal_fail(GCV_ERR_INVALID, "device index above 63");
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return gcv_internal_fail(GCV_ERR_CUDA, (std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                                                    cudaGetErrorString(e)).c_str());
        }
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return GCV_OK;
}

// Length of one knot interval from its derivative polynomial r: the same
// acceptance rule and depth-first order as k_length, without the leaf table.
template <int CODE>
__device__ double interval_length(const double* r, double rtol, int max_depth, unsigned long long* capped)
{
    const double eps50 = 50.0 * 2.220446049250313e-16;
    unsigned long long k = 0;
    int depth = 0;
    double cum = 0.0, tol_unit = 0.0;
    long long panels = 0;
    for (;;) {
        const double hw = pow2_neg(depth);
        const double vlo = fma(__ull2double_rn(k), 2.0 * hw, -1.0);
        double K, G, fend, qend;
        panel_k15<CODE>(r, vlo, hw, K, G, fend, qend);
        if (depth == 0) tol_unit = rtol * fabs(K);
        ++panels;
        const double err = fabs(K - G);
        const bool finite = isfinite(K) && isfinite(G);
        const bool at_cap = depth >= max_depth || panels >= PANEL_BUDGET;
        const bool ok = err <= fmax(tol_unit * hw, eps50 * fabs(K));
        if (ok || at_cap || !finite) {
            if (!ok && finite) ++*capped;
            cum += K;
            ++k;
            const int tz = __ffsll((long long)k) - 1;
            k >>= tz;
            depth -= tz;
            if (depth == 0) break;
        } else {
            k <<= 1;
            ++depth;
        }
    }
    return cum;
}

// first interval of curve c in the reference layout
__device__ __forceinline__ int64_t first_interval(const int* ko, int64_t c, int P)
{
    return (int64_t)ko[c] - (int64_t)(2 * P + 1) * c;
}

// error word of the header, read once per thread at kernel start (kernel 0
// finished before: same stream)
__device__ __forceinline__ bool offsets_bad(const double* scratch)
{
    return (*reinterpret_cast<const unsigned long long*>(scratch) & (NA_ERR_START | NA_ERR_OFFSETS)) != 0;
}

// kernel 0: knots_offset[0] == 0 and knots_offset[c + 1] - knots_offset[c] >=
// 2 P + 1 for every curve (then first_interval is non-decreasing from 0 to
// n_seg, and every interval's knots and control points lie inside the
// curve's own range)
__global__ void k_noalloc_check(int n_curve, int P, const int* __restrict__ ko, double* scratch)
{
    unsigned long long* hdr = reinterpret_cast<unsigned long long*>(scratch);
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_curve;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = ko[c], b = ko[c + 1];
        if (c == 0 && a != 0) atomicOr(hdr, NA_ERR_START);
        if (b - a < 2 * P + 1) {
            atomicOr(hdr, NA_ERR_OFFSETS);
            atomicMax(hdr + 2, (unsigned long long)(n_curve - c));  // the smallest bad c
        }
    }
}

template <int P, int D>
__global__ void __launch_bounds__(128) k_noalloc_intervals(int n_curve, const int* __restrict__ ko,
                                                           const double* __restrict__ knots,
                                                           const double* __restrict__ ctrl, double rtol,
                                                           int max_depth, int64_t n_seg, double* scratch)
{
    if (offsets_bad(scratch)) return;
    unsigned long long capped = 0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_seg;
         s += (int64_t)gridDim.x * blockDim.x) {
        // curve of interval s: the last c with first_interval(c) <= s
        int lo = 0, cnt = n_curve;
        while (cnt > 0) {
            const int h = cnt >> 1;
            if (first_interval(ko, lo + h, P) <= s) {
                lo += h + 1;
                cnt -= h + 1;
            } else {
                cnt = h;
            }
        }
        const int c = lo - 1;
        if (c < 0) continue;  // only with first_interval(0) > 0, which kernel 0 rules out
        const int span = int(s - first_interval(ko, c, P)) + P;
        const double* kv = knots + ko[c];
        const double* cp = ctrl + ((int64_t)ko[c] - (int64_t)(P + 1) * c) * D;
        const double ka = kv[span], kb = kv[span + 1];
        double len = 0.0;
        if (!(kb >= ka)) {
            atomicOr(reinterpret_cast<unsigned long long*>(scratch), (unsigned long long)ERR_BAD_KNOTS);
        } else if (kb > ka) {
            double cf[(P + 1) * D], der[P * D];
            bspline_setup<P, D>(kv, cp, span, cf);
            Eval<bs_code(P, D)>::load_speed(cf, der);
            len = interval_length<bs_code(P, D)>(der, rtol, max_depth, &capped);
        }
        scratch[HEADER_DOUBLES + s] = len;
    }
    if (capped) atomicAdd(reinterpret_cast<unsigned long long*>(scratch + 1), capped);
}

__global__ void k_noalloc_curves(int n_curve, int P, const int* __restrict__ ko, int64_t n_seg,
                                 const double* __restrict__ scratch, double* __restrict__ lengths)
{
    if (offsets_bad(scratch)) return;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_curve;
         c += (int64_t)gridDim.x * blockDim.x) {
        int64_t b = first_interval(ko, c, P), e = first_interval(ko, c + 1, P);
        // kernel 0 guarantees 0 <= b <= e <= n_seg; clamp all the same
        b = b < 0 ? 0 : (b > n_seg ? n_seg : b);
        e = e < b ? b : (e > n_seg ? n_seg : e);
        DD acc{0.0, 0.0};
        for (int64_t s = b; s < e; ++s) acc = dd_add(acc, DD{scratch[HEADER_DOUBLES + s], 0.0});
        lengths[c] = acc.hi + acc.lo;
    }
}

template <int P, int D>
cudaError_t launch(int n_curve, const int* ko, const double* knots, const double* ctrl, double rtol, int max_depth,
                   int64_t n_seg, double* scratch, cudaStream_t st)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n_seg + 127) / 128;
    const int grid = (int)(want < (int64_t)sms * 16 ? (want > 0 ? want : 1) : (int64_t)sms * 16);
    k_noalloc_intervals<P, D><<<grid, 128, 0, st>>>(n_curve, ko, knots, ctrl, rtol, max_depth, n_seg, scratch);
    return cudaGetLastError();
}

}  // namespace

extern "C" gcv_status gcv_bspline_lengths_noalloc(int n_curve, int degree, int dim, const int* knots_offset,
                                                  const double* knot_vector, const double* ctrl_pts, double rtol,
                                                  int max_depth, double* lengths, void* stream, int64_t* n_capped)
{
    if (n_capped) *n_capped = 0;
    if (n_curve < 0) return gcv_internal_fail(GCV_ERR_INVALID, "n_curve < 0");
    if (degree < 1 || degree > MAX_DEGREE) return gcv_internal_fail(GCV_ERR_INVALID, "degree must be in [1, 5]");
    if (dim != 2 && dim != 3) return gcv_internal_fail(GCV_ERR_INVALID, "dim must be 2 or 3");
    if (!(rtol > 0.0) || !(rtol < 1.0)) return gcv_internal_fail(GCV_ERR_INVALID, "rtol must be in (0, 1)");
    if (max_depth < 1 || max_depth > MAX_DEPTH_LIMIT)
        return gcv_internal_fail(GCV_ERR_INVALID, "max_depth must be in [1, 48]");
    if (n_curve == 0) return GCV_OK;
    if (!knots_offset || !knot_vector || !ctrl_pts || !lengths)
        return gcv_internal_fail(GCV_ERR_INVALID, "NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int kend = 0;
    cudaError_t e = cudaMemcpyAsync(&kend, knots_offset + n_curve, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gcv_internal_fail(GCV_ERR_CUDA, (std::string("reading knots_offset[n_curve]: ") + cudaGetErrorString(e)).c_str());
    }
    const int64_t n_seg = (int64_t)kend - (int64_t)(2 * degree + 1) * n_curve;
    if (n_seg < 0) return gcv_internal_fail(GCV_ERR_INVALID, "knots_offset[n_curve] < (2 degree + 1) n_curve");
    if (n_seg > NOALLOC_MAX_INTERVALS)
        return gcv_internal_fail(GCV_ERR_INVALID,
                                 (std::to_string(n_seg) + " knot intervals exceed the allocation-free limit of " +
                                  std::to_string(NOALLOC_MAX_INTERVALS) + " (GCV_NOALLOC_MAX_INTERVALS)").c_str());
    double* scratch = nullptr;
    gcv_status s = scratch_address(&scratch);
    if (s != GCV_OK) return s;
    // the header's error bits, capped count and bad-curve slot must start at
    // zero; the interval lengths are all rewritten below
    e = cudaMemsetAsync(scratch, 0, HEADER_DOUBLES * sizeof(double), st);
    const int curve_grid = (int)((n_curve + 127) / 128 < 4096 ? (n_curve + 127) / 128 : 4096);
    if (e == cudaSuccess) {
        k_noalloc_check<<<curve_grid, 128, 0, st>>>(n_curve, degree, knots_offset, scratch);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && n_seg > 0) {
        switch (degree * 4 + dim) {
#define GCV_NA_CASE(P, D)                                                                          \
    case P * 4 + D: e = launch<P, D>(n_curve, knots_offset, knot_vector, ctrl_pts, rtol, max_depth, n_seg, scratch, st); break;
            GCV_NA_CASE(1, 2) GCV_NA_CASE(2, 2) GCV_NA_CASE(3, 2) GCV_NA_CASE(4, 2) GCV_NA_CASE(5, 2)
            GCV_NA_CASE(1, 3) GCV_NA_CASE(2, 3) GCV_NA_CASE(3, 3) GCV_NA_CASE(4, 3) GCV_NA_CASE(5, 3)
#undef GCV_NA_CASE
        default: break;
        }
    }
    if (e == cudaSuccess) {
        k_noalloc_curves<<<curve_grid, 128, 0, st>>>(n_curve, degree, knots_offset, n_seg, scratch, lengths);
        e = cudaGetLastError();
    }
    unsigned long long hdr[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hdr, scratch, sizeof(hdr), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return gcv_internal_fail(GCV_ERR_CUDA, (std::string("allocation-free lengths: ") + cudaGetErrorString(e)).c_str());
    }
    // the allocating path's messages for the same offsets
    if (hdr[0] & NA_ERR_START) return gcv_internal_fail(GCV_ERR_INVALID, "offsets must start at 0");
    if (hdr[0] & NA_ERR_OFFSETS)
        return gcv_internal_fail(GCV_ERR_INVALID, ("curve " + std::to_string((int64_t)n_curve - (int64_t)hdr[2]) +
                                                   ": fewer than 2 * degree + 1 knots").c_str());
    if (hdr[0] & ERR_BAD_KNOTS) return gcv_internal_fail(GCV_ERR_INVALID, "knot vector decreases or holds NaN");
    if (n_capped) *n_capped = (int64_t)hdr[1];
    return GCV_OK;
}
