// Device views of a curve batch and of its arc-length table, and the
// counter slots the kernels share.
#pragma once

#include "gcv_device.cuh"

namespace gcv {

// ----------------------------------------------------------- device views
struct Batch {
    int64_t n_curve;
    int64_t n_seg;
    const uint8_t* kind;
    const uint8_t* degree;
    const uint8_t* dim;
    const int64_t* knot_off;
    const double* knots;
    const int64_t* ctrl_off;
    const double* ctrl;
    const int64_t* seg_off;   // [n_curve + 1] first segment of each curve
    const int64_t* coef_off;  // [n_curve + 1] first coefficient (double) of each curve
    const int* seg_curve;     // [n_seg] curve of each segment
};

// counters in one device array (reset before each phase that uses them)
enum Counter {
    C_WORK = 0,       // length work-queue head
    C_LEAF_TOP = 1,   // leaf-pool bump pointer
    C_DEEP = 2,       // number of segments on the deep list
    C_PANELS = 3,
    C_CAPPED = 4,
    C_NEWTON = 5,
    C_ERR = 6,        // error bits (ERR_*)
    C_NONFINITE = 7,
    C_SCAN_TILE = 8,  // scan tile ticket
    C_DEEP_LEAVES = 9,  // leaves of the deep list's intervals (count pass)
    C_WORK_CODE = 16,   // work-queue heads of the per-code main-pass launches
    C_COUNT = 32
};
enum ErrBits { ERR_POOL = 1, ERR_SCAN_TIMEOUT = 2, ERR_BAD_KNOTS = 4, ERR_DEEP_LIST = 8, ERR_BAD_COUNT = 16 };

struct Table {
    double* coef;      // per-segment evaluation data (code_stride doubles), FP64 path
    float2* coef_ff;   // the same as float-float pairs (mixed path; NULL otherwise)
    double* seg_t0;    // curve parameter at v = -1
    double* seg_t1;    // curve parameter at v = +1
    double* seg_f0;    // f(-1)
    double* seg_q0;    // (f f')(-1)
    double* seg_len;   // length of each segment
    double* seg_cum;   // cumulative length at the end of each segment (within its curve)
    double* curve_len;
    int64_t* leaf_off;
    int* leaf_cnt;
    double* leaf_v;    // right end (local v) of each leaf panel
    double* leaf_cum;  // cumulative length within the segment at that end
    float* leaf_f;     // f at that end (shapes the sampling guess only)
    float* leaf_q;     // f * df/dv at that end
    int64_t leaf_cap;
    int* deep_list;
    int64_t deep_cap;
    unsigned long long* ctr;
    int* scan_status;  // per scan tile: 0 none, 1 aggregate, 2 inclusive
    int* scan_flag;
    double* scan_hi;
    double* scan_lo;
};

// double-double value and its two-sum addition (compensated sums)
struct DD {
    double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b)
{
    const double s = a.hi + b.hi;
    const double bb = s - a.hi;
    double e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const double h = s + e;
    return DD{h, e - (h - s)};
}
__device__ __forceinline__ int curve_code(const Batch& b, int64_t c)
{
    return b.kind[c] == 0 ? CODE_ELLIPSE : bs_code(b.degree[c], b.dim[c]);
}

__device__ __forceinline__ void raise_err(const Table& t, unsigned bits)
{
    atomicOr(t.ctr + C_ERR, (unsigned long long)bits);
}

}  // namespace gcv
