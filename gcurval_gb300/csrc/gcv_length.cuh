// Adaptive length of every knot interval (FP64): persistent workers, one
// lane per knot interval.
//
// Each lane owns one segment at a time and refines it depth-first over the
// dyadic panels of v in [-1, 1].  A panel is named by (k, depth): it spans
// [-1 + k 2^(1-depth), -1 + (k+1) 2^(1-depth)], so the depth-first walk needs
// no stack: splitting goes to (2k, depth+1); after accepting a panel the next
// one is (k+1) with its trailing zero bits shifted out (climbing out of
// finished right children), and the walk ends when it climbs back to depth 0.
// Each panel is one 15-node Kronrod rule with its embedded 7-node Gauss rule
// plus the speed at the panel's right end, evaluated serially by the lane:
// accepted when |K15 - G7| is within the panel's share (half width) of
// rtol * |K15 of the whole interval|, or at max_depth / the panel budget.
// Accepted panels ("leaves") leave in parameter order; up to LCAP of them
// are staged in shared memory and copied to the leaf pool at an offset
// reserved by one atomic per warp.  Intervals with more leaves go to a deep
// list and are redone by the MODE 1 (count) and MODE 2 (write) passes, which
// write straight to the pool.
//
// This replaces the reference's breadth-first bisection (one GL3 task per
// thread, one launch and one host round trip per level,
// gcurval/detail/cuda/kernel/bfs.inl.cuh:9-125 driven from
// gcurval/detail/cuda/arclength_calculate.h:259-323).
#pragma once

#include "gcv_table.cuh"
#include "gcv_ff.cuh"

namespace gcv {

constexpr int LK_THREADS = 64;
constexpr int LCAP = 16;
constexpr long long PANEL_BUDGET = 1ll << 22;
constexpr int MAX_DEPTH_LIMIT = 48;

struct LengthParams {
    Batch b;
    Table t;
    double rtol;
    int max_depth;
    int collect;
    const int* list;  // segments to process; NULL: segments 0 .. n_items - 1
    int64_t n_items;
    const unsigned long long* n_items_dev;  // when set: the item count, read on the device
                                            // (graph launches; n_items then sizes the grid)
    const float2* coef_ff;  // float-float copy of the coefficients (PREC 1)
    unsigned long long* work;  // work-queue head of this launch (starts at 0)
    const uint32_t* starts;    // learned quarter start depths per segment (NULL: plain walk)
    // by_item (main pass of one curve code): the coefficients of work item i
    // are at coef_base + i * code_stride(CODE) and its learned start depths
    // at starts[i] (the table is laid out in the order of the grouped
    // segment list), so a lane starts its interval's first panel without
    // first loading the segment's curve and offsets
    int by_item;
    int64_t coef_base;
};

// Launches k_length<MODE, CODE, PREC> over P (persistent grid sized from the
// occupancy, capped at blocks_per_sm_cap per SM, and sm_count); defined with the kernel in gcv_length_impl.cuh and
// instantiated per curve code in the gcv_len_*.cu units.
//   MODE 0: main pass; MODE 1: count pass of the deep list; MODE 2: write pass.
//   CODE: curve code, or -1 for runtime dispatch per segment.
//   PREC 0: FP64 panels; 1: float-float panels.
template <int MODE, int CODE, int PREC>
cudaError_t length_launch(const LengthParams& P, cudaStream_t stream, int sm_count, int blocks_per_sm_cap);

// The main pass (MODE 0) with float-float panels and one half-warp per knot
// interval instead of one lane (gcv_length_hw.cuh); same table.
template <int CODE>
cudaError_t length_launch_hw(const LengthParams& P, cudaStream_t stream, int sm_count, int blocks_per_sm_cap);

}  // namespace gcv
