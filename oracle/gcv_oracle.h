/* Plain-C restatement of gcurval's CPU arc-length driver (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  The product path never links,
 * loads or calls it.
 *
 * Curve batch layout (shared with the CUDA library, see include/gcurval_gb300.h):
 *   kind[c]    0 = ellipse, 1 = B-spline
 *   degree[c]  B-spline degree (1..7); ignored for ellipses
 *   dim[c]     2 or 3 (ellipses are 2D)
 *   knots[knot_off[c] .. knot_off[c+1])   knot vector; ellipse: {0, 2*pi}
 *   ctrl[ctrl_off[c] .. ctrl_off[c+1])    B-spline: control points, dim
 *                                         doubles each; ellipse: a, b,
 *                                         rotation, centre x, centre y
 */
#ifndef GCV_ORACLE_H
#define GCV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gcvo_batch {
    int n_curve;
    const uint8_t* kind;
    const uint8_t* degree;
    const uint8_t* dim;
    const int64_t* knot_off;
    const double* knots;
    const int64_t* ctrl_off;
    const double* ctrl;
} gcvo_batch;

typedef struct gcvo_table gcvo_table;

/* Builds the adaptive (u, cumulative length, segment) table of every curve
 * exactly as ArclengthCalculateCpu::createArclengthTable does
 * (gcurval/detail/cpu/arclength_calculate.h:80-139).  max_error is the
 * reference's MAX_ERROR (1e-14 for double, gcurval/config.h:32), max_depth its
 * MaxRecursiveDepth (23 for double, gcurval/config.h:42).  The batch arrays
 * must outlive the table.  Returns NULL on bad input. */
gcvo_table* gcvo_build(const gcvo_batch* batch, double max_error, int max_depth, int nthreads);
void gcvo_free(gcvo_table* t);

/* getAllCurveArclengths (cpu/arclength_calculate.h:141-150,288-307). */
void gcvo_lengths(const gcvo_table* t, double* out);

/* arclengthReverse (cpu/arclength_calculate.h:152-238): n_per_curve[c]
 * samples for curve c, positions back to back (relative in [0,1] when
 * is_relative, else absolute arc lengths).  what = 0 writes parameters u,
 * what = 1 writes points (dim doubles each; a batch with mixed dims writes
 * 3 doubles per point, z = 0 for 2D curves). */
int gcvo_reverse(const gcvo_table* t, const int* n_per_curve, const double* pos, int is_relative,
                 int what, double* out, int nthreads);

/* Arc length from the start of curve cid to parameter u: the table entry
 * below u plus the reference's adaptive GL3 recursion on the remainder.  Used
 * to measure sample-position error |s(u) - target| / L. */
double gcvo_s_at(const gcvo_table* t, int cid, double u);
void gcvo_s_at_many(const gcvo_table* t, const int* n_per_curve, const double* u, double* out,
                    int nthreads);

/* |C'(u)| of curve cid at parameter u, and C(u) (dim doubles). */
double gcvo_speed(const gcvo_batch* b, int cid, double u);
void gcvo_point(const gcvo_batch* b, int cid, double u, double* out);
int gcvo_point_seg(const gcvo_batch* b, int cid, int segid, double u, double* out);

/* Work counters: total table entries, and total |C'| evaluations. */
int64_t gcvo_table_entries(const gcvo_table* t);
int64_t gcvo_evals(const gcvo_table* t);

/* Table of one curve (pointers into the table; valid until gcvo_free). */
int64_t gcvo_curve_table(const gcvo_table* t, int cid, const double** u, const double** al,
                         const int** segid);

#ifdef __cplusplus
}
#endif
#endif
