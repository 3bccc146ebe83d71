/* gcurval_gb300 Bundle reader: the reference's B-spline dataset files
 * (samples/sample2_bspline/dataset_loader.h:40-126, read_a_curve and
 * load_dataset) parsed and normalised on the GPU, into the device arrays
 * gcv_create_batch(..., GCV_DEVICE, ...) takes.
 *
 * Format, per curve, whitespace separated: "degree n_ctrl n_knots", the n_ctrl
 * x coordinates, the n_ctrl y coordinates, the n_knots knots
 * (dataset_loader.h:47-68).  The reference reads the numbers with
 * std::ifstream >> (correctly rounded decimal conversion); here every token
 * is converted by one thread with Clinger's exact fast path (an integer
 * significand below 2^53 times or over an exact power of ten up to 10^22,
 * one IEEE rounding), which gives the same double as a correctly rounded
 * conversion.  A number outside that path (more than 19 significant digits,
 * a significand above 2^53 or a decimal exponent beyond +-22) is rejected
 * with GCV_ERR_INVALID rather than converted inexactly.
 *
 * Normalisation (dataset_loader.h:77-103): each curve's control points are
 * centred on their mean (a sequential sum in point order divided by n_ctrl)
 * and divided by the largest |x| or |y| after centring.  A curve whose
 * centred coordinates are all zero is left centred (the reference would
 * divide by zero).  dim 3 appends z = 0 after normalising, as the
 * reference's 3D point type does.
 *
 * The reference loader takes the first 1,000 curves of each file
 * (dataset_loader.h:111-121); here every complete record of every file is
 * kept, files in order, up to max_curves curves in all.
 */
#ifndef GCURVAL_GB300_BUNDLE_H
#define GCURVAL_GB300_BUNDLE_H

#include "gcurval_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gcv_bundle gcv_bundle;

/* Tokenise and convert the n_files files laid end to end in `text`
 * (n_bytes bytes; host memory when where == GCV_HOST, else device memory),
 * file f spanning bytes [file_off[f], file_off[f + 1]) (a host array of
 * n_files + 1 offsets, file_off[0] = 0, file_off[n_files] = n_bytes), then
 * find every file's curve records.  Consecutive files must be separated by at
 * least one whitespace byte at the boundary.  Keeps the first max_curves
 * curves (max_curves < 0: all).  dim: 2 or 3.  Runs on `stream` (a
 * cudaStream_t, NULL: the legacy default stream) and returns when the record
 * count is known.  Malformed records (n_ctrl < degree + 1, n_knots !=
 * n_ctrl + degree + 1, a record cut short, trailing numbers, a token that is
 * not a number) fail with GCV_ERR_INVALID and a message naming the file and
 * the number's index.  On success *out owns the converted numbers until
 * gcv_bundle_destroy. */
gcv_status gcv_bundle_parse(const char* text, int64_t n_bytes, const int64_t* file_off, int n_files,
                            int64_t max_curves, int dim, int where, void* stream, gcv_bundle** out);

/* Sizes of the arrays gcv_bundle_fill writes: n_curve curves, n_knots
 * knots, n_ctrl_values control-point coordinates (sum of n_ctrl * dim). */
gcv_status gcv_bundle_sizes(const gcv_bundle* b, int64_t* n_curve, int64_t* n_knots, int64_t* n_ctrl_values);

/* Writes the batch into the caller's device arrays, in the layout of
 * gcv_create_batch: kind (n_curve, GCV_KIND_BSPLINE), degree, dim (n_curve
 * bytes each), knot_off and ctrl_off (n_curve + 1 int64 each), knots
 * (n_knots doubles), ctrl (n_ctrl_values doubles, x y [z] per point).
 * normalize != 0 applies the reference loader's centring and scaling.
 * Asynchronous on the stream given to gcv_bundle_parse. */
gcv_status gcv_bundle_fill(const gcv_bundle* b, int normalize, uint8_t* d_kind, uint8_t* d_degree, uint8_t* d_dim,
                           int64_t* d_knot_off, double* d_knots, int64_t* d_ctrl_off, double* d_ctrl);

/* Waits for the bundle's work on its stream and frees its device memory. */
void gcv_bundle_destroy(gcv_bundle* b);

#ifdef __cplusplus
}
#endif

#endif /* GCURVAL_GB300_BUNDLE_H */
