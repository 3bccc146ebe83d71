/* gcurval_gb300 C ABI: adaptive arc length and arc-length sampling of
 * parametric curves on one GB300 GPU (sm_103a).
 *
 * This is the drop-in boundary for gcurval's arc-length path.  Every entry
 * point replaces one member of the reference's driver class
 * gcurval::ArclengthCalculateCuda (gcurval/detail/cuda/arclength_calculate.h)
 * or one of the sample plugins' constructors; the citation is given beside
 * each declaration.  Plain pointers and sizes only: no CUDA or torch types
 * (a stream is passed as void*).
 *
 * Curve kinds built into the library:
 *   - ellipses  x = a cos t, y = b sin t, t in [0, 2 pi] (one knot interval),
 *               optionally rotated by `rot` and moved to (cx, cy)
 *               (samples/sample1_ellipse/ellipse.h);
 *   - B-splines of degree 1..5 in 2D or 3D over their knot vector, one knot
 *               interval per segment (samples/sample2_bspline/).
 * User-defined curve functors go through the header-only C++ path
 * include/gcurval_gb300/gcurval.cuh (ArclengthCalculateGpu<Curve, CurveTraits>),
 * whose kernels run the same adaptive walk, scan and Newton sampling
 * instantiated on the user's plugin types.
 *
 * Errors: every entry point returns a gcv_status; gcv_last_error() gives a
 * message for the calling thread.  The reference instead calls exit(-1) in
 * debug builds and ignores errors under NDEBUG
 * (gcurval/detail/cuda/util.h:14-34).
 *
 * Threading: a context is used by one host thread at a time.  All GPU work of
 * a context runs on its stream (options.stream, default the legacy default
 * stream), like the reference's single stream.
 */
#ifndef GCURVAL_GB300_H
#define GCURVAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gcv_status {
    GCV_OK = 0,
    GCV_ERR_INVALID = 1,      /* bad argument or curve data */
    GCV_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    GCV_ERR_OUT_OF_MEMORY = 3,
    GCV_ERR_STATE = 4,        /* e.g. sampling before the table exists */
    GCV_ERR_OVERFLOW = 5,     /* a fixed-capacity device structure overflowed */
    GCV_ERR_TIMEOUT = 6,      /* a bounded device-side wait gave up */
    GCV_ERR_NO_DEVICE = 7     /* no usable GPU / the kernels cannot run */
} gcv_status;

/* Mirrors gcurval::GcurvalEnum (gcurval/base/util.h:71-77): where a result
 * lives and what it holds.  The numeric values match the reference enum. */
typedef enum gcv_enum {
    GCV_DEVICE = 0,        /* gcurvalDevice */
    GCV_HOST = 1,          /* gcurvalHost */
    GCV_RETURN_US = 2,     /* gcurvalReverseReturnUs */
    GCV_RETURN_POINTS = 3  /* gcurvalReverseReturnPoints */
} gcv_enum;

typedef enum gcv_precision {
    GCV_PLAIN_FP64 = 0,    /* every step in FP64 */
    GCV_MIXED = 1          /* FP32 integrand and panels; FP64 prefix sum,
                              error test near tolerance and final Newton step */
} gcv_precision;

typedef enum gcv_kind { GCV_KIND_ELLIPSE = 0, GCV_KIND_BSPLINE = 1 } gcv_kind;

/* Run-time replacements of the reference's compile-time configuration
 * (gcurval/config.h: GCURVAL_MAX_ERROR, GCURVAL_MAX_RECURSIVE_DEPTH). */
typedef struct gcv_options {
    double rtol;          /* relative tolerance on every knot interval's length
                             (default 1e-10 for GCV_PLAIN_FP64, 1e-8 for GCV_MIXED) */
    int max_depth;        /* maximum bisection depth below one knot interval (default 30) */
    int precision;        /* gcv_precision */
    void* stream;         /* cudaStream_t; NULL = legacy default stream */
    int collect_stats;    /* nonzero: count panels and Newton steps (gcv_get_stats) */
    int learned;          /* nonzero: start B-spline intervals at the depths predicted by the
                             network installed with gcv_set_learned_model
                             (gcurval_gb300_learned.h); no effect without one */
    int mapping;          /* the length walk's main pass with float-float panels (GCV_MIXED):
                             GCV_MAP_LANE (default) one thread per knot interval, or
                             GCV_MAP_HALF_WARP 16 threads per knot interval, one panel node
                             each; the same table up to the summation order of each
                             panel's nodes (float-float rounding); no effect on GCV_PLAIN_FP64 */
    int host_in_place;    /* nonzero: gcv_create_batch with GCV_HOST does not copy page-locked
                             knot and control arrays (gcv_host_alloc, cudaMallocHost,
                             cudaHostRegister); every table build reads them in place over the
                             CPU-GPU link, so they must stay alive and unchanged for the life
                             of the context.  Pageable arrays are copied as without it. */
} gcv_options;

enum gcv_mapping { GCV_MAP_LANE = 0, GCV_MAP_HALF_WARP = 1 };

typedef struct gcv_ctx gcv_ctx;

/* Result of gcv_arclength_reverse; mirrors gcurval::ArclengthReverseResult
 * (gcurval/base/structs.inl.h:66-77).  `data` holds n_points parameters u, or
 * n_points points of point_dim doubles (x, y[, z]); it is device memory when
 * store_where == GCV_DEVICE, else host memory.  Release it with
 * gcv_free_result (the reference has no free helper and leaks it to the
 * caller, gcurval/detail/cuda/arclength_calculate.h:462-499). */
typedef struct gcv_result {
    int64_t n_points;
    int store_where;
    int store_what;
    int point_dim;
    double* data;
} gcv_result;

/* Counters of the last table build / sampling call (filled when
 * options.collect_stats is set; the timings always). */
#define GCV_N_CODE_SLOTS 11

typedef struct gcv_stats {
    int64_t n_curves;
    int64_t n_segments;       /* knot intervals */
    int64_t n_leaves;         /* accepted quadrature panels (table entries) */
    int64_t n_panels;         /* panels evaluated by the length kernel */
    int64_t n_deep_segments;  /* intervals that needed the deep (global-memory) path */
    int64_t n_capped;         /* panels accepted at max_depth without meeting rtol */
    int64_t n_samples;
    int64_t n_newton;         /* Newton iterations of the sampling kernel */
    double ms_setup, ms_length, ms_scan, ms_sample;  /* device time per phase */
    int64_t n_launches;       /* kernels launched by the context so far */
    double ms_learned;        /* network inference inside ms_length (learned form) */
    /* launch shapes in use, picked by the autotuner: the first three table
       builds and samplings of a batch shape new to the process each try one
       candidate, later ones use the fastest (tuned = 1) */
    int length_blocks_per_sm, sample_threads, sample_blocks_per_sm, tuned;
    /* persistent length workers per SM of each curve code's main pass, by
       slot: ellipse 0, degree 1..5 in 2D at 1..5, in 3D at 6..10 */
    int length_blocks_per_sm_code[GCV_N_CODE_SLOTS];
} gcv_stats;

const char* gcv_status_string(gcv_status s);
const char* gcv_last_error(void);
int gcv_version(void);

/* Fills *opt with the defaults for `precision`. */
gcv_status gcv_default_options(gcv_options* opt, int precision);

/* ---- construction ------------------------------------------------------ */

/* Ellipses.  Replaces the ellipse sample's
 * ArclengthCalculateGpu(int n_curve, Dt* a, Dt* b)
 * (samples/sample1_ellipse/ellipse.h:121-129) over
 * ArclengthCalculateCuda(int n_curve, int n_seg) (arclength_calculate.h:141-153).
 * rot, cx, cy may be NULL (0).  where = GCV_HOST copies the arrays to the
 * device; GCV_DEVICE uses the caller's device arrays, which must stay alive
 * and unchanged for the life of the context (the reference's subclass fills
 * d_curve with device pointers it owns, ellipse.h:121-135). */
gcv_status gcv_create_ellipses(gcv_ctx** out, int n_curve, const double* a, const double* b,
                               const double* rot, const double* cx, const double* cy, int where,
                               const gcv_options* opt);

/* B-splines of one degree and dimension in the reference sample's layout:
 * knots_offset[n_curve + 1] (int32, prefix of knot counts), knot vectors back
 * to back, control points back to back (dim doubles each; curve c's first
 * control point is knots_offset[c] - (degree + 1) * c).  Replaces
 * ArclengthCalculateGpu(int n_curve, int* knots_offset, Dt* knot_vector,
 * Vector* ctrl_ptrs) (samples/sample2_bspline/arclength_calculate.h:505-518)
 * with n_seg = knots_offset[n] - (2 degree + 1) n (:506). */
gcv_status gcv_create_bsplines(gcv_ctx** out, int n_curve, int degree, int dim,
                               const int* knots_offset, const double* knot_vector,
                               const double* ctrl_pts, int where, const gcv_options* opt);

/* A batch of uneven curves (any mix of ellipses and B-splines of degree 1..5,
 * 2D/3D): per-curve kind/degree/dim, int64 offsets into one knot array and
 * one control array (ellipses: knots {0, 2 pi}, control a, b, rot, cx, cy).
 * No reference counterpart: the reference fixes kind and degree per
 * template instantiation (gcurval/arclength_calculate.h:10-18). */
gcv_status gcv_create_batch(gcv_ctx** out, int n_curve, const uint8_t* kind, const uint8_t* degree,
                            const uint8_t* dim, const int64_t* knot_off, const double* knots,
                            const int64_t* ctrl_off, const double* ctrl, int where,
                            const gcv_options* opt);

/* ~ArclengthCalculateCuda (arclength_calculate.h:168-183). */
gcv_status gcv_destroy(gcv_ctx* ctx);

/* Changes rtol / max_depth / precision / stream of an existing context; the
 * next gcv_create_arclength_table uses them. */
gcv_status gcv_set_options(gcv_ctx* ctx, const gcv_options* opt);

/* ---- arc length ----------------------------------------------------------- */

/* createArclengthTable (arclength_calculate.h:185-210): adaptive length of
 * every knot interval, then the per-curve cumulative table.  Asynchronous on
 * the context's stream except for one device-to-host read of the table size. */
gcv_status gcv_create_arclength_table(gcv_ctx* ctx);

/* getAllCurveArclengths (arclength_calculate.h:212-216): total length of every
 * curve into out[n_curve] (host or device memory per `where`).  Unlike the
 * reference, the caller provides the buffer instead of receiving new[]. */
gcv_status gcv_get_all_curve_arclengths(gcv_ctx* ctx, double* out, int where);

/* getArclength (arclength_calculate.h:218-222). */
gcv_status gcv_get_arclength(gcv_ctx* ctx, int cid, double* out);

/* arclengthReverse (arclength_calculate.h:224-231,408-505): n_ptrs_for_curves
 * (n_curve ints) samples per curve at sample_position (sum of counts doubles;
 * fractions of each curve's length when is_relative, else absolute lengths).
 * Inputs are host memory, as in the reference.  The result is allocated by
 * the library in `where` memory (GCV_DEVICE, the reference's default, or
 * GCV_HOST) and holds parameters (GCV_RETURN_US) or points
 * (GCV_RETURN_POINTS). */
gcv_status gcv_arclength_reverse(gcv_ctx* ctx, const int* n_ptrs_for_curves,
                                 const double* sample_position, int is_relative, int where,
                                 int what, gcv_result* result);

/* The same into caller-provided memory: counts and positions in `in_where`
 * memory, output `out` (n points or n * point_dim doubles) in `out_where`
 * memory.  No allocation for the result.  Host positions and host outputs
 * are streamed through device buffers in chunks of curves, the copies of
 * neighbouring chunks overlapping the sampling of the current one; the call
 * returns after the results are in `out`. */
gcv_status gcv_arclength_reverse_into(gcv_ctx* ctx, const int* n_ptrs_for_curves,
                                      const double* sample_position, int is_relative,
                                      int in_where, int what, double* out, int out_where);

gcv_status gcv_free_result(gcv_result* result);

/* createArclengthTable followed by arclengthReverse of device-resident
 * counts / positions into device memory, as one CUDA graph on the context's
 * stream.  The first call builds the table the ordinary way (which sizes the
 * leaf pool and the deep list), captures the whole step - set-up, network
 * inference when the learned form is on, the length passes with their item
 * counts read on the device, the scan, a device scan of the sample counts
 * and the sampling launches - and replays it; later calls with the same
 * buffers, flags and options only replay it (a change captures again).
 * The counts' and positions' contents may change between calls.  A replay
 * whose data outgrew the pools is redone the ordinary way, which grows them,
 * and the next call captures again.  No reference counterpart: the reference
 * synchronises with the host after every kernel
 * (gcurval/detail/cuda/arclength_calculate.h:259-323). */
gcv_status gcv_step_graph(gcv_ctx* ctx, const int* d_counts, const double* d_pos, int is_relative,
                          int what, double* d_out);
/* Drops the captured step (the next gcv_step_graph captures again). */
gcv_status gcv_step_graph_reset(gcv_ctx* ctx);

/* clearArclength (arclength_calculate.h:233-237): drops the cached lengths. */
gcv_status gcv_clear_arclength(gcv_ctx* ctx);

/* ---- introspection -------------------------------------------------------- */

gcv_status gcv_synchronize(gcv_ctx* ctx);
gcv_status gcv_get_stats(gcv_ctx* ctx, gcv_stats* out);
/* n_curve, total knot intervals and point dimension of a context. */
gcv_status gcv_get_shape(gcv_ctx* ctx, int64_t* n_curve, int64_t* n_segments, int* point_dim);

/* Measures the current GPU's fused multiply-add throughput with a register-
 * only kernel (which = 0: FP64, 1: FP32) in TFLOP/s (an FMA counts 2).  Used
 * as the roofline denominator of the FP-pipe-bound kernels.  No reference
 * counterpart. */
gcv_status gcv_measure_fma_peak(int which, double* tflops);

/* Device memory kept for reuse: a destroyed context's buffers stay allocated
 * in a process-wide cache and serve the next context that needs a similar
 * size (the counterpart of the reference samples' optional RMM pool,
 * samples/sample1_ellipse/main.cpp:147-155).  An allocation that finds the
 * GPU full frees the cache first.  Set GCV_NO_MEMORY_CACHE=1 in the
 * environment to free buffers at once instead.  This call frees the cached
 * buffers of every device; *bytes (may be NULL) receives how many bytes. */
gcv_status gcv_release_cached_memory(int64_t* bytes);

/* Page-locked host memory for the host-side arrays of gcv_create_batch and
 * gcv_arclength_reverse_into (curve data, positions, results).  The copy
 * engines read and write such buffers directly, asynchronously and at the
 * link rate; pageable arrays are still accepted and are streamed through
 * the library's own pinned staging buffers by host threads.  *p receives
 * NULL when bytes is 0.  Free with gcv_host_free.  No reference
 * counterpart (the reference copies pageable arrays with cudaMemcpy). */
gcv_status gcv_host_alloc(size_t bytes, void** p);
gcv_status gcv_host_free(void* p);

/* ---- FP32 data ------------------------------------------------------------
 * The reference's float instantiation, ArclengthCalculateGpu<float> (the
 * samples' default, samples/sample1_ellipse/main.cpp:16-20,
 * samples/sample2_bspline/main.cpp:19): the same calls with float curve
 * data, positions, lengths, parameters and points.  Inputs are widened to
 * double and the work runs as for double data (options.precision and rtol as
 * given; GCV_MIXED with rtol 1e-6 matches the reference's float tolerance
 * MAX_ERROR_FLOAT, gcurval/config.h:31); results are rounded to float.
 * Device FP32 B-spline data is widened into buffers the context owns. */
typedef struct gcv_result_f32 {
    int64_t n_points;
    int store_where;
    int store_what;
    int point_dim;
    float* data;
} gcv_result_f32;

gcv_status gcv_create_ellipses_f32(gcv_ctx** out, int n_curve, const float* a, const float* b, const float* rot,
                                   const float* cx, const float* cy, int where, const gcv_options* opt);
gcv_status gcv_create_bsplines_f32(gcv_ctx** out, int n_curve, int degree, int dim, const int* knots_offset,
                                   const float* knot_vector, const float* ctrl_pts, int where, const gcv_options* opt);
gcv_status gcv_get_all_curve_arclengths_f32(gcv_ctx* ctx, float* out, int where);
gcv_status gcv_get_arclength_f32(gcv_ctx* ctx, int cid, float* out);
gcv_status gcv_arclength_reverse_into_f32(gcv_ctx* ctx, const int* n_ptrs_for_curves, const float* sample_position,
                                          int is_relative, int in_where, int what, float* out, int out_where);
gcv_status gcv_arclength_reverse_f32(gcv_ctx* ctx, const int* n_ptrs_for_curves, const float* sample_position,
                                     int is_relative, int where, int what, gcv_result_f32* result);
gcv_status gcv_free_result_f32(gcv_result_f32* result);

/* ---- allocation-free lengths ---------------------------------------------- */

/* Largest number of knot intervals gcv_bspline_lengths_noalloc accepts. */
#define GCV_NOALLOC_MAX_INTERVALS 1048576

/* Total length of every curve of a B-spline batch, for callers that cannot
 * allocate device memory: services that reserve a fixed device-memory budget
 * at start-up and forbid allocation afterwards, and code running inside
 * another library's allocator or memory-pool hooks, where a nested cudaMalloc
 * would recurse or fail.  No counterpart in the reference.
 *
 * Same layout as gcv_create_bsplines, but every array is DEVICE memory:
 * knots_offset[n_curve + 1], knot_vector, ctrl_pts, and the output
 * lengths[n_curve].  The result equals gcv_create_arclength_table +
 * gcv_get_all_curve_arclengths (FP64, same rtol / max_depth) to rounding.
 * knots_offset is checked on the device before anything reads through it:
 * it must start at 0 and give every curve at least 2 degree + 1 knots, else
 * GCV_ERR_INVALID with the allocating path's message.  n_capped (host
 * pointer, may be NULL) receives the number of panels accepted at max_depth
 * without meeting rtol, as gcv_stats.n_capped does for the allocating path.
 * The call allocates nothing: its working memory is one static device array
 * of GCV_NOALLOC_MAX_INTERVALS doubles plus a 256-byte header (about 8 MiB),
 * held by every GPU that loads the library until the process exits; batches
 * with more knot intervals return GCV_ERR_INVALID.  The first call on a device
 * looks up that array's address with the device current and keeps it for the
 * life of the process: make that first call before any stream capture begins,
 * and make no call on a device after cudaDeviceReset.  Runs on `stream`
 * (cudaStream_t, NULL = legacy default stream) and waits for that stream
 * before returning.  All calls share the array, so calls whose GPU work
 * overlaps race and must be serialised by the caller. */
gcv_status gcv_bspline_lengths_noalloc(int n_curve, int degree, int dim, const int* knots_offset,
                                       const double* knot_vector, const double* ctrl_pts, double rtol,
                                       int max_depth, double* lengths, void* stream, int64_t* n_capped);

#ifdef __cplusplus
}
#endif
#endif /* GCURVAL_GB300_H */
