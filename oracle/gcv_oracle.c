/* Plain-C restatement of gcurval's CPU arc-length driver (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; the CUDA library never links
 * or calls it.
 *
 * Parity: pinned against the reference's own CPU driver compiled from the
 * reference tree (oracle/_ref/libgcv_ref.so, built by oracle/Makefile) on
 * seeded ellipses and B-splines; the committed golden vectors in
 * tests/golden/ carry those reference outputs to machines without the
 * reference tree.  Compiled with -ffp-contract=off so results do not depend
 * on whether the host compiler fuses multiply-adds (x86 and Arm agree).
 *
 * What each piece follows (paths inside the reference project):
 *   gl3()            GaussLegendreQuadrature<Dt>, gcurval/base/functors.inl.h:39-66,
 *                    3-point nodes/weights gcurval/base/constants.inl.h:123,133
 *   eps_at()         Epsilon<Dt>::v host table, gcurval/base/constants.inl.h:21-30
 *   seg_recursive()  ArclengthCalculateCpu::arclengthRecursive,
 *                    gcurval/detail/cpu/arclength_calculate.h:242-278
 *   build_curve()    createArclengthTable, cpu/arclength_calculate.h:80-139,
 *                    Kahan offsetting gcurval/base/util.h:134-172
 *   target_recursive() arclengthRecursiveWithTarget_Paper,
 *                    cpu/arclength_calculate.h:378-439
 *   reverse_curve()  arclengthReverse, cpu/arclength_calculate.h:152-238
 *   bspline_deriv()  b_spline_derv_o1 + to_point,
 *                    samples/sample2_bspline/BSpline.h:49-96
 *   bspline_point()  b_spline_func_value + to_point, BSpline.h:26-47,87-96
 *   ellipse_*()      point / derv_o1, samples/sample1_ellipse/ellipse.h:5-15
 *                    (plus rotation and centre for points, which leave |C'|
 *                    unchanged)
 * Two deliberate differences: the reference starts the first table interval
 * at u = 0 (cpu/arclength_calculate.h:200); here it starts at the curve's
 * first parameter value (every curve generated by this project starts at 0,
 * where both agree).  And a zero-width knot span (a repeated knot) adds 0 to
 * the length, where the reference's de Boor divides 0 by 0 and returns NaN
 * for the whole curve (see build_curve).
 */
#define _GNU_SOURCE
#include "gcv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

static const double GL3_X[3] = {0.0, -0.7745966692414834, 0.7745966692414834};
static const double GL3_W[3] = {0.8888888888888889, 0.5555555555555556, 0.5555555555555556};
static const double TWO_PI = 6.283185307179586476925286766559;

/* ------------------------------------------------------------------------ */
/* curve evaluation                                                          */

typedef struct pack {
    int kind, p, dim, span;
    const double* kv; /* curve's knot vector */
    const double* cp; /* curve's control data */
    uint64_t* evals;
} pack_t;

/* The de Boor routines below take the degree p and dimension d as
 * arguments of always-inlined bodies; the dispatchers after them call the
 * bodies with constant (p, d), so each common case is compiled with its
 * loops unrolled, as the reference's degree-templated functions are
 * (same operations in the same order: the results do not change). */
#define GCVO_INLINE static inline __attribute__((always_inline))

GCVO_INLINE void bspline_deriv_pd(double u, const pack_t* pk, double* out, const int p, const int d)
{
    double f[9], left[9], right[9], saved, temp;
    const int span = pk->span;
    const double* kv = pk->kv;
    f[0] = 1.0;
    for (int j = 1; j < p; j++) {
        left[j] = u - kv[span + 1 - j];
        right[j] = kv[span + j] - u;
        saved = 0.0;
        for (int r = 0; r < j; r++) {
            temp = f[r] / (right[r + 1] + left[j - r]);
            f[r] = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        f[j] = saved;
    }
    left[p] = u - kv[span + 1 - p];
    right[p] = kv[span + p] - u;
    saved = 0.0;
    for (int r = 0; r < p; r++) {
        temp = (double)p * f[r] / (right[r + 1] + left[p - r]);
        f[r] = saved - temp;
        saved = temp;
    }
    f[p] = saved;
    const double* c0 = pk->cp + (size_t)(span - p) * d;
    for (int k = 0; k < d; k++) out[k] = c0[k] * f[0];
    for (int i = 1; i <= p; i++)
        for (int k = 0; k < d; k++) out[k] += c0[(size_t)i * d + k] * f[i];
}

GCVO_INLINE void bspline_point_pd(double u, const pack_t* pk, double* out, const int p, const int d)
{
    double f[9], left[9], right[9], saved, temp;
    const int span = pk->span;
    const double* kv = pk->kv;
    f[0] = 1.0;
    for (int j = 1; j <= p; j++) {
        left[j] = u - kv[span + 1 - j];
        right[j] = kv[span + j] - u;
        saved = 0.0;
        for (int r = 0; r < j; r++) {
            temp = f[r] / (right[r + 1] + left[j - r]);
            f[r] = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        f[j] = saved;
    }
    const double* c0 = pk->cp + (size_t)(span - p) * d;
    for (int k = 0; k < d; k++) out[k] = c0[k] * f[0];
    for (int i = 1; i <= p; i++)
        for (int k = 0; k < d; k++) out[k] += c0[(size_t)i * d + k] * f[i];
}

#define GCVO_PD_CASES(FN)                                                                        \
    case 1 * 4 + 2: FN(1, 2); return;                                                            \
    case 2 * 4 + 2: FN(2, 2); return;                                                            \
    case 3 * 4 + 2: FN(3, 2); return;                                                            \
    case 4 * 4 + 2: FN(4, 2); return;                                                            \
    case 5 * 4 + 2: FN(5, 2); return;                                                            \
    case 1 * 4 + 3: FN(1, 3); return;                                                            \
    case 2 * 4 + 3: FN(2, 3); return;                                                            \
    case 3 * 4 + 3: FN(3, 3); return;                                                            \
    case 4 * 4 + 3: FN(4, 3); return;                                                            \
    case 5 * 4 + 3: FN(5, 3); return;

static void bspline_point(double u, const pack_t* pk, double* out)
{
#define GCVO_P(P, D) bspline_point_pd(u, pk, out, P, D)
    switch (pk->p * 4 + pk->dim) {
        GCVO_PD_CASES(GCVO_P)
    default: bspline_point_pd(u, pk, out, pk->p, pk->dim); return;
    }
#undef GCVO_P
}

GCVO_INLINE double speed_pd(const pack_t* pk, double u, const int p, const int d)
{
    double v[3] = {0.0, 0.0, 0.0}, s = 0.0;
    bspline_deriv_pd(u, pk, v, p, d);
    for (int k = 0; k < d; k++) s += v[k] * v[k];
    return sqrt(s);
}

GCVO_INLINE double ellipse_speed(const pack_t* pk, double u)
{
    double v[2], s;
    v[0] = -1.0 * pk->cp[0] * sin(u);
    v[1] = pk->cp[1] * cos(u);
    s = v[0] * v[0];
    s += v[1] * v[1];
    return sqrt(s);
}

static double speed(const pack_t* pk, double u)
{
    if (pk->kind == 0) return ellipse_speed(pk, u);
    return speed_pd(pk, u, pk->p, pk->dim);
}

static void point(const pack_t* pk, double u, double* out)
{
    if (pk->kind == 0) {
        const double a = pk->cp[0], b = pk->cp[1], th = pk->cp[2];
        const double x = a * cos(u), y = b * sin(u);
        const double c = cos(th), s = sin(th);
        out[0] = c * x - s * y + pk->cp[3];
        out[1] = s * x + c * y + pk->cp[4];
        return;
    }
    bspline_point(u, pk, out);
}

/* GaussLegendreQuadrature with 3 nodes (gcurval/base/functors.inl.h:39-66);
 * the speed of each node is inlined for the curve's (p, d). */
#define GCVO_GL3_BODY(SPEED)                                                                     \
    do {                                                                                         \
        for (int j = 0; j < 3; j++) {                                                            \
            const double u = k * GL3_X[j] + b;                                                   \
            acc += GL3_W[j] * (SPEED);                                                           \
        }                                                                                        \
    } while (0)

static double gl3(const pack_t* pk, double begin, double end)
{
    const double k = (end - begin) / 2.0;
    const double b = (end + begin) / 2.0;
    double acc = 0.0;
    *pk->evals += 3;
    if (pk->kind == 0) {
        GCVO_GL3_BODY(ellipse_speed(pk, u));
    } else {
#define GCVO_G(P, D) GCVO_GL3_BODY(speed_pd(pk, u, P, D)); break
        switch (pk->p * 4 + pk->dim) {
        case 1 * 4 + 2: GCVO_G(1, 2);
        case 2 * 4 + 2: GCVO_G(2, 2);
        case 3 * 4 + 2: GCVO_G(3, 2);
        case 4 * 4 + 2: GCVO_G(4, 2);
        case 5 * 4 + 2: GCVO_G(5, 2);
        case 1 * 4 + 3: GCVO_G(1, 3);
        case 2 * 4 + 3: GCVO_G(2, 3);
        case 3 * 4 + 3: GCVO_G(3, 3);
        case 4 * 4 + 3: GCVO_G(4, 3);
        case 5 * 4 + 3: GCVO_G(5, 3);
        default: GCVO_GL3_BODY(speed_pd(pk, u, pk->p, pk->dim)); break;
        }
#undef GCVO_G
    }
    acc *= k;
    return acc;
}

/* ------------------------------------------------------------------------ */
/* batch helpers                                                              */

static int curve_segments(const gcvo_batch* b, int c)
{
    const int64_t nk = b->knot_off[c + 1] - b->knot_off[c];
    if (b->kind[c] == 0) return (int)(nk - 1);
    return (int)(nk - 2 * (int64_t)b->degree[c] - 1);
}

static pack_t make_pack(const gcvo_batch* b, int c, int segid, uint64_t* evals)
{
    pack_t pk;
    pk.kind = b->kind[c];
    pk.p = pk.kind == 0 ? 0 : b->degree[c];
    pk.dim = pk.kind == 0 ? 2 : b->dim[c];
    pk.span = segid + pk.p;
    pk.kv = b->knots + b->knot_off[c];
    pk.cp = b->ctrl + b->ctrl_off[c];
    pk.evals = evals;
    return pk;
}

/* ------------------------------------------------------------------------ */
/* tables                                                                     */

typedef struct curve_tab {
    int64_t n, cap;
    double* u;
    double* al;
    int* seg;
} curve_tab;

struct gcvo_table {
    const gcvo_batch* b;
    gcvo_batch bcopy;
    double max_error;
    double eps[64]; /* max_error * 2^-level, as the reference's per-level table */
    int max_depth;
    curve_tab* tabs;
    double* length;
    uint64_t evals;
    pthread_mutex_t lock;
};

static void tab_push(curve_tab* t, double u, double al, int seg)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->u = (double*)realloc(t->u, sizeof(double) * t->cap);
        t->al = (double*)realloc(t->al, sizeof(double) * t->cap);
        t->seg = (int*)realloc(t->seg, sizeof(int) * t->cap);
    }
    t->u[t->n] = u;
    t->al[t->n] = al;
    t->seg[t->n] = seg;
    t->n++;
}

static double eps_at(const gcvo_table* t, int level) { return t->eps[level]; }

/* arclengthRecursive: total_length is the length accumulated inside the
 * segment up to `begin` (passed by value, as in the reference). */
static double seg_recursive(const gcvo_table* t, const pack_t* pk, double begin, double end,
                            double parent, int level, double total_length, int segid,
                            curve_tab* tab)
{
    const double mid = (begin + end) / 2.0;
    double left = gl3(pk, begin, mid);
    double right = gl3(pk, mid, end);
    if (level < t->max_depth && fabs(left + right - parent) > eps_at(t, level)) {
        left = seg_recursive(t, pk, begin, mid, left, level + 1, total_length, segid, tab);
        total_length += left;
        if (tab) tab_push(tab, mid, total_length, segid);
        right = seg_recursive(t, pk, mid, end, right, level + 1, total_length, segid, tab);
    }
    return left + right;
}

static void build_curve(gcvo_table* t, int c, uint64_t* evals)
{
    const gcvo_batch* b = t->b;
    curve_tab* tab = &t->tabs[c];
    const int nseg = curve_segments(b, c);
    double acc_curve = 0.0, residual = 0.0; /* Kahan pair (util.h:153-172) */
    for (int segid = 0; segid < nseg; segid++) {
        pack_t pk = make_pack(b, c, segid, evals);
        const double sb = pk.kv[pk.span], se = pk.kv[pk.span + 1];
        if (se == sb) {
            /* Zero-width knot span (repeated knot).  The reference evaluates
             * de Boor here, divides 0 by 0 and turns the whole curve's length
             * into NaN; the span's length is 0, so it contributes 0 and one
             * table entry, as a guarded reference would. */
            tab_push(tab, se, acc_curve + (0.0 - residual), segid);
            continue;
        }
        const double parent = gl3(&pk, sb, se);
        const int64_t store_begin = tab->n;
        const double acc_seg = seg_recursive(t, &pk, sb, se, parent, 0, 0.0, segid, tab);
        tab_push(tab, se, acc_seg, segid);
        /* precisely_summation(sum, a, residual) = sum + (a - residual) */
        for (int64_t i = store_begin; i < tab->n; i++) tab->al[i] = acc_curve + (tab->al[i] - residual);
        /* precisely_summation_ref: Kahan step */
        const double y = acc_seg - residual;
        const double s = acc_curve + y;
        residual = (s - acc_curve) - y;
        acc_curve = s;
    }
    t->length[c] = tab->n > 0 ? tab->al[tab->n - 1] : 0.0;
}

/* ------------------------------------------------------------------------ */
/* threading                                                                  */

typedef struct job {
    void (*fn)(struct job*, int);
    gcvo_table* t;
    atomic_int* next; /* shared: the next curve to take */
    int n;
    const int* n_per_curve;
    const int64_t* off;
    const double* pos;
    const double* uin;
    int is_relative, what, pdim;
    double* out;
    uint64_t evals;
} job_t;

/* Curves are taken one at a time from a shared counter (dynamic
 * scheduling): per-curve costs are heavy-tailed (a 4,096-point curve costs
 * thousands of times a 4-point one), so static ranges leave most threads
 * idle behind the one that drew the largest curves. */
static void* job_main(void* arg)
{
    job_t* j = (job_t*)arg;
    for (;;) {
        const int c = atomic_fetch_add_explicit(j->next, 1, memory_order_relaxed);
        if (c >= j->n) break;
        j->fn(j, c);
    }
    return NULL;
}

static void run_jobs(job_t* proto, int n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > n) nthreads = n > 0 ? n : 1;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    atomic_int next;
    atomic_init(&next, 0);
    for (int i = 0; i < nthreads; i++) {
        jobs[i] = *proto;
        jobs[i].next = &next;
        jobs[i].n = n;
        jobs[i].evals = 0;
        if (nthreads > 1)
            pthread_create(&th[i], NULL, job_main, &jobs[i]);
        else
            job_main(&jobs[i]);
    }
    uint64_t ev = 0;
    for (int i = 0; i < nthreads; i++) {
        if (nthreads > 1) pthread_join(th[i], NULL);
        ev += jobs[i].evals;
    }
    proto->t->evals += ev;
    free(jobs);
    free(th);
}

static void build_job(job_t* j, int c) { build_curve(j->t, c, &j->evals); }

gcvo_table* gcvo_build(const gcvo_batch* batch, double max_error, int max_depth, int nthreads)
{
    if (!batch || batch->n_curve < 0 || max_depth < 0 || max_depth > 60 || !(max_error > 0.0)) return NULL;
    for (int c = 0; c < batch->n_curve; c++) {
        if (curve_segments(batch, c) < 0) return NULL;
        if (batch->kind[c] == 1 && (batch->degree[c] < 1 || batch->degree[c] > 7)) return NULL;
        if (batch->kind[c] == 1 && batch->dim[c] != 2 && batch->dim[c] != 3) return NULL;
    }
    gcvo_table* t = (gcvo_table*)calloc(1, sizeof(gcvo_table));
    t->bcopy = *batch;
    t->b = &t->bcopy;
    t->max_error = max_error;
    t->max_depth = max_depth;
    for (int k = 0; k < 64; k++) t->eps[k] = ldexp(max_error, -k);
    t->tabs = (curve_tab*)calloc((size_t)(batch->n_curve > 0 ? batch->n_curve : 1), sizeof(curve_tab));
    t->length = (double*)calloc((size_t)(batch->n_curve > 0 ? batch->n_curve : 1), sizeof(double));
    pthread_mutex_init(&t->lock, NULL);
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.fn = build_job;
    proto.t = t;
    run_jobs(&proto, batch->n_curve, nthreads);
    return t;
}

void gcvo_free(gcvo_table* t)
{
    if (!t) return;
    for (int c = 0; c < t->b->n_curve; c++) {
        free(t->tabs[c].u);
        free(t->tabs[c].al);
        free(t->tabs[c].seg);
    }
    free(t->tabs);
    free(t->length);
    pthread_mutex_destroy(&t->lock);
    free(t);
}

void gcvo_lengths(const gcvo_table* t, double* out)
{
    memcpy(out, t->length, sizeof(double) * (size_t)t->b->n_curve);
}

int64_t gcvo_table_entries(const gcvo_table* t)
{
    int64_t s = 0;
    for (int c = 0; c < t->b->n_curve; c++) s += t->tabs[c].n;
    return s;
}

int64_t gcvo_evals(const gcvo_table* t) { return (int64_t)t->evals; }

int64_t gcvo_curve_table(const gcvo_table* t, int cid, const double** u, const double** al,
                         const int** segid)
{
    const curve_tab* tab = &t->tabs[cid];
    if (u) *u = tab->u;
    if (al) *al = tab->al;
    if (segid) *segid = tab->seg;
    return tab->n;
}

/* ------------------------------------------------------------------------ */
/* sampling                                                                   */

/* arclengthRecursiveWithTarget_Paper; acc/residual are the wider-type Kahan
 * pair passed by value, as in the reference. */
static double target_recursive(const gcvo_table* t, const pack_t* pk, double begin, double end,
                               double parent, double target, double acc, double residual,
                               int level, double* u, int* found)
{
    const double mid = (begin + end) / 2.0;
    double left = gl3(pk, begin, mid);
    double right = gl3(pk, mid, end);
    if (level < t->max_depth && fabs((left + right) - parent) > eps_at(t, level)) {
        left = target_recursive(t, pk, begin, mid, left, target, acc, residual, level + 1, u, found);
        if (!*found) {
            const double y = left - residual;
            const double s = acc + y;
            residual = (s - acc) - y;
            acc = s;
            right = target_recursive(t, pk, mid, end, right, target, acc, residual, level + 1, u, found);
        }
    } else if (target <= acc + (left - residual)) {
        if (mid - begin < t->max_error || level == t->max_depth) {
            *u = (begin + mid) / 2.0;
            *found = 1;
        } else {
            left = target_recursive(t, pk, begin, mid, left, target, acc, residual, level + 1, u, found);
        }
    } else if (target <= acc + ((left + right) - residual)) {
        if (end - mid < t->max_error || level == t->max_depth) {
            *u = (mid + end) / 2.0;
            *found = 1;
        } else {
            const double y = left - residual;
            const double s = acc + y;
            residual = (s - acc) - y;
            acc = s;
            right = target_recursive(t, pk, mid, end, right, target, acc, residual, level + 1, u, found);
        }
    }
    return left + right;
}

static double curve_start(const gcvo_batch* b, int c)
{
    const double* kv = b->knots + b->knot_off[c];
    return b->kind[c] == 0 ? kv[0] : kv[b->degree[c]];
}

static int64_t lower_bound_d(const double* a, int64_t n, double v)
{
    int64_t lo = 0, cnt = n;
    while (cnt > 0) {
        const int64_t step = cnt >> 1;
        if (a[lo + step] < v) {
            lo += step + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    return lo;
}

static void reverse_job(job_t* j, int c)
{
    const gcvo_table* t = j->t;
    const gcvo_batch* b = t->b;
    const curve_tab* tab = &t->tabs[c];
    const double L = t->length[c];
    for (int64_t i = j->off[c]; i < j->off[c + 1]; i++) {
        double target = j->is_relative ? j->pos[i] * L : j->pos[i];
        double ures;
        int segid = 0;
        if (tab->n == 0) {
            ures = curve_start(b, c);
        } else {
            int64_t it = lower_bound_d(tab->al, tab->n, target);
            if (it == tab->n) it = tab->n - 1;
            double begin = curve_start(b, c), end;
            if (it > 0) {
                target -= tab->al[it - 1];
                begin = tab->u[it - 1];
                segid = tab->seg[it];
            }
            end = tab->u[it];
            pack_t pk = make_pack(b, c, segid, &j->evals);
            const double parent = gl3(&pk, begin, end);
            int found = 0;
            ures = end;
            target_recursive(t, &pk, begin, end, parent, target, 0.0, 0.0, 0, &ures, &found);
        }
        if (j->what == 0) {
            j->out[i] = ures;
        } else {
            pack_t pk = make_pack(b, c, segid, &j->evals);
            double p3[3] = {0.0, 0.0, 0.0};
            point(&pk, ures, p3);
            for (int k = 0; k < j->pdim; k++) j->out[i * j->pdim + k] = p3[k];
        }
    }
}

static int batch_point_dim(const gcvo_batch* b)
{
    int d = 0;
    for (int c = 0; c < b->n_curve; c++) {
        const int dc = b->kind[c] == 0 ? 2 : b->dim[c];
        if (d == 0) d = dc;
        else if (d != dc) return 3;
    }
    return d ? d : 2;
}

int gcvo_reverse(const gcvo_table* t, const int* n_per_curve, const double* pos, int is_relative,
                 int what, double* out, int nthreads)
{
    const int n = t->b->n_curve;
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    off[0] = 0;
    for (int c = 0; c < n; c++) off[c + 1] = off[c] + n_per_curve[c];
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.fn = reverse_job;
    proto.t = (gcvo_table*)t;
    proto.n_per_curve = n_per_curve;
    proto.off = off;
    proto.pos = pos;
    proto.is_relative = is_relative;
    proto.what = what;
    proto.pdim = batch_point_dim(t->b);
    proto.out = out;
    run_jobs(&proto, n, nthreads);
    free(off);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* arc length at a parameter                                                  */

static double s_at_impl(const gcvo_table* t, int c, double u, uint64_t* evals)
{
    const gcvo_batch* b = t->b;
    const curve_tab* tab = &t->tabs[c];
    if (tab->n == 0) return 0.0;
    int64_t it = lower_bound_d(tab->u, tab->n, u);
    if (it == tab->n) it = tab->n - 1;
    const double begin = it > 0 ? tab->u[it - 1] : curve_start(b, c);
    const double base = it > 0 ? tab->al[it - 1] : 0.0;
    pack_t pk = make_pack(b, c, tab->seg[it], evals);
    const double parent = gl3(&pk, begin, u);
    return base + seg_recursive(t, &pk, begin, u, parent, 0, 0.0, 0, NULL);
}

double gcvo_s_at(const gcvo_table* t, int cid, double u)
{
    uint64_t ev = 0;
    return s_at_impl(t, cid, u, &ev);
}

static void s_at_job(job_t* j, int c)
{
    for (int64_t i = j->off[c]; i < j->off[c + 1]; i++) j->out[i] = s_at_impl(j->t, c, j->uin[i], &j->evals);
}

void gcvo_s_at_many(const gcvo_table* t, const int* n_per_curve, const double* u, double* out,
                    int nthreads)
{
    const int n = t->b->n_curve;
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    off[0] = 0;
    for (int c = 0; c < n; c++) off[c + 1] = off[c] + n_per_curve[c];
    job_t proto;
    memset(&proto, 0, sizeof(proto));
    proto.fn = s_at_job;
    proto.t = (gcvo_table*)t;
    proto.off = off;
    proto.uin = u;
    proto.out = out;
    run_jobs(&proto, n, nthreads);
    free(off);
}

double gcvo_speed(const gcvo_batch* b, int cid, double u)
{
    uint64_t ev = 0;
    /* find the knot span containing u */
    const double* kv = b->knots + b->knot_off[cid];
    const int nseg = curve_segments(b, cid);
    const int p = b->kind[cid] == 0 ? 0 : b->degree[cid];
    int seg = 0;
    while (seg + 1 < nseg && u >= kv[seg + p + 1]) seg++;
    pack_t pk = make_pack(b, cid, seg, &ev);
    return speed(&pk, u);
}

void gcvo_point(const gcvo_batch* b, int cid, double u, double* out)
{
    uint64_t ev = 0;
    const double* kv = b->knots + b->knot_off[cid];
    const int nseg = curve_segments(b, cid);
    const int p = b->kind[cid] == 0 ? 0 : b->degree[cid];
    int seg = 0;
    while (seg + 1 < nseg && u >= kv[seg + p + 1]) seg++;
    pack_t pk = make_pack(b, cid, seg, &ev);
    point(&pk, u, out);
}

/* C(u) evaluated on knot interval segid of curve cid (span segid + degree),
 * as a plugin's GetPoint does with the pack of that interval
 * (samples/sample2_bspline/structs.h:165-174); -1 for a bad segid. */
int gcvo_point_seg(const gcvo_batch* b, int cid, int segid, double u, double* out)
{
    uint64_t ev = 0;
    if (segid < 0 || segid >= curve_segments(b, cid)) return -1;
    pack_t pk = make_pack(b, cid, segid, &ev);
    point(&pk, u, out);
    return 0;
}

/* the two-pi constant is part of the ellipse knot convention */
double gcvo_two_pi(void) { return TWO_PI; }
