// C ABI of the arc-length library (include/gcurval_gb300.h): contexts, device
// memory, and the host-side orchestration of the set-up, length, scan and
// sampling kernels on the context's stream.
#include "gcurval_gb300.h"
#include "gcurval_gb300_learned.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gcv_learned.cuh"
#include "gcv_length.cuh"
#include "gcv_sample.cuh"
#include "gcv_staging.h"
#include "gcv_table_kernels.cuh"

using namespace gcv;

namespace {

thread_local std::string g_err;

gcv_status fail(gcv_status s, const std::string& msg)
{
    g_err = msg;
    return s;
}

gcv_status cuda_fail(cudaError_t e, const char* what)
{
    cudaGetLastError();
    const gcv_status s = e == cudaErrorMemoryAllocation ? GCV_ERR_OUT_OF_MEMORY
                       : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
                           ? GCV_ERR_NO_DEVICE
                           : GCV_ERR_CUDA;
    return fail(s, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);                                        \
    } while (0)

#define CHECK(st)                                                                                  \
    do {                                                                                           \
        gcv_status s_ = (st);                                                                      \
        if (s_ != GCV_OK) return s_;                                                               \
    } while (0)

// ---------------------------------------------------- device memory cache
// A destroyed context hands its device buffers to a process-wide cache, and
// the next context that asks for a similar size (at most 1/8 larger) takes
// one from there instead of calling cudaMalloc: the counterpart of the
// memory pool the reference's samples can start (RMM,
// samples/sample1_ellipse/main.cpp:147-155).  Creating and destroying
// contexts of one batch shape then maps and unmaps none of the ~100 GB a
// 1M-curve table holds.  Buffers enter the cache only after a device-wide
// synchronisation (what cudaFree would have done), so a cached block is idle.
// A cudaMalloc that runs out of memory frees the oldest cached blocks (those
// least likely to be asked for again) until it succeeds.
// GCV_NO_MEMORY_CACHE=1 in the environment turns the cache off;
// gcv_release_cached_memory() frees it.
struct CachedBlock {
    void* p;
    int dev;
    unsigned long long seq;  // order of entry
};
std::mutex g_cache_m;
std::multimap<size_t, CachedBlock> g_cache;  // by size in bytes
unsigned long long g_cache_seq = 0;

bool cache_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("GCV_NO_MEMORY_CACHE");
        return !(v && v[0] && v[0] != '0');
    }();
    return on;
}

int current_device()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return dev;
}

// frees the cached blocks of device `dev` (-1: of every device); returns bytes
size_t release_cache(int dev)
{
    std::vector<std::pair<void*, int>> drop;
    size_t bytes = 0;
    {
        std::lock_guard<std::mutex> g(g_cache_m);
        for (auto it = g_cache.begin(); it != g_cache.end();) {
            if (dev < 0 || it->second.dev == dev) {
                drop.push_back({it->second.p, it->second.dev});
                bytes += it->first;
                it = g_cache.erase(it);
            } else {
                ++it;
            }
        }
    }
    const int cur = current_device();
    for (auto& d : drop) {
        if (d.second != cur) cudaSetDevice(d.second);
        cudaFree(d.first);
        if (d.second != cur) cudaSetDevice(cur);
    }
    return bytes;
}

// frees the oldest cached blocks of device `dev` until `want` bytes are
// freed (or none is left); returns the bytes freed
size_t release_oldest(int dev, size_t want)
{
    std::vector<void*> drop;
    size_t bytes = 0;
    {
        std::lock_guard<std::mutex> g(g_cache_m);
        while (bytes < want) {
            auto oldest = g_cache.end();
            for (auto it = g_cache.begin(); it != g_cache.end(); ++it)
                if (it->second.dev == dev && (oldest == g_cache.end() || it->second.seq < oldest->second.seq))
                    oldest = it;
            if (oldest == g_cache.end()) break;
            drop.push_back(oldest->second.p);
            bytes += oldest->first;
            g_cache.erase(oldest);
        }
    }
    for (void* q : drop) cudaFree(q);
    return bytes;
}

// a block of at least `bytes`; *got = its size
cudaError_t dev_alloc(void** p, size_t bytes, size_t* got)
{
    const int dev = current_device();
    if (cache_enabled()) {
        std::lock_guard<std::mutex> g(g_cache_m);
        for (auto it = g_cache.lower_bound(bytes); it != g_cache.end() && it->first <= bytes + bytes / 8; ++it) {
            if (it->second.dev == dev) {
                *p = it->second.p;
                *got = it->first;
                g_cache.erase(it);
                return cudaSuccess;
            }
        }
    }
    cudaError_t e = cudaMalloc(p, bytes);
    while (e == cudaErrorMemoryAllocation && cache_enabled()) {
        cudaGetLastError();
        if (release_oldest(dev, bytes) == 0) break;
        e = cudaMalloc(p, bytes);
    }
    *got = e == cudaSuccess ? bytes : 0;
    return e;
}

// an idle block into the cache (or freed when the cache is off)
void dev_recycle(void* p, size_t bytes)
{
    if (!p) return;
    if (!cache_enabled()) {
        cudaFree(p);
        return;
    }
    std::lock_guard<std::mutex> g(g_cache_m);
    g_cache.insert({bytes, CachedBlock{p, current_device(), ++g_cache_seq}});
}

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    size_t bytes = 0;  // size of the block behind p (owned blocks)
    bool owned = true;

    gcv_status reserve(size_t count)
    {
        if (count <= n && p) return GCV_OK;
        release();
        if (count == 0) count = 1;
        void* q = nullptr;
        size_t got = 0;
        cudaError_t e = dev_alloc(&q, count * sizeof(T), &got);
        if (e != cudaSuccess) {
            p = nullptr;
            n = 0;
            bytes = 0;
            return cuda_fail(e, "cudaMalloc");
        }
        p = static_cast<T*>(q);
        n = count;
        bytes = got;
        owned = true;
        return GCV_OK;
    }
    void borrow(const T* q, size_t count)
    {
        release();
        p = const_cast<T*>(q);
        n = count;
        bytes = 0;
        owned = false;
    }
    // frees at once (cudaFree synchronises the device): for buffers replaced
    // while the context's work may still be in flight
    void release()
    {
        if (p && owned) cudaFree(p);
        p = nullptr;
        n = 0;
        bytes = 0;
        owned = true;
    }
    // to the cache: only when the device is idle (context destruction)
    void recycle()
    {
        if (p && owned) dev_recycle(p, bytes);
        p = nullptr;
        n = 0;
        bytes = 0;
        owned = true;
    }
};

template <typename T>
gcv_status upload(DBuf<T>& b, const T* h, size_t count, cudaStream_t st)
{
    CHECK(b.reserve(count));
    if (count) CU(cudaMemcpyAsync(b.p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
    return GCV_OK;
}

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

// the curve codes' slots in per-code tables: ellipse 0, then degree 1-5 in
// 2D (1-5) and in 3D (6-10)
constexpr int N_CODE_SLOTS = GCV_N_CODE_SLOTS;
inline int code_slot(int code) { return code == CODE_ELLIPSE ? 0 : 1 + (code_dim(code) - 2) * 5 + (code_degree(code) - 1); }

// Launch shapes picked by the autotuner: persistent length workers per SM
// (cap on the occupancy) for each curve code's main pass and for the deep
// passes, and the sampling kernels' block size and blocks per SM.
struct Knobs {
    int length_cap[N_CODE_SLOTS];
    int deep_cap = 32;
    int sample_threads = 256;
    int sample_blocks_per_sm = 64;
    Knobs()
    {
        for (int& x : length_cap) x = 32;
    }
    bool operator==(const Knobs& o) const
    {
        return std::memcmp(length_cap, o.length_cap, sizeof(length_cap)) == 0 && deep_cap == o.deep_cap &&
               sample_threads == o.sample_threads && sample_blocks_per_sm == o.sample_blocks_per_sm;
    }
};
// The first TUNE_TRIALS table builds (and samplings) of a batch shape not seen
// before in the process each run one candidate; the fastest shapes, timed by
// the context's events, are kept for that shape (curve code, precision,
// learned form, log2 of the interval count).  The length walk is timed code
// by code (its main pass launches once per curve code), so each code of a
// batch that mixes codes keeps the persistent-worker count that was fastest
// for it.  The shapes change scheduling only: every result is the same
// under each, bit for bit.  (The half-warp-per-interval mapping of the main
// pass sums each panel's nodes in another order, so it is a user option,
// gcv_options.mapping, not a shape the tuner may pick.)
constexpr int TUNE_TRIALS = 3;
inline int trial_length_cap(int i) { return i == 1 ? 4 : (i == 2 ? 6 : 32); }
inline Knobs trial_knobs(int i)
{
    Knobs k;
    for (int& x : k.length_cap) x = trial_length_cap(i);
    k.deep_cap = trial_length_cap(i);
    if (i == 1) {
        k.sample_threads = 128;
        k.sample_blocks_per_sm = 128;
    } else if (i == 2) {
        k.sample_threads = 512;
        k.sample_blocks_per_sm = 16;
    }
    return k;
}
struct TuneKey {
    int code, precision, learned, log_seg;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(code, precision, learned, log_seg) < std::tie(o.code, o.precision, o.learned, o.log_seg);
    }
};
static std::mutex g_tune_m;
static std::map<TuneKey, Knobs> g_tuned;

constexpr int STREAM_EVENTS = 4;  // host-buffer sampling: events per stage, used round robin

struct CodeRange {
    int code;
    int64_t begin, end;  // range of the grouped segment list
    int64_t coef_base;   // coefficient index of the range's first segment
};

struct gcv_ctx {
    gcv_options opt{};
    cudaStream_t stream = nullptr;
    int64_t n_curve = 0, n_seg = 0, n_coef = 0;
    int point_dim = 2;
    int code = -1;  // common curve code, -1 when the batch mixes codes

    // batch (owned or borrowed)
    DBuf<uint8_t> kind, degree, dim;
    DBuf<int64_t> knot_off, ctrl_off;
    DBuf<double> knots, ctrl;
    // derived
    DBuf<int64_t> seg_off, coef_off;
    DBuf<int> seg_curve;
    std::vector<int64_t> h_seg_off;
    std::vector<uint8_t> h_kind, h_degree;
    std::vector<double> h_start;  // first parameter value of each curve
    // batches that mix curve codes: segments and curves grouped by code, one
    // range per code in each list
    DBuf<int> seg_list, curve_list;
    std::vector<CodeRange> code_ranges, curve_ranges;
    std::vector<int> h_curve_list;
    DBuf<int64_t> list_sample_off;  // sample-count prefix in curve_list order
    // learned form: the network's weight image and per-interval start depths
    void* mlp_w = nullptr;
    DBuf<uint32_t> starts;
    DBuf<uint4> feat16;  // bf16 feature rows of the B-spline intervals (2 uint4 each), written by set-up

    // table
    DBuf<double> coef, seg_t0, seg_t1, seg_f0, seg_q0, seg_len, seg_cum, curve_len;
    DBuf<int64_t> leaf_off;
    DBuf<int> leaf_cnt;
    DBuf<double> leaf_v, leaf_cum;
    DBuf<float> leaf_f, leaf_q;
    int64_t leaf_cap = 0;
    DBuf<int> deep_list;
    DBuf<unsigned long long> ctr;
    DBuf<int> scan_status, scan_flag;
    DBuf<double> scan_hi, scan_lo;
    bool table_ready = false;
    DBuf<float2> coef_ff;  // float-float copy of coef (GCV_MIXED)

    // sampling scratch
    DBuf<int64_t> sample_off;
    DBuf<int> sample_cnt;
    DBuf<double> sample_pos, sample_out;
    DBuf<float> f32_buf;  // float positions / results of the FP32 entry points
    std::vector<int64_t> h_sample_off;

    std::vector<double> h_len;
    bool h_len_valid = false;
    unsigned long long* h_ctr = nullptr;  // pinned
    // one-call steps captured as a CUDA graph (gcv_step_graph)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;  // capture stream when the context uses the legacy stream
    struct {
        const int* counts;
        const double* pos;
        double* out;
        int is_relative, what, learned;
        gcv_options opt;
    } gargs{};
    DBuf<int64_t> scan_blk;
    int64_t graph_kernels = 0;
    Knobs knobs, gknobs;  // launch shapes in use / in the captured step
    // autotuner progress of this context (-1: tuned, shapes from the table)
    int len_trial = 0, smp_trial = 0;
    double len_ms[TUNE_TRIALS] = {}, smp_ms[TUNE_TRIALS] = {};
    // per-code main-pass times of the tuning builds (ev_code: start / end of
    // each code's main-pass launch in the last build)
    double len_code_ms[TUNE_TRIALS][N_CODE_SLOTS] = {};
    cudaEvent_t ev_code[N_CODE_SLOTS][2] = {};
    bool code_timed[N_CODE_SLOTS] = {};
    TuneKey tune_key{-9, -9, -9, -9};
    // chunked host <-> device streaming of samples
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[STREAM_EVENTS] = {}, ev_done[STREAM_EVENTS] = {}, ev_out[STREAM_EVENTS] = {};
    gcv_stats stats{};
    cudaEvent_t ev[8] = {};
    bool ev_table = false, ev_sample = false;
    bool learned_ran = false;
};

namespace {

Batch batch_view(gcv_ctx* c)
{
    Batch b;
    b.n_curve = c->n_curve;
    b.n_seg = c->n_seg;
    b.kind = c->kind.p;
    b.degree = c->degree.p;
    b.dim = c->dim.p;
    b.knot_off = c->knot_off.p;
    b.knots = c->knots.p;
    b.ctrl_off = c->ctrl_off.p;
    b.ctrl = c->ctrl.p;
    b.seg_off = c->seg_off.p;
    b.coef_off = c->coef_off.p;
    b.seg_curve = c->seg_curve.p;
    return b;
}

Table table_view(gcv_ctx* c)
{
    Table t;
    t.coef = c->coef.p;
    t.coef_ff = c->opt.precision == GCV_MIXED ? c->coef_ff.p : nullptr;
    t.seg_t0 = c->seg_t0.p;
    t.seg_t1 = c->seg_t1.p;
    t.seg_f0 = c->seg_f0.p;
    t.seg_q0 = c->seg_q0.p;
    t.seg_len = c->seg_len.p;
    t.seg_cum = c->seg_cum.p;
    t.curve_len = c->curve_len.p;
    t.leaf_off = c->leaf_off.p;
    t.leaf_cnt = c->leaf_cnt.p;
    t.leaf_v = c->leaf_v.p;
    t.leaf_cum = c->leaf_cum.p;
    t.leaf_f = c->leaf_f.p;
    t.leaf_q = c->leaf_q.p;
    t.leaf_cap = c->leaf_cap;
    t.deep_list = c->deep_list.p;
    t.deep_cap = (int64_t)c->deep_list.n;
    t.ctr = c->ctr.p;
    t.scan_status = c->scan_status.p;
    t.scan_flag = c->scan_flag.p;
    t.scan_hi = c->scan_hi.p;
    t.scan_lo = c->scan_lo.p;
    return t;
}

gcv_status check_options(const gcv_options* o)
{
    if (!o) return fail(GCV_ERR_INVALID, "options are NULL");
    if (o->mapping != GCV_MAP_LANE && o->mapping != GCV_MAP_HALF_WARP)
        return fail(GCV_ERR_INVALID, "mapping must be GCV_MAP_LANE or GCV_MAP_HALF_WARP");
    if (!(o->rtol > 0.0) || !(o->rtol < 1.0)) return fail(GCV_ERR_INVALID, "rtol must be in (0, 1)");
    if (o->max_depth < 1 || o->max_depth > MAX_DEPTH_LIMIT)
        return fail(GCV_ERR_INVALID, "max_depth must be in [1, " + std::to_string(MAX_DEPTH_LIMIT) + "]");
    if (o->precision != GCV_PLAIN_FP64 && o->precision != GCV_MIXED)
        return fail(GCV_ERR_INVALID, "unknown precision mode");
    return GCV_OK;
}

void destroy_ctx(gcv_ctx* c)
{
    if (!c) return;
    // the context's buffers go to the memory cache idle, as cudaFree would
    // have left them
    if (cache_enabled()) cudaDeviceSynchronize();
    c->kind.recycle();
    c->degree.recycle();
    c->dim.recycle();
    c->knot_off.recycle();
    c->ctrl_off.recycle();
    c->knots.recycle();
    c->ctrl.recycle();
    c->seg_off.recycle();
    c->coef_off.recycle();
    c->seg_curve.recycle();
    c->seg_list.recycle();
    c->curve_list.recycle();
    c->starts.recycle();
    c->feat16.recycle();
    if (c->mlp_w) cudaFree(c->mlp_w);
    c->list_sample_off.recycle();
    c->coef.recycle();
    c->seg_t0.recycle();
    c->seg_t1.recycle();
    c->seg_f0.recycle();
    c->seg_q0.recycle();
    c->seg_len.recycle();
    c->seg_cum.recycle();
    c->curve_len.recycle();
    c->leaf_off.recycle();
    c->leaf_cnt.recycle();
    c->leaf_v.recycle();
    c->leaf_cum.recycle();
    c->leaf_f.recycle();
    c->leaf_q.recycle();
    c->deep_list.recycle();
    c->ctr.recycle();
    c->scan_status.recycle();
    c->scan_flag.recycle();
    c->scan_hi.recycle();
    c->scan_lo.recycle();
    c->sample_off.recycle();
    c->sample_cnt.recycle();
    c->sample_pos.recycle();
    c->sample_out.recycle();
    c->f32_buf.recycle();
    c->coef_ff.recycle();
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    for (int k = 0; k < STREAM_EVENTS; ++k) {
        if (c->ev_in[k]) cudaEventDestroy(c->ev_in[k]);
        if (c->ev_done[k]) cudaEventDestroy(c->ev_done[k]);
        if (c->ev_out[k]) cudaEventDestroy(c->ev_out[k]);
    }
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    if (c->gstream) cudaStreamDestroy(c->gstream);
    c->scan_blk.recycle();
    if (c->s_in) cudaStreamDestroy(c->s_in);
    if (c->s_out) cudaStreamDestroy(c->s_out);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& pair : c->ev_code)
        for (auto& e : pair)
            if (e) cudaEventDestroy(e);
    delete c;
}

// Validates per-curve metadata on the host and derives segment / coefficient
// offsets.  knot_off and ctrl_off are int64 prefix arrays of length n + 1.
gcv_status derive_layout(gcv_ctx* c, const uint8_t* kind, const uint8_t* degree, const uint8_t* dim,
                         const int64_t* knot_off, const int64_t* ctrl_off, std::vector<int64_t>& seg_off,
                         std::vector<int64_t>& coef_off)
{
    const int64_t n = c->n_curve;
    seg_off.assign(n + 1, 0);
    coef_off.assign(n + 1, 0);
    int common = -2, pdim = 0;
    bool mixed_dim = false;
    if (knot_off[0] != 0 || ctrl_off[0] != 0) return fail(GCV_ERR_INVALID, "offsets must start at 0");
    for (int64_t i = 0; i < n; ++i) {
        const int64_t nk = knot_off[i + 1] - knot_off[i];
        const int64_t nc = ctrl_off[i + 1] - ctrl_off[i];
        int64_t ns = 0;
        int code = 0, d = 2;
        if (kind[i] == GCV_KIND_ELLIPSE) {
            if (nk != 2 || nc != 5)
                return fail(GCV_ERR_INVALID, "curve " + std::to_string(i) + ": an ellipse has 2 knots and 5 control values");
            ns = ELLIPSE_PIECES;
            code = CODE_ELLIPSE;
        } else if (kind[i] == GCV_KIND_BSPLINE) {
            const int p = degree[i];
            d = dim[i];
            if (p < 1 || p > MAX_DEGREE)
                return fail(GCV_ERR_INVALID, "curve " + std::to_string(i) + ": degree must be in [1, 5]");
            if (d != 2 && d != 3) return fail(GCV_ERR_INVALID, "curve " + std::to_string(i) + ": dim must be 2 or 3");
            ns = nk - 2 * p - 1;
            if (ns < 0)
                return fail(GCV_ERR_INVALID, "curve " + std::to_string(i) + ": fewer than 2 * degree + 1 knots");
            if (nc != (nk - p - 1) * d)
                return fail(GCV_ERR_INVALID,
                            "curve " + std::to_string(i) + ": control values must be (knots - degree - 1) * dim");
            code = bs_code(p, d);
        } else {
            return fail(GCV_ERR_INVALID, "curve " + std::to_string(i) + ": unknown kind");
        }
        if (nk < 0 || nc < 0) return fail(GCV_ERR_INVALID, "offsets must be non-decreasing");
        seg_off[i + 1] = seg_off[i] + ns;
        coef_off[i + 1] = coef_off[i] + ns * code_stride(code);
        if (common == -2)
            common = code;
        else if (common != code)
            common = -1;
        if (pdim == 0)
            pdim = d;
        else if (pdim != d)
            mixed_dim = true;
    }
    c->n_seg = seg_off[n];
    c->n_coef = coef_off[n];
    c->code = common >= 0 ? common : -1;
    c->point_dim = mixed_dim ? 3 : (pdim ? pdim : 2);
    if (c->n_seg > (int64_t)0x7fffffff) return fail(GCV_ERR_INVALID, "more than 2^31 - 1 knot intervals");
    return GCV_OK;
}

gcv_status finish_create(gcv_ctx* c, const uint8_t* kind, const uint8_t* degree, const uint8_t* dim,
                         const int64_t* knot_off, const int64_t* ctrl_off, const double* knots_host_or_null)
{
    std::vector<int64_t> seg_off, coef_off;
    CHECK(derive_layout(c, kind, degree, dim, knot_off, ctrl_off, seg_off, coef_off));
    c->h_seg_off = seg_off;
    c->h_kind.assign(kind, kind + c->n_curve);
    c->h_degree.assign(degree, degree + c->n_curve);
    (void)knots_host_or_null;
    CHECK(upload(c->seg_off, seg_off.data(), seg_off.size(), c->stream));
    CHECK(upload(c->coef_off, coef_off.data(), coef_off.size(), c->stream));
    CHECK(c->seg_curve.reserve((size_t)std::max<int64_t>(c->n_seg, 1)));
    CHECK(c->ctr.reserve(C_COUNT));
    CU(cudaMallocHost(&c->h_ctr, C_COUNT * sizeof(unsigned long long)));
    for (auto& e : c->ev) CU(cudaEventCreate(&e));
    for (auto& pair : c->ev_code)
        for (auto& e : pair) CU(cudaEventCreate(&e));
    if (c->n_curve > 0) {
        const Batch b = batch_view(c);
        const int blocks = (int)std::min<int64_t>((c->n_curve + 255) / 256, 65535);
        k_seg_curve<<<blocks, 256, 0, c->stream>>>(b, c->seg_curve.p);
        CU(cudaGetLastError());
        c->stats.n_launches++;
    }
    if (c->code < 0 && c->n_seg > 0) {
        // Group the segments by curve code (stable within a code), so that
        // every main-pass launch runs one specialised kernel over one code.
        const int64_t n = c->n_curve;
        std::vector<int> code_of((size_t)n);
        std::vector<int64_t> per_code(64, 0);
        for (int64_t i = 0; i < n; ++i) {
            const int cd = kind[i] == GCV_KIND_ELLIPSE ? CODE_ELLIPSE : bs_code(degree[i], dim[i]);
            code_of[(size_t)i] = cd;
            per_code[(size_t)cd] += seg_off[(size_t)i + 1] - seg_off[(size_t)i];
        }
        std::vector<int64_t> base(64, 0);
        int64_t at = 0;
        c->code_ranges.clear();
        int64_t coef_at = 0;
        std::vector<int64_t> coef_base(64, 0);
        for (int cd = 0; cd < 64; ++cd) {
            base[(size_t)cd] = at;
            coef_base[(size_t)cd] = coef_at;
            if (per_code[(size_t)cd] > 0) {
                c->code_ranges.push_back(CodeRange{cd, at, at + per_code[(size_t)cd], coef_at});
                at += per_code[(size_t)cd];
                coef_at += per_code[(size_t)cd] * code_stride(cd);
            }
        }
        if (c->code_ranges.size() > (size_t)(C_COUNT - C_WORK_CODE))
            return fail(GCV_ERR_INVALID, "too many distinct curve codes in one batch");
        const std::vector<int64_t> range_begin = base;
        std::vector<int64_t> dst((size_t)n);
        for (int64_t i = 0; i < n; ++i) {
            const int cd = code_of[(size_t)i];
            int64_t& nb = base[(size_t)cd];
            // the coefficient table follows the grouped list: curve i's
            // first segment at its list position within the code's range
            coef_off[(size_t)i] = coef_base[(size_t)cd] + (nb - range_begin[(size_t)cd]) * code_stride(cd);
            dst[(size_t)i] = nb;
            nb += seg_off[(size_t)i + 1] - seg_off[(size_t)i];
        }
        CHECK(upload(c->coef_off, coef_off.data(), coef_off.size(), c->stream));
        // curves grouped the same way (sampling launches)
        std::vector<int64_t> curve_base(64, 0), per_code_curves(64, 0);
        for (int64_t i = 0; i < n; ++i) per_code_curves[(size_t)code_of[(size_t)i]]++;
        c->curve_ranges.clear();
        int64_t cat = 0;
        for (int cd = 0; cd < 64; ++cd) {
            curve_base[(size_t)cd] = cat;
            if (per_code_curves[(size_t)cd] > 0) {
                c->curve_ranges.push_back(CodeRange{cd, cat, cat + per_code_curves[(size_t)cd]});
                cat += per_code_curves[(size_t)cd];
            }
        }
        c->h_curve_list.assign((size_t)n, 0);
        for (int64_t i = 0; i < n; ++i) c->h_curve_list[(size_t)(curve_base[(size_t)code_of[(size_t)i]]++)] = (int)i;
        CHECK(upload(c->curve_list, c->h_curve_list.data(), (size_t)n, c->stream));
        DBuf<int64_t> d_dst;
        struct Release {
            DBuf<int64_t>& b;
            ~Release() { b.release(); }
        } release_dst{d_dst};
        CHECK(upload(d_dst, dst.data(), dst.size(), c->stream));
        CHECK(c->seg_list.reserve((size_t)c->n_seg));
        const int blocks = (int)std::min<int64_t>((c->n_seg + 255) / 256, (int64_t)sm_count() * 32);
        k_group_segments<<<blocks, 256, 0, c->stream>>>(batch_view(c), d_dst.p, c->seg_list.p);
        CU(cudaGetLastError());
        c->stats.n_launches++;
        CU(cudaStreamSynchronize(c->stream));
    }
    CU(cudaStreamSynchronize(c->stream));
    c->stats.n_curves = c->n_curve;
    c->stats.n_segments = c->n_seg;
    return GCV_OK;
}

gcv_status new_ctx(gcv_ctx** out, int n_curve, const gcv_options* opt, gcv_ctx** made)
{
    if (!out) return fail(GCV_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_curve < 0) return fail(GCV_ERR_INVALID, "n_curve < 0");
    gcv_options o;
    gcv_default_options(&o, opt ? opt->precision : GCV_PLAIN_FP64);
    if (opt) o = *opt;
    CHECK(check_options(&o));
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(GCV_ERR_NO_DEVICE, "no CUDA device is available");
    gcv_ctx* c = new gcv_ctx();
    c->opt = o;
    c->stream = (cudaStream_t)o.stream;
    c->n_curve = n_curve;
    *made = c;
    return GCV_OK;
}

template <typename T>
gcv_status to_host(const T* src, size_t n, int where, std::vector<T>& dst)
{
    dst.resize(n);
    if (!n) return GCV_OK;
    if (where == GCV_HOST)
        std::memcpy(dst.data(), src, n * sizeof(T));
    else
        CU(cudaMemcpy(dst.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost));
    return GCV_OK;
}

// ------------------------------------------------------------ table build

gcv_status ensure_table_buffers(gcv_ctx* c)
{
    const size_t ns = (size_t)std::max<int64_t>(c->n_seg, 1);
    // one copy of the coefficients: FP64, or float-float for the mixed path
    if (c->opt.precision == GCV_MIXED) {
        c->coef.release();
        CHECK(c->coef_ff.reserve((size_t)std::max<int64_t>(c->n_coef, 1)));
    } else {
        c->coef_ff.release();
        CHECK(c->coef.reserve((size_t)std::max<int64_t>(c->n_coef, 1)));
    }
    CHECK(c->seg_t0.reserve(ns));
    CHECK(c->seg_t1.reserve(ns));
    CHECK(c->seg_f0.reserve(ns));
    CHECK(c->seg_q0.reserve(ns));
    CHECK(c->seg_len.reserve(ns));
    CHECK(c->seg_cum.reserve(ns));
    CHECK(c->leaf_off.reserve(ns));
    CHECK(c->leaf_cnt.reserve(ns));
    CHECK(c->curve_len.reserve((size_t)std::max<int64_t>(c->n_curve, 1)));
    if (c->leaf_cap == 0) {
        // about three leaves per interval at the default tolerances; a pool
        // that turns out short sends the rest to the deep passes, which grow it
        c->leaf_cap = 3 * (int64_t)ns + 4096;
        CHECK(c->leaf_v.reserve((size_t)c->leaf_cap));
        CHECK(c->leaf_cum.reserve((size_t)c->leaf_cap));
        CHECK(c->leaf_f.reserve((size_t)c->leaf_cap));
        CHECK(c->leaf_q.reserve((size_t)c->leaf_cap));
    }
    if (c->deep_list.n == 0) CHECK(c->deep_list.reserve(ns / 16 + 1024));
    const size_t tiles = (ns + SCAN_TILE - 1) / SCAN_TILE;
    CHECK(c->scan_status.reserve(tiles));
    CHECK(c->scan_flag.reserve(tiles));
    CHECK(c->scan_hi.reserve(tiles));
    CHECK(c->scan_lo.reserve(tiles));
    return GCV_OK;
}

// grows the leaf pool to `cap`, keeping the first `keep` leaves
template <typename T>
gcv_status grow_buf(gcv_ctx* c, DBuf<T>& b, int64_t cap, int64_t keep)
{
    DBuf<T> nb;
    CHECK(nb.reserve((size_t)cap));
    if (keep > 0) CU(cudaMemcpyAsync(nb.p, b.p, (size_t)keep * sizeof(T), cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    b.release();
    b = nb;
    nb.p = nullptr;
    nb.n = 0;
    return GCV_OK;
}

gcv_status grow_pool(gcv_ctx* c, int64_t cap, int64_t keep)
{
    CHECK(grow_buf(c, c->leaf_v, cap, keep));
    CHECK(grow_buf(c, c->leaf_cum, cap, keep));
    CHECK(grow_buf(c, c->leaf_f, cap, keep));
    CHECK(grow_buf(c, c->leaf_q, cap, keep));
    c->leaf_cap = cap;
    return GCV_OK;
}

gcv_status read_counters(gcv_ctx* c)
{
    CU(cudaMemcpyAsync(c->h_ctr, c->ctr.p, C_COUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return GCV_OK;
}

// k_length over P for one curve code: every code has a specialised main
// pass; the deep passes are specialised for the common uniform batches and
// dispatch per segment otherwise (their lists mix codes)
template <int MODE, int PREC>
gcv_status launch_length_code(gcv_ctx* c, int code, const LengthParams& P)
{
    const int sms = sm_count();
    cudaError_t e = cudaErrorInvalidValue;
    if constexpr (MODE == 0) {
        const int cap = c->knobs.length_cap[code_slot(code)];
        const bool half_warp = PREC == 1 && c->opt.mapping == GCV_MAP_HALF_WARP;
        switch (code) {
#define GCV_CASE(C)                                                                                \
    case C:                                                                                        \
        e = half_warp ? length_launch_hw<C>(P, c->stream, sms, cap) : length_launch<0, C, PREC>(P, c->stream, sms, cap); \
        break;
            GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
        default: return fail(GCV_ERR_INVALID, "no length kernel for curve code " + std::to_string(code));
        }
    } else {
        const int cap = c->knobs.deep_cap;
        switch (code) {
        case CODE_ELLIPSE: e = length_launch<MODE, CODE_ELLIPSE, PREC>(P, c->stream, sms, cap); break;
        case bs_code(3, 2): e = length_launch<MODE, bs_code(3, 2), PREC>(P, c->stream, sms, cap); break;
        case bs_code(3, 3): e = length_launch<MODE, bs_code(3, 3), PREC>(P, c->stream, sms, cap); break;
        default: e = length_launch<MODE, -1, PREC>(P, c->stream, sms, cap); break;
        }
    }
    if (e != cudaSuccess) return cuda_fail(e, "length kernel launch");
    c->stats.n_launches++;
    return GCV_OK;
}

template <int MODE>
gcv_status launch_length(gcv_ctx* c, int code, const LengthParams& P)
{
    return c->opt.precision == GCV_MIXED ? launch_length_code<MODE, 1>(c, code, P)
                                         : launch_length_code<MODE, 0>(c, code, P);
}

// Main pass: one launch over all segments of a uniform batch, or one launch
// per curve code over that code's range of the grouped segment list; each
// code's launch is bracketed by its pair of timing events (as external event
// nodes under stream capture), which the autotuner reads.
gcv_status launch_main_pass(gcv_ctx* c, LengthParams P, bool capture = false)
{
    auto mark = [&](int code, int which) -> gcv_status {
        cudaEvent_t e = c->ev_code[code_slot(code)][which];
        CU(capture ? cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal) : cudaEventRecord(e, c->stream));
        c->code_timed[code_slot(code)] = true;
        return GCV_OK;
    };
    for (bool& x : c->code_timed) x = false;
    // work items in the order of the coefficient table and the learned
    // start depths (segment order for one code, the grouped list otherwise)
    P.by_item = 1;
    if (c->code >= 0) {
        P.list = nullptr;
        P.n_items = c->n_seg;
        P.work = c->ctr.p + C_WORK;
        P.coef_base = 0;
        CHECK(mark(c->code, 0));
        CHECK(launch_length<0>(c, c->code, P));
        return mark(c->code, 1);
    }
    const uint32_t* starts = P.starts;
    for (size_t k = 0; k < c->code_ranges.size(); ++k) {
        const CodeRange& r = c->code_ranges[k];
        if (r.end == r.begin) continue;
        P.list = c->seg_list.p + r.begin;
        P.n_items = r.end - r.begin;
        P.coef_base = r.coef_base;
        P.starts = starts ? starts + r.begin : nullptr;
        P.work = c->ctr.p + C_WORK_CODE + k;
        CHECK(mark(r.code, 0));
        CHECK(launch_length<0>(c, r.code, P));
        CHECK(mark(r.code, 1));
    }
    return GCV_OK;
}

// ---------------------------------------------------------- autotuner
TuneKey tune_key_of(gcv_ctx* c)
{
    int lg = 0;
    for (int64_t n = c->n_seg; n > 1; n >>= 1) ++lg;
    return TuneKey{c->code, c->opt.precision, c->opt.learned && c->mlp_w ? 1 : 0, lg};
}

// launch shapes for the next table build / sampling of this context
void select_knobs(gcv_ctx* c)
{
    const TuneKey key = tune_key_of(c);
    if (c->tune_key < key || key < c->tune_key) {  // a new shape: start over
        c->tune_key = key;
        c->len_trial = c->smp_trial = 0;
    }
    {
        std::lock_guard<std::mutex> g(g_tune_m);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            c->knobs = it->second;
            c->len_trial = c->smp_trial = -1;
            return;
        }
    }
    if (c->len_trial >= 0 && c->len_trial < TUNE_TRIALS) {
        const Knobs k = trial_knobs(c->len_trial);
        std::memcpy(c->knobs.length_cap, k.length_cap, sizeof(k.length_cap));
        c->knobs.deep_cap = k.deep_cap;
    }
    if (c->smp_trial >= 0 && c->smp_trial < TUNE_TRIALS) {
        const Knobs k = trial_knobs(c->smp_trial);
        c->knobs.sample_threads = k.sample_threads;
        c->knobs.sample_blocks_per_sm = k.sample_blocks_per_sm;
    }
}

int argmin3(const double* v)
{
    int b = 0;
    for (int i = 1; i < TUNE_TRIALS; ++i)
        if (v[i] < v[b]) b = i;
    return b;
}

// the length shapes of finished trials: each code its fastest trial, the
// deep passes the trial with the fastest length phase as a whole
void choose_length_knobs(gcv_ctx* c, Knobs& k)
{
    const int all = argmin3(c->len_ms);
    for (int sl = 0; sl < N_CODE_SLOTS; ++sl) {
        double v[TUNE_TRIALS];
        bool timed = true;
        for (int i = 0; i < TUNE_TRIALS; ++i) {
            v[i] = c->len_code_ms[i][sl];
            timed = timed && v[i] > 0.0;
        }
        k.length_cap[sl] = trial_length_cap(timed ? argmin3(v) : all);
    }
    k.deep_cap = trial_length_cap(all);
}

void tune_finish_if_done(gcv_ctx* c)
{
    if (c->len_trial == TUNE_TRIALS && c->smp_trial == TUNE_TRIALS) {
        Knobs k;
        choose_length_knobs(c, k);
        const Knobs ks = trial_knobs(argmin3(c->smp_ms));
        k.sample_threads = ks.sample_threads;
        k.sample_blocks_per_sm = ks.sample_blocks_per_sm;
        std::lock_guard<std::mutex> g(g_tune_m);
        g_tuned[c->tune_key] = k;
        c->knobs = k;
        c->len_trial = c->smp_trial = -1;
    }
}

// record the length passes' time (events ev[6] -> ev[2]) of a tuning build
gcv_status tune_after_table(gcv_ctx* c)
{
    if (c->len_trial < 0 || c->len_trial >= TUNE_TRIALS) return GCV_OK;
    CU(cudaEventSynchronize(c->ev[2]));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, c->ev[6], c->ev[2]));
    for (int sl = 0; sl < N_CODE_SLOTS; ++sl) {
        float mc = 0.f;
        c->len_code_ms[c->len_trial][sl] = 0.0;
        if (c->code_timed[sl] && cudaEventElapsedTime(&mc, c->ev_code[sl][0], c->ev_code[sl][1]) == cudaSuccess)
            c->len_code_ms[c->len_trial][sl] = std::max(mc, 1e-6f);
    }
    cudaGetLastError();
    c->len_ms[c->len_trial++] = ms;
    if (c->len_trial == TUNE_TRIALS && c->smp_trial >= 0 && c->smp_trial < TUNE_TRIALS) choose_length_knobs(c, c->knobs);
    tune_finish_if_done(c);
    return GCV_OK;
}

// record the sampling time (ev[4] -> ev[5]) of a tuning sampling call
gcv_status tune_after_sampling(gcv_ctx* c)
{
    if (c->smp_trial < 0 || c->smp_trial >= TUNE_TRIALS) return GCV_OK;
    CU(cudaEventSynchronize(c->ev[5]));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]));
    c->smp_ms[c->smp_trial++] = ms;
    tune_finish_if_done(c);
    return GCV_OK;
}

// feat16: the learned form's feature rows in grouped-list order (NULL otherwise)
gcv_status launch_setup_list(gcv_ctx* c, const CodeRange& r, uint4* feat16)
{
    const int64_t n = r.end - r.begin;
    if (n <= 0) return GCV_OK;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 64));
    const Batch b = batch_view(c);
    const Table t = table_view(c);
    const int* list = c->seg_list.p + r.begin;
    uint4* f16 = feat16 && r.code != CODE_ELLIPSE ? feat16 + 2 * r.begin : nullptr;
    const float rf = rtol_feature(c->opt.rtol);
    switch (r.code) {
#define GCV_CASE(C)                                                                                \
    case C: k_setup_list<C><<<blocks, 256, 0, c->stream>>>(b, t, list, n, f16, rf); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: return fail(GCV_ERR_INVALID, "no set-up kernel for curve code " + std::to_string(r.code));
    }
    CU(cudaGetLastError());
    c->stats.n_launches++;
    return GCV_OK;
}

gcv_status build_table(gcv_ctx* c)
{
    select_knobs(c);
    CHECK(ensure_table_buffers(c));
    const bool mixed = c->opt.precision == GCV_MIXED;
    const Batch b = batch_view(c);
    const int setup_blocks = (int)std::max<int64_t>(1, std::min<int64_t>((c->n_seg + 255) / 256, (int64_t)sm_count() * 64));
    const bool learned = c->opt.learned && c->mlp_w && c->n_seg > 0;
    // the learned form's set-up also writes each B-spline interval's features
    const bool with_features = learned && c->code != CODE_ELLIPSE;
    if (with_features) CHECK(c->feat16.reserve((size_t)c->n_seg * 2));
    uint4* feat16 = with_features ? c->feat16.p : nullptr;
    CU(cudaEventRecord(c->ev[0], c->stream));
    CU(cudaMemsetAsync(c->ctr.p, 0, C_COUNT * sizeof(unsigned long long), c->stream));
    if (c->n_seg > 0 && c->code >= 0) {
        k_setup<<<setup_blocks, 256, 0, c->stream>>>(b, table_view(c), feat16, rtol_feature(c->opt.rtol));
        CU(cudaGetLastError());
        c->stats.n_launches++;
    } else if (c->n_seg > 0) {
        for (const CodeRange& r : c->code_ranges) CHECK(launch_setup_list(c, r, feat16));
    }
    CU(cudaEventRecord(c->ev[1], c->stream));
    if (learned) {
        // start depths of every B-spline interval from the network (ellipse pieces keep 0)
        CHECK(c->starts.reserve((size_t)c->n_seg));
        CU(cudaMemsetAsync(c->starts.p, 0, (size_t)c->n_seg * sizeof(uint32_t), c->stream));
        const int md = mixed ? std::min(c->opt.max_depth, 44) : c->opt.max_depth;
        // start depths in the order of the work items (the grouped list)
        auto run = [&](const uint4* f16, uint32_t* starts, int64_t n) -> gcv_status {
            cudaError_t e = mlp_starts_launch_bf16(f16, nullptr, n, c->mlp_w, md, starts, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "network inference");
            c->stats.n_launches++;
            return GCV_OK;
        };
        if (c->code > 0) {
            CHECK(run(c->feat16.p, c->starts.p, c->n_seg));
        } else if (c->code < 0) {
            for (const CodeRange& r : c->code_ranges)
                if (r.code != CODE_ELLIPSE)
                    CHECK(run(c->feat16.p + 2 * r.begin, c->starts.p + r.begin, r.end - r.begin));
        }
    }
    CU(cudaEventRecord(c->ev[6], c->stream));
    for (int attempt = 0;; ++attempt) {
        if (attempt > 8) return fail(GCV_ERR_OVERFLOW, "deep list kept overflowing");
        // keep the set-up's error bits, clear the rest
        CU(cudaMemsetAsync(c->ctr.p, 0, C_ERR * sizeof(unsigned long long), c->stream));
        CU(cudaMemsetAsync(c->ctr.p + C_WORK_CODE, 0, (C_COUNT - C_WORK_CODE) * sizeof(unsigned long long), c->stream));
        LengthParams P{};
        P.b = b;
        P.t = table_view(c);
        P.rtol = c->opt.rtol;
        // float-float panel bounds are exact to depth 44
        P.max_depth = mixed ? std::min(c->opt.max_depth, 44) : c->opt.max_depth;
        P.collect = c->opt.collect_stats;
        P.list = nullptr;
        P.n_items = 0;
        P.coef_ff = c->coef_ff.p;
        P.work = c->ctr.p + C_WORK;
        P.starts = learned ? c->starts.p : nullptr;
        if (c->n_seg > 0) CHECK(launch_main_pass(c, P));
        CHECK(read_counters(c));
        const unsigned long long err = c->h_ctr[C_ERR];
        if (err & ERR_BAD_KNOTS) return fail(GCV_ERR_INVALID, "knot vector decreases or holds NaN");
        if (err & ERR_DEEP_LIST) {
            DBuf<int>& dl = c->deep_list;
            const size_t need = (size_t)(c->h_ctr[C_DEEP] * 1.25) + 1024;
            dl.release();
            CHECK(dl.reserve(need));
            CU(cudaMemsetAsync(c->ctr.p + C_ERR, 0, sizeof(unsigned long long), c->stream));
            continue;
        }
        const int64_t n_deep = (int64_t)c->h_ctr[C_DEEP];
        // Intervals whose leaves did not fit the pool went to the deep list;
        // what was reserved past the pool's end holds nothing.
        int64_t top = std::min<int64_t>((int64_t)c->h_ctr[C_LEAF_TOP], c->leaf_cap);
        if (n_deep > 0) {
            unsigned long long top_u = (unsigned long long)top;
            CU(cudaMemcpyAsync(c->ctr.p + C_LEAF_TOP, &top_u, sizeof(top_u), cudaMemcpyHostToDevice, c->stream));
            // count pass, then the leaves of the whole list summed on the device
            CU(cudaMemsetAsync(c->ctr.p + C_WORK, 0, sizeof(unsigned long long), c->stream));
            CU(cudaMemsetAsync(c->ctr.p + C_DEEP_LEAVES, 0, sizeof(unsigned long long), c->stream));
            LengthParams Q = P;
            Q.t = table_view(c);
            Q.list = c->deep_list.p;
            Q.n_items = n_deep;
            Q.collect = 0;
            Q.starts = nullptr;
            Q.work = c->ctr.p + C_WORK;
            CHECK(launch_length<1>(c, c->code, Q));
            const int rb = (int)std::min<int64_t>((n_deep + 255) / 256, (int64_t)sm_count() * 8);
            k_deep_total<<<rb, 256, 0, c->stream>>>(c->deep_list.p, n_deep, c->leaf_cnt.p, c->ctr.p + C_DEEP_LEAVES);
            CU(cudaGetLastError());
            c->stats.n_launches++;
            CHECK(read_counters(c));
            const int64_t extra = (int64_t)c->h_ctr[C_DEEP_LEAVES];
            if (top + extra > c->leaf_cap) CHECK(grow_pool(c, top + extra + (top + extra) / 16 + 4096, top));
            CU(cudaMemsetAsync(c->ctr.p + C_WORK, 0, sizeof(unsigned long long), c->stream));
            Q.t = table_view(c);
            Q.collect = P.collect;
            CHECK(launch_length<2>(c, c->code, Q));
            CHECK(read_counters(c));
            if (c->h_ctr[C_ERR] & ERR_POOL) return fail(GCV_ERR_OVERFLOW, "leaf pool overflow in the deep pass");
            top = (int64_t)c->h_ctr[C_LEAF_TOP];
        }
        c->stats.n_leaves = top;
        c->stats.n_deep_segments = n_deep;
        c->stats.n_panels = (int64_t)c->h_ctr[C_PANELS];
        c->stats.n_capped = (int64_t)c->h_ctr[C_CAPPED];
        break;
    }
    CU(cudaEventRecord(c->ev[2], c->stream));
    const int64_t tiles = (c->n_seg + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles > 0) {
        CU(cudaMemsetAsync(c->scan_status.p, 0, (size_t)tiles * sizeof(int), c->stream));
        CU(cudaMemsetAsync(c->ctr.p + C_SCAN_TILE, 0, sizeof(unsigned long long), c->stream));
        k_scan<<<(unsigned)tiles, SCAN_THREADS, 0, c->stream>>>(b, table_view(c), tiles);
        CU(cudaGetLastError());
        c->stats.n_launches++;
    }
    if (c->n_curve > 0) {
        k_curve_len<<<(unsigned)std::min<int64_t>((c->n_curve + 255) / 256, 65535), 256, 0, c->stream>>>(b, table_view(c));
        CU(cudaGetLastError());
        c->stats.n_launches++;
    }
    CU(cudaEventRecord(c->ev[3], c->stream));
    c->ev_table = true;
    if (learned) {
        unsigned err = 0;
        CU(cudaMemcpyAsync(&err, (uint8_t*)c->mlp_w + mlp_dev_bytes(), sizeof(err), cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        if (err) return fail(GCV_ERR_TIMEOUT, "network inference: a tensor-core wait gave up");
    }
    c->learned_ran = learned;
    CHECK(tune_after_table(c));
    return GCV_OK;
}

// ---------------------------------------------------------------- sampling

gcv_status launch_sampler(gcv_ctx* c, int code, const SampleParams& P, int64_t n)
{
    const int th = c->knobs.sample_threads;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + th - 1) / th,
                                                               (int64_t)sm_count() * c->knobs.sample_blocks_per_sm));
    const bool mixed = c->opt.precision == GCV_MIXED;
    const float2* cf = c->coef_ff.p;
    cudaError_t e = cudaErrorInvalidValue;
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: e = mixed ? sample_launch<C, 1>(P, cf, c->stream, grid, th) : sample_launch<C, 0>(P, cf, c->stream, grid, th); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: return fail(GCV_ERR_INVALID, "no sampling kernel for curve code " + std::to_string(code));
    }
    if (e != cudaSuccess) return cuda_fail(e, "sampling kernel launch");
    c->stats.n_launches++;
    return GCV_OK;
}

// sampling launches for the curves [c_lo, c_hi): one launch over their sample
// range (uniform batch), or one per curve code over the part of that code's
// grouped list (ascending curve ids) inside the range
gcv_status launch_sample_chunk(gcv_ctx* c, SampleParams P, int64_t c_lo, int64_t c_hi, const std::vector<int64_t>& lo)
{
    if (c->code >= 0) {
        P.curve_list = nullptr;
        P.s_begin = c->h_sample_off[(size_t)c_lo];
        P.s_end = c->h_sample_off[(size_t)c_hi];
        if (P.s_end > P.s_begin) CHECK(launch_sampler(c, c->code, P, P.s_end - P.s_begin));
        return GCV_OK;
    }
    P.curve_list = c->curve_list.p;
    P.list_off = c->list_sample_off.p;
    const int* L = c->h_curve_list.data();
    for (const CodeRange& r : c->curve_ranges) {
        const int64_t jb = std::lower_bound(L + r.begin, L + r.end, (int)c_lo) - L;
        const int64_t je = std::lower_bound(L + r.begin, L + r.end, (int)c_hi) - L;
        const int64_t ns = lo[(size_t)je] - lo[(size_t)jb];
        if (ns == 0) continue;
        P.cb = jb;
        P.ce = je;
        CHECK(launch_sampler(c, r.code, P, ns));
    }
    return GCV_OK;
}

gcv_status ensure_copy_streams(gcv_ctx* c)
{
    if (!c->s_in) CU(cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking));
    if (!c->s_out) CU(cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking));
    for (int k = 0; k < STREAM_EVENTS; ++k) {
        if (!c->ev_in[k]) CU(cudaEventCreateWithFlags(&c->ev_in[k], cudaEventDisableTiming));
        if (!c->ev_done[k]) CU(cudaEventCreateWithFlags(&c->ev_done[k], cudaEventDisableTiming));
        if (!c->ev_out[k]) CU(cudaEventCreateWithFlags(&c->ev_out[k], cudaEventDisableTiming));
    }
    return GCV_OK;
}

// Whether host memory at p is page-locked (cudaMallocHost, cudaHostAlloc or
// cudaHostRegister): the copy engines then move it directly, at the link
// rate and asynchronously to the host.
bool host_pinned(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The address under which the GPU reads and writes page-locked host memory
// at p directly (over the CPU-GPU link, without copies), or NULL when p is
// not page-locked and mapped.
void* host_mapped(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.hostPointer != p) return nullptr;
    return a.devicePointer;
}

// Samples into d_out from positions d_pos.  Host buffers (h_pos, h_out,
// either may be NULL) are streamed in chunks of curves: while chunk k is
// sampled, the copy engines bring in the positions of chunk k + 1 and take
// out the results of chunk k - 1.  Page-locked caller buffers are copied
// directly; pageable ones go through pinned staging buffers that a pool of
// host threads fills and drains.
gcv_status run_sampling(gcv_ctx* c, const int64_t* d_sample_off, double* d_pos, int64_t total, int is_relative,
                        int what, double* d_out, const double* h_pos = nullptr, double* h_out = nullptr)
{
    if (total == 0) return GCV_OK;
    const int width = what == GCV_RETURN_US ? 1 : c->point_dim;
    CU(cudaEventRecord(c->ev[4], c->stream));
    if (c->opt.collect_stats) CU(cudaMemsetAsync(c->ctr.p + C_NEWTON, 0, sizeof(unsigned long long), c->stream));
    SampleParams P{};
    P.b = batch_view(c);
    P.t = table_view(c);
    P.sample_off = d_sample_off;
    P.pos = d_pos;
    P.is_relative = is_relative;
    P.what = what;
    P.pdim = c->point_dim;
    P.out = d_out;
    P.n_samples = total;
    P.collect = c->opt.collect_stats;
    P.rtol = c->opt.rtol;
    P.eps_frac = (float)(SAMPLE_EPS_FRAC * c->opt.rtol);
    P.curve_list = nullptr;
    P.list_off = nullptr;
    P.cb = P.ce = 0;
    P.s_begin = 0;
    P.s_end = total;
    const int64_t n = c->n_curve;
    std::vector<int64_t> lo;
    if (c->code < 0) {
        // sample-count prefix in grouped-list order
        lo.assign((size_t)n + 1, 0);
        for (int64_t j = 0; j < n; ++j) {
            const int cj = c->h_curve_list[(size_t)j];
            lo[(size_t)j + 1] = lo[(size_t)j] + (c->h_sample_off[(size_t)cj + 1] - c->h_sample_off[(size_t)cj]);
        }
        CHECK(upload(c->list_sample_off, lo.data(), lo.size(), c->stream));
    }
    const int width_bytes = width * (int)sizeof(double);
    if (!h_pos && !h_out) {
        CHECK(launch_sample_chunk(c, P, 0, n, lo));
    } else if ((int64_t)total * width_bytes <= (int64_t)STAGE_CHUNK) {
        // one chunk's worth: plain copies around the kernels
        if (h_pos) CU(cudaMemcpyAsync(d_pos, h_pos, (size_t)total * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CHECK(launch_sample_chunk(c, P, 0, n, lo));
        if (h_out)
            CU(cudaMemcpyAsync(h_out, d_out, (size_t)total * width_bytes, cudaMemcpyDeviceToHost, c->stream));
    } else {
        // chunks of whole curves of about STAGE_CHUNK bytes of positions
        const int64_t per = (int64_t)(STAGE_CHUNK / sizeof(double));
        std::vector<int64_t> cut{0};
        while (cut.back() < n) {
            const int64_t want = c->h_sample_off[(size_t)cut.back()] + per;
            int64_t ci = std::upper_bound(c->h_sample_off.begin(), c->h_sample_off.end(), want) - c->h_sample_off.begin() - 1;
            ci = std::min<int64_t>(std::max<int64_t>(ci, cut.back() + 1), n);
            cut.push_back(ci);
        }
        const int chunks = (int)cut.size() - 1;
        int64_t max_s = 0;
        for (int k = 0; k < chunks; ++k)
            max_s = std::max<int64_t>(max_s, c->h_sample_off[(size_t)cut[(size_t)k + 1]] - c->h_sample_off[(size_t)cut[(size_t)k]]);
        CHECK(ensure_copy_streams(c));
        // page-locked caller buffers are copied directly: no staging, no host copies
        const bool pin_in = h_pos && host_pinned(h_pos), pin_out = h_out && host_pinned(h_out);
        std::unique_lock<std::mutex> lock;
        void* slot[STAGE_SLOTS] = {};
        if ((h_pos && !pin_in) || (h_out && !pin_out)) {
            lock = staging_lock();
            for (int i = 0; i < STAGE_SLOTS; ++i) {
                if (i < 2 ? !h_pos || pin_in : !h_out || pin_out) continue;
                const size_t bytes = (size_t)std::max<int64_t>(max_s, 1) * sizeof(double) * (i < 2 ? 1 : width);
                cudaError_t e = staging_slot(i, bytes, &slot[i]);
                if (e != cudaSuccess) return cuda_fail(e, "pinned staging buffer");
            }
        }
        auto s_of = [&](int k) { return c->h_sample_off[(size_t)cut[(size_t)k]]; };
        auto drain = [&](int k) -> gcv_status {  // results of chunk k -> caller (staged output only)
            CU(cudaEventSynchronize(c->ev_out[k % STREAM_EVENTS]));
            host_copy(h_out + s_of(k) * width, slot[2 + k % 2], (size_t)(s_of(k + 1) - s_of(k)) * width * sizeof(double));
            return GCV_OK;
        };
        for (int k = 0; k < chunks; ++k) {
            const int64_t s0 = s_of(k), s1 = s_of(k + 1);
            const int e = k % STREAM_EVENTS;
            if (h_pos && s1 > s0) {
                const double* src = h_pos + s0;
                if (!pin_in) {
                    if (k >= 2) CU(cudaEventSynchronize(c->ev_in[(k - 2) % STREAM_EVENTS]));  // buffer k % 2 is free
                    host_copy(slot[k % 2], h_pos + s0, (size_t)(s1 - s0) * sizeof(double));
                    src = (const double*)slot[k % 2];
                }
                CU(cudaMemcpyAsync(d_pos + s0, src, (size_t)(s1 - s0) * sizeof(double), cudaMemcpyHostToDevice, c->s_in));
                CU(cudaEventRecord(c->ev_in[e], c->s_in));
                CU(cudaStreamWaitEvent(c->stream, c->ev_in[e], 0));
            }
            CHECK(launch_sample_chunk(c, P, cut[(size_t)k], cut[(size_t)k + 1], lo));
            CU(cudaEventRecord(c->ev_done[e], c->stream));
            if (h_out) {
                // a staging buffer 2 + k % 2 was drained on the host before this point
                CU(cudaStreamWaitEvent(c->s_out, c->ev_done[e], 0));
                double* dst = pin_out ? h_out + s0 * width : (double*)slot[2 + k % 2];
                CU(cudaMemcpyAsync(dst, d_out + s0 * width, (size_t)(s1 - s0) * width * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->s_out));
                CU(cudaEventRecord(c->ev_out[e], c->s_out));
                if (k >= 1 && !pin_out) CHECK(drain(k - 1));
            }
        }
        if (h_out && !pin_out) {
            CHECK(drain(chunks - 1));
        } else if (h_out) {
            CU(cudaStreamSynchronize(c->s_out));
        } else {
            CU(cudaStreamSynchronize(c->s_in));
        }
    }
    CU(cudaEventRecord(c->ev[5], c->stream));
    c->ev_sample = true;
    c->stats.n_samples = total;
    CHECK(tune_after_sampling(c));
    return GCV_OK;
}

// ---------------------------------------------------------- graph step
// The table build and the sampling without host synchronisation, for stream
// capture (the phase events are recorded as external event nodes, so that
// the replays time the phases like the ordinary calls): the deep passes read their item count on the device, the sample
// offsets are scanned on the device, the sampling launches read their ranges
// on the device.  Pools keep the sizes an ordinary build gave them; an
// overflow is reported through the error word after the replay.
gcv_status enqueue_table_graph(gcv_ctx* c)
{
    const bool mixed = c->opt.precision == GCV_MIXED;
    const Batch b = batch_view(c);
    const bool learned = c->opt.learned && c->mlp_w && c->n_seg > 0;
    // feat16 is reserved before the capture (gcv_step_graph)
    uint4* feat16 = learned && c->code != CODE_ELLIPSE ? c->feat16.p : nullptr;
    CU(cudaEventRecordWithFlags(c->ev[0], c->stream, cudaEventRecordExternal));
    CU(cudaMemsetAsync(c->ctr.p, 0, C_COUNT * sizeof(unsigned long long), c->stream));
    if (c->n_seg > 0 && c->code >= 0) {
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((c->n_seg + 255) / 256, (int64_t)sm_count() * 64));
        k_setup<<<blocks, 256, 0, c->stream>>>(b, table_view(c), feat16, rtol_feature(c->opt.rtol));
        CU(cudaGetLastError());
    } else if (c->n_seg > 0) {
        for (const CodeRange& r : c->code_ranges) CHECK(launch_setup_list(c, r, feat16));
    }
    CU(cudaEventRecordWithFlags(c->ev[1], c->stream, cudaEventRecordExternal));
    if (learned) {
        CU(cudaMemsetAsync(c->starts.p, 0, (size_t)c->n_seg * sizeof(uint32_t), c->stream));
        const int md = mixed ? std::min(c->opt.max_depth, 44) : c->opt.max_depth;
        // start depths in the order of the work items (the grouped list)
        auto run = [&](const uint4* f16, uint32_t* starts, int64_t n) -> gcv_status {
            cudaError_t e = mlp_starts_launch_bf16(f16, nullptr, n, c->mlp_w, md, starts, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "network inference");
            return GCV_OK;
        };
        if (c->code > 0) {
            CHECK(run(c->feat16.p, c->starts.p, c->n_seg));
        } else if (c->code < 0) {
            for (const CodeRange& r : c->code_ranges)
                if (r.code != CODE_ELLIPSE)
                    CHECK(run(c->feat16.p + 2 * r.begin, c->starts.p + r.begin, r.end - r.begin));
        }
    }
    CU(cudaEventRecordWithFlags(c->ev[6], c->stream, cudaEventRecordExternal));
    if (c->n_seg > 0) {
        LengthParams P{};
        P.b = b;
        P.t = table_view(c);
        P.rtol = c->opt.rtol;
        P.max_depth = mixed ? std::min(c->opt.max_depth, 44) : c->opt.max_depth;
        P.collect = c->opt.collect_stats;
        P.coef_ff = c->coef_ff.p;
        P.starts = learned ? c->starts.p : nullptr;
        CHECK(launch_main_pass(c, P, true));
        // deep passes over the deep list, its length read on the device
        LengthParams Q = P;
        Q.list = c->deep_list.p;
        Q.n_items = (int64_t)c->deep_list.n;
        Q.n_items_dev = c->ctr.p + C_DEEP;
        Q.work = c->ctr.p + C_WORK;
        Q.starts = nullptr;
        Q.collect = 0;
        CU(cudaMemsetAsync(c->ctr.p + C_WORK, 0, sizeof(unsigned long long), c->stream));
        CHECK(launch_length<1>(c, c->code, Q));
        Q.collect = P.collect;
        CU(cudaMemsetAsync(c->ctr.p + C_WORK, 0, sizeof(unsigned long long), c->stream));
        CHECK(launch_length<2>(c, c->code, Q));
    }
    CU(cudaEventRecordWithFlags(c->ev[2], c->stream, cudaEventRecordExternal));
    const int64_t tiles = (c->n_seg + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles > 0) {
        CU(cudaMemsetAsync(c->scan_status.p, 0, (size_t)tiles * sizeof(int), c->stream));
        k_scan<<<(unsigned)tiles, SCAN_THREADS, 0, c->stream>>>(b, table_view(c), tiles);
        CU(cudaGetLastError());
    }
    if (c->n_curve > 0) {
        k_curve_len<<<(unsigned)std::min<int64_t>((c->n_curve + 255) / 256, 65535), 256, 0, c->stream>>>(b, table_view(c));
        CU(cudaGetLastError());
    }
    CU(cudaEventRecordWithFlags(c->ev[3], c->stream, cudaEventRecordExternal));
    return GCV_OK;
}

// exclusive prefix of the counts (gathered through idx when set) into out[0..n]
gcv_status enqueue_count_scan(gcv_ctx* c, const int* counts, const int* idx, int64_t* out)
{
    const int64_t n = c->n_curve;
    if (n == 0) return GCV_OK;
    const int64_t nb = (n + 1023) / 1024;
    k_count_block_sums<<<(unsigned)nb, 1024, 0, c->stream>>>(counts, idx, n, c->scan_blk.p, c->ctr.p + C_ERR);
    k_count_scan_blocks<<<1, 32, 0, c->stream>>>(c->scan_blk.p, nb);
    k_count_scan<<<(unsigned)nb, 1024, 0, c->stream>>>(counts, idx, n, c->scan_blk.p, out);
    CU(cudaGetLastError());
    return GCV_OK;
}

gcv_status enqueue_sampling_graph(gcv_ctx* c, const int* d_counts, const double* d_pos, int is_relative, int what,
                                  double* d_out)
{
    CU(cudaEventRecordWithFlags(c->ev[4], c->stream, cudaEventRecordExternal));
    if (c->n_curve == 0) {
        CU(cudaEventRecordWithFlags(c->ev[5], c->stream, cudaEventRecordExternal));
        return GCV_OK;
    }
    CHECK(enqueue_count_scan(c, d_counts, nullptr, c->sample_off.p));
    SampleParams P{};
    P.b = batch_view(c);
    P.t = table_view(c);
    P.sample_off = c->sample_off.p;
    P.pos = d_pos;
    P.is_relative = is_relative;
    P.what = what;
    P.pdim = c->point_dim;
    P.out = d_out;
    P.collect = c->opt.collect_stats;
    P.rtol = c->opt.rtol;
    P.eps_frac = (float)(SAMPLE_EPS_FRAC * c->opt.rtol);
    // grids for any sample count: the kernels loop over their ranges
    const int64_t nominal = (int64_t)sm_count() * c->knobs.sample_blocks_per_sm * c->knobs.sample_threads;
    if (c->code >= 0) {
        P.s_begin = 0;
        P.s_end_dev = c->sample_off.p + c->n_curve;
        CHECK(launch_sampler(c, c->code, P, nominal));
    } else {
        CHECK(enqueue_count_scan(c, d_counts, c->curve_list.p, c->list_sample_off.p));
        P.curve_list = c->curve_list.p;
        P.list_off = c->list_sample_off.p;
        for (const CodeRange& r : c->curve_ranges) {
            P.cb = r.begin;
            P.ce = r.end;
            CHECK(launch_sampler(c, r.code, P, nominal));
        }
    }
    CU(cudaEventRecordWithFlags(c->ev[5], c->stream, cudaEventRecordExternal));
    return GCV_OK;
}

void drop_graph(gcv_ctx* c)
{
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
}

gcv_status stage_counts(gcv_ctx* c, const int* n_ptrs, int in_where, int64_t* total)
{
    const int64_t n = c->n_curve;
    std::vector<int> cnt;
    CHECK(to_host(n_ptrs, (size_t)n, in_where, cnt));
    std::vector<int64_t>& off = c->h_sample_off;
    off.assign((size_t)n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (cnt[(size_t)i] < 0) return fail(GCV_ERR_INVALID, "negative sample count");
        off[(size_t)i + 1] = off[(size_t)i] + cnt[(size_t)i];
    }
    *total = off[(size_t)n];
    CHECK(upload(c->sample_off, off.data(), off.size(), c->stream));
    return GCV_OK;
}

// FP32 data: widened to double on the way in, rounded to float on the way out
__global__ void k_widen(const float* in, double* out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}
__global__ void k_narrow(const double* in, float* out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}
unsigned convert_grid(int64_t n)
{
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 32));
}

std::vector<double> widen_host(const float* p, size_t n)
{
    std::vector<double> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = (double)p[i];
    return v;
}

}  // namespace

// ===================================================================== ABI

extern "C" {

const char* gcv_status_string(gcv_status s)
{
    switch (s) {
    case GCV_OK: return "ok";
    case GCV_ERR_INVALID: return "invalid argument";
    case GCV_ERR_CUDA: return "CUDA error";
    case GCV_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GCV_ERR_STATE: return "invalid state";
    case GCV_ERR_OVERFLOW: return "device structure overflow";
    case GCV_ERR_TIMEOUT: return "bounded device wait timed out";
    case GCV_ERR_NO_DEVICE: return "no usable CUDA device";
    }
    return "unknown status";
}

const char* gcv_last_error(void) { return g_err.c_str(); }

// Sets the calling thread's gcv_last_error() message (used by the other
// translation units of the library; not part of the public header).
__attribute__((visibility("hidden"))) gcv_status gcv_internal_fail(gcv_status s, const char* msg)
{
    return fail(s, msg);
}

int gcv_version(void) { return 100; }

gcv_status gcv_default_options(gcv_options* opt, int precision)
{
    if (!opt) return fail(GCV_ERR_INVALID, "opt is NULL");
    std::memset(opt, 0, sizeof(*opt));
    opt->precision = precision;
    opt->rtol = precision == GCV_MIXED ? 1e-8 : 1e-10;
    opt->max_depth = 30;
    opt->stream = nullptr;
    opt->collect_stats = 0;
    return GCV_OK;
}

gcv_status gcv_create_batch(gcv_ctx** out, int n_curve, const uint8_t* kind, const uint8_t* degree, const uint8_t* dim,
                            const int64_t* knot_off, const double* knots, const int64_t* ctrl_off, const double* ctrl,
                            int where, const gcv_options* opt)
{
    gcv_ctx* c = nullptr;
    CHECK(new_ctx(out, n_curve, opt, &c));
    if (where != GCV_HOST && where != GCV_DEVICE) {
        destroy_ctx(c);
        return fail(GCV_ERR_INVALID, "where must be GCV_HOST or GCV_DEVICE");
    }
    if (n_curve > 0 && (!kind || !degree || !dim || !knot_off || !ctrl_off)) {
        destroy_ctx(c);
        return fail(GCV_ERR_INVALID, "NULL curve array");
    }
    std::vector<uint8_t> hk, hd, hm;
    std::vector<int64_t> hko, hco;
    gcv_status st;
    if ((st = to_host(kind, (size_t)n_curve, where, hk)) != GCV_OK ||
        (st = to_host(degree, (size_t)n_curve, where, hd)) != GCV_OK ||
        (st = to_host(dim, (size_t)n_curve, where, hm)) != GCV_OK ||
        (st = to_host(knot_off, (size_t)n_curve + 1, where, hko)) != GCV_OK ||
        (st = to_host(ctrl_off, (size_t)n_curve + 1, where, hco)) != GCV_OK) {
        destroy_ctx(c);
        return st;
    }
    if (n_curve == 0) {
        hko.assign(1, 0);
        hco.assign(1, 0);
    }
    const int64_t nk = hko[(size_t)n_curve], nc = hco[(size_t)n_curve];
    if ((nk > 0 && !knots) || (nc > 0 && !ctrl)) {
        destroy_ctx(c);
        return fail(GCV_ERR_INVALID, "NULL knots or control array");
    }
    // page-locked knot and control arrays read in place (opt.host_in_place)
    void* in_knots = where == GCV_HOST && c->opt.host_in_place && nk > 0 ? host_mapped(knots) : nullptr;
    void* in_ctrl = where == GCV_HOST && c->opt.host_in_place && nc > 0 ? host_mapped(ctrl) : nullptr;
    if (in_knots) c->knots.borrow((const double*)in_knots, (size_t)nk);
    if (in_ctrl) c->ctrl.borrow((const double*)in_ctrl, (size_t)nc);
    if (where == GCV_HOST) {
        // The knots and control points (nearly all of the bytes) go first, on
        // their own copy stream: from page-locked arrays the copy engines move
        // them while this thread derives the layout and groups the curves;
        // the create call still returns only once they have arrived.
        if ((st = ensure_copy_streams(c)) != GCV_OK ||
            (!in_knots && (st = upload(c->knots, knots, (size_t)nk, c->s_in)) != GCV_OK) ||
            (!in_ctrl && (st = upload(c->ctrl, ctrl, (size_t)nc, c->s_in)) != GCV_OK) ||
            (st = upload(c->kind, hk.data(), hk.size(), c->stream)) != GCV_OK ||
            (st = upload(c->degree, hd.data(), hd.size(), c->stream)) != GCV_OK ||
            (st = upload(c->dim, hm.data(), hm.size(), c->stream)) != GCV_OK ||
            (st = upload(c->knot_off, hko.data(), hko.size(), c->stream)) != GCV_OK ||
            (st = upload(c->ctrl_off, hco.data(), hco.size(), c->stream)) != GCV_OK) {
            if (c->s_in) cudaStreamSynchronize(c->s_in);
            destroy_ctx(c);
            return st;
        }
    } else {
        c->kind.borrow(kind, (size_t)n_curve);
        c->degree.borrow(degree, (size_t)n_curve);
        c->dim.borrow(dim, (size_t)n_curve);
        c->knot_off.borrow(knot_off, (size_t)n_curve + 1);
        c->ctrl_off.borrow(ctrl_off, (size_t)n_curve + 1);
        c->knots.borrow(knots, (size_t)nk);
        c->ctrl.borrow(ctrl, (size_t)nc);
    }
    st = finish_create(c, hk.data(), hd.data(), hm.data(), hko.data(), hco.data(), nullptr);
    if (where == GCV_HOST) {
        const cudaError_t e = cudaStreamSynchronize(c->s_in);
        if (st == GCV_OK && e != cudaSuccess) st = cuda_fail(e, "curve data upload");
    }
    if (st != GCV_OK) {
        destroy_ctx(c);
        return st;
    }
    *out = c;
    return GCV_OK;
}

gcv_status gcv_create_bsplines(gcv_ctx** out, int n_curve, int degree, int dim, const int* knots_offset,
                               const double* knot_vector, const double* ctrl_pts, int where, const gcv_options* opt)
{
    if (!out) return fail(GCV_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_curve < 0) return fail(GCV_ERR_INVALID, "n_curve < 0");
    if (degree < 1 || degree > MAX_DEGREE) return fail(GCV_ERR_INVALID, "degree must be in [1, 5]");
    if (dim != 2 && dim != 3) return fail(GCV_ERR_INVALID, "dim must be 2 or 3");
    if (!knots_offset) return fail(GCV_ERR_INVALID, "knots_offset is NULL");
    std::vector<int> ko;
    CHECK(to_host(knots_offset, (size_t)n_curve + 1, where == GCV_DEVICE ? GCV_DEVICE : GCV_HOST, ko));
    std::vector<uint8_t> k((size_t)n_curve, GCV_KIND_BSPLINE), dg((size_t)n_curve, (uint8_t)degree),
        dm((size_t)n_curve, (uint8_t)dim);
    std::vector<int64_t> knot_off((size_t)n_curve + 1), ctrl_off((size_t)n_curve + 1);
    for (int i = 0; i <= n_curve; ++i) {
        knot_off[(size_t)i] = ko[(size_t)i];
        // the sample's layout: curve c's control points start at knots_offset[c] - (degree + 1) c
        ctrl_off[(size_t)i] = ((int64_t)ko[(size_t)i] - (int64_t)(degree + 1) * i) * dim;
    }
    if (where == GCV_DEVICE) {
        // metadata is small: copy it, but keep the caller's knots and control points
        gcv_ctx* c = nullptr;
        CHECK(new_ctx(out, n_curve, opt, &c));
        gcv_status st;
        if ((st = upload(c->kind, k.data(), k.size(), c->stream)) != GCV_OK ||
            (st = upload(c->degree, dg.data(), dg.size(), c->stream)) != GCV_OK ||
            (st = upload(c->dim, dm.data(), dm.size(), c->stream)) != GCV_OK ||
            (st = upload(c->knot_off, knot_off.data(), knot_off.size(), c->stream)) != GCV_OK ||
            (st = upload(c->ctrl_off, ctrl_off.data(), ctrl_off.size(), c->stream)) != GCV_OK) {
            destroy_ctx(c);
            return st;
        }
        c->knots.borrow(knot_vector, (size_t)knot_off.back());
        c->ctrl.borrow(ctrl_pts, (size_t)ctrl_off.back());
        if ((st = finish_create(c, k.data(), dg.data(), dm.data(), knot_off.data(), ctrl_off.data(), nullptr)) != GCV_OK) {
            destroy_ctx(c);
            return st;
        }
        *out = c;
        return GCV_OK;
    }
    return gcv_create_batch(out, n_curve, k.data(), dg.data(), dm.data(), knot_off.data(), knot_vector, ctrl_off.data(),
                            ctrl_pts, GCV_HOST, opt);
}

gcv_status gcv_create_ellipses(gcv_ctx** out, int n_curve, const double* a, const double* b, const double* rot,
                               const double* cx, const double* cy, int where, const gcv_options* opt)
{
    if (!out) return fail(GCV_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_curve < 0) return fail(GCV_ERR_INVALID, "n_curve < 0");
    if (n_curve > 0 && (!a || !b)) return fail(GCV_ERR_INVALID, "a or b is NULL");
    const int w = where == GCV_DEVICE ? GCV_DEVICE : GCV_HOST;
    std::vector<double> ha, hb, hr, hx, hy;
    CHECK(to_host(a, (size_t)n_curve, w, ha));
    CHECK(to_host(b, (size_t)n_curve, w, hb));
    if (rot) CHECK(to_host(rot, (size_t)n_curve, w, hr));
    if (cx) CHECK(to_host(cx, (size_t)n_curve, w, hx));
    if (cy) CHECK(to_host(cy, (size_t)n_curve, w, hy));
    std::vector<uint8_t> k((size_t)n_curve, GCV_KIND_ELLIPSE), dg((size_t)n_curve, 0), dm((size_t)n_curve, 2);
    std::vector<int64_t> ko((size_t)n_curve + 1), co((size_t)n_curve + 1);
    std::vector<double> knots((size_t)n_curve * 2), ctrl((size_t)n_curve * 5);
    for (int i = 0; i < n_curve; ++i) {
        ko[(size_t)i] = 2 * (int64_t)i;
        co[(size_t)i] = 5 * (int64_t)i;
        knots[2 * (size_t)i] = 0.0;
        knots[2 * (size_t)i + 1] = 2.0 * PI;
        ctrl[5 * (size_t)i + 0] = ha[(size_t)i];
        ctrl[5 * (size_t)i + 1] = hb[(size_t)i];
        ctrl[5 * (size_t)i + 2] = rot ? hr[(size_t)i] : 0.0;
        ctrl[5 * (size_t)i + 3] = cx ? hx[(size_t)i] : 0.0;
        ctrl[5 * (size_t)i + 4] = cy ? hy[(size_t)i] : 0.0;
    }
    ko[(size_t)n_curve] = 2 * (int64_t)n_curve;
    co[(size_t)n_curve] = 5 * (int64_t)n_curve;
    return gcv_create_batch(out, n_curve, k.data(), dg.data(), dm.data(), ko.data(), knots.data(), co.data(), ctrl.data(),
                            GCV_HOST, opt);
}

gcv_status gcv_destroy(gcv_ctx* ctx)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    else cudaDeviceSynchronize();
    destroy_ctx(ctx);
    return GCV_OK;
}

gcv_status gcv_set_options(gcv_ctx* ctx, const gcv_options* opt)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    CHECK(check_options(opt));
    const bool rebuild = opt->precision != ctx->opt.precision || opt->rtol != ctx->opt.rtol ||
                         opt->max_depth != ctx->opt.max_depth || opt->mapping != ctx->opt.mapping;
    ctx->opt = *opt;
    ctx->stream = (cudaStream_t)opt->stream;
    if (rebuild) {
        ctx->table_ready = false;
        ctx->h_len_valid = false;
    }
    return GCV_OK;
}

gcv_status gcv_create_arclength_table(gcv_ctx* ctx)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    ctx->table_ready = false;
    ctx->h_len_valid = false;
    CHECK(build_table(ctx));
    ctx->table_ready = true;
    return GCV_OK;
}

gcv_status gcv_get_all_curve_arclengths(gcv_ctx* ctx, double* out, int where)
{
    if (!ctx || !out) return fail(GCV_ERR_INVALID, "NULL argument");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (ctx->n_curve == 0) return GCV_OK;
    const size_t bytes = (size_t)ctx->n_curve * sizeof(double);
    if (where == GCV_DEVICE) {
        CU(cudaMemcpyAsync(out, ctx->curve_len.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        CU(cudaMemcpyAsync(out, ctx->curve_len.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
    }
    return GCV_OK;
}

gcv_status gcv_get_arclength(gcv_ctx* ctx, int cid, double* out)
{
    if (!ctx || !out) return fail(GCV_ERR_INVALID, "NULL argument");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (cid < 0 || cid >= ctx->n_curve) return fail(GCV_ERR_INVALID, "cid out of range");
    if (!ctx->h_len_valid) {
        ctx->h_len.resize((size_t)ctx->n_curve);
        CHECK(gcv_get_all_curve_arclengths(ctx, ctx->h_len.data(), GCV_HOST));
        ctx->h_len_valid = true;
    }
    *out = ctx->h_len[(size_t)cid];
    return GCV_OK;
}

gcv_status gcv_clear_arclength(gcv_ctx* ctx)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    ctx->h_len.clear();
    ctx->h_len.shrink_to_fit();
    ctx->h_len_valid = false;
    return GCV_OK;
}

gcv_status gcv_arclength_reverse_into(gcv_ctx* ctx, const int* n_ptrs_for_curves, const double* sample_position,
                                      int is_relative, int in_where, int what, double* out, int out_where)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (what != GCV_RETURN_US && what != GCV_RETURN_POINTS) return fail(GCV_ERR_INVALID, "what must be RETURN_US or RETURN_POINTS");
    if (in_where != GCV_HOST && in_where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "bad in_where");
    if (out_where != GCV_HOST && out_where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "bad out_where");
    if (ctx->n_curve > 0 && !n_ptrs_for_curves) return fail(GCV_ERR_INVALID, "n_ptrs_for_curves is NULL");
    int64_t total = 0;
    CHECK(stage_counts(ctx, n_ptrs_for_curves, in_where, &total));
    if (total == 0) return GCV_OK;
    if (!sample_position || !out) return fail(GCV_ERR_INVALID, "NULL positions or output");
    // Page-locked host buffers are read and written by the sampling kernels
    // in place (each position and result crosses the link once, in the
    // kernels' own accesses); pageable ones are streamed through device
    // buffers in chunks, overlapped with the sampling kernels.
    const int width = what == GCV_RETURN_US ? 1 : ctx->point_dim;
    const double* h_pos = in_where == GCV_HOST ? sample_position : nullptr;
    double* h_out = out_where == GCV_HOST ? out : nullptr;
    double* d_pos = const_cast<double*>(sample_position);
    if (h_pos) {
        if (void* m = host_mapped(h_pos)) {
            d_pos = (double*)m;
            h_pos = nullptr;
        } else {
            CHECK(ctx->sample_pos.reserve((size_t)total));
            d_pos = ctx->sample_pos.p;
        }
    }
    double* d_out = out;
    if (h_out) {
        if (void* m = host_mapped(h_out)) {
            d_out = (double*)m;
            h_out = nullptr;
        } else {
            CHECK(ctx->sample_out.reserve((size_t)total * width));
            d_out = ctx->sample_out.p;
        }
    }
    CHECK(run_sampling(ctx, ctx->sample_off.p, d_pos, total, is_relative ? 1 : 0, what, d_out, h_pos, h_out));
    if (out_where == GCV_HOST) CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_arclength_reverse(gcv_ctx* ctx, const int* n_ptrs_for_curves, const double* sample_position,
                                 int is_relative, int where, int what, gcv_result* result)
{
    if (!ctx || !result) return fail(GCV_ERR_INVALID, "NULL argument");
    std::memset(result, 0, sizeof(*result));
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (where != GCV_HOST && where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "where must be GCV_HOST or GCV_DEVICE");
    if (what != GCV_RETURN_US && what != GCV_RETURN_POINTS) return fail(GCV_ERR_INVALID, "what must be RETURN_US or RETURN_POINTS");
    if (ctx->n_curve > 0 && !n_ptrs_for_curves) return fail(GCV_ERR_INVALID, "n_ptrs_for_curves is NULL");
    int64_t total = 0;
    for (int64_t i = 0; i < ctx->n_curve; ++i) {
        if (n_ptrs_for_curves[i] < 0) return fail(GCV_ERR_INVALID, "negative sample count");
        total += n_ptrs_for_curves[i];
    }
    const int width = what == GCV_RETURN_US ? 1 : ctx->point_dim;
    result->n_points = total;
    result->store_where = where;
    result->store_what = what;
    result->point_dim = what == GCV_RETURN_US ? 1 : ctx->point_dim;
    const size_t bytes = (size_t)std::max<int64_t>(total, 1) * width * sizeof(double);
    if (where == GCV_DEVICE) {
        CU(cudaMalloc(&result->data, bytes));
    } else {
        result->data = (double*)std::malloc(bytes);
        if (!result->data) return fail(GCV_ERR_OUT_OF_MEMORY, "host result allocation failed");
    }
    gcv_status st = gcv_arclength_reverse_into(ctx, n_ptrs_for_curves, sample_position, is_relative, GCV_HOST, what,
                                               result->data, where);
    if (st != GCV_OK) {
        gcv_free_result(result);
        return st;
    }
    if (where == GCV_DEVICE) CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_free_result(gcv_result* r)
{
    if (!r) return fail(GCV_ERR_INVALID, "result is NULL");
    if (r->data) {
        if (r->store_where == GCV_DEVICE)
            cudaFree(r->data);
        else
            std::free(r->data);
    }
    r->data = nullptr;
    r->n_points = 0;
    return GCV_OK;
}

// ----------------------------------------------------------- FP32 data
gcv_status gcv_create_ellipses_f32(gcv_ctx** out, int n_curve, const float* a, const float* b, const float* rot,
                                   const float* cx, const float* cy, int where, const gcv_options* opt)
{
    if (!out) return fail(GCV_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_curve < 0) return fail(GCV_ERR_INVALID, "n_curve < 0");
    if (n_curve > 0 && (!a || !b)) return fail(GCV_ERR_INVALID, "a or b is NULL");
    const int w = where == GCV_DEVICE ? GCV_DEVICE : GCV_HOST;
    std::vector<float> f[5];
    const float* src[5] = {a, b, rot, cx, cy};
    std::vector<double> d[5];
    for (int k = 0; k < 5; ++k) {
        if (!src[k]) continue;
        CHECK(to_host(src[k], (size_t)n_curve, w, f[k]));
        d[k] = widen_host(f[k].data(), f[k].size());
    }
    auto ptr = [&](int k) { return src[k] ? d[k].data() : nullptr; };
    return gcv_create_ellipses(out, n_curve, ptr(0), ptr(1), ptr(2), ptr(3), ptr(4), GCV_HOST, opt);
}

gcv_status gcv_create_bsplines_f32(gcv_ctx** out, int n_curve, int degree, int dim, const int* knots_offset,
                                   const float* knot_vector, const float* ctrl_pts, int where, const gcv_options* opt)
{
    if (!out) return fail(GCV_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (n_curve < 0) return fail(GCV_ERR_INVALID, "n_curve < 0");
    if (degree < 1 || degree > MAX_DEGREE) return fail(GCV_ERR_INVALID, "degree must be in [1, 5]");
    if (dim != 2 && dim != 3) return fail(GCV_ERR_INVALID, "dim must be 2 or 3");
    if (!knots_offset) return fail(GCV_ERR_INVALID, "knots_offset is NULL");
    const int w = where == GCV_DEVICE ? GCV_DEVICE : GCV_HOST;
    std::vector<int> ko;
    CHECK(to_host(knots_offset, (size_t)n_curve + 1, w, ko));
    const int64_t nk = ko[(size_t)n_curve];
    const int64_t nc = ((int64_t)ko[(size_t)n_curve] - (int64_t)(degree + 1) * n_curve) * dim;
    if (nk < 0 || nc < 0) return fail(GCV_ERR_INVALID, "knots_offset too small for the degree");
    if ((nk > 0 && !knot_vector) || (nc > 0 && !ctrl_pts)) return fail(GCV_ERR_INVALID, "NULL knots or control points");
    if (w == GCV_HOST) {
        const std::vector<double> kv = widen_host(knot_vector, (size_t)nk), cp = widen_host(ctrl_pts, (size_t)nc);
        return gcv_create_bsplines(out, n_curve, degree, dim, knots_offset, kv.data(), cp.data(), GCV_HOST, opt);
    }
    // device data: widened into buffers the context then owns
    DBuf<double> kv, cp;
    gcv_status r = kv.reserve((size_t)nk);
    if (r == GCV_OK) r = cp.reserve((size_t)nc);
    if (r == GCV_OK) {
        cudaStream_t st = opt ? (cudaStream_t)opt->stream : nullptr;
        if (nk) k_widen<<<convert_grid(nk), 256, 0, st>>>(knot_vector, kv.p, nk);
        if (nc) k_widen<<<convert_grid(nc), 256, 0, st>>>(ctrl_pts, cp.p, nc);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = cuda_fail(e, "widening the FP32 curve data");
    }
    gcv_ctx* c = nullptr;
    if (r == GCV_OK) r = gcv_create_bsplines(&c, n_curve, degree, dim, knots_offset, kv.p, cp.p, GCV_DEVICE, opt);
    if (r != GCV_OK) {
        kv.release();
        cp.release();
        return r;
    }
    // hand the widened arrays to the context (it borrowed them)
    c->knots.owned = true;
    c->knots.bytes = kv.bytes;
    c->ctrl.owned = true;
    c->ctrl.bytes = cp.bytes;
    kv.p = nullptr;
    cp.p = nullptr;
    *out = c;
    return GCV_OK;
}

gcv_status gcv_get_all_curve_arclengths_f32(gcv_ctx* ctx, float* out, int where)
{
    if (!ctx || !out) return fail(GCV_ERR_INVALID, "NULL argument");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    const int64_t n = ctx->n_curve;
    if (n == 0) return GCV_OK;
    float* d = out;
    if (where != GCV_DEVICE) {
        CHECK(ctx->f32_buf.reserve((size_t)n));
        d = ctx->f32_buf.p;
    }
    k_narrow<<<convert_grid(n), 256, 0, ctx->stream>>>(ctx->curve_len.p, d, n);
    CU(cudaGetLastError());
    if (where != GCV_DEVICE) {
        CU(cudaMemcpyAsync(out, d, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
    }
    return GCV_OK;
}

gcv_status gcv_get_arclength_f32(gcv_ctx* ctx, int cid, float* out)
{
    if (!out) return fail(GCV_ERR_INVALID, "NULL argument");
    double v = 0.0;
    CHECK(gcv_get_arclength(ctx, cid, &v));
    *out = (float)v;
    return GCV_OK;
}

gcv_status gcv_arclength_reverse_into_f32(gcv_ctx* ctx, const int* n_ptrs_for_curves, const float* sample_position,
                                          int is_relative, int in_where, int what, float* out, int out_where)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (what != GCV_RETURN_US && what != GCV_RETURN_POINTS) return fail(GCV_ERR_INVALID, "what must be RETURN_US or RETURN_POINTS");
    if (in_where != GCV_HOST && in_where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "bad in_where");
    if (out_where != GCV_HOST && out_where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "bad out_where");
    if (ctx->n_curve > 0 && !n_ptrs_for_curves) return fail(GCV_ERR_INVALID, "n_ptrs_for_curves is NULL");
    int64_t total = 0;
    CHECK(stage_counts(ctx, n_ptrs_for_curves, in_where, &total));
    if (total == 0) return GCV_OK;
    if (!sample_position || !out) return fail(GCV_ERR_INVALID, "NULL positions or output");
    const int width = what == GCV_RETURN_US ? 1 : ctx->point_dim;
    const int64_t n_out = total * width;
    CHECK(ctx->sample_pos.reserve((size_t)total));
    CHECK(ctx->sample_out.reserve((size_t)n_out));
    const int64_t n_f = std::max<int64_t>(in_where == GCV_HOST ? total : 0, out_where == GCV_HOST ? n_out : 0);
    if (n_f) CHECK(ctx->f32_buf.reserve((size_t)n_f));
    const float* d_in = sample_position;
    if (in_where == GCV_HOST) {
        CU(cudaMemcpyAsync(ctx->f32_buf.p, sample_position, (size_t)total * sizeof(float), cudaMemcpyHostToDevice,
                           ctx->stream));
        d_in = ctx->f32_buf.p;
    }
    k_widen<<<convert_grid(total), 256, 0, ctx->stream>>>(d_in, ctx->sample_pos.p, total);
    CU(cudaGetLastError());
    CHECK(run_sampling(ctx, ctx->sample_off.p, ctx->sample_pos.p, total, is_relative ? 1 : 0, what, ctx->sample_out.p,
                       nullptr, nullptr));
    float* d_out = out_where == GCV_DEVICE ? out : ctx->f32_buf.p;
    k_narrow<<<convert_grid(n_out), 256, 0, ctx->stream>>>(ctx->sample_out.p, d_out, n_out);
    CU(cudaGetLastError());
    if (out_where == GCV_HOST) {
        CU(cudaMemcpyAsync(out, d_out, (size_t)n_out * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
    }
    return GCV_OK;
}

gcv_status gcv_arclength_reverse_f32(gcv_ctx* ctx, const int* n_ptrs_for_curves, const float* sample_position,
                                     int is_relative, int where, int what, gcv_result_f32* result)
{
    if (!ctx || !result) return fail(GCV_ERR_INVALID, "NULL argument");
    std::memset(result, 0, sizeof(*result));
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (where != GCV_HOST && where != GCV_DEVICE) return fail(GCV_ERR_INVALID, "where must be GCV_HOST or GCV_DEVICE");
    if (what != GCV_RETURN_US && what != GCV_RETURN_POINTS) return fail(GCV_ERR_INVALID, "what must be RETURN_US or RETURN_POINTS");
    if (ctx->n_curve > 0 && !n_ptrs_for_curves) return fail(GCV_ERR_INVALID, "n_ptrs_for_curves is NULL");
    int64_t total = 0;
    for (int64_t i = 0; i < ctx->n_curve; ++i) {
        if (n_ptrs_for_curves[i] < 0) return fail(GCV_ERR_INVALID, "negative sample count");
        total += n_ptrs_for_curves[i];
    }
    const int width = what == GCV_RETURN_US ? 1 : ctx->point_dim;
    result->n_points = total;
    result->store_where = where;
    result->store_what = what;
    result->point_dim = width;
    const size_t bytes = (size_t)std::max<int64_t>(total, 1) * width * sizeof(float);
    if (where == GCV_DEVICE) {
        CU(cudaMalloc(&result->data, bytes));
    } else {
        result->data = (float*)std::malloc(bytes);
        if (!result->data) return fail(GCV_ERR_OUT_OF_MEMORY, "host result allocation failed");
    }
    gcv_status st = gcv_arclength_reverse_into_f32(ctx, n_ptrs_for_curves, sample_position, is_relative, GCV_HOST,
                                                   what, result->data, where);
    if (st != GCV_OK) {
        gcv_free_result_f32(result);
        return st;
    }
    if (where == GCV_DEVICE) CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_free_result_f32(gcv_result_f32* r)
{
    if (!r) return fail(GCV_ERR_INVALID, "result is NULL");
    if (r->data) {
        if (r->store_where == GCV_DEVICE)
            cudaFree(r->data);
        else
            std::free(r->data);
    }
    r->data = nullptr;
    r->n_points = 0;
    return GCV_OK;
}

gcv_status gcv_synchronize(gcv_ctx* ctx)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_get_stats(gcv_ctx* ctx, gcv_stats* out)
{
    if (!ctx || !out) return fail(GCV_ERR_INVALID, "NULL argument");
    CU(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    if (ctx->ev_table) {
        if (cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]) == cudaSuccess) ctx->stats.ms_setup = ms;
        if (cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]) == cudaSuccess) ctx->stats.ms_length = ms;
        ctx->stats.ms_learned = 0.0;
        if (ctx->learned_ran && cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[6]) == cudaSuccess)
            ctx->stats.ms_learned = ms;
        if (cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]) == cudaSuccess) ctx->stats.ms_scan = ms;
    }
    if (ctx->ev_sample) {
        if (cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]) == cudaSuccess) ctx->stats.ms_sample = ms;
        if (ctx->opt.collect_stats) {
            CHECK(read_counters(ctx));
            ctx->stats.n_newton = (int64_t)ctx->h_ctr[C_NEWTON];
        }
    }
    cudaGetLastError();
    ctx->stats.length_blocks_per_sm = ctx->code >= 0 ? ctx->knobs.length_cap[code_slot(ctx->code)] : ctx->knobs.deep_cap;
    for (int sl = 0; sl < N_CODE_SLOTS; ++sl) ctx->stats.length_blocks_per_sm_code[sl] = ctx->knobs.length_cap[sl];
    ctx->stats.sample_threads = ctx->knobs.sample_threads;
    ctx->stats.sample_blocks_per_sm = ctx->knobs.sample_blocks_per_sm;
    ctx->stats.tuned = ctx->len_trial < 0 ? 1 : 0;
    *out = ctx->stats;
    return GCV_OK;
}

gcv_status gcv_host_alloc(size_t bytes, void** p)
{
    if (!p) return fail(GCV_ERR_INVALID, "p is NULL");
    *p = nullptr;
    if (bytes == 0) return GCV_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(GCV_ERR_NO_DEVICE, "no CUDA device is available");
    CU(cudaMallocHost(p, bytes));
    return GCV_OK;
}

gcv_status gcv_host_free(void* p)
{
    if (p) CU(cudaFreeHost(p));
    return GCV_OK;
}

gcv_status gcv_release_cached_memory(int64_t* bytes)
{
    const size_t n = release_cache(-1);
    if (bytes) *bytes = (int64_t)n;
    return GCV_OK;
}

gcv_status gcv_measure_fma_peak(int which, double* tflops)
{
    if (!tflops || (which != 0 && which != 1)) return fail(GCV_ERR_INVALID, "which must be 0 (FP64) or 1 (FP32)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(GCV_ERR_NO_DEVICE, "no CUDA device is available");
    }
    const int threads = 256, blocks = sm_count() * 8;
    const int iters = which == 0 ? 256 : 16384;
    void* out = nullptr;
    CU(cudaMalloc(&out, 16));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        CU(cudaEventRecord(e0));
        if (which == 0)
            k_fma_probe<double><<<blocks, threads>>>((double*)out, iters, 1.0);
        else
            k_fma_probe<float><<<blocks, threads>>>((float*)out, iters, 1.0f);
        CU(cudaGetLastError());
        CU(cudaEventRecord(e1));
        CU(cudaEventSynchronize(e1));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return GCV_OK;
}

gcv_status gcv_get_shape(gcv_ctx* ctx, int64_t* n_curve, int64_t* n_segments, int* point_dim)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (n_curve) *n_curve = ctx->n_curve;
    if (n_segments) *n_segments = ctx->n_seg;
    if (point_dim) *point_dim = ctx->point_dim;
    return GCV_OK;
}

gcv_status gcv_step_graph(gcv_ctx* ctx, const int* d_counts, const double* d_pos, int is_relative, int what,
                          double* d_out)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (what != GCV_RETURN_US && what != GCV_RETURN_POINTS) return fail(GCV_ERR_INVALID, "what must be RETURN_US or RETURN_POINTS");
    if (ctx->n_curve > 0 && (!d_counts || !d_pos || !d_out)) return fail(GCV_ERR_INVALID, "NULL device buffer");
    gcv_ctx* c = ctx;
    // an ordinary build first: it sizes the leaf pool and the deep list
    if (!c->table_ready) {
        CHECK(build_table(c));
        c->table_ready = true;
        c->h_len_valid = false;
    }
    select_knobs(c);
    const bool same = c->gexec && c->gknobs == c->knobs && c->gargs.counts == d_counts && c->gargs.pos == d_pos && c->gargs.out == d_out &&
                      c->gargs.is_relative == is_relative && c->gargs.what == what &&
                      c->gargs.learned == (c->opt.learned && c->mlp_w ? 1 : 0) &&
                      std::memcmp(&c->gargs.opt, &c->opt, sizeof(gcv_options)) == 0;
    if (!same) {
        drop_graph(c);
        CHECK(c->sample_off.reserve((size_t)c->n_curve + 1));
        CHECK(c->list_sample_off.reserve((size_t)c->n_curve + 1));
        CHECK(c->scan_blk.reserve((size_t)(c->n_curve + 1023) / 1024 + 1));
        if (c->opt.learned && c->mlp_w) {
            CHECK(c->starts.reserve((size_t)std::max<int64_t>(c->n_seg, 1)));
            if (c->code != CODE_ELLIPSE) CHECK(c->feat16.reserve((size_t)std::max<int64_t>(c->n_seg, 1) * 2));
        }
        if (!c->stream && !c->gstream) CU(cudaStreamCreateWithFlags(&c->gstream, cudaStreamNonBlocking));
        cudaStream_t user = c->stream;
        cudaStream_t cap = c->stream ? c->stream : c->gstream;
        CU(cudaStreamSynchronize(user));
        c->stream = cap;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        gcv_status st = e == cudaSuccess ? GCV_OK : cuda_fail(e, "cudaStreamBeginCapture");
        if (st == GCV_OK) st = enqueue_table_graph(c);
        if (st == GCV_OK) st = enqueue_sampling_graph(c, d_counts, d_pos, is_relative, what, d_out);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cap, &g);
        c->stream = user;
        if (st != GCV_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        c->graph = g;
        e = cudaGraphInstantiate(&c->gexec, g, 0);
        if (e != cudaSuccess) {
            drop_graph(c);
            return cuda_fail(e, "cudaGraphInstantiate");
        }
        c->gargs.counts = d_counts;
        c->gargs.pos = d_pos;
        c->gargs.out = d_out;
        c->gargs.is_relative = is_relative;
        c->gargs.what = what;
        c->gargs.learned = c->opt.learned && c->mlp_w ? 1 : 0;
        std::memcpy(&c->gargs.opt, &c->opt, sizeof(gcv_options));
        c->gknobs = c->knobs;
        // kernels per replay, for the launch count
        size_t nn = 0;
        c->graph_kernels = 0;
        if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
            std::vector<cudaGraphNode_t> nodes(nn);
            if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
                for (cudaGraphNode_t nd : nodes) {
                    cudaGraphNodeType ty;
                    if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) c->graph_kernels++;
                }
        }
    }
    CU(cudaGraphLaunch(c->gexec, c->stream));
    c->stats.n_launches += c->graph_kernels;
    CHECK(read_counters(c));
    unsigned long long err = c->h_ctr[C_ERR];
    if (c->gargs.learned) {
        unsigned werr = 0;
        CU(cudaMemcpy(&werr, (uint8_t*)c->mlp_w + mlp_dev_bytes(), sizeof(werr), cudaMemcpyDeviceToHost));
        if (werr) return fail(GCV_ERR_TIMEOUT, "network inference: a tensor-core wait gave up");
    }
    if (err & ERR_BAD_KNOTS) return fail(GCV_ERR_INVALID, "knot vector decreases or holds NaN");
    if (err & ERR_BAD_COUNT) return fail(GCV_ERR_INVALID, "negative sample count");
    if (err & ERR_SCAN_TIMEOUT) return fail(GCV_ERR_TIMEOUT, "scan look-back gave up");
    if (err & (ERR_POOL | ERR_DEEP_LIST)) {
        // the pools were too small for this data: the ordinary path grows them,
        // and the next call captures again
        drop_graph(c);
        CHECK(build_table(c));
        int64_t total = 0;
        CHECK(stage_counts(c, d_counts, GCV_DEVICE, &total));
        CHECK(run_sampling(c, c->sample_off.p, const_cast<double*>(d_pos), total, is_relative, what, d_out));
        CU(cudaStreamSynchronize(c->stream));
        c->h_len_valid = false;
        return GCV_OK;
    }
    c->ev_table = c->ev_sample = true;
    c->learned_ran = c->gargs.learned != 0;
    c->stats.n_leaves = (int64_t)c->h_ctr[C_LEAF_TOP];
    c->stats.n_deep_segments = (int64_t)c->h_ctr[C_DEEP];
    c->stats.n_panels = (int64_t)c->h_ctr[C_PANELS];
    c->stats.n_capped = (int64_t)c->h_ctr[C_CAPPED];
    c->stats.n_newton = (int64_t)c->h_ctr[C_NEWTON];
    c->h_len_valid = false;
    CHECK(tune_after_table(c));
    CHECK(tune_after_sampling(c));
    return GCV_OK;
}

gcv_status gcv_step_graph_reset(gcv_ctx* ctx)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    drop_graph(ctx);
    return GCV_OK;
}

gcv_status gcv_learned_features(gcv_ctx* ctx, float* d_features)
{
    if (!ctx || (!d_features && ctx->n_seg > 0)) return fail(GCV_ERR_INVALID, "NULL argument");
    if (ctx->n_seg == 0) return GCV_OK;
    const int blocks = (int)std::min<int64_t>((ctx->n_seg + 255) / 256, (int64_t)sm_count() * 32);
    k_features<<<blocks, 256, 0, ctx->stream>>>(batch_view(ctx), rtol_feature(ctx->opt.rtol), d_features);
    CU(cudaGetLastError());
    ctx->stats.n_launches++;
    CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_learned_labels(gcv_ctx* ctx, int* d_depth, float* d_share, float* d_tguess)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    if (!ctx->table_ready) return fail(GCV_ERR_STATE, "createArclengthTable has not run");
    if (ctx->learned_ran) return fail(GCV_ERR_STATE, "labels come from a table built by the plain walk");
    if (ctx->n_seg == 0) return GCV_OK;
    if (!d_depth || !d_share || !d_tguess) return fail(GCV_ERR_INVALID, "NULL label array");
    const int blocks = (int)std::min<int64_t>((ctx->n_seg + 255) / 256, (int64_t)sm_count() * 32);
    k_labels<<<blocks, 256, 0, ctx->stream>>>(table_view(ctx), ctx->n_seg, d_depth, d_share, d_tguess);
    CU(cudaGetLastError());
    ctx->stats.n_launches++;
    CU(cudaStreamSynchronize(ctx->stream));
    return GCV_OK;
}

gcv_status gcv_set_learned_model(gcv_ctx* ctx, const float* host_weights)
{
    if (!ctx) return fail(GCV_ERR_INVALID, "ctx is NULL");
    CU(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);  // a captured step holds the old weights
    if (ctx->mlp_w) {
        cudaFree(ctx->mlp_w);
        ctx->mlp_w = nullptr;
    }
    if (!host_weights) return GCV_OK;
    for (int i = 0; i < MLP_NPARAM; ++i)
        if (!std::isfinite(host_weights[i])) return fail(GCV_ERR_INVALID, "network weights hold NaN or infinity");
    void* w = nullptr;
    cudaError_t e = mlp_upload_bf16(host_weights, &w);
    if (e != cudaSuccess) {
        if (w) cudaFree(w);
        return cuda_fail(e, "network upload");
    }
    ctx->mlp_w = w;
    return GCV_OK;
}

}  // extern "C"
