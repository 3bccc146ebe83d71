// Bundle text files (the reference's B-spline dataset format,
// samples/sample2_bspline/dataset_loader.h:40-126) parsed and normalised on
// the GPU: gcv_bundle_parse / gcv_bundle_sizes / gcv_bundle_fill /
// gcv_bundle_destroy (include/gcurval_gb300_bundle.h).
//
// Pipeline, all on the caller's stream:
//   1. k_tok_count: 4 KiB of text per block (16 bytes per thread), count the
//      token starts (a non-blank byte after a blank one);
//   2. k_scan_counts: exclusive prefix of the block counts (one block);
//   3. k_tok_parse: the same 16-byte ranges again; a block scan of the
//      per-thread counts gives each token its index, and the thread that
//      owns a token's first byte converts it, correctly rounded
//      (gcv_decimal.cuh), into vals[index];
//   4. k_file_tok: the index of each file's first token;
//   5. k_records: one thread per file walks its records header to header
//      (each header says how many numbers follow), checks them, counts them
//      and, on a second launch, writes each curve's first-token index,
//      degree and point count;
//   6. k_curve_offsets: knot and coordinate offsets of the kept curves
//      (one block, a running block scan);
//   7. k_fill (gcv_bundle_fill): one warp per curve copies knots and points
//      into the caller's arrays, centring and scaling the points like the
//      reference loader (dataset_loader.h:77-103).
// The host waits twice (for the token count and for the record counts);
// everything else is asynchronous.
#include "gcurval_gb300_bundle.h"

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <string>
#include <vector>

#include "gcv_decimal.cuh"

extern "C" gcv_status gcv_internal_fail(gcv_status s, const char* msg);

struct gcv_bundle {
    cudaStream_t stream = nullptr;
    int dim = 2;
    int64_t n_curve = 0, n_knots = 0, n_ctrl = 0;
    double* vals = nullptr;      // every number of the text, in order
    int64_t* rec_tok = nullptr;  // per kept curve: index of its header's first number
    int* rec_p = nullptr;        // degree
    int* rec_nc = nullptr;       // control points
    int64_t* knot_off = nullptr;  // n_curve + 1
    int64_t* ctrl_off = nullptr;  // n_curve + 1
};

namespace {

constexpr int TOK_THREADS = 256;
constexpr int TOK_BYTES = 16;
constexpr int64_t TOK_CHUNK = (int64_t)TOK_THREADS * TOK_BYTES;
constexpr int SCAN_THREADS = 1024;

// the blanks std::istream skips (isspace in the C locale)
__device__ __forceinline__ bool is_blank(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

__device__ __forceinline__ bool is_start(const unsigned char* t, int64_t i)
{
    return !is_blank(t[i]) && (i == 0 || is_blank(t[i - 1]));
}

// token starts in bytes [i0, min(i0 + 16, n))
__device__ __forceinline__ int count_starts(const unsigned char* t, int64_t n, int64_t i0)
{
    int c = 0;
    const int64_t e = i0 + TOK_BYTES < n ? i0 + TOK_BYTES : n;
    for (int64_t i = i0; i < e; ++i) c += is_start(t, i);
    return c;
}

// exclusive scan of one int per thread over a TOK_THREADS block
__device__ int block_excl_scan(int x)
{
    __shared__ int w[TOK_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int v = x;
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
    }
    if (lane == 31) w[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int t = lane < TOK_THREADS / 32 ? w[lane] : 0;
        for (int d = 1; d < TOK_THREADS / 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        if (lane < TOK_THREADS / 32) w[lane] = t;
    }
    __syncthreads();
    return (wid ? w[wid - 1] : 0) + v - x;
}

__global__ void __launch_bounds__(TOK_THREADS) k_tok_count(const unsigned char* t, int64_t n, int* blk_cnt)
{
    const int64_t i0 = (int64_t)blockIdx.x * TOK_CHUNK + (int64_t)threadIdx.x * TOK_BYTES;
    int c = i0 < n ? count_starts(t, n, i0) : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ int w[TOK_THREADS / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int i = 0; i < TOK_THREADS / 32; ++i) s += w[i];
        blk_cnt[blockIdx.x] = s;
    }
}

// out[i] = in[0] + ... + in[i - 1] for i in [0, n]; one block
template <typename F>
__device__ void running_scan(int64_t n, F value, int64_t* out)
{
    __shared__ long long w[SCAN_THREADS / 32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t base = 0; base < n; base += SCAN_THREADS) {
        const int64_t i = base + threadIdx.x;
        const long long x = i < n ? value(i) : 0;
        long long v = x;
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, v, d);
            if (lane >= d) v += y;
        }
        if (lane == 31) w[wid] = v;
        __syncthreads();
        if (wid == 0) {
            long long t = w[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            w[lane] = t;
        }
        __syncthreads();
        const long long incl = (wid ? w[wid - 1] : 0) + v;
        const long long c0 = carry;
        if (i < n) out[i] = c0 + incl - x;
        __syncthreads();
        if (threadIdx.x == SCAN_THREADS - 1) carry = c0 + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_counts(const int* cnt, int64_t n, int64_t* off)
{
    running_scan(n, [&](int64_t i) { return (long long)cnt[i]; }, off);
}

__global__ void __launch_bounds__(TOK_THREADS) k_tok_parse(const unsigned char* t, int64_t n, const int64_t* blk_off,
                                                          double* vals, long long* bad_number)
{
    const int64_t i0 = (int64_t)blockIdx.x * TOK_CHUNK + (int64_t)threadIdx.x * TOK_BYTES;
    const int c = i0 < n ? count_starts(t, n, i0) : 0;
    int64_t k = blk_off[blockIdx.x] + block_excl_scan(c);
    if (c == 0) return;
    const int64_t e = i0 + TOK_BYTES < n ? i0 + TOK_BYTES : n;
    for (int64_t i = i0; i < e; ++i) {
        if (!is_start(t, i)) continue;
        int64_t j = i + 1;
        while (j < n && !is_blank(t[j])) ++j;
        double v = 0.0;
        if (!gcv::parse_decimal(t + i, t + j, &v)) atomicMin(bad_number, (long long)k);
        vals[k++] = v;
    }
}

// ftok[f]: index of the first token at or after byte file_off[f]
// (ftok[n_files] = the token count); a token that runs across a file
// boundary is reported in *bad_sep
__global__ void k_file_tok(const unsigned char* t, int64_t n, const int64_t* file_off, int n_files,
                           const int64_t* blk_off, int64_t* ftok, long long* bad_sep)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f > n_files) return;
    const int64_t o = file_off[f];
    if (o >= n) {
        ftok[f] = blk_off[(n + TOK_CHUNK - 1) / TOK_CHUNK];
        return;
    }
    const int64_t b = o / TOK_CHUNK;
    int64_t k = blk_off[b];
    for (int64_t i = b * TOK_CHUNK; i < o; ++i) k += is_start(t, i);
    ftok[f] = k;
    if (o > 0 && !is_blank(t[o - 1]) && !is_blank(t[o])) atomicMin(bad_sep, (long long)f);
}

__device__ __forceinline__ bool as_count(double v, long long lo, long long hi, long long* out)
{
    if (!(v >= (double)lo && v <= (double)hi)) return false;
    const long long i = (long long)v;
    if ((double)i != v) return false;
    *out = i;
    return true;
}

// WRITE false: curve records per file into fcount; WRITE true: the kept
// curves' header index, degree and point count, file f's curves numbered
// from fcoff[f]
template <bool WRITE>
__global__ void k_records(const double* vals, const int64_t* ftok, int n_files, int* fcount, const int64_t* fcoff,
                          int64_t n_keep, int64_t* rec_tok, int* rec_p, int* rec_nc, long long* bad_record)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_files) return;
    int64_t t = ftok[f];
    const int64_t e = ftok[f + 1];
    int64_t c = 0;
    const int64_t base = WRITE ? fcoff[f] : 0;
    while (t < e) {
        long long p = 0, nc = 0, nk = 0;
        const bool ok = t + 3 <= e && as_count(vals[t], 1, 255, &p) && as_count(vals[t + 1], 2, INT_MAX / 4, &nc) &&
                        as_count(vals[t + 2], 3, INT_MAX / 2, &nk) && nc >= p + 1 && nk == nc + p + 1 &&
                        t + 3 + 2 * nc + nk <= e;
        if (!ok) {
            atomicMin(bad_record, (long long)t);
            break;
        }
        if (WRITE) {
            const int64_t g = base + c;
            if (g >= n_keep) break;
            rec_tok[g] = t;
            rec_p[g] = (int)p;
            rec_nc[g] = (int)nc;
        }
        ++c;
        t += 3 + 2 * nc + nk;
    }
    if (!WRITE) fcount[f] = (int)c;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_curve_offsets(const int* rec_p, const int* rec_nc, int64_t n, int dim,
                                                               int64_t* knot_off, int64_t* ctrl_off)
{
    running_scan(n, [&](int64_t i) { return (long long)rec_nc[i] + rec_p[i] + 1; }, knot_off);
    __syncthreads();
    running_scan(n, [&](int64_t i) { return (long long)rec_nc[i] * dim; }, ctrl_off);
}

// one warp per curve
__global__ void k_fill(const double* vals, const int64_t* rec_tok, const int* rec_p, const int* rec_nc,
                       const int64_t* knot_off, const int64_t* ctrl_off, int64_t n, int dim, int normalize,
                       uint8_t* kind, uint8_t* degree, uint8_t* dimv, double* knots, double* ctrl)
{
    const int lane = threadIdx.x & 31;
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= n) return;  // warp-uniform
    const int64_t t = rec_tok[c];
    const int p = rec_p[c], nc = rec_nc[c], nk = nc + p + 1;
    const double* x = vals + t + 3;
    const double* y = x + nc;
    const double* kv = y + nc;
    double* kn = knots + knot_off[c];
    for (int i = lane; i < nk; i += 32) kn[i] = kv[i];
    if (lane == 0) {
        kind[c] = (uint8_t)GCV_KIND_BSPLINE;
        degree[c] = (uint8_t)p;
        dimv[c] = (uint8_t)dim;
    }
    double cx = 0.0, cy = 0.0, m = 0.0;
    if (normalize) {
        // the mean point: a sequential sum in point order, then / n_ctrl
        if (lane == 0) {
            double sx = x[0], sy = y[0];
            for (int i = 1; i < nc; ++i) {
                sx = __dadd_rn(sx, x[i]);
                sy = __dadd_rn(sy, y[i]);
            }
            cx = __ddiv_rn(sx, (double)nc);
            cy = __ddiv_rn(sy, (double)nc);
        }
        cx = __shfl_sync(0xffffffffu, cx, 0);
        cy = __shfl_sync(0xffffffffu, cy, 0);
        for (int i = lane; i < nc; i += 32)
            m = fmax(m, fmax(fabs(__dsub_rn(x[i], cx)), fabs(__dsub_rn(y[i], cy))));
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    double* q = ctrl + ctrl_off[c];
    for (int i = lane; i < nc; i += 32) {
        double a = x[i], b = y[i];
        if (normalize) {
            a = __dsub_rn(a, cx);
            b = __dsub_rn(b, cy);
            if (m > 0.0) {
                a = __ddiv_rn(a, m);
                b = __ddiv_rn(b, m);
            }
        }
        q[(int64_t)i * dim] = a;
        q[(int64_t)i * dim + 1] = b;
        if (dim == 3) q[(int64_t)i * dim + 2] = 0.0;
    }
}

gcv_status cuda_status(cudaError_t e, const char* what)
{
    cudaGetLastError();
    const gcv_status s = e == cudaErrorMemoryAllocation ? GCV_ERR_OUT_OF_MEMORY
                       : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
                           ? GCV_ERR_NO_DEVICE
                           : GCV_ERR_CUDA;
    return gcv_internal_fail(s, (std::string("bundle: ") + what + ": " + cudaGetErrorString(e)).c_str());
}

#define BCU(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return cuda_status(e_, #call);                                      \
    } while (0)

// device memory released when the scope ends
struct DMem {
    void* p = nullptr;
    DMem() = default;
    DMem(const DMem&) = delete;
    DMem& operator=(const DMem&) = delete;
    ~DMem()
    {
        if (p) cudaFree(p);
    }
    template <typename T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
};

void free_bundle(gcv_bundle* b)
{
    if (!b) return;
    if (b->stream || b->vals) cudaStreamSynchronize(b->stream);
    cudaFree(b->vals);
    cudaFree(b->rec_tok);
    cudaFree(b->rec_p);
    cudaFree(b->rec_nc);
    cudaFree(b->knot_off);
    cudaFree(b->ctrl_off);
    delete b;
}

struct BundleGuard {
    gcv_bundle* b;
    ~BundleGuard() { free_bundle(b); }
};

gcv_status parse_into(gcv_bundle* b, const char* text, int64_t n, const int64_t* file_off, int n_files,
                      int64_t max_curves, int where)
{
    cudaStream_t s = b->stream;
    DMem d_text_own, d_blk_cnt, d_blk_off, d_file_off, d_ftok, d_fcount, d_fcoff, d_err;
    const unsigned char* t = reinterpret_cast<const unsigned char*>(text);
    if (where == GCV_HOST && n > 0) {
        BCU(d_text_own.alloc((size_t)n));
        BCU(cudaMemcpyAsync(d_text_own.p, text, (size_t)n, cudaMemcpyHostToDevice, s));
        t = d_text_own.as<unsigned char>();
    }
    const int64_t nb = (n + TOK_CHUNK - 1) / TOK_CHUNK;
    BCU(d_blk_cnt.alloc(sizeof(int) * (size_t)nb));
    BCU(d_blk_off.alloc(sizeof(int64_t) * (size_t)(nb + 1)));
    BCU(d_file_off.alloc(sizeof(int64_t) * (size_t)(n_files + 1)));
    BCU(d_ftok.alloc(sizeof(int64_t) * (size_t)(n_files + 1)));
    BCU(d_fcount.alloc(sizeof(int) * (size_t)n_files));
    BCU(d_fcoff.alloc(sizeof(int64_t) * (size_t)n_files));
    BCU(d_err.alloc(sizeof(long long) * 3));
    std::vector<long long> err(3, LLONG_MAX);
    BCU(cudaMemcpyAsync(d_err.p, err.data(), sizeof(long long) * 3, cudaMemcpyHostToDevice, s));
    BCU(cudaMemcpyAsync(d_file_off.p, file_off, sizeof(int64_t) * (size_t)(n_files + 1), cudaMemcpyHostToDevice, s));
    long long* d_bad = d_err.as<long long>();

    if (nb > 0) {
        k_tok_count<<<(unsigned)nb, TOK_THREADS, 0, s>>>(t, n, d_blk_cnt.as<int>());
        BCU(cudaGetLastError());
    }
    k_scan_counts<<<1, SCAN_THREADS, 0, s>>>(d_blk_cnt.as<int>(), nb, d_blk_off.as<int64_t>());
    BCU(cudaGetLastError());
    int64_t n_tok = 0;
    BCU(cudaMemcpyAsync(&n_tok, d_blk_off.as<int64_t>() + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    BCU(cudaStreamSynchronize(s));

    BCU(cudaMalloc(&b->vals, sizeof(double) * (size_t)(n_tok > 0 ? n_tok : 1)));
    if (nb > 0) {
        k_tok_parse<<<(unsigned)nb, TOK_THREADS, 0, s>>>(t, n, d_blk_off.as<int64_t>(), b->vals, d_bad);
        BCU(cudaGetLastError());
    }
    k_file_tok<<<(unsigned)((n_files + 1 + 127) / 128), 128, 0, s>>>(t, n, d_file_off.as<int64_t>(), n_files,
                                                                     d_blk_off.as<int64_t>(), d_ftok.as<int64_t>(),
                                                                     d_bad + 2);
    BCU(cudaGetLastError());
    k_records<false><<<(unsigned)((n_files + 127) / 128), 128, 0, s>>>(b->vals, d_ftok.as<int64_t>(), n_files,
                                                                       d_fcount.as<int>(), nullptr, 0, nullptr,
                                                                       nullptr, nullptr, d_bad + 1);
    BCU(cudaGetLastError());
    std::vector<int64_t> ftok((size_t)n_files + 1);
    std::vector<int> fcount((size_t)n_files);
    BCU(cudaMemcpyAsync(err.data(), d_bad, sizeof(long long) * 3, cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(ftok.data(), d_ftok.p, sizeof(int64_t) * ftok.size(), cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(fcount.data(), d_fcount.p, sizeof(int) * fcount.size(), cudaMemcpyDeviceToHost, s));
    BCU(cudaStreamSynchronize(s));

    // first problem in text order: file and number index within the file
    auto where_is = [&](long long tok) {
        int f = 0;
        while (f + 1 < n_files && ftok[(size_t)f + 1] <= tok) ++f;
        return "file " + std::to_string(f) + ", number " + std::to_string(tok - ftok[(size_t)f]);
    };
    if (err[2] != LLONG_MAX)
        return gcv_internal_fail(GCV_ERR_INVALID, ("bundle: a number runs across the start of file " +
                                                   std::to_string(err[2]) + " (files need a blank between them)")
                                                      .c_str());
    if (err[0] != LLONG_MAX && err[0] <= err[1])
        return gcv_internal_fail(GCV_ERR_INVALID,
                                 ("bundle: " + where_is(err[0]) +
                                  ": not a decimal number with at most 19 significant digits, a significand below "
                                  "2^53 and a decimal exponent within +-22")
                                     .c_str());
    if (err[1] != LLONG_MAX)
        return gcv_internal_fail(GCV_ERR_INVALID,
                                 ("bundle: " + where_is(err[1]) +
                                  ": malformed curve record (degree n_ctrl n_knots with n_ctrl >= degree + 1, "
                                  "n_knots = n_ctrl + degree + 1, then 2 n_ctrl + n_knots numbers)")
                                     .c_str());

    std::vector<int64_t> fcoff((size_t)n_files);
    int64_t total = 0;
    for (int f = 0; f < n_files; ++f) {
        fcoff[(size_t)f] = total;
        total += fcount[(size_t)f];
    }
    const int64_t n_keep = max_curves < 0 ? total : (max_curves < total ? max_curves : total);
    b->n_curve = n_keep;
    BCU(cudaMalloc(&b->rec_tok, sizeof(int64_t) * (size_t)(n_keep > 0 ? n_keep : 1)));
    BCU(cudaMalloc(&b->rec_p, sizeof(int) * (size_t)(n_keep > 0 ? n_keep : 1)));
    BCU(cudaMalloc(&b->rec_nc, sizeof(int) * (size_t)(n_keep > 0 ? n_keep : 1)));
    BCU(cudaMalloc(&b->knot_off, sizeof(int64_t) * (size_t)(n_keep + 1)));
    BCU(cudaMalloc(&b->ctrl_off, sizeof(int64_t) * (size_t)(n_keep + 1)));
    BCU(cudaMemcpyAsync(d_fcoff.p, fcoff.data(), sizeof(int64_t) * fcoff.size(), cudaMemcpyHostToDevice, s));
    k_records<true><<<(unsigned)((n_files + 127) / 128), 128, 0, s>>>(b->vals, d_ftok.as<int64_t>(), n_files, nullptr,
                                                                      d_fcoff.as<int64_t>(), n_keep, b->rec_tok,
                                                                      b->rec_p, b->rec_nc, d_bad + 1);
    BCU(cudaGetLastError());
    k_curve_offsets<<<1, SCAN_THREADS, 0, s>>>(b->rec_p, b->rec_nc, n_keep, b->dim, b->knot_off, b->ctrl_off);
    BCU(cudaGetLastError());
    int64_t sizes[2] = {0, 0};
    BCU(cudaMemcpyAsync(&sizes[0], b->knot_off + n_keep, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(&sizes[1], b->ctrl_off + n_keep, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    BCU(cudaStreamSynchronize(s));
    b->n_knots = sizes[0];
    b->n_ctrl = sizes[1];
    return GCV_OK;
}

}  // namespace

extern "C" {

gcv_status gcv_bundle_parse(const char* text, int64_t n_bytes, const int64_t* file_off, int n_files,
                            int64_t max_curves, int dim, int where, void* stream, gcv_bundle** out)
{
    if (!out) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: out is NULL");
    *out = nullptr;
    if (n_bytes < 0 || (n_bytes > 0 && !text)) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: bad text");
    if (n_files < 1 || !file_off) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: need at least one file offset range");
    if (file_off[0] != 0 || file_off[n_files] != n_bytes)
        return gcv_internal_fail(GCV_ERR_INVALID, "bundle: file_off must run from 0 to n_bytes");
    for (int f = 0; f < n_files; ++f)
        if (file_off[f + 1] < file_off[f]) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: file_off must not decrease");
    if (dim != 2 && dim != 3) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: dim must be 2 or 3");
    if (where != GCV_HOST && where != GCV_DEVICE)
        return gcv_internal_fail(GCV_ERR_INVALID, "bundle: where must be GCV_HOST or GCV_DEVICE");
    BundleGuard g{new gcv_bundle{}};
    g.b->stream = static_cast<cudaStream_t>(stream);
    g.b->dim = dim;
    const gcv_status st = parse_into(g.b, text, n_bytes, file_off, n_files, max_curves, where);
    if (st != GCV_OK) return st;
    *out = g.b;
    g.b = nullptr;
    return GCV_OK;
}

gcv_status gcv_bundle_sizes(const gcv_bundle* b, int64_t* n_curve, int64_t* n_knots, int64_t* n_ctrl_values)
{
    if (!b) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: NULL handle");
    if (n_curve) *n_curve = b->n_curve;
    if (n_knots) *n_knots = b->n_knots;
    if (n_ctrl_values) *n_ctrl_values = b->n_ctrl;
    return GCV_OK;
}

gcv_status gcv_bundle_fill(const gcv_bundle* b, int normalize, uint8_t* d_kind, uint8_t* d_degree, uint8_t* d_dim,
                           int64_t* d_knot_off, double* d_knots, int64_t* d_ctrl_off, double* d_ctrl)
{
    if (!b) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: NULL handle");
    if (!d_knot_off || !d_ctrl_off) return gcv_internal_fail(GCV_ERR_INVALID, "bundle: NULL offset array");
    cudaStream_t s = b->stream;
    const int64_t n = b->n_curve;
    BCU(cudaMemcpyAsync(d_knot_off, b->knot_off, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyDeviceToDevice, s));
    BCU(cudaMemcpyAsync(d_ctrl_off, b->ctrl_off, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyDeviceToDevice, s));
    if (n == 0) return GCV_OK;
    if (!d_kind || !d_degree || !d_dim || !d_knots || !d_ctrl)
        return gcv_internal_fail(GCV_ERR_INVALID, "bundle: NULL output array");
    const int64_t blocks = (n * 32 + 255) / 256;
    k_fill<<<(unsigned)blocks, 256, 0, s>>>(b->vals, b->rec_tok, b->rec_p, b->rec_nc, b->knot_off, b->ctrl_off, n,
                                            b->dim, normalize, d_kind, d_degree, d_dim, d_knots, d_ctrl);
    BCU(cudaGetLastError());
    return GCV_OK;
}

void gcv_bundle_destroy(gcv_bundle* b) { free_bundle(b); }

}  // extern "C"
