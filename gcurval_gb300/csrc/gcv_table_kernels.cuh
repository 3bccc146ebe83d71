// Kernels that build the arc-length table around the length pass: the
// per-segment set-up, the segment -> curve map, the grouping of segments by
// curve code, the deep-list leaf total, the compensated scan and the curve
// totals.  Included by gcv_api.cu only.
#pragma once

#include "gcv_ff_eval.cuh"
#include "gcv_kernels.cuh"
#include "gcv_learned.cuh"

namespace gcv {

// set-up of one B-spline interval for a mixed-path table: float-float
// coefficients straight from the float-float recursion
template <int P, int D>
__device__ void setup_bspline_seg_ff(const Batch& b, const Table& t, int64_t s, int64_t c)
{
    constexpr int N = code_stride(bs_code(P, D));
    const int64_t j = s - b.seg_off[c];
    const double* kv = b.knots + b.knot_off[c];
    const double* cp = b.ctrl + b.ctrl_off[c];
    const int span = int(j) + P;
    float2* at = t.coef_ff + b.coef_off[c] + j * N;
    const double ka = kv[span], kb = kv[span + 1];
    if (!(kb >= ka)) raise_err(t, ERR_BAD_KNOTS);
    if (kb > ka) {
        bspline_setup_ff<P, D>(kv, cp, span, at);
        t.seg_t0[s] = ka;
        t.seg_t1[s] = kb;
        ff r[P * D];
        float q0;
        EvalFF<bs_code(P, D)>::load(at, r);
        // the start speed and slope only shape the sampler's first guess: FP32
        t.seg_f0[s] = (double)EvalFF<bs_code(P, D)>::speed_slope32(r, -1.0f, q0);
        t.seg_q0[s] = (double)q0;
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) at[i] = make_float2(0.0f, 0.0f);
        t.seg_t0[s] = ka;
        t.seg_t1[s] = ka;
        t.seg_f0[s] = 0.0;
        t.seg_q0[s] = 0.0;
    }
}

template <int P, int D>
__device__ __forceinline__ void setup_bspline_any(const Batch& b, const Table& t, int64_t s, int64_t c)
{
    if (t.coef_ff)
        setup_bspline_seg_ff<P, D>(b, t, s, c);
    else
        setup_bspline_seg<P, D>(b, t, s, c);
}

// feat16 (learned form only, else NULL): bf16 feature row of every B-spline
// segment s at feat16[2 s]
static __global__ void k_setup(Batch b, Table t, uint4* __restrict__ feat16, float rtol_feat)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < b.n_seg;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = b.seg_curve[s];
        if (feat16 && b.kind[c] != 0) write_feature_row_bf16(b, s, rtol_feat, feat16 + 2 * s);
        switch (curve_code(b, c)) {
        case CODE_ELLIPSE: setup_ellipse_seg(b, t, s, c); break;
#define GCV_SETUP_CASE(P, D)                                                                       \
    case bs_code(P, D): setup_bspline_any<P, D>(b, t, s, c); break;
            GCV_SETUP_CASE(1, 2) GCV_SETUP_CASE(2, 2) GCV_SETUP_CASE(3, 2) GCV_SETUP_CASE(4, 2)
            GCV_SETUP_CASE(5, 2) GCV_SETUP_CASE(1, 3) GCV_SETUP_CASE(2, 3) GCV_SETUP_CASE(3, 3)
            GCV_SETUP_CASE(4, 3) GCV_SETUP_CASE(5, 3)
#undef GCV_SETUP_CASE
        default: break;
        }
    }
}

// set-up of the segments list[0 .. n) of one curve code (batches that mix
// codes); feat16 (learned form, B-spline codes; else NULL): the bf16 feature
// row of list[i] at feat16[2 i]
template <int CODE>
__global__ void k_setup_list(Batch b, Table t, const int* __restrict__ list, int64_t n, uint4* __restrict__ feat16,
                             float rtol_feat)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = list[i];
        const int64_t c = b.seg_curve[s];
        if constexpr (CODE == CODE_ELLIPSE) {
            setup_ellipse_seg(b, t, s, c);
        } else {
            if (feat16)
                write_feature_row_bf16<code_degree(CODE), code_dim(CODE)>(b, s, rtol_feat, feat16 + 2 * i);
            setup_bspline_any<code_degree(CODE), code_dim(CODE)>(b, t, s, c);
        }
    }
}

// segment -> curve map (thread per curve writes its range)
static __global__ void k_seg_curve(Batch b, int* seg_curve)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < b.n_curve;
         c += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t s = b.seg_off[c]; s < b.seg_off[c + 1]; ++s) seg_curve[s] = int(c);
    }
}

// grouped segment list: the segments of curve c go to dst[c], dst[c] + 1, ...
static __global__ void k_group_segments(Batch b, const int64_t* __restrict__ dst, int* __restrict__ list)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < b.n_seg;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int c = b.seg_curve[s];
        list[dst[c] + (s - b.seg_off[c])] = int(s);
    }
}

// sum of leaf_cnt over a list of segments (one atomic per warp)
static __global__ void k_deep_total(const int* __restrict__ list, int64_t n, const int* __restrict__ leaf_cnt,
                                    unsigned long long* __restrict__ out)
{
    unsigned long long acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += (unsigned long long)leaf_cnt[list[i]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// ------------------------------------------------- compensated scan
// Single-pass segmented inclusive scan of segment lengths (segments of one
// curve are contiguous; a curve's first segment starts a new sum) with
// decoupled look-back between tiles and double-double (two-sum) arithmetic,
// replacing the reference's per-segment Brent-Kung scan plus one thread per
// curve doing a sequential Kahan sum (gcurval/detail/cuda/kernel/generic.inl.cuh:52-137).
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 32;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr long long SCAN_SPIN_LIMIT = 1ll << 22;

struct SegVal {
    int flag;  // a curve starts inside this range
    DD v;      // sum since the last start
};
// a earlier, b later
__device__ __forceinline__ SegVal seg_combine(const SegVal& a, const SegVal& b)
{
    if (b.flag) return b;
    return SegVal{a.flag, dd_add(a.v, b.v)};
}
__device__ __forceinline__ SegVal shfl_up_sv(const SegVal& x, int d)
{
    SegVal y;
    y.flag = __shfl_up_sync(0xffffffffu, x.flag, d);
    y.v.hi = __shfl_up_sync(0xffffffffu, x.v.hi, d);
    y.v.lo = __shfl_up_sync(0xffffffffu, x.v.lo, d);
    return y;
}

static __global__ void __launch_bounds__(SCAN_THREADS) k_scan(Batch b, Table t, int64_t n_tiles)
{
    __shared__ int s_tile;
    __shared__ SegVal s_warp[SCAN_THREADS / 32];
    __shared__ SegVal s_prefix;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(t.ctr + C_SCAN_TILE, 1ull);
    __syncthreads();
    const int64_t tile = s_tile;
    if (tile >= n_tiles) return;
    const int64_t base = tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;

    // Within a warp: plain FP64 running sums of at most SCAN_ITEMS lengths
    // since the last curve start per thread, and a plain FP64 scan of the 32
    // thread sums (at most 1,024 lengths, rounding <= 37 ulp of the partial
    // sum); across warps, tiles and the look-back, where the sums grow long:
    // double-double.  The FP64 pipe bounds this kernel, and the warp-level
    // double-double carries were most of its FP64 operations.
    double part[SCAN_ITEMS];  // running sum since the last start within the thread
    unsigned heads = 0;       // bit k: item k starts a curve
    int prev_curve = base > 0 && base - 1 < b.n_seg ? b.seg_curve[base - 1] : -1;
    double run = 0.0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const int64_t s = base + k;
        double x = 0.0;
        if (s < b.n_seg) {
            x = t.seg_len[s];
            const int cc = b.seg_curve[s];
            if (s == 0 || cc != prev_curve) heads |= 1u << k;
            prev_curve = cc;
        }
        run = (heads >> k) & 1u ? x : run + x;
        part[k] = run;
    }
    // warp inclusive scan of the thread aggregates (seg_combine in FP64)
    int inc_flag = heads != 0;
    double inc_v = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int yf = __shfl_up_sync(0xffffffffu, inc_flag, d);
        const double yv = __shfl_up_sync(0xffffffffu, inc_v, d);
        if (lane >= d && !inc_flag) {
            inc_v = yv + inc_v;
            inc_flag = yf;
        }
    }
    if (lane == 31) s_warp[warp] = SegVal{inc_flag, DD{inc_v, 0.0}};
    __syncthreads();
    if (warp == 0) {
        SegVal w = lane < SCAN_THREADS / 32 ? s_warp[lane] : SegVal{0, DD{0.0, 0.0}};
#pragma unroll
        for (int d = 1; d < SCAN_THREADS / 32; d <<= 1) {
            const SegVal y = shfl_up_sv(w, d);
            if (lane >= d) w = seg_combine(y, w);
        }
        if (lane < SCAN_THREADS / 32) s_warp[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    // exclusive prefix of this thread inside the tile
    const int ex_flag = __shfl_up_sync(0xffffffffu, inc_flag, 1);
    const double ex_v = __shfl_up_sync(0xffffffffu, inc_v, 1);
    SegVal excl = lane == 0 ? SegVal{0, DD{0.0, 0.0}} : SegVal{ex_flag, DD{ex_v, 0.0}};
    if (warp > 0) excl = lane == 0 ? s_warp[warp - 1] : seg_combine(s_warp[warp - 1], excl);

    // decoupled look-back by thread 0
    if (threadIdx.x == 0) {
        const SegVal tile_agg = s_warp[SCAN_THREADS / 32 - 1];
        SegVal pre{0, DD{0.0, 0.0}};
        if (tile == 0) {
            pre = SegVal{1, DD{0.0, 0.0}};
        } else {
            t.scan_flag[tile] = tile_agg.flag;
            t.scan_hi[tile] = tile_agg.v.hi;
            t.scan_lo[tile] = tile_agg.v.lo;
            __threadfence();
            atomicExch(t.scan_status + tile, 1);
            bool done = false;
            for (int64_t j = tile - 1; j >= 0 && !done; --j) {
                int st = 0;
                for (long long it = 0; it < SCAN_SPIN_LIMIT; ++it) {
                    st = atomicAdd(t.scan_status + j, 0);
                    if (st) break;
                    __nanosleep(64);
                }
                if (!st) {
                    raise_err(t, ERR_SCAN_TIMEOUT);
                    break;
                }
                __threadfence();
                const SegVal pj{__ldcg(t.scan_flag + j), DD{__ldcg(t.scan_hi + j), __ldcg(t.scan_lo + j)}};
                pre = seg_combine(pj, pre);
                if (st == 2 || pj.flag) done = true;
            }
        }
        const SegVal incl = seg_combine(pre, tile_agg);
        t.scan_flag[tile] = 1;
        t.scan_hi[tile] = incl.v.hi;
        t.scan_lo[tile] = incl.v.lo;
        __threadfence();
        atomicExch(t.scan_status + tile, 2);
        s_prefix = pre;
    }
    __syncthreads();
    // items before the thread's first curve start add the exclusive prefix
    const SegVal pre = seg_combine(s_prefix, excl);
    const int first_head = heads ? __ffs(heads) - 1 : SCAN_ITEMS;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const int64_t s = base + k;
        if (s < b.n_seg) t.seg_cum[s] = k < first_head ? pre.v.hi + (pre.v.lo + part[k]) : part[k];
    }
}

static __global__ void k_curve_len(Batch b, Table t)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < b.n_curve;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = b.seg_off[c + 1];
        t.curve_len[c] = e > b.seg_off[c] ? t.seg_cum[e - 1] : 0.0;
    }
}

// ------------------------------------------- sample offsets on the device
// Exclusive prefix sums of n int32 sample counts, read through idx when set
// (counts of the curves idx[0..n) in that order), into out[0..n]; out[n] is
// the total.  Three launches: block totals (1024 counts per block), a serial
// scan of the block totals, block-local scans.  Negative counts count as 0
// and raise ERR_BAD_COUNT.
static __global__ void k_count_block_sums(const int* cnt, const int* idx, int64_t n, int64_t* blk, unsigned long long* err)
{
    __shared__ int64_t w[32];
    const int64_t base = (int64_t)blockIdx.x * 1024;
    int64_t x = 0;
    for (int i = threadIdx.x; i < 1024; i += blockDim.x)
        if (base + i < n) {
            const int v = cnt[idx ? idx[base + i] : base + i];
            if (v < 0) atomicOr(err, (unsigned long long)ERR_BAD_COUNT);
            x += v > 0 ? v : 0;
        }
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
        blk[blockIdx.x] = t;
    }
}
static __global__ void k_count_scan_blocks(int64_t* blk, int64_t nb)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int64_t run = 0;
        for (int64_t i = 0; i < nb; ++i) {
            const int64_t v = blk[i];
            blk[i] = run;
            run += v;
        }
        blk[nb] = run;
    }
}
static __global__ void __launch_bounds__(1024) k_count_scan(const int* cnt, const int* idx, int64_t n, const int64_t* blk,
                                                            int64_t* out)
{
    __shared__ int64_t w[32];
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    int64_t x = 0;
    if (i < n) {
        const int v = cnt[idx ? idx[i] : i];
        x = v > 0 ? v : 0;
    }
    int64_t v = x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
    }
    if (lane == 31) w[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int64_t t = w[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        w[lane] = t;
    }
    __syncthreads();
    if (i < n) out[i] = blk[blockIdx.x] + (wid ? w[wid - 1] : 0) + v - x;
    if (i == n - 1) out[n] = blk[gridDim.x];
}

// ------------------------------------------------- learned form: data
// features of every interval (16 floats each)
static __global__ void k_features(Batch b, float rtol_feat, float* __restrict__ out)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < b.n_seg; s += (int64_t)gridDim.x * blockDim.x) {
        float f[MLP_IN];
        interval_features(b, s, rtol_feat, f);
#pragma unroll
        for (int i = 0; i < MLP_IN; ++i) out[s * MLP_IN + i] = f[i];
    }
}

// labels from a plain table: shallowest leaf depth (capped), leaf share per
// quarter, and the local parameter at arc-length fractions (j + 1/2) / 8 by
// cubic Hermite interpolation of v(S) on the leaf (v' = 1 / f at its ends)
static __global__ void k_labels(Table t, int64_t n_seg, int* __restrict__ depth, float* __restrict__ share,
                                float* __restrict__ tg)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_seg; s += (int64_t)gridDim.x * blockDim.x) {
        const int64_t off = t.leaf_off[s];
        const int cnt = t.leaf_cnt[s];
        const double len = t.seg_len[s];
        if (!(t.seg_t1[s] > t.seg_t0[s]) || cnt <= 0 || !(len > 0.0)) {
            depth[s] = 0;
            for (int q = 0; q < 4; ++q) share[s * 4 + q] = 0.25f;
            for (int j = 0; j < 8; ++j) tg[s * 8 + j] = -1.0f + (2.0f * j + 1.0f) / 8.0f;
            continue;
        }
        int dmin = 64, qc[4] = {0, 0, 0, 0};
        double va = -1.0;
        for (int j = 0; j < cnt; ++j) {
            const double vb = t.leaf_v[off + j];
            const int d = 1 - ilogb(vb - va);  // width 2^(1 - d)
            dmin = min(dmin, d);
            qc[min(3, max(0, (int)((0.5 * (va + vb) + 1.0) * 2.0)))]++;
            va = vb;
        }
        depth[s] = min(dmin, MLP_MAX_DEPTH);
        for (int q = 0; q < 4; ++q) share[s * 4 + q] = (float)qc[q] / (float)cnt;
        int j = 0;
        for (int k8 = 0; k8 < 8; ++k8) {
            const double target = (k8 + 0.5) / 8.0 * len;
            while (j < cnt - 1 && t.leaf_cum[off + j] < target) ++j;
            const double base = j ? t.leaf_cum[off + j - 1] : 0.0, cb = t.leaf_cum[off + j];
            const double a = j ? t.leaf_v[off + j - 1] : -1.0, bv = t.leaf_v[off + j];
            const double fa = j ? (double)t.leaf_f[off + j - 1] : t.seg_f0[s], fb = (double)t.leaf_f[off + j];
            const double dS = cb - base;
            const double sg = dS > 0.0 ? fmin(fmax((target - base) / dS, 0.0), 1.0) : 0.0;
            double v = a + sg * (bv - a);
            if (fa > 0.0 && fb > 0.0) {
                const double s2 = sg * sg, s3 = s2 * sg;
                v = (2 * s3 - 3 * s2 + 1) * a + (-2 * s3 + 3 * s2) * bv + dS * ((s3 - 2 * s2 + sg) / fa + (s3 - s2) / fb);
                v = fmin(fmax(v, a), bv);
            }
            tg[s * 8 + k8] = (float)v;
        }
    }
}

}  // namespace gcv
