// Kernel and launcher of the adaptive length pass (see gcv_length.cuh);
// included only by the gcv_len_*.cu units that instantiate them.
#pragma once

#include <type_traits>

#include "gcv_ff_eval.cuh"
#include "gcv_learned.cuh"
#include "gcv_length.cuh"

namespace gcv {

// K15, G7 and the right-end speed of panel [vlo, vlo + 2 hw].
template <int CODE>
__device__ __forceinline__ void panel_k15(const double* r, double vlo, double hw, double& K, double& G,
                                          double& fend, double& qend)
{
    const double mid = vlo + hw;
    const double fc = Eval<CODE>::speed(r, mid);
    double k = gk_wk(7) * fc;
    double g = gk_wg(7) * fc;
    // unrolled: the FP64 integrands are compact (the float-float panels of
    // large integrands keep their node loop rolled, see panel_k15_ff)
    {
#pragma unroll
        for (int i = 0; i < 7; ++i) {
            const double dx = hw * gk_x(i);
            const double s = Eval<CODE>::speed(r, mid - dx) + Eval<CODE>::speed(r, mid + dx);
            k = fma(gk_wk(i), s, k);
            if (i & 1) g = fma(gk_wg(i), s, g);
        }
    }
    fend = Eval<CODE>::speed_slope(r, vlo + 2.0 * hw, qend);
    K = k * hw;
    G = g * hw;
}

__device__ __forceinline__ void panel_dyn(int code, const double* r, double vlo, double hw, double& K, double& G,
                                          double& fend, double& qend)
{
    switch (code) {
#define GCV_CASE(C)                                                                                \
    case C: panel_k15<C>(r, vlo, hw, K, G, fend, qend); break;
        GCV_FOR_EACH_CODE(GCV_CASE)
#undef GCV_CASE
    default: K = G = fend = qend = 0.0; break;
    }
}

__device__ __forceinline__ int warp_incl_scan(int x, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    return x;
}

// |C(1) - C(-1)| of a B-spline piece from its derivative polynomial
// b_m = (m + 1) a_{m+1}: C(1) - C(-1) = 2 sum_{m even} b_m / (m + 1).  A lower
// bound of the piece's length, so rtol * chord is a tolerance no looser than
// the plain walk's rtol * |K15 of the whole interval|.
template <int CODE, typename T>
__device__ __forceinline__ float chord_of(const T* r)
{
    constexpr int Pd = code_degree(CODE), D = code_dim(CODE);
    float c2 = 0.0f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        float acc = 0.0f;
#pragma unroll
        for (int m = 0; m < Pd; m += 2) {
            if constexpr (std::is_same<T, ff>::value)
                acc += r[m * D + d].hi / (float)(m + 1);
            else
                acc += (float)r[m * D + d] / (float)(m + 1);
        }
        c2 += 4.0f * acc * acc;
    }
    return sqrtf(c2);
}

// Resident blocks per SM the float-float main pass asks for, per curve code:
// 10 (at most 96 registers) for degree 3-5 in 3D, 12 (80) for the others.
// Single-code batches of the uneven 100k batch, main pass alone, at 12 / 10 /
// 8 blocks: degree 2-3 in 2D and degree 2 in 3D are fastest at 12 (3-14 %
// ahead of 8), degree 4-5 in 2D tie at 12 and 10, degree 3-5 in 3D gain 2-4 %
// at 10 (they spill 112-216 bytes at 80 registers, less at 96).
__host__ __device__ constexpr int length_ff_blocks(int code)
{
    return code > 0 && code_dim(code) == 3 && code_degree(code) >= 3 ? 10 : 12;
}

// PREC 0: FP64 panels; PREC 1: float-float panels (GCV_MIXED), whose K15 /
// G7 / end values enter the same FP64 bookkeeping (error test, leaf table).
template <int MODE, int CODE, int PREC = 0>
__global__ void __launch_bounds__(LK_THREADS, (MODE == 0 && PREC == 1) ? length_ff_blocks(CODE) : 1)
    k_length(LengthParams P)
{
    __shared__ double lf_v[MODE == 0 ? LCAP : 1][LK_THREADS];
    __shared__ double lf_c[MODE == 0 ? LCAP : 1][LK_THREADS];
    // the float-float path does not stage the leaves' end speed and slope:
    // it re-evaluates them in FP32 when it flushes the leaves (same values),
    // which leaves 16 of the 24 bytes per staged leaf and more blocks per SM
    constexpr int FQ_ROWS = MODE == 0 && PREC == 0 ? LCAP : 1;
    __shared__ float lf_f[FQ_ROWS][LK_THREADS];
    __shared__ float lf_q[FQ_ROWS][LK_THREADS];

    const Batch& b = P.b;
    const Table& t = P.t;
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x;
    const unsigned FULL = 0xffffffffu;
    const unsigned lt_mask = (1u << lane) - 1u;
    // round-off floor of the error test: 50 units of the working precision
    // (FP64: 2^-52; float-float: ~2^-46)
    const double eps50 = PREC == 1 ? 50.0 * 1.4210854715202004e-14 : 50.0 * 2.220446049250313e-16;

    const int64_t n_items = P.n_items_dev ? (int64_t)*P.n_items_dev : P.n_items;
    bool active = false, exhausted = false;
    int64_t s = 0, pool = 0;
    int code = CODE >= 0 ? CODE : 0;
    double r[PREC == 0 ? MAX_COEF : 1];
    // float-float path: the interval's coefficients are reloaded for every
    // panel (L1 hits) rather than kept in registers: the panel shifts its
    // copy in place, and the registers go to occupancy
    const float2* cff = nullptr;
    unsigned long long k = 0;
    int depth = 0, nleaf = 0;
    double cum = 0.0, tol_unit = 0.0;
    ff cumf{0.0f, 0.0f};  // float-float running sum (PREC 1)
    float tol_f = 0.0f;
    uint32_t dq = 0;  // learned quarter start depths of the segment (0: plain walk)
    long long panels = 0;
    unsigned long long my_panels = 0, my_capped = 0, my_nonfinite = 0;

    for (;;) {
        bool fin = false, ovf = false;
        // ---- refill idle lanes with one atomic per warp
        const bool need = !active && !exhausted;
        const unsigned m = __ballot_sync(FULL, need);
        if (m) {
            const int leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(P.work, (unsigned long long)__popc(m));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const int64_t item = (int64_t)base + __popc(m & lt_mask);
                if (item >= n_items) {
                    exhausted = true;
                } else {
                    s = P.list ? (int64_t)P.list[item] : item;
                    // the main pass of one code addresses the table by work
                    // item (no dependent loads before the first panel)
                    const bool by_item = MODE == 0 && CODE >= 0 && P.by_item;
                    int64_t ci;
                    if (by_item) {
                        ci = P.coef_base + item * code_stride(code);
                    } else {
                        const int64_t c = b.seg_curve[s];
                        if (CODE < 0) code = curve_code(b, c);
                        ci = b.coef_off[c] + (s - b.seg_off[c]) * code_stride(code);
                    }
                    if constexpr (PREC == 1) {
                        cff = P.coef_ff + ci;
                    } else {
                        if constexpr (CODE >= 0)
                            Eval<(CODE >= 0 ? CODE : 0)>::load_speed(t.coef + ci, r);
                        else
                            load_speed_dyn(code, t.coef + ci, r);
                    }
                    k = 0;
                    depth = 0;
                    nleaf = 0;
                    cum = 0.0;
                    cumf = ff{0.0f, 0.0f};
                    panels = 0;
                    dq = 0;
                    if constexpr (MODE == 0 && CODE > 0) {
                        // learned start: the predicted depths, tolerance from the chord
                        if (P.starts) {
                            const uint32_t q = P.starts[by_item ? item : s];
                            float ch;
                            if constexpr (PREC == 1) {
                                ff rc[MAX_COEF];
                                EvalFF<(CODE > 0 ? CODE : 16 + 4 + 2)>::load(cff, rc);
                                ch = chord_of<CODE>(rc);
                            } else {
                                ch = chord_of<CODE>(r);
                            }
                            if (q != 0u && ch > 0.0f) {
                                dq = q;
                                tol_unit = P.rtol * (double)ch;
                                tol_f = (float)tol_unit;
                                learned_descend(dq, k, depth);
                            }
                        }
                    }
                    if (MODE == 2) {
                        pool = (int64_t)atomicAdd(t.ctr + C_LEAF_TOP, (unsigned long long)t.leaf_cnt[s]);
                        if (pool + t.leaf_cnt[s] > t.leaf_cap) {
                            raise_err(t, ERR_POOL);
                            pool = -1;
                        }
                    }
                    // zero-width knot interval: one empty leaf (the main pass
                    // by work item walks it: its coefficients are zero, so the
                    // root panel is accepted with length 0 and the same leaf)
                    if (!by_item && t.seg_t1[s] == t.seg_t0[s]) {
                        if (MODE == 0) {
                            lf_v[0][tid] = 1.0;
                            lf_c[0][tid] = 0.0;
                            if constexpr (PREC == 0) {
                                lf_f[0][tid] = 0.0f;
                                lf_q[0][tid] = 0.0f;
                            }
                        } else if (MODE == 2 && pool >= 0) {
                            t.leaf_v[pool] = 1.0;
                            t.leaf_cum[pool] = 0.0;
                            t.leaf_f[pool] = 0.0f;
                            t.leaf_q[pool] = 0.0f;
                        }
                        nleaf = 1;
                        fin = true;
                    } else if (MODE != 2 || pool >= 0) {
                        active = true;
                    }
                }
            }
        }
        // ---- one panel per active lane
        if (active) {
            // panel values: K15, the error test, and (for leaves) the right-end
            // speed f and slope q, in FP64; the float-float path keeps its
            // values in FP32 pairs, evaluates f and q of leaves in plain FP32,
            // and touches FP64 only for leaves' sums and for error tests that
            // land within 1 % of the threshold
            bool ok, finite;
            double K = 0.0, fend = 0.0, qend = 0.0;
            ff Kf{0.0f, 0.0f};
            if constexpr (PREC == 1) {
                ff Gf;
                ff rl[MAX_COEF];
                if constexpr (CODE >= 0) {
                    EvalFF<(CODE >= 0 ? CODE : 0)>::load(cff, rl);
                    panel_ff<(CODE >= 0 ? CODE : 0)>(rl, k, depth, Kf, Gf);
                } else {
                    load_ff_dyn(code, cff, rl);
                    panel_ff_dyn(code, rl, k, depth, Kf, Gf);
                }
                if (depth == 0) {
                    tol_unit = P.rtol * fabs(ff_to_double(Kf));
                    tol_f = (float)tol_unit;
                }
                const ff dkg = ff_add(Kf, ff_neg(Gf));
                const float hwf = __int_as_float((127 - depth) << 23);  // 2^-depth
                const float errf = fabsf(dkg.hi);
                const float thr = fmaxf(tol_f * hwf, (float)eps50 * fabsf(Kf.hi));
                finite = isfinite(Kf.hi) && isfinite(Gf.hi);
                if (errf < 0.99f * thr) {
                    ok = true;
                } else if (errf > 1.01f * thr && thr > 1e-30f) {
                    ok = false;
                } else {  // near the tolerance (or below FP32 range): the FP64 test
                    const double Kd = ff_to_double(Kf);
                    ok = fabs(ff_to_double(dkg)) <= fmax(tol_unit * pow2_neg(depth), eps50 * fabs(Kd));
                }
            } else {
                const double hw = pow2_neg(depth);
                const double vlo = fma(__ull2double_rn(k), 2.0 * hw, -1.0);
                double G;
                if constexpr (CODE >= 0)
                    panel_k15<(CODE >= 0 ? CODE : 0)>(r, vlo, hw, K, G, fend, qend);
                else
                    panel_dyn(code, r, vlo, hw, K, G, fend, qend);
                if (depth == 0) tol_unit = P.rtol * fabs(K);
                finite = isfinite(K) && isfinite(G);
                ok = fabs(K - G) <= fmax(tol_unit * hw, eps50 * fabs(K));
            }
            ++panels;
            const bool at_cap = depth >= P.max_depth || panels >= PANEL_BUDGET;
            if (ok || at_cap || !finite) {
                if (!ok && finite) ++my_capped;
                if (!finite) ++my_nonfinite;
                if constexpr (PREC == 1) {
                    cumf = ff_add(cumf, Kf);
                    cum = ff_to_double(cumf);
                    if constexpr (MODE == 2) {
                        // the leaf's right-end speed and slope (FP32: they only
                        // shape the sampler's guess), -1 + (k + 1) 2^(1 - depth)
                        const float vr32 = fmaf((float)(k + 1), __int_as_float((128 - depth) << 23), -1.0f);
                        float q32;
                        ff rl[MAX_COEF];
                        if constexpr (CODE >= 0)
                            EvalFF<(CODE >= 0 ? CODE : 0)>::load(cff, rl);
                        else
                            load_ff_dyn(code, cff, rl);
                        fend = (double)speed_slope32_of<CODE>(code, rl, vr32, q32);
                        qend = (double)q32;
                    }
                } else {
                    cum += K;
                }
                // right end -1 + (k + 1) 2^(1 - depth): exact
                const double vr = fma(__ull2double_rn(k + 1), 2.0 * pow2_neg(depth), -1.0);
                if (MODE == 0) {
                    if (nleaf < LCAP) {
                        lf_v[nleaf][tid] = vr;
                        lf_c[nleaf][tid] = cum;
                        if constexpr (PREC == 0) {
                            lf_f[nleaf][tid] = (float)fend;
                            lf_q[nleaf][tid] = (float)qend;
                        }
                    } else {
                        ovf = true;
                    }
                } else if (MODE == 2) {
                    t.leaf_v[pool + nleaf] = vr;
                    t.leaf_cum[pool + nleaf] = cum;
                    t.leaf_f[pool + nleaf] = (float)fend;
                    t.leaf_q[pool + nleaf] = (float)qend;
                }
                ++nleaf;
                ++k;
                const int tz = __ffsll((long long)k) - 1;
                k >>= tz;
                depth -= tz;
                if (dq && depth > 0) learned_descend(dq, k, depth);
                if (ovf) {
                    active = false;
                } else if (depth == 0) {
                    active = false;
                    fin = true;
                }
            } else {
                k <<= 1;
                ++depth;
            }
            if (!active) my_panels += (unsigned long long)panels;
        }
        // ---- finished segments: outputs (leaf-pool offsets reserved per warp)
        if (MODE == 0) {
            const unsigned fm = __ballot_sync(FULL, fin);
            if (fm) {
                const int x = fin ? nleaf : 0;
                const int incl = warp_incl_scan(x, lane);
                const int total = __shfl_sync(FULL, incl, 31);
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(t.ctr + C_LEAF_TOP, (unsigned long long)total);
                base = __shfl_sync(FULL, base, 0);
                const int64_t off = (int64_t)base + incl - x;  // this lane's first pool slot
                const bool fits = off + nleaf <= t.leaf_cap;
                __syncwarp(FULL);  // the lanes' staged leaves, written this iteration, are read across lanes
                // The warp writes the finished lanes' leaves together, leaf
                // g of the warp's total going to lane g % 32, instead of each
                // finished lane writing its own while the others wait: the
                // owner of leaf g is the first lane whose inclusive count
                // exceeds g (a five-step search over the counts).
                for (int g0 = 0; g0 < total; g0 += 32) {
                    const int gi = g0 + lane;
                    int owner = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1)
                        if (__shfl_sync(FULL, incl, owner + step - 1) <= gi) owner += step;
                    const int o_first = __shfl_sync(FULL, incl - x, owner);
                    const bool o_fits = __shfl_sync(FULL, (int)fits, owner) != 0;
                    const int64_t o_off = (int64_t)__shfl_sync(FULL, (unsigned long long)off, owner);
                    const int i = gi - o_first;          // the leaf's index in its interval
                    const int otid = (tid & ~31) + owner;  // the owner's staging column
                    if constexpr (PREC == 1) {
                        const float2* o_cff = reinterpret_cast<const float2*>(
                            __shfl_sync(FULL, reinterpret_cast<unsigned long long>(cff), owner));
                        const int o_code = CODE >= 0 ? CODE : __shfl_sync(FULL, code, owner);
                        if (gi < total && o_fits) {
                            ff rl[MAX_COEF];
                            if constexpr (CODE >= 0)
                                EvalFF<(CODE >= 0 ? CODE : 0)>::load(o_cff, rl);
                            else
                                load_ff_dyn(o_code, o_cff, rl);
                            const double vi = lf_v[i][otid];
                            float q32;
                            const float f32 = speed_slope32_of<CODE>(o_code, rl, (float)vi, q32);
                            t.leaf_v[o_off + i] = vi;
                            t.leaf_cum[o_off + i] = lf_c[i][otid];
                            t.leaf_f[o_off + i] = f32;
                            t.leaf_q[o_off + i] = q32;
                        }
                    } else {
                        if (gi < total && o_fits) {
                            t.leaf_v[o_off + i] = lf_v[i][otid];
                            t.leaf_cum[o_off + i] = lf_c[i][otid];
                            t.leaf_f[o_off + i] = lf_f[i][otid];
                            t.leaf_q[o_off + i] = lf_q[i][otid];
                        }
                    }
                }
                if (fin) {
                    if (!fits) {
                        // the pool is full: the deep passes redo this interval
                        const unsigned long long o = atomicAdd(t.ctr + C_DEEP, 1ull);
                        if ((int64_t)o < t.deep_cap)
                            t.deep_list[o] = int(s);
                        else
                            raise_err(t, ERR_DEEP_LIST);
                    }
                    t.seg_len[s] = nleaf == 1 && t.seg_t1[s] == t.seg_t0[s] ? 0.0 : cum;
                    t.leaf_off[s] = off;
                    t.leaf_cnt[s] = nleaf;
                }
            }
            if (ovf) {
                const unsigned long long o = atomicAdd(t.ctr + C_DEEP, 1ull);
                if ((int64_t)o < t.deep_cap)
                    t.deep_list[o] = int(s);
                else
                    raise_err(t, ERR_DEEP_LIST);
            }
        } else if (fin) {
            if (MODE == 1) t.leaf_cnt[s] = nleaf;
            if (MODE == 2) {
                t.seg_len[s] = t.seg_t1[s] == t.seg_t0[s] ? 0.0 : cum;
                t.leaf_off[s] = pool;
            }
        }
        if (__all_sync(FULL, exhausted && !active)) break;
    }
    // ---- statistics
    for (int o = 16; o > 0; o >>= 1) {
        my_panels += __shfl_xor_sync(FULL, my_panels, o);
        my_capped += __shfl_xor_sync(FULL, my_capped, o);
        my_nonfinite += __shfl_xor_sync(FULL, my_nonfinite, o);
    }
    if (lane == 0) {
        if (P.collect && my_panels) atomicAdd(t.ctr + C_PANELS, my_panels);
        if (my_capped) atomicAdd(t.ctr + C_CAPPED, my_capped);
        if (my_nonfinite) atomicAdd(t.ctr + C_NONFINITE, my_nonfinite);
    }
}

template <int MODE, int CODE, int PREC>
cudaError_t length_launch(const LengthParams& P, cudaStream_t stream, int sm_count, int blocks_per_sm_cap)
{
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_length<MODE, CODE, PREC>, LK_THREADS, 0);
    if (e != cudaSuccess) return e;
    const int cap = blocks_per_sm_cap < 1 ? 1 : blocks_per_sm_cap;
    occ = occ < 1 ? 1 : (occ > cap ? cap : occ);
    // persistent: fill the GPU, but no more lanes than there are intervals
    const int64_t want = (P.n_items + LK_THREADS - 1) / LK_THREADS;
    int64_t grid = (int64_t)sm_count * occ;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    k_length<MODE, CODE, PREC><<<(unsigned)grid, LK_THREADS, 0, stream>>>(P);
    return cudaGetLastError();
}

#define GCV_LENGTH_INST(MODE, CODE, PREC)                                                          \
    template cudaError_t length_launch<MODE, CODE, PREC>(const LengthParams&, cudaStream_t, int, int);
// both precisions of one (MODE, CODE)
#define GCV_LENGTH_INST2(MODE, CODE) GCV_LENGTH_INST(MODE, CODE, 0) GCV_LENGTH_INST(MODE, CODE, 1)

}  // namespace gcv
