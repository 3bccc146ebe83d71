// The length pass with one half-warp per knot interval (float-float panels):
// the alternative mapping to k_length's one lane per interval, chosen by the
// caller through gcv_options.mapping (GCV_MAP_HALF_WARP).  It is not an
// autotuner choice: the two mappings sum K15 and G7 in different orders, and
// a tuner's choice must leave every result bit-identical.
//
// The 16 lanes of a half-warp walk one interval's dyadic panels together:
// in each panel lane hl evaluates one node (gk_lane: the 15 Kronrod nodes,
// lane 15 idle), the half-warp sums K15 and G7 by shuffles, and the walk's
// state (panel (k, depth), running sums, tolerance) is the same in all its
// lanes.  Lane 0 of the half stages accepted leaves in shared memory; the
// lanes write them out together when the interval is done.  The acceptance
// test, the learned start, the leaf table and the deep-list hand-over are
// those of k_length<0, CODE, 1>, so both mappings build the same table (up
// to the summation order of K15 and G7).
//
// Per panel this mapping spends 16 lanes on one node each plus the
// shuffle reductions, where k_length spends one lane on seven node pairs
// (gcv_ff_eval.cuh, panel_k15_ff_pairs); it holds far less state per lane
// and finishes each interval 16 times sooner.
#pragma once

#include "gcv_length_impl.cuh"  // chord_of and the shared parameter block

namespace gcv {

// float-float sum over the 16 lanes of each half-warp (every lane of the
// warp takes part), then lane 0's result for the whole half
__device__ __forceinline__ ff half_warp_sum(ff a, int half_base)
{
#pragma unroll
    for (int o = 8; o > 0; o >>= 1)
        a = ff_add(a, ff{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
    return ff{__shfl_sync(0xffffffffu, a.hi, half_base), __shfl_sync(0xffffffffu, a.lo, half_base)};
}

template <int CODE>
__global__ void __launch_bounds__(LK_THREADS) k_length_hw(LengthParams P)
{
    static_assert(LK_THREADS % 32 == 0, "whole warps");
    constexpr int HALVES = LK_THREADS / 16;
    __shared__ double lf_v[LCAP][HALVES];
    __shared__ double lf_c[LCAP][HALVES];

    const Batch& b = P.b;
    const Table& t = P.t;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, hl = lane & 15, half_base = lane & 16, half = threadIdx.x >> 4;
    const unsigned half_mask = half_base ? 0xffff0000u : 0x0000ffffu;
    const double eps50 = 50.0 * 1.4210854715202004e-14;  // round-off floor: 50 float-float units

    // this lane's node and weights
    double xd, wkd, wgd;
    gk_lane(hl, xd, wkd, wgd);
    const ff xn = ff_from_double(xd), wk = ff_from_double(wkd), wg = ff_from_double(wgd);

    const int64_t n_items = P.n_items_dev ? (int64_t)*P.n_items_dev : P.n_items;
    bool active = false, exhausted = false;
    int64_t s = 0;
    const float2* cff = nullptr;
    unsigned long long k = 0;
    int depth = 0, nleaf = 0;
    double cum = 0.0, tol_unit = 0.0;
    ff cumf{0.0f, 0.0f};
    float tol_f = 0.0f;
    uint32_t dq = 0;
    long long panels = 0;
    unsigned long long my_panels = 0, my_capped = 0, my_nonfinite = 0;

    for (;;) {
        bool fin = false, ovf = false;
        // ---- refill: lane 0 of each idle half takes the next interval
        const bool need = !active && !exhausted;  // the same in all lanes of a half
        unsigned long long item = 0;
        if (need && hl == 0) item = atomicAdd(P.work, 1ull);
        item = __shfl_sync(FULL, item, half_base);
        if (need) {
            if ((int64_t)item >= n_items) {
                exhausted = true;
            } else {
                s = P.list ? (int64_t)P.list[item] : (int64_t)item;
                if (P.by_item) {
                    cff = P.coef_ff + P.coef_base + (int64_t)item * code_stride(CODE);
                } else {
                    const int64_t c = b.seg_curve[s];
                    cff = P.coef_ff + b.coef_off[c] + (s - b.seg_off[c]) * code_stride(CODE);
                }
                k = 0;
                depth = 0;
                nleaf = 0;
                cum = 0.0;
                cumf = ff{0.0f, 0.0f};
                panels = 0;
                dq = 0;
                if constexpr (CODE > 0) {
                    if (P.starts) {
                        const uint32_t q = P.starts[P.by_item ? (int64_t)item : s];
                        ff rc[MAX_COEF];
                        EvalFF<CODE>::load(cff, rc);
                        const float ch = chord_of<CODE>(rc);
                        if (q != 0u && ch > 0.0f) {
                            dq = q;
                            tol_unit = P.rtol * (double)ch;
                            tol_f = (float)tol_unit;
                            learned_descend(dq, k, depth);
                        }
                    }
                }
                if (t.seg_t1[s] == t.seg_t0[s]) {  // zero-width knot interval: one empty leaf
                    if (hl == 0) {
                        lf_v[0][half] = 1.0;
                        lf_c[0][half] = 0.0;
                    }
                    nleaf = 1;
                    fin = true;
                } else {
                    active = true;
                }
            }
        }
        // ---- one panel per active half: each lane one node
        const float hwf = __int_as_float((127 - depth) << 23);  // 2^-depth
        ff Kf{0.0f, 0.0f}, Gf{0.0f, 0.0f};
        if (active && hl < 15) {
            const float kh = (float)(unsigned)(k >> 24), kl = (float)(unsigned)(k & 0xFFFFFFull);
            const float sh = __int_as_float((127 + 25 - depth) << 23), sl = 2.0f * hwf;
            const ff vlo = ff_add_f(two_sum(-1.0f, kh * sh), kl * sl);
            const ff v = ff_add(ff_add_f(vlo, hwf), ff_scale(xn, hwf));
            ff rl[MAX_COEF];
            EvalFF<CODE>::load(cff, rl);
            const ff f = EvalFF<CODE>::speed(rl, v);
            Kf = ff_mul(wk, f);
            Gf = ff_mul(wg, f);
        }
        Kf = half_warp_sum(Kf, half_base);
        Gf = half_warp_sum(Gf, half_base);
        if (active) {
            Kf = ff_scale(Kf, hwf);
            Gf = ff_scale(Gf, hwf);
            if (depth == 0) {
                tol_unit = P.rtol * fabs(ff_to_double(Kf));
                tol_f = (float)tol_unit;
            }
            const ff dkg = ff_add(Kf, ff_neg(Gf));
            const float errf = fabsf(dkg.hi);
            const float thr = fmaxf(tol_f * hwf, (float)eps50 * fabsf(Kf.hi));
            const bool finite = isfinite(Kf.hi) && isfinite(Gf.hi);
            bool ok;
            if (errf < 0.99f * thr) {
                ok = true;
            } else if (errf > 1.01f * thr && thr > 1e-30f) {
                ok = false;
            } else {
                const double Kd = ff_to_double(Kf);
                ok = fabs(ff_to_double(dkg)) <= fmax(tol_unit * pow2_neg(depth), eps50 * fabs(Kd));
            }
            ++panels;
            const bool at_cap = depth >= P.max_depth || panels >= PANEL_BUDGET;
            if (ok || at_cap || !finite) {
                if (!ok && finite) ++my_capped;
                if (!finite) ++my_nonfinite;
                cumf = ff_add(cumf, Kf);
                cum = ff_to_double(cumf);
                const double vr = fma(__ull2double_rn(k + 1), 2.0 * pow2_neg(depth), -1.0);
                if (nleaf < LCAP) {
                    if (hl == 0) {
                        lf_v[nleaf][half] = vr;
                        lf_c[nleaf][half] = cum;
                    }
                } else {
                    ovf = true;
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
            if (!active && hl == 0) my_panels += (unsigned long long)panels;
        }
        // ---- finished intervals: the half writes its leaves together
        if (fin) {
            __syncwarp(half_mask);  // lane 0's staged leaves are visible to the half
            unsigned long long base = 0;
            if (hl == 0) base = atomicAdd(t.ctr + C_LEAF_TOP, (unsigned long long)nleaf);
            base = __shfl_sync(half_mask, base, half_base);
            const int64_t off = (int64_t)base;
            if (off + nleaf <= t.leaf_cap) {
                ff rl[MAX_COEF];
                EvalFF<CODE>::load(cff, rl);
                for (int i = hl; i < nleaf; i += 16) {
                    const double vi = lf_v[i][half];
                    float q32;
                    const float f32 = EvalFF<CODE>::speed_slope32(rl, (float)vi, q32);
                    t.leaf_v[off + i] = vi;
                    t.leaf_cum[off + i] = lf_c[i][half];
                    t.leaf_f[off + i] = f32;
                    t.leaf_q[off + i] = q32;
                }
            } else if (hl == 0) {
                // the pool is full: the deep passes redo this interval
                const unsigned long long o = atomicAdd(t.ctr + C_DEEP, 1ull);
                if ((int64_t)o < t.deep_cap)
                    t.deep_list[o] = int(s);
                else
                    raise_err(t, ERR_DEEP_LIST);
            }
            if (hl == 0) {
                t.seg_len[s] = nleaf == 1 && t.seg_t1[s] == t.seg_t0[s] ? 0.0 : cum;
                t.leaf_off[s] = off;
                t.leaf_cnt[s] = nleaf;
            }
            __syncwarp(half_mask);  // the staging slots are free for the next interval
        }
        if (ovf && hl == 0) {
            const unsigned long long o = atomicAdd(t.ctr + C_DEEP, 1ull);
            if ((int64_t)o < t.deep_cap)
                t.deep_list[o] = int(s);
            else
                raise_err(t, ERR_DEEP_LIST);
        }
        if (__all_sync(FULL, exhausted && !active)) break;
    }
    // ---- statistics (lane 0 of each half holds its counts)
    if (hl != 0) my_panels = my_capped = my_nonfinite = 0;
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

template <int CODE>
cudaError_t length_launch_hw(const LengthParams& P, cudaStream_t stream, int sm_count, int blocks_per_sm_cap)
{
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_length_hw<CODE>, LK_THREADS, 0);
    if (e != cudaSuccess) return e;
    const int cap = blocks_per_sm_cap < 1 ? 1 : blocks_per_sm_cap;
    occ = occ < 1 ? 1 : (occ > cap ? cap : occ);
    const int64_t want = (P.n_items + LK_THREADS / 16 - 1) / (LK_THREADS / 16);
    int64_t grid = (int64_t)sm_count * occ;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    k_length_hw<CODE><<<(unsigned)grid, LK_THREADS, 0, stream>>>(P);
    return cudaGetLastError();
}

#define GCV_LENGTH_HW_INST(CODE)                                                                  \
    template cudaError_t length_launch_hw<CODE>(const LengthParams&, cudaStream_t, int, int);

}  // namespace gcv
