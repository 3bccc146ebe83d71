// Learned form: a small MLP (16 features -> 3 x 128 GELU -> 32 outputs) that
// predicts, per B-spline knot interval, the depth of the shallowest leaf of
// the adaptive walk (13 classes), the share of leaves in each quarter of the
// interval ("panel split fractions") and 8 local parameters at arc-length
// fractions (j + 1/2) / 8 of the interval.  The length walk starts at the
// predicted depths instead of the whole interval; every panel is still
// checked with the Kronrod error estimate and split further when it misses
// the tolerance, so the plain adaptive method keeps the final say.
//
// This header: sizes, the packed weight layout, the per-interval features and
// the start-depth rule shared by the kernels.
#pragma once

#include <cmath>

#include "gcv_table.cuh"

namespace gcv {

constexpr int MLP_IN = 16;
constexpr int MLP_H = 128;
constexpr int MLP_OUT = 32;
constexpr int MLP_DEPTHS = 13;  // depth classes 0 .. 12
constexpr int MLP_O_SPLIT = 13;  // 4 quarter logits
constexpr int MLP_O_T = 17;      // 8 local parameters
constexpr int MLP_MAX_DEPTH = 12;

// packed FP32 weights, row-major W[in][out] then the bias of each layer
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_IN * MLP_H;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H * MLP_H;
constexpr int MLP_OFF_W4 = MLP_OFF_B3 + MLP_H;
constexpr int MLP_OFF_B4 = MLP_OFF_W4 + MLP_H * MLP_OUT;
constexpr int MLP_NPARAM = MLP_OFF_B4 + MLP_OUT;

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
constexpr float GELU_C = 0.7978845608028654f;
constexpr float GELU_A = 0.044715f;

// x to float by its bit pattern, truncated (integer instructions only: on
// GB300 a conversion on the FP64 pipe costs as much issue time as dozens of
// FP32 instructions); |x| below 2^-126 gives 0, above 2^127 the largest float.
// Precise enough for the network's features.
__device__ __forceinline__ float float_of(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned top = (unsigned)(b >> 32), sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7FFu) - 1023;
    if (e < -126) return __uint_as_float(sign);
    if (e > 127) return __uint_as_float(sign | 0x7F7FFFFFu);
    return __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7FFFFFull));
}

// Features of interval s (a B-spline knot interval; anything else gets
// zeros), FP32:
//   0 degree / 5, 1 dim - 2,
//   2..6 control-polygon edge lengths of the interval's p + 1 control points,
//        over their sum (zero-padded),
//   7..10 cosines of the turning angles between consecutive edges (one-padded),
//   11 interval width over the support of its basis functions,
//   12, 13 log2 of the left / right neighbour width over the width, clamped
//        to [-8, 8], / 8,
//   14 log2(polygon length / chord) clamped to [0, 8], / 4,
//   15 -log10(rtol) / 10.
// Computed in FP32 from the knots and control points converted by float_of.
__device__ inline void interval_features(const Batch& b, int64_t s, float log_rtol_feature, float* f)
{
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) f[i] = 0.0f;
    const int64_t c = b.seg_curve[s];
    if (b.kind[c] == 0) return;
    const int p = b.degree[c], D = b.dim[c];
    const int64_t j = s - b.seg_off[c];
    const double* kv = b.knots + b.knot_off[c];
    const double* cp = b.ctrl + b.ctrl_off[c];
    const int span = int(j) + p;
    const double k0 = kv[span];
    const float fk0 = float_of(k0);
    const float w = float_of(kv[span + 1]) - fk0;
    f[0] = p * 0.2f;
    f[1] = (float)(D - 2);
    f[15] = log_rtol_feature;
    if (!(w > 0.0f)) return;
    // control polygon of the interval, relative to its first point
    float q[6][3], base[3];
    for (int d = 0; d < 3; ++d) base[d] = d < D ? float_of(cp[(size_t)(span - p) * D + d]) : 0.0f;
    for (int i = 0; i <= p; ++i)
        for (int d = 0; d < 3; ++d) q[i][d] = d < D ? float_of(cp[(size_t)(span - p + i) * D + d]) - base[d] : 0.0f;
    float e[5], sum = 0.0f;
    for (int i = 0; i < p; ++i) {
        const float dx = q[i + 1][0] - q[i][0], dy = q[i + 1][1] - q[i][1], dz = q[i + 1][2] - q[i][2];
        e[i] = sqrtf(dx * dx + dy * dy + dz * dz);
        sum += e[i];
    }
    for (int i = 0; i < 4; ++i) f[7 + i] = 1.0f;
    if (sum > 0.0f) {
        const float inv = 1.0f / sum;
        for (int i = 0; i < p; ++i) f[2 + i] = e[i] * inv;
        for (int i = 0; i + 1 < p; ++i) {
            float dot = 0.0f;
            for (int d = 0; d < 3; ++d) dot += (q[i + 1][d] - q[i][d]) * (q[i + 2][d] - q[i + 1][d]);
            const float den = e[i] * e[i + 1];
            f[7 + i] = den > 0.0f ? fminf(fmaxf(dot / den, -1.0f), 1.0f) : 1.0f;
        }
        const float cx = q[p][0], cy = q[p][1], cz = q[p][2];
        const float chord = sqrtf(cx * cx + cy * cy + cz * cz);
        f[14] = chord > 0.0f ? fminf(fmaxf(__log2f(sum / chord), 0.0f), 8.0f) * 0.25f : 2.0f;
    }
    const float support = float_of(kv[span + p + 1]) - float_of(kv[span - p]);
    f[11] = support > 0.0f ? w / support : 0.0f;
    const float wl = fk0 - float_of(kv[span - 1]), wr = float_of(kv[span + 2]) - float_of(kv[span + 1]);
    f[12] = wl > 0.0f ? fminf(fmaxf(__log2f(wl / w), -8.0f), 8.0f) * 0.125f : -1.0f;
    f[13] = wr > 0.0f ? fminf(fmaxf(__log2f(wr / w), -8.0f), 8.0f) * 0.125f : -1.0f;
}

// interval_features for a B-spline interval of compile-time degree P and
// dimension D (the per-code set-up kernels): the same operations in the same
// order, with the loops unrolled and the polygon held in registers.
template <int P, int D>
__device__ __forceinline__ void interval_features_pd(const Batch& b, int64_t s, float log_rtol_feature, float* f)
{
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) f[i] = 0.0f;
    const int64_t c = b.seg_curve[s];
    const int64_t j = s - b.seg_off[c];
    const double* kv = b.knots + b.knot_off[c];
    const double* cp = b.ctrl + b.ctrl_off[c];
    const int span = int(j) + P;
    const double k0 = kv[span];
    const float fk0 = float_of(k0);
    const float w = float_of(kv[span + 1]) - fk0;
    f[0] = P * 0.2f;
    f[1] = (float)(D - 2);
    f[15] = log_rtol_feature;
    if (!(w > 0.0f)) return;
    float q[P + 1][3], base[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) base[d] = d < D ? float_of(cp[(size_t)(span - P) * D + d]) : 0.0f;
#pragma unroll
    for (int i = 0; i <= P; ++i)
#pragma unroll
        for (int d = 0; d < 3; ++d) q[i][d] = d < D ? float_of(cp[(size_t)(span - P + i) * D + d]) - base[d] : 0.0f;
    float e[P], sum = 0.0f;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const float dx = q[i + 1][0] - q[i][0], dy = q[i + 1][1] - q[i][1], dz = q[i + 1][2] - q[i][2];
        e[i] = sqrtf(dx * dx + dy * dy + dz * dz);
        sum += e[i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) f[7 + i] = 1.0f;
    if (sum > 0.0f) {
        const float inv = 1.0f / sum;
#pragma unroll
        for (int i = 0; i < P; ++i) f[2 + i] = e[i] * inv;
#pragma unroll
        for (int i = 0; i + 1 < P; ++i) {
            float dot = 0.0f;
#pragma unroll
            for (int d = 0; d < 3; ++d) dot += (q[i + 1][d] - q[i][d]) * (q[i + 2][d] - q[i + 1][d]);
            const float den = e[i] * e[i + 1];
            f[7 + i] = den > 0.0f ? fminf(fmaxf(dot / den, -1.0f), 1.0f) : 1.0f;
        }
        const float cx = q[P][0], cy = q[P][1], cz = q[P][2];
        const float chord = sqrtf(cx * cx + cy * cy + cz * cz);
        f[14] = chord > 0.0f ? fminf(fmaxf(__log2f(sum / chord), 0.0f), 8.0f) * 0.25f : 2.0f;
    }
    const float support = float_of(kv[span + P + 1]) - float_of(kv[span - P]);
    f[11] = support > 0.0f ? w / support : 0.0f;
    const float wl = fk0 - float_of(kv[span - 1]), wr = float_of(kv[span + 2]) - float_of(kv[span + 1]);
    f[12] = wl > 0.0f ? fminf(fmaxf(__log2f(wl / w), -8.0f), 8.0f) * 0.125f : -1.0f;
    f[13] = wr > 0.0f ? fminf(fmaxf(__log2f(wr / w), -8.0f), 8.0f) * 0.125f : -1.0f;
}

// feature 15: -log10(rtol) / 10
inline float rtol_feature(double rtol) { return (float)(-std::log10(rtol) * 0.1); }

// The features of interval s as one bf16 row (16 values, 32 bytes, rounded
// to nearest: the same bf16 values the network kernel would make of the FP32
// row), written by the set-up kernels of the learned form so that no separate
// pass gathers the knots and control points again.
// P > 0: the interval's curve has compile-time degree P and dimension D;
// P == 0: read them from the batch
template <int P = 0, int D = 0>
__device__ __forceinline__ void write_feature_row_bf16(const Batch& b, int64_t s, float log_rtol_feature,
                                                       uint4* __restrict__ row)
{
    float f[MLP_IN];
    if constexpr (P > 0)
        interval_features_pd<P, D>(b, s, log_rtol_feature, f);
    else
        interval_features(b, s, log_rtol_feature, f);
    uint32_t w[MLP_IN / 2];
#pragma unroll
    for (int i = 0; i < MLP_IN / 2; ++i) {
        uint32_t h;
        asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(h) : "f"(f[2 * i]), "f"(f[2 * i + 1]));
        w[i] = h;
    }
    row[0] = make_uint4(w[0], w[1], w[2], w[3]);
    row[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// Start depth of the learned walk for the node (k, depth): the quarter
// depths dq (one byte each) of the quarters the node covers (their minimum
// above depth 2).
__device__ __forceinline__ int learned_start(uint32_t dq, unsigned long long k, int depth)
{
    if (depth >= 2) return (int)((dq >> (8 * (int)(k >> (depth - 2)))) & 0xffu);
    const int q0 = (int)(k << (2 - depth)), nq = 1 << (2 - depth);
    int m = 255;
    for (int q = q0; q < q0 + nq; ++q) m = min(m, (int)((dq >> (8 * q)) & 0xffu));
    return m;
}

// descend from (k, depth) to the leftmost node at the learned start depth
__device__ __forceinline__ void learned_descend(uint32_t dq, unsigned long long& k, int& depth)
{
    for (int guard = 0; guard < 16 && depth < learned_start(dq, k, depth); ++guard) {
        k <<= 1;
        ++depth;
    }
}

// quarter depths from the network's outputs: the predicted shallowest leaf
// depth d, raised in quarters that hold more than their share of leaves,
// d + round(log2(4 share)), capped by max_depth
__device__ __forceinline__ uint32_t quarter_depths(const float* o, int max_depth)
{
    int d = 0;
    float best = o[0];
    for (int i = 1; i < MLP_DEPTHS; ++i)
        if (o[i] > best) {
            best = o[i];
            d = i;
        }
    float mx = o[MLP_O_SPLIT];
    for (int q = 1; q < 4; ++q) mx = fmaxf(mx, o[MLP_O_SPLIT + q]);
    float e[4], z = 0.0f;
    for (int q = 0; q < 4; ++q) {
        e[q] = __expf(o[MLP_O_SPLIT + q] - mx);
        z += e[q];
    }
    uint32_t out = 0;
    for (int q = 0; q < 4; ++q) {
        int dq = d;
        if (d >= 2) dq += max(0, __float2int_rn(log2f(fmaxf(4.0f * e[q] / z, 1e-6f))));
        dq = min(dq, min(max_depth, MLP_MAX_DEPTH));
        out |= (uint32_t)dq << (8 * q);
    }
    return out;
}

// Start depths of the intervals list[0 .. n) (list NULL: 0 .. n - 1) from
// their bf16 feature rows feat16[0 .. n) (two uint4 each, written by the
// set-up kernels): one launch of the tcgen05 network.
cudaError_t mlp_starts_launch_bf16(const uint4* feat16, const int* list, int64_t n, const void* w_dev, int max_depth,
                                   uint32_t* starts, cudaStream_t stream);
// device copy of the packed FP32 weights in the inference kernel's layout
cudaError_t mlp_upload_bf16(const float* host_w, void** w_dev);
size_t mlp_dev_bytes();

}  // namespace gcv
