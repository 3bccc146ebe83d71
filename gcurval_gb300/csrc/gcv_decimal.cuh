// Decimal text to binary64, correctly rounded (round to nearest, ties to
// even), for the numbers of the Bundle dataset files.  Host and device.
//
// A token [sign] digits [. digits] [(e|E) [sign] digits] is read as an
// integer significand m of at most 19 significant digits (leading zeros
// skipped, trailing zeros folded into the exponent) and a decimal exponent
// k, value = m * 10^k.  Then:
//   * m <= 2^53 and |k| <= 22: Clinger's fast path, one IEEE multiply or
//     divide of two exact doubles, which is correctly rounded;
//   * 0 < k <= 38 and m * 10^k < 2^128: the product is formed exactly in
//     128-bit integers and rounded once;
//   * -38 <= k < 0: m / 10^-k by restoring binary long division, 64
//     quotient bits plus a sticky bit for the remainder, rounded once.
// Anything else (more significant digits, larger exponents, no digits,
// stray characters) is rejected.  Within that range every result is a
// normal double, so rounding only has to handle the significand.
#pragma once

#include <cstdint>

namespace gcv {

#ifdef __CUDACC__
#define GCV_DEC_HD __host__ __device__ __forceinline__
#else
#define GCV_DEC_HD inline
#endif

typedef unsigned __int128 u128;

GCV_DEC_HD int clz64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

GCV_DEC_HD double bits_to_double(unsigned long long b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double d;
    __builtin_memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// the double nearest to q * 2^(t - 63), 2^63 <= q < 2^64, `sticky` when
// nonzero bits lie below q; ties to even; t within the normal range
GCV_DEC_HD double round_q64(unsigned long long q, int t, bool sticky)
{
    unsigned long long hi = q >> 11;  // 53 bits, bit 52 set
    const unsigned low = (unsigned)(q & 0x7FFu);
    if (low > 0x400u || (low == 0x400u && (sticky || (hi & 1u)))) ++hi;
    if (hi == (1ull << 53)) {
        hi >>= 1;
        ++t;
    }
    return bits_to_double(((unsigned long long)(t + 1023) << 52) | (hi & ((1ull << 52) - 1)));
}

GCV_DEC_HD u128 pow10_u128(int k)
{
    u128 p = 1;
    for (int i = 0; i < k; ++i) p *= 10u;
    return p;
}

// m * 10^k, 1 <= k <= 38; false when the product reaches 2^128
GCV_DEC_HD bool exact_mul(unsigned long long m, int k, double* out)
{
    const u128 p = pow10_u128(k);
    const unsigned long long ph = (unsigned long long)(p >> 64), pl = (unsigned long long)p;
    const u128 lo = (u128)m * pl;
    const u128 mid = (u128)m * ph;
    if ((mid >> 64) != 0) return false;
    const unsigned long long top = (unsigned long long)mid + (unsigned long long)(lo >> 64);
    if (top < (unsigned long long)mid) return false;
    const u128 n = ((u128)top << 64) | (unsigned long long)lo;
    const unsigned long long nh = (unsigned long long)(n >> 64);
    const int t = nh ? 127 - clz64(nh) : 63 - clz64((unsigned long long)n);
    unsigned long long q;
    bool sticky = false;
    if (t >= 63) {
        q = (unsigned long long)(n >> (t - 63));
        sticky = t > 63 && (n & (((u128)1 << (t - 63)) - 1)) != 0;
    } else {
        q = (unsigned long long)n << (63 - t);
    }
    *out = round_q64(q, t, sticky);
    return true;
}

// m / 10^j, 1 <= j <= 38
GCV_DEC_HD double exact_div(unsigned long long m, int j)
{
    u128 d = pow10_u128(j), r = m;
    int t = 0;
    if (r >= d) {
        while ((d << 1) <= r) {
            d <<= 1;
            ++t;
        }
    } else {
        while (r < d) {
            r <<= 1;
            --t;
        }
    }
    // d <= r < 2d: the quotient's leading bit is 2^t
    unsigned long long q = 0;
    for (int i = 0; i < 64; ++i) {
        q <<= 1;
        if (r >= d) {
            q |= 1u;
            r -= d;
        }
        r <<= 1;
    }
    return round_q64(q, t, r != 0);
}

// [s, end) to the nearest double; false when the token is not a number of
// the supported form
GCV_DEC_HD bool parse_decimal(const unsigned char* s, const unsigned char* end, double* out)
{
    bool neg = false;
    if (s < end && (*s == '+' || *s == '-')) {
        neg = *s == '-';
        ++s;
    }
    unsigned long long m = 0;
    int nd = 0, zeros = 0, nfrac = 0;
    bool digits = false, frac = false;
    for (; s < end; ++s) {
        const unsigned char ch = *s;
        if (ch == '.' && !frac) {
            frac = true;
            continue;
        }
        if (ch < '0' || ch > '9') break;
        digits = true;
        nfrac += frac;
        const unsigned d = ch - '0';
        if (d == 0) {
            zeros += nd > 0;  // zeros after the first nonzero digit wait here
            continue;
        }
        if (nd + zeros + 1 > 19) return false;
        nd += zeros + 1;
        for (; zeros > 0; --zeros) m *= 10u;
        m = m * 10u + d;
    }
    if (!digits) return false;
    int x = 0;
    if (s < end && (*s == 'e' || *s == 'E')) {
        ++s;
        bool eneg = false;
        if (s < end && (*s == '+' || *s == '-')) {
            eneg = *s == '-';
            ++s;
        }
        bool ed = false;
        for (; s < end && *s >= '0' && *s <= '9'; ++s) {
            ed = true;
            if (x < 100000) x = x * 10 + (*s - '0');
        }
        if (!ed) return false;
        if (eneg) x = -x;
    }
    if (s != end) return false;
    if (m == 0) {
        *out = neg ? -0.0 : 0.0;
        return true;
    }
    const int k = x - nfrac + zeros;
    double v;
    if (m <= (1ull << 53) && k >= -22 && k <= 22) {
        // exact powers of ten 10^0 .. 10^22
        double p = 1.0;
        for (int i = 0; i < (k < 0 ? -k : k); ++i) p *= 10.0;
#ifdef __CUDA_ARCH__
        const double mv = __ull2double_rn(m);
        v = k >= 0 ? __dmul_rn(mv, p) : __ddiv_rn(mv, p);
#else
        const double mv = (double)m;
        v = k >= 0 ? mv * p : mv / p;
#endif
    } else if (k > 0 && k <= 38) {
        if (!exact_mul(m, k, &v)) return false;
    } else if (k < 0 && k >= -38) {
        v = exact_div(m, -k);
    } else if (k == 0) {
        // m > 2^53: round the integer itself
        const int t = 63 - clz64(m);
        v = round_q64(m << (63 - t), t, false);
    } else {
        return false;
    }
    *out = neg ? -v : v;
    return true;
}

#undef GCV_DEC_HD

}  // namespace gcv
