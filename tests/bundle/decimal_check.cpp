// Checks gcv::parse_decimal (the Bundle reader's number conversion) against
// the C library's correctly rounded strtod on the host: random doubles
// printed with 1-19 significant digits in %g, %e and %f forms, random digit
// strings with exponents across the supported range, and hand-picked
// halfway and boundary cases.  Prints "checked N rejected R mismatched M"
// and exits non-zero on any mismatch or on a rejection inside the
// supported range.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#include "gcv_decimal.cuh"

static long long n_checked = 0, n_rejected = 0, n_bad = 0;

static void check(const std::string& s, bool must_accept)
{
    const unsigned char* b = reinterpret_cast<const unsigned char*>(s.data());
    double ours = 0.0;
    const bool ok = gcv::parse_decimal(b, b + s.size(), &ours);
    ++n_checked;
    if (!ok) {
        ++n_rejected;
        if (must_accept) {
            ++n_bad;
            if (n_bad < 20) std::printf("rejected %s\n", s.c_str());
        }
        return;
    }
    const double ref = std::strtod(s.c_str(), nullptr);
    uint64_t a, r;
    std::memcpy(&a, &ours, 8);
    std::memcpy(&r, &ref, 8);
    if (a != r) {
        ++n_bad;
        static int shown = 0;
        if (shown++ < 20) std::printf("mismatch %s: %.17g vs %.17g\n", s.c_str(), ours, ref);
    }
}

int main(int argc, char** argv)
{
    const long long n = argc > 1 ? std::atoll(argv[1]) : 200000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    // |v| within 1e-18 .. 1e18: at most 19 significant digits keep the
    // decimal exponent of the last digit within -38 .. 18
    std::uniform_real_distribution<double> lg(-18.0, 18.0);
    std::uniform_int_distribution<int> wide(-40, 40), nd(1, 19), form(0, 2);
    char buf[128];
    for (long long i = 0; i < n; ++i) {
        const double v = (u(rng) < 0 ? -1.0 : 1.0) * std::pow(10.0, lg(rng));
        const int d = nd(rng), f = form(rng);
        if (f == 0) std::snprintf(buf, sizeof buf, "%.*g", d, v);
        else if (f == 1) std::snprintf(buf, sizeof buf, "%.*e", d - 1, v);
        else std::snprintf(buf, sizeof buf, "%.*f", d, v);
        // inside the supported range unless %f wrote more than 19 significant digits
        std::string s(buf);
        int sig = 0;
        bool lead = true;
        for (char c : s)
            if (c >= '0' && c <= '9') {
                if (c != '0') lead = false;
                if (!lead) ++sig;
            } else if (c == 'e') {
                break;
            }
        check(s, sig <= 19);
        // wider magnitudes: whatever is accepted must match
        std::snprintf(buf, sizeof buf, "%.*g", d, u(rng) * std::pow(10.0, wide(rng)));
        check(buf, false);
    }
    // random digit strings: up to 19 digits, exponents -38 .. 19 keep m * 10^k
    // inside the supported range
    std::uniform_int_distribution<int> dig(0, 9), ke(-38, 19);
    for (long long i = 0; i < n; ++i) {
        std::string s;
        const int len = nd(rng);
        for (int j = 0; j < len; ++j) s += char('0' + dig(rng));
        s += "e" + std::to_string(ke(rng) - 0);
        check(s, true);
    }
    // halfway cases between neighbouring doubles near 1, 2^53 and 10^-5
    const char* fixed[] = {"9007199254740993", "9007199254740995", "1.00000000000000011102230246251565",
                           "0.1", "0.2", "0.3", "1e22", "1e23", "5e-324", "2.2250738585072014e-308",
                           "123456789012345678", "1234567890123456789", "0.000852558", "-0", "+7", ".5", "5.",
                           "1.5E+3", "8.82678", "17976931348623157", "4.9406564584124654e-18",
                           "9.999999999999999e37", "1e38", "1e-38", "3.4028236692093846346e38"};
    for (const char* s : fixed) check(s, false);
    // malformed tokens must be rejected
    const char* bad[] = {"", "-", ".", "e5", "1e", "1e+", "1.2.3", "0x10", "nan", "inf", "1,5", "--1", "12a"};
    for (const char* s : bad) {
        const unsigned char* b = reinterpret_cast<const unsigned char*>(s);
        double v;
        if (gcv::parse_decimal(b, b + std::strlen(s), &v)) {
            ++n_bad;
            std::printf("accepted malformed %s\n", s);
        }
    }
    std::printf("checked %lld rejected %lld mismatched %lld\n", n_checked, n_rejected, n_bad);
    return n_bad == 0 ? 0 : 1;
}
