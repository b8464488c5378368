// Host check of csrc/exact_int.h: mul6 and mul_pow2 against the host's IEEE
// binary64 multiply (round to nearest even), bit for bit, on random bit
// patterns, random moderate values, constructed rounding ties at every
// exponent near the ends of the range, and the special values.  Prints the
// count checked and the count that differ; exits non-zero on a difference.
#include "../1dsweptcuda_gb300/csrc/exact_int.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using sw::f64_bits;
using sw::f64_from_bits;

static long n_checked = 0, n_bad = 0;

static bool same(double a, double b) { return f64_bits(a) == f64_bits(b) || (std::isnan(a) && std::isnan(b)); }

static void check(double x) {
    ++n_checked;
    if (!same(sw::mul6(x), x * 6.0)) {
        if (n_bad++ < 5) std::printf("mul6(%a) = %a, multiply gives %a\n", x, sw::mul6(x), x * 6.0);
    }
    for (int k = -3; k <= 5; ++k) {
        const double f = std::ldexp(1.0, k);
        if (!same(sw::mul_pow2(x, f, k), x * f)) {
            if (n_bad++ < 5) std::printf("mul_pow2(%a, 2^%d) = %a, multiply gives %a\n", x, k, sw::mul_pow2(x, f, k), x * f);
        }
    }
}

int main(int argc, char **argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 g(20261204);
    for (long i = 0; i < n; ++i) check(f64_from_bits(g()));
    for (long i = 0; i < n; ++i) {
        const double m = std::ldexp((double)(g() >> 11), -53);
        check((g() & 1 ? 1.0 : -1.0) * std::ldexp(m, (int)(g() % 40) - 20));
    }
    const int exps[] = {1, 2, 3, 1000, 1023, 2040, 2041, 2042, 2043, 2044, 2045, 2046};
    for (long i = 0; i < n / 10; ++i) {
        const uint64_t m = g() & 0x000ffffffffffffcull;
        for (uint64_t lo = 0; lo < 4; ++lo)
            for (int e : exps) {
                const double x = f64_from_bits(((uint64_t)e << 52) | m | lo);
                check(x);
                check(-x);
            }
    }
    const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 4.9e-324, 2.2250738585072014e-308,
                              2.225073858507201e-308, 1.7976931348623157e308, 1e308 / 6, 3e307, 1.0, -1.0, 0.5};
    for (double x : special) check(x);
    std::printf("checked %ld, differ %ld\n", n_checked, n_bad);
    return n_bad != 0;
}
