// Host check of csrc/exact_int.h against the host's IEEE binary64 operations
// (round to nearest even), bit for bit: mul6, mul_pow2 and mul_int against
// the multiply, and mul_int_fast's result wherever it does not flag the
// operands as its caller's to recompute (zero operands included).  Operands:
// random bit patterns, random moderate values, significands with few bits set
// (exact products and ties), exponents near the ends of the range, and the
// special values.  Prints the count
// checked and the count that differ; exits non-zero on a difference.
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

static long n_fast = 0;
static void check2(double x, double y) {
    ++n_checked;
    const double want = x * y;
    if (!same(sw::mul_int(x, y), want)) {
        if (n_bad++ < 8) std::printf("mul_int(%a, %a) = %a, multiply gives %a\n", x, y, sw::mul_int(x, y), want);
    }
    uint32_t bad = 0;
    const double fast = sw::mul_int_fast(x, y, bad);
    if (!bad) {
        ++n_fast;
        if (!same(fast, want)) {
            if (n_bad++ < 8) std::printf("mul_int_fast(%a, %a) = %a unflagged, multiply gives %a\n", x, y, fast, want);
        }
    }
}

static double with_exp(std::mt19937_64 &g, uint64_t mant, int e) {
    return f64_from_bits(((g() & 1) ? 0x8000000000000000ull : 0) | ((uint64_t)e << 52) | (mant & 0x000fffffffffffffull));
}

static void check_pairs(std::mt19937_64 &g, long n) {
    for (long i = 0; i < n; ++i) check2(f64_from_bits(g()), f64_from_bits(g()));
    for (long i = 0; i < n; ++i) {  // moderate values
        const int e = 1023 + (int)(g() % 41) - 20, d = (int)(g() % 41) - 20;
        check2(with_exp(g, g(), e), with_exp(g, g(), e + d));
    }
    for (long i = 0; i < n; ++i) {  // few significand bits set: exact products and ties
        const int e = 1023 + (int)(g() % 21) - 10;
        const uint64_t ma = g() & (g() & 0x000fffffffffffffull) & (g() | 0x000ff00000000000ull);
        const uint64_t mb = (g() & 0x000f000000000000ull) | (g() & 1) | ((g() & 1) << 1);
        check2(with_exp(g, ma, e), with_exp(g, mb, e - (int)(g() % 5)));
        check2(with_exp(g, ma >> (g() % 52), e), with_exp(g, ma, e));
        const double v = with_exp(g, ma, e);
        check2(v, v);  // squares
    }
    const int ends[] = {1, 2, 3, 4, 5, 50, 51, 52, 53, 54, 55, 60, 500, 511, 512, 513, 1000, 1022, 1023, 1024,
                        1534, 1535, 1536, 2040, 2043, 2044, 2045, 2046};
    for (long i = 0; i < n / 4; ++i) {  // exponents near the ends of the range, and products near them
        const int e1 = ends[g() % 28], e2 = ends[g() % 28];
        check2(with_exp(g, g(), e1), with_exp(g, g(), e2));
        check2(with_exp(g, g() | 0x000fffffffff0000ull, e1), with_exp(g, g() | 0x000fffffffff0000ull, e2));
        check2(with_exp(g, g() & 0x00000000ffffffffull, e1), with_exp(g, g() & 0x00000000ffffffffull, e2));
    }
    const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 4.9e-324, 2.2250738585072014e-308,
                              2.225073858507201e-308, 1.7976931348623157e308, 8.98846567431158e307, 1.0, -1.0, 0.5,
                              1.0 + 0x1p-52, 1.0 - 0x1p-53, 3.0, 0x1p-1022, 0x1p1023, 0x1p-511, 0x1p512, 1.5e-154, 1.4e154};
    for (double x : special)
        for (double y : special) {
            check2(x, y);
            check2(x, -y);
        }
}

int main(int argc, char **argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    std::mt19937_64 g(20261204);
    check_pairs(g, n);
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
    std::printf("checked %ld (%ld unflagged fast products), differ %ld\n", n_checked, n_fast, n_bad);
    return n_bad != 0;
}
