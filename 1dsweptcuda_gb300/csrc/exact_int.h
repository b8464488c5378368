// FP64 products formed on the integer pipe, rounded exactly as the FP64
// multiply rounds them (IEEE 754 binary64, round to nearest even).
//
// On GB300 an FP64 warp instruction holds its SM sub-partition's FP64 pipe for
// 64 cycles, while integer instructions issue at up to one per cycle on
// another pipe.  The FP64 stencils are bound by the FP64 pipe, so a product
// that can be formed from the operand's bits with a handful of integer
// instructions frees FP64 time without changing a bit of the result:
//
//  * mul_pow2(x, f, k): x * f for f = 2^k.  For a normal x whose product is
//    normal, the product is exact and only adds k to the exponent field.
//  * mul6(x): x * 6.  The significand M (53 bits, leading one included) times
//    3 has 54 or 55 bits; it is shifted back to 53 bits and rounded to nearest,
//    ties to even, from the bits shifted out, and the exponent grows by the
//    shift plus one (the factor 2 of 6 = 2 * 3, exact).
//
// Zeros, subnormals, infinities, NaNs and products outside the normal range
// take the FP64 multiply itself (volatile inline PTX, so the compiler keeps
// that multiply inside its branch instead of computing it for every lane).
// The same functions compile for the host, where tests compare them with the
// host's multiply over random and edge-case operands.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SW_HD __host__ __device__ __forceinline__
#else
#define SW_HD inline
#endif

namespace sw {

SW_HD uint64_t f64_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
SW_HD double f64_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}
// The FP64 multiply, kept where it is written.
SW_HD double f64_mul_pipe(double a, double b) {
#if defined(__CUDA_ARCH__)
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
#else
    volatile double va = a;
    return va * b;
#endif
}

// x * f with f = 2^k (|k| < 1023).
SW_HD double mul_pow2(double x, double f, int k) {
    const uint64_t b = f64_bits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((unsigned)(e - 1) < 2046u && (unsigned)(e + k - 1) < 2046u)
        return f64_from_bits(b + ((uint64_t)(int64_t)k << 52));
    return f64_mul_pipe(x, f);
}

// x * 6.
SW_HD double mul6(double x) {
    const uint64_t b = f64_bits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((unsigned)(e - 1) < 2043u) {  // normal x and a normal product: e + 3 <= 2046
        const uint64_t m = (b & 0x000fffffffffffffull) | 0x0010000000000000ull;  // 53-bit significand
        const uint64_t p = m * 3u;                                               // 54 or 55 bits
        const int s = (p >> 54) ? 2 : 1;                                         // bits to drop
        uint64_t q = p >> s;
        const uint64_t rem = p & ((1ull << s) - 1), half = 1ull << (s - 1);
        q += (rem > half || (rem == half && (q & 1))) ? 1u : 0u;
        int ex = e + s;  // 3x's exponent ...
        if (q >> 53) {   // rounding carried into a 54th bit
            q >>= 1;
            ++ex;
        }
        ex += 1;  // ... times 2
        return f64_from_bits((b & 0x8000000000000000ull) | ((uint64_t)ex << 52) | (q & 0x000fffffffffffffull));
    }
    return f64_mul_pipe(x, 6.0);
}

// ---- the general product on the integer pipe
//
// mul_int_fast(x, y, bad) = x * y, rounded once, for normal operands whose
// product is normal (biased exponent at most 2045 before rounding).  The two
// significands, each shifted to bit 63, give a 128-bit product whose upper
// word holds the leading 64 bits (the leading one at bit 63 or 62); the lower
// word only decides whether the discarded part is zero (the sticky bit of
// round to nearest, ties to even).  For anything else -- zeros, subnormals,
// infinities, NaNs, a product near or outside the ends of the normal range --
// it sets bad and its result is meaningless: the caller recomputes that value
// with the FP64 multiply.  No FP64 instruction sits on its path, so none is
// issued: a predicated-off FP64 instruction still holds the FP64 pipe, and a
// fallback inside this function measured as slow as the multiply it replaces.
// The check is kept to three comparisons: the integer pipe is nearly as busy
// as the FP64 pipe in the KS kernels, and handling zeros here (rare in those
// products) cost more than it saved.
// mul_int(x, y) is the same product with that fallback inside (host checks).
SW_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

constexpr uint64_t kSign = 0x8000000000000000ull, kAbs = 0x7fffffffffffffffull;
constexpr uint64_t kMant = 0x000fffffffffffffull, kHidden = 0x0010000000000000ull;

SW_HD double mul_int_fast(double x, double y, uint32_t &bad) {
    const uint64_t a = f64_bits(x), b = f64_bits(y);
    const int ea = (int)(a >> 52) & 0x7ff, eb = (int)(b >> 52) & 0x7ff;
    const uint64_t A = ((a & kMant) | kHidden) << 11, B = ((b & kMant) | kHidden) << 11;
    const uint64_t hi = umulhi64(A, B), lo = A * B;
    const int top = (int)(hi >> 63);  // the product's leading one at bit 127 (else 126)
    const uint64_t n = top ? hi : (hi << 1) | (lo >> 63), below = top ? lo : lo << 1;
    uint64_t m = n >> 11;
    const uint32_t rem = (uint32_t)n & 0x7ffu;
    m += (uint64_t)((rem > 0x400u) | ((rem == 0x400u) & ((below != 0) | ((uint32_t)m & 1u))));
    const int er = ea + eb - 1023 + top;
    // er <= 2045: a rounding carry leaves the exponent field at most 2046
    bad |= (uint32_t)!((unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && (unsigned)(er - 1) < 2045u);
    return f64_from_bits(((a ^ b) & kSign) | (((uint64_t)(int64_t)(er - 1) << 52) + m));
}

SW_HD double mul_int(double x, double y) {
    uint32_t bad = 0;
    const double r = mul_int_fast(x, y, bad);
    return bad ? f64_mul_pipe(x, y) : r;
}

}  // namespace sw
