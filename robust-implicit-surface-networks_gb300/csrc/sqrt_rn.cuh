// Correctly rounded FP64 square root on the integer and FP32 pipes (device code; also compiled
// for the host in a test-only harness).
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and the sampled formulas take up to two square roots
// per value.  IEEE 754 defines the square root as the exact value rounded to nearest, so any
// method that delivers that rounding gives the same bits.  This one is the textbook integer
// square root (Newton's method, finished from the exact remainder) in 64-bit integer arithmetic:
//
//   s = x * 2^e, x a 53-bit integer; e made even by doubling x, so x is in [2^52, 2^54)
//   sqrt(s) = sqrt(M) * 2^(e/2 - 26), M = x * 2^52 (105 or 106 bits), sqrt(M) in [2^52, 2^53)
//   seed    R0 = rsqrt(x / 2^52) * 2^31 from the FP32 reciprocal square root; q = x * R0 * 2^-31
//   Newton  q += (M - q^2) * R0 * 2^-84, twice (1/(2q) taken as R0 * 2^-84); for a seed good to
//           2^-20 the first step leaves q within about 2^14 of sqrt(M), the second within a few units
//   fix-up  q = floor(sqrt(M)) from the exact remainder r = M - q^2, stepped until 0 <= r <= 2q
//   round   y = q + (r > q): sqrt(M) >= q + 1/2 exactly when M >= q^2 + q + 1/4, that is r >= q + 1
//           (a tie would need M = q^2 + q + 1/4, never an integer)
//   bits    ((e/2 + 1048) << 52) + y; y = 2^53 carries into the exponent
//
// Subnormal inputs are normalised first (x = m * 2^k with the leading bit moved to bit 52).  Zero,
// negative, infinite and NaN inputs are answered from their bits as IEEE 754 defines them: sqrt(+-0)
// = +-0, sqrt(+inf) = +inf, a NaN stays a (quiet) NaN, a negative input gives a NaN.  So no FP64
// instruction runs in this function.
#pragma once
#include "exact.cuh"

namespace ria {

RIA_HD uint64_t mul_hi_u64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

RIA_HD float rsqrt_seed(float u) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(u);
#else
    return 1.0f / std::sqrt(u);
#endif
}

// R0 = rsqrt(x / 2^52) * 2^31 (about 31 significant bits, as accurate as the FP32 estimate)
RIA_HD uint64_t sqrt_seed(uint64_t x) {
    const uint32_t w = (uint32_t)(x >> 53);  // 0: x / 2^52 in [1, 2); 1: in [2, 4)
    const uint32_t ub = ((127u + w) << 23) | (uint32_t)((x >> (29 + w)) & 0x7FFFFFu);
    float u;
    std::memcpy(&u, &ub, 4);
    const float r = rsqrt_seed(u);  // near (0.5, 1]
    uint32_t rb;
    std::memcpy(&rb, &r, 4);
    const int ex = (int)(rb >> 23);  // r = mantissa * 2^(ex - 150)
    return (uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << (ex - 119);
}

// M - q^2 as a 128-bit two's complement value (hi, lo), M = x * 2^52, x and q below 2^54
RIA_HD void sqrt_rem(uint64_t x, uint64_t q, int64_t& hi, uint64_t& lo) {
    const uint64_t mlo = x << 52, mhi = x >> 12;
    const uint64_t qlo = q * q, qhi = mul_hi_u64(q, q);
    lo = mlo - qlo;
    hi = (int64_t)(mhi - qhi - (mlo < qlo ? 1u : 0u));
}

// one Newton step q + (M - q^2) * R0 * 2^-84, for |M - q^2| < 2^89
RIA_HD uint64_t sqrt_newton(uint64_t x, uint64_t q, uint64_t r0) {
    int64_t hi;
    uint64_t lo;
    sqrt_rem(x, q, hi, lo);
    const int64_t d = (int64_t)(((uint64_t)hi << 38) | (lo >> 26));  // (M - q^2) >> 26
    const uint64_t mag = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
    const uint64_t step = mul_hi_u64(mag, r0 << 6);
    return d < 0 ? q - step : q + step;
}

// the square root of x * 2^e (x in [2^52, 2^54), e even) from the seed r0
RIA_HD double sqrt_rn_finish(uint64_t x, int e, uint64_t r0) {
    uint64_t q = mul_hi_u64(x << 10, r0 << 23);
    q = sqrt_newton(x, q, r0);
    q = sqrt_newton(x, q, r0);
    int64_t hi;
    uint64_t lo;
    sqrt_rem(x, q, hi, lo);
    int64_t r = (int64_t)lo;  // |M - q^2| is far below 2^63 here
    for (int i = 0; i < 8 && r < 0; ++i) {
        --q;
        r += (int64_t)(2 * q + 1);
    }
    for (int i = 0; i < 8 && r > (int64_t)(2 * q); ++i) {
        r -= (int64_t)(2 * q + 1);
        ++q;
    }
    const uint64_t y = q + (r > (int64_t)q ? 1u : 0u);
    const uint64_t out = ((uint64_t)(e / 2 + 1048) << 52) + y;
    double v;
    std::memcpy(&v, &out, 8);
    return v;
}

RIA_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// s split into x * 2^e with e even and x in [2^52, 2^54); false for zero, negative, infinite and NaN
RIA_HD bool sqrt_split(double s, uint64_t& x, int& e) {
    uint64_t b;
    std::memcpy(&b, &s, 8);
    if (b >> 63) return false;  // negative, -0 included
    const uint64_t E = b >> 52, m = b & ((1ull << 52) - 1);
    if (E == 2047) return false;  // infinite or NaN
    if (E == 0) {
        if (m == 0) return false;  // +0
        const int sh = clz64(m) - 11;  // subnormal m * 2^-1074: move the leading bit to bit 52
        x = m << sh;
        e = -1074 - sh;
    } else {
        x = m | (1ull << 52);
        e = (int)E - 1075;
    }
    if (e & 1) {
        x <<= 1;
        e -= 1;
    }
    return true;
}

// the inputs sqrt_split leaves out: +-0, +inf, NaN (quieted), negatives (a quiet NaN)
RIA_HD double sqrt_special(double s) {
    uint64_t b;
    std::memcpy(&b, &s, 8);
    const uint64_t mag = b & 0x7FFFFFFFFFFFFFFFull;
    uint64_t out = b;
    if (mag > 0x7FF0000000000000ull) out = b | (1ull << 51);  // NaN: keep its payload, quiet it
    else if (mag != 0 && (b >> 63)) out = 0x7FF8000000000000ull;  // negative: the default NaN
    double v;
    std::memcpy(&v, &out, 8);
    return v;
}

RIA_HD double sqrt_rn(double s) {
    uint64_t x;
    int e;
    if (!sqrt_split(s, x, e)) return sqrt_special(s);
    return sqrt_rn_finish(x, e, sqrt_seed(x));
}

}  // namespace ria
