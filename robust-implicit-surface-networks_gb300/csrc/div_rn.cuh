// Correctly rounded FP64 division on the integer and FP32 pipes (device code; also compiled for the
// host in a test-only harness).
//
// The vertex coordinates divide by the differences of the function values, and GB300 issues FP64 at
// a small fraction of its integer rate: a division on the FP64 pipe is a chain of about a dozen FP64
// operations, which bound the vertex emission.  IEEE 754 defines the quotient as the exact value
// rounded to nearest even, so any method that delivers that rounding gives the same bits.  This one
// is the textbook reciprocal method in 64-bit integer arithmetic, finished from the exact remainder:
//
//   a = ma * 2^(ea-1075), b = mb * 2^(eb-1075), ma and mb 53-bit integers in [2^52, 2^53)
//   n = ma (or 2 ma when ma < mb), so that n / mb is in [1, 2)
//   R ~ 2^115 / mb in (2^62, 2^63]: seed from the FP32 reciprocal of mb's leading 24 bits (about 21
//     correct bits), then two Newton steps R += R (2^115 - mb R) / 2^115 (about 42, then about 60 bits)
//   q = floor(n 2^53 / mb) in [2^53, 2^54): first n R / 2^62 (off by at most a few units), then fixed
//     from the exact remainder r = n 2^53 - q mb (its low 64 bits suffice: |r| is far below 2^63)
//     until 0 <= r < mb
//   round   the 53-bit significand is q >> 1; it rounds up when the dropped half (q & 1, with r as the
//           sticky part) exceeds one half, or equals it and the significand is odd
//   bits    sign | ((E - 1) << 52) + significand, E = ea - eb + 1023 (1022 when n = 2 ma); a carry
//           to 2^53 moves into the exponent
//
// Zero, subnormal, infinite and NaN operands, and quotients outside the normal range, go to the FP64
// instruction, which defines them.
#pragma once
#include "sqrt_rn.cuh"

namespace ria {

RIA_HD double div_f64_pipe(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}

RIA_HD float rcp_seed(float u) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(u);
#else
    return 1.0f / u;
#endif
}

// R0 ~ 2^115 / mb from the FP32 reciprocal of mb / 2^29 (exact: mb's leading 24 bits)
RIA_HD uint64_t div_seed(uint64_t mb) {
    const float f = (float)(uint32_t)(mb >> 29);  // in [2^23, 2^24)
    const float r = rcp_seed(f);                  // in (2^-24, 2^-23]
    uint32_t rb;
    std::memcpy(&rb, &r, 4);
    const int ex = (int)(rb >> 23);  // r = mant * 2^(ex - 150)
    const uint64_t mant = (rb & 0x7FFFFFu) | 0x800000u;
    // R0 = r * 2^86 = mant * 2^(ex - 64)
    return mant << (ex - 64);
}

// one Newton step of the reciprocal R ~ 2^115 / mb
RIA_HD uint64_t div_newton(uint64_t mb, uint64_t R) {
    const uint64_t plo = mb * R, phi = mul_hi_u64(mb, R);  // mb R, about 2^115
    // e = 2^115 - mb R as a 128-bit two's complement value, then e >> 31 (|e| < 2^94)
    const uint64_t elo = (uint64_t)0 - plo;
    const uint64_t ehi = (1ull << 51) - phi - (plo != 0 ? 1u : 0u);
    const int64_t e = (int64_t)((ehi << 33) | (elo >> 31));
    const uint64_t mag = e < 0 ? (uint64_t)0 - (uint64_t)e : (uint64_t)e;
    const uint64_t corr = mul_hi_u64(R, mag) >> 20;  // R e / 2^115
    return e < 0 ? R - corr : R + corr;
}

// a / b, rounded to nearest even, on the integer and FP32 pipes
RIA_HD double div_rn(double a, double b) {
    uint64_t x, y;
    std::memcpy(&x, &a, 8);
    std::memcpy(&y, &b, 8);
    const uint32_t ex = (uint32_t)(x >> 52) & 0x7FF, ey = (uint32_t)(y >> 52) & 0x7FF;
    // exponent fields 1..2046 only: zeros, subnormals, infinities and NaNs go to the FP64 pipe
    if (ex - 1 >= 2046u || ey - 1 >= 2046u) return div_f64_pipe(a, b);
    const uint64_t frac = (1ull << 52) - 1;
    const uint64_t ma = (x & frac) | (1ull << 52), mb = (y & frac) | (1ull << 52);
    const bool lower = ma < mb;
    const uint64_t n = lower ? ma << 1 : ma;  // n / mb in [1, 2)
    const int E = (int)ex - (int)ey + (lower ? 1022 : 1023);
    if (E < 1 || E > 2045) return div_f64_pipe(a, b);  // subnormal or (near) overflowing quotient
    uint64_t R = div_seed(mb);
    R = div_newton(mb, R);
    R = div_newton(mb, R);
    uint64_t q = mul_hi_u64(n << 2, R);  // n 2^53 / mb, within a few units
    int64_t r = (int64_t)((n << 53) - q * mb);
    for (int i = 0; i < 8 && r < 0; ++i) {
        --q;
        r += (int64_t)mb;
    }
    for (int i = 0; i < 8 && r >= (int64_t)mb; ++i) {
        ++q;
        r -= (int64_t)mb;
    }
    const uint64_t m = q >> 1;
    const uint64_t up = ((q & 1) && (r != 0 || (m & 1))) ? 1u : 0u;
    const uint64_t out = ((x ^ y) & (1ull << 63)) | (((uint64_t)(E - 1) << 52) + m + up);
    double v;
    std::memcpy(&v, &out, 8);
    return v;
}

}  // namespace ria
