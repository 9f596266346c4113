// IEEE 754 binary64 multiplication and addition, round to nearest even, computed with integer
// operations.
//
// On this GPU FP64 instructions issue on a narrow pipe (two lanes per cycle per SM), while the
// integer pipes are many times wider. A gate pass that keeps the FP64 pipe saturated can give
// part of its multiplications and additions to these routines: both pipes then work at once,
// and the results are the same bits, because each routine rounds exactly as IEEE 754 requires.
//
// Method: the textbook construction of correctly rounded binary floating point (see J.-M. Muller
// et al., "Handbook of Floating-Point Arithmetic", ch. 7-8, and J. Hauser's SoftFloat):
//   * unpack sign, biased exponent and the 53-bit significand with its implicit leading 1;
//   * multiply: the exact 106-bit significand product from four 32x32-bit partial products;
//     add: align the smaller operand's significand to the larger one's exponent, keeping every
//     shifted-out bit as a "sticky" bit jammed into the lowest position, then add or subtract;
//   * normalise so the leading 1 sits at bit 63 of a 64-bit word; bits 63..11 are the result's
//     significand, bit 10 the round bit, bits 9..0 (with the jammed sticky) decide ties;
//   * round to nearest, ties to even, and repack; a carry out of the significand on rounding
//     lands in the exponent field by itself.
// Operands and results that are not normal numbers or zero (subnormals, infinities, NaNs, an
// exponent that would overflow or underflow) take the hardware instruction instead, so every
// input gives the IEEE result. Zero operands are handled on the integer path.
//
// Both routines are __host__ __device__: the host build is checked bit for bit against the
// host's IEEE arithmetic on random and edge-case operands.
#pragma once
#include <cstdint>
#ifdef __CUDACC__
#define SQC_HD __host__ __device__ __forceinline__
#else
#define SQC_HD inline
#endif

namespace sqc {
namespace emu {

constexpr uint64_t kSign = 0x8000000000000000ULL;
constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFULL;
constexpr uint64_t kHidden = 0x0010000000000000ULL;

SQC_HD uint64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    __builtin_memcpy(&u, &x, 8);
    return u;
#endif
}
SQC_HD double double_of(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, 8);
    return x;
#endif
}

SQC_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// The hardware operations, used for the operands the integer path does not cover.
SQC_HD double hw_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
SQC_HD double hw_add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}

// Round the normalised word x (leading 1 at bit 63; bits 9..0 include the sticky bit) to a
// 53-bit significand, ties to even, and pack it with exponent field e (1..2045) and sign s.
SQC_HD uint64_t round_pack(uint64_t s, int e, uint64_t x) {
    uint64_t m = x >> 11;
    const uint64_t rb = (x >> 10) & 1ULL;
    const uint64_t st = (x & 0x3FFULL) != 0 ? 1ULL : 0ULL;
    m += rb & (st | (m & 1ULL));
    // m is in [2^52, 2^53]; adding it to (e - 1) << 52 puts its leading 1 into the exponent
    // field (a rounding carry to 2^53 raises the exponent by one, with a zero fraction)
    return s | ((((uint64_t)(e - 1)) << 52) + m);
}

// a * b, correctly rounded (round to nearest, ties to even).
SQC_HD double mul(double a, double b) {
    const uint64_t ua = bits_of(a), ub = bits_of(b);
    const uint64_t s = (ua ^ ub) & kSign;
    const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
    const bool za = (ua << 1) == 0, zb = (ub << 1) == 0;
    if (za || zb) {
        if (ea != 0x7FF && eb != 0x7FF) return double_of(s);   // zero times a finite number
        return hw_mul(a, b);
    }
    const int e = ea + eb - 1023;
    // normal operands whose product stays normal (e + 1 is the largest exponent it can take)
    if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(e - 1) >= 2044u)
        return hw_mul(a, b);
    const uint64_t ma = (ua & kFrac) | kHidden, mb = (ub & kFrac) | kHidden;
    const uint32_t al = (uint32_t)ma, ah = (uint32_t)(ma >> 32);
    const uint32_t bl = (uint32_t)mb, bh = (uint32_t)(mb >> 32);
    const uint64_t ll = (uint64_t)al * bl;
    const uint64_t mid = (uint64_t)al * bh + (uint64_t)ah * bl;   // < 2^54
    const uint64_t hh = (uint64_t)ah * bh;
    const uint64_t lo = ll + (mid << 32);
    const uint64_t hi = hh + (mid >> 32) + (lo < ll ? 1ULL : 0ULL);
    // the product hi:lo lies in [2^104, 2^106); keep its top 64 bits, the rest as a sticky bit
    uint64_t x = (hi << 22) | (lo >> 42);
    x |= (lo & ((1ULL << 42) - 1)) != 0 ? 1ULL : 0ULL;
    const int t = (int)(x >> 63);   // product >= 2^105
    if (!t) x <<= 1;
    return double_of(round_pack(s, e + t, x));
}

// a + b, correctly rounded (round to nearest, ties to even).
SQC_HD double add(double a, double b) {
    uint64_t ua = bits_of(a), ub = bits_of(b);
    uint64_t aa = ua & ~kSign, ab = ub & ~kSign;
    if (aa < ab) {   // a is the operand of larger magnitude
        const uint64_t t0 = ua; ua = ub; ub = t0;
        const uint64_t t1 = aa; aa = ab; ab = t1;
    }
    const int ea = (int)(aa >> 52), eb = (int)(ab >> 52);
    if (ab == 0) {
        if (aa != 0) return double_of(ua);          // x + (+-0) = x
        return double_of(ua & ub & kSign);          // +-0 + +-0: -0 only when both are -0
    }
    // both normal (the smaller one nonzero), the result's exponent at most ea + 1 <= 2045
    if ((unsigned)(eb - 1) >= 2046u || ea >= 2045) return hw_add(a, b);
    const int d = ea - eb;
    const uint64_t A = ((aa & kFrac) | kHidden) << 9;   // leading 1 at bit 61
    uint64_t B = ((ab & kFrac) | kHidden) << 9;
    if (d >= 64) {
        B = 1;                                      // entirely below the round bit: sticky only
    } else if (d > 0) {
        const uint64_t lost = B << (64 - d);
        B = (B >> d) | (lost != 0 ? 1ULL : 0ULL);
    }
    const bool sub = ((ua ^ ub) & kSign) != 0;
    const uint64_t S = sub ? A - B : A + B;
    if (S == 0) return 0.0;                          // exact cancellation gives +0
    const int lz = clz64(S);
    const int e = ea + 2 - lz;
    if (e < 1) return hw_add(a, b);                  // the result is subnormal
    return double_of(round_pack(ua & kSign, e, S << lz));
}

SQC_HD double sub(double a, double b) { return add(a, double_of(bits_of(b) ^ kSign)); }

}  // namespace emu
}  // namespace sqc
