// Exact, order-independent sums of products on the device (norms, probabilities, state
// comparisons).
//
// The live-bucket list, and so the order in which a kernel meets the keys, depends on how
// concurrent claims interleaved. A floating-point sum over that order differs in its last bits
// from run to run, and a measurement outcome decided by p1 = |proj|^2 / norm could follow it.
// Here every product x*y is added exactly (its full 106-bit significand product) to a
// fixed-point number whose least significant bit is 2^kSumLsb; the number is kept as
// kSumChunks 32-bit pieces in 64-bit counters, added as integers (associative and
// commutative) and carried on the host. Products below 2^kSumLsb lose their low bits the same
// way in every order; the range is |sum| < 2^63. A negative product is added as its two's
// complement modulo 2^(32 * kSumChunks). The host rounds the exact total to the nearest double
// once (exact_sum_value), so the result depends only on the set of (key, amplitude) entries.
#pragma once
#include <cstdint>
#include "sqc_types.h"

namespace sqc {

#ifdef __CUDACC__
// acc += x * y exactly (x, y finite).
__device__ __forceinline__ void exact_add_prod(unsigned long long (&acc)[kSumChunks], double x, double y) {
    const unsigned long long ux = (unsigned long long)__double_as_longlong(x);
    const unsigned long long uy = (unsigned long long)__double_as_longlong(y);
    const unsigned long long ax = ux & 0x7FFFFFFFFFFFFFFFULL, ay = uy & 0x7FFFFFFFFFFFFFFFULL;
    if (!ax || !ay) return;
    const int ex = (int)(ax >> 52), ey = (int)(ay >> 52);
    const unsigned long long mx = (ax & 0x000FFFFFFFFFFFFFULL) | (ex ? 0x0010000000000000ULL : 0ULL);
    const unsigned long long my = (ay & 0x000FFFFFFFFFFFFFULL) | (ey ? 0x0010000000000000ULL : 0ULL);
    unsigned long long lo = mx * my, hi = __umul64hi(mx, my);   // the exact product, < 2^106
    // position of the product's least significant bit relative to 2^kSumLsb
    int pos = (ex ? ex : 1) + (ey ? ey : 1) - 2 * 1075 - kSumLsb;
    if (pos < 0) {   // bits below 2^kSumLsb are dropped
        const int r = -pos;
        if (r >= 128) return;
        if (r >= 64) { lo = hi >> (r - 64); hi = 0; }
        else { lo = (lo >> r) | (r ? hi << (64 - r) : 0ULL); hi = r ? hi >> r : hi; }
        pos = 0;
        if (!lo && !hi) return;
    }
    const int k = pos >> 5, sh = pos & 31;
    // (hi:lo) << sh as five 32-bit words w0..w4 (at most 137 bits)
    const unsigned long long l2 = lo << sh;
    const unsigned long long h2 = (hi << sh) | (sh ? lo >> (64 - sh) : 0ULL);
    const unsigned long long w0 = l2 & 0xFFFFFFFFULL, w1 = l2 >> 32, w2 = h2 & 0xFFFFFFFFULL, w3 = h2 >> 32;
    const unsigned long long w4 = sh ? (hi >> (64 - sh)) : 0ULL;
    const bool negative = ((ux ^ uy) >> 63) != 0;
    // a negative product goes in as ~P + 1 modulo 2^(32 * kSumChunks): the complement of every
    // 32-bit piece (0xFFFFFFFF where P has none), plus one at the lowest piece
#pragma unroll
    for (int i = 0; i < kSumChunks; ++i) {
        const int d = i - k;
        unsigned long long w = d == 0 ? w0 : d == 1 ? w1 : d == 2 ? w2 : d == 3 ? w3 : d == 4 ? w4 : 0ULL;
        if (negative) w = (~w & 0xFFFFFFFFULL) + (i == 0 ? 1ULL : 0ULL);
        acc[i] += w;
    }
}

// Add a warp's accumulators into the global sum (every lane calls it).
__device__ __forceinline__ void exact_flush(unsigned long long (&acc)[kSumChunks], unsigned long long* out) {
#pragma unroll
    for (int i = 0; i < kSumChunks; ++i) {
        unsigned long long v = acc[i];
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(out + i, v);
    }
}
#endif

// The exact total of an accumulator (its pieces carried, read as a two's complement number),
// rounded to the nearest double, ties to even. Host code.
double exact_sum_value(const unsigned long long* acc);

}  // namespace sqc
