// 96-bit two's-complement accumulators of the exact (Ozaki) GEMM epilogue and
// their conversion to float64, written for host and device alike so that the
// conversion can be checked on the CPU against exact rational arithmetic.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define MGB_HD __host__ __device__ __forceinline__
#else
#define MGB_HD inline
#endif

namespace mgb {

MGB_HD int x96_clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __clz((int)v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}
MGB_HD int x96_clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
MGB_HD double x96_bits_to_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

// X * 2^E for the 96-bit two's-complement integer X = w2:w1:w0 (|X| < 2^95),
// rounded to nearest, ties to even, including subnormal results and overflow
// to infinity; X = 0 gives +0. Integer operations only: GB300 retires about
// two FP64 operations per cycle per SM, and a short-K tile writes thousands
// of outputs per CTA.
MGB_HD double x96_ldexp_rn(uint32_t w0, uint32_t w1, uint32_t w2, int E) {
    const uint64_t neg = w2 >> 31;
    uint64_t lo = ((uint64_t)w1 << 32) | w0;
    uint32_t hi = w2;
    if (neg) {  // |X| = ~X + 1 over 96 bits
        lo = ~lo + 1;
        hi = ~hi + (lo == 0 ? 1u : 0u);
    }
    int p;  // position of the leading one of |X|
    if (hi) p = 64 + 31 - x96_clz32(hi);
    else if (lo) p = 63 - x96_clz64(lo);
    else return 0.0;
    // biased exponent of a normal result; subnormals keep the fixed unit 2^-1074
    const int be = p + E + 1023;
    int field = be - 1;
    int sh = p - 52;  // right shift that leaves the 53-bit significand
    if (be < 1) {
        sh += 1 - be;
        field = 0;
    }
    uint64_t m;
    if (sh <= 0) {
        m = lo << (-sh);  // p <= 52: |X| lies in lo
    } else if (sh >= 96) {
        m = 0;  // |X| < 2^95 <= half of the last kept unit
    } else {
        m = sh < 64 ? (lo >> sh) | (sh ? (uint64_t)hi << (64 - sh) : 0) : (uint64_t)(hi >> (sh - 64));
        const int gb = sh - 1;  // guard bit, then the sticky bits below it
        const uint64_t guard = gb < 64 ? (lo >> gb) & 1u : (uint64_t)(hi >> (gb - 64)) & 1u;
        bool sticky;
        if (gb == 0) sticky = false;
        else if (gb < 64) sticky = (lo & ((uint64_t(1) << gb) - 1)) != 0;
        else if (gb == 64) sticky = lo != 0;
        else sticky = lo != 0 || (hi & ((1u << (gb - 64)) - 1)) != 0;
        m += guard & (uint64_t)(sticky || (m & 1u));
    }
    uint64_t bits;
    if (field >= 2047) bits = 0x7FF0000000000000ull;
    else bits = ((uint64_t)field << 52) + m;  // a carry out of the significand bumps the exponent
    if (bits > 0x7FF0000000000000ull) bits = 0x7FF0000000000000ull;
    return x96_bits_to_double(bits | (neg << 63));
}

}  // namespace mgb
