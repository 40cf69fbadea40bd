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

// The most significant 32 bits of hi:lo shifted left by c (0 <= c < 32).
MGB_HD uint32_t x96_shl_funnel(uint32_t lo, uint32_t hi, int c) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, (unsigned)c);
#else
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << c) >> 32);
#endif
}

// X * 2^E for the 96-bit two's-complement integer X = w2:w1:w0 (|X| < 2^95),
// rounded to nearest, ties to even, including subnormal results and overflow
// to infinity; X = 0 gives +0. Integer operations only: GB300 retires about
// two FP64 operations per cycle per SM, and a short-K tile writes thousands
// of outputs per CTA. This is the general routine with a branch per case;
// the epilogue runs x96_ldexp_bits_fast and comes here only for subnormal
// results.
MGB_HD double x96_ldexp_rn_general(uint32_t w0, uint32_t w1, uint32_t w2, int E) {
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

// The bits of x96_ldexp_rn(w0, w1, w2, E) as straight-line code for every
// result that is not subnormal (normal, infinite, or +0 for X = 0); raises
// `slow` for a subnormal result, whose bits it does not compute. |X| is
// normalised so that its leading one is bit 95 (whole words by selects, then
// a funnel shift), which puts the 53-bit significand, the guard bit and the
// sticky bits at fixed places. Without branches, the conversions of the
// columns a thread writes are independent instruction streams that the
// compiler interleaves.
MGB_HD uint64_t x96_ldexp_bits_fast(uint32_t w0, uint32_t w1, uint32_t w2, int E, bool &slow) {
    const uint32_t neg = w2 >> 31, flip = 0u - neg;
    // |X| = (X ^ flip) + neg over 96 bits
    uint32_t a0 = w0 ^ flip, a1 = w1 ^ flip, a2 = w2 ^ flip;
    uint64_t t = (uint64_t)a0 + neg;
    a0 = (uint32_t)t;
    t = (uint64_t)a1 + (t >> 32);
    a1 = (uint32_t)t;
    a2 += (uint32_t)(t >> 32);
    int words = 0;  // 32-bit words shifted in from below
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const bool up = a2 == 0;
        a2 = up ? a1 : a2;
        a1 = up ? a0 : a1;
        a0 = up ? 0u : a0;
        words += up ? 1 : 0;
    }
    const int c = x96_clz32(a2) & 31;  // a2 is zero only for X = 0
    a2 = x96_shl_funnel(a1, a2, c);
    a1 = x96_shl_funnel(a0, a1, c);
    a0 <<= c;
    const int be = 95 - 32 * words - c + E + 1023;  // biased exponent of a normal result
    const uint64_t sig = ((uint64_t)a2 << 21) | (a1 >> 11);  // bits 95..43
    const uint32_t guard = (a1 >> 10) & 1u;                 // bit 42
    const uint32_t sticky = ((a1 & 0x3FFu) | a0) != 0u;      // bits 41..0
    const uint64_t m = sig + (guard & (sticky | (uint32_t)(sig & 1u)));
    const uint64_t inf = 0x7FF0000000000000ull;
    // a carry out of the significand bumps the exponent field
    uint64_t bits = ((uint64_t)(uint32_t)(be - 1) << 52) + m;
    bits = (be >= 2047 || bits > inf) ? inf : bits;
    const bool zero = (w0 | w1 | w2) == 0u;
    slow = slow || (!zero && be < 1);
    return zero ? 0ull : bits | ((uint64_t)neg << 63);
}

MGB_HD double x96_ldexp_rn(uint32_t w0, uint32_t w1, uint32_t w2, int E) {
    bool slow = false;
    const uint64_t b = x96_ldexp_bits_fast(w0, w1, w2, E, slow);
    return slow ? x96_ldexp_rn_general(w0, w1, w2, E) : x96_bits_to_double(b);
}

}  // namespace mgb
