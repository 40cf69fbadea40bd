// Fixed-point sums of float64 values on the integer pipes, for the unary
// reductions (traces, partial sums) of Float64 / ComplexF64 tensors. GB300
// retires about two FP64 operations per clock per SM, so a sum that adds one
// FP64 value per element is bound by the FP64 pipe at about half the HBM
// rate. Here each value is aligned to the running largest exponent and added
// into a 128-bit two's-complement integer with integer instructions only.
//
// The sum is A * 2^(e - 1075 - kFxFrac): e is the largest biased exponent
// seen (at least 1, the exponent of the subnormals), A a 128-bit integer.
// A value with biased exponent be contributes its 53-bit significand shifted
// left by kFxFrac - (e - be) (right when that is negative); values within
// kFxFrac binades of the largest are added exactly, smaller ones are
// truncated below 2^-kFxFrac units in the last place of the largest (a
// relative 2^-62 of the largest term per term, where an FP64 sum rounds by
// up to 2^-53 of the running sum per term). Contributions stay below 2^63,
// so 2^63 of them cannot overflow A. The result is rounded once, to nearest
// with ties to even. Inf and NaN elements set flags that decide the result
// as in an FP64 sum (Inf, -Inf, or NaN for NaN or Inf - Inf). Host and
// device alike, so that the arithmetic is checked on the CPU against exact
// rational sums.
#pragma once

#include <cstdint>
#include <cstring>

#include "mgb_x96.h"

namespace mgb {

constexpr int kFxFrac = 10;

// Non-finite elements seen, as flags (integer work, so that no FP64
// instruction sits in the per-element path, not even a predicated one).
constexpr uint32_t kFxPosInf = 1, kFxNegInf = 2, kFxNaN = 4;

struct FxSum {
    uint64_t lo;
    int64_t hi;
    int32_t e;
    uint32_t flags;  // kFxPosInf | kFxNegInf | kFxNaN
};

MGB_HD uint64_t fx_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

MGB_HD FxSum fx_zero() { return FxSum{0ull, 0ll, 1, 0u}; }

// A >>= d (arithmetic, d >= 0)
MGB_HD void fx_shr(FxSum &a, int d) {
    if (d <= 0) return;
    if (d >= 128) {
        a.lo = a.hi < 0 ? ~0ull : 0ull;
        a.hi = a.hi < 0 ? -1ll : 0ll;
    } else if (d >= 64) {
        a.lo = (uint64_t)(a.hi >> (d - 64));
        a.hi = a.hi >> 63;
    } else {
        a.lo = (a.lo >> d) | ((uint64_t)a.hi << (64 - d));
        a.hi = a.hi >> d;
    }
}

MGB_HD void fx_add128(FxSum &a, uint64_t lo, uint64_t hi) {
    const uint64_t s = a.lo + lo;
    const uint64_t carry = s < lo ? 1ull : 0ull;
    a.lo = s;
    a.hi = (int64_t)((uint64_t)a.hi + hi + carry);
}

// The signed significand scaled by 2^kFxFrac (below 2^63), shifted right
// (arithmetically) by the distance to the largest exponent, and added into
// the 128-bit sum with its sign extended. Straight-line apart from the two
// rare cases: a non-finite value, a new largest exponent.
MGB_HD void fx_push(FxSum &a, double x) {
    const uint64_t b = fx_bits(x);
    const int be = (int)((b >> 52) & 0x7FF);
    if (be == 0x7FF) {
        a.flags |= (b & 0xFFFFFFFFFFFFFull) ? kFxNaN : ((b >> 63) ? kFxNegInf : kFxPosInf);
        return;
    }
    const int bn = be ? be : 1;  // subnormals share the exponent of 2^-1022
    if (bn > a.e) {
        fx_shr(a, bn - a.e);
        a.e = bn;
    }
    const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | ((uint64_t)(be != 0) << 52);
    const int64_t sgn = (int64_t)b >> 63;  // 0 or -1
    const int64_t v = ((int64_t)(m << kFxFrac) ^ sgn) - sgn;
    const int d = a.e - bn < 63 ? a.e - bn : 63;
    const int64_t c = v >> d;
    fx_add128(a, (uint64_t)c, (uint64_t)(c >> 63));
}

MGB_HD void fx_merge(FxSum &a, FxSum b) {
    if (b.e > a.e) {
        fx_shr(a, b.e - a.e);
        a.e = b.e;
    } else {
        fx_shr(b, a.e - b.e);
    }
    fx_add128(a, b.lo, (uint64_t)b.hi);
    a.flags |= b.flags;
}

// A * 2^(e - 1075 - kFxFrac) rounded to float64 (nearest, ties to even),
// with overflow to infinity and subnormal results; a zero sum gives +0.
MGB_HD double fx_value(const FxSum &a) {
    if (a.flags) {  // as an FP64 sum: Inf - Inf and any NaN give NaN
        const bool nan = (a.flags & kFxNaN) || (a.flags & (kFxPosInf | kFxNegInf)) == (kFxPosInf | kFxNegInf);
        return x96_bits_to_double(nan ? 0x7FF8000000000000ull
                                      : ((a.flags & kFxNegInf) ? 0xFFF0000000000000ull : 0x7FF0000000000000ull));
    }
    const bool neg = a.hi < 0;
    uint64_t ml = a.lo, mh = (uint64_t)a.hi;
    if (neg) {
        ml = ~ml + 1ull;
        mh = ~mh + (ml == 0 ? 1ull : 0ull);
    }
    if (mh == 0 && ml == 0) return 0.0;
    const int p = mh ? 127 - x96_clz64(mh) : 63 - x96_clz64(ml);  // leading one
    int be = p + a.e - 1075 - kFxFrac + 1023;                      // biased exponent of the result
    uint64_t bits;
    if (be >= 1) {
        const int sh = 127 - p;  // leading one to bit 127
        uint64_t nh, nl;
        if (sh >= 64) {
            nh = ml << (sh - 64);
            nl = 0;
        } else if (sh > 0) {
            nh = (mh << sh) | (ml >> (64 - sh));
            nl = ml << sh;
        } else {
            nh = mh;
            nl = ml;
        }
        uint64_t mant = nh >> 11;  // bits 127..75: 53 bits with the leading one
        const bool round = (nh >> 10) & 1ull;
        const bool sticky = (nh & 0x3FFull) != 0 || nl != 0;
        if (round && (sticky || (mant & 1ull))) {
            ++mant;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                ++be;
            }
        }
        if (be >= 2047) return x96_bits_to_double((neg ? 1ull << 63 : 0ull) | 0x7FF0000000000000ull);
        bits = ((uint64_t)be << 52) | (mant & 0xFFFFFFFFFFFFFull);
    } else {
        // subnormal: round(|A| * 2^(e - 1 - kFxFrac)) units of 2^-1074
        const int sh = kFxFrac + 1 - a.e;
        uint64_t q;
        if (sh <= 0) {
            q = ml << (-sh);  // exact: the result is below 2^52 units
        } else {
            q = (ml >> sh) | (sh < 64 ? (mh << (64 - sh)) : 0ull);
            const bool round = (ml >> (sh - 1)) & 1ull;
            const bool sticky = sh > 1 && (ml & ((1ull << (sh - 1)) - 1ull)) != 0;
            if (round && (sticky || (q & 1ull))) ++q;  // 2^52 becomes the smallest normal
        }
        bits = q;
    }
    if (neg) bits |= 1ull << 63;
    return x96_bits_to_double(bits);
}

}  // namespace mgb
