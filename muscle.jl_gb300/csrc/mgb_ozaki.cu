// Emulated forms on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// OZAKI (Float64 / ComplexF64 results)
//   Each row m of A and column n of B gets a power-of-two scale from its
//   largest exponent; the scaled value a in [-1, 1] is cut into S signed
//   W-bit digits by round-to-nearest:  a = sum_i s_i 2^(-W i) + r,
//   |s_1| <= 2^W, |s_i| <= 2^(W-1), |r| <= 2^(-W S - 1).  W = 8 for S <= 6
//   and W = 7 for S >= 7: every digit is an integer that bf16 holds exactly,
//   every digit product is exact, and a float32 accumulator stays exact
//   while the sum of the absolute products it receives is <= 2^24.
//   Products s_i t_j with i + j = d share the scale 2^(-W d) and go to one
//   TMEM accumulator per d ("group"); pairs with i + j > S + 1 are dropped
//   (Ozaki scheme I).  Every KC embedded k (KC = 256 for W = 7, 128 for
//   W = 8) the epilogue warps read every group's float32 partial sums (exact
//   integers), convert them to int and add them, shifted left by
//   W (S + 1 - d), into one exact 96-bit integer per output element
//   (|X| < 2^(log2 K + W (S + 1) + 1) < 2^95 for any K below 2^31). X times
//   the row and column scales is rounded to float64 with integer operations
//   only (x96_ldexp_rn): no float64 arithmetic at all, since GB300's FP64
//   pipe retires about two operations per cycle per SM.
//   Group bound per k: max(d + 1, 4) * 2^(2W-2); KC * bound <= 2^24 for
//   d <= 15 (W = 7) and d <= 7 (W = 8), which covers every group of every
//   supported S (d <= S + 1).
//
// BF16X3 (Float32 / ComplexF32 results)
//   x = hi + mid + lo, three bf16 pieces (exact for normal floats); the six
//   products with piece-index sum <= 2 (0-based) are kept. The tensor core
//   accumulates in float32 with truncation, whose bias grows with the number
//   of accumulations, so the products are grouped by piece-index sum like
//   the digit groups (hi*hi alone, then sums 1 and 2), read out every
//   KC = 256 k and summed in registers with Kahan compensation.
//
// Complex operands are embedded as real GEMMs: A_e[m][2k+p] = part_p(A[m,k]),
// B_e[2n+q][2k+p] holds [[Br, -Bi], [Bi, Br]] so that C_e[m][2n+q] is part q
// of C[m,n] (4 real products per complex product, as zgemm's 4M form).
//
// Pipeline per CTA (128 x BN embedded outputs per tile, BN = 32, or 64 for
// BF16X3; a persistent grid of one CTA per SM, each walking the tiles b,
// b + grid, ... of one contraction or of a group's job table):
//   warp 0       TMA producer: one 3-D box per operand per 32-wide k block
//                loads all S slices at once into a 64B-swizzled stage;
//   warp 1       TMEM allocation, then one thread issues, per 16 k, one
//                tcgen05.mma.cta_group::1.kind::f16 per A slice i with
//                M = 128, N = BN (S - i): B slices 0 .. S-1-i lie back to
//                back in the stage and their accumulators (digit groups
//                i .. S-1) lie back to back in TMEM;
//   warp 10      (OZAKI) a second issuing thread: the two take alternate
//                k blocks;
//   warps 2..9   epilogue: tcgen05.ld 32x32b.x16 per group and column half
//                from the bank the MMAs are not writing, then tcgen05.st of
//                zeros into what was read.
// Every mbarrier wait is bounded; on timeout the CTA records
// MGB_ERR_DEVICE_TIMEOUT in the device status word, drains its copies and
// MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <map>
#include <tuple>
#include <type_traits>
#include <cstring>
#include <cmath>
#include <mutex>
#include <vector>

#include "mgb_internal.h"
#include "mgb_ptx.h"
#include "mgb_x96.h"

namespace mgb {

constexpr int OZ_KC = 256;     // BF16X3: embedded k between readouts
constexpr int OZ_BM = 128;     // rows of A per CTA (TMEM lanes)
constexpr int OZ_BK = 32;      // k per stage (64-byte swizzled rows)
constexpr int OZ_EPI_WARPS = 8;
// Row tiles per rasterisation band. The resident CTAs drift apart in k over
// many waves, so L2 keeps a band's A slices only while they are small: on the
// 8192^3 ComplexF64 case (S = 6) DRAM traffic per launch is 222 GB for bands
// of 1, 135 GB for 2, 124 GB for 3, 145 GB for 4 and 187-224 GB for 8. The
// default is the widest band up to 3 whose A slices (band x 128 rows x all
// of K x S slices) stay within OZ_BAND_BYTES: on the same case S = 8 (two
// stages, so exposed to every L2 miss) ran 173 ms with bands of 3 (96 MiB),
// 133 ms with 2 and 142 ms with 1, while S = 6 (72 MiB at 3) ran 76.0 ms
// with 3 and 78.0 ms with 2.
constexpr int OZ_GROUP_M = 3;
constexpr int64_t OZ_BAND_BYTES = 90ll << 20;  // S = 7 at K_e = 16384: 84 MiB; S = 8: 96 MiB
// warp 0 TMA, warp 1 MMA issuer (and TMEM owner), warps 2..9 epilogue,
// warp 10 second MMA issuer
constexpr int OZ_THREADS = 96 + 32 * OZ_EPI_WARPS;
constexpr int OZ_ISSUER2_WARP = 2 + OZ_EPI_WARPS;
constexpr int OZ_A_TILE = OZ_BM * OZ_BK * 2;  // 8192 bytes per slice
constexpr int OZ_SMEM_BUDGET = 220 * 1024;
constexpr int OZ_MAX_STAGES = 6;

// Columns per digit group (= embedded rows of B per CTA): two banks of S
// groups must fit the 512 TMEM columns, and one MMA covers at most 256.
// BF16X3 (S = 3, two float registers per column) takes 64; the exact forms
// keep 32, where their three 32-bit words per column stay in registers.
__host__ __device__ constexpr int oz_bn(int S, bool exact) { return (!exact && S <= 3) ? 64 : 32; }
__host__ __device__ constexpr int oz_b_tile(int S, bool exact) { return oz_bn(S, exact) * OZ_BK * 2; }  // bytes per slice
__host__ __device__ constexpr int oz_stage_bytes(int S, bool exact) { return S * (OZ_A_TILE + oz_b_tile(S, exact)); }
// Digit width and exact chunk length (in 32-wide k blocks) per slice count.
// W = 8 for S <= 6: |s1| <= 256, |si| <= 128, group bound max(d+1,4) 2^14, so a
// float32 accumulator stays exact over 4 blocks (128 k) for every d <= 7.
// W = 7 for S >= 7: group bound max(d+1,4) 2^12, exact over 8 blocks (256 k)
// for d <= 15. Both hold about the same number of mantissa bits (W S = 48 / 49).
__host__ __device__ constexpr int oz_digit_bits(int S) { return S <= 6 ? 8 : 7; }
__host__ __device__ constexpr int oz_chunk_blocks(int S) { return oz_digit_bits(S) == 8 ? 4 : 8; }
__host__ __device__ constexpr int oz_stages(int S, bool exact) {
    return (OZ_SMEM_BUDGET / oz_stage_bytes(S, exact)) < OZ_MAX_STAGES ? (OZ_SMEM_BUDGET / oz_stage_bytes(S, exact))
                                                                       : OZ_MAX_STAGES;
}
// two banks of S groups of oz_bn columns; bank bases at columns 0 and 256
__host__ __device__ constexpr int oz_tmem_cols(int) { return 512; }
// More than half of the SM's shared memory for every S, so one CTA (and one
// TMEM allocation) per SM.
__host__ __device__ constexpr int oz_smem_bytes(int S, bool exact) {
    return oz_stages(S, exact) * oz_stage_bytes(S, exact) + 1024 /*align*/ + 256 /*barriers*/;
}
static_assert(2 * oz_smem_bytes(3, true) > 228 * 1024 && 2 * oz_smem_bytes(8, true) > 228 * 1024 &&
                  2 * oz_smem_bytes(3, false) > 228 * 1024,
              "one CTA per SM");

// =============================================================================
// PTX wrappers
// =============================================================================
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *tm, int c0, int c1,
                                            int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// tcgen05.ld of 16 consecutive columns of this warp's 32 lanes (no wait)
__device__ __forceinline__ void tc_ld16_issue(uint32_t taddr, uint32_t *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
          "=r"(v[14]), "=r"(v[15])
        : "r"(taddr)
        : "memory");
}
// zeroes 16 consecutive columns of this warp's 32 lanes (no wait)
__device__ __forceinline__ void tc_st16_zero(uint32_t taddr) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr),
        "r"(0u)
        : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// NC consecutive columns (a multiple of 16), then wait for the loads
template <int NC>
__device__ __forceinline__ void tc_ld(uint32_t taddr, uint32_t (&v)[NC]) {
#pragma unroll
    for (int c = 0; c < NC; c += 16) tc_ld16_issue(taddr + c, v + c);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 96-bit two's-complement accumulation (carry chain) and conversion.
__device__ __forceinline__ void add96(uint32_t &w0, uint32_t &w1, uint32_t &w2, uint32_t a0, uint32_t a1,
                                      uint32_t a2) {
    asm("add.cc.u32 %0, %0, %3;\n\taddc.cc.u32 %1, %1, %4;\n\taddc.u32 %2, %2, %5;"
        : "+r"(w0), "+r"(w1), "+r"(w2)
        : "r"(a0), "r"(a1), "r"(a2));
}
__device__ __forceinline__ void add64hi(uint32_t &w1, uint32_t &w2, uint32_t a1, uint32_t a2) {
    asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, %3;" : "+r"(w1), "+r"(w2) : "r"(a1), "r"(a2));
}

// K-major operand tile, 64-byte swizzle: rows of 64 B, 8-row atoms of 512 B.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused here)
    d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset: 8 rows x 64 B
    d |= (uint64_t)1 << 46;                   // descriptor version (sm_100 family)
    d |= (uint64_t)4 << 61;                   // swizzle mode: 64 B
    return d;
}
// kind::f16 instruction descriptor: f32 accumulate, bf16 A and B, both
// K-major, M = 128, N = n (a multiple of 16 up to 256).
__host__ __device__ constexpr uint32_t oz_idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(OZ_BM >> 4) << 24);
}

// =============================================================================
// Pre-pass 1: largest biased exponent per row of an operand
// =============================================================================
struct OpGeom {
    ModeGroup gr, gk, gl;  // rows, contracted, batch
    const void *const *ptrs;  // per-batch-entry base pointers (grouped execution) or null
    int t;                 // tensor index inside the groups (0 = A, 1 = B)
    int64_t R, K;
    int rows_fast;         // operand's unit-stride mode is a row mode
};

__device__ __forceinline__ int bexp(double v) {
    return (int)((__double_as_longlong(v) >> 52) & 0x7FF);
}
__device__ __forceinline__ int bexp_of(double v) { return bexp(v); }
__device__ __forceinline__ int bexp_of(double2 v) { return max(bexp(v.x), bexp(v.y)); }
// Float32 operands of a Float64 / ComplexF64 contraction (promote_eltype),
// widened exactly
__device__ __forceinline__ int bexp_of(float v) { return bexp((double)v); }
__device__ __forceinline__ int bexp_of(float2 v) { return max(bexp((double)v.x), bexp((double)v.y)); }

// `emax` (nullable): also the largest exponent of the whole operand.
// 2^(2 d) as a float (0 below 2^-126)
__device__ __forceinline__ float pow4f(int d) { return d >= -63 ? __int_as_float((127 + 2 * d) << 23) : 0.f; }

// k per tile of the exponent scan: each thread issues eight loads before
// the first reduction.
constexpr int OZ_SCAN_KT = 64;

struct ScaleSmem {
    int64_t roff[32], koff[OZ_SCAN_KT];
    int red[8][33];
    int cmax[8][OZ_SCAN_KT + 1];    // partials: per-warp column maxima
    float csum[8][OZ_SCAN_KT + 1];  // partials: per-warp column sums
    int tmax[OZ_SCAN_KT];           // partials: column maxima over the tile
};

// |x|^2 4^-(t - 1023), from the exponent and the top of the mantissa, for an
// element whose biased exponent is at most t (zero, subnormal and non-finite
// elements give 0: negligible, or flagged through the exponent table)
__device__ __forceinline__ float sq_tile(double x, int t) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7FF);
    if (be == 0 || be == 0x7FF) return 0.f;
    const float f = __int_as_float(0x3F800000 | (uint32_t)((b >> 29) & 0x7FFFFF));
    return f * f * pow4f(be - t);
}
__device__ __forceinline__ float sq_tile(double2 x, int t) { return sq_tile(x.x, t) + sq_tile(x.y, t); }
__device__ __forceinline__ float sq_tile(float x, int t) { return sq_tile((double)x, t); }
__device__ __forceinline__ float sq_tile(float2 x, int t) { return sq_tile((double)x.x, t) + sq_tile((double)x.y, t); }
template <typename T>
// One 32-row x 64-k tile. `part` (nullable, adaptive plans): per 32-row tile
// and k, the tile's largest exponent t and the sum of |x|^2 4^-(t - 1023)
// over its rows, at part[(l * ceil(R / 32) + tile) * K + k].
__device__ __forceinline__ void oz_scale_tile(const T *__restrict__ X, const OpGeom &g, int32_t *exps,
                                              int32_t *emax, int2 *part, int64_t blk, int64_t l, ScaleSmem &sm) {
    constexpr int KT = OZ_SCAN_KT;
    int64_t tiles_k = (g.K + KT - 1) / KT;
    int64_t tr = blk / tiles_k, tk = blk - tr * tiles_k;
    int64_t r0 = tr * 32, k0 = tk * KT;
    int tid = threadIdx.x, tx = tid % 32, ty = tid / 32;
    if (tid < 32) sm.roff[tid] = (r0 + tid < g.R) ? group_offset(g.gr, g.t, r0 + tid) : 0;
    else if (tid < 32 + KT) sm.koff[tid - 32] = (k0 + tid - 32 < g.K) ? group_offset(g.gk, g.t, k0 + tid - 32) : 0;
    const T *Xl = g.ptrs ? (const T *)g.ptrs[l] : X + group_offset(g.gl, g.t, l);
    __syncthreads();
    const int64_t R32 = (g.R + 31) / 32;
    int2 *pt = part ? part + (l * R32 + tr) * g.K + k0 : nullptr;  // this tile's partials
    if (g.rows_fast) {  // lanes walk rows; thread column kk = ty + 8 j
        constexpr int NJ = KT / 8;
        const bool rin = r0 + tx < g.R;
        T v[NJ];
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            memset(&v[j], 0, sizeof(T));
            if (rin && k0 + ty + 8 * j < g.K) v[j] = __ldg(Xl + sm.roff[tx] + sm.koff[ty + 8 * j]);
        }
        int e = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            const int be = bexp_of(v[j]);  // zero-filled outside the operand: 0
            e = max(e, be);
            if (pt) {
                int t = be;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) t = max(t, __shfl_xor_sync(0xffffffffu, t, d));
                float q = sq_tile(v[j], t);
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) q += __shfl_xor_sync(0xffffffffu, q, d);
                if (tx == 0 && k0 + ty + 8 * j < g.K) pt[ty + 8 * j] = make_int2(t, __float_as_int(q));
            }
        }
        sm.red[ty][tx] = e;
    } else {  // lanes walk k: columns tx and tx + 32, rows ty + 8 j
        T v[4][2];
        int be[4][2];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                memset(&v[j][h], 0, sizeof(T));
                if (r0 + ty + 8 * j < g.R && k0 + tx + 32 * h < g.K)
                    v[j][h] = __ldg(Xl + sm.roff[ty + 8 * j] + sm.koff[tx + 32 * h]);
            }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            be[j][0] = bexp_of(v[j][0]);
            be[j][1] = bexp_of(v[j][1]);
            int e = max(be[j][0], be[j][1]);
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, d));
            if (tx == 0) sm.red[j][ty + 8 * j] = e;  // rows ty + 8 j are distinct per (ty, j)
        }
        if (pt) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
                sm.cmax[ty][tx + 32 * h] = max(max(be[0][h], be[1][h]), max(be[2][h], be[3][h]));
            __syncthreads();
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int t = 0;
#pragma unroll
                for (int y = 0; y < 8; ++y) t = max(t, sm.cmax[y][tx + 32 * h]);
                float q = 0.f;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (be[j][h] > 0) q += sq_tile(v[j][h], t);
                sm.csum[ty][tx + 32 * h] = q;
                if (ty == 0) sm.tmax[tx + 32 * h] = t;
            }
            __syncthreads();
            if (ty < 2) {
                const int c = tx + 32 * ty;
                if (k0 + c < g.K) {
                    float s2 = 0.f;
#pragma unroll
                    for (int y = 0; y < 8; ++y) s2 += sm.csum[y][c];
                    pt[c] = make_int2(sm.tmax[c], __float_as_int(s2));
                }
            }
        }
    }
    __syncthreads();
    if (tid < 32) {
        int e = 0;
        if (r0 + tid < g.R) {
            if (g.rows_fast) {
                for (int j = 0; j < 8; ++j) e = max(e, sm.red[j][tid]);
            } else {
                e = sm.red[tid / 8 % 4][tid];  // written by ty = tid % 8, j = tid / 8
            }
            if (e > 0) atomicMax(exps + l * g.R + r0 + tid, e);
        }
        if (emax) {
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, d));
            if (tid == 0 && e > 0) atomicMax(emax, e);
        }
    }
}
template <typename T>
__global__ void __launch_bounds__(256, 4) k_oz_scale(const T *__restrict__ X, OpGeom g, int32_t *exps, int32_t *emax,
                                                  int2 *part) {
    __shared__ ScaleSmem sm;
    oz_scale_tile<T>(X, g, exps, emax, part, blockIdx.x, blockIdx.y, sm);
}

// =============================================================================
// Adaptive slice count: operand statistics and the choice
// =============================================================================
// Error model of the OZAKI form with S digits of W bits (u = 2^-(W S)), for
// row scales 2^e_i of A and column scales 2^f_j of B:
//   * each scaled element is represented to within u/2 (round-to-nearest
//     digits), an error of variance u^2/12 per real part: over C this sums to
//     u^2/12 sum_ij (4^e_i |b_j|^2 + 4^f_j |a_i|^2) = u^2/12 (P_A Q_B + P_B Q_A)
//     with P = sum of the squared scales and Q = squared Frobenius norm;
//   * the dropped digit pairs (i + j = S, 0-based) are S - 1 products of
//     digits of at most 2^(W-1) at weight 2^-(W (S+2)): variance at most
//     (S - 1) u^2 / 144 per k per real product, (S - 1) u^2/144 K P_A P_B;
//   * without cancellation, ||C||^2 = sum_k q_A[k] q_B[k] with q_A[k] the
//     squared norm of A's column k and q_B[k] of B's row k.
// Complex products count twice (re and im parts) in the first term and four
// times in the second. A numpy emulation of the digit scheme gave estimate /
// actual error between 1.0 (Gaussian data) and 5 (log-uniform magnitudes over
// 2^-60..2^60) for every slice count. Everything is measured relative to the
// operand's largest exponent, so the sums stay in float range.
struct OzStats {
    int32_t sel;        // chosen slice count, 0 = plain
    int32_t nonfinite;  // an operand holds Inf / NaN
    int32_t emax[2];    // largest biased exponent of A and B
    float est[9];       // estimated error per candidate slice count
    int32_t pad[3];
    // sums over k and batch entries (cleared with the header every call):
    // P_A sum q_B + P_B sum q_A, sum q_A q_B, K P_A P_B
    double acc[3];
    double pad2;
};
static_assert(sizeof(OzStats) == 96, "stats header");



// Statistics of one operand from the exponent scan's partials, once the
// operand's largest exponent is known. Blocks [0, ceil(K / 256)) of batch
// entry l write q[l][k], the squared norm of column k relative to 4^(be_max
// + 1 - 1023); the blocks after them add the rows' squared scales
// 4^(be_i - be_max) to P[l] and flag non-finite rows.
struct StatSmem {
    float red[32];
};
__device__ __forceinline__ void oz_stat_block(const int2 *__restrict__ part, const int32_t *__restrict__ exps,
                                              OzStats *st, int t, float *q, float *P, int64_t R, int64_t K,
                                              int64_t blk, int64_t l, StatSmem &sm) {
    const int be_max = st->emax[t];
    const int64_t nq = (K + 255) / 256, R32 = (R + 31) / 32;
    if (blk < nq) {
        const int64_t k = blk * 256 + threadIdx.x;
        if (k < K) {
            const int2 *p = part + l * R32 * K + k;
            float acc = 0.f;
            for (int64_t tr = 0; tr < R32; ++tr) {
                const int2 v = __ldg(p + tr * K);
                const float x = __int_as_float(v.y);
                if (x != 0.f) acc += x * pow4f(v.x - be_max - 1);
            }
            q[l * K + k] = acc;
        }
        return;
    }
    const int64_t i = (blk - nq) * 256 + threadIdx.x;
    float w = 0.f;
    if (i < R) {
        const int be = exps[l * R + i];
        if (be == 0x7FF) st->nonfinite = 1;
        else if (be > 0) w = pow4f(be - be_max);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) w += __shfl_xor_sync(0xffffffffu, w, d);
    if (threadIdx.x % 32 == 0) sm.red[threadIdx.x / 32] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s2 = 0.f;
        for (int y = 0; y < (int)blockDim.x / 32; ++y) s2 += sm.red[y];
        if (s2 != 0.f) atomicAdd(P + l, s2);
    }
}
__global__ void __launch_bounds__(256) k_oz_stat(const int2 *__restrict__ part, const int32_t *__restrict__ exps,
                                                 OzStats *st, int t, float *q, float *P, int64_t R, int64_t K) {
    __shared__ StatSmem sm;
    oz_stat_block(part, exps, st, t, q, P, R, K, blockIdx.x, blockIdx.y, sm);
}
__host__ __device__ inline int64_t oz_stat_blocks(int64_t R, int64_t K) { return (K + 255) / 256 + (R + 255) / 256; }

// The sums behind the estimate, spread over the GPU: block b of batch entry
// l (flattened as l * blocks + b) covers OZ_EST_K values of k and adds its
// part of P_A sum q_B + P_B sum q_A and of sum q_A q_B into the header in
// double; the entry's first block adds K P_A P_B.
constexpr int OZ_EST_K = 2048;
__host__ __device__ inline int64_t oz_est_blocks(int64_t K) { return (K + OZ_EST_K - 1) / OZ_EST_K; }
__device__ __forceinline__ void oz_est_block(OzStats *st, const float *__restrict__ qa, const float *__restrict__ qb,
                                             const float *__restrict__ pa, const float *__restrict__ pb, int64_t K,
                                             int64_t blk, int64_t l, double (&red)[2][8]) {
    double sa = 0.0, sb = 0.0, d = 0.0;
    const int64_t k1 = min(K, (blk + 1) * OZ_EST_K);
    for (int64_t k = blk * OZ_EST_K + threadIdx.x; k < k1; k += blockDim.x) {
        const float x = __ldg(qa + l * K + k), y = __ldg(qb + l * K + k);
        sa += x;
        sb += y;
        d += (double)x * y;
    }
    const double Pa = pa[l], Pb = pb[l];
    double tr = Pa * sb + Pb * sa;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tr += __shfl_xor_sync(0xffffffffu, tr, o);
        d += __shfl_xor_sync(0xffffffffu, d, o);
    }
    const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
    if (lane == 0) {
        red[0][w] = tr;
        red[1][w] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        tr = d = 0.0;
        for (int i = 0; i < (int)blockDim.x / 32; ++i) {
            tr += red[0][i];
            d += red[1][i];
        }
        if (tr != 0.0) atomicAdd(&st->acc[0], tr);
        if (d != 0.0) atomicAdd(&st->acc[1], d);
        if (blk == 0 && Pa * Pb != 0.0) atomicAdd(&st->acc[2], (double)K * Pa * Pb);
    }
}
__global__ void __launch_bounds__(256) k_oz_est(OzStats *st, const float *__restrict__ qa, const float *__restrict__ qb,
                                                const float *__restrict__ pa, const float *__restrict__ pb, int64_t K) {
    __shared__ double red[2][8];
    const int64_t nb = oz_est_blocks(K), l = blockIdx.x / nb;
    oz_est_block(st, qa, qb, pa, pb, K, blockIdx.x - l * nb, l, red);
}

// One thread: the error estimate of every candidate slice count (bit S of
// `cand`) from the sums, and the choice, the smallest count within `tol`,
// else 0 (plain).
__device__ __forceinline__ void oz_choose_final(OzStats *st, uint32_t cand, double tol, double margin, int cx) {
    const double trunc = st->acc[0], den = st->acc[1], drop = st->acc[2];
    const double f1 = cx ? 2.0 : 1.0, f2 = cx ? 4.0 : 1.0;
    int sel = 0;
    for (int S = 8; S >= 1; --S) {
        st->est[S] = 0.f;
        if (!(cand & (1u << S))) continue;
        const int W = S <= 6 ? 8 : 7;
        const double u = ldexp(1.0, -W * S);
        const double num = u * u * (f1 / 12.0 * trunc + f2 * (S - 1) / 144.0 * drop);
        double e;
        if (num == 0.0) e = 0.0;                 // an operand is zero: every form is exact
        else if (den == 0.0) e = INFINITY;       // no overlap the estimate can rest on
        else e = sqrt(num / den) * margin;
        st->est[S] = (float)e;
        if (e <= tol && !st->nonfinite) sel = S;  // scanning down: ends at the smallest
    }
    st->est[0] = 0.f;
    st->sel = sel;
}
__global__ void k_oz_choose(OzStats *st, uint32_t cand, double tol, double margin, int cx) {
    if (threadIdx.x == 0) oz_choose_final(st, cand, tol, margin, cx);
}

// =============================================================================
// Pre-pass 2: slices (OZAKI digits or BF16X3 pieces), permutation fused
// =============================================================================
// Output words (2 x bf16) of slice plane s: out[((l*S + s) * rows_e + row) * kw + word].
//   MODE_REAL : row = r,        word w holds k = 2w, 2w+1
//   MODE_CA   : row = r,        word k holds (re, im)           (A side)
//   MODE_CB   : rows 2r, 2r+1,  word k holds (re, -im), (im, re) (B side)
enum { MODE_REAL = 0, MODE_CA = 1, MODE_CB = 2 };

__device__ __forceinline__ uint32_t bf16_bits_of_int(int d) {
    float f = __int_as_float(0x4B400000 + d) - 12582912.0f;  // exact for |d| < 2^22
    return __float_as_uint(f) >> 16;                         // exact in bf16 for |d| <= 256
}
__device__ __forceinline__ uint32_t pack2(uint32_t lo, uint32_t hi) { return lo | (hi << 16); }

// x * 2^(62 - e) truncated to a signed 62-bit fixed-point integer (|x| < 2^e).
__device__ __forceinline__ int64_t oz_fixed(double x, int e) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7FF);
    int64_t m = (int64_t)(b & 0xFFFFFFFFFFFFFull);
    int ex;
    if (be) {
        m |= (int64_t)1 << 52;
        ex = be - 1075;
    } else {
        ex = -1074;
    }
    const int sh = ex + 62 - e;  // Q = m * 2^sh < 2^62
    int64_t Q;
    if (sh >= 0) Q = m << sh;
    else if (sh > -63) Q = m >> (-sh);
    else Q = 0;
    return (b >> 63) ? -Q : Q;
}
// Signed digits of Q, most significant first, rounded to nearest (balanced):
// with B = half a unit of the last digit plus 2^(W-1) at every digit position
// after the first, digit s >= 1 is the W-bit window of Q + B at its position
// minus 2^(W-1), and the leading digit is everything above its position
// (signed). |d_0| <= 2^W, |d_s| <= 2^(W-1), and the remainder below the last
// digit lies in [-1/2, 1/2) units of it: the rounding of taking the digits
// one at a time, with one 64-bit add for all of them instead of an add, a
// shift and a subtract per digit.
__host__ __device__ constexpr int64_t oz_digit_bias(int S, int W) {
    int64_t b = (int64_t)1 << (62 - W * S - 1);
    for (int s = 1; s < S; ++s) b += (int64_t)1 << (62 - W * (s + 1) + W - 1);
    return b;
}
// Digit s of a biased value Qb (Q + oz_digit_bias) as an exact float. The
// leading digit (signed, |d| <= 2^W) goes through 1.5 * 2^23 + d; a later
// digit's W-bit window u becomes the mantissa of 2^23 + u, from which
// 2^23 + 2^(W-1) is subtracted: a funnel shift, a mask-and-or and one add,
// with no integer-to-float conversion. NEG gives -d (+0 for d = 0, as d).
template <int W, int s, bool NEG = false>
__device__ __forceinline__ float oz_digit_f(int64_t Qb) {
    constexpr int sh = 62 - W * (s + 1);
    if constexpr (s == 0) {
        const float m = __int_as_float(0x4B400000 + (int)(Qb >> sh));
        return NEG ? 12582912.0f - m : m - 12582912.0f;
    } else {
        constexpr float c = 8388608.0f + (float)(1 << (W - 1));
        const float m = __uint_as_float(0x4B000000u | ((uint32_t)((uint64_t)Qb >> sh) & ((1u << W) - 1u)));
        return NEG ? c - m : m - c;
    }
}
// Two floats that bf16 holds exactly (the digits: integers of at most 8
// significant bits) as one packed word, `lo` in the low half. Their bf16
// bits are the upper halves of their float bits, so one byte permute on the
// integer pipe packs them (no conversion instruction).
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}
// f(integral_constant<int, s>) for s = 0 .. N-1, unrolled at compile time.
template <int N, int s = 0, typename F>
__device__ __forceinline__ void oz_static_for(F &&f) {
    if constexpr (s < N) {
        f(std::integral_constant<int, s>{});
        oz_static_for<N, s + 1>(f);
    }
}

// Three bf16 pieces of a float: x = hi + mid + lo (to ~2^-24 relative).
__device__ __forceinline__ void bf3_pieces(float x, uint32_t (&p)[8]) {
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    float r = x - __bfloat162float(h);
    __nv_bfloat16 m = __float2bfloat16_rn(r);
    r = r - __bfloat162float(m);
    __nv_bfloat16 l = __float2bfloat16_rn(r);
    p[0] = __bfloat16_as_ushort(h);
    p[1] = __bfloat16_as_ushort(m);
    p[2] = __bfloat16_as_ushort(l);
}

template <typename T>
struct OzIn;
template <>
struct OzIn<double> {
    static constexpr bool cx = false;
    __device__ static double re(double v) { return v; }
    __device__ static double im(double) { return 0.0; }
};
template <>
struct OzIn<double2> {
    static constexpr bool cx = true;
    __device__ static double re(double2 v) { return v.x; }
    __device__ static double im(double2 v) { return v.y; }
};
template <>
struct OzIn<float> {
    static constexpr bool cx = false;
    __device__ static float re(float v) { return v; }
    __device__ static float im(float) { return 0.f; }
};
template <>
struct OzIn<float2> {
    static constexpr bool cx = true;
    __device__ static float re(float2 v) { return v.x; }
    __device__ static float im(float2 v) { return v.y; }
};

// BF3 = true: float inputs split into bf16 pieces; otherwise Ozaki digits.
template <typename T, int KT>
struct SliceSmem {
    T tile[32][KT + 1];
    int64_t roff[32], koff[KT];
    int rexp[32];
};
// k per slicer tile: eight loads per thread before the barrier
constexpr int OZ_SLICE_KT = 64;
template <typename T, int MODE>
using SliceSmemOf = SliceSmem<T, OZ_SLICE_KT>;

// BF16x3: three bf16 pieces per float, one thread per (row, k word).
template <typename T, int MODE>
__device__ __forceinline__ void oz_write_pieces(const SliceSmemOf<T, MODE> &sm, const OpGeom &g, uint32_t *outl,
                                                int64_t plane, int64_t kw, int64_t r0, int64_t k0) {
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    for (int j = 0; j < 4; ++j) {
        const int r = ty + 8 * j;
        const int64_t row = r0 + r;
        if (row >= g.R) continue;
        if constexpr (MODE == MODE_REAL) {
            const int64_t word = k0 / 2 + tx;
            if (word >= kw) continue;
            uint32_t *o = outl + row * kw + word;
            uint32_t p0[8], p1[8];
            bf3_pieces((float)OzIn<T>::re(sm.tile[r][2 * tx]), p0);
            bf3_pieces((float)OzIn<T>::re(sm.tile[r][2 * tx + 1]), p1);
#pragma unroll
            for (int s = 0; s < 3; ++s) o[s * plane] = pack2(p0[s], p1[s]);
        } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int kk = tx + 32 * h;
                const int64_t word = k0 + kk;
                if (word >= kw) continue;
                // MODE_CA: row r; MODE_CB: rows 2r (re, -im) and 2r + 1 (im, re)
                uint32_t *o = outl + (MODE == MODE_CB ? 2 * row : row) * kw + word;
                const T v = sm.tile[r][kk];
                uint32_t pr[8], pi[8], pn[8];
                bf3_pieces((float)OzIn<T>::re(v), pr);
                bf3_pieces((float)OzIn<T>::im(v), pi);
                bf3_pieces(-(float)OzIn<T>::im(v), pn);
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    if (MODE == MODE_CA) {
                        o[s * plane] = pack2(pr[s], pi[s]);
                    } else {
                        o[s * plane] = pack2(pr[s], pn[s]);
                        o[s * plane + kw] = pack2(pi[s], pr[s]);
                    }
                }
            }
        }
    }
}

// Ozaki digits with the slice count fixed at compile time: every digit plane
// is written as soon as it is known, from two biased fixed-point values per
// thread.
template <int S, typename T, int MODE>
__device__ __forceinline__ void oz_write_digits(const SliceSmemOf<T, MODE> &sm, const OpGeom &g, uint32_t *outl,
                                                int64_t plane, int64_t kw, int64_t r0, int64_t k0) {
    constexpr int W = oz_digit_bits(S);
    constexpr int64_t bias = oz_digit_bias(S, W);
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    for (int j = 0; j < 4; ++j) {
        const int r = ty + 8 * j;
        const int64_t row = r0 + r;
        if (row >= g.R) continue;
        int e = sm.rexp[r];
        const bool bad = e == 0x7FFFFFFF;
        if (bad) e = 0;
        if constexpr (MODE == MODE_REAL) {
            const int64_t word = k0 / 2 + tx;
            if (word >= kw) continue;
            uint32_t *o = outl + row * kw + word;
            const int64_t q0 = oz_fixed(bad ? 0.0 : (double)OzIn<T>::re(sm.tile[r][2 * tx]), e) + bias;
            const int64_t q1 = oz_fixed(bad ? 0.0 : (double)OzIn<T>::re(sm.tile[r][2 * tx + 1]), e) + bias;
            oz_static_for<S>([&](auto sc) {
                constexpr int s = decltype(sc)::value;
                o[s * plane] = pack_bf16x2(oz_digit_f<W, s>(q0), oz_digit_f<W, s>(q1));
            });
        } else {
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                const int kk = tx + 32 * h;
                const int64_t word = k0 + kk;
                if (word >= kw) continue;
                uint32_t *o = outl + (MODE == MODE_CB ? 2 * row : row) * kw + word;
                const T v = sm.tile[r][kk];  // one shared-memory read of the whole element
                const int64_t qr = oz_fixed(bad ? 0.0 : (double)OzIn<T>::re(v), e) + bias;
                const int64_t qi = oz_fixed(bad ? 0.0 : (double)OzIn<T>::im(v), e) + bias;
                oz_static_for<S>([&](auto sc) {
                    constexpr int s = decltype(sc)::value;
                    const float dr = oz_digit_f<W, s>(qr), di = oz_digit_f<W, s>(qi);
                    if constexpr (MODE == MODE_CA) {
                        o[s * plane] = pack_bf16x2(dr, di);
                    } else {
                        o[s * plane] = pack_bf16x2(dr, oz_digit_f<W, s, true>(qi));
                        o[s * plane + kw] = pack_bf16x2(di, dr);
                    }
                });
            }
        }
    }
}

// One 32-row tile of an operand: staged through shared memory (coalesced
// reads whichever mode is contiguous), then written as digit (or piece)
// planes [L][S][rows_e][kw] with K contiguous.
template <typename T, int MODE, bool BF3>
__device__ __forceinline__ void oz_slice_tile(const T *__restrict__ X, const OpGeom &g,
                                              const int32_t *__restrict__ exps, int S,
                                              uint32_t *__restrict__ out, int64_t rows_e, int64_t kw, int64_t blk,
                                              int64_t l, SliceSmemOf<T, MODE> &sm) {
    constexpr int KT = OZ_SLICE_KT;
    int64_t tiles_k = (g.K + KT - 1) / KT;
    int64_t tr = blk / tiles_k, tk = blk - tr * tiles_k;
    int64_t r0 = tr * 32, k0 = tk * KT;
    int tid = threadIdx.x;
    if (tid < 32) {
        sm.roff[tid] = (r0 + tid < g.R) ? group_offset(g.gr, g.t, r0 + tid) : 0;
        if (!BF3) {
            int be = (r0 + tid < g.R) ? exps[l * g.R + r0 + tid] : 0;
            sm.rexp[tid] = be == 0x7FF ? 0x7FFFFFFF : (be == 0 ? -1022 : be - 1022);
        }
    }
    if (tid < KT) sm.koff[tid] = (k0 + tid < g.K) ? group_offset(g.gk, g.t, k0 + tid) : 0;
    const T *Xl = g.ptrs ? (const T *)g.ptrs[l] : X + group_offset(g.gl, g.t, l);
    __syncthreads();
    for (int idx = tid; idx < 32 * KT; idx += 256) {
        int r, kk;
        if (g.rows_fast) {
            r = idx % 32;
            kk = idx / 32;
        } else {
            kk = idx % KT;
            r = idx / KT;
        }
        T v;
        memset(&v, 0, sizeof(T));
        if (r0 + r < g.R && k0 + kk < g.K) v = __ldg(Xl + sm.roff[r] + sm.koff[kk]);
        sm.tile[r][kk] = v;
    }
    __syncthreads();
    const int64_t plane = rows_e * kw;
    uint32_t *outl = out + l * (int64_t)S * plane;
    if constexpr (BF3) {
        oz_write_pieces<T, MODE>(sm, g, outl, plane, kw, r0, k0);
    } else {
        switch (S) {
        case 3: oz_write_digits<3, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        case 4: oz_write_digits<4, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        case 5: oz_write_digits<5, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        case 6: oz_write_digits<6, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        case 7: oz_write_digits<7, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        case 8: oz_write_digits<8, T, MODE>(sm, g, outl, plane, kw, r0, k0); break;
        default: break;  // plans hold 3..8
        }
    }
}

// `sel` (nullable): the adaptive choice; the slice count is read from it and
// the launch does nothing when it is 0 (plain).
template <typename T, int MODE, bool BF3>
__global__ void __launch_bounds__(256, 4) k_oz_slice(const T *__restrict__ X, OpGeom g,
                                                  const int32_t *__restrict__ exps, int S,
                                                  uint32_t *__restrict__ out, int64_t rows_e,
                                                  int64_t kw, const int32_t *__restrict__ sel) {
    if (sel) {
        S = *sel;
        if (S == 0) return;
    }
    __shared__ SliceSmemOf<T, MODE> sm;
    oz_slice_tile<T, MODE, BF3>(X, g, exps, S, out, rows_e, kw, blockIdx.x, blockIdx.y, sm);
}

// =============================================================================
// The tcgen05 GEMM over slices
// =============================================================================
struct OzGemmArgs {
    int64_t M, Ne, N;      // rows of A, embedded rows of B, un-embedded N
    int32_t nkb;           // number of 32-wide k blocks
    int32_t kcb;           // k blocks per chunk (exact readout interval)
    int32_t S;             // slices (digits / pieces)
    const int32_t *expA;   // [L][M] biased exponents (OZAKI)
    const int32_t *expB;   // [L][N]
    void *C;
    void *const *cptr;     // per-batch-entry output pointers (grouped execution) or null
    int32_t band;          // row tiles per rasterisation band
    ModeGroup gm, gn, gl;  // C offsets live in tensor slot 2
    int32_t *status;
    const int32_t *sel;    // adaptive choice (nullable): run only when it holds S
};

// One contraction (or one bucket of a group) as the GEMM sees it: the slice
// tensor maps, the arguments and its tile grid (column tiles x row tiles x
// batch entries).
struct OzJob {  // aligned as its tensor maps
    CUtensorMap tmA, tmB;
    OzGemmArgs a;
    int32_t tiles_n, tiles_m, L;
};

// Tile sources of the kernel: one job in the parameter space, or a table of
// jobs in global memory (a group) whose tiles are numbered consecutively.
// `hint` is the caller's job index of its previous tile (0 at first): a CTA
// visits its tiles in increasing order, so the next tile usually lies in the
// same job or the one after it.
struct OzOneJob {
    static constexpr bool kTable = false;
    const OzJob *j;
    __device__ int64_t tiles() const { return (int64_t)j->tiles_n * j->tiles_m * j->L; }
    __device__ const OzJob &job(int64_t t, int64_t &local, int &) const {
        local = t;
        return *j;
    }
};
struct OzJobTable {
    static constexpr bool kTable = true;  // jobs may carry their own adaptive choice (skipped unless it is S)
    const OzJob *jobs;
    const int64_t *start;  // [n + 1]: first tile of each job, then the total
    int n;
    __device__ int64_t tiles() const { return start[n]; }
    __device__ const OzJob &job(int64_t t, int64_t &local, int &hint) const {
        int lo = hint;  // the last job with start <= t, at or after the hint
        if (lo + 1 < n && start[lo + 1] <= t) {
            ++lo;
            if (lo + 1 < n && start[lo + 1] <= t) {
                int hi = n - 1;
                ++lo;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) / 2;
                    if (start[mid] <= t) lo = mid;
                    else hi = mid - 1;
                }
            }
        }
        hint = lo;
        local = t - start[lo];
        return jobs[lo];
    }
    // The first tile after job `hint` that the CTA striding by `grid` from
    // `first` visits: a skipped job costs one step, not one per tile.
    __device__ int64_t after_job(int hint, int64_t first, int64_t grid) const {
        const int64_t e = start[hint + 1];
        return e + (((first - e) % grid) + grid) % grid;
    }
};

// The tile before this CTA's first tile after job `hint` (the tile loop then
// adds the grid stride): every role of the CTA skips a job of another slice
// count in one step, and all roles see the same choice, so their tile
// sequences stay equal.
template <typename Src>
__device__ __forceinline__ int64_t skip_job(const Src &src, int hint, int64_t t) {
    if constexpr (Src::kTable) return src.after_job(hint, blockIdx.x, gridDim.x) - gridDim.x;
    return t;
}

// Tile `local` of a job: batch entry, then grouped rasterisation within the
// entry, so that consecutive tiles walk a band of `band` row tiles across all
// column tiles and the CTAs resident at the same time share slices in L2.
template <typename I>
__device__ __forceinline__ void oz_tile_t(I local, I nn, I nm, I gm, int bn, int64_t &m0, int64_t &n0, int &l) {
    const I per = nn * nm;
    const I ll = local / per;
    const I t = local - ll * per;
    const I band = t / (gm * nn);
    const I first = band * gm;
    const I rows = min(gm, nm - first);
    const I r = t - band * gm * nn;
    l = (int)ll;
    m0 = (int64_t)(first + r % rows) * OZ_BM;
    n0 = (int64_t)(r / rows) * bn;
}
__device__ __forceinline__ void oz_tile(const OzJob &J, int64_t local, int bn, int64_t &m0, int64_t &n0, int &l) {
    const int64_t nn = J.tiles_n, nm = J.tiles_m, gm = J.a.band;
    // 32-bit divisions whenever the job's tile numbers fit (a 64-bit division
    // is a long software sequence)
    if (local <= INT32_MAX && (int64_t)J.L * nn * nm <= INT32_MAX && gm * nn <= INT32_MAX)
        oz_tile_t<uint32_t>((uint32_t)local, (uint32_t)nn, (uint32_t)nm, (uint32_t)gm, bn, m0, n0, l);
    else
        oz_tile_t<int64_t>(local, nn, nm, gm, bn, m0, n0, l);
}

// One CTA computes 128 x BN tiles of the embedded output, in turn for the
// tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...: the stage ring, the
// TMEM banks and their barriers run on across tiles, so the loads of the
// next tile overlap the MMAs and the readout of the current one. Digit group
// g = i + j (0-based slice indices of A and B) owns BN TMEM columns; the S
// groups of a chunk form one bank of BN S columns, and two banks alternate
// so that the epilogue reads chunk c while the MMAs fill chunk c + 1.
// The B slices of a stage lie back to back (BN rows each), so the products
// of A slice i with B slices 0 .. S-1-i are ONE tcgen05.mma with
// N = BN (S - i) whose accumulator columns are exactly groups i .. S-1:
// S wide MMAs per 16 k instead of S (S+1)/2 narrow ones, and every A slice
// is read from shared memory once per 16 k. BN = 64 for BF16X3 and 32 for
// the exact forms: the widest that two banks leave room for while the
// epilogue's accumulators (96-bit integers, or float sums and their
// compensations) stay in registers.
template <int S, bool EXACT, bool CX, typename Src>
__device__ __forceinline__ void oz_gemm_body(const Src &src) {
    constexpr int W = oz_digit_bits(S);  // digit width (EXACT)
    constexpr int NST = oz_stages(S, EXACT);
    constexpr int STAGE = oz_stage_bytes(S, EXACT);
    constexpr int BN = oz_bn(S, EXACT);  // columns per digit group, embedded B rows per CTA
    constexpr int HALF = BN / 2;     // columns per group read by one epilogue warp
    constexpr int TCOLS = oz_tmem_cols(S);
    constexpr int BANK = TCOLS / 2;  // TMEM column offset of the second bank
    static_assert(NST >= 2, "need at least two pipeline stages");
    static_assert(BN * S <= BANK && TCOLS <= 512, "two banks must fit in TMEM");
    static_assert(BN * S <= 256, "one MMA covers at most 256 columns");
    static_assert(HALF % 16 == 0, "epilogue reads 16 columns at a time");
    // MMA-issuing threads. Each mbarrier poll by an issuing thread stalls it
    // for ~150 cycles while the tensor core's queue holds only ~200 cycles of
    // MMAs, so a single issuer leaves a bubble at every k block. Two issuers
    // (warps 1 and 10) take alternate k blocks and keep the queue fed while
    // the other polls. Their MMAs into a bank interleave in an unspecified
    // order, which changes nothing for the exact integer sums of the OZAKI
    // form; BF16X3 sums round, so it keeps one issuer and stays deterministic.
    constexpr int NI = EXACT ? 2 : 1;

    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + NST * STAGE);
    uint64_t *full = bars;               // [2 NST] see full_idx
    uint64_t *empty = bars + 2 * NST;    // [NST]
    uint64_t *acc_full = bars + 3 * NST; // [2] bank filled (one commit per issuer)
    uint64_t *acc_empty = acc_full + 2;  // [2] bank read and cleared (one arrive per epilogue warp)
    uint64_t *done = acc_empty + 2;      // [2] per issuer: all its MMAs complete
    uint32_t *tmem_slot = (uint32_t *)(done + 2);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

    // Stage-landed barriers, indexed by the CTA's running k-block count g
    // (across its tiles). Each barrier is waited on by a single issuer and in
    // order of its phases: an mbarrier parity wait cannot tell phase r from
    // phase r - 2, so a waiter that could run two phases ahead of a barrier
    // would pass early. With two issuers and an odd stage count the rounds of
    // a stage alternate between the issuers, so every stage gets one barrier
    // per issuer (index 2 s + g % 2) and each of those is used every other
    // round; otherwise stage s always has the same issuer (index 2 s + s % 2,
    // or 2 s for one issuer), used every round.
    auto full_idx = [](uint32_t g) { return 2 * (int)(g % NST) + (NI == 2 ? (int)(g & 1u) : 0); };
    auto full_par = [](uint32_t g) {
        const uint32_t r = g / NST;
        return (NI == 2 && (NST & 1)) ? (r >> 1) & 1u : r & 1u;
    };
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int64_t T = src.tiles();
    int32_t *status;
    {
        int64_t unused;
        int h0 = 0;
        const OzGemmArgs &a0 = src.job(0, unused, h0).a;
        // an adaptive plan launches every candidate; all but the chosen one
        // return before touching shared memory or TMEM
        if (!Src::kTable && a0.sel && *a0.sel != S) return;
        status = a0.status;
    }

    if (tid == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(smem_u32(full + 2 * s), 1);
            mbar_init(smem_u32(full + 2 * s + 1), 1);
            mbar_init(smem_u32(empty + s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(acc_full + b), NI);
            mbar_init(smem_u32(acc_empty + b), OZ_EPI_WARPS);
            mbar_init(smem_u32(done + b), 1);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"((uint32_t)TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // Every MMA accumulates (the issuers' order within a bank is free); the
    // epilogue warps clear both banks here and each bank again after reading it.
    if (warp >= 2 && warp < 2 + OZ_EPI_WARPS) {
        const int q = warp % 4, h = (warp - 2) / 4;
        for (int c = 0; c < TCOLS / 2; c += 16) tc_st16_zero(tmem + ((uint32_t)(32 * q) << 16) + h * (TCOLS / 2) + c);
        tc_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t g = 0;  // k blocks issued so far, over all tiles of this CTA
            bool ok = true;
            int hint = 0;
            for (int64_t t = blockIdx.x; t < T && ok; t += gridDim.x) {
                int64_t local;
                const OzJob &J = src.job(t, local, hint);
                if (Src::kTable && J.a.sel && *J.a.sel != S) {  // a job of another slice count
                    t = skip_job(src, hint, t);
                    continue;
                }
                int64_t m0, n0;
                int l;
                oz_tile(J, local, BN, m0, n0, l);
                for (int kb = 0; kb < J.a.nkb; ++kb, ++g) {
                    const int s = (int)(g % NST);
                    const uint32_t round = g / NST;
                    if (!mbar_wait(smem_u32(empty + s), (round & 1) ^ 1, abort_flag, status)) {
                        ok = false;
                        break;
                    }
                    uint8_t *st = smem + s * STAGE;
                    const uint32_t fb = smem_u32(full + full_idx(g));
                    mbar_expect_tx(fb, STAGE);
                    tma_load_3d(smem_u32(st), &J.tmA, kb * OZ_BK, (int)m0, l * S, fb);
                    tma_load_3d(smem_u32(st + S * OZ_A_TILE), &J.tmB, kb * OZ_BK, (int)n0, l * S, fb);
                }
            }
            // make sure no bulk copy is still writing into shared memory
            for (uint32_t gg = g > (uint32_t)NST ? g - NST : 0u; gg < g; ++gg)
                mbar_drain(smem_u32(full + full_idx(gg)), full_par(gg));
        }
    } else if (warp == 1 || (NI == 2 && warp == OZ_ISSUER2_WARP)) {
        // ---------------- MMA issuers ----------------
        // Issuer `me` takes the k blocks whose running count g has g % NI == me.
        // Per chunk C (counted over all tiles) it waits until the epilogue has
        // read and cleared the bank's previous chunk (C - 2), issues its k
        // blocks, and commits the chunk's acc_full barrier once (also when it
        // owns no k block of it).
        if (lane == 0) {
            const int me = warp == 1 ? 0 : 1;
            bool ok = true;
            uint32_t g = 0, C = 0;
            int hint = 0;
            for (int64_t t = blockIdx.x; t < T && ok; t += gridDim.x) {
                int64_t local;
                const OzJob &J = src.job(t, local, hint);
                if (Src::kTable && J.a.sel && *J.a.sel != S) {  // a job of another slice count
                    t = skip_job(src, hint, t);
                    continue;
                }
                const int nkb = J.a.nkb, kcb = J.a.kcb;
                for (int c0 = 0; c0 < nkb && ok; c0 += kcb, ++C) {
                    const uint32_t bank = C & 1u;
                    if (!mbar_wait(smem_u32(acc_empty + bank), ((C >> 1) & 1u) ^ 1u, abort_flag, status)) {
                        ok = false;
                        break;
                    }
                    const int c1 = min(nkb, c0 + kcb);
                    for (int kb = c0; kb < c1; ++kb) {
                        const uint32_t gg = g + (uint32_t)kb;
                        if (NI == 2 && (int)(gg & 1u) != me) continue;
                        const int s = (int)(gg % NST);
                        if (!mbar_wait(smem_u32(full + full_idx(gg)), full_par(gg), abort_flag, status)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t a_base = smem_u32(smem + s * STAGE);
                        const uint64_t ad0 = sw64_desc(a_base);
                        const uint64_t bd0 = sw64_desc(a_base + S * OZ_A_TILE);
                        const uint32_t d0 = tmem + bank * BANK;
#pragma unroll
                        for (int k16 = 0; k16 < OZ_BK / 16; ++k16)
#pragma unroll
                            for (int i = 0; i < S; ++i)
                                tc_mma(d0 + BN * i, ad0 + (uint64_t)((i * OZ_A_TILE + k16 * 32) >> 4),
                                       bd0 + (uint64_t)((k16 * 32) >> 4), oz_idesc(BN * (S - i)), 1u);
                        tc_commit(smem_u32(empty + s));
                    }
                    if (ok) tc_commit(smem_u32(acc_full + bank));
                }
                g += (uint32_t)nkb;
            }
            // wait for every MMA this thread issued before TMEM is released
            tc_commit(smem_u32(done + me));
            mbar_drain(smem_u32(done + me), 0);
        }
    } else if (warp < 2 + OZ_EPI_WARPS) {
        // ---------------- epilogue ----------------
        const int q = warp % 4;        // TMEM lane quarter this warp may access
        const int h = (warp - 2) / 4;  // column half (HALF columns) of each group
        const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + HALF * h;
        bool ok = true;
        uint32_t C = 0;  // chunks read so far, over all tiles of this CTA
        int hint = 0;
        for (int64_t t = blockIdx.x; t < T && ok; t += gridDim.x) {
            int64_t local;
            const OzJob &J = src.job(t, local, hint);
            if (Src::kTable && J.a.sel && *J.a.sel != S) {  // a job of another slice count
                t = skip_job(src, hint, t);
                continue;
            }
            const OzGemmArgs &args = J.a;
            int64_t m0, n0;
            int l;
            oz_tile(J, local, BN, m0, n0, l);
            const int64_t row = m0 + 32 * q + lane;
            const int nchunks = (args.nkb + args.kcb - 1) / args.kcb;
            // Output addressing of the tile, fetched before the first chunk
            // wait so that its loads overlap the MMAs: the thread's row (offset
            // and exponent), and one output column per lane (lane j < NCOL
            // holds column j of this warp's half, broadcast by shuffles).
            constexpr int NCOL = CX ? HALF / 2 : HALF;
            const bool row_ok = row < args.M;
            int64_t rowoff = 0;
            int erow = 0;
            bool badrow = false;
            if (row_ok) {
                rowoff = (args.cptr ? 0 : group_offset(args.gl, 2, l)) + group_offset(args.gm, 2, row);
                if (EXACT) {
                    const int be = args.expA[(int64_t)l * args.M + row];
                    badrow = be == 0x7FF;
                    erow = be == 0 ? -1022 : be - 1022;
                }
            }
            long long lcoff = 0;
            int lexp = -1;  // the column's exponent (0 without one), -1 beyond the output
            {
                const int64_t ne = n0 + HALF * h + (int64_t)lane * (CX ? 2 : 1);
                if (lane < NCOL && ne < args.Ne) {
                    const int64_t n = CX ? (ne >> 1) : ne;
                    lcoff = group_offset(args.gn, 2, n);
                    lexp = EXACT ? args.expB[(int64_t)l * args.N + n] : 0;
                }
            }
            void *const Cl = args.cptr ? args.cptr[l] : args.C;
            // EXACT: one 96-bit two's-complement integer per output column,
            // X = sum_d G_d 2^(W (S + 1 - d)), held in w0 (bits 0-31), w1, w2.
            uint32_t w0[EXACT ? HALF : 1], w1[EXACT ? HALF : 1], w2[EXACT ? HALF : 1];
            // BF16X3: Kahan-compensated float32 sum over the chunks
            float accf[EXACT ? 1 : HALF], comp[EXACT ? 1 : HALF];
#pragma unroll
            for (int j = 0; j < HALF; ++j) {
                if (EXACT) {
                    w0[j] = 0;
                    w1[j] = 0;
                    w2[j] = 0;
                } else {
                    accf[j] = 0.f;
                    comp[j] = 0.f;
                }
            }
#pragma unroll 1
            for (int c = 0; c < nchunks; ++c, ++C) {
                const uint32_t bank = C & 1u;
                // warp-uniform outcome: the warp-collective loads below need every lane
                if (!__all_sync(0xffffffffu, mbar_wait(smem_u32(acc_full + bank), (C >> 1) & 1u, abort_flag, status))) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t tb = tbase + bank * BANK;
                if constexpr (EXACT) {
#pragma unroll
                    for (int g = 0; g < S; ++g) {
                        uint32_t v[HALF];
                        tc_ld<HALF>(tb + BN * g, v);
#pragma unroll
                        for (int c2 = 0; c2 < HALF; c2 += 16) tc_st16_zero(tb + BN * g + c2);
                        if (g == S - 1) {  // every group of the bank read and cleared
                            tc_wait_st();
                            tc_fence_before();
                            __syncwarp();
                            if (lane == 0) mbar_arrive(smem_u32(acc_empty + bank));
                        }
                        const int sh = W * (S - 1 - g);  // W (S + 1 - d), d = g + 2
                        if (sh < 32) {
#pragma unroll
                            for (int j = 0; j < HALF; ++j) {
                                int64_t x = (int64_t)__float2int_rn(__uint_as_float(v[j])) << sh;
                                add96(w0[j], w1[j], w2[j], (uint32_t)x, (uint32_t)((uint64_t)x >> 32),
                                      x < 0 ? 0xFFFFFFFFu : 0u);
                            }
                        } else {
#pragma unroll
                            for (int j = 0; j < HALF; ++j) {
                                int64_t x = (int64_t)__float2int_rn(__uint_as_float(v[j])) << (sh - 32);
                                add64hi(w1[j], w2[j], (uint32_t)x, (uint32_t)((uint64_t)x >> 32));
                            }
                        }
                    }
                } else {
                    // pieces hi*hi, then the products of piece-index sum 1 and 2;
                    // 16 columns at a time, so that the three groups' registers
                    // stay beside the running sums and their compensations
#pragma unroll
                    for (int c2 = 0; c2 < HALF; c2 += 16) {
                        uint32_t v0[16], v1[16], v2[16];
                        tc_ld<16>(tb + c2, v0);
                        tc_ld<16>(tb + BN + c2, v1);
                        tc_ld<16>(tb + 2 * BN + c2, v2);
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            float x = __uint_as_float(v0[j]) + (__uint_as_float(v1[j]) + __uint_as_float(v2[j]));
                            float y = x - comp[c2 + j];
                            float s2 = accf[c2 + j] + y;
                            comp[c2 + j] = (s2 - accf[c2 + j]) - y;
                            accf[c2 + j] = s2;
                        }
                    }
#pragma unroll
                    for (int g = 0; g < 3; ++g)
#pragma unroll
                        for (int c2 = 0; c2 < HALF; c2 += 16) tc_st16_zero(tb + BN * g + c2);
                    tc_wait_st();
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(smem_u32(acc_empty + bank));
                }
            }
            if (!ok) break;
            if constexpr (EXACT) {
                // Four conversions at a time through the straight-line routine,
                // so that their integer sequences interleave (one conversion
                // alone is a chain of dependent instructions); a group with a
                // subnormal result (rare) goes through the general routine;
                // then the group's stores.
                constexpr int GQ = CX ? 2 : 4;  // output columns per group
                constexpr int NP = CX ? 2 : 1;  // parts per output column
                const uint64_t nanb = 0x7FF8000000000000ull;
#pragma unroll
                for (int j0 = 0; j0 < NCOL; j0 += GQ) {
                    uint64_t bits[GQ][NP];
                    int Eq[GQ];
                    bool slow = false;
#pragma unroll
                    for (int q2 = 0; q2 < GQ; ++q2) {
                        const int bc = __shfl_sync(0xffffffffu, lexp, j0 + q2);
                        Eq[q2] = erow + (bc == 0 ? -1022 : bc - 1022) - W * (S + 1);
#pragma unroll
                        for (int pp = 0; pp < NP; ++pp) {
                            const int j = NP * (j0 + q2) + pp;
                            bits[q2][pp] = x96_ldexp_bits_fast(w0[j], w1[j], w2[j], Eq[q2], slow);
                        }
                    }
                    if (slow) {
#pragma unroll
                        for (int q2 = 0; q2 < GQ; ++q2)
#pragma unroll
                            for (int pp = 0; pp < NP; ++pp) {
                                const int j = NP * (j0 + q2) + pp;
                                bits[q2][pp] =
                                    (uint64_t)__double_as_longlong(x96_ldexp_rn_general(w0[j], w1[j], w2[j], Eq[q2]));
                            }
                    }
#pragma unroll
                    for (int q2 = 0; q2 < GQ; ++q2) {
                        const int jj = j0 + q2;
                        const int64_t coff = __shfl_sync(0xffffffffu, lcoff, jj);
                        const int bc = __shfl_sync(0xffffffffu, lexp, jj);
                        if (!row_ok || bc < 0) continue;
                        const int64_t off = rowoff + coff;
                        const bool bad = badrow || bc == 0x7FF;
                        const double v0 = __longlong_as_double((long long)(bad ? nanb : bits[q2][0]));
                        if constexpr (CX) {
                            const double v1 = __longlong_as_double((long long)(bad ? nanb : bits[q2][NP - 1]));
                            ((double2 *)Cl)[off] = make_double2(v0, v1);
                        } else {
                            ((double *)Cl)[off] = v0;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int jj = 0; jj < NCOL; ++jj) {
                    const int64_t coff = __shfl_sync(0xffffffffu, lcoff, jj);
                    const int bc = __shfl_sync(0xffffffffu, lexp, jj);
                    if (!row_ok || bc < 0) continue;
                    const int j = CX ? 2 * jj : jj;
                    const int64_t off = rowoff + coff;
                    if (CX) ((float2 *)Cl)[off] = make_float2(accf[j], accf[j + 1]);
                    else ((float *)Cl)[off] = accf[j];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((uint32_t)TCOLS)
                     : "memory");
}

// A single contraction: its job in the parameter space (the tensor maps
// must lie in param, const or global memory for TMA).
template <int S, bool EXACT, bool CX>
__global__ void __launch_bounds__(OZ_THREADS, 1) k_oz_gemm(const __grid_constant__ OzJob job) {
    oz_gemm_body<S, EXACT, CX>(OzOneJob{&job});
}

// A group: every bucket of one kernel variant in one persistent launch.
template <int S, bool EXACT, bool CX>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_oz_gemm_grouped(const OzJob *__restrict__ jobs, const int64_t *__restrict__ start, int njobs) {
    oz_gemm_body<S, EXACT, CX>(OzJobTable{jobs, start, njobs});
}

// =============================================================================
// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing
// completes, with the production wait routine, and must come back with
// MGB_ERR_DEVICE_TIMEOUT in the status word.
// =============================================================================
__global__ void k_wait_selftest(int32_t *status) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) (void)mbar_wait(smem_u32(&bar), 0, &abort_flag, status);
    __syncthreads();
}

int selftest_wait_timeout(cudaStream_t s) {
    int32_t *status = device_status_ptr();
    if (!status) return fail(MGB_ERR_CUDA, "device status word unavailable");
    k_wait_selftest<<<1, 32, 0, s>>>(status);
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

// =============================================================================
// Host side
// =============================================================================
static uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

// |X| <= k_e * 2^(2W) * 2^(W(S-1)) * (1 + small) must stay below 2^95.
static bool oz_fits(int64_t k_e, int S) {
    const int W = oz_digit_bits(S);
    return std::log2((double)std::max<int64_t>(k_e, 1)) + 2 * W + W * (S - 1) + 1 < 94;
}

// Candidate slice counts of an adaptive plan: those whose exact accumulator
// holds K and whose digits could reach the tolerance at all (2^-(W S) within
// 64 tol; the estimate is at least about u for any data).
static uint32_t oz_candidates(int64_t k_e, double tol) {
    uint32_t m = 0;
    for (int S = 3; S <= 8; ++S)
        if (oz_fits(k_e, S) && std::ldexp(1.0, -oz_digit_bits(S) * S) <= 64.0 * tol) m |= 1u << S;
    return m;
}

// A plan's tensor-core tiles are 128 rows of A by oz_bn embedded columns of
// B (complex B embeds two columns per column). When A has few rows and B many
// columns, most of each 128-row tile is empty; C^T = B^T A^T puts the long
// side on the rows. The exact forms give the same digits and the same exact
// sums either way (the kept digit pairs and the adaptive error estimate are
// symmetric in A and B), so only the tile count decides.
void ozaki_orient(ContractionPlan &p) {
    if (p.form == MGB_FORM_PLAIN || p.swapped) return;
    const bool exact = p.form == MGB_FORM_OZAKI, cx = is_complex(p.compute_dtype);
    const int64_t bn = oz_bn(exact ? p.slices : 3, exact);
    auto tiles = [&](int64_t rows, int64_t cols) {
        return ((rows + OZ_BM - 1) / OZ_BM) * (((cx ? 2 : 1) * cols + bn - 1) / bn);
    };
    if (tiles(p.N, p.M) >= tiles(p.M, p.N)) return;
    std::swap(p.a, p.b);
    std::swap(p.gm, p.gn);
    for (ModeGroup *g : {&p.gm, &p.gn, &p.gk, &p.gl})
        for (int i = 0; i < kMaxRank; ++i) std::swap(g->str[0][i], g->str[1][i]);
    std::swap(p.M, p.N);
    std::swap(p.convert_a, p.convert_b);
    std::swap(p.pa, p.pb);
    p.swapped = true;
}

void ozaki_setup(ContractionPlan &p) {
    bool cx = is_complex(p.compute_dtype);
    if (p.adaptive) {
        const int64_t k_e = cx ? 2 * p.K : p.K;
        p.cand_mask = oz_candidates(k_e, p.tol);
        // the workspace holds the slices of the largest count that fits K, so
        // that a later tolerance never needs more
        p.slices = 0;
        for (int S = 8; S >= 3 && !p.slices; --S)
            if (oz_fits(k_e, S)) p.slices = S;
        if (!p.slices) p.slices = 3;  // K too long for any count: ozaki_setup reports it below
    }
    int S = p.slices;
    p.m_e = p.M;
    p.n_e = cx ? 2 * p.N : p.N;
    p.k_e = cx ? 2 * p.K : p.K;
    p.kpad = (p.k_e + 7) / 8 * 8;
    p.oz_w = oz_digit_bits(S);
    p.oz_kc = p.form == MGB_FORM_OZAKI ? 32 * oz_chunk_blocks(S) : OZ_KC;
    uint64_t off = 0;
    p.ws_a = off;
    off = align256(off + (uint64_t)p.L * S * p.m_e * p.kpad * 2);
    p.ws_b = off;
    off = align256(off + (uint64_t)p.L * S * p.n_e * p.kpad * 2);
    if (p.form == MGB_FORM_OZAKI) {
        p.ws_scale_a = off;
        off = align256(off + (uint64_t)p.L * p.M * 4);
        p.ws_scale_b = off;
        off = align256(off + (uint64_t)p.L * p.N * 4);
        p.oz_R = oz_fits(p.k_e, S) ? 0 : -1;  // -1: K too long for the exact accumulator
        if (p.adaptive) {
            // OzStats, P_A[L], P_B[L], q_A[L][K], q_B[L][K] (cleared every
            // call), then the exponent scan's partials of A and B
            // ([L][ceil(R / 32)][K] pairs, every one written every call)
            p.ws_stat = off;
            off = align256(off + sizeof(OzStats) + 2 * (uint64_t)p.L * 4);
            off = align256(off + 2 * (uint64_t)p.L * p.K * 4);
            off = align256(off + (uint64_t)p.L * ((p.M + 31) / 32) * p.K * 8);
            off = align256(off + (uint64_t)p.L * ((p.N + 31) / 32) * p.K * 8);
        }
    }
    p.ws_bytes = off;
}

// Statistics area of an adaptive plan inside the workspace.
struct OzStatArea {
    OzStats *st;
    float *pa, *pb, *qa, *qb;
    int2 *parta, *partb;
};
static OzStatArea stat_area(const ContractionPlan &p, void *ws) {
    OzStatArea a;
    uint8_t *w = (uint8_t *)ws + p.ws_stat;
    a.st = (OzStats *)w;
    a.pa = (float *)(w + sizeof(OzStats));
    a.pb = a.pa + p.L;
    uint64_t off = align256(p.ws_stat + sizeof(OzStats) + 2 * (uint64_t)p.L * 4);
    a.qa = (float *)((uint8_t *)ws + off);
    a.qb = a.qa + p.L * p.K;
    off = align256(off + 2 * (uint64_t)p.L * p.K * 4);
    a.parta = (int2 *)((uint8_t *)ws + off);
    off = align256(off + (uint64_t)p.L * ((p.M + 31) / 32) * p.K * 8);
    a.partb = (int2 *)((uint8_t *)ws + off);
    return a;
}
static uint64_t stat_bytes(const ContractionPlan &p) {
    return align256(align256(sizeof(OzStats) + 2 * (uint64_t)p.L * 4) + 2 * (uint64_t)p.L * p.K * 4);
}

PFN_encodeTiled_t tensor_map_encoder() {
    static PFN_encodeTiled_t fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_encodeTiled_t)p;
    });
    return fn;
}

static int make_map(CUtensorMap *tm, void *base, int64_t k_e, int64_t rows, int64_t planes,
                    int64_t kpad, int box_rows, int S) {
    PFN_encodeTiled_t enc = tensor_map_encoder();
    if (!enc) return fail(MGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)k_e, (cuuint64_t)rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)(kpad * 2 * rows)};
    cuuint32_t box[3] = {OZ_BK, (cuuint32_t)box_rows, (cuuint32_t)S};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(MGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return MGB_OK;
}

// Per-device caches, safe for concurrent callers: the values are idempotent,
// so a race only repeats the query or the attribute call.
constexpr int OZ_MAX_DEVICES = 64;

static int sm_count() {
    static std::atomic<int> count[OZ_MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    const bool cached = dev >= 0 && dev < OZ_MAX_DEVICES;
    int n = cached ? count[dev].load(std::memory_order_relaxed) : 0;
    if (n <= 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
        if (cached) count[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

template <typename K>
static int set_smem_attr(K kern, int smem, std::atomic<bool> (&done)[OZ_MAX_DEVICES]) {
    int dev = 0;
    cudaGetDevice(&dev);
    const bool cached = dev >= 0 && dev < OZ_MAX_DEVICES;
    if (!cached || !done[dev].load(std::memory_order_acquire)) {
        MGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        if (cached) done[dev].store(true, std::memory_order_release);
    }
    return MGB_OK;
}

// Persistent grids: one CTA per SM (the shared memory of a CTA exceeds half
// of an SM's), each walking its share of the tiles.
template <int S, bool EXACT, bool CX>
static int launch_gemm_t(const OzJob &job, int64_t tiles, cudaStream_t s) {
    auto kern = k_oz_gemm<S, EXACT, CX>;
    constexpr int smem = oz_smem_bytes(S, EXACT);
    static std::atomic<bool> attr_set[OZ_MAX_DEVICES];
    if (int st = set_smem_attr(kern, smem, attr_set)) return st;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, sm_count());
    kern<<<grid, OZ_THREADS, smem, s>>>(job);
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

template <int S, bool EXACT, bool CX>
static int launch_grouped_t(const OzJob *jobs, const int64_t *start, int njobs, int64_t tiles, cudaStream_t s) {
    auto kern = k_oz_gemm_grouped<S, EXACT, CX>;
    constexpr int smem = oz_smem_bytes(S, EXACT);
    static std::atomic<bool> attr_set[OZ_MAX_DEVICES];
    if (int st = set_smem_attr(kern, smem, attr_set)) return st;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, sm_count());
    kern<<<grid, OZ_THREADS, smem, s>>>(jobs, start, njobs);
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

// Dispatch on (slices, exact, complex): BF16X3 is S = 3 and not exact.
#define OZ_DISPATCH(CALL)                                                        \
    if (!exact) return cx ? CALL(3, false, true) : CALL(3, false, false);       \
    switch (S) {                                                                 \
    case 3: return cx ? CALL(3, true, true) : CALL(3, true, false);             \
    case 4: return cx ? CALL(4, true, true) : CALL(4, true, false);             \
    case 5: return cx ? CALL(5, true, true) : CALL(5, true, false);             \
    case 6: return cx ? CALL(6, true, true) : CALL(6, true, false);             \
    case 7: return cx ? CALL(7, true, true) : CALL(7, true, false);             \
    case 8: return cx ? CALL(8, true, true) : CALL(8, true, false);             \
    }                                                                            \
    return fail(MGB_ERR_ARGUMENT, "unsupported slice count");

static int launch_gemm(int S, bool exact, bool cx, const OzJob &job, int64_t tiles, cudaStream_t s) {
#define OZ_ONE(SS, EX, CC) launch_gemm_t<SS, EX, CC>(job, tiles, s)
    OZ_DISPATCH(OZ_ONE)
#undef OZ_ONE
}

static int launch_grouped(int S, bool exact, bool cx, const OzJob *jobs, const int64_t *start, int njobs,
                          int64_t tiles, cudaStream_t s) {
#define OZ_GRP(SS, EX, CC) launch_grouped_t<SS, EX, CC>(jobs, start, njobs, tiles, s)
    OZ_DISPATCH(OZ_GRP)
#undef OZ_GRP
}
#undef OZ_DISPATCH

static int unit_row_fast(const ModeGroup &gr, const ModeGroup &gk, int t) {
    int64_t sr = gr.n > 0 ? std::llabs(gr.str[t][0]) : INT64_MAX;
    int64_t sk = gk.n > 0 ? std::llabs(gk.str[t][0]) : INT64_MAX;
    return sr <= sk ? 1 : 0;
}

template <typename T, bool BF3>
static int run_prepass(const OpGeom &g, int mode, const void *X, int32_t *exps, int S, uint32_t *out,
                       int64_t rows_e, int64_t kw, int64_t L, cudaStream_t s, const int32_t *sel = nullptr) {
    int64_t tiles = ((g.R + 31) / 32) * ((g.K + OZ_SLICE_KT - 1) / OZ_SLICE_KT);
    if (tiles > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "operand too large for the slicer grid");
    dim3 grid((unsigned)tiles, (unsigned)L);
    const T *x = (const T *)X;
    switch (mode) {
    case MODE_REAL: k_oz_slice<T, MODE_REAL, BF3><<<grid, 256, 0, s>>>(x, g, exps, S, out, rows_e, kw, sel); break;
    case MODE_CA: k_oz_slice<T, MODE_CA, BF3><<<grid, 256, 0, s>>>(x, g, exps, S, out, rows_e, kw, sel); break;
    default: k_oz_slice<T, MODE_CB, BF3><<<grid, 256, 0, s>>>(x, g, exps, S, out, rows_e, kw, sel); break;
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

template <typename T>
static int run_scale(const OpGeom &g, const void *X, int32_t *exps, int64_t L, cudaStream_t s,
                     int32_t *emax = nullptr, int2 *part = nullptr) {
    int64_t tiles = ((g.R + 31) / 32) * ((g.K + OZ_SCAN_KT - 1) / OZ_SCAN_KT);
    if (tiles > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "operand too large for the scale grid");
    dim3 grid((unsigned)tiles, (unsigned)L);
    k_oz_scale<T><<<grid, 256, 0, s>>>((const T *)X, g, exps, emax, part);
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

static int run_stat(const int2 *part, const int32_t *exps, OzStats *st, int t, float *q, float *P, int64_t R,
                    int64_t K, int64_t L, cudaStream_t s) {
    const int64_t blocks = oz_stat_blocks(R, K);
    if (blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "operand too large for the statistics grid");
    k_oz_stat<<<dim3((unsigned)blocks, (unsigned)L), 256, 0, s>>>(part, exps, st, t, q, P, R, K);
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}
// Calls f with a null pointer of the operand's element type.
template <typename F>
static int by_type(int dtype, F &&f) {
    switch (dtype) {
    case MGB_F64: return f((double *)nullptr);
    case MGB_C64: return f((double2 *)nullptr);
    case MGB_F32: return f((float *)nullptr);
    default: return f((float2 *)nullptr);
    }
}
template <typename P>
using TypeOf = typename std::remove_pointer<P>::type;

// Pre-pass of the emulated forms: exponents (OZAKI) and slices of A and B
// into the workspace.
int ozaki_prepass(const ContractionPlan &p, const void *A, const void *B, void *ws, cudaStream_t s) {
    if (((uintptr_t)ws & 255) != 0) return fail(MGB_ERR_WORKSPACE, "workspace must be 256-byte aligned");
    const bool exact = p.form == MGB_FORM_OZAKI;
    const bool cx = is_complex(p.compute_dtype);
    const int S = p.slices;
    uint8_t *w = (uint8_t *)ws;
    uint32_t *sa = (uint32_t *)(w + p.ws_a), *sb = (uint32_t *)(w + p.ws_b);
    int32_t *ea = exact ? (int32_t *)(w + p.ws_scale_a) : nullptr;
    int32_t *eb = exact ? (int32_t *)(w + p.ws_scale_b) : nullptr;

    OpGeom ga, gb;
    ga.ptrs = p.pa;
    gb.ptrs = p.pb;
    ga.gr = p.gm; ga.gk = p.gk; ga.gl = p.gl; ga.t = 0; ga.R = p.M; ga.K = p.K;
    ga.rows_fast = unit_row_fast(p.gm, p.gk, 0);
    gb.gr = p.gn; gb.gk = p.gk; gb.gl = p.gl; gb.t = 1; gb.R = p.N; gb.K = p.K;
    gb.rows_fast = unit_row_fast(p.gn, p.gk, 1);
    const int64_t kw = p.kpad / 2;
    const int mode_a = cx ? MODE_CA : MODE_REAL, mode_b = cx ? MODE_CB : MODE_REAL;
    int st;
    if (exact) {
        MGB_CUDA_CHECK(cudaMemsetAsync(ea, 0, (size_t)p.L * p.M * 4, s));
        MGB_CUDA_CHECK(cudaMemsetAsync(eb, 0, (size_t)p.L * p.N * 4, s));
        OzStatArea sa_ = {};
        const int32_t *sel = nullptr;
        if (p.adaptive) {
            sa_ = stat_area(p, ws);
            MGB_CUDA_CHECK(cudaMemsetAsync(sa_.st, 0, stat_bytes(p), s));
            sel = &sa_.st->sel;
        }
        int32_t *emax_a = p.adaptive ? &sa_.st->emax[0] : nullptr, *emax_b = p.adaptive ? &sa_.st->emax[1] : nullptr;
        st = by_type(p.a.dtype,
                     [&](auto tag) { return run_scale<TypeOf<decltype(tag)>>(ga, A, ea, p.L, s, emax_a, sa_.parta); });
        if (st) return st;
        st = by_type(p.b.dtype,
                     [&](auto tag) { return run_scale<TypeOf<decltype(tag)>>(gb, B, eb, p.L, s, emax_b, sa_.partb); });
        if (st) return st;
        if (p.adaptive) {
            if ((st = run_stat(sa_.parta, ea, sa_.st, 0, sa_.qa, sa_.pa, p.M, p.K, p.L, s))) return st;
            if ((st = run_stat(sa_.partb, eb, sa_.st, 1, sa_.qb, sa_.pb, p.N, p.K, p.L, s))) return st;
            // Fluctuations of a Frobenius norm over few outputs: a margin that
            // vanishes for large results.
            const double margin = 1.0 + 2.0 / std::sqrt((double)std::max<int64_t>(p.M * p.N * p.L, 1));
            const int64_t eb = oz_est_blocks(p.K) * p.L;
            if (eb > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "operand too large for the estimate grid");
            k_oz_est<<<(unsigned)eb, 256, 0, s>>>(sa_.st, sa_.qa, sa_.qb, sa_.pa, sa_.pb, p.K);
            MGB_CUDA_CHECK(cudaGetLastError());
            k_oz_choose<<<1, 32, 0, s>>>(sa_.st, p.cand_mask, p.tol, margin, cx ? 1 : 0);
            MGB_CUDA_CHECK(cudaGetLastError());
        }
        st = by_type(p.a.dtype, [&](auto tag) {
            return run_prepass<TypeOf<decltype(tag)>, false>(ga, mode_a, A, ea, S, sa, p.m_e, kw, p.L, s, sel);
        });
        if (st) return st;
        st = by_type(p.b.dtype, [&](auto tag) {
            return run_prepass<TypeOf<decltype(tag)>, false>(gb, mode_b, B, eb, S, sb, p.n_e, kw, p.L, s, sel);
        });
        if (st) return st;
    } else {
        st = p.a.dtype == MGB_C32 ? run_prepass<float2, true>(ga, mode_a, A, nullptr, 3, sa, p.m_e, kw, p.L, s)
                                  : run_prepass<float, true>(ga, mode_a, A, nullptr, 3, sa, p.m_e, kw, p.L, s);
        if (st) return st;
        st = p.b.dtype == MGB_C32 ? run_prepass<float2, true>(gb, mode_b, B, nullptr, 3, sb, p.n_e, kw, p.L, s)
                                  : run_prepass<float, true>(gb, mode_b, B, nullptr, 3, sb, p.n_e, kw, p.L, s);
        if (st) return st;
    }
    return MGB_OK;
}

// The GEMM's view of a plan whose slices lie in `ws`.
static int ozaki_job(const ContractionPlan &p, void *C, void *ws, OzJob &job, int64_t &tiles, int S = 0,
                     const int32_t *sel = nullptr) {
    const bool exact = p.form == MGB_FORM_OZAKI;
    if (S == 0) S = p.slices;
    uint8_t *w = (uint8_t *)ws;
    uint32_t *sa = (uint32_t *)(w + p.ws_a), *sb = (uint32_t *)(w + p.ws_b);
    int32_t *status = device_status_ptr();
    if (!status) return fail(MGB_ERR_CUDA, "device status word unavailable");
    std::memset(&job, 0, sizeof(job));
    int st;
    if ((st = make_map(&job.tmA, sa, p.k_e, p.m_e, p.L * S, p.kpad, OZ_BM, S))) return st;
    const int bn = oz_bn(S, exact);
    if ((st = make_map(&job.tmB, sb, p.k_e, p.n_e, p.L * S, p.kpad, bn, S))) return st;
    OzGemmArgs &a = job.a;
    a.M = p.M;
    a.Ne = p.n_e;
    a.N = p.N;
    a.nkb = (int32_t)((p.k_e + OZ_BK - 1) / OZ_BK);
    a.kcb = exact ? oz_chunk_blocks(S) : OZ_KC / OZ_BK;
    a.S = S;
    a.expA = exact ? (int32_t *)(w + p.ws_scale_a) : nullptr;
    a.expB = exact ? (int32_t *)(w + p.ws_scale_b) : nullptr;
    a.C = C;
    a.cptr = p.pc;
    if (p.band > 0) {
        a.band = p.band;
    } else {
        a.band = OZ_GROUP_M;
        while (a.band > 1 && (int64_t)a.band * OZ_BM * p.kpad * S * 2 > OZ_BAND_BYTES) --a.band;
    }
    a.gm = p.gm;
    a.gn = p.gn;
    a.gl = p.gl;
    a.status = status;
    a.sel = sel;
    if (a.gm.n == 0) { a.gm.n = 1; a.gm.ext[0] = 1; for (int t = 0; t < 3; ++t) a.gm.str[t][0] = 0; }
    if (a.gn.n == 0) { a.gn.n = 1; a.gn.ext[0] = 1; for (int t = 0; t < 3; ++t) a.gn.str[t][0] = 0; }
    job.tiles_n = (int32_t)((p.n_e + bn - 1) / bn);
    job.tiles_m = (int32_t)((p.M + OZ_BM - 1) / OZ_BM);
    job.L = (int32_t)p.L;
    if ((p.n_e + bn - 1) / bn > INT32_MAX || (p.M + OZ_BM - 1) / OZ_BM > INT32_MAX || p.L > INT32_MAX)
        return fail(MGB_ERR_UNSUPPORTED, "contraction too large for the tile grid");
    tiles = (int64_t)job.tiles_n * job.tiles_m * job.L;
    return MGB_OK;
}

int ozaki_gemm(const ContractionPlan &p, const void *A, const void *B, void *C, void *ws, cudaStream_t s) {
    int st;
    OzJob job;
    int64_t tiles = 0;
    if (!p.adaptive) {
        if ((st = ozaki_job(p, C, ws, job, tiles))) return st;
        return launch_gemm(p.slices, p.form == MGB_FORM_OZAKI, is_complex(p.compute_dtype), job, tiles, s);
    }
    // Every candidate is launched; the kernel of the chosen count works and
    // the others return at once. With no count chosen the plain form runs.
    const int32_t *sel = &stat_area(p, ws).st->sel;
    for (int S = 3; S <= 8; ++S) {
        if (!(p.cand_mask & (1u << S))) continue;
        if ((st = ozaki_job(p, C, ws, job, tiles, S, sel))) return st;
        if ((st = launch_gemm(S, true, is_complex(p.compute_dtype), job, tiles, s))) return st;
    }
    return launch_plain_gemm(p, A, B, C, s, sel);
}

int launch_ozaki(const ContractionPlan &p, const void *A, const void *B, void *C, void *ws,
                 cudaStream_t s, cudaEvent_t mid) {
    int st = ozaki_prepass(p, A, B, ws, s);
    if (st) return st;
    if (mid) MGB_CUDA_CHECK(cudaEventRecord(mid, s));
    return ozaki_gemm(p, A, B, C, ws, s);
}

int ozaki_adaptive_report(const ContractionPlan &p, const void *ws, cudaStream_t s, mgb_adaptive_report *out) {
    if (!p.adaptive) return fail(MGB_ERR_ARGUMENT, "adaptive report: the plan has a fixed slice count");
    if (!ws) return fail(MGB_ERR_ARGUMENT, "adaptive report: null workspace");
    OzStats h;
    MGB_CUDA_CHECK(cudaMemcpyAsync(&h, stat_area(p, const_cast<void *>(ws)).st, sizeof(h), cudaMemcpyDeviceToHost, s));
    MGB_CUDA_CHECK(cudaStreamSynchronize(s));
    std::memset(out, 0, sizeof(*out));
    out->slices = h.sel;
    out->nonfinite = h.nonfinite;
    for (int S = 0; S <= 8; ++S) out->estimate[S] = (p.cand_mask & (1u << S)) ? (double)h.est[S] : 0.0;
    out->tolerance = p.tol;
    return MGB_OK;
}

int ozaki_set_tolerance(ContractionPlan &p, double tol) {
    if (!p.adaptive) return fail(MGB_ERR_ARGUMENT, "tolerance: the plan has a fixed slice count");
    if (!(tol > 0.0)) return fail(MGB_ERR_ARGUMENT, "tolerance must be positive");
    p.tol = tol;
    p.cand_mask = oz_candidates(is_complex(p.compute_dtype) ? 2 * p.K : p.K, tol);
    return MGB_OK;
}

// ---- one persistent GEMM launch for several plans of one kernel variant ----
struct OzGrouped {
    int S = 0;
    bool exact = false, cx = false;
    int njobs = 0;
    int64_t tiles = 0;
    OzJob *jobs = nullptr;     // device
    int64_t *start = nullptr;  // device [njobs + 1]
};

int ozaki_grouped_create(const std::vector<const ContractionPlan *> &plans, const std::vector<void *> &ws, int S,
                         bool exact, bool cx, OzGrouped **out) {
    *out = nullptr;
    if (plans.empty()) return fail(MGB_ERR_ARGUMENT, "grouped GEMM: no plans");
    auto *g = new OzGrouped();
    g->S = S;
    g->exact = exact;
    g->cx = cx;
    std::vector<OzJob> host(plans.size());
    std::vector<int64_t> start(plans.size() + 1, 0);
    for (size_t i = 0; i < plans.size(); ++i) {
        const ContractionPlan &p = *plans[i];
        const bool variant_ok = (p.form == MGB_FORM_OZAKI) == exact && is_complex(p.compute_dtype) == cx &&
                                (p.adaptive ? exact && (p.cand_mask & (1u << S)) != 0 : p.slices == S);
        if (!variant_ok) {
            delete g;
            return fail(MGB_ERR_ARGUMENT, "grouped GEMM: plans of different kernel variants");
        }
        int64_t t = 0;
        // an adaptive plan's job works only when its device choice is S
        const int st = p.adaptive ? ozaki_job(p, nullptr, ws[i], host[i], t, S, &stat_area(p, ws[i]).st->sel)
                                  : ozaki_job(p, nullptr, ws[i], host[i], t);
        if (st) {
            delete g;
            return st;
        }
        start[i + 1] = start[i] + t;
    }
    g->njobs = (int)plans.size();
    g->tiles = start.back();
    cudaError_t e = cudaMalloc((void **)&g->jobs, host.size() * sizeof(OzJob));
    if (e == cudaSuccess) e = cudaMalloc((void **)&g->start, start.size() * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMemcpy(g->jobs, host.data(), host.size() * sizeof(OzJob), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(g->start, start.data(), start.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        ozaki_grouped_destroy(g);
        return cuda_fail(e, "grouped GEMM job table");
    }
    *out = g;
    return MGB_OK;
}

int ozaki_grouped_launch(const OzGrouped *g, cudaStream_t s) {
    if (g->tiles == 0) return MGB_OK;
    return launch_grouped(g->S, g->exact, g->cx, g->jobs, g->start, g->njobs, g->tiles, s);
}

void ozaki_grouped_destroy(OzGrouped *g) {
    if (!g) return;
    if (g->jobs) cudaFree(g->jobs);
    if (g->start) cudaFree(g->start);
    delete g;
}


// =============================================================================
// Batched execution of many different contractions (the serving form): one
// launch per pre-pass phase over a table of operands, one multi-job chooser,
// and one persistent tensor-core launch per kernel variant over a table of
// (contraction, slice count) jobs.
// =============================================================================
enum { PRE_ZERO = 0, PRE_SCALE = 1, PRE_STAT = 2, PRE_SLICE = 3, PRE_PHASES = 4 };

// One operand of one contraction.
struct PreJob {
    OpGeom g;
    const void *X;
    int32_t dtype;      // the operand's element type
    int32_t mode;       // MODE_REAL / MODE_CA / MODE_CB
    int32_t bf3;        // BF16X3 pieces instead of Ozaki digits
    int32_t S;          // slice count when `sel` is null
    int32_t t;          // 0 = A, 1 = B
    int32_t L;
    int32_t *exps;      // [L][R] (Ozaki)
    int32_t *emax;      // largest exponent of the operand (adaptive) or null
    uint32_t *out;      // slice planes
    int64_t rows_e, kw;
    const int32_t *sel; // adaptive choice of the contraction, or null
    OzStats *st;        // its statistics (adaptive) or null
    float *q, *P;       // this operand's per-k norms and squared scales
    int2 *part;         // the exponent scan's partials of this operand (adaptive) or null
    void *zero[2];      // regions cleared by PRE_ZERO (exponents; statistics for t == 0)
    int64_t zero_words[2];
    int64_t tiles[PRE_PHASES];  // blocks of every phase
};

// One adaptive contraction for the multi-job chooser.
struct ChooseJob {
    OzStats *st;
    const float *qa, *qb, *pa, *pb;
    int64_t K, L;
    uint32_t cand;
    int32_t cx;
    double tol, margin;
};

union PreSmem {
    ScaleSmem scale;
    StatSmem stat;
    SliceSmemOf<double, MODE_REAL> s_dr;
    SliceSmemOf<double2, MODE_CA> s_zc;
    SliceSmemOf<double, MODE_CA> s_dc;
    SliceSmemOf<float, MODE_REAL> s_fr;
    SliceSmemOf<float2, MODE_CA> s_cc;
    SliceSmemOf<float, MODE_CA> s_fc;
};

template <typename T, bool BF3>
__device__ __forceinline__ void pre_slice_typed(const PreJob &J, int S, int64_t blk, int64_t l, PreSmem &sm) {
    const T *X = (const T *)J.X;
    switch (J.mode) {
    case MODE_REAL:
        if constexpr (!OzIn<T>::cx)
            oz_slice_tile<T, MODE_REAL, BF3>(X, J.g, J.exps, S, J.out, J.rows_e, J.kw, blk, l,
                                             *reinterpret_cast<SliceSmemOf<T, MODE_REAL> *>(&sm));
        break;
    case MODE_CA:
        oz_slice_tile<T, MODE_CA, BF3>(X, J.g, J.exps, S, J.out, J.rows_e, J.kw, blk, l,
                                       *reinterpret_cast<SliceSmemOf<T, MODE_CA> *>(&sm));
        break;
    default:
        oz_slice_tile<T, MODE_CB, BF3>(X, J.g, J.exps, S, J.out, J.rows_e, J.kw, blk, l,
                                       *reinterpret_cast<SliceSmemOf<T, MODE_CB> *>(&sm));
        break;
    }
}

__global__ void __launch_bounds__(256, 3) k_oz_pre_multi(const PreJob *__restrict__ jobs,
                                                         const int64_t *__restrict__ start, int njobs, int phase) {
    __shared__ __align__(16) PreSmem sm;
    const int64_t b = blockIdx.x;
    int lo = 0, hi = njobs - 1;  // the last job whose first block is <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (start[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const PreJob &J = jobs[lo];
    const int64_t local = b - start[lo];
    if (phase == PRE_ZERO) {
        for (int r = 0; r < 2; ++r) {  // this job's blocks clear both regions
            int32_t *z = (int32_t *)J.zero[r];
            const int64_t n = J.zero_words[r], nb = J.tiles[PRE_ZERO];
            for (int64_t w = local * blockDim.x + threadIdx.x; w < n; w += nb * blockDim.x) z[w] = 0;
        }
        return;
    }
    const int64_t per_l = J.tiles[phase] / max(J.L, 1);
    const int64_t l = local / per_l, blk = local - l * per_l;
    if (phase == PRE_SCALE) {
        switch (J.dtype) {
        case MGB_F64: oz_scale_tile<double>((const double *)J.X, J.g, J.exps, J.emax, J.part, blk, l, sm.scale); break;
        case MGB_C64: oz_scale_tile<double2>((const double2 *)J.X, J.g, J.exps, J.emax, J.part, blk, l, sm.scale); break;
        case MGB_F32: oz_scale_tile<float>((const float *)J.X, J.g, J.exps, J.emax, J.part, blk, l, sm.scale); break;
        default: oz_scale_tile<float2>((const float2 *)J.X, J.g, J.exps, J.emax, J.part, blk, l, sm.scale); break;
        }
    } else if (phase == PRE_STAT) {
        oz_stat_block(J.part, J.exps, J.st, J.t, J.q, J.P, J.g.R, J.g.K, blk, l, sm.stat);
    } else {
        int S = J.S;
        if (J.sel) {
            S = *J.sel;
            if (S == 0) return;  // the plain form will run this contraction
        }
        if (J.bf3) {
            if (J.dtype == MGB_C32) pre_slice_typed<float2, true>(J, 3, blk, l, sm);
            else pre_slice_typed<float, true>(J, 3, blk, l, sm);
        } else {
            switch (J.dtype) {
            case MGB_F64: pre_slice_typed<double, false>(J, S, blk, l, sm); break;
            case MGB_C64: pre_slice_typed<double2, false>(J, S, blk, l, sm); break;
            case MGB_F32: pre_slice_typed<float, false>(J, S, blk, l, sm); break;
            default: pre_slice_typed<float2, false>(J, S, blk, l, sm); break;
            }
        }
    }
}

// dst[i] = *src[i]: every item's slice count after the choice
// The last job of a table whose first block is <= b.
__device__ __forceinline__ int multi_job(const int64_t *__restrict__ start, int njobs, int64_t b) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (start[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Exponent scan over a table of operand jobs of one element type: the same
// tile routine, shared memory and occupancy as the single-plan scan, for
// many operands in one launch (no launch per operand, one tail for all).
template <typename T>
__global__ void __launch_bounds__(256, 4) k_oz_scale_multi(const PreJob *__restrict__ jobs,
                                                        const int64_t *__restrict__ start, int njobs) {
    __shared__ ScaleSmem sm;
    const int j = multi_job(start, njobs, blockIdx.x);
    const PreJob &J = jobs[j];
    const int64_t local = blockIdx.x - start[j];
    const int64_t per_l = J.tiles[PRE_SCALE] / max(J.L, 1);
    const int64_t l = local / per_l;
    oz_scale_tile<T>((const T *)J.X, J.g, J.exps, J.emax, J.part, local - l * per_l, l, sm);
}

// Slicing over a table of operand jobs of one element type, embedding and
// form, as the single-plan slicer does it.
template <typename T, int MODE, bool BF3>
__global__ void __launch_bounds__(256, 4) k_oz_slice_multi(const PreJob *__restrict__ jobs,
                                                        const int64_t *__restrict__ start, int njobs) {
    __shared__ SliceSmemOf<T, MODE> sm;
    const int j = multi_job(start, njobs, blockIdx.x);
    const PreJob &J = jobs[j];
    int S = J.S;
    if (J.sel) {
        S = *J.sel;
        if (S == 0) return;  // the plain form will run this contraction
    }
    const int64_t local = blockIdx.x - start[j];
    const int64_t per_l = J.tiles[PRE_SLICE] / max(J.L, 1);
    const int64_t l = local / per_l;
    oz_slice_tile<T, MODE, BF3>((const T *)J.X, J.g, J.exps, S, J.out, J.rows_e, J.kw, local - l * per_l, l, sm);
}

__global__ void k_gather_sel(const int32_t *const *__restrict__ src, int32_t *__restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = *src[i];
}

// One block per adaptive contraction (the body of k_oz_choose).
// The estimate's sums of every adaptive contraction of a batch: job j owns
// blocks [start[j], start[j + 1]) (oz_est_blocks(K) per batch entry).
__global__ void __launch_bounds__(256) k_oz_est_multi(const ChooseJob *__restrict__ jobs,
                                                      const int64_t *__restrict__ start, int njobs) {
    __shared__ double red[2][8];
    const int64_t b = blockIdx.x;
    int lo = 0, hi = njobs - 1;  // the last job whose first block is <= b
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (start[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const ChooseJob &c = jobs[lo];
    const int64_t local = b - start[lo], nb = oz_est_blocks(c.K), l = local / nb;
    oz_est_block(c.st, c.qa, c.qb, c.pa, c.pb, c.K, local - l * nb, l, red);
}
// One thread per adaptive contraction: its estimate and choice.
__global__ void k_oz_choose_multi(const ChooseJob *__restrict__ jobs, int njobs) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < njobs) oz_choose_final(jobs[j].st, jobs[j].cand, jobs[j].tol, jobs[j].margin, jobs[j].cx);
}

struct OzBatchBuffers {
    // device tables and their pinned staging, grown on demand
    uint8_t *dev = nullptr, *host = nullptr;
    size_t cap = 0;
    cudaEvent_t staged = nullptr;  // the last upload has left the staging area
};

OzBatchBuffers *ozaki_batch_buffers_create() { return new OzBatchBuffers(); }

void ozaki_batch_buffers_destroy(OzBatchBuffers *b) {
    if (!b) return;
    if (b->staged) cudaEventSynchronize(b->staged), cudaEventDestroy(b->staged);
    if (b->dev) cudaFree(b->dev);
    if (b->host) cudaFreeHost(b->host);
    delete b;
}

static int batch_reserve(OzBatchBuffers *b, size_t bytes) {
    if (b->staged) MGB_CUDA_CHECK(cudaEventSynchronize(b->staged));  // the previous upload read the staging
    if (bytes <= b->cap) return MGB_OK;
    size_t cap = std::max(bytes, 2 * b->cap);
    if (b->dev) cudaFree(b->dev);
    if (b->host) cudaFreeHost(b->host);
    b->dev = b->host = nullptr;
    b->cap = 0;
    MGB_CUDA_CHECK(cudaMalloc((void **)&b->dev, cap));
    MGB_CUDA_CHECK(cudaMallocHost((void **)&b->host, cap));
    b->cap = cap;
    if (!b->staged) MGB_CUDA_CHECK(cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming));
    return MGB_OK;
}

static void fill_prejob(PreJob &J, const ContractionPlan &p, int t, const void *X, void *ws) {
    std::memset(&J, 0, sizeof(J));
    const bool cx = is_complex(p.compute_dtype), exact = p.form == MGB_FORM_OZAKI;
    uint8_t *w = (uint8_t *)ws;
    // one operand, or (X null) the plan's per-batch-entry pointer table
    J.g.ptrs = X ? nullptr : (t == 0 ? p.pa : p.pb);
    J.g.gr = t == 0 ? p.gm : p.gn;
    J.g.gk = p.gk;
    J.g.gl = p.gl;
    J.g.t = t;
    J.g.R = t == 0 ? p.M : p.N;
    J.g.K = p.K;
    J.g.rows_fast = unit_row_fast(J.g.gr, p.gk, t);
    J.X = X;
    J.dtype = t == 0 ? p.a.dtype : p.b.dtype;
    J.mode = cx ? (t == 0 ? MODE_CA : MODE_CB) : MODE_REAL;
    J.bf3 = exact ? 0 : 1;
    J.S = exact ? p.slices : 3;
    J.t = t;
    J.L = (int32_t)p.L;
    J.exps = exact ? (int32_t *)(w + (t == 0 ? p.ws_scale_a : p.ws_scale_b)) : nullptr;
    J.out = (uint32_t *)(w + (t == 0 ? p.ws_a : p.ws_b));
    J.rows_e = t == 0 ? p.m_e : p.n_e;
    J.kw = p.kpad / 2;
    const int64_t R = J.g.R, K = p.K, L = p.L;
    int64_t zw = 0;
    if (exact) {
        J.zero[0] = J.exps;
        J.zero_words[0] = L * R;
        zw += L * R;
        if (p.adaptive) {
            OzStatArea a = stat_area(p, ws);
            J.sel = &a.st->sel;
            J.st = a.st;
            J.emax = &a.st->emax[t];
            J.q = t == 0 ? a.qa : a.qb;
            J.P = t == 0 ? a.pa : a.pb;
            J.part = t == 0 ? a.parta : a.partb;
            if (t == 0) {
                J.zero[1] = a.st;
                J.zero_words[1] = (int64_t)(stat_bytes(p) / 4);
                zw += J.zero_words[1];
            }
        }
    }
    J.tiles[PRE_ZERO] = zw ? std::min<int64_t>((zw + 1023) / 1024, 64) : 0;
    J.tiles[PRE_SCALE] = exact ? ((R + 31) / 32) * ((K + OZ_SCAN_KT - 1) / OZ_SCAN_KT) * L : 0;
    J.tiles[PRE_STAT] = (exact && p.adaptive) ? oz_stat_blocks(R, K) * L : 0;
    J.tiles[PRE_SLICE] = ((R + 31) / 32) * ((K + OZ_SLICE_KT - 1) / OZ_SLICE_KT) * L;
}

// The chooser's job for an adaptive plan whose statistics lie in `ws`.
static ChooseJob choose_job(const ContractionPlan &p, void *ws) {
    OzStatArea a = stat_area(p, ws);
    ChooseJob c;
    c.st = a.st;
    c.qa = a.qa;
    c.qb = a.qb;
    c.pa = a.pa;
    c.pb = a.pb;
    c.K = p.K;
    c.L = p.L;
    c.cand = p.cand_mask;
    c.cx = is_complex(p.compute_dtype) ? 1 : 0;
    c.tol = p.tol;
    c.margin = 1.0 + 2.0 / std::sqrt((double)std::max<int64_t>(p.M * p.N * p.L, 1));
    return c;
}

// Pre-pass tables of emulated items: two operand jobs per item (operands
// given by pointer, or, when null, by the plan's pointer tables), one
// chooser job per adaptive item.
static int pre_tables(const std::vector<OzBatchItem> &items, std::vector<PreJob> &pre, std::vector<ChooseJob> &choose) {
    pre.assign(2 * items.size(), PreJob{});
    choose.clear();
    for (size_t i = 0; i < items.size(); ++i) {
        const OzBatchItem &it = items[i];
        const ContractionPlan &p = *it.p;
        if (p.form == MGB_FORM_PLAIN) return fail(MGB_ERR_ARGUMENT, "batch: plain-form plans are not batched");
        if (((uintptr_t)it.ws & 255) != 0) return fail(MGB_ERR_WORKSPACE, "batch: workspace must be 256-byte aligned");
        fill_prejob(pre[2 * i], p, 0, p.swapped ? it.B : it.A, it.ws);
        fill_prejob(pre[2 * i + 1], p, 1, p.swapped ? it.A : it.B, it.ws);
        if (p.adaptive) choose.push_back(choose_job(p, it.ws));
    }
    // operand jobs of one (form, element type, embedding) lie together: the
    // scan and the slicer run one launch per such segment
    std::stable_sort(pre.begin(), pre.end(), [](const PreJob &u, const PreJob &v) {
        return std::make_tuple(u.bf3, u.dtype, u.mode) < std::make_tuple(v.bf3, v.dtype, v.mode);
    });
    return MGB_OK;
}

// Byte offsets of the pre-pass tables in one device area: [pre jobs]
// [block starts of each phase][chooser jobs][their estimate blocks' starts].
struct PreSegment {
    int first = 0, count = 0;  // operand jobs [first, first + count)
    int32_t bf3 = 0, dtype = 0, mode = 0;
    size_t o_scale = 0, o_slice = 0;  // their block starts of the scan and the slicer
    int64_t scale_blocks = 0, slice_blocks = 0;
};
struct PreLayout {
    size_t o_pre = 0, o_pst = 0, o_ch = 0, o_cs = 0, end = 0;
    int64_t blocks[PRE_PHASES] = {};
    int64_t est_blocks = 0;
    std::vector<PreSegment> seg;  // runs of jobs with one (form, element type, embedding)
};
static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
static PreLayout pre_layout(const std::vector<PreJob> &pre, const std::vector<ChooseJob> &choose, size_t base) {
    PreLayout L;
    size_t off = base;
    L.o_pre = off;
    off = al256(off + pre.size() * sizeof(PreJob));
    L.o_pst = off;
    off = al256(off + PRE_PHASES * (pre.size() + 1) * sizeof(int64_t));
    L.o_ch = off;
    off = al256(off + choose.size() * sizeof(ChooseJob));
    L.o_cs = off;
    off = al256(off + (choose.size() + 1) * sizeof(int64_t));
    for (size_t j = 0; j < pre.size();) {
        PreSegment g;
        g.first = (int)j;
        g.bf3 = pre[j].bf3;
        g.dtype = pre[j].dtype;
        g.mode = pre[j].mode;
        while (j < pre.size() && pre[j].bf3 == g.bf3 && pre[j].dtype == g.dtype && pre[j].mode == g.mode) ++j;
        g.count = (int)j - g.first;
        g.o_scale = off;
        off = al256(off + (g.count + 1) * sizeof(int64_t));
        g.o_slice = off;
        off = al256(off + (g.count + 1) * sizeof(int64_t));
        L.seg.push_back(g);
    }
    L.end = off;
    return L;
}
// Writes the tables at their offsets of host area `h` and fills the block counts.
static void pre_write(PreLayout &L, const std::vector<PreJob> &pre, const std::vector<ChooseJob> &choose, uint8_t *h) {
    std::memcpy(h + L.o_pre, pre.data(), pre.size() * sizeof(PreJob));
    int64_t *pst = (int64_t *)(h + L.o_pst);
    for (int ph = 0; ph < PRE_PHASES; ++ph) {
        int64_t *st = pst + ph * (pre.size() + 1);
        st[0] = 0;
        for (size_t j = 0; j < pre.size(); ++j) st[j + 1] = st[j] + pre[j].tiles[ph];
        L.blocks[ph] = st[pre.size()];
    }
    for (PreSegment &g : L.seg) {
        int64_t *a = (int64_t *)(h + g.o_scale), *b = (int64_t *)(h + g.o_slice);
        a[0] = b[0] = 0;
        for (int j = 0; j < g.count; ++j) {
            a[j + 1] = a[j] + pre[g.first + j].tiles[PRE_SCALE];
            b[j + 1] = b[j] + pre[g.first + j].tiles[PRE_SLICE];
        }
        g.scale_blocks = a[g.count];
        g.slice_blocks = b[g.count];
    }
    std::memcpy(h + L.o_ch, choose.data(), choose.size() * sizeof(ChooseJob));
    int64_t *cst = (int64_t *)(h + L.o_cs);
    cst[0] = 0;
    for (size_t j = 0; j < choose.size(); ++j) cst[j + 1] = cst[j] + oz_est_blocks(choose[j].K) * choose[j].L;
    L.est_blocks = cst[choose.size()];
}
// One typed launch of phase `ph` (scan or slicing) over segment `g`.
static int seg_launch(const PreSegment &g, int ph, const PreJob *dpre, const uint8_t *d, cudaStream_t s) {
    const int64_t blocks = ph == PRE_SCALE ? g.scale_blocks : g.slice_blocks;
    if (blocks == 0) return MGB_OK;
    if (blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "batch: pre-pass grid too large");
    const PreJob *jobs = dpre + g.first;
    const int64_t *st = (const int64_t *)(d + (ph == PRE_SCALE ? g.o_scale : g.o_slice));
    const unsigned nb = (unsigned)blocks;
    if (ph == PRE_SCALE) {
        switch (g.dtype) {
        case MGB_F64: k_oz_scale_multi<double><<<nb, 256, 0, s>>>(jobs, st, g.count); break;
        case MGB_C64: k_oz_scale_multi<double2><<<nb, 256, 0, s>>>(jobs, st, g.count); break;
        case MGB_F32: k_oz_scale_multi<float><<<nb, 256, 0, s>>>(jobs, st, g.count); break;
        default: k_oz_scale_multi<float2><<<nb, 256, 0, s>>>(jobs, st, g.count); break;
        }
    } else {
#define MGB_SLICE_MULTI(T, MODE, BF3) k_oz_slice_multi<T, MODE, BF3><<<nb, 256, 0, s>>>(jobs, st, g.count)
        auto by_mode = [&](auto tag, bool bf3) {
            using T = typename std::remove_pointer<decltype(tag)>::type;
            if (bf3) {
                if constexpr (std::is_same<T, float>::value || std::is_same<T, float2>::value) {
                    if (g.mode == MODE_CA) MGB_SLICE_MULTI(T, MODE_CA, true);
                    else if (g.mode == MODE_CB) MGB_SLICE_MULTI(T, MODE_CB, true);
                    else if constexpr (!OzIn<T>::cx) MGB_SLICE_MULTI(T, MODE_REAL, true);
                }
            } else {
                if (g.mode == MODE_CA) MGB_SLICE_MULTI(T, MODE_CA, false);
                else if (g.mode == MODE_CB) MGB_SLICE_MULTI(T, MODE_CB, false);
                else if constexpr (!OzIn<T>::cx) MGB_SLICE_MULTI(T, MODE_REAL, false);
            }
        };
#undef MGB_SLICE_MULTI
        switch (g.dtype) {
        case MGB_F64: by_mode((double *)nullptr, g.bf3 != 0); break;
        case MGB_C64: by_mode((double2 *)nullptr, g.bf3 != 0); break;
        case MGB_F32: by_mode((float *)nullptr, g.bf3 != 0); break;
        default: by_mode((float2 *)nullptr, g.bf3 != 0); break;
        }
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

// Every pre-pass phase over the tables at device area `d`: clearing and the
// statistics as one launch each, the scan and the slicing as one typed
// launch per segment, the estimate and the choice before the slicing.
static int pre_launch(const PreLayout &L, size_t npre, size_t nch, const uint8_t *d, cudaStream_t s) {
    const PreJob *dpre = (const PreJob *)(d + L.o_pre);
    for (int ph = 0; ph < PRE_PHASES; ++ph) {
        if (ph == PRE_SLICE && nch > 0) {
            if (L.est_blocks > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "batch: estimate grid too large");
            if (L.est_blocks > 0) {
                k_oz_est_multi<<<(unsigned)L.est_blocks, 256, 0, s>>>((const ChooseJob *)(d + L.o_ch),
                                                                      (const int64_t *)(d + L.o_cs), (int)nch);
                MGB_CUDA_CHECK(cudaGetLastError());
            }
            k_oz_choose_multi<<<((int)nch + 127) / 128, 128, 0, s>>>((const ChooseJob *)(d + L.o_ch), (int)nch);
            MGB_CUDA_CHECK(cudaGetLastError());
        }
        if (ph == PRE_SCALE || ph == PRE_SLICE) {
            for (const PreSegment &g : L.seg)
                if (int st = seg_launch(g, ph, dpre, d, s)) return st;
            continue;
        }
        if (L.blocks[ph] == 0) continue;
        if (L.blocks[ph] > INT32_MAX) return fail(MGB_ERR_UNSUPPORTED, "batch: pre-pass grid too large");
        k_oz_pre_multi<<<(unsigned)L.blocks[ph], 256, 0, s>>>(dpre, (const int64_t *)(d + L.o_pst) + ph * (npre + 1),
                                                              (int)npre, ph);
        MGB_CUDA_CHECK(cudaGetLastError());
    }
    return MGB_OK;
}

// The plain-form candidate of an adaptive plan (runs only when the device
// chose no slice count), after its pre-pass into `ws`.
int ozaki_plain_fallback(const ContractionPlan &p, const void *A, const void *B, void *C, void *ws, cudaStream_t s) {
    if (!p.adaptive) return MGB_OK;
    return launch_plain_gemm(p, A, B, C, s, &stat_area(p, ws).st->sel);
}

int ozaki_batch_launch(const std::vector<OzBatchItem> &items, OzBatchBuffers *buf, cudaStream_t s,
                       int32_t *sel_dev_out, const std::function<int()> &after_prepass,
                       const std::function<int(int S, bool exact, bool cx)> &after_variant) {
    const int n = (int)items.size();
    if (n == 0) return MGB_OK;
    int32_t *status = device_status_ptr();
    if (!status) return fail(MGB_ERR_CUDA, "device status word unavailable");
    // ---- host tables
    std::vector<PreJob> pre;
    std::vector<ChooseJob> choose;
    if (int st = pre_tables(items, pre, choose)) return st;
    // GEMM jobs per variant: key (S, exact, cx) ordered cheapest first
    std::map<std::tuple<int, int, int>, std::vector<OzJob>> gem;
    for (int i = 0; i < n; ++i) {
        const OzBatchItem &it = items[i];
        const ContractionPlan &p = *it.p;
        const bool exact = p.form == MGB_FORM_OZAKI, cx = is_complex(p.compute_dtype);
        if (p.adaptive) {
            OzStatArea a = stat_area(p, it.ws);
            for (int S = 3; S <= 8; ++S) {
                if (!(p.cand_mask & (1u << S))) continue;
                OzJob job;
                int64_t tiles;
                if (int st = ozaki_job(p, it.C, it.ws, job, tiles, S, &a.st->sel)) return st;
                gem[std::make_tuple(S, 1, cx ? 1 : 0)].push_back(job);
            }
        } else {
            OzJob job;
            int64_t tiles;
            if (int st = ozaki_job(p, it.C, it.ws, job, tiles)) return st;
            gem[std::make_tuple(exact ? p.slices : 3, exact ? 1 : 0, cx ? 1 : 0)].push_back(job);
        }
    }
    // longest tiles first in every variant's launch: each CTA ends its walk
    // on short tiles, which even out the CTAs' finishing times
    for (auto &kv : gem)
        std::stable_sort(kv.second.begin(), kv.second.end(),
                         [](const OzJob &u, const OzJob &v) { return u.a.nkb > v.a.nkb; });
    // ---- one staging area: [pre-pass tables][per item: fixed slice count,
    //      address of its slice count][per variant: jobs, starts]
    auto al = al256;
    PreLayout PL = pre_layout(pre, choose, 0);
    size_t off = PL.end;
    // per item: the address of its slice count (adaptive: the choice; else
    // the fixed count stored here)
    const size_t o_fix = off;
    off = al(off + n * sizeof(int32_t));
    const size_t o_sp = off;
    off = al(off + n * sizeof(void *));
    std::vector<size_t> o_gj, o_gs;
    for (auto &kv : gem) {
        o_gj.push_back(off);
        off = al(off + kv.second.size() * sizeof(OzJob));
        o_gs.push_back(off);
        off = al(off + (kv.second.size() + 1) * sizeof(int64_t));
    }
    if (int st = batch_reserve(buf, off)) return st;
    uint8_t *h = buf->host, *d = buf->dev;
    pre_write(PL, pre, choose, h);
    for (int i = 0; i < n; ++i) {
        const ContractionPlan &p = *items[i].p;
        ((int32_t *)(h + o_fix))[i] = p.form == MGB_FORM_OZAKI ? p.slices : 3;
        ((const int32_t **)(h + o_sp))[i] =
            p.adaptive ? &stat_area(p, items[i].ws).st->sel : (const int32_t *)(d + o_fix) + i;
    }
    size_t vi = 0;
    std::vector<int64_t> vtiles;
    for (auto &kv : gem) {
        std::memcpy(h + o_gj[vi], kv.second.data(), kv.second.size() * sizeof(OzJob));
        int64_t *st = (int64_t *)(h + o_gs[vi]);
        st[0] = 0;
        for (size_t j = 0; j < kv.second.size(); ++j)
            st[j + 1] = st[j] + (int64_t)kv.second[j].tiles_n * kv.second[j].tiles_m * kv.second[j].L;
        vtiles.push_back(st[kv.second.size()]);
        ++vi;
    }
    MGB_CUDA_CHECK(cudaMemcpyAsync(d, h, off, cudaMemcpyHostToDevice, s));
    MGB_CUDA_CHECK(cudaEventRecord(buf->staged, s));
    // ---- pre-pass phases
    if (int st = pre_launch(PL, pre.size(), choose.size(), d, s)) return st;
    // every item's slice count (its fixed count, or the device's choice; 0 = plain)
    if (sel_dev_out) {
        k_gather_sel<<<(n + 255) / 256, 256, 0, s>>>((const int32_t *const *)(d + o_sp), sel_dev_out, n);
        MGB_CUDA_CHECK(cudaGetLastError());
    }
    if (after_prepass)
        if (int st = after_prepass()) return st;
    // ---- one persistent launch per kernel variant
    vi = 0;
    for (auto &kv : gem) {
        const int S = std::get<0>(kv.first);
        const bool exact = std::get<1>(kv.first) != 0, cx = std::get<2>(kv.first) != 0;
        if (vtiles[vi] > 0)
            if (int st = launch_grouped(S, exact, cx, (const OzJob *)(d + o_gj[vi]), (const int64_t *)(d + o_gs[vi]),
                                        (int)kv.second.size(), vtiles[vi], s))
                return st;
        if (after_variant)
            if (int st = after_variant(S, exact, cx)) return st;
        ++vi;
    }
    return MGB_OK;
}
}  // namespace mgb
