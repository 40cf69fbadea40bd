// PLAIN form: native-precision contraction C[l][m][n] = sum_k A[l][m][k] B[l][k][n]
// (src/Operations/binary_einsum.jl:76-96 computes the same with permute ->
// BLAS gemm -> permute). Here the operands are read in place through their
// folded mode groups (a direct GETT), so no permutation pass is needed.
//
//  * Float64 / ComplexF64: FP64 tensor cores, mma.sync m16n8k16 .f64 (DMMA).
//    Complex uses the 4-real-product form (4M), as zgemm does.
//  * Float32 / ComplexF32: FP32 FFMA on CUDA cores.
// The FP64 pipe of GB300 is the roofline of this form.
#include <algorithm>
#include <type_traits>

#include "mgb_internal.h"

namespace mgb {

struct GemmArgs {
    ModeGroup gm, gn, gk, gl;  // tensor 0 = A, 1 = B, 2 = C
    const void *const *pa, *const *pb;  // per-batch-entry pointers (grouped execution) or null
    void *const *pc;
    int64_t M, N, K;
    int a_kfast;  // A's unit-stride mode is contracted (else left)
    int b_kfast;  // B's unit-stride mode is contracted (else right)
    const int32_t *sel;  // adaptive choice (nullable): run only when it holds 0
};

template <typename T>
struct Cx;
template <>
struct Cx<double> {
    static constexpr bool complex = false;
    __device__ static double re(double v) { return v; }
    __device__ static double im(double) { return 0.0; }
};
template <>
struct Cx<double2> {
    static constexpr bool complex = true;
    __device__ static double re(double2 v) { return v.x; }
    __device__ static double im(double2 v) { return v.y; }
};
template <>
struct Cx<float> {
    static constexpr bool complex = false;
    __device__ static float re(float v) { return v; }
    __device__ static float im(float) { return 0.f; }
};
template <>
struct Cx<float2> {
    static constexpr bool complex = true;
    __device__ static float re(float2 v) { return v.x; }
    __device__ static float im(float2 v) { return v.y; }
};

__device__ __forceinline__ void dmma16816(double (&c)[4], const double (&a)[8], const double (&b)[4]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
        "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
        : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
        : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
          "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
}

constexpr int BM = 64, BN = 64, BK = 16, PADD = 4;

// Tile loader shared by both kernels: fills sre/sim[k][r] (r = m or n) from an
// operand whose row group is `gr` and contracted group `gk` (tensor t). A
// real operand of a complex contraction (promote_eltype, src/Muscle.jl:47)
// is widened here, with zero imaginary parts (CXR: complex result).
template <typename T, typename R, int NT, bool CXR>
__device__ __forceinline__ void load_tile(const T *__restrict__ base, const int64_t *rowoff,
                                          const int64_t *koff, int64_t rows_left, int64_t k_left,
                                          int kfast, R (*sre)[BM + PADD], R (*sim)[BM + PADD]) {
    for (int idx = threadIdx.x; idx < BM * BK; idx += NT) {
        int r, k;
        if (kfast) {
            k = idx % BK;
            r = idx / BK;
        } else {
            r = idx % BM;
            k = idx / BM;
        }
        R vr = 0, vi = 0;
        if (r < rows_left && k < k_left) {
            T v = __ldg(base + rowoff[r] + koff[k]);
            vr = (R)Cx<T>::re(v);
            vi = (R)Cx<T>::im(v);
        }
        sre[k][r] = vr;
        if (CXR) sim[k][r] = vi;
    }
}

// ---------------------------------------------------------------- DMMA (FP64)
template <typename TA, typename TB, typename T>
__global__ void __launch_bounds__(128) k_plain_dmma(const TA *__restrict__ A, const TB *__restrict__ B,
                                                    T *__restrict__ C, GemmArgs g) {
    constexpr bool CX = Cx<T>::complex;
    if (g.sel && *g.sel != 0) return;
    __shared__ double As_re[BK][BM + PADD], Bs_re[BK][BN + PADD];
    __shared__ double As_im[CX ? BK : 1][BM + PADD], Bs_im[CX ? BK : 1][BN + PADD];
    __shared__ int64_t rowA[BM], colB[BN], kA[BK], kB[BK];

    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    const int64_t l = blockIdx.z;
    const TA *Ab = g.pa ? (const TA *)g.pa[l] : A + group_offset(g.gl, 0, l);
    const TB *Bb = g.pb ? (const TB *)g.pb[l] : B + group_offset(g.gl, 1, l);
    T *Cb = g.pc ? (T *)g.pc[l] : C + group_offset(g.gl, 2, l);
    int tid = threadIdx.x;
    if (tid < BM) rowA[tid] = (m0 + tid < g.M) ? group_offset(g.gm, 0, m0 + tid) : 0;
    else colB[tid - BM] = (n0 + tid - BM < g.N) ? group_offset(g.gn, 1, n0 + tid - BM) : 0;

    int warp = tid / 32, lane = tid % 32;
    int wm = (warp / 2) * 32, wn = (warp % 2) * 32;
    int gq = lane >> 2, tq = lane & 3;
    double acc_re[2][4][4], acc_im[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc_re[i][j][q] = acc_im[i][j][q] = 0.0;

    for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
        __syncthreads();
        if (tid < BK) kA[tid] = (k0 + tid < g.K) ? group_offset(g.gk, 0, k0 + tid) : 0;
        else if (tid < 2 * BK) kB[tid - BK] = (k0 + tid - BK < g.K) ? group_offset(g.gk, 1, k0 + tid - BK) : 0;
        __syncthreads();
        load_tile<TA, double, 128, CX>(Ab, rowA, kA, g.M - m0, g.K - k0, g.a_kfast, As_re, As_im);
        // B rows are n: element (k, n) at colB[n] + kB[k]
        load_tile<TB, double, 128, CX>(Bb, colB, kB, g.N - n0, g.K - k0, g.b_kfast, Bs_re, Bs_im);
        __syncthreads();
        double bre[4][4], bim[4][4];
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                bre[ni][i] = Bs_re[tq + 4 * i][wn + ni * 8 + gq];
                if (CX) bim[ni][i] = Bs_im[tq + 4 * i][wn + ni * 8 + gq];
            }
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
            double are[8], aim[8], ain[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                int r = wm + mi * 16 + gq + 8 * (i % 2), c = tq + 4 * (i / 2);
                are[i] = As_re[c][r];
                if (CX) {
                    aim[i] = As_im[c][r];
                    ain[i] = -aim[i];
                }
            }
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                dmma16816(acc_re[mi][ni], are, bre[ni]);
                if (CX) {
                    dmma16816(acc_re[mi][ni], ain, bim[ni]);
                    dmma16816(acc_im[mi][ni], are, bim[ni]);
                    dmma16816(acc_im[mi][ni], aim, bre[ni]);
                }
            }
        }
    }
    // epilogue
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            int64_t m = m0 + wm + mi * 16 + gq + 8 * h;
            if (m >= g.M) continue;
            int64_t om = group_offset(g.gm, 2, m);
#pragma unroll
            for (int ni = 0; ni < 4; ++ni)
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    int64_t n = n0 + wn + ni * 8 + 2 * tq + e;
                    if (n >= g.N) continue;
                    int64_t off = om + group_offset(g.gn, 2, n);
                    double vr = acc_re[mi][ni][2 * h + e];
                    if constexpr (CX) {
                        Cb[off] = make_double2(vr, acc_im[mi][ni][2 * h + e]);
                    } else {
                        Cb[off] = vr;
                    }
                }
        }
}

// ---------------------------------------------------------------- FFMA (FP32)
template <typename TA, typename TB, typename T>
__global__ void __launch_bounds__(256) k_plain_ffma(const TA *__restrict__ A, const TB *__restrict__ B,
                                                    T *__restrict__ C, GemmArgs g) {
    constexpr bool CX = Cx<T>::complex;
    if (g.sel && *g.sel != 0) return;
    __shared__ float As_re[BK][BM + PADD], Bs_re[BK][BN + PADD];
    __shared__ float As_im[CX ? BK : 1][BM + PADD], Bs_im[CX ? BK : 1][BN + PADD];
    __shared__ int64_t rowA[BM], colB[BN], kA[BK], kB[BK];
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    const int64_t l = blockIdx.z;
    const TA *Ab = g.pa ? (const TA *)g.pa[l] : A + group_offset(g.gl, 0, l);
    const TB *Bb = g.pb ? (const TB *)g.pb[l] : B + group_offset(g.gl, 1, l);
    T *Cb = g.pc ? (T *)g.pc[l] : C + group_offset(g.gl, 2, l);
    int tid = threadIdx.x;
    if (tid < BM) rowA[tid] = (m0 + tid < g.M) ? group_offset(g.gm, 0, m0 + tid) : 0;
    else if (tid < BM + BN) colB[tid - BM] = (n0 + tid - BM < g.N) ? group_offset(g.gn, 1, n0 + tid - BM) : 0;
    int tr = tid / 16, tc = tid % 16;  // 4x4 outputs: rows tr + 16 i, cols tc + 16 j
    float cr[4][4], ci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cr[i][j] = ci[i][j] = 0.f;
    for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
        __syncthreads();
        if (tid < BK) kA[tid] = (k0 + tid < g.K) ? group_offset(g.gk, 0, k0 + tid) : 0;
        else if (tid < 2 * BK) kB[tid - BK] = (k0 + tid - BK < g.K) ? group_offset(g.gk, 1, k0 + tid - BK) : 0;
        __syncthreads();
        load_tile<TA, float, 256, CX>(Ab, rowA, kA, g.M - m0, g.K - k0, g.a_kfast, As_re, As_im);
        load_tile<TB, float, 256, CX>(Bb, colB, kB, g.N - n0, g.K - k0, g.b_kfast, Bs_re, Bs_im);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            float ar[4], ai[4], br[4], bi[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ar[i] = As_re[k][tr + 16 * i];
                br[i] = Bs_re[k][tc + 16 * i];
                if (CX) {
                    ai[i] = As_im[k][tr + 16 * i];
                    bi[i] = Bs_im[k][tc + 16 * i];
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    cr[i][j] = fmaf(ar[i], br[j], cr[i][j]);
                    if (CX) {
                        cr[i][j] = fmaf(-ai[i], bi[j], cr[i][j]);
                        ci[i][j] = fmaf(ar[i], bi[j], ci[i][j]);
                        ci[i][j] = fmaf(ai[i], br[j], ci[i][j]);
                    }
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int64_t m = m0 + tr + 16 * i;
        if (m >= g.M) continue;
        int64_t om = group_offset(g.gm, 2, m);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int64_t n = n0 + tc + 16 * j;
            if (n >= g.N) continue;
            int64_t off = om + group_offset(g.gn, 2, n);
            if constexpr (CX) Cb[off] = make_float2(cr[i][j], ci[i][j]);
            else Cb[off] = cr[i][j];
        }
    }
}

static int unit_stride_in(const ModeGroup &g, int t) {
    return g.n > 0 && (g.str[t][0] == 1 || g.str[t][0] == -1);
}

template <typename T>
constexpr bool is_dbl() {
    return std::is_same<T, double>::value || std::is_same<T, double2>::value;
}
// (TA, TB) -> T is Julia's promote_eltype over {Float32, Float64, ComplexF32, ComplexF64}
template <typename TA, typename TB, typename T>
constexpr bool promotes_to() {
    return (Cx<TA>::complex || Cx<TB>::complex) == Cx<T>::complex && (is_dbl<TA>() || is_dbl<TB>()) == is_dbl<T>();
}

template <typename TA, typename TB, typename T>
static void launch_typed(dim3 grid, const void *A, const void *B, void *C, const GemmArgs &g, cudaStream_t s) {
    if constexpr (promotes_to<TA, TB, T>()) {
        if constexpr (is_dbl<T>())
            k_plain_dmma<TA, TB, T><<<grid, 128, 0, s>>>((const TA *)A, (const TB *)B, (T *)C, g);
        else
            k_plain_ffma<TA, TB, T><<<grid, 256, 0, s>>>((const TA *)A, (const TB *)B, (T *)C, g);
    }
}

// Operand element type `d` as the kernels' load type.
template <typename T>
struct AsType {
    typedef T type;
};

template <typename F>
static bool with_type(int d, F &&f) {
    switch (d) {
    case MGB_F32: f(AsType<float>{}); return true;
    case MGB_F64: f(AsType<double>{}); return true;
    case MGB_C32: f(AsType<float2>{}); return true;
    case MGB_C64: f(AsType<double2>{}); return true;
    }
    return false;
}

int launch_plain_gemm(const ContractionPlan &p, const void *A, const void *B, void *C,
                      cudaStream_t s, const int32_t *sel) {
    GemmArgs g;
    g.gm = p.gm;
    g.gn = p.gn;
    g.gk = p.gk;
    g.gl = p.gl;
    g.M = p.M;
    g.N = p.N;
    g.K = p.K;
    g.pa = p.pa;
    g.pb = p.pb;
    g.pc = p.pc;
    g.sel = sel;
    g.a_kfast = unit_stride_in(p.gk, 0) && !unit_stride_in(p.gm, 0);
    g.b_kfast = unit_stride_in(p.gk, 1) && !unit_stride_in(p.gn, 1);
    int64_t gx = (p.N + BN - 1) / BN, gy = (p.M + BM - 1) / BM;
    if (gy > 65535) return fail(MGB_ERR_UNSUPPORTED, "plain: M too large for the grid");
    dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)p.L);
    // Operands are read in their own element types (a real operand of a
    // complex contraction, or Float32 in a Float64 one, is widened on load).
    bool ok = false;
    auto go = [&](auto tc) {
        typedef typename decltype(tc)::type T;
        with_type(p.a.dtype, [&](auto ta) {
            typedef typename decltype(ta)::type TA;
            with_type(p.b.dtype, [&](auto tb) {
                typedef typename decltype(tb)::type TB;
                launch_typed<TA, TB, T>(grid, A, B, C, g, s);
                ok = promotes_to<TA, TB, T>();
            });
        });
    };
    switch (p.compute_dtype) {
    case MGB_F64: go(AsType<double>{}); break;
    case MGB_C64: go(AsType<double2>{}); break;
    case MGB_F32: go(AsType<float>{}); break;
    case MGB_C32: go(AsType<float2>{}); break;
    }
    if (!ok) return fail(MGB_ERR_ARGUMENT, "plain: bad dtype");
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

}  // namespace mgb
