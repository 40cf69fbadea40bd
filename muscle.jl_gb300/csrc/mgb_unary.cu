// unary_einsum: Y[out] = sum over the remaining labels of X, where a label
// repeated in X walks the diagonal (src/Operations/unary_einsum.jl:26-46,
// ext/MuscleOMEinsumExt.jl:25-38; cases pinned by
// test/integration/omeinsum.jl:6-100: axis sum, full sum, ii->i, iji->ij,
// ii->, iji->j). The plan folds each distinct label into one mode whose X
// stride is the sum of its positions' strides, so the kernel is a strided
// reduction: y(o) = sum_r x(off_o + off_r). Memory-bound.
#include <algorithm>

#include "mgb_fxsum.h"
#include "mgb_internal.h"

namespace mgb {

constexpr int UU = 4;  // loads in flight per thread

// Accumulators. Float32 / ComplexF32 add in FP32 into UU independent partial
// sums. Float64 / ComplexF64 add into fixed-point sums on the integer pipes
// (mgb_fxsum.h): GB300's FP64 pipe would bound an FP64 sum at about half the
// HBM rate, and the fixed-point sum is also exact within 10 binades of the
// largest term and independent of the order. One such sum per thread and component.
template <typename T>
struct Acc;
template <typename F>
struct AccFp {
    using V = F;
    static constexpr int kParts = UU;
    __device__ static V zero() { return F(0); }
    __device__ static void push(V &a, F x) { a += x; }
    __device__ static void merge(V &a, V b) { a += b; }
    __device__ static V shfl(V a, int d) { return __shfl_down_sync(0xffffffffu, a, d); }
    __device__ static F out(V a) { return a; }
};
template <>
struct Acc<float> : AccFp<float> {};
template <>
struct Acc<float2> {
    using V = float2;
    static constexpr int kParts = UU;
    __device__ static V zero() { return make_float2(0.f, 0.f); }
    __device__ static void push(V &a, float2 x) {
        a.x += x.x;
        a.y += x.y;
    }
    __device__ static void merge(V &a, V b) { push(a, b); }
    __device__ static V shfl(V a, int d) {
        return make_float2(__shfl_down_sync(0xffffffffu, a.x, d), __shfl_down_sync(0xffffffffu, a.y, d));
    }
    __device__ static float2 out(V a) { return a; }
};
__device__ __forceinline__ FxSum fx_shfl(const FxSum &a, int d) {
    FxSum r;
    r.lo = __shfl_down_sync(0xffffffffu, (unsigned long long)a.lo, d);
    r.hi = __shfl_down_sync(0xffffffffu, (long long)a.hi, d);
    r.e = __shfl_down_sync(0xffffffffu, a.e, d);
    r.flags = __shfl_down_sync(0xffffffffu, a.flags, d);
    return r;
}
template <>
struct Acc<double> {
    using V = FxSum;
    static constexpr int kParts = 1;
    __device__ static V zero() { return fx_zero(); }
    __device__ static void push(V &a, double x) { fx_push(a, x); }
    __device__ static void merge(V &a, const V &b) { fx_merge(a, b); }
    __device__ static V shfl(const V &a, int d) { return fx_shfl(a, d); }
    __device__ static double out(const V &a) { return fx_value(a); }
};
struct FxSum2 {
    FxSum re, im;
};
template <>
struct Acc<double2> {
    using V = FxSum2;
    static constexpr int kParts = 1;
    __device__ static V zero() { return FxSum2{fx_zero(), fx_zero()}; }
    __device__ static void push(V &a, double2 x) {
        fx_push(a.re, x.x);
        fx_push(a.im, x.y);
    }
    __device__ static void merge(V &a, const V &b) {
        fx_merge(a.re, b.re);
        fx_merge(a.im, b.im);
    }
    __device__ static V shfl(const V &a, int d) { return FxSum2{fx_shfl(a.re, d), fx_shfl(a.im, d)}; }
    __device__ static double2 out(const V &a) { return make_double2(fx_value(a.re), fx_value(a.im)); }
};

// Kernel arguments, in the parameter space (__grid_constant__): the mode
// groups are indexed where they lie, never copied to local memory.
struct UnaryArgs {
    ModeGroup go;        // outputs: tensor 0 = X stride, 1 = Y stride
    ModeGroup rest;      // reduced modes after the fastest one (X strides)
    int64_t e0, s0;      // fastest reduced mode: extent and X stride
    int64_t O, outer;    // outputs; rest.size()
};

// One thread per output: consecutive threads take consecutive outputs, so
// the loads are coalesced when Y's fastest mode is also X's (a sum over a
// slower label); the fastest reduced mode is walked without division, four
// loads in flight.
template <typename T>
__global__ void __launch_bounds__(256) k_unary_thread(const T *__restrict__ x, T *__restrict__ y,
                                                      const __grid_constant__ UnaryArgs a) {
    using A = Acc<T>;
    const int64_t e0 = a.e0, s0 = a.s0;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < a.O;
         o += (int64_t)gridDim.x * blockDim.x) {
        const T *xo = x + group_offset(a.go, 0, o);
        typename A::V acc[A::kParts];
#pragma unroll
        for (int u = 0; u < A::kParts; ++u) acc[u] = A::zero();
        for (int64_t q = 0; q < a.outer; ++q) {
            const T *xq = xo + group_offset(a.rest, 0, q);
            int64_t r = 0;
            for (; r + UU <= e0; r += UU) {
                T v[UU];
#pragma unroll
                for (int u = 0; u < UU; ++u) v[u] = __ldg(xq + (r + u) * s0);
#pragma unroll
                for (int u = 0; u < UU; ++u) A::push(acc[u % A::kParts], v[u]);
            }
            for (; r < e0; ++r) A::push(acc[0], __ldg(xq + r * s0));
        }
#pragma unroll
        for (int u = 1; u < A::kParts; ++u) A::merge(acc[0], acc[u]);
        y[group_offset(a.go, 1, o)] = A::out(acc[0]);
    }
}

// One warp per output (long reductions): lanes take every 32nd element of
// the fastest reduced mode, four loads in flight; the lanes' sums are merged
// by shuffles.
template <typename T>
__global__ void __launch_bounds__(256) k_unary_warp(const T *__restrict__ x, T *__restrict__ y,
                                                    const __grid_constant__ UnaryArgs a) {
    using A = Acc<T>;
    const int lane = threadIdx.x % 32;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
    const int64_t e0 = a.e0, s0 = a.s0;
    for (int64_t o = warp; o < a.O; o += nwarps) {
        const T *xo = x + group_offset(a.go, 0, o);
        typename A::V acc[A::kParts];
#pragma unroll
        for (int u = 0; u < A::kParts; ++u) acc[u] = A::zero();
        for (int64_t q = 0; q < a.outer; ++q) {
            const T *xq = xo + group_offset(a.rest, 0, q);
            int64_t r = lane;
            for (; r + 32 * (UU - 1) < e0; r += 32 * UU) {
                T v[UU];
#pragma unroll
                for (int u = 0; u < UU; ++u) v[u] = __ldg(xq + (r + 32 * u) * s0);
#pragma unroll
                for (int u = 0; u < UU; ++u) A::push(acc[u % A::kParts], v[u]);
            }
            for (; r < e0; r += 32) A::push(acc[0], __ldg(xq + r * s0));
        }
#pragma unroll
        for (int u = 1; u < A::kParts; ++u) A::merge(acc[0], acc[u]);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) A::merge(acc[0], A::shfl(acc[0], d));
        if (lane == 0) y[group_offset(a.go, 1, o)] = A::out(acc[0]);
    }
}

template <typename T>
static int run_unary(const UnaryPlan &p, const T *x, T *y, cudaStream_t s) {
    UnaryArgs a;
    a.go = p.go;
    ModeGroup gr = p.gr;
    if (a.go.n == 0) {
        a.go.n = 1;
        a.go.ext[0] = 1;
        a.go.str[0][0] = a.go.str[1][0] = a.go.str[2][0] = 0;
    }
    if (gr.n == 0) {
        gr.n = 1;
        gr.ext[0] = 1;
        gr.str[0][0] = gr.str[1][0] = gr.str[2][0] = 0;
    }
    a.e0 = gr.ext[0];
    a.s0 = gr.str[0][0];
    a.rest.n = gr.n - 1;
    for (int i = 0; i + 1 < gr.n; ++i) {
        a.rest.ext[i] = gr.ext[i + 1];
        for (int t = 0; t < 3; ++t) a.rest.str[t][i] = gr.str[t][i + 1];
    }
    a.O = p.O;
    a.outer = a.e0 > 0 ? p.R / a.e0 : 0;
    // a warp per output when the reduction runs along X's contiguous mode (or
    // no mode of the output is contiguous in X and the reduction is long);
    // otherwise a thread per output, coalesced over the outputs
    const bool red_contig = std::llabs(gr.str[0][0]) == 1 && gr.ext[0] > 1;
    const bool out_contig = std::llabs(a.go.str[0][0]) == 1 && a.go.ext[0] > 1;
    if (p.R >= 64 && (red_contig || !out_contig)) {
        int64_t blocks = std::min<int64_t>((p.O * 32 + 255) / 256, 152 * 16);
        k_unary_warp<T><<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(x, y, a);
    } else {
        int64_t blocks = std::min<int64_t>((p.O + 255) / 256, 152 * 16);
        k_unary_thread<T><<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, s>>>(x, y, a);
    }
    MGB_CUDA_CHECK(cudaGetLastError());
    return MGB_OK;
}

int launch_unary(const UnaryPlan &p, const void *X, void *Y, cudaStream_t s) {
    switch (p.x.dtype) {
    case MGB_F32: return run_unary<float>(p, (const float *)X, (float *)Y, s);
    case MGB_F64: return run_unary<double>(p, (const double *)X, (double *)Y, s);
    case MGB_C32: return run_unary<float2>(p, (const float2 *)X, (float2 *)Y, s);
    case MGB_C64: return run_unary<double2>(p, (const double2 *)X, (double2 *)Y, s);
    }
    return fail(MGB_ERR_ARGUMENT, "unary: bad dtype");
}

}  // namespace mgb
