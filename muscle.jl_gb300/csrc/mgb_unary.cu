// unary_einsum: Y[out] = sum over the remaining labels of X, where a label
// repeated in X walks the diagonal (src/Operations/unary_einsum.jl:26-46,
// ext/MuscleOMEinsumExt.jl:25-38; cases pinned by
// test/integration/omeinsum.jl:6-100: axis sum, full sum, ii->i, iji->ij,
// ii->, iji->j). The plan folds each distinct label into one mode whose X
// stride is the sum of its positions' strides, so the kernel is a strided
// reduction: y(o) = sum_r x(off_o + off_r). Memory-bound.
#include <algorithm>

#include "mgb_internal.h"

namespace mgb {

template <typename T>
struct Acc;
template <>
struct Acc<float> {
    using V = float;
    __device__ static V zero() { return 0.f; }
    __device__ static V add(V a, V b) { return a + b; }
};
template <>
struct Acc<double> {
    using V = double;
    __device__ static V zero() { return 0.0; }
    __device__ static V add(V a, V b) { return a + b; }
};
template <>
struct Acc<float2> {
    using V = float2;
    __device__ static V zero() { return make_float2(0.f, 0.f); }
    __device__ static V add(V a, V b) { return make_float2(a.x + b.x, a.y + b.y); }
};
template <>
struct Acc<double2> {
    using V = double2;
    __device__ static V zero() { return make_double2(0.0, 0.0); }
    __device__ static V add(V a, V b) { return make_double2(a.x + b.x, a.y + b.y); }
};

template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d);
template <>
__device__ __forceinline__ float shfl_down(float v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
template <>
__device__ __forceinline__ double shfl_down(double v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
template <>
__device__ __forceinline__ float2 shfl_down(float2 v, int d) {
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
template <>
__device__ __forceinline__ double2 shfl_down(double2 v, int d) {
    return make_double2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}

// Kernel arguments, in the parameter space (__grid_constant__): the mode
// groups are indexed where they lie, never copied to local memory.
struct UnaryArgs {
    ModeGroup go;        // outputs: tensor 0 = X stride, 1 = Y stride
    ModeGroup rest;      // reduced modes after the fastest one (X strides)
    int64_t e0, s0;      // fastest reduced mode: extent and X stride
    int64_t O, outer;    // outputs; rest.size()
};

constexpr int UU = 4;  // independent partial sums (loads in flight) per thread

// One thread per output: consecutive threads take consecutive outputs, so
// the loads are coalesced when Y's fastest mode is also X's (a sum over a
// slower label); the fastest reduced mode is walked without division, four
// elements at a time into independent partial sums.
template <typename T>
__global__ void __launch_bounds__(256) k_unary_thread(const T *__restrict__ x, T *__restrict__ y,
                                                      const __grid_constant__ UnaryArgs a) {
    const int64_t e0 = a.e0, s0 = a.s0;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < a.O;
         o += (int64_t)gridDim.x * blockDim.x) {
        const T *xo = x + group_offset(a.go, 0, o);
        T acc[UU];
#pragma unroll
        for (int u = 0; u < UU; ++u) acc[u] = Acc<T>::zero();
        for (int64_t q = 0; q < a.outer; ++q) {
            const T *xq = xo + group_offset(a.rest, 0, q);
            int64_t r = 0;
            for (; r + UU <= e0; r += UU) {
                T v[UU];
#pragma unroll
                for (int u = 0; u < UU; ++u) v[u] = __ldg(xq + (r + u) * s0);
#pragma unroll
                for (int u = 0; u < UU; ++u) acc[u] = Acc<T>::add(acc[u], v[u]);
            }
            for (; r < e0; ++r) acc[0] = Acc<T>::add(acc[0], __ldg(xq + r * s0));
        }
        y[group_offset(a.go, 1, o)] = Acc<T>::add(Acc<T>::add(acc[0], acc[1]), Acc<T>::add(acc[2], acc[3]));
    }
}

// One warp per output (long reductions): lanes take every 32nd element of
// the fastest reduced mode, four at a time into independent partial sums.
template <typename T>
__global__ void __launch_bounds__(256) k_unary_warp(const T *__restrict__ x, T *__restrict__ y,
                                                    const __grid_constant__ UnaryArgs a) {
    const int lane = threadIdx.x % 32;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
    const int64_t nwarps = (int64_t)gridDim.x * blockDim.x / 32;
    const int64_t e0 = a.e0, s0 = a.s0;
    for (int64_t o = warp; o < a.O; o += nwarps) {
        const T *xo = x + group_offset(a.go, 0, o);
        T acc[UU];
#pragma unroll
        for (int u = 0; u < UU; ++u) acc[u] = Acc<T>::zero();
        for (int64_t q = 0; q < a.outer; ++q) {
            const T *xq = xo + group_offset(a.rest, 0, q);
            int64_t r = lane;
            for (; r + 32 * (UU - 1) < e0; r += 32 * UU) {
                T v[UU];
#pragma unroll
                for (int u = 0; u < UU; ++u) v[u] = __ldg(xq + (r + 32 * u) * s0);
#pragma unroll
                for (int u = 0; u < UU; ++u) acc[u] = Acc<T>::add(acc[u], v[u]);
            }
            for (; r < e0; r += 32) acc[0] = Acc<T>::add(acc[0], __ldg(xq + r * s0));
        }
        T s = Acc<T>::add(Acc<T>::add(acc[0], acc[1]), Acc<T>::add(acc[2], acc[3]));
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) s = Acc<T>::add(s, shfl_down(s, d));
        if (lane == 0) y[group_offset(a.go, 1, o)] = s;
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
