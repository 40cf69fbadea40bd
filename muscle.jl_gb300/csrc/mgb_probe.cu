// Roofline probes: the measured rates of the FP64 pipes that bound the plain
// form (DMMA) and the complex double-precision memory kernels (DFMA, DADD).
// GB300 carries far less FP64 throughput than its predecessors, and no
// datasheet figure is trusted here: the benchmarks divide by these rates.
// Each probe runs independent dependency chains in every warp of a grid of
// `blocks` x `threads`, long enough that launch overhead is negligible, and
// writes one value per thread (never a real output) so that nothing is
// optimised away.
#include <algorithm>

#include "mgb_internal.h"

namespace mgb {

__device__ __forceinline__ void probe_dmma(double (&c)[4], const double (&a)[8], const double (&b)[4]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
        "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
        : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
        : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
          "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
}

// 4 independent m16n8k16 accumulators per warp: 4 x 4096 flops per iteration
__global__ void k_probe_dmma(double *out, int64_t iters) {
    double a[8], b[4], c[4][4];
    const double t = 1.0 + threadIdx.x * 1e-9;
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = t * (i + 1) * 1e-3;
#pragma unroll
    for (int i = 0; i < 4; ++i) b[i] = t * (i + 2) * 1e-3;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) c[j][i] = 0.0;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < 4; ++j) probe_dmma(c[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) s += c[j][i];
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

// 8 independent fma (or add) chains per thread: 8 instructions per iteration
template <bool FMA>
__global__ void k_probe_fp64(double *out, int64_t iters) {
    double x[8];
    const double m = 1.0 - 1e-12, d = 1e-12 * (1 + threadIdx.x % 7);
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = 1.0 + i * 1e-3 + threadIdx.x * 1e-9;
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = FMA ? fma(x[i], m, d) : x[i] + d;
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace mgb

using namespace mgb;

extern "C" int mgb_probe_fp64(int32_t op, int64_t iters, int32_t blocks, int32_t threads, void *scratch,
                              uint64_t scratch_bytes, void *stream, double *tflops) {
    if (!tflops || op < 0 || op > 2 || iters <= 0 || blocks <= 0 || threads <= 0 || threads > 1024 || threads % 32)
        return fail(MGB_ERR_ARGUMENT, "probe: bad arguments");
    if (!scratch || scratch_bytes < (uint64_t)blocks * threads * sizeof(double))
        return fail(MGB_ERR_WORKSPACE, "probe: scratch holds one double per thread");
    cudaStream_t s = (cudaStream_t)stream;
    double *out = (double *)scratch;
    cudaEvent_t e0, e1;
    MGB_CUDA_CHECK(cudaEventCreate(&e0));
    MGB_CUDA_CHECK(cudaEventCreate(&e1));
    auto launch = [&](int64_t n) {
        if (op == 0) k_probe_dmma<<<blocks, threads, 0, s>>>(out, n);
        else if (op == 1) k_probe_fp64<true><<<blocks, threads, 0, s>>>(out, n);
        else k_probe_fp64<false><<<blocks, threads, 0, s>>>(out, n);
    };
    launch(std::max<int64_t>(iters / 16, 1));  // warm-up
    cudaEventRecord(e0, s);
    launch(iters);
    cudaEventRecord(e1, s);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return cuda_fail(err, "probe");
    const double warps = (double)blocks * threads / 32.0;
    double flops;
    if (op == 0) flops = warps * iters * 4.0 * 4096.0;                        // 4 m16n8k16 per warp-iteration
    else flops = (double)blocks * threads * iters * 8.0 * (op == 1 ? 2.0 : 1.0);  // 8 fma (2 flops) or add
    *tflops = flops / (ms * 1e-3) / 1e12;
    return MGB_OK;
}
