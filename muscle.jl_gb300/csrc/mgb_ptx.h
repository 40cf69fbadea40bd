// Inline-PTX wrappers shared by the kernels that stage tiles with TMA:
// mbarrier set-up, arrivals and bounded waits, and the tensor-map encoder
// reached through the runtime's driver entry point (no -lcuda).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "muscle_gb300.h"

namespace mgb {

// A bounded wait gives up after this many clock64 cycles (~1 s at 2 GHz).
constexpr long long kWaitTimeoutCycles = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false when the CTA aborted or this wait timed out (about a
// second of clock64 cycles, checked every 256 tries). A timeout raises the
// CTA's abort flag and records MGB_ERR_DEVICE_TIMEOUT in `status`.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                          int32_t *status) {
    if (mbar_try(bar, parity)) return true;
    long long t0 = clock64();
    for (uint32_t n = 1;; ++n) {
        if (mbar_try(bar, parity)) return true;
        if ((n & 255) == 0) {
            if (*abort_flag) return false;
            if (clock64() - t0 > kWaitTimeoutCycles) {
                *abort_flag = 1;
                atomicCAS(status, 0, (int32_t)MGB_ERR_DEVICE_TIMEOUT);
                return false;
            }
        }
    }
}
// Drain wait used after an abort: bounded, never raises the abort flag.
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
    long long t0 = clock64();
    while (!mbar_try(bar, parity))
        if (clock64() - t0 > kWaitTimeoutCycles) return;
}
// 5-D tiled TMA load into shared memory, completing `bytes` on `bar`.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *tm, int c0, int c1, int c2,
                                            int c3, int c4, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}

typedef CUresult (*PFN_encodeTiled_t)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                      const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                      const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                      CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
// cuTensorMapEncodeTiled, or nullptr when the driver lacks it (resolved once).
PFN_encodeTiled_t tensor_map_encoder();

}  // namespace mgb
