// mgb_contract_noalloc: the contraction entry point for callers that cannot
// allocate device memory themselves.
//
// Who needs it: callers that own every byte of device memory through their own
// allocator and must not see the library grow its footprint (a serving loop
// that admits requests against a fixed HBM byte budget, or a host runtime whose
// pooled allocator must not be bypassed), and callers on paths where a
// cudaMalloc and the device synchronisation it may imply are not acceptable.
// Such callers cannot hand mgb_contract a workspace, so this entry point uses a
// scratch array of fixed size that the library itself holds in device memory.
//
// Limits and behaviour:
//  * the scratch is MGB_NOALLOC_SCRATCH_BYTES bytes; a plan whose workspace
//    (mgb_plan_workspace_size) is larger is rejected with MGB_ERR_WORKSPACE;
//  * every GPU that loads the library holds the array until the process exits;
//  * all calls share the array, so calls whose kernels overlap on the GPU
//    (different streams, or different host threads) race on it; serialise them;
//  * the array keeps the previous call's contents; the kernels rewrite every
//    slice they read and clear the exponent tables they accumulate into;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <atomic>

#include "mgb_internal.h"

namespace {

// The scratch itself: device memory of every GPU that loads the library.
static __device__ __align__(256) unsigned char mgb_noalloc_scratch[MGB_NOALLOC_SCRATCH_BYTES];

// Device address of the array per device (host code cannot use the symbol as
// a pointer: on the host it only names a stand-in object).
// Lock-free per-device cache (the lookup is idempotent).
int scratch_address(void **out) {
    static std::atomic<void *> addr[128];
    int dev = 0;
    MGB_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return mgb::fail(MGB_ERR_CUDA, "device ordinal out of range");
    void *p = addr[dev].load(std::memory_order_acquire);
    if (!p) {
        cudaError_t e = cudaGetSymbolAddress(&p, mgb_noalloc_scratch);
        if (e != cudaSuccess) return mgb::cuda_fail(e, "cudaGetSymbolAddress(mgb_noalloc_scratch)");
        addr[dev].store(p, std::memory_order_release);
    }
    *out = p;
    return MGB_OK;
}

}  // namespace

extern "C" int mgb_contract_noalloc(mgb_plan plan, const void *A, const void *B, void *C, void *stream) {
    if (!plan || plan->kind != mgb::PlanKind::Contraction)
        return mgb::fail(MGB_ERR_ARGUMENT, "not a contraction plan");
    const uint64_t need = plan->cp.ws_bytes;
    if (need > (uint64_t)MGB_NOALLOC_SCRATCH_BYTES)
        return mgb::fail(MGB_ERR_WORKSPACE,
                         "contraction needs " + std::to_string(need) +
                             " bytes of scratch; mgb_contract_noalloc holds at most " +
                             std::to_string((uint64_t)MGB_NOALLOC_SCRATCH_BYTES) +
                             " bytes (use mgb_contract with a caller workspace)");
    void *scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st) return st;
    return mgb_contract(plan, A, B, C, scratch, (uint64_t)MGB_NOALLOC_SCRATCH_BYTES, stream);
}
