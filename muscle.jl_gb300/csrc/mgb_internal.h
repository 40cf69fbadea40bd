// Internal declarations shared by the libmuscle_gb300 translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "muscle_gb300.h"

namespace mgb {

constexpr int kMaxRank = MGB_MAX_RANK;

// Per-thread error message behind mgb_last_error().
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t err, const char *what);

#define MGB_CUDA_CHECK(expr)                                  \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return ::mgb::cuda_fail(_e, #expr); \
    } while (0)

inline int elem_bytes(int dtype) {
    switch (dtype) {
    case MGB_F32: return 4;
    case MGB_F64: return 8;
    case MGB_C32: return 8;
    case MGB_C64: return 16;
    }
    return 0;
}
inline bool is_complex(int dtype) { return dtype == MGB_C32 || dtype == MGB_C64; }
inline bool is_double(int dtype) { return dtype == MGB_F64 || dtype == MGB_C64; }
inline bool valid_dtype(int dtype) { return dtype >= MGB_F32 && dtype <= MGB_C64; }
// Base.promote_eltype over {Float32, Float64, ComplexF32, ComplexF64}.
inline int promote(int a, int b) {
    bool c = is_complex(a) || is_complex(b);
    bool d = is_double(a) || is_double(b);
    return c ? (d ? MGB_C64 : MGB_C32) : (d ? MGB_F64 : MGB_F32);
}

// A folded group of modes and the strides it has in up to three tensors.
// Linear index i in [0, size) decomposes mixed-radix with mode 0 fastest.
struct ModeGroup {
    int32_t n = 0;
    int64_t ext[kMaxRank];
    int64_t str[3][kMaxRank];  // stride in tensor 0/1/2 (elements), 0 when absent
    int64_t size() const {
        int64_t s = 1;
        for (int i = 0; i < n; ++i) s *= ext[i];
        return s;
    }
};

// Device-side decomposition: offset of linear index `idx` (0 <= idx < size())
// in tensor `t`. The slowest mode needs no division, and indices below 2^31
// divide in 32 bits (a 64-bit division is a long software sequence on the GPU).
__host__ __device__ inline int64_t group_offset(const ModeGroup &g, int t, int64_t idx) {
    int64_t off = 0;
    for (int i = 0; i + 1 < g.n; ++i) {
        const int64_t e = g.ext[i];
        int64_t q;
        if ((uint64_t)idx <= 0x7FFFFFFFu && (uint64_t)e <= 0x7FFFFFFFu) q = (int64_t)((uint32_t)idx / (uint32_t)e);
        else q = idx / e;
        off += (idx - q * e) * g.str[t][i];
        idx = q;
    }
    if (g.n > 0) off += idx * g.str[t][g.n - 1];
    return off;
}

// Internal tensor description with owned arrays.
struct Desc {
    int dtype = MGB_F64;
    int rank = 0;
    int32_t modes[kMaxRank];
    int64_t ext[kMaxRank];
    int64_t str[kMaxRank];
};
int read_desc(const mgb_tensor_desc *d, Desc &out, const char *name);
bool has_repeats(const Desc &d);
int find_mode(const Desc &d, int label);  // position of `label` in d, or -1

// One label of a contraction or broadcast with its extent and its stride in
// up to three tensors (0 where the tensor lacks it).
struct ModeRec {
    int label;
    int64_t ext;
    int64_t str[3];
};
ModeGroup fold_group(std::vector<ModeRec> modes, const bool present[3], int primary);

enum class PlanKind { Contraction, Unary };

// Resolved binary contraction: GEMM view C[l][m][n] = sum_k A[l][m][k] B[l][k][n].
struct ContractionPlan {
    Desc a, b, c;
    int compute_dtype = MGB_F64;
    int form = MGB_FORM_PLAIN;
    int slices = 0;
    // Groups: tensor index 0 = A, 1 = B, 2 = C.
    ModeGroup gm, gn, gk, gl;
    int64_t M = 1, N = 1, K = 1, L = 1;
    // Kept for mgb_plan_info's permute flags: always false, since the plain
    // kernels read operands of any element type in place.
    bool convert_a = false, convert_b = false;
    // Ozaki / bf16x3 parameters.
    int oz_w = 7;          // slice width in bits
    int oz_kc = 256;       // k-chunk (embedded elements) between exact readouts
    int oz_R = 0;          // -1 when K is too long for the exact accumulator
    // Adaptive OZAKI (slices = 0 at plan creation): every call measures the
    // operands and picks the smallest slice count in `cand_mask` (bit S)
    // whose estimated relative Frobenius error is within `tol`, or the plain
    // form when none is. `slices` then holds the largest candidate (the
    // workspace is sized for it).
    bool adaptive = false;
    uint32_t cand_mask = 0;
    double tol = 1e-13;
    uint64_t ws_stat = 0;  // statistics and the choice (OzStats, then P and q arrays)
    uint64_t ws_conv = 0;  // mixed real x complex operands widened to complex (adaptive only)
    // Grouped execution: per-batch-entry operand / output pointers (device
    // arrays of L pointers) replace the batch strides when set.
    const void *const *pa = nullptr, *const *pb = nullptr;
    void *const *pc = nullptr;
    int band = 0;          // tensor-core kernel: row tiles per rasterisation band (0: default)
    // The emulated forms may compute C^T = B^T A^T instead: A and B (their
    // descriptors, mode strides, extents and pointer tables) are then stored
    // exchanged, and every entry point passes the caller's B where the plan
    // says A. Set at plan creation when it fills more of the 128-row tiles.
    bool swapped = false;
    uint64_t ws_bytes = 0;
    // workspace layout (byte offsets)
    uint64_t ws_a = 0, ws_b = 0, ws_scale_a = 0, ws_scale_b = 0;
    int64_t kpad = 0;      // padded embedded K of the slice buffers
    int64_t m_e = 0, n_e = 0, k_e = 0;  // embedded GEMM extents
};

struct UnaryPlan {
    Desc x, y;
    ModeGroup go;  // output modes: tensor 0 = X stride, 1 = Y stride
    ModeGroup gr;  // reduced modes: tensor 0 = X stride
    int64_t O = 1, R = 1;
};

}  // namespace mgb

struct mgb_plan_s {
    mgb::PlanKind kind;
    mgb::ContractionPlan cp;
    mgb::UnaryPlan up;
    // optional phase timing (mgb_plan_set_timing)
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    ~mgb_plan_s() {
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
};

namespace mgb {
// Kernel launchers (each returns an mgb_status).
int launch_permute(const Desc &x, const Desc &y, const void *X, void *Y, cudaStream_t s);
int launch_fill_zero(void *p, int64_t count, int dtype, const Desc &d, cudaStream_t s);
// `sel` (nullable): a device word; the launch does nothing unless it holds 0
// (the adaptive choice "plain").
int launch_plain_gemm(const ContractionPlan &p, const void *A, const void *B, void *C,
                      cudaStream_t s, const int32_t *sel = nullptr);
int launch_ozaki(const ContractionPlan &p, const void *A, const void *B, void *C,
                 void *ws, cudaStream_t s, cudaEvent_t mid = nullptr);
int launch_unary(const UnaryPlan &p, const void *X, void *Y, cudaStream_t s);
int selftest_wait_timeout(cudaStream_t s);
// Emulated forms split for groups: the pre-pass of one plan, and one
// persistent GEMM launch for several plans of one kernel variant (same
// slices, form and real/complex) whose slices lie in the given workspaces.
int ozaki_prepass(const ContractionPlan &p, const void *A, const void *B, void *ws, cudaStream_t s);
// The tensor-core part of one plan whose pre-pass has run into `ws` (for an
// adaptive plan: one launch per candidate slice count, of which only the
// chosen one works, and the plain form as the fallback).
int ozaki_gemm(const ContractionPlan &p, const void *A, const void *B, void *C, void *ws, cudaStream_t s);
// Reads the adaptive choice of the last call that ran with `ws` (synchronises s).
int ozaki_adaptive_report(const ContractionPlan &p, const void *ws, cudaStream_t s, mgb_adaptive_report *out);
int ozaki_set_tolerance(ContractionPlan &p, double tol);
// Batched execution of different emulated-form contractions (each with its
// own workspace `ws`, sized by its plan): one launch per pre-pass phase over
// all operands, one chooser launch for the adaptive ones, and one persistent
// tensor-core launch per kernel variant. `sel_dev_out` (device, one int32 per
// item, nullable) receives each item's slice count (0: an adaptive item chose
// the plain form, which the caller must then run). `after_prepass` is called
// on the host once the pre-pass and `sel_dev_out` are queued and before any
// tensor-core launch, `after_variant` after each variant's launch (slice
// count, exact form, complex), e.g. to queue copies or record events.
// Plain-form plans are rejected.
struct OzBatchItem {
    const ContractionPlan *p;
    const void *A, *B;
    void *C;
    void *ws;
};
struct OzBatchBuffers;
OzBatchBuffers *ozaki_batch_buffers_create();
void ozaki_batch_buffers_destroy(OzBatchBuffers *b);
int ozaki_batch_launch(const std::vector<OzBatchItem> &items, OzBatchBuffers *buf, cudaStream_t s,
                       int32_t *sel_dev_out, const std::function<int()> &after_prepass,
                       const std::function<int(int S, bool exact, bool cx)> &after_variant);
// One persistent GEMM launch of kernel variant (S, exact, cx) over plans
// whose slices lie in `ws`: fixed plans of that variant, and adaptive plans
// that hold S among their candidates (their jobs work only when the device
// chose S).
struct OzGrouped;
int ozaki_grouped_create(const std::vector<const ContractionPlan *> &plans, const std::vector<void *> &ws, int S,
                         bool exact, bool cx, OzGrouped **out);
int ozaki_grouped_launch(const OzGrouped *g, cudaStream_t s);
void ozaki_grouped_destroy(OzGrouped *g);
// The plain-form candidate of an adaptive plan after its pre-pass into `ws`
// (works only when the device chose the plain form; nothing for fixed plans).
int ozaki_plain_fallback(const ContractionPlan &p, const void *A, const void *B, void *C, void *ws, cudaStream_t s);
int launch_hadamard(const ModeGroup &g, int ta, int tb, int tc, const void *A, const void *B, void *C,
                    cudaStream_t s);
int32_t *device_status_ptr();  // per-device status word
uint64_t ozaki_workspace(ContractionPlan &p);
void ozaki_setup(ContractionPlan &p);
// Emulated forms: exchanges the roles of A and B (see `swapped`) when the
// tensor-core tiles of C^T = B^T A^T are fewer than those of C = A B.
void ozaki_orient(ContractionPlan &p);
}  // namespace mgb
