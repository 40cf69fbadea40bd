/*
 * muscle_gb300.h — C ABI of libmuscle_gb300.so, a GB300 (sm_103a) backend for
 * Muscle.jl's tensor contractions.
 *
 * The library replaces the device branch of Muscle.jl's operation front-ends:
 *   binary_einsum(::Backend, inds_c, a, b)  src/Operations/binary_einsum.jl:50
 *   binary_einsum!(::Backend, c, a, b)      src/Operations/binary_einsum.jl:68
 *   unary_einsum(::Backend, inds_y, x)      src/Operations/unary_einsum.jl:35
 *   unary_einsum!(::Backend, y, x)          src/Operations/unary_einsum.jl:44
 * whose CUDA implementation is cuTENSOR.contract! in ext/MuscleCUDAExt.jl:10-41
 * (label -> integer mode mapping at :24-27, alpha = 1, beta = 0 at :29-38).
 *
 * Conventions
 *  - A tensor is described by its element type, rank, integer mode labels,
 *    extents and strides in ELEMENTS (Julia's `strides`, column-major when the
 *    array is dense). strides == NULL means dense column-major.
 *  - Device buffers are owned by the caller; the library never frees them.
 *  - Every entry returns an mgb_status; MGB_OK == 0. A per-thread message is
 *    available from mgb_last_error().
 *  - Streams are passed as `void*` (a cudaStream_t; NULL = legacy default).
 *  - Plans are immutable after creation and may be executed concurrently on
 *    different streams with different workspaces.
 */
#ifndef MUSCLE_GB300_H
#define MUSCLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGB_MAX_RANK 16

typedef enum mgb_status {
    MGB_OK = 0,
    MGB_ERR_ARGUMENT = 1,           /* Julia ArgumentError (binary_einsum.jl:54,82-83) */
    MGB_ERR_DIMENSION_MISMATCH = 2, /* Julia DimensionMismatch (Tensor.jl:23)          */
    MGB_ERR_UNSUPPORTED = 3,        /* combination not implemented by the chosen form  */
    MGB_ERR_WORKSPACE = 4,          /* workspace missing or too small                  */
    MGB_ERR_CUDA = 5,               /* CUDA runtime error (message has details)        */
    MGB_ERR_DEVICE_TIMEOUT = 6,     /* a bounded device-side wait gave up              */
    MGB_ERR_OUT_OF_MEMORY = 7,      /* byte budget exceeded (serving admission)        */
    MGB_ERR_NOT_FINITE = 8          /* non-finite input met by an emulated form        */
} mgb_status;

typedef enum mgb_dtype {
    MGB_F32 = 0, /* Float32     */
    MGB_F64 = 1, /* Float64     */
    MGB_C32 = 2, /* ComplexF32  */
    MGB_C64 = 3  /* ComplexF64  */
} mgb_dtype;

typedef enum mgb_form {
    MGB_FORM_AUTO = 0,   /* OZAKI for F64/C64 results, BF16X3 for F32/C32        */
    MGB_FORM_PLAIN = 1,  /* native arithmetic: FP64 DMMA / FP32 FFMA              */
    MGB_FORM_OZAKI = 2,  /* FP64/C64 as exact bf16 integer slices on tcgen05      */
    MGB_FORM_BF16X3 = 3  /* FP32/C32 as 3-piece bf16 split products on tcgen05    */
} mgb_form;

typedef struct mgb_tensor_desc {
    int32_t dtype;            /* mgb_dtype                                    */
    int32_t rank;             /* 0 .. MGB_MAX_RANK                            */
    const int32_t *modes;     /* rank integer labels                          */
    const int64_t *extents;   /* rank extents (>= 0)                          */
    const int64_t *strides;   /* rank strides in elements, or NULL (dense)    */
} mgb_tensor_desc;

typedef struct mgb_plan_s *mgb_plan;

/* Summary of a plan, for callers that report work or pick workspaces. */
typedef struct mgb_plan_info {
    int64_t m, n, k, batch;   /* folded GEMM view: left, right, contracted, hyper */
    int32_t form;             /* resolved mgb_form                               */
    int32_t slices;           /* Ozaki slice count (0: not emulated, or adaptive) */
    int32_t compute_dtype;    /* promoted element type of the result             */
    int32_t permute_a, permute_b, permute_c; /* 1 when PLAIN stages a permute     */
    double flops;             /* algorithmic: 8MNK complex, 2MNK real (x batch)  */
    uint64_t workspace_bytes; /* bytes mgb_contract needs                        */
} mgb_plan_info;

/* ---- binary contraction: C[modes_c] = sum A[modes_a] * B[modes_b] ---------
 * Mode classes follow cuTENSOR semantics used by ext/MuscleCUDAExt.jl:36-38:
 * a mode in A and B but not C is contracted; a mode in A, B and C is a batch
 * (hyper) mode; a mode in exactly one operand and C is free. Any other pattern
 * is MGB_ERR_ARGUMENT. The result element type is promote_eltype(A, B)
 * (ext/MuscleCUDAExt.jl:16) and C must have it. alpha = 1, beta = 0.
 * slices: Ozaki slice count 3..8, or 0 = adaptive (AUTO and OZAKI forms of
 * a Float64 / ComplexF64 result): every mgb_contract then measures the
 * operands on the device (per-row and per-column exponents, and the norms
 * that bound the digit truncation and the dropped digit pairs) and runs the
 * smallest slice count whose estimated relative Frobenius error is within
 * the plan's tolerance (1e-13 unless mgb_plan_set_tolerance changed it), or
 * the plain FP64 form when none is, e.g. for operands with Inf or NaN. The
 * choice happens on the device: the call stays asynchronous and can be
 * captured in a CUDA graph, each replay choosing again for its data. The
 * workspace is sized for the largest candidate. Ignored by other forms.   */
int mgb_contraction_plan(mgb_plan *plan, const mgb_tensor_desc *a,
                         const mgb_tensor_desc *b, const mgb_tensor_desc *c,
                         int32_t form, int32_t slices);
int mgb_contract(mgb_plan plan, const void *A, const void *B, void *C,
                 void *workspace, uint64_t workspace_bytes, void *stream);

/* ---- unary contraction: Y[modes_y] = sum over the other modes of X --------
 * Repeated labels in X select a diagonal (test/integration/omeinsum.jl:6-100,
 * ext/MuscleOMEinsumExt.jl:25-38). modes_y must be distinct and a subset of
 * modes_x (ext/MuscleOMEinsumExt.jl:32). X and Y share the element type.
 * Float64 / ComplexF64 sums are fixed-point integers rounded once: exact
 * while the terms lie within 10 binades of the largest one (otherwise within
 * 2^-62 of the largest term per term), independent of the summation order,
 * Inf / NaN as in an FP64 sum. Float32 / ComplexF32 add in FP32.           */
int mgb_unary_plan(mgb_plan *plan, const mgb_tensor_desc *x,
                   const mgb_tensor_desc *y);
int mgb_unary(mgb_plan plan, const void *X, void *Y, void *workspace,
              uint64_t workspace_bytes, void *stream);

/* ---- permutation: Y[modes_y] = X[modes_x], modes_y a permutation of modes_x
 * (Base.permutedims via src/Tensor.jl:316-319). Element types may differ only
 * by real -> complex promotion of the same precision or F32 -> F64.        */
int mgb_permute(const mgb_tensor_desc *x, const mgb_tensor_desc *y,
                const void *X, void *Y, void *stream);

/* ---- Hadamard (broadcast element-wise) product: C = A .* B -----------------
 * Replaces hadamard / hadamard! of BackendBase (src/Operations/hadamard.jl:
 * 34-77) on device arrays. modes_b must be distinct and a subset of modes_a
 * (hadamard.jl:10,24), B is broadcast along A's other labels, and C carries
 * A's labels in A's order (hadamard.jl:23). The product is formed in the
 * promoted type of A and B and stored in C's type; a complex product into a
 * real C is rejected. C may alias A (hadamard!(a, a, b)) when the two have
 * the same layout and element type; other overlaps are not allowed.     */
int mgb_hadamard(const mgb_tensor_desc *a, const mgb_tensor_desc *b,
                 const mgb_tensor_desc *c, const void *A, const void *B,
                 void *C, void *stream);

int mgb_plan_info_get(mgb_plan plan, mgb_plan_info *info);
/* Phase timing for benchmarks. When enabled, mgb_contract records CUDA events
 * on its launch stream before its pre-pass kernels (scales, slices or
 * operand conversion), before its main contraction kernel and after it;
 * mgb_plan_timing synchronises on the last call's events and returns the two
 * elapsed times in milliseconds. The events belong to the plan: while timing
 * is enabled, execute the plan from one thread and one stream at a time. */
int mgb_plan_set_timing(mgb_plan plan, int32_t enable);
int mgb_plan_timing(mgb_plan plan, float *prepass_ms, float *main_ms);
/* Rasterisation band of the emulated forms' tensor-core kernel: the number
 * of row tiles (1..64) that consecutive tiles walk across all column tiles;
 * 0 = the library's default. Changes the schedule only, never the result.
 * No counterpart in the reference. */
int mgb_plan_set_band(mgb_plan plan, int32_t band);
/* *swapped = 1 when an emulated-form plan computes C^T = B^T A^T (A's and
 * B's roles exchanged inside the library, because A has fewer rows than a
 * tensor-core tile and B many columns), else 0. Callers pass A and B as
 * always; the result is the same contraction. Diagnostic only. No
 * counterpart in the reference. */
int mgb_plan_operands_swapped(mgb_plan plan, int32_t *swapped);
/* Target relative Frobenius error (> 0) of an adaptive plan's slice choice;
 * the default 1e-13 is the tolerance Muscle.jl's Float64 results are held
 * to. Set it before executing the plan, not while executions are in flight.
 * MGB_ERR_ARGUMENT for plans that are not adaptive. No counterpart in the
 * reference. */
int mgb_plan_set_tolerance(mgb_plan plan, double tolerance);
/* The choice of the last mgb_contract of an adaptive plan that ran with
 * `workspace`, read from that workspace after synchronising `stream`.
 * estimate[S] is the estimated relative Frobenius error with S slices for
 * every candidate S (0 elsewhere); slices is the chosen count, 0 when the
 * plain form ran. No counterpart in the reference.                       */
typedef struct mgb_adaptive_report {
    int32_t slices;        /* chosen slice count; 0: the plain FP64 form ran     */
    int32_t nonfinite;     /* 1 when an operand holds Inf or NaN                  */
    double estimate[9];    /* estimated relative error per candidate slice count */
    double tolerance;      /* the plan's target                                   */
} mgb_adaptive_report;
int mgb_plan_adaptive_report(mgb_plan plan, const void *workspace, void *stream,
                             mgb_adaptive_report *report);
int mgb_plan_workspace_size(mgb_plan plan, uint64_t *bytes);
int mgb_plan_destroy(mgb_plan plan);

/* ---- grouped (batched) contractions ---------------------------------------
 * Many independent contractions on one stream. Members that share a plan
 * handle (same shapes, strides, element types and form) run as one batched
 * launch per kernel, the batch index selecting the member's operand and
 * output pointers from a device array; other members run one by one. The
 * group copies the pointer arrays at creation into device memory;
 * mgb_group_update replaces them (a CUDA-graph replay of mgb_group_execute
 * then reads the new pointers) after waiting for the executions and graph
 * replays of the group already launched: every execution records an event
 * on its stream, captured as an external event node in a graph. Operand
 * pointers are device pointers.
 * Device state that a captured graph launches with (pointer arrays, job
 * tables) stays valid until mgb_group_destroy.
 * The ensemble of a PEPS sweep is the motivating case
 * (ext/MuscleDaggerExt/binary_einsum.jl:64-119 runs such independent pairs
 * as separate tasks).                                                      */
typedef struct mgb_group_s *mgb_group;
int mgb_group_create(mgb_group *group, const mgb_plan *plans, int32_t count,
                     const void *const *A, const void *const *B,
                     void *const *C);
int mgb_group_update(mgb_group group, const void *const *A,
                     const void *const *B, void *const *C);
int mgb_group_workspace_size(mgb_group group, uint64_t *bytes);
/* Runs every member on `stream`: the pre-passes of the emulated buckets and
 * the plain buckets, then ONE persistent tensor-core launch per kernel
 * variant over all emulated buckets (each CTA walks tiles of every bucket;
 * an adaptive bucket has a job in the launch of each candidate slice count,
 * which works only for the count its device choice names), then the
 * plain-form fallback of adaptive buckets and members that run alone. The
 * first execution with a given workspace (and the first after
 * mgb_group_set_tiles) uploads the persistent launches' job tables with a
 * synchronous copy; capture the group in a CUDA graph after such a warm-up
 * execution.                                                               */
int mgb_group_execute(mgb_group group, void *workspace,
                      uint64_t workspace_bytes, void *stream);
/* mgb_group_execute in two steps, so that the first can run on several
 * streams: mgb_group_prepare_part runs the pre-passes of the emulated
 * buckets and the plain buckets of part `part` of `nparts` (dealt as in
 * mgb_group_execute_part); once every part has finished, mgb_group_finish
 * runs the persistent tensor-core launches and the members that run alone.
 * No counterpart in the reference.                                        */
int mgb_group_prepare_part(mgb_group group, int32_t part, int32_t nparts,
                           void *workspace, uint64_t workspace_bytes,
                           void *stream);
int mgb_group_finish(mgb_group group, void *workspace,
                     uint64_t workspace_bytes, void *stream);
/* The members of part `part` of `nparts` (0 <= part < nparts). The work units
 * (batched buckets and single members) are dealt, largest first, to the part
 * with the least work so far. Parts touch disjoint outputs and workspace
 * slices, so they may run at the same time on different streams, e.g. as
 * parallel branches of one CUDA graph. No counterpart in the reference.   */
int mgb_group_execute_part(mgb_group group, int32_t part, int32_t nparts,
                           void *workspace, uint64_t workspace_bytes,
                           void *stream);
/* Tile schedule of the batched tensor-core launches: per member, an index
 * 0..5 into the rasterisation bands {1, 2, 3, 4, 8, 16} (row tiles walked
 * together across all column tiles); a bucket takes its first member's
 * value; any other index = the library's default band (3). Written by the
 * host-side autotuner.                                                    */
int mgb_group_set_tiles(mgb_group group, const int32_t *tile_per_plan);
int mgb_group_destroy(mgb_group group);

/* ---- serving loop -----------------------------------------------------------
 * Contractions submitted as they arrive are admitted against a device-memory
 * byte budget and dispatched with continuous batching onto `nstreams`
 * streams by a scheduler thread of the library: while earlier batches run,
 * later arrivals are admitted as budget frees up and launched on the other
 * streams, so their work overlaps on the GPU. A request's admitted bytes are
 * the caller-declared resident bytes (operands and output, which stay in
 * device memory owned by the caller) plus its workspace, which the server
 * allocates from its own stream-ordered pool. A request larger than the
 * whole budget finishes at once with MGB_ERR_OUT_OF_MEMORY. `dep_stream`
 * (may be NULL) is a caller stream whose work so far the request waits for
 * (e.g. the kernels that produced its operands). Plans and buffers must stay
 * alive until mgb_server_wait has returned for the ticket. This is the
 * request loop of the serving form; the reference has no counterpart.     */
typedef struct mgb_server_s *mgb_server;
typedef struct mgb_server_stats {
    uint64_t submitted, completed, rejected, batches, pending, used_bytes;
    double p50_ms, p99_ms, max_ms;  /* latency: submission -> completion seen */
    double elapsed_s;               /* since creation or the last reset         */
} mgb_server_stats;
int mgb_server_create(mgb_server *server, uint64_t budget_bytes, int32_t nstreams,
                      int32_t max_batch);
int mgb_server_submit(mgb_server server, mgb_plan plan, const void *A,
                      const void *B, void *C, uint64_t resident_bytes,
                      void *dep_stream, int64_t *ticket);
/* Blocks until the ticket's request finished (timeout_s < 0: no timeout);
 * *status is its mgb_status. Each ticket is waited for once.              */
int mgb_server_wait(mgb_server server, int64_t ticket, double timeout_s,
                    int32_t *status);
int mgb_server_get_stats(mgb_server server, mgb_server_stats *stats);
int mgb_server_reset_stats(mgb_server server);
/* Waits for queued and running requests, then frees streams and the pool.  */
int mgb_server_destroy(mgb_server server);

/* ---- contraction without a caller workspace --------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory (a fixed byte budget owned by their own allocator, or a path where a
 * cudaMalloc and its implicit synchronisation are not acceptable): runs the
 * plan exactly like mgb_contract, with the workspace taken from a scratch
 * array of MGB_NOALLOC_SCRATCH_BYTES bytes that the library keeps in the
 * device memory of every GPU that loads it, until the process exits. Plans
 * that need more scratch fail with MGB_ERR_WORKSPACE. Calls share the array:
 * calls that overlap on the GPU race. The first call on a device looks up the
 * array's address; make it before any stream capture. Allocates nothing.   */
#define MGB_NOALLOC_SCRATCH_BYTES (32u << 20)
int mgb_contract_noalloc(mgb_plan plan, const void *A, const void *B, void *C,
                         void *stream);

/* ---- status ---------------------------------------------------------------*/
const char *mgb_last_error(void);
/* Reads and clears, in one atomic exchange ordered on `stream`, the status
 * word of the current device written by bounded waits of the library's
 * kernels. The word is per device: it collects what kernels on every stream
 * and host thread recorded. Synchronises `stream`.                         */
int mgb_device_status(void *stream, int32_t *status);
/* Self-test of the bounded device waits (no counterpart in the reference):
 * launches one CTA whose mbarrier wait nothing ever completes, through the
 * same wait routine the contraction kernels use. The wait gives up after its
 * limit (about a second), records MGB_ERR_DEVICE_TIMEOUT in the device status
 * word and the kernel returns normally, so the context stays usable. Read the
 * word with mgb_device_status afterwards.                                  */
int mgb_selftest_wait_timeout(void *stream);
/* ---- thin singular value decomposition ---------------------------------------
 * The factorisation of simple_update (src/Operations/simple_update.jl:56-60),
 * done on the host by LinearAlgebra.svd in tensor_svd_thin
 * (src/Operations/tensor_svd.jl:98-125) and on CUDA by cuTensorNet (:34).
 * A (m x n, column-major with leading dimension lda, Float64 or ComplexF64)
 * = U diag(s) V^H with k = min(m, n) and s descending (Float64). Writes the
 * first `keep` triplets (keep <= 0 or > k: all k): U m x keep, s keep, V
 * n x keep, column-major and dense. Flags: MGB_SVD_NORMALIZE scales the kept
 * s to unit 2-norm (normalize! of simple_update); MGB_SVD_CONJ_V writes
 * conj(V), the right factor as tensor_svd_thin labels it; MGB_SVD_SQRT_S
 * writes sqrt of the (normalised) s, for an equal absorb. One-sided Jacobi
 * rotations in one thread block on the device: min(m, n) <= 1024, m n <=
 * 2^28. Left vectors of exactly zero singular values are completed to an
 * orthonormal set. The workspace comes from mgb_svd_workspace_size.        */
#define MGB_SVD_NORMALIZE 1
#define MGB_SVD_CONJ_V 2
#define MGB_SVD_SQRT_S 4
int mgb_svd_workspace_size(int32_t dtype, int64_t m, int64_t n, uint64_t *bytes);
int mgb_svd(int32_t dtype, int64_t m, int64_t n, const void *A, int64_t lda, void *U, void *s,
            void *V, int32_t keep, int32_t flags, void *workspace, uint64_t workspace_bytes,
            void *stream);

/* Roofline probe (no counterpart in the reference): the measured rate of an
 * FP64 pipe of the current device, the denominator of the plain form's and
 * the double-precision memory kernels' roofline fractions. op 0 = DMMA
 * (mma.sync m16n8k16 .f64, 4096 flops per warp instruction), 1 = DFMA (two
 * flops), 2 = DADD (one flop). Runs `iters` iterations of independent chains
 * in every thread of `blocks` x `threads` (a multiple of 32), timed with CUDA
 * events on `stream` (synchronised), and returns TFLOP/s. `scratch` (device,
 * one double per thread) receives values that keep the work alive.        */
int mgb_probe_fp64(int32_t op, int64_t iters, int32_t blocks, int32_t threads, void *scratch,
                   uint64_t scratch_bytes, void *stream, double *tflops);
/* Library version string. */
const char *mgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MUSCLE_GB300_H */
