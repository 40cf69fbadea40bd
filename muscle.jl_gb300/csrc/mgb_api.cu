// C ABI entry points, plan construction (label algebra, mode folding) and
// error reporting for libmuscle_gb300.
//
// Label algebra follows Muscle.jl:
//  * contracted = labels shared by A and B and absent from C
//    (src/Operations/binary_einsum.jl:34,77, cuTENSOR semantics of
//    ext/MuscleCUDAExt.jl:24-38);
//  * labels shared by A, B and C are batch (hyper) labels, which the CUDA
//    path supports (test/integration/cuda.jl:126-145);
//  * result eltype = promote_eltype(a, b) (ext/MuscleCUDAExt.jl:16);
//  * repeated labels must have equal extents (src/Tensor.jl:20-24).
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "mgb_internal.h"

namespace mgb {

static thread_local std::string g_last_error;

// Device status word written by bounded waits of the tcgen05 kernels; read
// and cleared by mgb_device_status(). Its address is looked up once per device.
// One word per device, shared by every stream and host thread; it is
// element 0 of the array, and the elements after it receive the values that
// mgb_device_status exchanges out (a ring of slots, one per call, so that
// concurrent callers on different streams do not share an output).
constexpr int kStatusSlots = 64;
__device__ int32_t mgb_status_word[1 + kStatusSlots];
static std::atomic<uint32_t> g_status_slot{0};

// Read-and-clear in one atomic exchange, so that a timeout recorded by a
// kernel on another stream between a read and a clear cannot be lost.
__global__ void k_status_exchange(int32_t *word, int32_t *out) { *out = atomicExch(word, 0); }

// Lock-free: the lookup is idempotent, so concurrent first calls at worst
// repeat it, and later launches take no lock.
int32_t *device_status_ptr() {
    static std::atomic<int32_t *> ptrs[128];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return nullptr;
    int32_t *p = ptrs[dev].load(std::memory_order_acquire);
    if (!p) {
        void *q = nullptr;
        if (cudaGetSymbolAddress(&q, mgb_status_word) != cudaSuccess) return nullptr;
        p = (int32_t *)q;
        ptrs[dev].store(p, std::memory_order_release);
    }
    return p;
}

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int status, const std::string &msg) {
    set_error(msg);
    return status;
}
int cuda_fail(cudaError_t err, const char *what) {
    set_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(err));
    return MGB_ERR_CUDA;
}

int read_desc(const mgb_tensor_desc *d, Desc &out, const char *name) {
    if (!d) return fail(MGB_ERR_ARGUMENT, std::string(name) + ": null descriptor");
    if (!valid_dtype(d->dtype))
        return fail(MGB_ERR_ARGUMENT, std::string(name) + ": unknown dtype");
    if (d->rank < 0 || d->rank > kMaxRank)
        return fail(MGB_ERR_ARGUMENT, std::string(name) + ": rank out of range");
    if (d->rank > 0 && (!d->modes || !d->extents))
        return fail(MGB_ERR_ARGUMENT, std::string(name) + ": null modes/extents");
    out.dtype = d->dtype;
    out.rank = d->rank;
    int64_t dense = 1;
    for (int i = 0; i < d->rank; ++i) {
        out.modes[i] = d->modes[i];
        out.ext[i] = d->extents[i];
        if (out.ext[i] < 0) return fail(MGB_ERR_ARGUMENT, std::string(name) + ": negative extent");
        out.str[i] = d->strides ? d->strides[i] : dense;
        dense *= std::max<int64_t>(out.ext[i], 1);
    }
    return MGB_OK;
}

// ---------------------------------------------------------------------------
// Mode folding.
// Builds a folded ModeGroup. `present[t]` marks tensors that carry the group.
// Modes are ordered by |stride| in tensor `primary`, extent-1 modes dropped,
// and neighbours merged when they are linear in every present tensor.
ModeGroup fold_group(std::vector<ModeRec> modes, const bool present[3], int primary) {
    ModeGroup g;
    bool empty = false;
    std::vector<ModeRec> kept;
    for (auto &m : modes) {
        if (m.ext == 0) empty = true;
        if (m.ext != 1) kept.push_back(m);
    }
    if (empty) {
        g.n = 1;
        g.ext[0] = 0;
        for (int t = 0; t < 3; ++t) g.str[t][0] = 0;
        return g;
    }
    std::stable_sort(kept.begin(), kept.end(), [&](const ModeRec &x, const ModeRec &y) {
        return std::llabs(x.str[primary]) < std::llabs(y.str[primary]);
    });
    std::vector<ModeRec> out;
    for (auto &m : kept) {
        if (!out.empty()) {
            ModeRec &p = out.back();
            bool lin = true;
            for (int t = 0; t < 3; ++t)
                if (present[t] && m.str[t] != p.str[t] * p.ext) lin = false;
            if (lin) {
                p.ext *= m.ext;
                continue;
            }
        }
        out.push_back(m);
    }
    g.n = (int)out.size();
    for (int i = 0; i < g.n; ++i) {
        g.ext[i] = out[i].ext;
        for (int t = 0; t < 3; ++t) g.str[t][i] = present[t] ? out[i].str[t] : 0;
    }
    return g;
}

static int64_t min_stride_label(const Desc &d) {
    int64_t best = INT64_MAX;
    int lab = INT32_MIN;
    for (int i = 0; i < d.rank; ++i)
        if (d.ext[i] > 1 && std::llabs(d.str[i]) < best) {
            best = std::llabs(d.str[i]);
            lab = d.modes[i];
        }
    return lab;
}

bool has_repeats(const Desc &d) {
    for (int i = 0; i < d.rank; ++i)
        for (int j = i + 1; j < d.rank; ++j)
            if (d.modes[i] == d.modes[j]) return true;
    return false;
}

int find_mode(const Desc &d, int label) {
    for (int i = 0; i < d.rank; ++i)
        if (d.modes[i] == label) return i;
    return -1;
}

static int build_contraction(ContractionPlan &p) {
    const Desc *T[3] = {&p.a, &p.b, &p.c};
    const char *names[3] = {"A", "B", "C"};
    for (int t = 0; t < 3; ++t)
        if (has_repeats(*T[t]))
            return fail(MGB_ERR_UNSUPPORTED,
                        std::string("binary contraction: repeated label in ") + names[t] +
                            " (take the diagonal with unary_einsum first)");
    p.compute_dtype = promote(p.a.dtype, p.b.dtype);
    if (p.c.dtype != p.compute_dtype)
        return fail(MGB_ERR_ARGUMENT, "C must have the promoted element type of A and B");
    // distinct labels in order of first appearance (A, then B, then C)
    std::vector<int> labels;
    for (int t = 0; t < 3; ++t)
        for (int i = 0; i < T[t]->rank; ++i)
            if (std::find(labels.begin(), labels.end(), T[t]->modes[i]) == labels.end())
                labels.push_back(T[t]->modes[i]);
    std::vector<ModeRec> left, right, contr, batch;
    for (int lab : labels) {
        int pos[3];
        int64_t ext = -1;
        ModeRec r;
        r.label = lab;
        for (int t = 0; t < 3; ++t) {
            pos[t] = find_mode(*T[t], lab);
            r.str[t] = 0;
            if (pos[t] >= 0) {
                int64_t e = T[t]->ext[pos[t]];
                if (ext >= 0 && e != ext)
                    return fail(MGB_ERR_DIMENSION_MISMATCH,
                                "label " + std::to_string(lab) + " has different extents");
                ext = e;
                r.str[t] = T[t]->str[pos[t]];
            }
        }
        r.ext = ext;
        bool ia = pos[0] >= 0, ib = pos[1] >= 0, ic = pos[2] >= 0;
        if (ia && ib && ic) batch.push_back(r);
        else if (ia && ib) contr.push_back(r);
        else if (ia && ic) left.push_back(r);
        else if (ib && ic) right.push_back(r);
        else if (ic)
            return fail(MGB_ERR_ARGUMENT,
                        "output label " + std::to_string(lab) + " is in neither operand");
        else
            return fail(MGB_ERR_ARGUMENT,
                        "label " + std::to_string(lab) +
                            " appears in one operand only and not in the output");
    }
    bool pm[3] = {true, false, true}, pn[3] = {false, true, true}, pk[3] = {true, true, false},
         pl[3] = {true, true, true};
    p.gm = fold_group(left, pm, 0);
    p.gn = fold_group(right, pn, 1);
    // contracted order follows the operand whose unit-stride mode is contracted
    int prim_k = 0;
    {
        int la = (int)min_stride_label(p.a), lb = (int)min_stride_label(p.b);
        auto in_k = [&](int lab) {
            for (auto &r : contr)
                if (r.label == lab) return true;
            return false;
        };
        if (!in_k(la) && in_k(lb)) prim_k = 1;
    }
    p.gk = fold_group(contr, pk, prim_k);
    p.gl = fold_group(batch, pl, 2);
    p.M = p.gm.size();
    p.N = p.gn.size();
    p.K = p.gk.size();
    p.L = p.gl.size();
    if (p.L > 65535) return fail(MGB_ERR_UNSUPPORTED, "more than 65535 batch entries");
    return MGB_OK;
}

static int resolve_form(ContractionPlan &p, int form, int slices) {
    bool dbl = is_double(p.compute_dtype);
    if (form == MGB_FORM_AUTO) form = dbl ? MGB_FORM_OZAKI : MGB_FORM_BF16X3;
    if (form == MGB_FORM_OZAKI && !dbl)
        return fail(MGB_ERR_UNSUPPORTED, "OZAKI form needs a Float64/ComplexF64 result");
    if (form == MGB_FORM_BF16X3 && dbl)
        return fail(MGB_ERR_UNSUPPORTED, "BF16X3 form needs a Float32/ComplexF32 result");
    if (form != MGB_FORM_PLAIN && form != MGB_FORM_OZAKI && form != MGB_FORM_BF16X3)
        return fail(MGB_ERR_ARGUMENT, "unknown form");
    p.form = form;
    if (form == MGB_FORM_OZAKI) {
        if (slices == 0) {
            p.adaptive = true;  // chosen per call from the operands (ozaki_setup sizes for the largest)
            p.slices = 8;
            return MGB_OK;
        }
        if (slices < 3 || slices > 8) return fail(MGB_ERR_ARGUMENT, "OZAKI slices must be in 3..8, or 0 (adaptive)");
        p.slices = slices;
    } else if (form == MGB_FORM_BF16X3) {
        p.slices = 3;
    } else {
        p.slices = 0;
    }
    return MGB_OK;
}

static uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

// The plain kernels read operands of any element type in place (widening on
// load), so the plain form needs no workspace.
static void plain_workspace(ContractionPlan &p) {
    p.convert_a = p.convert_b = false;
    p.ws_bytes = 0;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

const char *mgb_last_error(void) { return g_last_error.c_str(); }

const char *mgb_version(void) { return "muscle_gb300 0.1.0 (sm_103a)"; }

int mgb_contraction_plan(mgb_plan *plan, const mgb_tensor_desc *a, const mgb_tensor_desc *b,
                         const mgb_tensor_desc *c, int32_t form, int32_t slices) {
    if (!plan) return fail(MGB_ERR_ARGUMENT, "plan output pointer is null");
    *plan = nullptr;
    auto *p = new mgb_plan_s();
    p->kind = PlanKind::Contraction;
    ContractionPlan &cp = p->cp;
    int st;
    if ((st = read_desc(a, cp.a, "A")) || (st = read_desc(b, cp.b, "B")) ||
        (st = read_desc(c, cp.c, "C")) || (st = build_contraction(cp)) ||
        (st = resolve_form(cp, form, slices))) {
        delete p;
        return st;
    }
    if (cp.form == MGB_FORM_PLAIN) {
        plain_workspace(cp);
    } else {
        ozaki_orient(cp);
        ozaki_setup(cp);
    }
    if (cp.adaptive && cp.oz_R < 0) {  // no slice count holds K exactly: the plain form
        cp.adaptive = false;
        cp.form = MGB_FORM_PLAIN;
        cp.slices = 0;
        cp.oz_R = 0;
        plain_workspace(cp);
    }
    if (cp.oz_R < 0) {
        delete p;
        return fail(MGB_ERR_UNSUPPORTED, "contracted extent too long for the exact OZAKI accumulator");
    }
    *plan = p;
    return MGB_OK;
}

int mgb_plan_destroy(mgb_plan plan) {
    delete plan;
    return MGB_OK;
}

int mgb_plan_workspace_size(mgb_plan plan, uint64_t *bytes) {
    if (!plan || !bytes) return fail(MGB_ERR_ARGUMENT, "null argument");
    *bytes = plan->kind == PlanKind::Contraction ? plan->cp.ws_bytes : 0;
    return MGB_OK;
}

int mgb_plan_info_get(mgb_plan plan, mgb_plan_info *info) {
    if (!plan || !info) return fail(MGB_ERR_ARGUMENT, "null argument");
    std::memset(info, 0, sizeof(*info));
    if (plan->kind == PlanKind::Unary) {
        info->m = plan->up.O;
        info->k = plan->up.R;
        info->n = info->batch = 1;
        info->form = MGB_FORM_PLAIN;
        info->compute_dtype = plan->up.x.dtype;
        info->flops = (double)plan->up.O * (double)plan->up.R * (is_complex(plan->up.x.dtype) ? 2 : 1);
        return MGB_OK;
    }
    const ContractionPlan &cp = plan->cp;
    info->m = cp.swapped ? cp.N : cp.M;  // the caller's A and B
    info->n = cp.swapped ? cp.M : cp.N;
    info->k = cp.K;
    info->batch = cp.L;
    info->form = cp.form;
    info->slices = (cp.form == MGB_FORM_OZAKI && !cp.adaptive) ? cp.slices : 0;
    info->compute_dtype = cp.compute_dtype;
    info->permute_a = cp.swapped ? cp.convert_b : cp.convert_a;
    info->permute_b = cp.swapped ? cp.convert_a : cp.convert_b;
    info->permute_c = 0;
    info->flops = (is_complex(cp.compute_dtype) ? 8.0 : 2.0) * (double)cp.M * (double)cp.N *
                  (double)cp.K * (double)cp.L;
    info->workspace_bytes = cp.ws_bytes;
    return MGB_OK;
}

static int contract_impl(mgb_plan plan, const void *A, const void *B, void *C, void *workspace,
                         uint64_t workspace_bytes, void *stream);

int mgb_contract(mgb_plan plan, const void *A, const void *B, void *C, void *workspace,
                 uint64_t workspace_bytes, void *stream) {
    if (!plan || plan->kind != PlanKind::Contraction)
        return fail(MGB_ERR_ARGUMENT, "not a contraction plan");
    if (!plan->timing) return contract_impl(plan, A, B, C, workspace, workspace_bytes, stream);
    cudaStream_t s = (cudaStream_t)stream;
    for (auto &e : plan->ev)
        if (!e) MGB_CUDA_CHECK(cudaEventCreate(&e));
    MGB_CUDA_CHECK(cudaEventRecord(plan->ev[0], s));
    int st = contract_impl(plan, A, B, C, workspace, workspace_bytes, stream);
    if (st) return st;
    MGB_CUDA_CHECK(cudaEventRecord(plan->ev[2], s));
    return MGB_OK;
}

static int contract_impl(mgb_plan plan, const void *A, const void *B, void *C, void *workspace,
                         uint64_t workspace_bytes, void *stream) {
    const ContractionPlan &cp = plan->cp;
    cudaStream_t s = (cudaStream_t)stream;
    if (workspace_bytes < cp.ws_bytes || (cp.ws_bytes && !workspace))
        return fail(MGB_ERR_WORKSPACE, "workspace smaller than mgb_plan_workspace_size");
    int64_t nc = cp.M * cp.N * cp.L;
    if (nc == 0) {
        if (plan->timing) MGB_CUDA_CHECK(cudaEventRecord(plan->ev[1], s));
        return MGB_OK;
    }
    if (!C) return fail(MGB_ERR_ARGUMENT, "null output pointer");
    if (plan->timing) MGB_CUDA_CHECK(cudaEventRecord(plan->ev[1], s));
    if (cp.K == 0) return launch_fill_zero(C, nc, cp.c.dtype, cp.c, s);  // empty sum
    if (!A || !B) return fail(MGB_ERR_ARGUMENT, "null operand pointer");
    if (cp.swapped) std::swap(A, B);  // the plan computes C^T = B^T A^T
    if (cp.form == MGB_FORM_PLAIN) return launch_plain_gemm(cp, A, B, C, s);
    return launch_ozaki(cp, A, B, C, workspace, s, plan->timing ? plan->ev[1] : nullptr);
}

int mgb_plan_set_timing(mgb_plan plan, int32_t enable) {
    if (!plan) return fail(MGB_ERR_ARGUMENT, "null plan");
    plan->timing = enable != 0;
    return MGB_OK;
}

int mgb_plan_operands_swapped(mgb_plan plan, int32_t *swapped) {
    if (!plan || !swapped || plan->kind != PlanKind::Contraction)
        return fail(MGB_ERR_ARGUMENT, "operands_swapped: needs a contraction plan and an output");
    *swapped = plan->cp.swapped ? 1 : 0;
    return MGB_OK;
}

int mgb_plan_set_band(mgb_plan plan, int32_t band) {
    if (!plan || plan->kind != PlanKind::Contraction) return fail(MGB_ERR_ARGUMENT, "band: not a contraction plan");
    if (band < 0 || band > 64) return fail(MGB_ERR_ARGUMENT, "band must be in 0..64");
    plan->cp.band = band;
    return MGB_OK;
}

int mgb_plan_set_tolerance(mgb_plan plan, double tolerance) {
    if (!plan || plan->kind != PlanKind::Contraction)
        return fail(MGB_ERR_ARGUMENT, "tolerance: not a contraction plan");
    return ozaki_set_tolerance(plan->cp, tolerance);
}

int mgb_plan_adaptive_report(mgb_plan plan, const void *workspace, void *stream, mgb_adaptive_report *report) {
    if (!plan || !report || plan->kind != PlanKind::Contraction)
        return fail(MGB_ERR_ARGUMENT, "adaptive report: null argument or not a contraction plan");
    return ozaki_adaptive_report(plan->cp, workspace, (cudaStream_t)stream, report);
}

int mgb_plan_timing(mgb_plan plan, float *prepass_ms, float *main_ms) {
    if (!plan || !prepass_ms || !main_ms) return fail(MGB_ERR_ARGUMENT, "null argument");
    if (!plan->timing || !plan->ev[0]) return fail(MGB_ERR_ARGUMENT, "timing was not enabled");
    MGB_CUDA_CHECK(cudaEventSynchronize(plan->ev[2]));
    MGB_CUDA_CHECK(cudaEventElapsedTime(prepass_ms, plan->ev[0], plan->ev[1]));
    MGB_CUDA_CHECK(cudaEventElapsedTime(main_ms, plan->ev[1], plan->ev[2]));
    return MGB_OK;
}

int mgb_permute(const mgb_tensor_desc *x, const mgb_tensor_desc *y, const void *X, void *Y,
                void *stream) {
    Desc dx, dy;
    int st;
    if ((st = read_desc(x, dx, "X")) || (st = read_desc(y, dy, "Y"))) return st;
    if (dx.rank != dy.rank) return fail(MGB_ERR_ARGUMENT, "permute: ranks differ");
    if (has_repeats(dx) || has_repeats(dy))
        return fail(MGB_ERR_ARGUMENT, "permute: repeated labels");
    for (int i = 0; i < dy.rank; ++i) {
        int j = find_mode(dx, dy.modes[i]);
        if (j < 0) return fail(MGB_ERR_ARGUMENT, "permute: output label missing from input");
        if (dx.ext[j] != dy.ext[i]) return fail(MGB_ERR_DIMENSION_MISMATCH, "permute: extents differ");
    }
    bool ok = dx.dtype == dy.dtype || (dx.dtype == MGB_F32 && dy.dtype != MGB_F32) ||
              (dx.dtype == MGB_F64 && dy.dtype == MGB_C64) ||
              (dx.dtype == MGB_C32 && dy.dtype == MGB_C64);
    if (!ok) return fail(MGB_ERR_ARGUMENT, "permute: only widening conversions are allowed");
    return launch_permute(dx, dy, X, Y, (cudaStream_t)stream);
}

// ---- unary ---------------------------------------------------------------
int mgb_unary_plan(mgb_plan *plan, const mgb_tensor_desc *x, const mgb_tensor_desc *y) {
    if (!plan) return fail(MGB_ERR_ARGUMENT, "plan output pointer is null");
    *plan = nullptr;
    auto *p = new mgb_plan_s();
    p->kind = PlanKind::Unary;
    UnaryPlan &up = p->up;
    int st;
    if ((st = read_desc(x, up.x, "X")) || (st = read_desc(y, up.y, "Y"))) {
        delete p;
        return st;
    }
    if (up.x.dtype != up.y.dtype) {
        delete p;
        return fail(MGB_ERR_ARGUMENT, "unary: X and Y must share the element type");
    }
    if (has_repeats(up.y)) {
        delete p;
        return fail(MGB_ERR_ARGUMENT, "unary: output labels must be distinct");
    }
    // distinct labels of X with summed strides (a repeated label walks the diagonal)
    std::vector<ModeRec> outm, redm;
    std::vector<int> seen;
    for (int i = 0; i < up.x.rank; ++i) {
        int lab = up.x.modes[i];
        if (std::find(seen.begin(), seen.end(), lab) != seen.end()) continue;
        seen.push_back(lab);
        ModeRec r;
        r.label = lab;
        r.ext = up.x.ext[i];
        r.str[0] = 0;
        r.str[1] = 0;
        r.str[2] = 0;
        for (int j = 0; j < up.x.rank; ++j)
            if (up.x.modes[j] == lab) {
                if (up.x.ext[j] != r.ext) {
                    delete p;
                    return fail(MGB_ERR_DIMENSION_MISMATCH, "nonuniform size of repeated indices");
                }
                r.str[0] += up.x.str[j];
            }
        int jy = find_mode(up.y, lab);
        if (jy >= 0) {
            if (up.y.ext[jy] != r.ext) {
                delete p;
                return fail(MGB_ERR_DIMENSION_MISMATCH, "unary: output extent differs");
            }
            r.str[1] = up.y.str[jy];
            outm.push_back(r);
        } else {
            redm.push_back(r);
        }
    }
    for (int i = 0; i < up.y.rank; ++i)
        if (find_mode(up.x, up.y.modes[i]) < 0) {
            delete p;
            return fail(MGB_ERR_ARGUMENT, "Output indices must be a subset of input indices");
        }
    bool po[3] = {true, true, false}, pr[3] = {true, false, false};
    up.go = fold_group(outm, po, 1);
    up.gr = fold_group(redm, pr, 0);
    up.O = up.go.size();
    up.R = up.gr.size();
    *plan = p;
    return MGB_OK;
}

int mgb_unary(mgb_plan plan, const void *X, void *Y, void *workspace, uint64_t workspace_bytes,
              void *stream) {
    (void)workspace;
    (void)workspace_bytes;
    if (!plan || plan->kind != PlanKind::Unary) return fail(MGB_ERR_ARGUMENT, "not a unary plan");
    const UnaryPlan &up = plan->up;
    if (up.O == 0) return MGB_OK;
    if (!X || !Y) return fail(MGB_ERR_ARGUMENT, "null operand pointer");
    return launch_unary(up, X, Y, (cudaStream_t)stream);
}

int mgb_selftest_wait_timeout(void *stream) { return selftest_wait_timeout((cudaStream_t)stream); }

int mgb_device_status(void *stream, int32_t *status) {
    if (!status) return fail(MGB_ERR_ARGUMENT, "null status pointer");
    cudaStream_t s = (cudaStream_t)stream;
    int32_t *d = device_status_ptr();
    if (!d) return fail(MGB_ERR_CUDA, "device status word unavailable");
    int32_t *out = d + 1 + (int)(g_status_slot.fetch_add(1, std::memory_order_relaxed) % kStatusSlots);
    k_status_exchange<<<1, 1, 0, s>>>(d, out);
    MGB_CUDA_CHECK(cudaGetLastError());
    int32_t v = 0;
    MGB_CUDA_CHECK(cudaMemcpyAsync(&v, out, sizeof(v), cudaMemcpyDeviceToHost, s));
    MGB_CUDA_CHECK(cudaStreamSynchronize(s));
    *status = v;
    return MGB_OK;
}

}  // extern "C"
