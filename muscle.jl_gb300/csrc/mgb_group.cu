// Grouped execution of many independent contraction plans.
//
// Members that share a plan (same shapes, strides, element types and form;
// callers that cache plans by descriptor get this for free) form a bucket. A
// bucket runs as one batched launch of each kernel of its form: the batch
// index selects the member, whose operand and output pointers come from a
// device array instead of a batch stride. A PEPS sweep (thousands of pairs of
// a handful of shape classes) therefore costs a handful of launches per
// class, all on one stream, so the caller can capture the group in one CUDA
// graph. Members that cannot be batched (an empty contraction, a plan that is
// already batched) run one by one through mgb_contract. The workspace is carved into per-bucket and
// per-member slices.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "mgb_internal.h"

namespace {

struct Bucket {
    mgb_plan plan = nullptr;        // the shared member plan
    std::vector<int> members;
    mgb::ContractionPlan cp;        // batched copy: L = members, pointer arrays
    void **dptr = nullptr;          // device: A[L], B[L], C[L]
    uint64_t ws_off = 0;
};

struct Single {
    int member;
    uint64_t ws_off;
};

const int kBands[6] = {1, 2, 3, 4, 8, 16};

}  // namespace

struct mgb_group_s {
    std::vector<mgb_plan> plans;
    std::vector<const void *> A, B;
    std::vector<void *> C;
    std::vector<Bucket> buckets;
    std::vector<Single> singles;
    uint64_t ws_bytes = 0;
    // One persistent GEMM launch per kernel variant of the emulated buckets;
    // its job table holds slice addresses inside the workspace, so it is
    // built on the first execution with a workspace and rebuilt when the
    // workspace moves.
    void *grouped_ws = nullptr;
    std::vector<mgb::OzGrouped *> grouped;
    // Tables of earlier builds: a CUDA graph captured before the rebuild may
    // still launch with them, so they live until the group is destroyed.
    std::vector<mgb::OzGrouped *> retired;
    // One event per stream an execution ran on, recorded at its end (inside a
    // CUDA graph as an external event node, so replays record it too):
    // mgb_group_update waits for them before it rewrites the pointer arrays.
    std::vector<std::pair<cudaStream_t, cudaEvent_t>> done;
    std::mutex done_mu;
};

using namespace mgb;

static bool batchable(const mgb_plan p) {
    const ContractionPlan &cp = p->cp;
    if (cp.L != 1 || cp.K == 0 || cp.M * cp.N == 0) return false;
    return true;
}

static int upload(mgb_group g) {
    for (auto &b : g->buckets) {
        const size_t n = b.members.size();
        std::vector<void *> h(3 * n);
        const bool sw = b.cp.swapped;  // the plan computes C^T = B^T A^T
        for (size_t i = 0; i < n; ++i) {
            const int m = b.members[i];
            h[i] = const_cast<void *>(sw ? g->B[m] : g->A[m]);
            h[n + i] = const_cast<void *>(sw ? g->A[m] : g->B[m]);
            h[2 * n + i] = g->C[m];
        }
        MGB_CUDA_CHECK(cudaMemcpy(b.dptr, h.data(), 3 * n * sizeof(void *), cudaMemcpyHostToDevice));
    }
    return MGB_OK;
}

static void free_grouped(mgb_group g) {
    for (auto *x : g->grouped) ozaki_grouped_destroy(x);
    for (auto *x : g->retired) ozaki_grouped_destroy(x);
    g->grouped.clear();
    g->retired.clear();
    g->grouped_ws = nullptr;
}

// Records the end of an execution on `s` (see mgb_group_s::done).
static int mark_done(mgb_group g, cudaStream_t s) {
    cudaEvent_t ev = nullptr;
    {
        std::lock_guard<std::mutex> lk(g->done_mu);
        for (auto &x : g->done)
            if (x.first == s) ev = x.second;
        if (!ev) {
            MGB_CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            g->done.push_back({s, ev});
        }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    MGB_CUDA_CHECK(cudaStreamIsCapturing(s, &cap));
    if (cap == cudaStreamCaptureStatusActive) MGB_CUDA_CHECK(cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal));
    else MGB_CUDA_CHECK(cudaEventRecord(ev, s));
    return MGB_OK;
}

static void free_group(mgb_group g) {
    for (auto &x : g->done) cudaEventDestroy(x.second);
    free_grouped(g);
    for (auto &b : g->buckets)
        if (b.dptr) cudaFree(b.dptr);
    delete g;
}

// Job tables of the persistent GEMM launches, one per kernel variant
// (slices, form, real or complex) of the emulated buckets. An adaptive
// bucket has a job in the launch of every candidate slice count, each of
// which works only when the device chose that count.
static int build_grouped(mgb_group g, void *workspace) {
    g->retired.insert(g->retired.end(), g->grouped.begin(), g->grouped.end());
    g->grouped.clear();
    g->grouped_ws = nullptr;
    std::map<std::tuple<int, int, int>, std::pair<std::vector<const ContractionPlan *>, std::vector<void *>>> sets;
    for (auto &b : g->buckets) {
        if (b.cp.form == MGB_FORM_PLAIN) continue;  // no tensor-core part
        const int cx = is_complex(b.cp.compute_dtype) ? 1 : 0;
        for (int S = 3; S <= 8; ++S) {
            if (b.cp.adaptive ? !(b.cp.cand_mask & (1u << S)) : S != b.cp.slices) continue;
            auto &e = sets[std::make_tuple(S, b.cp.form, cx)];
            e.first.push_back(&b.cp);
            e.second.push_back((char *)workspace + b.ws_off);
        }
    }
    for (auto &kv : sets) {
        // longest tiles first: each CTA then ends its walk on short tiles,
        // which even out the CTAs' finishing times
        {
            auto &pl = kv.second.first;
            auto &wl = kv.second.second;
            std::vector<size_t> ord(pl.size());
            for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
            std::stable_sort(ord.begin(), ord.end(), [&](size_t u, size_t v) { return pl[u]->k_e > pl[v]->k_e; });
            std::vector<const ContractionPlan *> p2;
            std::vector<void *> w2;
            for (size_t i : ord) {
                p2.push_back(pl[i]);
                w2.push_back(wl[i]);
            }
            pl.swap(p2);
            wl.swap(w2);
        }
        OzGrouped *x = nullptr;
        const int S = std::get<0>(kv.first);
        const bool exact = std::get<1>(kv.first) == MGB_FORM_OZAKI, cx = std::get<2>(kv.first) != 0;
        if (int st = ozaki_grouped_create(kv.second.first, kv.second.second, S, exact, cx, &x)) {
            for (auto *y : g->grouped) ozaki_grouped_destroy(y);  // never launched
            g->grouped.clear();
            return st;
        }
        g->grouped.push_back(x);
    }
    g->grouped_ws = workspace;
    return MGB_OK;
}

extern "C" {

int mgb_group_create(mgb_group *group, const mgb_plan *plans, int32_t count, const void *const *A,
                     const void *const *B, void *const *C) {
    if (!group) return fail(MGB_ERR_ARGUMENT, "group output pointer is null");
    *group = nullptr;
    if (count < 0 || (count > 0 && (!plans || !A || !B || !C)))
        return fail(MGB_ERR_ARGUMENT, "group: null arrays");
    auto *g = new mgb_group_s();
    std::map<mgb_plan, int> index;
    for (int i = 0; i < count; ++i) {
        if (!plans[i] || plans[i]->kind != PlanKind::Contraction) {
            free_group(g);
            return fail(MGB_ERR_ARGUMENT, "group: member " + std::to_string(i) + " is not a contraction plan");
        }
        g->plans.push_back(plans[i]);
        g->A.push_back(A[i]);
        g->B.push_back(B[i]);
        g->C.push_back(C[i]);
        if (batchable(plans[i])) {
            auto it = index.find(plans[i]);
            if (it == index.end()) {
                index[plans[i]] = (int)g->buckets.size();
                g->buckets.emplace_back();
                g->buckets.back().plan = plans[i];
            }
            g->buckets[index[plans[i]]].members.push_back(i);
        } else {
            g->singles.push_back({i, 0});
        }
    }
    uint64_t off = 0;
    for (auto &b : g->buckets) {
        const int64_t n = (int64_t)b.members.size();
        if (n > 65535) {
            free_group(g);
            return fail(MGB_ERR_UNSUPPORTED, "group: more than 65535 members share one plan");
        }
        b.cp = b.plan->cp;
        b.cp.L = n;
        b.cp.gl.n = 1;
        b.cp.gl.ext[0] = n;
        for (int t = 0; t < 3; ++t) b.cp.gl.str[t][0] = 0;
        if (b.cp.form != MGB_FORM_PLAIN) ozaki_setup(b.cp);  // workspace for L members
        else b.cp.ws_bytes = 0;
        cudaError_t e = cudaMalloc((void **)&b.dptr, 3 * n * sizeof(void *));
        if (e != cudaSuccess) {
            b.dptr = nullptr;
            free_group(g);
            return cuda_fail(e, "cudaMalloc(group pointer arrays)");
        }
        b.cp.pa = (const void *const *)b.dptr;
        b.cp.pb = (const void *const *)(b.dptr + n);
        b.cp.pc = b.dptr + 2 * n;
        b.ws_off = off;
        off += (b.cp.ws_bytes + 255) & ~uint64_t(255);
    }
    for (auto &s : g->singles) {
        s.ws_off = off;
        off += (g->plans[s.member]->cp.ws_bytes + 255) & ~uint64_t(255);
    }
    g->ws_bytes = off;
    int st = upload(g);
    if (st) {
        free_group(g);
        return st;
    }
    *group = g;
    return MGB_OK;
}

int mgb_group_update(mgb_group group, const void *const *A, const void *const *B, void *const *C) {
    if (!group || !A || !B || !C) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    {
        // executions (and graph replays) still reading the pointer arrays
        std::lock_guard<std::mutex> lk(group->done_mu);
        for (auto &x : group->done) MGB_CUDA_CHECK(cudaEventSynchronize(x.second));
    }
    for (size_t i = 0; i < group->plans.size(); ++i) {
        group->A[i] = A[i];
        group->B[i] = B[i];
        group->C[i] = C[i];
    }
    return upload(group);
}

int mgb_group_workspace_size(mgb_group group, uint64_t *bytes) {
    if (!group || !bytes) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    *bytes = group->ws_bytes;
    return MGB_OK;
}

int mgb_group_set_tiles(mgb_group group, const int32_t *tile_per_plan) {
    if (!group || !tile_per_plan) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    for (auto &b : group->buckets) {
        const int t = tile_per_plan[b.members.front()];
        b.cp.band = (t >= 0 && t < 6) ? kBands[t] : 0;
    }
    group->grouped_ws = nullptr;  // the job tables embed the bands: rebuild on the next execution
    return MGB_OK;
}

// Work units (buckets, then singles) of part `part` of `nparts`: units are
// dealt in decreasing order of flops to the part with the least work so far.
static std::vector<int> part_units(const mgb_group_s *g, int part, int nparts) {
    const int nb = (int)g->buckets.size(), nu = nb + (int)g->singles.size();
    std::vector<std::pair<double, int>> w(nu);
    for (int u = 0; u < nu; ++u) {
        const ContractionPlan &cp = u < nb ? g->buckets[u].cp : g->plans[g->singles[u - nb].member]->cp;
        w[u] = {(double)cp.M * (double)cp.N * (double)std::max<int64_t>(cp.K, 1) * (double)cp.L, u};
    }
    std::stable_sort(w.begin(), w.end(), [](const std::pair<double, int> &x, const std::pair<double, int> &y) {
        return x.first > y.first;
    });
    std::vector<double> load(nparts, 0.0);
    std::vector<int> mine;
    for (auto &x : w) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += x.first;
        if (k == part) mine.push_back(x.second);
    }
    std::sort(mine.begin(), mine.end());
    return mine;
}

static int run_unit(mgb_group g, int u, void *workspace, cudaStream_t s) {
    const int nb = (int)g->buckets.size();
    if (u < nb) {
        Bucket &b = g->buckets[u];
        return b.cp.form == MGB_FORM_PLAIN ? launch_plain_gemm(b.cp, nullptr, nullptr, nullptr, s)
                                           : launch_ozaki(b.cp, nullptr, nullptr, nullptr, (char *)workspace + b.ws_off, s);
    }
    const Single &m = g->singles[u - nb];
    const mgb_plan p = g->plans[m.member];
    void *w = p->cp.ws_bytes ? (char *)workspace + m.ws_off : nullptr;
    return mgb_contract(p, g->A[m.member], g->B[m.member], g->C[m.member], w, p->cp.ws_bytes, s);
}

static int check_ws(mgb_group group, void *workspace, uint64_t workspace_bytes) {
    if (!group) return fail(MGB_ERR_ARGUMENT, "group: null argument");
    if (workspace_bytes < group->ws_bytes || (group->ws_bytes && !workspace))
        return fail(MGB_ERR_WORKSPACE, "group workspace smaller than mgb_group_workspace_size");
    return MGB_OK;
}

int mgb_group_prepare_part(mgb_group group, int32_t part, int32_t nparts, void *workspace, uint64_t workspace_bytes,
                           void *stream) {
    if (int st = check_ws(group, workspace, workspace_bytes)) return st;
    if (nparts < 1 || part < 0 || part >= nparts) return fail(MGB_ERR_ARGUMENT, "group: part out of range");
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = (int)group->buckets.size();
    auto one = [&](int u) -> int {
        Bucket &b = group->buckets[u];
        return b.cp.form == MGB_FORM_PLAIN ? launch_plain_gemm(b.cp, nullptr, nullptr, nullptr, s)
                                           : ozaki_prepass(b.cp, nullptr, nullptr, (char *)workspace + b.ws_off, s);
    };
    if (nparts == 1) {
        for (int u = 0; u < nb; ++u)
            if (int st = one(u)) return st;
        return mark_done(group, s);
    }
    for (int u : part_units(group, part, nparts))
        if (u < nb)
            if (int st = one(u)) return st;
    return mark_done(group, s);
}

int mgb_group_finish(mgb_group group, void *workspace, uint64_t workspace_bytes, void *stream) {
    if (int st = check_ws(group, workspace, workspace_bytes)) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (group->grouped_ws != workspace)
        if (int st = build_grouped(group, workspace)) return st;
    for (auto *x : group->grouped)
        if (int st = ozaki_grouped_launch(x, s)) return st;
    // adaptive buckets whose device choice was the plain form
    for (auto &b : group->buckets)
        if (b.cp.adaptive)
            if (int st = ozaki_plain_fallback(b.cp, nullptr, nullptr, nullptr, (char *)workspace + b.ws_off, s))
                return st;
    const int nb = (int)group->buckets.size(), nu = nb + (int)group->singles.size();
    for (int u = nb; u < nu; ++u)
        if (int st = run_unit(group, u, workspace, s)) return st;
    return mark_done(group, s);
}

int mgb_group_execute(mgb_group group, void *workspace, uint64_t workspace_bytes, void *stream) {
    if (int st = check_ws(group, workspace, workspace_bytes)) return st;
    // build the job tables before any launch, so that a failure leaves no work queued
    if (group->grouped_ws != workspace)
        if (int st = build_grouped(group, workspace)) return st;
    if (int st = mgb_group_prepare_part(group, 0, 1, workspace, workspace_bytes, stream)) return st;
    return mgb_group_finish(group, workspace, workspace_bytes, stream);
}

int mgb_group_execute_part(mgb_group group, int32_t part, int32_t nparts, void *workspace, uint64_t workspace_bytes,
                           void *stream) {
    if (int st = check_ws(group, workspace, workspace_bytes)) return st;
    if (nparts < 1 || part < 0 || part >= nparts) return fail(MGB_ERR_ARGUMENT, "group: part out of range");
    cudaStream_t s = (cudaStream_t)stream;
    if (nparts == 1) {
        const int nu = (int)(group->buckets.size() + group->singles.size());
        for (int u = 0; u < nu; ++u)
            if (int st = run_unit(group, u, workspace, s)) return st;
        return mark_done(group, s);
    }
    for (int u : part_units(group, part, nparts))
        if (int st = run_unit(group, u, workspace, s)) return st;
    return mark_done(group, s);
}

int mgb_group_destroy(mgb_group group) {
    if (group) free_group(group);
    return MGB_OK;
}

}  // extern "C"
