// Serving loop: contractions submitted as they arrive, admitted against a
// device-memory byte budget, and run as batched launches with continuous
// batching over several streams, so that requests arriving while others run
// join the next batch and overlap with the running ones on the GPU.
//
// A scheduler thread owned by the server repeatedly
//   1. retires finished requests one by one: every request waits on the event
//      of the launch that computed it, not on the whole batch;
//   2. admits queued requests in arrival order while the bytes of admitted,
//      unfinished requests (operands, output and workspace) stay within the
//      budget, and launches them as one batch on an idle stream:
//        - the emulated-form requests (Ozaki, BF16x3; each with its own
//          shapes) through the batched path: one launch per pre-pass phase
//          over all of their operands, the adaptive slice choices in one
//          launch, and one persistent tensor-core launch per kernel variant,
//          each followed by an event that retires the requests it computed;
//        - plain-form requests one launch each, each with its own event;
//      a batch takes one workspace block from the server's stream-ordered
//      memory pool (cudaMallocFromPoolAsync, no device synchronisation);
//   3. re-runs through mgb_contract the adaptive requests whose device
//      choice was the plain form (their estimate met no slice count);
//   4. sleeps briefly when there is nothing to do.
// A request finishes with MGB_ERR_DEVICE_TIMEOUT when the device status word
// (bounded waits of the kernels) is set at its retirement. Latency is measured
// from submission to the moment the scheduler sees the request finished.
// Plans and device buffers stay owned by the caller, who must keep them alive
// until the request is finished.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "mgb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t ticket;
    mgb_plan plan;
    const void *A, *B;
    void *C;
    uint64_t bytes;      // admitted bytes: caller-declared resident bytes + workspace
    cudaEvent_t dep;     // caller-stream event the request waits on (or null)
    Clock::time_point t0;
    cudaEvent_t done = nullptr;    // the launch that computes it (set once known)
    bool own_done = false;         // `done` belongs to this request alone
    const int32_t *status_word = nullptr;  // pinned snapshot of the device status after its launch
    int32_t status = MGB_OK;
};

// A kernel variant of the batched tensor-core launches: slice count, exact
// (Ozaki) or not (BF16x3), complex or real.
typedef std::tuple<int, int, int> Variant;
constexpr int kMaxVariants = 16;

struct Batch {
    std::vector<Req> emu;        // emulated-form requests (batched path)
    std::vector<Req> plain;      // plain-form requests (own launches)
    std::map<Variant, std::pair<cudaEvent_t, int32_t *>> variant;  // event and status snapshot after its launch
    cudaEvent_t chosen = nullptr;  // the slice counts have reached sel_host
    bool mapped = false;           // every emulated request knows its launch
    void *ws = nullptr;
    int32_t *sel_dev = nullptr, *sel_host = nullptr;  // per emulated request
    size_t sel_cap = 0;
    int32_t *status_host = nullptr;  // pinned: [0] after the plain launches, [1 + v] after variant v
    cudaEvent_t end = nullptr;       // after everything of the batch
    mgb::OzBatchBuffers *buf = nullptr;
    bool busy = false;
};

}  // namespace

struct mgb_server_s {
    int device = 0;
    uint64_t budget = 0, used = 0;
    int max_batch = 256;
    cudaMemPool_t pool = nullptr;
    std::vector<cudaStream_t> streams;
    std::vector<Batch> slots;  // one in-flight batch per stream
    std::deque<Req> pending;
    std::unordered_map<int64_t, int32_t> finished;  // ticket -> status
    std::vector<double> latency_ms;
    std::vector<cudaEvent_t> event_pool;
    std::mutex mu;     // queue, results, statistics and budget
    std::mutex ev_mu;  // event pool (never held while taking mu)
    std::condition_variable cv_work, cv_done;
    std::atomic<bool> stop{false};
    std::thread worker;
    int64_t next_ticket = 1;
    uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0;
    Clock::time_point started;
};

using namespace mgb;

static cudaEvent_t take_event(mgb_server_s *s) {
    {
        std::lock_guard<std::mutex> lk(s->ev_mu);
        if (!s->event_pool.empty()) {
            cudaEvent_t e = s->event_pool.back();
            s->event_pool.pop_back();
            return e;
        }
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

static void give_event(mgb_server_s *s, cudaEvent_t e) {
    if (!e) return;
    std::lock_guard<std::mutex> lk(s->ev_mu);
    s->event_pool.push_back(e);
}

static void finish(mgb_server_s *s, const Req &r, int32_t status) {
    // caller holds s->mu
    s->finished[r.ticket] = status;
    s->latency_ms.push_back(std::chrono::duration<double, std::milli>(Clock::now() - r.t0).count());
    s->used -= r.bytes;
    ++s->completed;
    give_event(s, r.dep);
}

static int alloc_ws(mgb_server_s *s, void **p, uint64_t bytes, cudaStream_t st) {
    *p = nullptr;
    if (!bytes) return MGB_OK;
    return cudaMallocFromPoolAsync(p, bytes, s->pool, st) == cudaSuccess ? MGB_OK : MGB_ERR_OUT_OF_MEMORY;
}

static Variant variant_of(const ContractionPlan &cp, int S) {
    return Variant(S, cp.form == MGB_FORM_OZAKI ? 1 : 0, is_complex(cp.compute_dtype) ? 1 : 0);
}

// Launches the emulated requests of slot k's batch; returns an mgb_status.
static int launch_emulated(mgb_server_s *s, size_t k) {
    Batch &b = s->slots[k];
    cudaStream_t st = s->streams[k];
    std::vector<uint64_t> off(b.emu.size());
    uint64_t total = 0;
    for (size_t i = 0; i < b.emu.size(); ++i) {
        off[i] = total;
        total += (b.emu[i].plan->cp.ws_bytes + 255) & ~uint64_t(255);
    }
    if (b.sel_cap < b.emu.size()) {
        if (b.sel_dev) cudaFree(b.sel_dev);
        if (b.sel_host) cudaFreeHost(b.sel_host);
        b.sel_dev = b.sel_host = nullptr;
        b.sel_cap = 0;
        const size_t cap = std::max<size_t>(b.emu.size(), 64);
        MGB_CUDA_CHECK(cudaMalloc((void **)&b.sel_dev, cap * 4));
        MGB_CUDA_CHECK(cudaMallocHost((void **)&b.sel_host, cap * 4));
        b.sel_cap = cap;
    }
    int rc = alloc_ws(s, &b.ws, total, st);
    if (rc) return rc;
    std::vector<OzBatchItem> items(b.emu.size());
    for (size_t i = 0; i < b.emu.size(); ++i)
        items[i] = {&b.emu[i].plan->cp, b.emu[i].A, b.emu[i].B, b.emu[i].C, (char *)b.ws + off[i]};
    int nv = 0;
    rc = ozaki_batch_launch(
        items, b.buf, st, b.sel_dev,
        [&]() -> int {  // the slice counts reach the host before any tensor-core launch
            MGB_CUDA_CHECK(cudaMemcpyAsync(b.sel_host, b.sel_dev, b.emu.size() * 4, cudaMemcpyDeviceToHost, st));
            b.chosen = take_event(s);
            MGB_CUDA_CHECK(cudaEventRecord(b.chosen, st));
            return MGB_OK;
        },
        [&](int S, bool exact, bool cx) -> int {
            if (nv >= kMaxVariants) return fail(MGB_ERR_UNSUPPORTED, "server: too many kernel variants in a batch");
            int32_t *snap = b.status_host + 1 + nv++;
            MGB_CUDA_CHECK(cudaMemcpyAsync(snap, device_status_ptr(), 4, cudaMemcpyDeviceToHost, st));
            cudaEvent_t e = take_event(s);
            MGB_CUDA_CHECK(cudaEventRecord(e, st));
            b.variant[Variant(S, exact ? 1 : 0, cx ? 1 : 0)] = {e, snap};
            return MGB_OK;
        });
    cudaFreeAsync(b.ws, st);  // stream-ordered: reusable once the batch has passed this point
    b.ws = nullptr;
    return rc;
}

// Launches one admitted batch on stream k. Requests that fail to launch are
// finished at once with their error.
static void launch_batch(mgb_server_s *s, size_t k, std::vector<Req> &reqs) {
    Batch &b = s->slots[k];
    cudaStream_t st = s->streams[k];
    for (auto &r : reqs)
        if (r.dep) cudaStreamWaitEvent(st, r.dep, 0);
    std::vector<Req> failed;
    for (auto &r : reqs) (r.plan->cp.form == MGB_FORM_PLAIN ? b.plain : b.emu).push_back(r);
    if (!b.emu.empty()) {
        if (int rc = launch_emulated(s, k)) {
            for (auto &r : b.emu) {
                r.status = rc;
                failed.push_back(r);
            }
            b.emu.clear();
            for (auto &kv : b.variant) give_event(s, kv.second.first);
            b.variant.clear();
            give_event(s, b.chosen);
            b.chosen = nullptr;
        }
    }
    std::vector<Req> ok;
    for (auto &r : b.plain) {
        // the plain form reads its operands in place and needs no workspace
        if (int rc = mgb_contract(r.plan, r.A, r.B, r.C, nullptr, 0, st)) {
            r.status = rc;
            failed.push_back(r);
            continue;
        }
        r.done = take_event(s);
        r.own_done = true;
        r.status_word = b.status_host;  // plain kernels have no bounded waits; the snapshot is taken below
        cudaEventRecord(r.done, st);
        ok.push_back(r);
    }
    b.plain.swap(ok);
    cudaMemcpyAsync(b.status_host, device_status_ptr(), 4, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(b.end, st);
    b.mapped = b.emu.empty();
    b.busy = true;
    ++s->batches;
    if (!failed.empty()) {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &r : failed) finish(s, r, r.status);
        s->cv_done.notify_all();
    }
}

// Retires what finished in slot k; returns true when something changed.
static bool retire(mgb_server_s *s, size_t k) {
    Batch &b = s->slots[k];
    if (!b.busy) return false;
    bool progressed = false;
    cudaStream_t st = s->streams[k];
    if (!b.mapped && cudaEventQuery(b.chosen) != cudaErrorNotReady) {
        // every emulated request now knows the launch that computes it;
        // adaptive ones that chose the plain form run again through mgb_contract
        bool redo = false;
        for (size_t i = 0; i < b.emu.size(); ++i) {
            Req &r = b.emu[i];
            const int S = b.sel_host[i];
            auto it = S > 0 ? b.variant.find(variant_of(r.plan->cp, S)) : b.variant.end();
            if (it != b.variant.end()) {
                r.done = it->second.first;
                r.status_word = it->second.second;
                continue;
            }
            void *ws = nullptr;
            int rc = alloc_ws(s, &ws, r.plan->cp.ws_bytes, st);
            if (rc == MGB_OK) rc = mgb_contract(r.plan, r.A, r.B, r.C, ws, r.plan->cp.ws_bytes, st);
            if (ws) cudaFreeAsync(ws, st);
            r.status = rc;
            r.done = take_event(s);
            r.own_done = true;
            r.status_word = b.status_host;
            cudaEventRecord(r.done, st);
            redo = true;
        }
        if (redo) {  // the batch now ends after the re-runs
            cudaMemcpyAsync(b.status_host, device_status_ptr(), 4, cudaMemcpyDeviceToHost, st);
            cudaEventRecord(b.end, st);
        }
        b.mapped = true;
        progressed = true;
    }
    // one by one: requests whose own launch has completed (the requests of
    // one variant share its event: each event is queried once per sweep)
    std::vector<std::pair<Req, int32_t>> done;
    std::vector<std::pair<cudaEvent_t, cudaError_t>> seen;
    auto query = [&](cudaEvent_t e) {
        for (auto &x : seen)
            if (x.first == e) return x.second;
        const cudaError_t q = cudaEventQuery(e);
        seen.push_back({e, q});
        return q;
    };
    auto sweep = [&](std::vector<Req> &v) {
        std::vector<Req> keep;
        for (auto &r : v) {
            cudaError_t q = r.done ? query(r.done) : cudaErrorNotReady;
            // own events of plain launches and re-runs: their status snapshot
            // is taken at the batch's end
            if (q == cudaSuccess && r.own_done && query(b.end) == cudaErrorNotReady) q = cudaErrorNotReady;
            if (q == cudaErrorNotReady) {
                keep.push_back(r);
                continue;
            }
            int32_t stv = r.status;
            if (stv == MGB_OK && q != cudaSuccess) stv = MGB_ERR_CUDA;
            // a bounded device wait gave up on this device since the word was
            // last cleared: the result of this request is suspect
            if (stv == MGB_OK && r.status_word && *r.status_word != 0) stv = MGB_ERR_DEVICE_TIMEOUT;
            done.push_back({r, stv});
            if (r.own_done) give_event(s, r.done);
        }
        v.swap(keep);
    };
    if (b.mapped) sweep(b.emu);
    sweep(b.plain);
    const bool all = b.mapped && b.emu.empty() && b.plain.empty() && cudaEventQuery(b.end) != cudaErrorNotReady;
    if (all) {
        for (auto &kv : b.variant) give_event(s, kv.second.first);
        b.variant.clear();
        give_event(s, b.chosen);
        b.chosen = nullptr;
        b.busy = false;
        progressed = true;
    }
    if (!done.empty()) {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &x : done) finish(s, x.first, x.second);
        s->cv_done.notify_all();
        progressed = true;
    }
    return progressed;
}

static void serve_loop(mgb_server_s *s) {
    cudaSetDevice(s->device);
    while (!s->stop.load()) {
        bool progressed = false;
        for (size_t k = 0; k < s->slots.size(); ++k) progressed |= retire(s, k);
        for (size_t k = 0; k < s->slots.size(); ++k) {
            if (s->slots[k].busy) continue;
            std::vector<Req> reqs;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                while (!s->pending.empty() && (int)reqs.size() < s->max_batch) {
                    Req &r = s->pending.front();
                    if (s->used + r.bytes > s->budget) break;  // wait for budget (FIFO)
                    s->used += r.bytes;
                    reqs.push_back(r);
                    s->pending.pop_front();
                }
            }
            if (reqs.empty()) break;
            launch_batch(s, k, reqs);
            progressed = true;
        }
        if (!progressed) {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
    }
}

extern "C" {

int mgb_server_create(mgb_server *server, uint64_t budget_bytes, int32_t nstreams, int32_t max_batch) {
    if (!server) return fail(MGB_ERR_ARGUMENT, "server output pointer is null");
    *server = nullptr;
    if (nstreams < 1 || nstreams > 64 || max_batch < 1) return fail(MGB_ERR_ARGUMENT, "server: bad stream/batch count");
    auto *s = new mgb_server_s();
    s->budget = budget_bytes;
    s->max_batch = max_batch;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaGetDevice");
    }
    if (!device_status_ptr()) {
        delete s;
        return fail(MGB_ERR_CUDA, "device status word unavailable");
    }
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if ((e = cudaMemPoolCreate(&s->pool, &props)) != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaMemPoolCreate");
    }
    uint64_t keep = budget_bytes;  // keep freed blocks for reuse instead of returning them
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    s->streams.resize(nstreams);
    s->slots.resize(nstreams);
    for (int i = 0; i < nstreams; ++i) {
        cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking);
        Batch &b = s->slots[i];
        cudaEventCreateWithFlags(&b.end, cudaEventDisableTiming);
        b.buf = ozaki_batch_buffers_create();
        if (cudaMallocHost((void **)&b.status_host, (1 + kMaxVariants) * 4) == cudaSuccess)
            std::memset(b.status_host, 0, (1 + kMaxVariants) * 4);
    }
    s->started = Clock::now();
    s->worker = std::thread(serve_loop, s);
    *server = s;
    return MGB_OK;
}

int mgb_server_submit(mgb_server server, mgb_plan plan, const void *A, const void *B, void *C,
                      uint64_t resident_bytes, void *dep_stream, int64_t *ticket) {
    if (!server || !plan || !ticket || plan->kind != PlanKind::Contraction)
        return fail(MGB_ERR_ARGUMENT, "server: bad submit arguments");
    Req r;
    r.plan = plan;
    r.A = A;
    r.B = B;
    r.C = C;
    r.bytes = resident_bytes + plan->cp.ws_bytes;
    r.dep = nullptr;
    r.t0 = Clock::now();
    std::lock_guard<std::mutex> lk(server->mu);
    r.ticket = server->next_ticket++;
    *ticket = r.ticket;
    ++server->submitted;
    if (r.bytes > server->budget) {
        ++server->rejected;
        server->finished[r.ticket] = MGB_ERR_OUT_OF_MEMORY;
        server->latency_ms.push_back(0.0);
        ++server->completed;
        return MGB_OK;  // the ticket reports MGB_ERR_OUT_OF_MEMORY
    }
    if (dep_stream) {
        r.dep = take_event(server);
        cudaEventRecord(r.dep, (cudaStream_t)dep_stream);
    }
    server->pending.push_back(r);
    server->cv_work.notify_one();
    return MGB_OK;
}

int mgb_server_wait(mgb_server server, int64_t ticket, double timeout_s, int32_t *status) {
    if (!server || !status) return fail(MGB_ERR_ARGUMENT, "server: null argument");
    std::unique_lock<std::mutex> lk(server->mu);
    auto pred = [&] { return server->finished.count(ticket) != 0; };
    if (timeout_s < 0) server->cv_done.wait(lk, pred);
    else if (!server->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
        return fail(MGB_ERR_DEVICE_TIMEOUT, "server: request not finished before the timeout");
    *status = server->finished[ticket];
    server->finished.erase(ticket);
    return MGB_OK;
}

int mgb_server_get_stats(mgb_server server, mgb_server_stats *out) {
    if (!server || !out) return fail(MGB_ERR_ARGUMENT, "server: null argument");
    std::lock_guard<std::mutex> lk(server->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = server->submitted;
    out->completed = server->completed;
    out->rejected = server->rejected;
    out->batches = server->batches;
    out->pending = server->pending.size();
    out->used_bytes = server->used;
    std::vector<double> v = server->latency_ms;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = v.back();
    }
    out->elapsed_s = std::chrono::duration<double>(Clock::now() - server->started).count();
    return MGB_OK;
}

int mgb_server_reset_stats(mgb_server server) {
    if (!server) return fail(MGB_ERR_ARGUMENT, "server: null argument");
    std::lock_guard<std::mutex> lk(server->mu);
    server->latency_ms.clear();
    server->submitted = server->completed = server->rejected = server->batches = 0;
    server->started = Clock::now();
    return MGB_OK;
}

int mgb_server_destroy(mgb_server server) {
    if (!server) return MGB_OK;
    {
        // let queued work finish so caller buffers are not written after return
        std::unique_lock<std::mutex> lk(server->mu);
        server->cv_done.wait_for(lk, std::chrono::seconds(600), [&] {
            bool idle = server->pending.empty();
            return idle && server->used == 0;
        });
    }
    server->stop.store(true);
    server->cv_work.notify_all();
    if (server->worker.joinable()) server->worker.join();
    for (size_t i = 0; i < server->streams.size(); ++i) {
        cudaStreamSynchronize(server->streams[i]);
        cudaStreamDestroy(server->streams[i]);
        Batch &b = server->slots[i];
        cudaEventDestroy(b.end);
        for (auto &kv : b.variant) cudaEventDestroy(kv.second.first);
        if (b.chosen) cudaEventDestroy(b.chosen);
        ozaki_batch_buffers_destroy(b.buf);
        if (b.sel_dev) cudaFree(b.sel_dev);
        if (b.sel_host) cudaFreeHost(b.sel_host);
        if (b.status_host) cudaFreeHost(b.status_host);
    }
    for (auto e : server->event_pool) cudaEventDestroy(e);
    if (server->pool) cudaMemPoolDestroy(server->pool);
    delete server;
    return MGB_OK;
}

}  // extern "C"
