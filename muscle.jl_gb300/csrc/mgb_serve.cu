// Serving loop: contractions submitted as they arrive, admitted against a
// device-memory byte budget, and dispatched with continuous batching onto
// several streams so that requests arriving while others run overlap with
// them on the GPU.
//
// A scheduler thread owned by the server repeatedly
//   1. retires finished batches (event query), releasing their budget and
//      waking the waiters of their requests;
//   2. admits queued requests in arrival order while the bytes of admitted,
//      unfinished requests (operands, output and workspace) stay within the
//      budget, and launches them as one batch on an idle stream: every
//      request's workspace comes from the server's stream-ordered memory pool
//      (cudaMallocAsync / cudaFreeAsync, no device synchronisation);
//   3. sleeps briefly when there is nothing to do.
// Latency is measured from submission to the moment the scheduler sees the
// request's batch finished. Plans and device buffers stay owned by the caller,
// who must keep them alive until the request is finished.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
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
};

struct Batch {
    std::vector<Req> reqs;
    cudaEvent_t done = nullptr;
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
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::atomic<bool> stop{false};
    std::thread worker;
    int64_t next_ticket = 1;
    uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0;
    double busy_ms = 0;
    Clock::time_point started;
};

using namespace mgb;

static cudaEvent_t take_event(mgb_server_s *s) {
    if (!s->event_pool.empty()) {
        cudaEvent_t e = s->event_pool.back();
        s->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

static void finish(mgb_server_s *s, const Req &r, int32_t status) {
    // caller holds s->mu
    s->finished[r.ticket] = status;
    s->latency_ms.push_back(std::chrono::duration<double, std::milli>(Clock::now() - r.t0).count());
    s->used -= r.bytes;
    ++s->completed;
    if (r.dep) s->event_pool.push_back(r.dep);
}

static void serve_loop(mgb_server_s *s) {
    cudaSetDevice(s->device);
    while (!s->stop.load()) {
        bool progressed = false;
        // 1. retire finished batches
        for (size_t k = 0; k < s->slots.size(); ++k) {
            Batch &b = s->slots[k];
            if (!b.busy) continue;
            cudaError_t q = cudaEventQuery(b.done);
            if (q == cudaErrorNotReady) continue;
            std::lock_guard<std::mutex> lk(s->mu);
            for (auto &r : b.reqs) finish(s, r, q == cudaSuccess ? MGB_OK : MGB_ERR_CUDA);
            b.reqs.clear();
            b.busy = false;
            progressed = true;
            s->cv_done.notify_all();
        }
        // 2. admit and launch on idle streams
        for (size_t k = 0; k < s->slots.size(); ++k) {
            Batch &b = s->slots[k];
            if (b.busy) continue;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                while (!s->pending.empty() && (int)b.reqs.size() < s->max_batch) {
                    Req &r = s->pending.front();
                    if (s->used + r.bytes > s->budget) break;  // wait for budget (FIFO)
                    s->used += r.bytes;
                    b.reqs.push_back(r);
                    s->pending.pop_front();
                }
            }
            if (b.reqs.empty()) break;
            cudaStream_t st = s->streams[k];
            std::vector<std::pair<size_t, int32_t>> failed;
            for (size_t i = 0; i < b.reqs.size(); ++i) {
                Req &r = b.reqs[i];
                if (r.dep) cudaStreamWaitEvent(st, r.dep, 0);
                void *ws = nullptr;
                const uint64_t wsb = r.plan->cp.ws_bytes;
                if (wsb && cudaMallocFromPoolAsync(&ws, wsb, s->pool, st) != cudaSuccess) {
                    failed.push_back({i, MGB_ERR_OUT_OF_MEMORY});
                    continue;
                }
                int rc = mgb_contract(r.plan, r.A, r.B, r.C, ws, wsb, st);
                if (ws) cudaFreeAsync(ws, st);
                if (rc) failed.push_back({i, rc});
            }
            cudaEventRecord(b.done, st);
            b.busy = true;
            ++s->batches;
            progressed = true;
            if (!failed.empty()) {
                // finished (with an error) right away; the rest completes with the batch
                std::lock_guard<std::mutex> lk(s->mu);
                std::vector<Req> keep;
                size_t fi = 0;
                for (size_t i = 0; i < b.reqs.size(); ++i) {
                    if (fi < failed.size() && failed[fi].first == i) {
                        finish(s, b.reqs[i], failed[fi].second);
                        ++fi;
                    } else {
                        keep.push_back(b.reqs[i]);
                    }
                }
                b.reqs.swap(keep);
                s->cv_done.notify_all();
            }
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
        cudaEventCreateWithFlags(&s->slots[i].done, cudaEventDisableTiming);
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
        cudaEventDestroy(server->slots[i].done);
    }
    for (auto e : server->event_pool) cudaEventDestroy(e);
    if (server->pool) cudaMemPoolDestroy(server->pool);
    delete server;
    return MGB_OK;
}

}  // extern "C"
