// cj_serve.cpp -- a parse server with continuous batching (C ABI).
//
// No counterpart in the reference, which parses one document per blocking
// call.  Requests (one standard or JSON-Lines document each) are queued by
// any host thread.  One scheduler thread turns the queue into batches and
// keeps up to `slots` batches in flight, each on its own context (device
// arena + stream):
//
//   - whenever a slot is free, it takes the oldest waiting request's kind
//     (standard or JSON Lines), and admits further waiting requests of that
//     kind, oldest first, while the batch stays within max_batch_docs and the
//     slot's share of the device-memory budget (memory_budget / slots, with
//     the per-byte arena cost of a batch); then stages the batch (H2D on the
//     slot's stream) and launches it;
//   - while one slot's kernels run, the next batch is staged on another, so
//     copies and kernels of consecutive batches overlap on the device;
//   - a finished slot hands every request its verdict and its result in the
//     reference layout and is free again.
// Requests that arrive while batches are in flight join the next batch as
// soon as a slot frees up.  Every request is parsed as an independent
// document, so its result is the same alone and in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cj_device.cuh"
#include "cujson_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

// Device bytes one document of `size` bytes adds to a batch arena: input
// padded to 1 KiB, int32 positions and pair row, 8-byte bracket records and
// 4-byte spine slots per chunk-aligned byte, the int32 result layout, region
// tables and work list (104 bytes per region of the smallest size), the emit
// masks (half a byte per input byte and 8 KiB per document); times the arena's
// 1/8 growth headroom.
uint64_t doc_device_bytes(size_t size)
{
    const uint64_t b = size;
    const uint64_t chunked = (b + 511) / 512 * 512 + 512;
    const uint64_t regions = b / ((uint64_t)cj::kRegionStepsAllowed[0] * cj::kStepBytes) + 2;
    const uint64_t raw = (b + 1024) + 8 * (b + 1) + 8 * chunked + 4 * chunked + 4 * (2 * b + 4) +
                         104 * regions + b / 2 + 8192 + 64;
    return raw + raw / 8;
}

struct Request {
    uint64_t id = 0;
    const uint8_t* data = nullptr;
    size_t size = 0;
    bool lines = false;
    Clock::time_point t_submit, t_done;
    bool done = false;
    cj_parse_info info{};
    std::vector<int32_t> result;   // reference layout
};

struct Slot {
    cj_context* ctx = nullptr;
    cudaEvent_t done_ev = nullptr;
    bool busy = false;
    std::vector<std::shared_ptr<Request>> reqs;
    int32_t* pinned_out = nullptr;   // layouts of the batch in flight
    size_t pinned_cap = 0;
};

}  // namespace

struct cj_server {
    cj_server_config cfg{};
    uint64_t slot_budget = 0;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> live;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    // statistics
    uint64_t batches = 0, docs = 0, bytes = 0, max_batch = 0, peak_admitted_bytes = 0;
    cj_status fault = CJ_OK;
};

namespace {

void fail_all(cj_server* s, std::vector<std::shared_ptr<Request>>& reqs, cj_status st)
{
    const auto now = Clock::now();
    for (auto& r : reqs) {
        r->info = cj_parse_info{};
        r->info.status = st;
        r->t_done = now;
        r->done = true;
    }
    s->cv_done.notify_all();
}

// Stage and launch one batch on a free slot (called without the lock held).
cj_status launch(cj_server* s, Slot& sl)
{
    const size_t n = sl.reqs.size();
    std::vector<const uint8_t*> ptrs(n);
    std::vector<size_t> sizes(n);
    for (size_t i = 0; i < n; i++) {
        ptrs[i] = sl.reqs[i]->data;
        sizes[i] = sl.reqs[i]->size;
    }
    cj_status st = cj_stage_batch(sl.ctx, ptrs.data(), sizes.data(), n, sl.reqs[0]->lines ? 1 : 0);
    if (!st) st = cj_run_staged(sl.ctx);
    if (!st && cudaEventRecord(sl.done_ev, (cudaStream_t)cj_context_stream(sl.ctx)) != cudaSuccess)
        st = CJ_ERR_CUDA;
    return st;
}

// Collect a finished slot's results into its requests.
cj_status complete(cj_server* s, Slot& sl)
{
    const size_t n = sl.reqs.size();
    std::vector<int32_t> status(n), depth(n);
    std::vector<int64_t> S(n), off(n + 1);
    cj_status st = cj_batch_info(sl.ctx, status.data(), S.data(), depth.data(), off.data(), n);
    if (st) return st;
    const size_t total = (size_t)off[n];
    if (total > sl.pinned_cap) {
        if (sl.pinned_out) cudaFreeHost(sl.pinned_out);
        sl.pinned_out = nullptr;
        sl.pinned_cap = 0;
        const size_t want = total + total / 4 + 1024;
        if (cudaMallocHost((void**)&sl.pinned_out, want * sizeof(int32_t)) != cudaSuccess)
            return CJ_ERR_OUT_OF_MEMORY;
        sl.pinned_cap = want;
    }
    st = cj_copy_batch_result(sl.ctx, sl.pinned_out, sl.pinned_cap);
    if (st) return st;
    const auto now = Clock::now();
    for (size_t i = 0; i < n; i++) {
        Request& r = *sl.reqs[i];
        r.info = cj_parse_info{};
        r.info.status = status[i];
        r.info.n_structural = S[i];
        r.info.max_depth = depth[i];
        r.info.n_segments = 1;
        if (status[i] == CJ_OK)
            r.result.assign(sl.pinned_out + off[i], sl.pinned_out + off[i + 1]);
        r.t_done = now;
    }
    return CJ_OK;
}

void worker_loop(cj_server* s)
{
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        bool progress = false;
        // 1. finished slots
        for (Slot& sl : s->slots) {
            if (!sl.busy) continue;
            if (cudaEventQuery(sl.done_ev) == cudaErrorNotReady) continue;
            lk.unlock();
            cj_status st = complete(s, sl);
            lk.lock();
            if (st) {
                fail_all(s, sl.reqs, st);
                if (!s->fault) s->fault = st;
            } else {
                for (auto& r : sl.reqs) r->done = true;
                s->cv_done.notify_all();
            }
            sl.reqs.clear();
            sl.busy = false;
            progress = true;
        }
        // 2. a free slot takes the next batch
        if (!s->queue.empty()) {
            for (Slot& sl : s->slots) {
                if (sl.busy || s->queue.empty()) continue;
                const bool lines = s->queue.front()->lines;
                uint64_t need = 0;
                for (auto it = s->queue.begin(); it != s->queue.end() && sl.reqs.size() < s->cfg.max_batch_docs;) {
                    Request& r = **it;
                    if (r.lines != lines) { ++it; continue; }
                    const uint64_t b = doc_device_bytes(r.size);
                    if (!sl.reqs.empty() && need + b > s->slot_budget) break;
                    need += b;
                    sl.reqs.push_back(*it);
                    it = s->queue.erase(it);
                }
                s->batches++;
                s->docs += sl.reqs.size();
                s->max_batch = std::max<uint64_t>(s->max_batch, sl.reqs.size());
                s->peak_admitted_bytes = std::max<uint64_t>(s->peak_admitted_bytes, need);
                for (auto& r : sl.reqs) s->bytes += r->size;
                sl.busy = true;
                lk.unlock();
                cj_status st = launch(s, sl);
                lk.lock();
                if (st) {
                    fail_all(s, sl.reqs, st);
                    sl.reqs.clear();
                    sl.busy = false;
                    if (!s->fault) s->fault = st;
                }
                progress = true;
            }
        }
        bool any_busy = false;
        for (Slot& sl : s->slots) any_busy |= sl.busy;
        if (s->stop && s->queue.empty() && !any_busy) break;
        if (!progress) {
            if (any_busy) s->cv_work.wait_for(lk, std::chrono::microseconds(20));
            else s->cv_work.wait(lk, [s] { return s->stop || !s->queue.empty(); });
        }
    }
}

}  // namespace

extern "C" {

cj_status cj_server_create(const cj_server_config* cfg, cj_server** out)
{
    if (!cfg || !out) return CJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cj_server* s = new cj_server();
    s->cfg = *cfg;
    if (s->cfg.slots == 0) s->cfg.slots = 2;
    if (s->cfg.slots > 8) s->cfg.slots = 8;
    if (s->cfg.max_batch_docs == 0) s->cfg.max_batch_docs = 1024;
    if (s->cfg.memory_budget == 0) s->cfg.memory_budget = 16ull << 30;
    s->slot_budget = s->cfg.memory_budget / s->cfg.slots;
    s->slots.resize(s->cfg.slots);
    for (Slot& sl : s->slots) {
        cj_status st = cj_context_create(s->cfg.device, &sl.ctx);
        // the slots' streams share the GPU: a dependent kernel of one slot
        // waiting on its SMs would hold resources the other slot's kernels need
        if (!st) st = cj_context_set_dependent_launch(sl.ctx, 0);
        if (!st && cudaEventCreateWithFlags(&sl.done_ev, cudaEventDisableTiming) != cudaSuccess) st = CJ_ERR_CUDA;
        if (st) {
            cj_server_destroy(s);
            return st;
        }
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return CJ_OK;
}

void cj_server_destroy(cj_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (Slot& sl : s->slots) {
        if (sl.done_ev) cudaEventDestroy(sl.done_ev);
        if (sl.pinned_out) cudaFreeHost(sl.pinned_out);
        if (sl.ctx) cj_context_destroy(sl.ctx);
    }
    delete s;
}

cj_status cj_server_submit(cj_server* s, const uint8_t* data, size_t size, int lines_mode, uint64_t* ticket)
{
    if (!s || !data || size == 0 || !ticket) return CJ_ERR_INVALID_ARGUMENT;
    if (size > CJ_MAX_INPUT_BYTES) return CJ_ERR_TOO_LARGE;
    if (doc_device_bytes(size) > s->slot_budget) return CJ_ERR_TOO_LARGE;   // would never be admitted
    auto r = std::make_shared<Request>();
    r->data = data;
    r->size = size;
    r->lines = lines_mode != 0;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> g(s->mu);
        r->id = s->next_id++;
        s->live[r->id] = r;
        s->queue.push_back(r);
    }
    s->cv_work.notify_one();
    *ticket = r->id;
    return CJ_OK;
}

cj_status cj_server_wait(cj_server* s, uint64_t ticket, int64_t timeout_ms, cj_parse_info* info,
                         double* latency_s)
{
    if (!s) return CJ_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->live.find(ticket);
    if (it == s->live.end()) return CJ_ERR_INVALID_ARGUMENT;
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return CJ_ERR_TIMEOUT;
    if (info) *info = r->info;
    if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    return CJ_OK;
}

cj_status cj_server_take(cj_server* s, uint64_t ticket, int32_t* host_out, size_t out_cap)
{
    if (!s) return CJ_ERR_INVALID_ARGUMENT;
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->live.find(ticket);
        if (it == s->live.end() || !it->second->done) return CJ_ERR_INVALID_ARGUMENT;
        r = it->second;
        if (host_out && r->result.size() > out_cap) return CJ_ERR_CAPACITY;
        s->live.erase(it);
    }
    if (host_out && !r->result.empty()) memcpy(host_out, r->result.data(), r->result.size() * sizeof(int32_t));
    return (cj_status)r->info.status;
}

cj_status cj_server_get_stats(cj_server* s, cj_server_stats* out)
{
    if (!s || !out) return CJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    out->batches = s->batches;
    out->docs = s->docs;
    out->bytes = s->bytes;
    out->max_batch_docs = s->max_batch;
    out->peak_admitted_bytes = s->peak_admitted_bytes;
    uint64_t dev = 0;
    for (Slot& sl : s->slots) dev += cj_context_device_bytes(sl.ctx);
    out->device_bytes = dev;
    out->fault = s->fault;
    return CJ_OK;
}

cj_status cj_server_replay(cj_server* s, const uint8_t* const* docs, const size_t* sizes, const int32_t* lines,
                           const double* arrival_s, size_t n, int32_t* status, double* latency_s,
                           double* makespan_s)
{
    if (!s || !docs || !sizes || !arrival_s || n == 0) return CJ_ERR_INVALID_ARGUMENT;
    std::vector<uint64_t> tickets(n, 0);
    std::vector<cj_status> sub(n, CJ_OK);
    const auto t0 = Clock::now();
    for (size_t i = 0; i < n; i++) {
        const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
        while (Clock::now() < due) {
            const auto left = due - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
        }
        sub[i] = cj_server_submit(s, docs[i], sizes[i], lines ? lines[i] : 0, &tickets[i]);
    }
    Clock::time_point last = t0;
    for (size_t i = 0; i < n; i++) {
        if (sub[i]) {
            if (status) status[i] = sub[i];
            if (latency_s) latency_s[i] = 0.0;
            continue;
        }
        cj_parse_info info;
        double lat = 0.0;
        cj_status st = cj_server_wait(s, tickets[i], -1, &info, &lat);
        {
            std::lock_guard<std::mutex> g(s->mu);
            auto it = s->live.find(tickets[i]);
            if (it != s->live.end()) {
                last = std::max(last, it->second->t_done);
                s->live.erase(it);
            }
        }
        if (status) status[i] = st ? st : info.status;
        if (latency_s) latency_s[i] = lat;
    }
    if (makespan_s) *makespan_s = std::chrono::duration<double>(last - t0).count();
    return CJ_OK;
}

}  // extern "C"
