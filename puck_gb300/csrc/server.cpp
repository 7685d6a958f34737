// Serving loop: continuous batching of search requests on CUDA graphs.
//
// Requests (n queries each, their own top-k) are queued by pgpu_server_submit.
// A scheduler thread owns S slots; each slot has its own scratch, stream, pinned
// staging buffers and, per (batch-size bucket, top-k), a CUDA graph holding the
// whole pass: query upload, the search kernels, result download. Whenever a
// slot is free the scheduler fills it from the head of the queue with requests of
// the same top-k (several requests share one batch), pads the batch to the next
// bucket with copies of its first query, and launches the slot's graph on the
// slot's stream. Slots run concurrently, so requests that arrive while others are
// on the GPU are admitted as soon as a slot frees up and their work overlaps on
// the device. The number of slots is set by a scratch-memory budget. Each query's
// result depends only on that query, so a request's results are bit-identical
// alone or in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pgpu_internal.h"

struct pgpu_index;  // defined in capi.cpp; the server reads its device index and config

namespace pgpu {
const DeviceIndex& index_device(const pgpu_index* h);
const SearchConfig& index_config(const pgpu_index* h);
int index_device_ordinal(const pgpu_index* h);
}  // namespace pgpu

namespace {

using clock_type = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    uint32_t n = 0, topk = 0;
    const float* q = nullptr;
    float* dist = nullptr;
    uint32_t* ids = nullptr;
    int32_t* status = nullptr;
    int state = 0;  // 0 queued, 1 on the GPU, 2 done
    int rc = 0;
    clock_type::time_point t_submit, t_done;
};

struct Slot {
    pgpu::Scratch s;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    float* h_q = nullptr;
    float* h_dist = nullptr;
    uint32_t* h_ids = nullptr;
    int32_t* h_status = nullptr;
    float* d_q = nullptr;
    float* d_dist = nullptr;
    uint32_t* d_ids = nullptr;
    int32_t* d_status = nullptr;
    std::map<std::pair<uint32_t, uint32_t>, cudaGraphExec_t> graphs;  // (bucket, topk)
    std::vector<Request*> reqs;
    uint32_t used = 0, topk = 0;
    bool busy = false;
};

}  // namespace

struct pgpu_server {
    pgpu_index* index = nullptr;
    int device = 0;
    uint32_t cap = 0, topk_max = 0, d = 0;
    std::vector<uint32_t> buckets;
    std::vector<std::unique_ptr<Slot>> slots;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t next_ticket = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread sched;
    bool stop = false;
    int sched_error = 0;
    std::string sched_msg;
    pgpu_server_stats stats{};
};

namespace {

void free_slot(Slot* sl) {
    for (auto& kv : sl->graphs) cudaGraphExecDestroy(kv.second);
    sl->graphs.clear();
    pgpu::free_scratch(&sl->s);
    if (sl->stream) cudaStreamDestroy(sl->stream);
    if (sl->done) cudaEventDestroy(sl->done);
    void* hp[] = {sl->h_q, sl->h_dist, sl->h_ids, sl->h_status};
    for (void* p : hp)
        if (p) cudaFreeHost(p);
    void* dp[] = {sl->d_q, sl->d_dist, sl->d_ids, sl->d_status};
    for (void* p : dp)
        if (p) cudaFree(p);
}

uint64_t staging_bytes(uint32_t cap, uint32_t d, uint32_t kmax) {
    return (uint64_t)cap * (d * 4ull + kmax * 8ull + 4ull);
}

int alloc_slot(pgpu_server* sv, Slot* sl, std::string* err) {
    const auto& ix = pgpu::index_device(sv->index);
    const auto& cfg = pgpu::index_config(sv->index);
    if (int rc = pgpu::alloc_scratch(ix, cfg, sv->cap, &sl->s, err)) return rc;
    const uint64_t C = sv->cap, d = sv->d, K = sv->topk_max;
    cudaError_t e = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl->h_q, 4 * C * d);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl->h_dist, 4 * C * K);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl->h_ids, 4 * C * K);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&sl->h_status, 4 * C);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl->d_q, 4 * C * d);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl->d_dist, 4 * C * K);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl->d_ids, 4 * C * K);
    if (e == cudaSuccess) e = cudaMalloc((void**)&sl->d_status, 4 * C);
    if (e != cudaSuccess) {
        *err = std::string("server slot allocation: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
    }
    return PGPU_OK;
}

// Enqueues one pass (upload, kernels, download) of `bucket` queries on the slot.
cudaError_t enqueue_pass(pgpu_server* sv, Slot* sl, uint32_t bucket, uint32_t topk,
                         const char** what) {
    const auto& ix = pgpu::index_device(sv->index);
    const auto& cfg = pgpu::index_config(sv->index);
    cudaError_t e = cudaMemcpyAsync(sl->d_q, sl->h_q, 4ull * bucket * sv->d, cudaMemcpyHostToDevice,
                                    sl->stream);
    if (e != cudaSuccess) {
        *what = "query upload";
        return e;
    }
    int launched = 0;
    e = pgpu::run_pipeline(ix, cfg, sl->s, bucket, sl->d_q, topk, sl->d_dist, sl->d_ids,
                           sl->d_status, sl->stream, nullptr, &launched, what);
    if (e != cudaSuccess) return e;
    *what = "result download";
    if ((e = cudaMemcpyAsync(sl->h_dist, sl->d_dist, 4ull * bucket * topk, cudaMemcpyDeviceToHost,
                             sl->stream)))
        return e;
    if ((e = cudaMemcpyAsync(sl->h_ids, sl->d_ids, 4ull * bucket * topk, cudaMemcpyDeviceToHost,
                             sl->stream)))
        return e;
    return cudaMemcpyAsync(sl->h_status, sl->d_status, 4ull * bucket, cudaMemcpyDeviceToHost,
                           sl->stream);
}

// The slot's graph for (bucket, topk), captured on first use.
cudaError_t slot_graph(pgpu_server* sv, Slot* sl, uint32_t bucket, uint32_t topk,
                       cudaGraphExec_t* out, const char** what) {
    auto key = std::make_pair(bucket, topk);
    auto it = sl->graphs.find(key);
    if (it != sl->graphs.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    // one uncaptured pass first: kernels set their launch attributes on first use
    cudaError_t e = enqueue_pass(sv, sl, bucket, topk, what);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sl->stream);
    if (e != cudaSuccess) return e;
    cudaGraph_t g = nullptr;
    *what = "graph capture";
    if ((e = cudaStreamBeginCapture(sl->stream, cudaStreamCaptureModeThreadLocal))) return e;
    cudaError_t ep = enqueue_pass(sv, sl, bucket, topk, what);
    e = cudaStreamEndCapture(sl->stream, &g);
    if (ep != cudaSuccess) e = ep;
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return e;
    }
    cudaGraphExec_t ex = nullptr;
    *what = "graph instantiate";
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return e;
    sl->graphs[key] = ex;
    sv->stats.graphs_captured += 1;
    *out = ex;
    return cudaSuccess;
}

uint32_t bucket_for(const pgpu_server* sv, uint32_t n) {
    for (uint32_t b : sv->buckets)
        if (b >= n) return b;
    return sv->cap;
}

void deliver(pgpu_server* sv, Slot* sl) {
    const auto now = clock_type::now();
    uint32_t off = 0;
    for (Request* r : sl->reqs) {
        const uint32_t k = sl->topk;
        for (uint32_t i = 0; i < r->n; ++i) {
            std::memcpy(r->dist + (uint64_t)i * r->topk, sl->h_dist + (uint64_t)(off + i) * k,
                        4ull * r->topk);
            std::memcpy(r->ids + (uint64_t)i * r->topk, sl->h_ids + (uint64_t)(off + i) * k,
                        4ull * r->topk);
        }
        if (r->status) std::memcpy(r->status, sl->h_status + off, 4ull * r->n);
        off += r->n;
        r->state = 2;
        r->t_done = now;
        const double us =
            std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
        sv->stats.requests_done += 1;
        sv->stats.queries_done += r->n;
        sv->stats.latency_us_sum += us;
    }
    sl->reqs.clear();
    sl->busy = false;
}

void fail_all(pgpu_server* sv, int rc, const std::string& msg) {
    sv->sched_error = rc;
    sv->sched_msg = msg;
    for (auto& kv : sv->reqs)
        if (kv.second->state != 2) {
            kv.second->state = 2;
            kv.second->rc = rc;
        }
    sv->queue.clear();
}

void scheduler(pgpu_server* sv) {
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    while (true) {
        bool any_busy = false, delivered = false;
        for (auto& sp : sv->slots) {
            Slot* sl = sp.get();
            if (!sl->busy) continue;
            cudaError_t q = cudaEventQuery(sl->done);
            if (q == cudaSuccess) {
                deliver(sv, sl);
                delivered = true;
            } else if (q == cudaErrorNotReady) {
                any_busy = true;
            } else {
                fail_all(sv, PGPU_E_CUDA, std::string("search pass: ") + cudaGetErrorString(q));
                sl->busy = false;
                delivered = true;
            }
        }
        if (delivered) sv->cv_done.notify_all();
        // admit queued requests into free slots
        for (auto& sp : sv->slots) {
            Slot* sl = sp.get();
            if (sl->busy || sv->queue.empty() || sv->sched_error) continue;
            const uint32_t k = sv->queue.front()->topk;
            uint32_t used = 0;
            while (!sv->queue.empty() && sv->queue.front()->topk == k &&
                   used + sv->queue.front()->n <= sv->cap) {
                Request* r = sv->queue.front();
                sv->queue.pop_front();
                std::memcpy(sl->h_q + (uint64_t)used * sv->d, r->q, 4ull * r->n * sv->d);
                used += r->n;
                r->state = 1;
                sl->reqs.push_back(r);
            }
            const uint32_t bucket = bucket_for(sv, used);
            for (uint32_t i = used; i < bucket; ++i)  // pad with copies of the first query
                std::memcpy(sl->h_q + (uint64_t)i * sv->d, sl->h_q, 4ull * sv->d);
            sl->used = used;
            sl->topk = k;
            cudaGraphExec_t g = nullptr;
            const char* what = "";
            cudaError_t e = slot_graph(sv, sl, bucket, k, &g, &what);
            if (e == cudaSuccess) e = cudaGraphLaunch(g, sl->stream);
            if (e == cudaSuccess) e = cudaEventRecord(sl->done, sl->stream);
            if (e != cudaSuccess) {
                fail_all(sv, PGPU_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
                sl->reqs.clear();
                sv->cv_done.notify_all();
                continue;
            }
            sl->busy = true;
            any_busy = true;
            sv->stats.batches += 1;
            sv->stats.graph_launches += 1;
            sv->stats.padded_queries += bucket - used;
        }
        if (sv->stop && sv->queue.empty() && !any_busy) break;
        if (any_busy) {
            // results are polled: release the lock briefly so submitters get in
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        } else if (sv->queue.empty() && !sv->stop) {
            sv->cv_work.wait(lk);
        }
    }
}

int sfail(int code, const std::string& msg) { return pgpu::set_last_error(code, msg); }

}  // namespace

extern "C" {

void pgpu_server_params_default(pgpu_server_params* p) {
    p->max_batch = 1024;
    p->scratch_budget_bytes = 1ull << 30;
    p->max_slots = 4;
}

int pgpu_server_create(pgpu_index* index, const pgpu_server_params* params, pgpu_server** out) {
    if (index == nullptr || out == nullptr) return sfail(PGPU_E_INVALID, "null argument");
    pgpu_server_params p;
    if (params) p = *params;
    else pgpu_server_params_default(&p);
    if (p.max_batch == 0 || p.max_slots == 0) return sfail(PGPU_E_INVALID, "max_batch and max_slots must be positive");
    const auto& ix = pgpu::index_device(index);
    const auto& cfg = pgpu::index_config(index);
    auto sv = std::make_unique<pgpu_server>();
    sv->index = index;
    sv->device = pgpu::index_device_ordinal(index);
    sv->cap = p.max_batch;
    sv->topk_max = cfg.topk_max;
    sv->d = ix.qdim;  // floats per caller query
    for (uint32_t b = 32; b < sv->cap; b <<= 1) sv->buckets.push_back(b);
    sv->buckets.push_back(sv->cap);
    const uint64_t per_slot = pgpu::scratch_bytes(ix, cfg, sv->cap) +
                              staging_bytes(sv->cap, sv->d, sv->topk_max);
    const uint64_t fit = p.scratch_budget_bytes / per_slot;
    if (fit == 0)
        return sfail(PGPU_E_LIMIT, "scratch budget below one slot (" + std::to_string(per_slot) +
                                       " bytes for max_batch " + std::to_string(sv->cap) + ")");
    const uint32_t nslots = (uint32_t)std::min<uint64_t>(fit, p.max_slots);
    cudaSetDevice(sv->device);
    for (uint32_t i = 0; i < nslots; ++i) {
        auto sl = std::make_unique<Slot>();
        std::string err;
        if (int rc = alloc_slot(sv.get(), sl.get(), &err)) {
            free_slot(sl.get());
            for (auto& s2 : sv->slots) free_slot(s2.get());
            return sfail(rc, err);
        }
        sv->slots.push_back(std::move(sl));
    }
    sv->stats.slots = nslots;
    sv->stats.slot_bytes = per_slot;
    pgpu_server* raw = sv.release();
    raw->sched = std::thread(scheduler, raw);
    *out = raw;
    return PGPU_OK;
}

int pgpu_server_submit(pgpu_server* sv, uint32_t n, const float* query, uint32_t topk,
                       float* distance, uint32_t* labels, int32_t* status, uint64_t* ticket) {
    if (sv == nullptr || query == nullptr || distance == nullptr || labels == nullptr ||
        ticket == nullptr)
        return sfail(PGPU_E_INVALID, "null argument");
    if (n == 0 || n > sv->cap)
        return sfail(PGPU_E_LIMIT, "a request holds 1.." + std::to_string(sv->cap) + " queries");
    if (topk == 0 || topk > sv->topk_max)
        return sfail(PGPU_E_INVALID, "topk should <= topk, topk = " + std::to_string(sv->topk_max));
    auto r = std::make_unique<Request>();
    r->n = n;
    r->topk = topk;
    r->q = query;
    r->dist = distance;
    r->ids = labels;
    r->status = status;
    r->t_submit = clock_type::now();
    {
        std::lock_guard<std::mutex> g(sv->mu);
        if (sv->sched_error) return sfail(sv->sched_error, sv->sched_msg);
        r->ticket = sv->next_ticket++;
        *ticket = r->ticket;
        sv->queue.push_back(r.get());
        sv->reqs[r->ticket] = std::move(r);
        sv->stats.requests_submitted += 1;
    }
    sv->cv_work.notify_one();
    return PGPU_OK;
}

int pgpu_server_wait(pgpu_server* sv, uint64_t ticket, int32_t timeout_ms, double* latency_us) {
    if (sv == nullptr) return sfail(PGPU_E_INVALID, "null server");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return sfail(PGPU_E_INVALID, "unknown ticket");
    Request* r = it->second.get();
    auto ready = [&] { return r->state == 2; };
    if (timeout_ms < 0) {
        sv->cv_done.wait(lk, ready);
    } else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return sfail(PGPU_E_TIMEOUT, "request not finished within the timeout");
    }
    const int rc = r->rc;
    if (latency_us)
        *latency_us = std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
    sv->reqs.erase(it);
    if (rc) return sfail(rc, sv->sched_msg);
    return PGPU_OK;
}

int pgpu_server_stats_get(pgpu_server* sv, pgpu_server_stats* out) {
    if (sv == nullptr || out == nullptr) return sfail(PGPU_E_INVALID, "null argument");
    std::lock_guard<std::mutex> g(sv->mu);
    *out = sv->stats;
    return PGPU_OK;
}

int pgpu_server_destroy(pgpu_server* sv) {
    if (sv == nullptr) return PGPU_OK;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->sched.joinable()) sv->sched.join();
    cudaSetDevice(sv->device);
    for (auto& sl : sv->slots) {
        cudaStreamSynchronize(sl->stream);
        free_slot(sl.get());
    }
    delete sv;
    return PGPU_OK;
}

}  // extern "C"
