// extern "C" entry points of libpuck_gb300 (declared in include/puck_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pgpu_internal.h"

struct pgpu_index {
    int device = 0;
    pgpu::DeviceIndex ix;
    pgpu::Scratch s;
    pgpu::SearchConfig cfg;
    uint32_t max_batch = 8192;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    // staging for host-buffer searches
    float* d_qin = nullptr;
    float* d_dist = nullptr;
    uint32_t* d_ids = nullptr;
    int32_t* d_status = nullptr;
    uint32_t stage_topk = 0;
    uint64_t kernels = 0, records = 0, cells = 0;
    uint64_t walk_counters[pgpu::kNumWalkCounters] = {};
    // optional per-stage timing with CUDA events on the launching stream
    bool profiling = false;
    cudaEvent_t ev[PGPU_NUM_STAGES + 1] = {};
    float stage_ms[PGPU_NUM_STAGES] = {};
    bool stage_pending = false;
    pgpu::RealtimeHost rt;  // host mirrors of the realtime insert lists
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

void free_staging(pgpu_index* h) {
    void* ptrs[] = {h->d_qin, h->d_dist, h->d_ids, h->d_status};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    h->d_qin = nullptr;
    h->d_dist = nullptr;
    h->d_ids = nullptr;
    h->d_status = nullptr;
    h->stage_topk = 0;
}

template <class T>
cudaError_t alloc(T** p, uint64_t count, uint64_t* bytes) {
    const size_t sz = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc((void**)p, sz);
    if (e == cudaSuccess) *bytes += sz;
    return e;
}

int alloc_scratch(pgpu_index* h) {
    std::string err;
    if (int rc = pgpu::alloc_scratch(h->ix, h->cfg, h->max_batch, &h->s, &err)) return fail(rc, err);
    return PGPU_OK;
}

int check_config(const pgpu_index* h, const pgpu_params* p) {
    // IndexConf::adaptive_search_param (puck/index_conf.cpp:152-199)
    if (p->radius_rate < 1.0) return fail(PGPU_E_INVALID, "radius_rate should >= 1.0");
    if (p->filter_topk < p->topk) return fail(PGPU_E_INVALID, "filter_topk should >= topk");
    if (p->search_coarse_count == 0 || p->filter_topk == 0)
        return fail(PGPU_E_INVALID, "search_coarse_count and filter_topk must be positive");
    if (p->filter_topk > pgpu::kMaxFilterTopk)
        return fail(PGPU_E_LIMIT, "filter_topk above " + std::to_string(pgpu::kMaxFilterTopk));
    if (p->topk > pgpu::kMaxFilterTopk)
        return fail(PGPU_E_LIMIT, "topk above " + std::to_string(pgpu::kMaxFilterTopk));
    if (p->max_batch == 0) return fail(PGPU_E_INVALID, "max_batch must be positive");
    if (p->mode != PGPU_MODE_EXACT && p->mode != PGPU_MODE_SCAN)
        return fail(PGPU_E_INVALID, "unknown search mode");
    if (p->precision != PGPU_PRECISION_FP32 && p->precision != PGPU_PRECISION_BF16)
        return fail(PGPU_E_INVALID, "unknown precision");
    if (p->precision == PGPU_PRECISION_BF16 && p->mode != PGPU_MODE_SCAN)
        return fail(PGPU_E_INVALID, "BF16 precision needs scan mode");
    const uint64_t keep =
        (uint64_t)p->filter_topk + (p->precision == PGPU_PRECISION_BF16 ? p->filter_margin : 0);
    if (p->mode == PGPU_MODE_SCAN && keep > pgpu::scan_max_filter_topk())
        return fail(PGPU_E_LIMIT, "filter_topk + filter_margin above " +
                                      std::to_string(pgpu::scan_max_filter_topk()) + " in scan mode");
    if (h != nullptr && h->cfg.probe != nullptr && p->mode != PGPU_MODE_SCAN)
        return fail(PGPU_E_INVALID, "a learned probe is attached: scan mode only");
    if (h != nullptr) {
        const bool bf16 = p->precision == PGPU_PRECISION_BF16;
        if (pgpu::walk_smem_bytes(h->ix, p->filter_topk) > 220 * 1024 ||
            (bf16 ? pgpu::scan_smem_bytes_half(h->ix, (uint32_t)keep)
                  : pgpu::scan_smem_bytes(h->ix, (uint32_t)keep)) > 220 * 1024 ||
            (bf16 && h->ix.pq_nsq == 0
                 ? pgpu::rerank_screen_smem_bytes(h->ix, (uint32_t)keep, p->topk)
                  : pgpu::rerank_smem_bytes(h->ix, (uint32_t)keep, p->topk)) > 220 * 1024)
            return fail(PGPU_E_LIMIT, "filter_topk/topk/filter_nsq exceed the shared-memory budget");
    }
    return PGPU_OK;
}

void apply_config(pgpu_index* h, const pgpu_params* p) {
    h->cfg.P = p->search_coarse_count;
    h->cfg.T = p->filter_topk;
    h->cfg.topk_max = p->topk;
    h->cfg.radius_rate = p->radius_rate;
    h->cfg.mode = p->mode;
    h->cfg.precision = p->precision;
    h->cfg.margin = p->filter_margin;
    h->max_batch = p->max_batch;
}

int ensure_precision_data(pgpu_index* h) {
    std::string err;
    // the scan's interleaved code copy (both precisions)
    if (h->cfg.mode == PGPU_MODE_SCAN)
        if (int rc = pgpu::ensure_interleaved_codes(&h->ix, &err)) return fail(rc, err);
    if (h->cfg.precision != PGPU_PRECISION_BF16) return PGPU_OK;
    // the BF16 screen reranks original vectors; a PQ index reranks by its PQ
    if (h->ix.pq_nsq != 0) return PGPU_OK;
    if (int rc = pgpu::ensure_bf16_features(&h->ix, &err)) return fail(rc, err);
    return PGPU_OK;
}

int ensure_staging(pgpu_index* h, uint32_t topk) {
    if (h->d_qin != nullptr && h->stage_topk >= topk) return PGPU_OK;
    free_staging(h);
    const uint64_t B = h->max_batch;
    uint64_t b = 0;
    cudaError_t e = alloc(&h->d_qin, B * h->ix.d, &b);
    if (e == cudaSuccess) e = alloc(&h->d_dist, B * std::max(1u, topk), &b);
    if (e == cudaSuccess) e = alloc(&h->d_ids, B * std::max(1u, topk), &b);
    if (e == cudaSuccess) e = alloc(&h->d_status, B, &b);
    if (e != cudaSuccess) {
        free_staging(h);
        return cuda_fail(e, "staging allocation");
    }
    h->stage_topk = topk;
    return PGPU_OK;
}

// Accumulates the previous call's stage times once its events have completed.
void collect_stage_times(pgpu_index* h) {
    if (!h->stage_pending) return;
    cudaEventSynchronize(h->ev[PGPU_NUM_STAGES]);
    for (int i = 0; i < PGPU_NUM_STAGES; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, h->ev[i], h->ev[i + 1]) == cudaSuccess) h->stage_ms[i] += ms;
    }
    h->stage_pending = false;
}

// One pass of <= max_batch queries, all buffers on the device.
int run_pass(pgpu_index* h, uint32_t n, const float* d_q, uint32_t topk, float* d_dist,
             uint32_t* d_ids, int32_t* d_status, cudaStream_t st) {
    const bool prof = h->profiling;
    if (prof) collect_stage_times(h);
    int launched = 0;
    const char* what = "";
    cudaError_t e = pgpu::run_pipeline(h->ix, h->cfg, h->s, n, d_q, topk, d_dist, d_ids, d_status,
                                       st, prof ? h->ev : nullptr, &launched, &what);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (prof) h->stage_pending = true;
    h->kernels += launched;
    return PGPU_OK;
}

int open_common(const pgpu_index_arrays& a, const pgpu_params* params, pgpu_index** out) {
    pgpu_params p;
    if (params) p = *params;
    else pgpu_params_default(&p);
    if (int rc = check_config(nullptr, &p)) return rc;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(PGPU_E_CUDA, "no CUDA device available");
    if (p.device < 0 || p.device >= ndev) return fail(PGPU_E_INVALID, "device ordinal out of range");
    if ((e = cudaSetDevice(p.device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pgpu::HostIndex hidx;
    std::string err;
    if (int rc = pgpu::build_host_index(a, &hidx, &err)) return fail(rc, err);
    auto* h = new pgpu_index();
    h->device = p.device;
    if (int rc = pgpu::upload_index_with_base(hidx, a.base, &h->ix, &err)) {
        delete h;
        return fail(rc, err);
    }
    if (int rc = check_config(h, &p)) {
        pgpu::free_device_index(&h->ix);
        delete h;
        return rc;
    }
    apply_config(h, &p);
    if (int rc = ensure_precision_data(h)) {
        pgpu::free_device_index(&h->ix);
        delete h;
        return rc;
    }
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        pgpu::free_device_index(&h->ix);
        delete h;
        return cuda_fail(e, "stream create");
    }
    if (int rc = alloc_scratch(h)) {
        cudaStreamDestroy(h->stream);
        pgpu::free_device_index(&h->ix);
        delete h;
        return rc;
    }
    *out = h;
    return PGPU_OK;
}

}  // namespace

namespace pgpu {
int set_last_error(int code, const std::string& msg) { return fail(code, msg); }
const DeviceIndex& index_device(const pgpu_index* h) { return h->ix; }
const SearchConfig& index_config(const pgpu_index* h) { return h->cfg; }
int index_device_ordinal(const pgpu_index* h) { return h->device; }
}  // namespace pgpu

extern "C" {

void pgpu_params_default(pgpu_params* p) {
    p->search_coarse_count = 200;
    p->topk = 100;
    p->filter_topk = 1100;
    p->radius_rate = 1.0;
    p->device = 0;
    p->max_batch = 8192;
    p->mode = PGPU_MODE_EXACT;
    p->precision = PGPU_PRECISION_FP32;
    p->filter_margin = 0;
}

const char* pgpu_last_error(void) { return g_last_error.c_str(); }

int pgpu_open_arrays(const pgpu_index_arrays* arrays, const pgpu_params* params,
                     pgpu_index** out) {
    if (arrays == nullptr || out == nullptr) return fail(PGPU_E_INVALID, "null argument");
    *out = nullptr;
    return open_common(*arrays, params, out);
}

int pgpu_open(const char* index_path, const pgpu_params* params, pgpu_index** out) {
    if (index_path == nullptr || out == nullptr) return fail(PGPU_E_INVALID, "null argument");
    *out = nullptr;
    if (params != nullptr)
        if (int rc = check_config(nullptr, params)) return rc;
    pgpu_index_arrays a;
    std::memset(&a, 0, sizeof(a));
    std::vector<char> storage;
    std::string err;
    if (int rc = pgpu::read_index_files(index_path, &a, storage, &err)) return fail(rc, err);
    return open_common(a, params, out);
}

int pgpu_set_search_params(pgpu_index* h, const pgpu_params* params) {
    if (h == nullptr || params == nullptr) return fail(PGPU_E_INVALID, "null argument");
    std::lock_guard<std::mutex> g(h->mu);
    if (int rc = check_config(h, params)) return rc;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    apply_config(h, params);
    if (int rc = ensure_precision_data(h)) return rc;
    free_staging(h);
    return alloc_scratch(h);
}

int pgpu_search_batch_device(pgpu_index* h, uint32_t n, const float* query, uint32_t topk,
                             float* distance, uint32_t* labels, int32_t* status, void* stream) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    if (n == 0 || topk == 0) return PGPU_OK;
    if (query == nullptr || distance == nullptr || labels == nullptr)
        return fail(PGPU_E_INVALID, "feature is nullptr");
    if (topk > h->cfg.topk_max)
        return fail(PGPU_E_INVALID, "topk should <= topk, topk = " + std::to_string(h->cfg.topk_max));
    std::lock_guard<std::mutex> g(h->mu);
    cudaSetDevice(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    collect_stage_times(h);
    h->kernels = 0;
    for (float& v : h->stage_ms) v = 0.0f;
    const uint32_t d = h->ix.qdim;  // floats per caller query
    for (uint32_t off = 0; off < n; off += h->max_batch) {
        const uint32_t m = std::min(h->max_batch, n - off);
        if (int rc = run_pass(h, m, query + (uint64_t)off * d, topk, distance + (uint64_t)off * topk,
                              labels + (uint64_t)off * topk, status ? status + off : nullptr, st))
            return rc;
    }
    return PGPU_OK;
}

int pgpu_search_batch(pgpu_index* h, uint32_t n, const float* query, uint32_t topk,
                      float* distance, uint32_t* labels, int32_t* status) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    if (n == 0 || topk == 0) return PGPU_OK;
    if (query == nullptr || distance == nullptr || labels == nullptr)
        return fail(PGPU_E_INVALID, "feature is nullptr");
    if (topk > h->cfg.topk_max) {
        if (status)
            for (uint32_t i = 0; i < n; ++i) status[i] = PGPU_E_INVALID;
        return fail(PGPU_E_INVALID, "topk should <= topk, topk = " + std::to_string(h->cfg.topk_max));
    }
    std::lock_guard<std::mutex> g(h->mu);
    cudaSetDevice(h->device);
    if (int rc = ensure_staging(h, topk)) return rc;
    const uint32_t d = h->ix.qdim;  // floats per caller query
    cudaStream_t st = h->stream;
    collect_stage_times(h);
    h->kernels = 0;
    for (float& v : h->stage_ms) v = 0.0f;
    h->records = 0;
    h->cells = 0;
    for (uint64_t& c : h->walk_counters) c = 0;
    cudaError_t e;
    for (uint32_t off = 0; off < n; off += h->max_batch) {
        const uint32_t m = std::min(h->max_batch, n - off);
        if ((e = cudaMemcpyAsync(h->d_qin, query + (uint64_t)off * d, sizeof(float) * m * d,
                                 cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_fail(e, "query upload");
        if (int rc = run_pass(h, m, h->d_qin, topk, h->d_dist, h->d_ids, h->d_status, st)) return rc;
        if ((e = cudaMemcpyAsync(distance + (uint64_t)off * topk, h->d_dist,
                                 sizeof(float) * m * topk, cudaMemcpyDeviceToHost, st)) ||
            (e = cudaMemcpyAsync(labels + (uint64_t)off * topk, h->d_ids,
                                 sizeof(uint32_t) * m * topk, cudaMemcpyDeviceToHost, st)))
            return cuda_fail(e, "result download");
        if (status && (e = cudaMemcpyAsync(status + off, h->d_status, sizeof(int32_t) * m,
                                           cudaMemcpyDeviceToHost, st)))
            return cuda_fail(e, "status download");
        unsigned long long cnt[pgpu::kNumWalkCounters];
        if ((e = cudaMemcpyAsync(cnt, h->s.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaStreamSynchronize(st)))
            return cuda_fail(e, "search");
        h->records += cnt[0];
        h->cells += cnt[1];
        for (int i = 0; i < pgpu::kNumWalkCounters; ++i) h->walk_counters[i] += cnt[i];
    }
    return PGPU_OK;
}

int pgpu_search(pgpu_index* h, const float* feature, uint32_t topk, float* distance,
                uint32_t* local_idx, uint32_t* result_num) {
    if (h == nullptr || feature == nullptr) return fail(PGPU_E_INVALID, "feature is nullptr");
    if (topk > h->cfg.topk_max)
        return fail(PGPU_E_INVALID, "topk should <= topk, topk = " + std::to_string(h->cfg.topk_max));
    if (topk == 0) {
        if (result_num) *result_num = 0;
        return PGPU_OK;
    }
    int32_t status = 0;
    if (int rc = pgpu_search_batch(h, 1, feature, topk, distance, local_idx, &status)) return rc;
    if (result_num) {
        uint32_t rn = 0;
        while (rn < topk && local_idx[rn] != pgpu::kNoLabel) ++rn;
        *result_num = rn;
    }
    if (status != 0) return fail(status, "query rejected (zero norm)");
    return PGPU_OK;
}

int pgpu_index_info_get(const pgpu_index* h, pgpu_index_info* info) {
    if (h == nullptr || info == nullptr) return fail(PGPU_E_INVALID, "null argument");
    info->feature_dim = h->ix.d;
    info->query_dim = h->ix.qdim;
    info->ip2cos = h->ix.ip2cos;
    info->total_point_count = h->ix.n;
    info->coarse_cluster_count = h->ix.C;
    info->fine_cluster_count = h->ix.F;
    info->filter_nsq = h->ix.nsq;
    info->lsq = h->ix.lsq;
    info->whether_norm = h->ix.whether_norm;
    info->device_bytes = h->ix.bytes;
    return PGPU_OK;
}

int pgpu_last_stats(const pgpu_index* h, uint64_t* kernels_launched, uint64_t* records_scanned,
                    uint64_t* cells_scanned) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    if (kernels_launched) *kernels_launched = h->kernels;
    if (records_scanned) *records_scanned = h->records;
    if (cells_scanned) *cells_scanned = h->cells;
    return PGPU_OK;
}

int pgpu_walk_counters(const pgpu_index* h, uint64_t* out, uint32_t n) {
    if (h == nullptr || out == nullptr) return fail(PGPU_E_INVALID, "null argument");
    for (uint32_t i = 0; i < n && i < (uint32_t)pgpu::kNumWalkCounters; ++i) out[i] = h->walk_counters[i];
    return PGPU_OK;
}

int pgpu_realtime_open(pgpu_index* h, uint32_t capacity) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    if (h->ix.ip2cos) return fail(PGPU_E_UNSUPPORTED, "inserts into an ip2cos index");
    std::lock_guard<std::mutex> g(h->mu);
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    std::string err;
    if (int rc = pgpu::realtime_open(&h->ix, &h->rt, capacity, &err)) return fail(rc, err);
    return PGPU_OK;
}

int pgpu_insert(pgpu_index* h, uint32_t n, const float* feature, int64_t* local_idx) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    if (n == 0) return PGPU_OK;
    if (feature == nullptr || local_idx == nullptr) return fail(PGPU_E_INVALID, "null argument");
    if (h->ix.ins_cap == 0) return fail(PGPU_E_INVALID, "pgpu_realtime_open was not called");
    std::lock_guard<std::mutex> g(h->mu);
    cudaSetDevice(h->device);
    if (int rc = ensure_staging(h, 1)) return rc;
    const uint32_t d = h->ix.qdim;
    cudaStream_t st = h->stream;
    std::vector<int32_t> status(h->max_batch);
    for (uint32_t off = 0; off < n; off += h->max_batch) {
        const uint32_t m = std::min(h->max_batch, n - off);
        cudaError_t e = cudaMemcpyAsync(h->d_qin, feature + (uint64_t)off * d,
                                        sizeof(float) * m * d, cudaMemcpyHostToDevice, st);
        // single_build's normalisation (hierarchical_cluster_index.cpp:1513-1536); a
        // non-finite or zero-norm feature is not inserted (local id -1)
        if (e == cudaSuccess) e = pgpu::launch_prep_queries(h->ix, h->d_qin, m, h->s, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(status.data(), h->s.status, sizeof(int32_t) * m,
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "insert");
        for (uint32_t i = 0; i < m; ++i) status[i] = status[i] == 0 ? 1 : 0;
        std::string err;
        if (int rc = pgpu::realtime_insert(&h->ix, &h->rt, m, h->s.q, status.data(),
                                           local_idx + off, st, &err))
            return fail(rc, err);
    }
    return PGPU_OK;
}

int pgpu_close(pgpu_index* h) {
    if (h == nullptr) return PGPU_OK;
    cudaSetDevice(h->device);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    free_staging(h);
    pgpu::free_scratch(&h->s);
    pgpu::free_device_index(&h->ix);
    if (h->ev[0])
        for (auto& e : h->ev) cudaEventDestroy(e);
    delete h;
    return PGPU_OK;
}

int pgpu_set_profiling(pgpu_index* h, int enable) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    std::lock_guard<std::mutex> g(h->mu);
    cudaSetDevice(h->device);
    if (enable && h->ev[0] == nullptr) {
        for (auto& e : h->ev) {
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return cuda_fail(r, "event create");
        }
    }
    h->profiling = enable != 0;
    h->stage_pending = false;
    for (float& v : h->stage_ms) v = 0.0f;
    return PGPU_OK;
}

int pgpu_stage_times(pgpu_index* h, float* ms, uint32_t n_stages) {
    if (h == nullptr || ms == nullptr) return fail(PGPU_E_INVALID, "null argument");
    std::lock_guard<std::mutex> g(h->mu);
    if (!h->profiling) return fail(PGPU_E_INVALID, "profiling is not enabled");
    cudaSetDevice(h->device);
    collect_stage_times(h);
    for (uint32_t i = 0; i < n_stages && i < (uint32_t)PGPU_NUM_STAGES; ++i) ms[i] = h->stage_ms[i];
    return PGPU_OK;
}

int pgpu_nearest_center(uint32_t dim, const float* centroids, uint64_t k, const float* points,
                        uint64_t n, int32_t* assign, float* distance, void* stream) {
    if (dim == 0 || k == 0 || centroids == nullptr || points == nullptr || assign == nullptr ||
        distance == nullptr)
        return fail(PGPU_E_INVALID, "invalid argument");
    if (n == 0) return PGPU_OK;
    if (k > 0xFFFFFFFFull) return fail(PGPU_E_LIMIT, "more than 2^32-1 centroids");
    cudaError_t e = pgpu::launch_nearest_center_tc(dim, centroids, k, points, n, assign, distance,
                                                   (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "nearest_center");
    return PGPU_OK;
}

int pgpu_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C, const float* fine,
                             uint32_t F, const float* points, uint64_t n, uint32_t* cell,
                             float* distance, void* stream) {
    if (dim == 0 || C == 0 || F == 0 || coarse == nullptr || fine == nullptr ||
        points == nullptr || cell == nullptr || distance == nullptr)
        return fail(PGPU_E_INVALID, "invalid argument");
    if ((uint64_t)C * F > 0xFFFFFFFFull) return fail(PGPU_E_LIMIT, "C * F above 2^32 - 1");
    if (n == 0) return PGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = pgpu::launch_nearest_cell_assign(dim, coarse, C, fine, F, points, n, cell,
                                                     distance, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "nearest_cell_assign");
    return PGPU_OK;
}

int pgpu_filter_candidates(pgpu_index* h, uint32_t n, const float* query, uint32_t* labels,
                           float* distance, uint32_t* count) {
    if (h == nullptr || query == nullptr || labels == nullptr || distance == nullptr ||
        count == nullptr)
        return fail(PGPU_E_INVALID, "null argument");
    if (n == 0) return PGPU_OK;
    std::lock_guard<std::mutex> g(h->mu);
    if (n > h->max_batch) return fail(PGPU_E_LIMIT, "n above max_batch");
    if (h->cfg.mode != PGPU_MODE_SCAN) return fail(PGPU_E_INVALID, "scan mode only");
    cudaSetDevice(h->device);
    const uint32_t topk = 1;
    if (int rc = ensure_staging(h, topk)) return rc;
    cudaStream_t st = h->stream;
    const uint32_t keep = h->s.T;
    cudaError_t e = cudaMemcpyAsync(h->d_qin, query, sizeof(float) * n * h->ix.qdim,
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "query upload");
    if (int rc = run_pass(h, n, h->d_qin, topk, h->d_dist, h->d_ids, h->d_status, st)) return rc;
    uint32_t* ids = nullptr;
    e = cudaMallocAsync(&ids, sizeof(uint32_t) * (uint64_t)n * keep, st);
    if (e == cudaSuccess) e = pgpu::launch_gather_u32(h->s.htag, (uint64_t)n * keep, h->ix.mem2local, ids, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(labels, ids, sizeof(uint32_t) * (uint64_t)n * keep,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(distance, h->s.hdist, sizeof(float) * (uint64_t)n * keep,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(count, h->s.hcnt, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st);
    if (ids) cudaFreeAsync(ids, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "filter_candidates");
    return PGPU_OK;
}

int pgpu_set_probe(pgpu_index* h, pgpu_probe* probe, float mass, uint32_t max_probe) {
    if (h == nullptr) return fail(PGPU_E_INVALID, "null index");
    std::lock_guard<std::mutex> g(h->mu);
    if (probe != nullptr) {
        const pgpu::ProbeNet* net = pgpu::probe_net(probe);
        if (h->cfg.mode != PGPU_MODE_SCAN) return fail(PGPU_E_INVALID, "the learned probe needs scan mode");
        if (pgpu::probe_device(probe) != h->device)
            return fail(PGPU_E_INVALID, "probe and index are on different devices");
        if (net->d != h->ix.d || net->C != h->ix.C)
            return fail(PGPU_E_INVALID, "probe dimension or cluster count does not match the index");
        if (!(mass > 0.0f && mass <= 1.0f)) return fail(PGPU_E_INVALID, "mass must be in (0, 1]");
        if (max_probe == 0 || max_probe > 64 || max_probe > h->ix.C)
            return fail(PGPU_E_INVALID, "max_probe must be in [1, min(64, coarse_cluster_count)]");
    }
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    h->cfg.probe = probe ? pgpu::probe_net(probe) : nullptr;
    h->cfg.probe_mass = mass;
    h->cfg.probe_max = probe ? max_probe : 0;
    free_staging(h);
    return alloc_scratch(h);
}

int pgpu_knn(const float* base, uint64_t n, uint32_t dim, const float* queries, uint32_t nq,
             uint32_t k, uint32_t* labels, float* distance, void* stream) {
    if (base == nullptr || queries == nullptr || labels == nullptr || distance == nullptr ||
        dim == 0 || k == 0)
        return fail(PGPU_E_INVALID, "invalid argument");
    if (k > 64) return fail(PGPU_E_LIMIT, "k above 64");
    if (n > 0xFFFFFFFFull) return fail(PGPU_E_LIMIT, "more than 2^32-1 base points");
    if (n == 0 || nq == 0) return PGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int* err = nullptr;
    cudaError_t e = cudaMallocAsync(&err, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e == cudaSuccess) e = pgpu::launch_knn(base, n, dim, queries, nq, k, labels, distance, err, st);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (err) cudaFreeAsync(err, st);
    if (e != cudaSuccess) return cuda_fail(e, "knn");
    if (flag) return fail(PGPU_E_TIMEOUT, "tensor-core wait expired");
    return PGPU_OK;
}

int pgpu_contract_bf16(int32_t mode, uint32_t na, uint32_t nb, uint32_t k, const float* a,
                       uint64_t a_rs, uint64_t a_ks, const float* b, uint64_t b_rs, uint64_t b_ks,
                       const float* bias, const float* aux, uint64_t ld_aux, float* out,
                       uint64_t ld_out, float* out2, float alpha, float beta, void* stream) {
    if (mode < PGPU_CONTRACT_SCORE || mode > PGPU_CONTRACT_GELU_BWD || k == 0 || a == nullptr ||
        b == nullptr || out == nullptr || ld_out < nb)
        return fail(PGPU_E_INVALID, "invalid argument");
    if ((na + 127u) / 128u > 65535u) return fail(PGPU_E_LIMIT, "na above 8388480");
    cudaStream_t st = (cudaStream_t)stream;
    int* err = nullptr;
    cudaError_t e = cudaMallocAsync(&err, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "contract_bf16");
    e = cudaMemsetAsync(err, 0, sizeof(int), st);
    pgpu::TcOperand A{a, a_rs, a_ks, na};
    pgpu::TcOperand B{b, b_rs, b_ks, nb};
    pgpu::TcEpilogue ep{};
    ep.mode = mode;
    ep.out = out;
    ep.ld = ld_out;
    ep.bias = bias;
    ep.aux = aux;
    ep.ld_aux = ld_aux;
    ep.out2 = out2;
    ep.alpha = alpha;
    ep.beta = beta;
    if (e == cudaSuccess) e = pgpu::launch_tc_gemm(A, B, k, ep, err, st);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(err, st);
    if (e == cudaErrorInvalidValue) return fail(PGPU_E_INVALID, "invalid contraction operands");
    if (e != cudaSuccess) return cuda_fail(e, "contract_bf16");
    if (flag) return fail(PGPU_E_TIMEOUT, "tensor-core wait expired");
    return PGPU_OK;
}

int pgpu_contract_bf16_rows(int32_t mode, uint32_t na, uint32_t nb, uint32_t k,
                            const uint16_t* a, uint64_t a_rs, const uint16_t* b, uint64_t b_rs,
                            const float* bias, const float* aux, uint64_t ld_aux, float* out,
                            uint64_t ld_out, float* out2, float alpha, float beta, void* stream) {
    if (mode < PGPU_CONTRACT_SCORE || mode > PGPU_CONTRACT_GELU_BWD || k == 0 || a == nullptr ||
        b == nullptr || out == nullptr || ld_out < nb)
        return fail(PGPU_E_INVALID, "invalid argument");
    if ((na + 127u) / 128u > 65535u) return fail(PGPU_E_LIMIT, "na above 8388480");
    cudaStream_t st = (cudaStream_t)stream;
    int* err = nullptr;
    cudaError_t e = cudaMallocAsync(&err, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "contract_bf16_rows");
    e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (a_rs < k || b_rs < k) return fail(PGPU_E_INVALID, "row stride below k");
    pgpu::TcOperand A{nullptr, a_rs, 1, na, a};
    pgpu::TcOperand B{nullptr, b_rs, 1, nb, b};
    pgpu::TcEpilogue ep{};
    ep.mode = mode;
    ep.out = out;
    ep.ld = ld_out;
    ep.bias = bias;
    ep.aux = aux;
    ep.ld_aux = ld_aux;
    ep.out2 = out2;
    ep.alpha = alpha;
    ep.beta = beta;
    if (e == cudaSuccess) e = pgpu::launch_tc_gemm(A, B, k, ep, err, st);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(err, st);
    if (e == cudaErrorInvalidValue) return fail(PGPU_E_INVALID, "invalid contraction operands");
    if (e != cudaSuccess) return cuda_fail(e, "contract_bf16_rows");
    if (flag) return fail(PGPU_E_TIMEOUT, "tensor-core wait expired");
    return PGPU_OK;
}

}  // extern "C"
