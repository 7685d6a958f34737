// C entry points over the reference's own Puck code (compiled from the
// reference sources by oracle/ref/Makefile into oracle/_ref/libpuckref.so).
// Test infrastructure only: used here to build small reference indexes and to
// dump golden search outputs. Nothing in the product links this library.
//
// ref_search drives py_puck_api::PySearcher::search
// (pyapi_wrapper/py_api_wrapper.cpp:154-170), i.e. the reference's batch
// entry point, unchanged. ref_probe subclasses puck::PuckIndex to call its own
// stages (puck/puck/puck_index.cpp:559-600) one at a time and copy the
// per-query SearchContext buffers out (coarse list, filter heap).
#include <cstring>
#include <memory>
#include <vector>

#include "gflags/gflags.h"
#include "puck/gflags/puck_gflags.h"
#include "puck/puck/puck_index.h"
#include "puck/puck/realtime_insert_puck_index.h"
#include "puck/search_context.h"
#include "pyapi_wrapper/py_api_wrapper.h"

namespace {
class ProbeIndex : public puck::PuckIndex {
public:
    // Runs normalization -> coarse -> filter scan exactly as PuckIndex::search
    // does, and copies the intermediate buffers out.
    int probe(const float* q, uint32_t* coarse_tag, float* coarse_dist, uint32_t* filter_tag,
              float* filter_dist, uint32_t* filter_cnt, float* lut) {
        puck::DataHandler<puck::SearchContext> context(_context_pool);
        if (context->reset(_conf) != 0) return -1;
        const float* feature = normalization(context.get(), q);
        if (feature == nullptr) return -2;
        if (search_nearest_coarse_cluster(context.get(), feature, _conf.search_coarse_count) != 0)
            return -3;
        auto& cell = context->get_search_cell_data();
        std::memcpy(coarse_tag, cell.coarse_tag, sizeof(uint32_t) * _conf.search_coarse_count);
        std::memcpy(coarse_dist, cell.coarse_distance, sizeof(float) * _conf.search_coarse_count);
        int cnt = search_nearest_filter_points(context.get(), feature);
        if (cnt < 0) return -4;
        auto& pt = context->get_search_point_data();
        *filter_cnt = (uint32_t)cnt;
        std::memcpy(filter_tag, pt.result_tag, sizeof(uint32_t) * _conf.filter_topk);
        std::memcpy(filter_dist, pt.result_distance, sizeof(float) * _conf.filter_topk);
        if (lut != nullptr) {
            std::memcpy(lut, pt.pq_dist_table, sizeof(float) * _conf.filter_nsq * _conf.ks);
        }
        return 0;
    }
    const uint32_t* memory_to_local() const { return _memory_to_local; }
    uint32_t search_coarse_count() const { return _conf.search_coarse_count; }
    uint32_t filter_topk() const { return _conf.filter_topk; }
    uint32_t total_point_count() const { return _conf.total_point_count; }
};
}  // namespace

extern "C" {

int ref_set_flag(const char* name, const char* value) {
    return google::SetCommandLineOption(name, value).empty() ? -1 : 0;
}

// train() then build() of a PuckIndex, as tools/train.cpp and tools/build.cpp do.
int ref_train_build() {
    {
        puck::PuckIndex index;
        if (index.train() != 0) return -1;
    }
    {
        puck::PuckIndex index;
        if (index.build() != 0) return -2;
    }
    return 0;
}

void* ref_open_searcher() {
    auto* s = new py_puck_api::PySearcher();
    if (s->init() != 0) {
        delete s;
        return nullptr;
    }
    return s;
}

int ref_search(void* h, uint32_t n, const float* q, uint32_t topk, float* dist, uint32_t* labels) {
    return static_cast<py_puck_api::PySearcher*>(h)->search(n, q, topk, dist, labels);
}

void ref_close_searcher(void* h) { delete static_cast<py_puck_api::PySearcher*>(h); }

void* ref_open_probe() {
    auto* p = new ProbeIndex();
    if (p->init() != 0) {
        delete p;
        return nullptr;
    }
    return p;
}

int ref_probe(void* h, const float* q, uint32_t* coarse_tag, float* coarse_dist,
              uint32_t* filter_tag, float* filter_dist, uint32_t* filter_cnt, float* lut) {
    return static_cast<ProbeIndex*>(h)->probe(q, coarse_tag, coarse_dist, filter_tag, filter_dist,
                                              filter_cnt, lut);
}

// One query through the reference's Index::search(const Request*, Response*)
// (puck/index.h:46, puck/puck/puck_index.cpp:559-600) on the probe's index and context
// pool. On an ip2cos index PySearcher's contexts can hold a stale last query float
// (normalization's memset counts bytes, hierarchical_cluster_index.cpp:1519); the probe's
// contexts are only ever written through that same path, so their last float stays as
// allocated, which the caller checks against the probe's own filter tables.
int ref_search_one(void* h, const float* q, uint32_t topk, float* dist, uint32_t* labels,
                   uint32_t* result_num) {
    puck::Request req;
    req.topk = topk;
    req.feature = q;
    puck::Response resp;
    resp.distance = dist;
    resp.local_idx = labels;
    resp.result_num = 0;
    const int rc = static_cast<ProbeIndex*>(h)->search(&req, &resp);
    *result_num = resp.result_num;
    return rc;
}

// The reference's RealtimeInsertPuckIndex (puck/puck/realtime_insert_puck_index.cpp):
// init() over an index directory holding the label file, insert() of one point, and
// Index::search over the base and inserted points.
void* ref_open_realtime() {
    auto* p = new puck::RealtimeInsertPuckIndex();
    if (p->init() != 0) {
        delete p;
        return nullptr;
    }
    return p;
}

int ref_realtime_insert(void* h, const float* feature, uint32_t dim, const char* label) {
    puck::InsertRequest req;
    req.label = label;
    req.feature = feature;
    req.dim = dim;
    return static_cast<puck::RealtimeInsertPuckIndex*>(h)->insert(&req);
}

int ref_realtime_search(void* h, const float* q, uint32_t topk, float* dist, uint32_t* labels,
                        uint32_t* result_num) {
    puck::Request req;
    req.topk = topk;
    req.feature = q;
    puck::Response resp;
    resp.distance = dist;
    resp.local_idx = labels;
    resp.result_num = 0;
    const int rc = static_cast<puck::RealtimeInsertPuckIndex*>(h)->search(&req, &resp);
    *result_num = resp.result_num;
    return rc;
}

void ref_close_realtime(void* h) { delete static_cast<puck::RealtimeInsertPuckIndex*>(h); }

int ref_probe_sizes(void* h, uint32_t* search_coarse_count, uint32_t* filter_topk,
                    uint32_t* total_point_count) {
    auto* p = static_cast<ProbeIndex*>(h);
    *search_coarse_count = p->search_coarse_count();
    *filter_topk = p->filter_topk();
    *total_point_count = p->total_point_count();
    return 0;
}

int ref_memory_to_local(void* h, uint32_t* out) {
    auto* p = static_cast<ProbeIndex*>(h);
    std::memcpy(out, p->memory_to_local(), sizeof(uint32_t) * p->total_point_count());
    return 0;
}

void ref_close_probe(void* h) { delete static_cast<ProbeIndex*>(h); }
}
