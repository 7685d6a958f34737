// One search pass on the device: query prep, coarse scores, coarse top-P, fine
// terms (+ full fine order in exact mode), filter stage (exact walk or scan),
// rerank. Shared by the synchronous entry points and the serving loop.
#include <algorithm>
#include <mutex>
#include <set>
#include <string>
#include <tuple>

#include "pgpu_internal.h"

namespace pgpu {
namespace {
template <class T>
cudaError_t alloc(T** p, uint64_t count, uint64_t* bytes) {
    const size_t sz = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc((void**)p, sz);
    if (e == cudaSuccess) *bytes += sz;
    return e;
}
}  // namespace

void ensure_max_dynamic_smem(const void* kernel, int bytes) {
    static std::mutex mu;
    static std::set<std::tuple<const void*, int, int>> done;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(kernel, dev, bytes);
    std::lock_guard<std::mutex> g(mu);
    if (done.count(key)) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
        done.insert(key);
}

void free_scratch(Scratch* s) {
    void* ptrs[] = {s->q, s->qb, s->qnorm, s->status, s->dots, s->cdist, s->ctag, s->fdist,
                    s->ftag, s->hdist, s->htag, s->hcnt, s->counters, s->tc_err,
                    s->ph1, s->ph2, s->pconf, s->pz, s->order, s->wbucket, s->ulist, s->ucount,
                    s->tbuf, s->qcnt, s->qoff, s->qflag, s->cut};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    *s = Scratch();
}

// Split scan buffer: room for 40960 record distances per query of the batch (about
// 1.6 times the mean record count of a coarse cluster at 100M points and 4000
// clusters), at least 2^20 and at most 2^30. A query whose records do not fit runs
// the fused scan kernel instead.
uint64_t split_capacity(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t B) {
    if (cfg.mode != PGPU_MODE_SCAN || !scan_split_possible(ix, cfg.filter_keep())) return 0;
    uint64_t c = (uint64_t)B * 40960ull;
    if (c < (1ull << 20)) c = 1ull << 20;
    if (c > (1ull << 30)) c = 1ull << 30;
    return c;
}

uint64_t scratch_bytes(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t B) {
    const uint64_t P = cfg.coarse_slots(ix.C), T = cfg.filter_keep();
    const uint64_t probe = cfg.probe ? (uint64_t)B * (cfg.probe->h * 4 + 8 + ix.C * 4ull) + 4 : 0;
    const uint64_t fine_order = cfg.mode == PGPU_MODE_EXACT ? (uint64_t)B * ix.F * 8 : 8;
    const uint64_t tables = cfg.mode == PGPU_MODE_SCAN ? (uint64_t)B * 5 : 0;  // launch order
    const uint64_t tcap = split_capacity(ix, cfg, B);
    const uint64_t split = tcap ? tcap * 4 + (uint64_t)B * (12 + sizeof(SplitCut)) : 0;
    return (uint64_t)B * (ix.d * 6 + 4 + 4 + std::max(ix.C, ix.F) * 4ull + P * 8 + T * 8 + 4) +
           fine_order + tables + split + probe + kNumWalkCounters * 8 + 4;
}

int alloc_scratch(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t B, Scratch* out,
                  std::string* err) {
    free_scratch(out);
    Scratch& s = *out;
    s.P = cfg.coarse_slots(ix.C);
    s.Pfix = std::min(cfg.P, ix.C);
    s.T = cfg.filter_keep();
    // the full fine order is only read by the exact walk
    const uint64_t fine_rows = cfg.mode == PGPU_MODE_EXACT ? (uint64_t)B * ix.F : 1;
    uint64_t b = 0;
    cudaError_t e = cudaSuccess;
#define PGPU_ALLOC(ptr, cnt)                                                        \
    if (e == cudaSuccess) e = alloc(&(ptr), (cnt), &b);
    PGPU_ALLOC(s.q, (uint64_t)B * ix.d);
    PGPU_ALLOC(s.qb, (uint64_t)B * ix.d);
    PGPU_ALLOC(s.qnorm, B);
    PGPU_ALLOC(s.status, B);
    PGPU_ALLOC(s.dots, (uint64_t)B * std::max(ix.C, ix.F));
    PGPU_ALLOC(s.cdist, (uint64_t)B * s.P);
    PGPU_ALLOC(s.ctag, (uint64_t)B * s.P);
    PGPU_ALLOC(s.fdist, fine_rows);
    PGPU_ALLOC(s.ftag, fine_rows);
    PGPU_ALLOC(s.hdist, (uint64_t)B * s.T);
    PGPU_ALLOC(s.htag, (uint64_t)B * s.T);
    PGPU_ALLOC(s.hcnt, B);
    PGPU_ALLOC(s.counters, kNumWalkCounters);
    PGPU_ALLOC(s.tc_err, 1);
    if (cfg.mode == PGPU_MODE_SCAN) {
        PGPU_ALLOC(s.order, B);
        PGPU_ALLOC(s.wbucket, B);
        const uint64_t tcap = split_capacity(ix, cfg, B);
        if (tcap) {
            PGPU_ALLOC(s.tbuf, tcap);
            PGPU_ALLOC(s.qcnt, B);
            PGPU_ALLOC(s.qoff, B);
            PGPU_ALLOC(s.qflag, B);
            PGPU_ALLOC(s.cut, B);
            s.tcap = tcap;
        }
    }
    if (cfg.probe) {
        PGPU_ALLOC(s.ulist, B);
        PGPU_ALLOC(s.ucount, 1);
        PGPU_ALLOC(s.ph1, (uint64_t)B * cfg.probe->h);
        PGPU_ALLOC(s.ph2, (uint64_t)B * cfg.probe->h);
        PGPU_ALLOC(s.pconf, B);
        PGPU_ALLOC(s.pz, (uint64_t)B * ix.C);
    }
#undef PGPU_ALLOC
    if (e != cudaSuccess) {
        free_scratch(&s);
        *err = std::string("scratch allocation: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
    }
    s.cap = B;
    s.bytes = b;
    return PGPU_OK;
}

cudaError_t run_pipeline(const DeviceIndex& ix, const SearchConfig& cfg, Scratch& s, uint32_t n,
                         const float* d_q, uint32_t topk, float* d_dist, uint32_t* d_ids,
                         int32_t* d_status, cudaStream_t st, cudaEvent_t* ev, int* launched,
                         const char** what) {
    cudaError_t e;
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], st);
    };
#define PGPU_STEP(call, name)           \
    if ((e = (call)) != cudaSuccess) {  \
        *what = name;                   \
        return e;                       \
    }
    PGPU_STEP(cudaMemsetAsync(s.counters, 0, sizeof(unsigned long long) * kNumWalkCounters, st),
              "memset");
    PGPU_STEP(cudaMemsetAsync(s.tc_err, 0, sizeof(int), st), "memset");
    mark(0);
    PGPU_STEP(launch_prep_queries(ix, d_q, n, s, st), "prep_queries");
    mark(1);
    int probe_kernels = 0;
    if (cfg.probe) {
        // learned probe first: scores of the coarse clusters, then the adaptive choice.
        // The fixed-count selection (tensor-core screen + exact window) then runs only
        // for the queries the probe leaves to it (s.ulist, s.ucount on the device): with
        // a confident probe the coarse screen has nothing to do.
        PGPU_STEP(cudaMemsetAsync(s.ucount, 0, sizeof(uint32_t), st), "memset");
        float* pz = s.pz;
        PGPU_STEP(probe_infer(*cfg.probe, s.q, s.qb, n, s.ph1, s.ph2, pz, s.tc_err, st),
                  "probe forward");
        PGPU_STEP(launch_probe_select(*cfg.probe, ix, n, pz, cfg.probe_mass, cfg.probe_max, s, st),
                  "probe select");
        probe_kernels = 4;
    }
    // coarse: BF16 tensor-core screen, then the exact top-P from an FP32 window
    PGPU_STEP(launch_coarse_tc(ix, n, s, st), "coarse scores");
    mark(2);
    PGPU_STEP(launch_coarse_window(ix, n, s, st), "coarse select");
    mark(3);
    const bool bf16 = cfg.precision == PGPU_PRECISION_BF16;
    if (bf16) {
        // precision form: -q.f from the BF16 tensor-core contraction
        TcOperand A{nullptr, ix.d, 1, n, s.qb};
        TcOperand B{nullptr, ix.d, 1, ix.F, ix.fine_bf16};
        TcEpilogue ep{};
        ep.mode = TC_EPI_NEG;
        ep.out = s.dots;
        ep.ld = ix.F;
        PGPU_STEP(launch_tc_gemm(A, B, ix.d, ep, s.tc_err, st), "fine scores");
    } else {
        PGPU_STEP(launch_centroid_scores(s.q, n, ix.fine, ix.F, ix.d, nullptr, true, s.dots, ix.F,
                                         st),
                  "fine scores");
    }
    mark(4);
    int k = 6;
    if (cfg.mode == PGPU_MODE_EXACT) {
        PGPU_STEP(launch_topsort_status(s.dots, n, ix.F, ix.F, ix.F, s.fdist, s.ftag, s.status, st),
                  "fine order");
        k = 7;
    } else {
        PGPU_STEP(launch_scan_order(ix, n, s, st), "scan order");
        PGPU_STEP(launch_scan_prepare(ix, n, s, bf16, st), "scan prepare");
    }
    mark(5);
    if (cfg.mode == PGPU_MODE_EXACT) {
        PGPU_STEP(launch_walk_scan(ix, cfg, n, s, st), "walk_scan");
    } else {
        PGPU_STEP(launch_scan_records(ix, n, s, bf16, st), "scan records");
    }
    mark(6);
    if (cfg.mode == PGPU_MODE_SCAN) PGPU_STEP(launch_scan_finish(ix, n, s, bf16, st), "scan finish");
    mark(7);
    if (bf16 && ix.pq_nsq == 0) {
        PGPU_STEP(launch_rerank_screen(ix, n, topk, s, d_dist, d_ids, d_status, st), "rerank");
    } else {  // the original vectors, or the second-level PQ
        PGPU_STEP(launch_rerank(ix, cfg, n, topk, s, d_dist, d_ids, d_status, st), "rerank");
    }
    mark(8);
#undef PGPU_STEP
    // scan mode adds the two launch-order kernels, and the split scan three more
    // (k_split_counts, k_split_offsets, k_scan_score; the fused kernel is counted in k)
    if (launched)
        *launched = k + probe_kernels +
                    (cfg.mode == PGPU_MODE_SCAN ? 2 + (scan_split_applies(ix, s) ? 3 : 0) : 0);
    return cudaSuccess;
}

}  // namespace pgpu
