// k_walk_scan: the cell walk and filter-PQ ADC scan of
// PuckIndex::search_nearest_filter_points (puck/puck/puck_index.cpp:485-557) and
// compute_quantized_distance (puck_index.cpp:346-390), bit-exact.
//
// The reference walks, for each probed coarse cluster c (ascending coarse term),
// the fine cells k in ascending fine-term order fd, breaks when
// fd + min_dist >= pivot, skips cells with stationary[c][k] >= max_stationary_dist,
// and scans the others into a bounded max-heap; pivot and max_stationary_dist only
// decrease as the heap fills. One block per query reproduces it:
//
//   candidate generation (all threads, against the current pivot/max_stat, which
//   bound every later value):
//     enumeration: cells of c in ascending stationary order (sorted at load) below
//                  max_stat and before the break, re-ordered by fine rank. Used
//                  when they fit one block-wide chunk of the sorted row.
//     fd-order   : 128 consecutive fine ranks per chunk, break/skip tests per cell
//                  (the heap-fill phase, where nothing is pruned yet).
//   speculative ADC: every point of every candidate cell (one thread per point).
//   replay (thread 0): the candidates in fine-rank order with the exact pivot,
//     max_stationary_dist and heap; it only prunes further, never adds.
// Every test is monotone in pivot/max_stat, so the replay scans exactly the cells
// and points the sequential walk scans, in the same order.
#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr int kThreads = 128;   // block size = candidate slots per round
constexpr int kWarps = kThreads / 32;
constexpr int kPointBuf = 1024; // points whose ADC is precomputed per batch

struct WalkParams {
    const float* q;
    const float* qnorm;
    const int32_t* status;
    const float* cdist;
    const uint32_t* ctag;
    const float* fdist;       // [B][F] fine terms in ascending (rank) order
    const uint32_t* ftag;     // [B][F] fine id at each rank
    const float* fd_by_fine;  // [B][F] fine term indexed by fine id
    float* hdist;
    uint32_t* htag;
    uint32_t* hcnt;
    const float* stationary;  // [C][F]
    const float* stat_sorted; // [C][F] stationary ascending per coarse row
    const uint32_t* stat_fine;// [C][F] fine id of each sorted entry
    const uint32_t* cell_start;
    const float* mdo;
    const float* offsets;
    const uint8_t* codes;
    const float* codebook;
    unsigned long long* counters;
    const int32_t* ins_head;  // realtime: [C*F] newest insert of each cell, or null
    const int32_t* ins_next;
    uint32_t n_base;          // memory id of insert 0
    uint32_t d, C, F, nsq, lsq, code_stride, P, T;
    double rr;
};

// Diagnostic counters accumulated per launch (pgpu_walk_counters): records and
// cells scanned, fd-order chunks, enumerations, fd-order coarse clusters, heap
// inserts, and thread-0 clock cycles spent in replay / whole walk / prologue /
// candidate generation / speculative ADC.
enum { kCntRecords, kCntCells, kCntChunks, kCntEnum, kCntFdOrder, kCntInserts, kCycReplay,
       kCycTotal, kCycPrologue, kCycCand, kCycAdc, kNumCounters };

struct WalkState {
    float pivot, max_stat, min_dist, cdl;
    uint32_t c, dpc, broke, n_used, big, npts;
    uint32_t warp_tot[kWarps];
    unsigned long long cnt[kNumCounters];
};

struct Cand {  // per-candidate arrays, kThreads entries each (+1 for pref)
    uint32_t* fine;
    uint32_t* rank;
    float* fd;
    float* stat;
    float* dist;
    uint32_t* start;
    uint32_t* cnt;
    uint32_t* pref;
};

// Scans candidates [0, n) (sorted by fine rank) in batches whose points fit the
// point buffer. Returns true when the walk broke inside this coarse cluster.
__device__ bool process_candidates(const WalkParams& p, WalkState& st, const Cand& cd, uint32_t n,
                                   const float* lut, float* hv, uint32_t* ht, float* pt0,
                                   float* ptf, const uint32_t* cs, float qn) {
    const int tid = threadIdx.x;
    const float cdl = st.cdl;
    if ((uint32_t)tid < n) {
        const uint32_t k = cd.fine[tid];
        const uint32_t s0 = cs[k];
        cd.start[tid] = s0;
        cd.cnt[tid] = cs[k + 1] - s0;
        cd.dist[tid] = __fadd_rn(__fadd_rn(cdl, cd.stat[tid]), cd.fd[tid]);
    }
    __syncthreads();
    uint32_t b0 = 0;
    while (b0 < n) {
        const bool mine = (uint32_t)tid >= b0 && (uint32_t)tid < n;
        const uint32_t cnt = mine ? cd.cnt[tid] : 0u;
        uint32_t total;
        const uint32_t incl = block_scan_incl<kWarps>(cnt, st.warp_tot, &total);
        if (mine) cd.pref[tid] = incl - cnt;
        const int fits = __syncthreads_count(mine && incl <= (uint32_t)kPointBuf);
        if (tid == 0) {
            st.n_used = fits > 0 ? (uint32_t)fits : 1u;
            st.big = fits > 0 ? 0u : 1u;
        }
        __syncthreads();
        long long t_adc = clock64();
        const uint32_t n_used = st.n_used;
        const uint32_t last = b0 + n_used - 1;
        const uint32_t npts = st.big ? 0u : cd.pref[last] + cd.cnt[last];
        for (uint32_t j = tid; j < npts; j += kThreads) {
            uint32_t lo = b0, hi = b0 + n_used;  // last candidate with pref <= j
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (cd.pref[mid] <= j) lo = mid;
                else hi = mid;
            }
            const uint32_t mi = cd.start[lo] + (j - cd.pref[lo]);
            const float t0 = adc_base(cd.dist[lo], p.offsets[mi]);
            pt0[j] = t0;
            ptf[j] = __fadd_rn(t0, lut_sum(p.codes + (uint64_t)mi * p.code_stride, lut, p.nsq));
        }
        __syncthreads();
        if (tid == 0) {
            const long long t_rep = clock64();
            st.cnt[kCycAdc] += (unsigned long long)(t_rep - t_adc);
            float pivot = st.pivot, max_stat = st.max_stat;
            const float md = st.min_dist;
            uint32_t dpc = st.dpc;
            bool broke = false;
            unsigned long long sp = 0, sc = 0, ins = 0;
            for (uint32_t i = b0; i <= last; ++i) {
                const float fdi = cd.fd[i];
                if (__fadd_rn(fdi, md) >= pivot) {
                    broke = true;
                    break;
                }
                if (cd.stat[i] >= max_stat) continue;
                uint32_t upd = 0;
                const uint32_t s0 = cd.start[i], nc = cd.cnt[i];
                ++sc;
                for (uint32_t pp = 0; pp < nc; ++pp) {
                    float t0, tf;
                    if (st.big) {
                        t0 = adc_base(cd.dist[i], p.offsets[s0 + pp]);
                        if (t0 >= hv[1]) break;
                        tf = __fadd_rn(t0, lut_sum(p.codes + (uint64_t)(s0 + pp) * p.code_stride,
                                                   lut, p.nsq));
                    } else {
                        t0 = pt0[cd.pref[i] + pp];
                        if (t0 >= hv[1]) break;
                        tf = ptf[cd.pref[i] + pp];
                    }
                    ++sp;
                    if (heap_update(hv, ht, p.T, dpc, tf, s0 + pp)) ++upd;
                }
                if (p.ins_head) {
                    // realtime: the cell's inserted points, newest first, none skipped,
                    // each counted as an update (realtime_insert_puck_index.cpp:398-453)
                    const uint64_t cell = (uint64_t)st.c * p.F + cd.fine[i];
                    for (int32_t id = p.ins_head[cell]; id >= 0; id = p.ins_next[id]) {
                        const uint32_t mi = p.n_base + (uint32_t)id;
                        const float t0 = adc_base(cd.dist[i], p.offsets[mi]);
                        const float tf = __fadd_rn(
                            t0, lut_sum(p.codes + (uint64_t)mi * p.code_stride, lut, p.nsq));
                        ++sp;
                        ++upd;
                        heap_update(hv, ht, p.T, dpc, tf, mi);
                    }
                }
                ins += upd;
                if (upd > 0) pivot = pivot_of(hv[1], qn, p.rr);
                const float cand_ms = __fsub_rn(__fsub_rn(pivot, cdl), fdi);
                if (cand_ms < max_stat) max_stat = cand_ms;
            }
            st.pivot = pivot;
            st.max_stat = max_stat;
            st.dpc = dpc;
            st.broke = broke ? 1u : 0u;
            st.cnt[kCntRecords] += sp;
            st.cnt[kCntCells] += sc;
            st.cnt[kCntInserts] += ins;
            st.cnt[kCycReplay] += (unsigned long long)(clock64() - t_rep);
        }
        __syncthreads();
        if (st.broke) return true;
        b0 += n_used;
    }
    return false;
}

__global__ __launch_bounds__(kThreads) void k_walk_scan(WalkParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ WalkState st;
    const uint32_t qi = blockIdx.x;
    const int tid = threadIdx.x;
    const uint32_t nsq = p.nsq, T = p.T, F = p.F;
    float* lut = reinterpret_cast<float*>(smem);
    float* hv = lut + nsq * 256;  // 1-based [1..T]
    uint32_t* ht = reinterpret_cast<uint32_t*>(hv + T + 1);
    float* qv = reinterpret_cast<float*>(ht + T + 1);
    uint32_t* rank_s = reinterpret_cast<uint32_t*>(qv + p.d);  // [F] fine id -> rank
    uint32_t* cbase = rank_s + F;
    Cand cd;
    cd.fine = cbase;
    cd.rank = cbase + kThreads;
    cd.fd = reinterpret_cast<float*>(cbase + 2 * kThreads);
    cd.stat = reinterpret_cast<float*>(cbase + 3 * kThreads);
    cd.dist = reinterpret_cast<float*>(cbase + 4 * kThreads);
    cd.start = cbase + 5 * kThreads;
    cd.cnt = cbase + 6 * kThreads;
    cd.pref = cbase + 7 * kThreads;  // kThreads + 1
    uint32_t* e_fine = cbase + 8 * kThreads + 1;  // enumeration staging
    uint32_t* e_rank = e_fine + kThreads;
    float* e_fd = reinterpret_cast<float*>(e_rank + kThreads);
    float* e_stat = e_fd + kThreads;
    float* pt0 = e_stat + kThreads;
    float* ptf = pt0 + kPointBuf;

    if (p.status[qi] != 0) {
        if (tid == 0) p.hcnt[qi] = 0;
        return;
    }
    const long long t_start = clock64();
    const float* fd = p.fdist + (uint64_t)qi * F;
    const uint32_t* ftag = p.ftag + (uint64_t)qi * F;
    const float* fdk = p.fd_by_fine + (uint64_t)qi * F;
    for (uint32_t i = tid; i < p.d; i += kThreads) qv[i] = p.q[(uint64_t)qi * p.d + i];
    for (uint32_t i = tid; i <= T; i += kThreads) hv[i] = sentinel_f();
    for (uint32_t i = tid; i < F; i += kThreads) {
        const uint32_t k = ftag[i];
        if (k < F) rank_s[k] = i;
    }
    __syncthreads();
    // get_dist_table (quantization.cpp:260-270)
    build_lut(lut, qv, p.codebook, nsq, p.lsq, kThreads);
    const float qn = p.qnorm[qi];
    if (tid == 0) {
        st.dpc = T;
        st.pivot = pivot_of(sentinel_f(), qn, p.rr);
        for (int i = 0; i < kNumCounters; ++i) st.cnt[i] = 0;
        st.cnt[kCycPrologue] = (unsigned long long)(clock64() - t_start);
    }
    __syncthreads();

    for (uint32_t l = 0; l < p.P; ++l) {
        if (tid == 0) {
            const uint32_t c = p.ctag[(uint64_t)qi * p.P + l];
            const float cdl = p.cdist[(uint64_t)qi * p.P + l];
            st.c = c < p.C ? c : 0u;
            st.cdl = cdl;
            st.min_dist = c < p.C ? __fadd_rn(p.mdo[c], cdl) : 0.0f;
            st.max_stat = __fsub_rn(__fsub_rn(st.pivot, cdl), fd[0]);
            st.broke = c < p.C ? 0u : 1u;  // never taken for finite queries
        }
        __syncthreads();
        if (st.broke) {
            __syncthreads();
            continue;
        }
        const uint32_t c = st.c;
        const uint32_t* cs = p.cell_start + (uint64_t)c * F;
        float pv = st.pivot, ms = st.max_stat;
        const float md = st.min_dist;
        long long t_cand = clock64();

        // ---- enumeration through the stationary-sorted row of c
        bool below = false;
        uint32_t k = 0;
        float sv = 0.0f;
        if ((uint32_t)tid < F) {
            sv = p.stat_sorted[(uint64_t)c * F + tid];
            k = p.stat_fine[(uint64_t)c * F + tid];
            below = sv < ms;
        }
        const bool fallback = __syncthreads_and(below) && F > (uint32_t)kThreads;
        if (!fallback) {
            bool cand = false;
            float fv = 0.0f;
            uint32_t r = 0;
            if (below && k < F) {
                fv = fdk[k];
                r = rank_s[k];
                cand = !(__fadd_rn(fv, md) >= pv);
            }
            uint32_t n;
            const uint32_t pos = block_scan_incl<kWarps>(cand ? 1u : 0u, st.warp_tot, &n) - 1;
            if (cand) {
                e_fine[pos] = k;
                e_rank[pos] = r;
                e_fd[pos] = fv;
                e_stat[pos] = sv;
            }
            __syncthreads();
            if ((uint32_t)tid < n) {  // order by fine rank (ranks are distinct)
                const uint32_t myr = e_rank[tid];
                uint32_t o = 0;
                for (uint32_t j = 0; j < n; ++j) o += e_rank[j] < myr;
                cd.fine[o] = e_fine[tid];
                cd.rank[o] = myr;
                cd.fd[o] = e_fd[tid];
                cd.stat[o] = e_stat[tid];
            }
            __syncthreads();
            if (tid == 0) {
                st.cnt[kCntEnum] += 1;
                st.cnt[kCycCand] += (unsigned long long)(clock64() - t_cand);
            }
            process_candidates(p, st, cd, n, lut, hv, ht, pt0, ptf, cs, qn);
            __syncthreads();
            continue;
        }
        if (tid == 0) st.cnt[kCntFdOrder] += 1;

        // ---- fd-order chunks (nothing pruned yet)
        const float* statrow = p.stationary + (uint64_t)c * F;
        for (uint32_t base = 0; base < F;) {
            t_cand = clock64();
            pv = st.pivot;
            ms = st.max_stat;
            const uint32_t idx = base + tid;
            const bool valid = idx < F;
            const float fdv = valid ? fd[idx] : 0.0f;
            const bool brk = !valid || (__fadd_rn(fdv, md) >= pv);
            // first break position in the chunk: everything before it is a candidate
            // unless skipped
            const uint32_t nbrk_before = __syncthreads_count(!brk);
            // breaks are monotone in idx, so the non-breaking threads are a prefix
            const uint32_t bpos = nbrk_before;
            bool cand = false;
            float stv = 0.0f;
            uint32_t kk = 0;
            if ((uint32_t)tid < bpos) {
                kk = ftag[idx];
                if (kk >= F) kk = 0;  // never taken for finite queries
                stv = statrow[kk];
                cand = !(stv >= ms);
            }
            uint32_t n;
            const uint32_t pos = block_scan_incl<kWarps>(cand ? 1u : 0u, st.warp_tot, &n) - 1;
            if (cand) {
                cd.fine[pos] = kk;
                cd.rank[pos] = idx;
                cd.fd[pos] = fdv;
                cd.stat[pos] = stv;
            }
            __syncthreads();
            if (tid == 0) {
                st.cnt[kCntChunks] += 1;
                st.cnt[kCycCand] += (unsigned long long)(clock64() - t_cand);
            }
            const bool broke = process_candidates(p, st, cd, n, lut, hv, ht, pt0, ptf, cs, qn);
            if (broke || bpos < (uint32_t)kThreads) break;
            base += kThreads;
        }
        __syncthreads();
    }
    if (tid == 0) {
        const uint32_t cnt = T - st.dpc;
        if (cnt < T) heap_reorder(hv, ht, T);
        p.hcnt[qi] = cnt;
        st.cnt[kCycTotal] = (unsigned long long)(clock64() - t_start);
        if (p.counters)
            for (int i = 0; i < kNumCounters; ++i) atomicAdd(p.counters + i, st.cnt[i]);
    }
    __syncthreads();
    for (uint32_t i = tid; i < T; i += kThreads) {
        p.hdist[(uint64_t)qi * T + i] = hv[i + 1];
        p.htag[(uint64_t)qi * T + i] = ht[i + 1];
    }
}

}  // namespace

size_t walk_smem_bytes(const DeviceIndex& ix, uint32_t T) {
    return sizeof(float) * ix.nsq * 256 + (sizeof(float) + sizeof(uint32_t)) * (T + 1) +
           sizeof(float) * ix.d + sizeof(uint32_t) * ix.F + sizeof(uint32_t) * (12 * kThreads + 1) +
           sizeof(float) * 2 * kPointBuf;
}

cudaError_t launch_walk_scan(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t n,
                             Scratch& s, cudaStream_t stream) {
    WalkParams p;
    p.q = s.q;
    p.qnorm = s.qnorm;
    p.status = s.status;
    p.cdist = s.cdist;
    p.ctag = s.ctag;
    p.fdist = s.fdist;
    p.ftag = s.ftag;
    p.fd_by_fine = s.dots;
    p.hdist = s.hdist;
    p.htag = s.htag;
    p.hcnt = s.hcnt;
    p.stationary = ix.stationary;
    p.ins_head = ix.ins_n ? ix.ins_head : nullptr;
    p.ins_next = ix.ins_next;
    p.n_base = ix.n;
    p.stat_sorted = ix.stat_sorted;
    p.stat_fine = ix.stat_fine;
    p.cell_start = ix.cell_start;
    p.mdo = ix.min_dist_offset;
    p.offsets = ix.offsets;
    p.codes = ix.codes;
    p.codebook = ix.codebook;
    p.counters = s.counters;
    p.d = ix.d;
    p.C = ix.C;
    p.F = ix.F;
    p.nsq = ix.nsq;
    p.lsq = ix.lsq;
    p.code_stride = ix.code_stride;
    p.P = s.P;
    p.T = s.T;
    p.rr = cfg.radius_rate;
    const size_t smem = walk_smem_bytes(ix, s.T);
    ensure_max_dynamic_smem(k_walk_scan, 220 * 1024);
    k_walk_scan<<<n, kThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace pgpu
