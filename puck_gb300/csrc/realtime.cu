// Realtime insert on the device: RealtimeInsertPuckIndex
// (puck/puck/realtime_insert_puck_index.cpp) over a loaded index.
//
// The reference keeps inserted points in their own memory groups and, per fine
// cell, a list of them newest first (InsertFineCluster, :398-453); its searches
// scan a cell's base records (with the walk's break) and then every inserted point
// of the cell, with memory id n + insert id. Here:
//   * every per-record device array (filter offsets and codes, the scan's
//     interleaved code copy, fine ids, the vectors or the second-level PQ records, the memory ->
//     local map, the BF16 copy) is widened once, at open, to n + capacity rows, and
//     an inserted point's records are written to row n + insert id; nothing that
//     reads a record by memory id needs to know whether it was inserted;
//   * per cell, the newest insert (ins_head) and a link to the next older one
//     (ins_next): the exact walk's order (walk_scan.cu);
//   * per coarse cluster, its inserted memory ids (ins_cl_start / ins_cl_ids): the
//     scan's extra records of a probed cluster (scan_select.cu).
// An insert is single_build (normalisation, the nearest cell on the index's live
// stationary terms, hierarchical_cluster_index.cpp:1455-1494) and
// puck_single_assign (puck_index.cpp:938-988), i.e. launch_nearest_cell_assign and
// the build's encoder for one point; a cell whose count becomes 1 gets the
// stationary term c.f - f.f (:322-333). Each cell's count starts at its base count,
// so only a cell empty in the base is rewritten, and it is chosen only if its
// sqrt(FLT_MAX) stationary term still wins; a batch is cut there and assigned again
// after the rewrite, so batches give the one-at-a-time results.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

template <class T>
cudaError_t grow(T** p, uint64_t old_count, uint64_t new_count, uint64_t* bytes) {
    if (*p == nullptr) return cudaSuccess;
    T* q = nullptr;
    cudaError_t e = cudaMalloc((void**)&q, sizeof(T) * (new_count ? new_count : 1));
    if (e != cudaSuccess) return e;
    if (old_count) e = cudaMemcpy(q, *p, sizeof(T) * old_count, cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
        cudaFree(q);
        return e;
    }
    cudaFree(*p);
    *p = q;
    *bytes += sizeof(T) * (new_count - old_count);
    return cudaSuccess;
}

// Records of m inserted points into rows base_row + i of the index's arrays: filter
// offset and codes (packed nsq bytes -> code_stride rows),
// fine id, memory -> local id, second-level PQ, vector.
__global__ void k_ins_records(uint32_t m, uint64_t base_row, const uint32_t* __restrict__ cell,
                              uint32_t F, const float* __restrict__ f_off,
                              const uint8_t* __restrict__ f_codes, uint32_t nsq, uint32_t stride,
                              const float* __restrict__ p_off, const uint8_t* __restrict__ p_codes,
                              uint32_t pnsq, uint32_t pstride, const float* __restrict__ x,
                              uint32_t d, DeviceIndex ix) {
    const uint32_t i = blockIdx.x;
    if (i >= m) return;
    const uint64_t r = base_row + i;
    const int t = threadIdx.x;
    if (t == 0) {
        ix.offsets[r] = f_off[i];
        ix.rec_fine[r] = (uint16_t)(cell[i] % F);
        ix.mem2local[r] = (uint32_t)r;
        if (pnsq) ix.pq_offsets[r] = p_off[i];
    }
    for (uint32_t s = t; s < stride; s += blockDim.x)
        ix.codes[r * stride + s] = s < nsq ? f_codes[(uint64_t)i * nsq + s] : 0;
    for (uint32_t s = t; pnsq && s < pstride; s += blockDim.x)
        ix.pq_codes[r * pstride + s] = s < pnsq ? p_codes[(uint64_t)i * pnsq + s] : 0;
    if (ix.feat) {
        for (uint32_t k = t; k < d; k += blockDim.x) ix.feat[r * d + k] = x[(uint64_t)i * d + k];
    }
}

// stationary[cell] = c.f - f.f, each dot sequential (realtime_insert_puck_index.cpp:322-333)
__global__ void k_rewrite_stationary(const float* __restrict__ coarse,
                                     const float* __restrict__ fine, uint32_t d, uint32_t F,
                                     uint32_t cell, float* __restrict__ stationary) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float* c = coarse + (uint64_t)(cell / F) * d;
    const float* f = fine + (uint64_t)(cell % F) * d;
    stationary[cell] = __fsub_rn(dot_seq(c, f, d), dot_seq(f, f, d));
}

__global__ void k_set_i32(int32_t* __restrict__ a, const uint32_t* __restrict__ at,
                          const int32_t* __restrict__ v, uint32_t m) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) a[at[i]] = v[i];
}

}  // namespace

int realtime_open(DeviceIndex* ix, RealtimeHost* rh, uint32_t cap, std::string* err) {
    if (ix->ins_cap != 0) {
        *err = "the index is already open for inserts";
        return PGPU_E_INVALID;
    }
    if (cap == 0 || (uint64_t)ix->n + cap > 0xFFFFFFFEull) {
        *err = "capacity must be in [1, 2^32 - 2 - point count]";
        return PGPU_E_LIMIT;
    }
    const uint64_t n = ix->n, N = n + cap, cells = (uint64_t)ix->C * ix->F;
    uint64_t bytes = 0;
    cudaError_t e = cudaDeviceSynchronize();
#define PGPU_GROW(ptr, per)                                         \
    if (e == cudaSuccess) e = grow(&(ptr), n * (per), N * (per), &bytes);
    PGPU_GROW(ix->offsets, 1);
    PGPU_GROW(ix->codes, ix->code_stride);
    if (e == cudaSuccess)
        e = grow(&ix->codes_il, il_bytes(n, ix->nsq), il_bytes(N, ix->nsq), &bytes);
    PGPU_GROW(ix->rec_fine, 1);
    PGPU_GROW(ix->mem2local, 1);
    PGPU_GROW(ix->feat, ix->d);
    PGPU_GROW(ix->feat_bf16, ix->d);
    PGPU_GROW(ix->feat_abs, 1);
    PGPU_GROW(ix->pq_offsets, 1);
    PGPU_GROW(ix->pq_codes, ix->pq_code_stride);
#undef PGPU_GROW
    auto dalloc = [&](void** p, uint64_t b) {
        if (e == cudaSuccess) e = cudaMalloc(p, b ? b : 1);
        if (e == cudaSuccess) bytes += b;
    };
    dalloc((void**)&ix->ins_head, sizeof(int32_t) * cells);
    dalloc((void**)&ix->ins_next, sizeof(int32_t) * cap);
    dalloc((void**)&ix->ins_cl_start, sizeof(uint32_t) * (ix->C + 1ull));
    dalloc((void**)&ix->ins_cl_ids, sizeof(uint32_t) * cap);
    if (e == cudaSuccess) e = cudaMemset(ix->ins_head, 0xFF, sizeof(int32_t) * cells);
    if (e == cudaSuccess) e = cudaMemset(ix->ins_cl_start, 0, sizeof(uint32_t) * (ix->C + 1ull));
    std::vector<uint32_t> cs(cells + 1);
    if (e == cudaSuccess)
        e = cudaMemcpy(cs.data(), ix->cell_start, sizeof(uint32_t) * (cells + 1),
                       cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        *err = std::string("realtime open: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
    }
    rh->head.assign(cells, -1);
    rh->next.clear();
    rh->cluster.clear();
    rh->cnt.resize(cells);
    for (uint64_t c = 0; c < cells; ++c) rh->cnt[c] = cs[c + 1] - cs[c];
    ix->ins_cap = cap;
    ix->ins_n = 0;
    ix->bytes += bytes;
    return PGPU_OK;
}

int realtime_insert(DeviceIndex* ix, RealtimeHost* rh, uint32_t m, const float* x,
                    const int32_t* ok, int64_t* ids, cudaStream_t st, std::string* err) {
    const uint32_t d = ix->d, F = ix->F;
    uint32_t valid = 0;
    for (uint32_t i = 0; i < m; ++i) valid += ok[i] ? 1u : 0u;
    if ((uint64_t)ix->ins_n + valid > ix->ins_cap) {
        *err = "insert capacity exceeded";
        return PGPU_E_LIMIT;
    }
    // the valid rows, packed, in order
    std::vector<uint32_t> rows;
    for (uint32_t i = 0; i < m; ++i)
        if (ok[i]) rows.push_back(i);
    for (uint32_t i = 0; i < m; ++i) ids[i] = -1;
    if (rows.empty()) return PGPU_OK;
    const uint32_t v = (uint32_t)rows.size();
    const uint32_t fnsq = ix->nsq, pnsq = ix->pq_nsq;
    float *xs = nullptr, *dist = nullptr, *f_off = nullptr, *p_off = nullptr;
    uint32_t *cell = nullptr, *at = nullptr;
    int32_t* val = nullptr;
    uint8_t *f_codes = nullptr, *p_codes = nullptr;
    cudaError_t e = cudaSuccess;
    auto dalloc = [&](void** p, uint64_t b) {
        if (e == cudaSuccess) e = cudaMallocAsync(p, b ? b : 1, st);
    };
    dalloc((void**)&xs, sizeof(float) * (uint64_t)v * d);
    dalloc((void**)&dist, sizeof(float) * v);
    dalloc((void**)&cell, sizeof(uint32_t) * v);
    dalloc((void**)&f_off, sizeof(float) * v);
    dalloc((void**)&f_codes, (uint64_t)v * fnsq);
    dalloc((void**)&p_off, sizeof(float) * v);
    dalloc((void**)&p_codes, (uint64_t)v * (pnsq ? pnsq : 1));
    dalloc((void**)&at, sizeof(uint32_t) * ((uint64_t)v + ix->C + 1));
    dalloc((void**)&val, sizeof(int32_t) * v);
    for (uint32_t j = 0; e == cudaSuccess && j < v; ++j)
        e = cudaMemcpyAsync(xs + (uint64_t)j * d, x + (uint64_t)rows[j] * d, sizeof(float) * d,
                            cudaMemcpyDeviceToDevice, st);
    std::vector<uint32_t> hcell(v);
    uint32_t done = 0;
    int rc = PGPU_OK;
    while (e == cudaSuccess && rc == PGPU_OK && done < v) {
        // cells of the remaining points on the live stationary terms
        const uint32_t rest = v - done;
        e = launch_nearest_cell_assign(d, ix->coarse, ix->C, ix->fine, F, xs + (uint64_t)done * d,
                                       rest, cell + done, dist + done, st, ix->stationary);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hcell.data() + done, cell + done, sizeof(uint32_t) * rest,
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        uint32_t next_done = v;
        for (uint32_t j = done; j < v; ++j) {
            const uint32_t c = hcell[j];
            if (c >= (uint64_t)ix->C * F) {
                *err = "no cell found for an inserted point";
                rc = PGPU_E_INVALID;
                break;
            }
            if (++rh->cnt[c] == 1) {
                // the cell was empty: its stationary term changes for the later points
                k_rewrite_stationary<<<1, 32, 0, st>>>(ix->coarse, ix->fine, d, F, c,
                                                       ix->stationary);
                e = cudaGetLastError();
                // the exact walk's ascending stationary row of that coarse cluster
                const uint64_t row = (uint64_t)(c / F) * F;
                if (e == cudaSuccess)
                    e = launch_topsort(ix->stationary + row, 1, F, F, F, ix->stat_sorted + row,
                                       ix->stat_fine + row, st);
                next_done = j + 1;
                break;
            }
        }
        done = next_done;
    }
    if (e == cudaSuccess && rc == PGPU_OK) {
        // the build's encoder for the inserted points (puck_single_assign)
        rc = pgpu_puck_assign(d, v, xs, cell, ix->coarse, ix->C, ix->fine, F, ix->codebook, fnsq,
                              pnsq ? ix->pq_codebook : nullptr, pnsq, f_off, f_codes,
                              pnsq ? p_off : nullptr, pnsq ? p_codes : nullptr, st);
        if (rc != PGPU_OK) *err = std::string("encoder: ") + pgpu_last_error();
    }
    const uint64_t row0 = (uint64_t)ix->n + ix->ins_n;
    if (e == cudaSuccess && rc == PGPU_OK) {
        k_ins_records<<<v, 128, 0, st>>>(v, row0, cell, F, f_off, f_codes, fnsq, ix->code_stride,
                                         p_off, p_codes, pnsq, ix->pq_code_stride, xs, d, *ix);
        e = cudaGetLastError();
        if (e == cudaSuccess && ix->codes_il)
            e = launch_interleave_codes(*ix, row0, v, st);
        if (e == cudaSuccess && ix->feat_bf16)
            e = launch_bf16_rows(ix->feat + row0 * d, v, d, ix->feat_bf16 + row0 * d,
                                 ix->feat_abs + row0, st);
    }
    if (e == cudaSuccess && rc == PGPU_OK) {
        // the cells' lists (newest first) and the clusters' inserted ids
        std::vector<uint32_t> hat;
        std::vector<int32_t> hval;
        for (uint32_t j = 0; j < v; ++j) {
            const uint32_t id = ix->ins_n + j;
            rh->next.push_back(rh->head[hcell[j]]);
            rh->head[hcell[j]] = (int32_t)id;
            rh->cluster.push_back(hcell[j] / F);
            ids[rows[j]] = (int64_t)ix->n + id;
        }
        hat = hcell;  // each touched cell's final head, once
        std::sort(hat.begin(), hat.end());
        hat.erase(std::unique(hat.begin(), hat.end()), hat.end());
        for (uint32_t c : hat) hval.push_back(rh->head[c]);
        const uint32_t total = ix->ins_n + v;
        std::vector<uint32_t> cl_start(ix->C + 1, 0), cl_ids(total);
        for (uint32_t id = 0; id < total; ++id) ++cl_start[rh->cluster[id] + 1];
        for (uint32_t c = 0; c < ix->C; ++c) cl_start[c + 1] += cl_start[c];
        {
            std::vector<uint32_t> fill(cl_start.begin(), cl_start.end() - 1);
            for (uint32_t id = 0; id < total; ++id) cl_ids[fill[rh->cluster[id]]++] = ix->n + id;
        }
        // uploads (synchronous: the host vectors are temporaries)
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess)
            e = cudaMemcpy(ix->ins_next + ix->ins_n, rh->next.data() + ix->ins_n,
                           sizeof(int32_t) * v, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(ix->ins_cl_start, cl_start.data(), sizeof(uint32_t) * (ix->C + 1ull),
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(ix->ins_cl_ids, cl_ids.data(), sizeof(uint32_t) * total,
                           cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(at, hat.data(), sizeof(uint32_t) * hat.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(val, hval.data(), sizeof(int32_t) * hval.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            k_set_i32<<<(unsigned)((hat.size() + 255) / 256), 256, 0, st>>>(
                ix->ins_head, at, val, (uint32_t)hat.size());
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) ix->ins_n = total;
    }
    for (void* p : {(void*)xs, (void*)dist, (void*)cell, (void*)f_off, (void*)f_codes,
                    (void*)p_off, (void*)p_codes, (void*)at, (void*)val})
        if (p) cudaFreeAsync(p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (rc != PGPU_OK) return rc;
    if (e != cudaSuccess) {
        *err = std::string("insert: ") + cudaGetErrorString(e);
        return PGPU_E_CUDA;
    }
    return PGPU_OK;
}

}  // namespace pgpu
