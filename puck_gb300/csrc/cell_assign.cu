// Exact nearest-cell assignment of the build (HierarchicalClusterIndex::
// nearest_cell_assign, puck/hierarchical_cluster/hierarchical_cluster_index.cpp:
// 1042-1085, driven by assign :1087-1138): for each point x the cell c * F + f
// with the smallest
//     score = ((0.5|c|^2 - x.c) + 0.5|x|^2 - x.f) + stationary[c][f],
// walking the coarse clusters in ascending (coarse term, id) order and, inside
// each, the fine clusters in index order (descending norm at train time), with the
// reference's break test sqrt(best) - fneg[f] < sqrt(coarse term)
// (fneg[f] = -sqrt(0.5|f|^2)) and its strict-< update (first minimum wins).
//
// Every dot product is the reference's sequential FP32 sum (k_centroid_scores), so
// cells and distances are bit-identical to the sequential walk. The walk itself:
//   * one warp per point; the coarse terms of all C clusters, then the first
//     cluster (the smallest term) walked in full;
//   * after it, best can only decrease, and every test above is monotone in best,
//     so a cluster whose f = 0 test already breaks with the first cluster's best
//     breaks at its turn too and changes nothing; the walk order puts every such
//     cluster after all others. The remaining clusters (usually a handful) are
//     collected, sorted by (term, id) and walked in that order;
//   * a cluster walk takes 32 fine ids per step: each lane's break test uses the
//     best before it, the exclusive prefix minimum over the earlier lanes' scores
//     (the only values that could have changed best), so the first breaking lane
//     and the update are the sequential walk's.
#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr int kWalkWarps = 8;
constexpr uint32_t kMaxNear = 64;  // collected clusters per point before the slow path

// (value, id) as one ordered 64-bit key: float order, then id.
__device__ __forceinline__ uint64_t term_key(float v, uint32_t id) {
    return ((uint64_t)ordered_key(v) << 32) | id;
}

// Walks coarse cluster c (term t) from fine id 0 in order, with the reference's
// break test and strict-< update; best / best_id on every lane.
__device__ __forceinline__ void walk_cluster(uint32_t c, float t, const float* __restrict__ fip,
                                             const float* __restrict__ fneg,
                                             const float* __restrict__ stat, uint32_t F,
                                             float& best, int32_t& best_id) {
    const int lane = threadIdx.x & 31;
    const float st = __fsqrt_rn(t);
    const float* srow = stat + (uint64_t)c * F;
    for (uint32_t f0 = 0; f0 < F; f0 += 32) {
        const uint32_t f = f0 + lane;
        const bool valid = f < F;
        // fip holds -x.f (k_centroid_scores MODE 1): negation is exact
        const float score = valid ? __fadd_rn(__fsub_rn(t, -fip[f]), srow[f]) : FLT_MAX;
        // best before this lane: min(best, scores of the earlier lanes)
        float pre = score;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float u = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= o) pre = fminf(pre, u);
        }
        float before = __shfl_up_sync(0xffffffffu, pre, 1);
        before = lane == 0 ? best : fminf(best, before);
        const bool brk = valid && __fsub_rn(__fsqrt_rn(before), fneg[f]) < st;
        const unsigned bb = __ballot_sync(0xffffffffu, brk);
        const int stop = bb ? __ffs(bb) - 1 : 32;  // lanes < stop are walked
        const bool walked = valid && lane < stop;
        float m = walked ? score : FLT_MAX;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (m < best) {
            // the first walked lane reaching the minimum sets best (strict <)
            const unsigned at = __ballot_sync(0xffffffffu, walked && score == m);
            best = m;
            best_id = (int32_t)(c * F + f0 + (__ffs(at) - 1));
        }
        if (bb) return;
    }
}

// One warp per point. ctm: [rows][C] 0.5|c|^2 - x.c; fip: [rows][F] -x.f; qn: [rows]
// 0.5|x|^2 (all in the reference's sequential order).
__global__ __launch_bounds__(kWalkWarps * 32) void k_cell_walk(
    const float* __restrict__ ctm, const float* __restrict__ fip, const float* __restrict__ qn,
    uint32_t rows, uint32_t C, uint32_t F, const float* __restrict__ fneg,
    const float* __restrict__ stat, uint32_t* __restrict__ cell, float* __restrict__ dist) {
    __shared__ uint64_t near[kWalkWarps][kMaxNear];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * kWalkWarps + warp;
    if (i >= rows) return;  // whole warps only
    const float* cr = ctm + (uint64_t)i * C;
    const float* fr = fip + (uint64_t)i * F;
    const float q = qn[i];
    // the first cluster: smallest (term, id)
    uint64_t kmin = ~0ull;
    for (uint32_t c = lane; c < C; c += 32) {
        const uint64_t k = term_key(__fadd_rn(cr[c], q), c);
        kmin = k < kmin ? k : kmin;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t u = __shfl_xor_sync(0xffffffffu, kmin, o);
        kmin = u < kmin ? u : kmin;
    }
    float best = FLT_MAX;
    int32_t best_id = -1;
    const uint32_t c1 = (uint32_t)kmin;
    walk_cluster(c1, key_to_float((uint32_t)(kmin >> 32)), fr, fneg, stat, F, best, best_id);
    // the clusters whose f = 0 test does not break with this best
    const float th = __fsub_rn(__fsqrt_rn(best), fneg[0]);
    uint32_t cnt = 0;
    for (uint32_t c0 = 0; c0 < C; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool in = false;
        uint64_t k = 0;
        if (c < C && c != c1) {
            const float t = __fadd_rn(cr[c], q);
            in = !(th < __fsqrt_rn(t));
            k = term_key(t, c);
        }
        const unsigned b = __ballot_sync(0xffffffffu, in);
        if (in) {
            const uint32_t pos = cnt + __popc(b & ((1u << lane) - 1));
            if (pos < kMaxNear) near[warp][pos] = k;
        }
        cnt += __popc(b);
    }
    __syncwarp();
    if (cnt <= kMaxNear) {
        // sort the collected keys (at most kMaxNear; odd-even transposition over lanes)
        for (uint32_t r = 0; r < cnt; ++r) {
            for (uint32_t j = 2 * lane + (r & 1); j + 1 < cnt; j += 64) {
                const uint64_t a = near[warp][j], b = near[warp][j + 1];
                if (b < a) {
                    near[warp][j] = b;
                    near[warp][j + 1] = a;
                }
            }
            __syncwarp();
        }
        for (uint32_t r = 0; r < cnt; ++r) {
            const uint64_t k = near[warp][r];
            walk_cluster((uint32_t)k, key_to_float((uint32_t)(k >> 32)), fr, fneg, stat, F, best,
                         best_id);
        }
    } else {
        // many near clusters: take them in order by repeated selection
        uint64_t prev = kmin;
        for (uint32_t r = 0; r < cnt; ++r) {
            uint64_t next = ~0ull;
            for (uint32_t c = lane; c < C; c += 32) {
                const float t = __fadd_rn(cr[c], q);
                const uint64_t k = term_key(t, c);
                if (k > prev && !(th < __fsqrt_rn(t))) next = k < next ? k : next;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t u = __shfl_xor_sync(0xffffffffu, next, o);
                next = u < next ? u : next;
            }
            walk_cluster((uint32_t)next, key_to_float((uint32_t)(next >> 32)), fr, fneg, stat, F,
                         best, best_id);
            prev = next;
        }
    }
    if (lane == 0) {
        cell[i] = (uint32_t)best_id;
        dist[i] = best;
    }
}

// fneg[f] = 0 - sqrt(0.5|f|^2) (hierarchical_cluster_index.cpp:1186-1194)
__global__ void k_fneg(const float* __restrict__ fn, uint32_t F, float* __restrict__ fneg) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < F) fneg[f] = 0.0f - __fsqrt_rn(fn[f]);
}

}  // namespace

cudaError_t launch_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C,
                                       const float* fine, uint32_t F, const float* x, uint64_t n,
                                       uint32_t* cell, float* dist, cudaStream_t stream,
                                       const float* stat_in) {
    if (n == 0) return cudaSuccess;
    // per-chunk scratch of at most 512 MiB for the two term matrices
    uint64_t chunk = (512ull << 20) / (4ull * (C + F) + 4);
    chunk = chunk < 32 ? 32 : (chunk / 32) * 32;
    if (chunk > n) chunk = n;
    if (chunk > 65535ull * 64) chunk = 65535ull * 64;  // the score kernels' grid.y
    float *cn = nullptr, *fn = nullptr, *fneg = nullptr, *stat = nullptr, *ctm = nullptr,
          *fip = nullptr, *qn = nullptr;
    cudaError_t e = cudaMallocAsync(&cn, sizeof(float) * C, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&fn, sizeof(float) * F, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&fneg, sizeof(float) * F, stream);
    if (e == cudaSuccess && stat_in == nullptr)
        e = cudaMallocAsync(&stat, sizeof(float) * (uint64_t)C * F, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&ctm, sizeof(float) * chunk * C, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&fip, sizeof(float) * chunk * F, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&qn, sizeof(float) * chunk, stream);
    if (e == cudaSuccess) e = launch_half_norms(coarse, C, dim, cn, stream);
    if (e == cudaSuccess) e = launch_half_norms(fine, F, dim, fn, stream);
    if (e == cudaSuccess) {
        k_fneg<<<(F + 255) / 256, 256, 0, stream>>>(fn, F, fneg);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && stat_in == nullptr)
        e = launch_stationary(coarse, C, fine, F, dim, fn, stat, stream);
    const float* sp = stat_in ? stat_in : stat;
    for (uint64_t r0 = 0; e == cudaSuccess && r0 < n; r0 += chunk) {
        const uint32_t rows = (uint32_t)(n - r0 < chunk ? n - r0 : chunk);
        const float* xr = x + r0 * dim;
        e = launch_centroid_scores(xr, rows, coarse, C, dim, cn, false, ctm, C, stream);
        if (e == cudaSuccess)
            e = launch_centroid_scores(xr, rows, fine, F, dim, nullptr, true, fip, F, stream);
        if (e == cudaSuccess) e = launch_half_norms(xr, rows, dim, qn, stream);
        if (e == cudaSuccess) {
            k_cell_walk<<<(rows + kWalkWarps - 1) / kWalkWarps, kWalkWarps * 32, 0, stream>>>(
                ctm, fip, qn, rows, C, F, fneg, sp, cell + r0, dist + r0);
            e = cudaGetLastError();
        }
    }
    for (float* p : {cn, fn, fneg, stat, ctm, fip, qn})
        if (p) cudaFreeAsync(p, stream);
    return e;
}

}  // namespace pgpu
