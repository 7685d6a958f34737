// The throughput-mode filter stage (scan mode). For one query it streams every
// filter record of its probed coarse clusters (each cluster is one contiguous
// range in memory order) and keeps the filter_topk smallest ADC distances. Three
// kernels: the split scan (k_scan_score, "split scan" below), which answers every
// query whose records fit the per-pass distance buffer; the fused k_scan_il
// (interleaved layout) for the rest; k_scan_select for nsq not a multiple of 4.
//
// Per record the distance is the reference's own expression for a scanned point
// (puck/puck/puck_index.cpp:360-368 with cell_dist from :539-540):
//     cell_dist = (coarse_term + stationary[c][f]) + fine_term[f]
//     t         = (float)(2 * cell_dist + offset) + lookup_dist_table(codes)
// so every t is bit-identical to the value PuckIndex::search would compute for
// that point. Unlike the reference's pivot-pruned cell walk, no cell of a probed
// cluster is skipped: the result is the exact top-filter_topk by (t, memory id)
// over all records of the probed clusters, a superset search of the same cells.
//
// Table: each block builds its query's table in shared memory
// (get_dist_table, quantization.cpp:260-270, in the reference's lane order):
// thread j computes codeword j of every subspace from one coalesced 16-byte
// codebook load per subspace (the codebook stays in L2).
//
// Selection: a buffer of (t, id) keys in shared memory, sized from filter_topk,
// with a running threshold tau, a key with at least filter_topk kept keys below
// it; records whose (2*cell_dist + offset, id) key is not below tau are dropped
// before the table lookups (t can only grow). When the buffer could not take
// another round, one histogram pass over the buffer's float values (1024 linear
// bins between the smallest and the largest) finds the bin holding the
// filter_topk-th key; the keys above that bin are dropped and tau becomes the
// bin's upper edge. A last exact radix select leaves the set of the filter_topk
// smallest (t, id) keys, unordered.
//
// Blocks start in launch order longest scan first (k_scan_work, k_scan_order),
// one block per query.
//
// Precision form (FP16 tables): the table is stored in FP16, scaled per query by a
// power of two 2^e chosen from the bound (|q| + max |codeword|)^2 >= every entry
// so that all entries stay below 32768; lookups are accumulated in FP32 and the
// sum is multiplied by 2^-e. Entries are non-negative, so t >= t0 still holds and
// the threshold test before the lookups stays valid.
//
// Interleaved kernel (k_scan_il; nsq a multiple of 4, at most 32: every index
// the library builds for its configurations). The codes come from the interleaved
// copy (DeviceIndex::codes_il, pgpu_internal.h): record r's codes rotated by
// l = r & 31, its lane in a block of 32 records. Thread t of a round takes the
// records whose memory id is congruent to t mod 32, so every 8-byte code load of a
// warp reads one whole 256-byte line, and at lookup step s lane l reads table
// column s + l. The table holds, for each code c (a row) and each column
// m' < nsq + 31, the entry of subspace m' mod nsq at word c * 64 + m' (FP32) or
// half c * 64 + m' (FP16): the 32 lanes of a warp read 32 distinct banks at every
// lookup, whatever the codes (the reference's [subspace][code] table costs about
// 3.4 shared-memory wavefronts per warp-wide lookup of random codes). A lookup is
// one PRMT (the address (c << 8) | 4l from the code word and the lane), one load
// and one add. The sum runs in the rotated order: lookup step s goes to partial
// s mod 4, and t = t0 + ((a0 + a1) + (a2 + a3)), FP32 throughout; the oracle's
// scan mode restates that order (the reference's own order, partial m mod 4 over
// subspaces m, holds for the other kernel, k_scan_select). This kernel has no
// threshold test before the lookups: t0 lacks the table's |q|^2 share, so the test
// passes for almost every record. Loads are double-buffered: a round's records are
// fetched while the previous round is scored.
#include <cuda_fp16.h>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

// Block shape of the scan (compile-time; -D overrides for tuning sweeps).
#ifndef PGPU_SCAN_THREADS
#define PGPU_SCAN_THREADS 256
#endif
#ifndef PGPU_SCAN_RECORDS
#define PGPU_SCAN_RECORDS 4
#endif
#ifndef PGPU_SCAN_MIN_BLOCKS
#define PGPU_SCAN_MIN_BLOCKS 3
#endif
constexpr int kThreads = PGPU_SCAN_THREADS;
constexpr int kRecPerThread = PGPU_SCAN_RECORDS;
constexpr int kRound = kThreads * kRecPerThread;  // records per round
// Candidate buffer: at most kMaxCap keys (kCapPer per thread in the compaction);
// sized per launch from filter_topk (scan_cap).
constexpr int kCapPer = 16;
constexpr uint32_t kMaxCap = kThreads * kCapPer;
constexpr uint32_t kHistBins = 1024;  // bins of the cut-back histogram
static_assert(kHistBins % kThreads == 0, "bins split evenly over the threads");

// Buffer size for filter_topk T: T + a round + room for max(1024, T) more keys
// before the next cut, in whole multiples of the block, at most kMaxCap.
__host__ __device__ inline uint32_t scan_cap(uint32_t T) {
    uint32_t room = T > 1024 ? T : 1024;
    uint32_t c = T + kRound + room;
    c = (c + kThreads - 1) / kThreads * kThreads;
    return c > kMaxCap ? kMaxCap : c;
}

struct ScanParams {
    const float* q;
    const float* qnorm;
    const int32_t* status;
    const float* cdist;
    const uint32_t* ctag;
    const float* fd_by_fine;  // [B][F]
    float* hdist;
    uint32_t* htag;
    uint32_t* hcnt;
    const float* stationary;  // [C][F]
    const uint32_t* cell_start;
    const uint16_t* rec_fine; // [n] fine id of each record
    const float* offsets;
    const uint8_t* codes;
    const uint8_t* codes_il;    // interleaved copy (k_scan_il)
    const float* codebook;
    unsigned long long* counters;
    const uint32_t* order;      // [B] query of each block
    int* err;                   // set when a bulk copy's wait expired
    const uint32_t* ins_cl_start;  // realtime: [C+1] inserted records per cluster, or null
    const uint32_t* ins_cl_ids;    // their memory ids
    const uint32_t* done;          // [B] 1: the split scan has answered the query, or null
    uint32_t d, C, F, nsq, lsq, code_stride, P, T, cap;
    float codebook_max;
};

// Power-of-two scale of the FP16 table: 2^e with every entry * 2^e < 32768, from
// the bound (|q| + max |codeword|)^2 on |q_m - c|^2.
__device__ __forceinline__ int half_lut_exponent(float qnorm, float codebook_max) {
    const float qa = sqrtf(qnorm) + codebook_max;
    const float bound = qa * qa * 1.0001f + 1e-30f;
    int e = (int)floorf(log2f(32768.0f / bound));
    return e < -60 ? -60 : (e > 60 ? 60 : e);
}

// get_dist_table (quantization.cpp:260-270) for one query into shared memory:
// thread j computes codeword j of every subspace (one coalesced 16-byte codebook
// load per subspace when lsq = 4), in the reference's lane order (l2sqr_sse).
// Table variants: FP32 (the reference's values and order), FP16 in the same
// layout, FP16 in the rotated one-bank-per-subspace layout.
enum { kTabF32 = 0, kTabF16 = 1 };

template <int TAB>
__device__ __forceinline__ void build_table(void* lut, const float* qv,
                                            const float* __restrict__ cb, uint32_t nsq,
                                            uint32_t lsq, float scale) {
    for (uint32_t j = threadIdx.x; j < 256; j += kThreads) {
        auto store = [&](uint32_t m, float v) {
            if (TAB == kTabF16)
                reinterpret_cast<__half*>(lut)[m * 256 + j] = __float2half_rn(v * scale);
            else
                reinterpret_cast<float*>(lut)[m * 256 + j] = v;
        };
        if (lsq == 4) {
            const float4* cb4 = reinterpret_cast<const float4*>(cb);
            for (uint32_t m0 = 0; m0 < nsq; m0 += 8) {
                float4 y[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (m0 + u < nsq) y[u] = __ldg(cb4 + (uint64_t)(m0 + u) * 256 + j);
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const uint32_t m = m0 + u;
                    if (m >= nsq) break;
                    const float* x = qv + m * 4;
                    const float t0 = __fsub_rn(x[0], y[u].x), t1 = __fsub_rn(x[1], y[u].y);
                    const float t2 = __fsub_rn(x[2], y[u].z), t3 = __fsub_rn(x[3], y[u].w);
                    store(m, __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)),
                                       __fadd_rn(__fmul_rn(t2, t2), __fmul_rn(t3, t3))));
                }
            }
        } else {
            for (uint32_t m = 0; m < nsq; ++m)
                store(m, l2sqr_sse(qv + m * lsq, cb + ((uint64_t)m * 256 + j) * lsq, lsq));
        }
    }
}

template <int NW>
__device__ __forceinline__ float lut_sum_words_half(const uint32_t (&w)[NW], const __half* lut,
                                                    uint32_t nsq) {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        const uint32_t m = 4u * i;
        if (m >= nsq) break;
        const uint32_t c = w[i];
        a0 += __half2float(lut[(m + 0) * 256 + (c & 0xff)]);
        if (m + 1 < nsq) a1 += __half2float(lut[(m + 1) * 256 + ((c >> 8) & 0xff)]);
        if (m + 2 < nsq) a2 += __half2float(lut[(m + 2) * 256 + ((c >> 16) & 0xff)]);
        if (m + 3 < nsq) a3 += __half2float(lut[(m + 3) * 256 + (c >> 24)]);
    }
    return (a0 + a1) + (a2 + a3);
}

__device__ __forceinline__ float key_value(uint64_t k) {
    uint32_t b = (uint32_t)(k >> 32);
    b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    return __uint_as_float(b);
}

constexpr uint64_t kKeyMax = ~0ull;

// The K-th smallest (1-based) of keys[0..count), all distinct: MSB-first radix
// select with 8-bit digits, stopping as soon as the chosen digit's bucket holds
// one key (usually after the 2nd or 3rd digit of the float). `hist` has 256
// slots, `sel` 4. All threads call it.
// max_digits > 0 stops after that many digit passes and returns the largest key of
// the bucket reached: then at least K keys are <= the result (a cut-back bound, not
// the K-th itself).
template <int NT>
__device__ uint64_t block_select_kth(const uint64_t* keys, uint32_t count, uint32_t K,
                                     uint32_t* hist, uint64_t* sel, int max_digits = 0) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the leading bits every key shares need no pass: start at the digit where the
    // smallest and the largest key first differ
    uint64_t lo = ~0ull, hi = 0;
    for (uint32_t i = tid; i < count; i += NT) {
        const uint64_t x = keys[i];
        lo = x < lo ? x : lo;
        hi = x > hi ? x : hi;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t a = __shfl_xor_sync(0xffffffffu, lo, o);
        const uint64_t b = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    __shared__ uint64_t red_lo[NT / 32], red_hi[NT / 32];
    if (lane == 0) {
        red_lo[warp] = lo;
        red_hi[warp] = hi;
    }
    __syncthreads();
    lo = red_lo[0];
    hi = red_hi[0];
    for (int w = 1; w < NT / 32; ++w) {
        lo = red_lo[w] < lo ? red_lo[w] : lo;
        hi = red_hi[w] > hi ? red_hi[w] : hi;
    }
    __syncthreads();
    int top = 56;
    if (lo != hi) {
        const int msb = 63 - __clzll((long long)(lo ^ hi));
        top = (msb / 8) * 8;
    } else {
        top = 0;
    }
    uint64_t mask = top >= 56 ? 0ull : ~((1ull << (top + 8)) - 1);
    uint64_t prefix = lo & mask;
    uint32_t k = K;
    for (int shift = top; shift >= 0; shift -= 8) {
        for (int i = tid; i < 256; i += NT) hist[i] = 0;
        __syncthreads();
        for (uint32_t i0 = 0; i0 < count; i0 += NT) {
            const uint32_t i = i0 + tid;
            bool in = false;
            uint32_t digit = 0;
            if (i < count) {
                const uint64_t key = keys[i];
                in = (key & mask) == prefix;
                digit = (uint32_t)(key >> shift) & 255u;
            }
            // one atomic per distinct digit in the warp
            const unsigned active = __ballot_sync(0xffffffffu, in);
            if (in) {
                const unsigned same = __match_any_sync(active, digit);
                if (lane == __ffs(same) - 1) atomicAdd(&hist[digit], (uint32_t)__popc(same));
            }
        }
        __syncthreads();
        if (tid < 32) {
            // digit d with (count below d) < k <= (count up to d)
            uint32_t c[8], run = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                c[j] = hist[tid * 8 + j];
                run += c[j];
            }
            uint32_t incl = run;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += u;
            }
            uint32_t below = incl - run;
            if (below < k && k <= incl) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (below < k && k <= below + c[j]) {
                        sel[0] = (uint64_t)(tid * 8 + j);
                        sel[1] = k - below;
                        sel[2] = c[j];
                    }
                    below += c[j];
                }
            }
        }
        __syncthreads();
        prefix |= sel[0] << shift;
        mask |= 255ull << shift;
        k = (uint32_t)sel[1];
        const bool unique = sel[2] == 1;
        __syncthreads();
        if (!unique && max_digits > 0 && --max_digits == 0 && shift > 0)
            return prefix | ~mask;
        if (unique && shift > 0) {
            // the one key under this prefix is the K-th
            for (uint32_t i = tid; i < count; i += NT)
                if ((keys[i] & mask) == prefix) sel[3] = keys[i];
            __syncthreads();
            const uint64_t r = sel[3];
            __syncthreads();
            return r;
        }
    }
    return prefix;
}

// Cut-back bound of the buffer: keys[0..count) hold at least K keys. One pass
// of a kHistBins-bin histogram of the keys' float parts, linear between the
// smallest and the largest, finds the bin holding the K-th smallest; the result
// is the (exclusive) upper edge of that bin as a key: at least K keys lie below
// it, and only the keys of that one bin above the K-th are kept in excess.
// Returns kKeyMax when the float parts are all equal (no cut possible). `hist`
// has kHistBins slots, `red` 2 * (kThreads / 32) + 2. All threads call it.
template <int NT>
__device__ uint64_t block_cut_bound(const uint64_t* keys, uint32_t count, uint32_t K,
                                    uint32_t* hist, uint32_t* red) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kW = NT / 32;
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    for (uint32_t i = tid; i < count; i += NT) {
        const uint32_t h = (uint32_t)(keys[i] >> 32);
        lo = h < lo ? h : lo;
        hi = h > hi ? h : hi;
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
        red[warp] = lo;
        red[kW + warp] = hi;
    }
    for (uint32_t b = tid; b < kHistBins; b += NT) hist[b] = 0;
    __syncthreads();
    lo = red[0];
    hi = red[kW];
#pragma unroll
    for (int w = 1; w < kW; ++w) {
        lo = red[w] < lo ? red[w] : lo;
        hi = red[kW + w] > hi ? red[kW + w] : hi;
    }
    if (lo == hi) {
        __syncthreads();
        return kKeyMax;
    }
    int shift = 0;
    while (((hi - lo) >> shift) >= kHistBins) ++shift;
    for (uint32_t i = tid; i < count; i += NT)
        atomicAdd(&hist[((uint32_t)(keys[i] >> 32) - lo) >> shift], 1u);
    __syncthreads();
    // thread t owns bins [t * per, (t + 1) * per): the bin where the running count reaches K
    constexpr uint32_t per = kHistBins / NT;
    uint32_t c[per], run = 0;
#pragma unroll
    for (uint32_t j = 0; j < per; ++j) {
        c[j] = hist[tid * per + j];
        run += c[j];
    }
    uint32_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) red[warp] = incl;  // red's min/max were read before the histogram barrier
    __syncthreads();
    uint32_t below = incl - run;
    for (int w = 0; w < warp; ++w) below += red[w];
    if (below < K && K <= below + run) {
#pragma unroll
        for (uint32_t j = 0; j < per; ++j) {
            if (below < K && K <= below + c[j]) red[2 * kW + 1] = tid * per + j;
            below += c[j];
        }
    }
    __syncthreads();
    const uint32_t bin = red[2 * kW + 1];
    __syncthreads();
    const uint64_t edge = (uint64_t)lo + ((uint64_t)(bin + 1) << shift);
    return edge > 0xFFFFFFFFull ? kKeyMax : (edge << 32);
}

// The K-th smallest (1-based) of keys[0..count), all distinct, K <= count: one
// histogram pass of kHistBins linear bins over the keys' float parts (as
// block_cut_bound) finds the bin holding the K-th; the keys of that bin (at most
// kHistBins / 2 of them: `hist` then holds them as 64-bit keys) are ranked by
// counting, and the one of rank K - (keys below the bin) is the result. A bin
// holding more keys, or all float parts equal, goes to block_select_kth. `red` has
// 2 * (NT / 32) + 2 slots, `cnt` is a shared counter. All threads call it.
template <int NT>
__device__ uint64_t block_kth_hist(const uint64_t* keys, uint32_t count, uint32_t K, uint32_t* hist,
                                   uint32_t* red, uint32_t* cnt, uint32_t* hist256, uint64_t* sel) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kW = NT / 32;
    uint32_t lo = 0xFFFFFFFFu, hi = 0;
    for (uint32_t i = tid; i < count; i += NT) {
        const uint32_t h = (uint32_t)(keys[i] >> 32);
        lo = h < lo ? h : lo;
        hi = h > hi ? h : hi;
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
        red[warp] = lo;
        red[kW + warp] = hi;
    }
    for (uint32_t b = tid; b < kHistBins; b += NT) hist[b] = 0;
    if (tid == 0) *cnt = 0;
    __syncthreads();
    lo = red[0];
    hi = red[kW];
#pragma unroll
    for (int w = 1; w < kW; ++w) {
        lo = red[w] < lo ? red[w] : lo;
        hi = red[kW + w] > hi ? red[kW + w] : hi;
    }
    if (lo == hi) {
        __syncthreads();
        return block_select_kth<NT>(keys, count, K, hist256, sel);
    }
    int shift = 0;
    while (((hi - lo) >> shift) >= kHistBins) ++shift;
    for (uint32_t i = tid; i < count; i += NT)
        atomicAdd(&hist[((uint32_t)(keys[i] >> 32) - lo) >> shift], 1u);
    __syncthreads();
    constexpr uint32_t per = kHistBins / NT;
    uint32_t c[per], run = 0;
#pragma unroll
    for (uint32_t j = 0; j < per; ++j) {
        c[j] = hist[tid * per + j];
        run += c[j];
    }
    uint32_t incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) red[warp] = incl;
    __syncthreads();
    uint32_t below = incl - run;
    for (int w = 0; w < warp; ++w) below += red[w];
    if (below < K && K <= below + run) {
#pragma unroll
        for (uint32_t j = 0; j < per; ++j) {
            if (below < K && K <= below + c[j]) {
                red[2 * kW] = tid * per + j;  // the bin
                red[2 * kW + 1] = below;      // keys below it
                sel[0] = c[j];                // keys in it
            }
            below += c[j];
        }
    }
    __syncthreads();
    const uint32_t bin = red[2 * kW], nbelow = red[2 * kW + 1], m = (uint32_t)sel[0];
    if (m > kHistBins / 2) {
        __syncthreads();
        return block_select_kth<NT>(keys, count, K, hist256, sel);
    }
    // the bin's keys into hist (as 64-bit keys), then the one of rank K - nbelow
    uint64_t* bk = reinterpret_cast<uint64_t*>(hist);
    for (uint32_t i = tid; i < count; i += NT) {
        const uint64_t k = keys[i];
        if ((((uint32_t)(k >> 32) - lo) >> shift) == bin) bk[atomicAdd(cnt, 1u)] = k;
    }
    __syncthreads();
    const uint32_t want = K - nbelow - 1;  // 0-based rank in the bin
    for (uint32_t i = tid; i < m; i += NT) {
        const uint64_t k = bk[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < m; ++j) rank += bk[j] < k ? 1u : 0u;
        if (rank == want) sel[1] = k;
    }
    __syncthreads();
    const uint64_t r = sel[1];
    __syncthreads();
    return r;
}

// Keeps the keys < bound at the front (in arbitrary order); returns their count.
// `cnt` is a shared counter. All threads call it.
template <int NT, int PER = (int)(kMaxCap / NT)>
__device__ uint32_t block_compact_lt(uint64_t* keys, uint32_t count, uint64_t bound, uint32_t* cnt) {
    const int tid = threadIdx.x, lane = tid & 31;
    uint64_t mine[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const uint32_t i = tid + j * NT;
        mine[j] = i < count ? keys[i] : ~0ull;
    }
    if (tid == 0) *cnt = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const bool keep = mine[j] < bound;
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        uint32_t base = 0;
        if (b) {
            if (lane == __ffs(b) - 1) base = atomicAdd(cnt, (uint32_t)__popc(b));
            base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
        }
        if (keep) keys[base + __popc(b & ((1u << lane) - 1))] = mine[j];
    }
    __syncthreads();
    const uint32_t r = *cnt;
    __syncthreads();
    return r;
}

// Diagnostic counters (pgpu_walk_counters slots, summed per launch): 0 records
// evaluated, 1 records past the cell-distance test (table lookups), 2 records kept, 3 compactions, 5 max records of one query, and
// thread-0 clock cycles: 6 prologue (table, query), 7 whole block, 8 record
// rounds, 9 compactions, 10 final select + output.
enum { kScRecords = 0, kScLookups = 1, kScKept = 2, kScCompactions = 3, kScMaxRecords = 5, kScCycPrologue = 6,
       kScCycTotal = 7, kScCycRounds = 8, kScCycCompact = 9, kScCycFinal = 10 };

struct ScanState {
    uint64_t tau;
    uint64_t sel[4];
    uint32_t hist[256];
    uint32_t red[2 * (512 / 32) + 2];  // for blocks of up to 512 threads
    uint32_t ccount;
    uint32_t count;
    uint32_t c;
    float cdl;
    uint32_t r0, r1, i0, i1;
    unsigned long long evaluated, looked, passed;
    unsigned long long cyc_rounds, cyc_compact, n_compact, n_records;
};

// Slot l of query qi's probed clusters into st (all threads; barriers on both
// sides): false when the slot is empty (the probed clusters fill a prefix).
__device__ __forceinline__ bool scan_cluster_begin(const ScanParams& p, ScanState& st, uint32_t qi,
                                                   uint32_t l) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t c = p.ctag[(uint64_t)qi * p.P + l];
        st.c = c;
        st.cdl = p.cdist[(uint64_t)qi * p.P + l];
        st.i0 = st.i1 = 0;
        st.r0 = st.r1 = 0;
        if (c < p.C) {
            st.r0 = p.cell_start[(uint64_t)c * p.F];
            st.r1 = p.cell_start[(uint64_t)c * p.F + p.F];
            if (p.ins_cl_start) {
                st.i0 = p.ins_cl_start[c];
                st.i1 = p.ins_cl_start[c + 1];
            }
        }
    }
    __syncthreads();
    return st.c < p.C;
}

// srow[f] = 2 * cell_dist of cluster c's cell f, cell_dist = (cd + stationary) + fd
// (puck_index.cpp:539-540); all threads, barrier after.
__device__ __forceinline__ void scan_fill_srow(const ScanParams& p, float* srow, const float* fdk,
                                               uint32_t c, float cdl) {
    const uint32_t F = p.F;
    if ((F & 3u) == 0) {
        // 16-byte rows (F % 4 == 0): one float4 of each row per step
        const float4* st4 = reinterpret_cast<const float4*>(p.stationary + (uint64_t)c * F);
        const float4* fd4 = reinterpret_cast<const float4*>(fdk);
        float4* s4 = reinterpret_cast<float4*>(srow);
        for (uint32_t i = threadIdx.x; i < (F >> 2); i += blockDim.x) {
            const float4 a = __ldg(st4 + i), b = __ldg(fd4 + i);
            s4[i] = make_float4(2.0f * __fadd_rn(__fadd_rn(cdl, a.x), b.x),
                                2.0f * __fadd_rn(__fadd_rn(cdl, a.y), b.y),
                                2.0f * __fadd_rn(__fadd_rn(cdl, a.z), b.z),
                                2.0f * __fadd_rn(__fadd_rn(cdl, a.w), b.w));
        }
    } else {
        for (uint32_t i = threadIdx.x; i < F; i += blockDim.x)
            srow[i] = 2.0f * __fadd_rn(__fadd_rn(cdl, p.stationary[(uint64_t)c * F + i]), fdk[i]);
    }
    __syncthreads();
}

// Buffer insert of one round slot: the kept keys of the warp take consecutive
// slots (one shared atomic per warp). The capacity is kept >= count + a round by
// the cut in scan_after_round.
__device__ __forceinline__ void scan_insert(ScanState& st, uint64_t* keys, bool keep, uint64_t key,
                                            unsigned long long& my_pass) {
    const unsigned ballot = __ballot_sync(0xffffffffu, keep);
    if (ballot) {
        const int lane = threadIdx.x & 31;
        uint32_t base_slot = 0;
        if (lane == __ffs(ballot) - 1) base_slot = atomicAdd(&st.count, (uint32_t)__popc(ballot));
        base_slot = __shfl_sync(0xffffffffu, base_slot, __ffs(ballot) - 1);
        if (keep) {
            keys[base_slot + __popc(ballot & ((1u << lane) - 1))] = key;
            ++my_pass;
        }
    }
}

// After a round (all threads): cut the buffer back when it could not take another
// round of `round` keys. One histogram pass gives a bound with at least T keys below
// it (the final select is exact); tau = that bound. If the cut kept too many to take
// another round, cut exactly to T.
template <int NT>
__device__ __forceinline__ void scan_after_round(ScanState& st, uint64_t* keys, uint32_t* hist,
                                                 uint32_t cap, uint32_t round, uint32_t T,
                                                 uint64_t tau, long long t_round) {
    __syncthreads();
    const long long t_round_end = clock64();
    if (threadIdx.x == 0) st.cyc_rounds += (unsigned long long)(t_round_end - t_round);
    if (st.count > cap - round) {
        const uint32_t cnt = st.count;
        uint64_t bound = block_cut_bound<NT>(keys, cnt, T, hist, st.red);
        uint32_t kept = bound == kKeyMax ? cnt : block_compact_lt<NT>(keys, cnt, bound, &st.ccount);
        if (kept > cap - round) {
            const uint64_t kth = block_select_kth<NT>(keys, kept, T, st.hist, st.sel);
            bound = kth + 1;  // kth < kKeyMax: keys are distinct by id
            kept = block_compact_lt<NT>(keys, kept, bound, &st.ccount);
        }
        if (threadIdx.x == 0) {
            st.count = kept;
            st.tau = bound < tau ? bound : tau;
            st.n_compact += 1;
            st.cyc_compact += (unsigned long long)(clock64() - t_round_end);
        }
        __syncthreads();
    }
}

// The block's last steps: the exact T smallest keys of the buffer, written out
// unordered (only the rerank's tie path needs their (t, id) order, and it sorts
// them itself), and the diagnostic counters.
template <int NT>
__device__ void scan_finish(const ScanParams& p, ScanState& st, uint64_t* keys, uint32_t* hist,
                            uint32_t qi,
                            unsigned long long my_eval, unsigned long long my_look,
                            unsigned long long my_pass, long long t_start, long long t_pro) {
    const int tid = threadIdx.x;
    const uint32_t T = p.T;
    __syncthreads();
    const long long t_final = clock64();
    uint32_t count = st.count;
    if (count > T) {
        const uint64_t kth =
            block_kth_hist<NT>(keys, count, T, hist, st.red, &st.ccount, st.hist, st.sel);
        block_compact_lt<NT>(keys, count, kth + 1, &st.ccount);
        count = T;
    }
    const uint32_t out = count < T ? count : T;
    for (uint32_t i = tid; i < T; i += NT) {
        p.hdist[(uint64_t)qi * T + i] = i < out ? key_value(keys[i]) : sentinel_f();
        p.htag[(uint64_t)qi * T + i] = i < out ? (uint32_t)keys[i] : kNoLabel;
    }
    if (tid == 0) p.hcnt[qi] = out;
    if (p.counters) {
        // records evaluated / looked up / kept: summed over the block first, so each
        // counter takes one global atomic per block (the counters share one sector,
        // and atomics on it from every thread of the grid serialise in L2)
        const unsigned we = __reduce_add_sync(0xffffffffu, (unsigned)my_eval);
        const unsigned wl = __reduce_add_sync(0xffffffffu, (unsigned)my_look);
        const unsigned wp = __reduce_add_sync(0xffffffffu, (unsigned)my_pass);
        if ((tid & 31) == 0) {
            atomicAdd(&st.evaluated, (unsigned long long)we);
            atomicAdd(&st.looked, (unsigned long long)wl);
            atomicAdd(&st.passed, (unsigned long long)wp);
        }
        __syncthreads();
        if (tid == 0) {
            const long long t_end = clock64();
            atomicAdd(p.counters + kScRecords, st.evaluated);
            atomicAdd(p.counters + kScLookups, st.looked);
            atomicAdd(p.counters + kScKept, st.passed);
            atomicAdd(p.counters + kScCompactions, st.n_compact);
            atomicMax(p.counters + kScMaxRecords, st.n_records);
            atomicAdd(p.counters + kScCycPrologue, (unsigned long long)(t_pro - t_start));
            atomicAdd(p.counters + kScCycTotal, (unsigned long long)(t_end - t_start));
            atomicAdd(p.counters + kScCycRounds, st.cyc_rounds);
            atomicAdd(p.counters + kScCycCompact, st.cyc_compact);
            atomicAdd(p.counters + kScCycFinal, (unsigned long long)(t_end - t_final));
        }
    }
}

// Loads the NW code words of record `mr` (8-byte loads when the row stride allows).
template <int NW>
__device__ __forceinline__ void load_codes(const uint8_t* codes, uint32_t stride, uint32_t mr,
                                           uint32_t (&w)[NW]) {
    if ((NW & 1) == 0 && (stride & 7u) == 0) {
        const uint2* cw = reinterpret_cast<const uint2*>(codes + (uint64_t)mr * stride);
#pragma unroll
        for (int i = 0; i < NW / 2; ++i) {
            const uint2 v = __ldg(cw + i);
            w[2 * i] = v.x;
            w[2 * i + 1] = v.y;
        }
    } else {
        const uint32_t* cw = reinterpret_cast<const uint32_t*>(codes + (uint64_t)mr * stride);
#pragma unroll
        for (int i = 0; i < NW; ++i) w[i] = __ldg(cw + i);
    }
}

// NW = code words per record (code_stride / 4); TAB = table variant.
template <int NW, int TAB>
__global__ __launch_bounds__(kThreads, PGPU_SCAN_MIN_BLOCKS) void k_scan_select(ScanParams p) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ ScanState st;
    const uint32_t qi = p.order[blockIdx.x];
    const int tid = threadIdx.x;
    const uint32_t nsq = p.nsq, F = p.F, T = p.T, cap = p.cap;
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem);  // [cap], first (8-byte aligned)
    uint32_t* hist = reinterpret_cast<uint32_t*>(keys + cap);  // [kHistBins]
    float* lut = reinterpret_cast<float*>(hist + kHistBins);
    __half* luth = reinterpret_cast<__half*>(lut);
    constexpr bool HALF = TAB != kTabF32;
    // [F] 2 * cell_dist of the current cluster's cells, after the table
    float* srow = HALF ? reinterpret_cast<float*>(luth + nsq * 256) : lut + nsq * 256;
    float* qv = srow + F;                  // [d]

    if (p.done && p.done[qi]) return;  // answered by the split scan
    if (p.status[qi] != 0) {
        if (tid == 0) p.hcnt[qi] = 0;
        return;
    }
    const long long t_start = clock64();
    for (uint32_t i = tid; i < p.d; i += kThreads) qv[i] = p.q[(uint64_t)qi * p.d + i];
    const float* fdk = p.fd_by_fine + (uint64_t)qi * F;  // fine terms of this query
    if (tid == 0) {
        st.tau = kKeyMax;
        st.count = 0;
        st.evaluated = 0;
        st.looked = 0;
        st.passed = 0;
        st.cyc_rounds = st.cyc_compact = st.n_compact = st.n_records = 0;
    }
    const int lut_e = HALF ? half_lut_exponent(p.qnorm[qi], p.codebook_max) : 0;
    const float inv_scale = HALF ? ldexpf(1.0f, -lut_e) : 1.0f;
    __syncthreads();
    build_table<TAB>(lut, qv, p.codebook, nsq, p.lsq, HALF ? ldexpf(1.0f, lut_e) : 1.0f);
    unsigned long long my_eval = 0, my_look = 0, my_pass = 0;
    const long long t_pro = clock64();
    for (uint32_t l = 0; l < p.P; ++l) {
        // the probed clusters fill a prefix of the slots (the learned probe leaves the
        // rest empty): the first empty slot ends the walk
        if (!scan_cluster_begin(p, st, qi, l)) break;
        const uint32_t r0 = st.r0, i0 = st.i0;
        // the cluster's base records [r0, r1), then its inserted ones (realtime)
        const uint32_t nb = st.r1 - r0, nall = nb + (st.i1 - st.i0);
        if (nall == 0) continue;
        scan_fill_srow(p, srow, fdk, st.c, st.cdl);
        if (tid == 0) st.n_records += nall;
        for (uint32_t base = 0; base < nall; base += kRound) {
            const long long t_round = clock64();
            const uint64_t tau = st.tau;
            // all loads of the thread's records first, so their latencies overlap
            uint32_t fine_id[kRecPerThread];
            float off[kRecPerThread];
            uint32_t words[kRecPerThread][NW];
            uint32_t mem[kRecPerThread];
#pragma unroll
            for (int j = 0; j < kRecPerThread; ++j) {
                const uint32_t v = base + tid + j * kThreads;
                const uint32_t mr = v < nb ? r0 + v : (v < nall ? p.ins_cl_ids[i0 + v - nb] : r0);
                mem[j] = mr;
                fine_id[j] = p.rec_fine[mr];
                off[j] = p.offsets[mr];
                load_codes<NW>(p.codes, p.code_stride, mr, words[j]);
            }
#pragma unroll
            for (int j = 0; j < kRecPerThread; ++j) {
                const uint32_t mi = mem[j];
                bool keep = false;
                uint64_t key = 0;
                if (base + tid + j * kThreads < nall) {
                    // (float)(2.0 * cell_dist + offset): one float add of the exact
                    // 2 * cell_dist (see adc_base)
                    const float t0 = __fadd_rn(srow[fine_id[j]], off[j]);
                    ++my_eval;
                    if (filter_key(t0, mi) < tau) {  // t can only grow past t0
                        ++my_look;
                        float t;
                        if (TAB == kTabF16)
                            t = t0 + lut_sum_words_half<NW>(words[j], luth, nsq) * inv_scale;
                        else
                            t = __fadd_rn(t0, lut_sum_words<NW>(words[j], lut, nsq));
                        key = filter_key(t, mi);
                        keep = key < tau;
                    }
                }
                scan_insert(st, keys, keep, key, my_pass);
            }
            scan_after_round<kThreads>(st, keys, hist, cap, kRound, T, tau, t_round);
        }
    }
    scan_finish<kThreads>(p, st, keys, hist, qi, my_eval, my_look, my_pass, t_start, t_pro);
}

// ------------------------------------------------------------ interleaved kernel
// One block per query. A round is 2 * NT / 32 interleaved record blocks, 2 * NT
// records: thread t takes lane t & 31 of blocks t >> 5 and (t >> 5) + NT / 32, and
// scores the two records together. Rounds arrive in a ring of shared-memory slots
// by one bulk copy each (cp.async.bulk, completion on the slot's mbarrier), issued
// by thread 0 up to a ring's length ahead; the first copies go out before the
// table is built.
//   FP32 table (64 KB): 512 threads, 3 slots, one block per SM.
//   FP16 table (32 KB): 256 threads, 2 slots, two blocks per SM, so one block's
//   table build, cuts and final select overlap the other's rounds.
#ifndef PGPU_SCAN_IL_REC
#define PGPU_SCAN_IL_REC 2
#endif
#ifndef PGPU_SCAN_IL_STAGES32
#define PGPU_SCAN_IL_STAGES32 3
#endif
#ifndef PGPU_SCAN_IL_STAGES16
#define PGPU_SCAN_IL_STAGES16 2
#endif
constexpr int kIlRec = PGPU_SCAN_IL_REC;  // records per thread and round
template <bool HALF>
struct IlShape {
    static constexpr int kThreads = HALF ? 256 : 512;
    static constexpr int kStages = HALF ? PGPU_SCAN_IL_STAGES16 : PGPU_SCAN_IL_STAGES32;
    static constexpr int kMinBlocks = HALF ? 2 : 1;
    static constexpr uint32_t kBlocksPerRound = kThreads / 32 * kIlRec;
    static constexpr int kRound = kThreads * kIlRec;  // records per round
    static_assert(kMaxCap % kThreads == 0 && kHistBins % kThreads == 0, "helper shapes");
};
constexpr uint32_t kIlWaitLimit = 1u << 22;

// Buffer size of the interleaved kernel for filter_topk T (see scan_cap).
template <bool HALF>
__host__ __device__ inline uint32_t il_cap(uint32_t T) {
    constexpr uint32_t NT = IlShape<HALF>::kThreads;
    uint32_t room = T > 1024 ? T : 1024;
    uint32_t c = T + IlShape<HALF>::kRound + room;
    c = (c + NT - 1) / NT * NT;
    return c > kMaxCap ? kMaxCap : c;
}
__host__ __device__ constexpr uint32_t il_table_bytes(bool half) {
    return half ? 256u * 64u * 2u : 256u * 64u * 4u;
}
// Shared memory after the table: the query, the ring, then either the compact table
// being built ([nsq][257] floats) or the cluster's cell terms, the key buffer and the
// cut histogram.
__host__ __device__ inline uint32_t il_query_bytes(uint32_t d) { return (d * 4u + 15u) & ~15u; }
__host__ __device__ inline uint32_t il_srow_bytes(uint32_t F) { return (F * 4u + 7u) & ~7u; }
template <bool HALF>
__host__ __device__ inline uint32_t il_slot_bytes(uint32_t nsq) {
    return IlShape<HALF>::kBlocksPerRound * il_block_bytes(nsq);
}

// Bounded wait on a slot's mbarrier phase. A try_wait may suspend the thread for up
// to PGPU_SCAN_WAIT_HINT ns (0: no hint) while the copy is outstanding.
#ifndef PGPU_SCAN_WAIT_HINT
#define PGPU_SCAN_WAIT_HINT 0
#endif
__device__ __forceinline__ bool il_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < kIlWaitLimit; ++it) {
        uint32_t ok;
        if (PGPU_SCAN_WAIT_HINT > 0)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
                "selp.b32 %0, 1, 0, p;\n}"
                : "=r"(ok)
                : "r"(bar), "r"(parity), "n"(PGPU_SCAN_WAIT_HINT)
                : "memory");
        else
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                "selp.b32 %0, 1, 0, p;\n}"
                : "=r"(ok)
                : "r"(bar), "r"(parity)
                : "memory");
        if (ok) return true;
    }
    return false;
}

// get_dist_table (quantization.cpp:260-270) of the query qv in the reference's lane
// order, staged as stage[m * 257 + j] (row pitch 257: the expansion reads it without
// bank conflicts), then expanded into the rotated table: column m' < NSQ + 31 of row
// c holds subspace m' mod NSQ (FP32), or the same scaled by 2^lut_e in FP16. Each
// codeword's subspaces go in two halves, a thread per half (NT = 512) or both halves
// by one thread (NT = 256). All NT threads; one barrier inside (after the staging),
// none after the expansion.
template <int NSQ, bool HALF, int NT, bool WIDE = false>
__device__ __forceinline__ void il_build_table(unsigned char* tab, float* stage, const float* qv,
                                               const float* __restrict__ codebook, uint32_t lsq,
                                               int lut_e) {
    static_assert(NT % 256 == 0, "a thread per codeword and half");
    const int tid = threadIdx.x;
    for (uint32_t h2 = tid >> 8; h2 < 2; h2 += NT / 256) {
        const uint32_t j = tid & 255u;
        const int mh = (int)h2 * (NSQ / 2);
        if (lsq == 4) {
            const float4* cb4 = reinterpret_cast<const float4*>(codebook);
#pragma unroll
            for (int m0 = 0; m0 < NSQ / 2; m0 += 2) {
                float4 y[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) y[u] = __ldg(cb4 + (uint64_t)(mh + m0 + u) * 256 + j);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int m = mh + m0 + u;
                    const float* x = qv + m * 4;
                    const float t0 = __fsub_rn(x[0], y[u].x), t1 = __fsub_rn(x[1], y[u].y);
                    const float t2 = __fsub_rn(x[2], y[u].z), t3 = __fsub_rn(x[3], y[u].w);
                    stage[m * 257 + j] = __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)),
                                                   __fadd_rn(__fmul_rn(t2, t2), __fmul_rn(t3, t3)));
                }
            }
        } else {
            for (int m = mh; m < mh + NSQ / 2; ++m)
                stage[m * 257 + j] =
                    l2sqr_sse(qv + m * lsq, codebook + ((uint64_t)m * 256 + j) * lsq, lsq);
        }
    }
    __syncthreads();
    if (HALF && WIDE) {
        // each FP16 entry in its own 4-byte slot (the FP32 table's addresses)
        const float scale = ldexpf(1.0f, lut_e);
        uint32_t* tw = reinterpret_cast<uint32_t*>(tab);
        for (uint32_t w = tid; w < 256 * 64; w += NT) {
            const uint32_t c = w >> 6, m = w & 63;
            const float v = m < NSQ + 31 ? stage[(m % NSQ) * 257 + c] : 0.0f;
            tw[w] = (uint32_t)__half_as_ushort(__float2half_rn(v * scale));
        }
    } else if (HALF) {
        const float scale = ldexpf(1.0f, lut_e);
        uint32_t* tw = reinterpret_cast<uint32_t*>(tab);
        for (uint32_t w = tid; w < 256 * 32; w += NT) {
            const uint32_t c = w >> 5, m0 = (w & 31) * 2;
            const float v0 = m0 < NSQ + 31 ? stage[(m0 % NSQ) * 257 + c] : 0.0f;
            const float v1 = m0 + 1 < NSQ + 31 ? stage[((m0 + 1) % NSQ) * 257 + c] : 0.0f;
            const __half2 h = __halves2half2(__float2half_rn(v0 * scale), __float2half_rn(v1 * scale));
            tw[w] = *reinterpret_cast<const uint32_t*>(&h);
        }
    } else {
        float* tf = reinterpret_cast<float*>(tab);
        for (uint32_t w = tid; w < 256 * 64; w += NT) {
            const uint32_t c = w >> 6, m = w & 63;
            tf[w] = m < NSQ + 31 ? stage[(m % NSQ) * 257 + c] : 0.0f;
        }
    }
}

// t of R records (memory ids mr, lanes mr & 31) from their codes (8-byte granules
// of the rotated layout), offsets and fine ids, with srow[f] = 2 * cell_dist of the
// record's cell; the R lookup chains are interleaved. Lookup step s goes to partial
// s mod 4 in FP32; t = (srow[f] + offset) + ((a0 + a1) + (a2 + a3)) (the FP16 table's
// sum scaled back by inv_scale).
template <int NSQ, bool HALF, int R, bool WIDE = false>
__device__ __forceinline__ void il_score(const unsigned char* tab, const float* srow,
                                         const uint2 (&gr)[R][(NSQ + 7) / 8], const float (&off)[R],
                                         const uint32_t (&fine)[R], const uint32_t (&mr)[R],
                                         float inv_scale, float (&t)[R]) {
    float a[R][4];
    uint32_t lb[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        lb[j] = (mr[j] & 31u) << 2;  // byte 0 of the table address
        a[j][0] = a[j][1] = a[j][2] = a[j][3] = 0.0f;
    }
#pragma unroll
    for (int s2 = 0; s2 < NSQ; ++s2) {
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const uint32_t w = (s2 & 4) ? gr[j][s2 >> 3].y : gr[j][s2 >> 3].x;
            // (code << 8) | 4 * lane: the entry of column s2 + lane
            const uint32_t addr = __byte_perm(w, lb[j], 0x5504u | ((uint32_t)(s2 & 3) << 4));
            if (HALF) {
                // compact table: 2-byte entries (one shift); WIDE: one entry per 4-byte slot
                const unsigned short h =
                    WIDE ? *reinterpret_cast<const unsigned short*>(tab + addr + 4 * s2)
                         : *reinterpret_cast<const unsigned short*>(tab + (addr >> 1) + 2 * s2);
                asm("add.f32.f16 %0, %1, %0;" : "+f"(a[j][s2 & 3]) : "h"(h));
            } else {
                a[j][s2 & 3] =
                    __fadd_rn(a[j][s2 & 3], *reinterpret_cast<const float*>(tab + addr + 4 * s2));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const float t0 = __fadd_rn(srow[fine[j]], off[j]);  // (float)(2.0 * cell_dist + offset)
        const float sum = __fadd_rn(__fadd_rn(a[j][0], a[j][1]), __fadd_rn(a[j][2], a[j][3]));
        t[j] = HALF ? t0 + sum * inv_scale : __fadd_rn(t0, sum);
    }
}

template <int NSQ, bool HALF>
__global__ __launch_bounds__(IlShape<HALF>::kThreads, IlShape<HALF>::kMinBlocks) void k_scan_il(
    ScanParams p) {
    constexpr int kIlThreads = IlShape<HALF>::kThreads;
    constexpr int kIlStages = IlShape<HALF>::kStages;
    constexpr uint32_t kIlBlocksPerRound = IlShape<HALF>::kBlocksPerRound;
    constexpr int kIlRound = IlShape<HALF>::kRound;
    static_assert(NSQ % 4 == 0 && NSQ <= 32, "interleaved layout: nsq a multiple of 4, <= 32");
    constexpr int NG = (NSQ + 7) / 8;  // 8-byte code granules per record
    constexpr uint32_t kG = NG * 8;
    constexpr uint32_t kBlk = 32 * kG + 192;  // il_block_bytes
    constexpr uint32_t kSlot = kIlBlocksPerRound * kBlk;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ ScanState st;
    __shared__ __align__(8) uint64_t full[kIlStages];
    __shared__ int il_failed;
    const uint32_t qi = p.order[blockIdx.x];
    const int tid = threadIdx.x;
    const uint32_t F = p.F, T = p.T, cap = p.cap;
    unsigned char* tab = smem;  // the rotated table, at offset 0
    float* qv = reinterpret_cast<float*>(smem + il_table_bytes(HALF));
    unsigned char* ring = smem + il_table_bytes(HALF) + il_query_bytes(p.d);  // [kIlStages][kSlot]
    unsigned char* rest = ring + kIlStages * kSlot;
    float* stage = reinterpret_cast<float*>(rest);  // [NSQ][257] while the table is built
    float* srow = reinterpret_cast<float*>(rest);   // [F] afterwards
    uint64_t* keys = reinterpret_cast<uint64_t*>(rest + il_srow_bytes(F));  // [cap]
    uint32_t* hist = reinterpret_cast<uint32_t*>(keys + cap);              // [kHistBins]

    if (p.done && p.done[qi]) return;  // answered by the split scan
    if (p.status[qi] != 0) {
        if (tid == 0) p.hcnt[qi] = 0;
        return;
    }
    const long long t_start = clock64();
    // rounds issued and consumed over the whole block (slot g % S, parity (g / S) & 1)
    uint32_t g_issued = 0, g_done = 0;
    auto bar_of = [&](uint32_t g) { return (uint32_t)__cvta_generic_to_shared(&full[g % kIlStages]); };
    // thread 0: bulk copy of record blocks [blk0, blk0 + nblk) into round g's slot
    auto issue = [&](uint32_t g, uint64_t blk0, uint32_t nblk) {
        const uint32_t bar = bar_of(g);
        const uint32_t bytes = nblk * kBlk;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(ring + (g % kIlStages) * kSlot);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                "r"(dst),
            "l"(p.codes_il + blk0 * kBlk), "r"(bytes), "r"(bar)
            : "memory");
    };
    if (tid == 0) {
        for (int i = 0; i < kIlStages; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_of(i)), "r"(1u));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        st.tau = kKeyMax;
        st.count = 0;
        st.evaluated = st.looked = st.passed = 0;
        st.cyc_rounds = st.cyc_compact = st.n_compact = st.n_records = 0;
        il_failed = 0;
    }
    // the first cluster's first rounds go out before the table is built
    uint32_t primed_blk0 = 0, primed_blocks = 0;
    if (tid == 0) {
        const uint32_t c = p.ctag[(uint64_t)qi * p.P];
        if (c < p.C) {
            const uint32_t r0 = p.cell_start[(uint64_t)c * F], r1 = p.cell_start[(uint64_t)c * F + F];
            if (r1 > r0) {
                const uint32_t b0 = r0 >> 5, nblk = ((r1 - 1) >> 5) - b0 + 1;
                primed_blk0 = b0;
                for (uint32_t k = 0; k < (uint32_t)kIlStages && k * kIlBlocksPerRound < nblk; ++k) {
                    const uint32_t m = min(kIlBlocksPerRound, nblk - k * kIlBlocksPerRound);
                    issue(g_issued++, (uint64_t)b0 + k * kIlBlocksPerRound, m);
                    primed_blocks += m;
                }
            }
        }
    }
    for (uint32_t i = tid; i < p.d; i += kIlThreads) qv[i] = p.q[(uint64_t)qi * p.d + i];
    const float* fdk = p.fd_by_fine + (uint64_t)qi * F;
    // the first cluster's stationary row and this query's fine terms are loaded now,
    // so their latency overlaps the table build (srow is written after it)
    constexpr int kPre = 2;  // float4 per thread and row (F <= kPre * 4 * kIlThreads)
    const uint32_t c_first = p.ctag[(uint64_t)qi * p.P];
    const bool pre = c_first < p.C && (F & 3u) == 0 && F <= kPre * 4 * kIlThreads;
    float4 pre_st[kPre], pre_fd[kPre];
#pragma unroll
    for (int u = 0; u < kPre; ++u) {
        const uint32_t i = tid + u * kIlThreads;
        if (pre && i < (F >> 2)) {
            pre_st[u] = __ldg(reinterpret_cast<const float4*>(p.stationary + (uint64_t)c_first * F) + i);
            pre_fd[u] = __ldg(reinterpret_cast<const float4*>(fdk) + i);
        }
    }
    const int lut_e = HALF ? half_lut_exponent(p.qnorm[qi], p.codebook_max) : 0;
    const float inv_scale = HALF ? ldexpf(1.0f, -lut_e) : 1.0f;
    __syncthreads();
    il_build_table<NSQ, HALF, kIlThreads>(tab, stage, qv, p.codebook, p.lsq, lut_e);
    unsigned long long my_eval = 0, my_pass = 0;
    const long long t_pro = clock64();

    auto score_records = [&](const uint2 (&gr)[kIlRec][NG], const float (&off)[kIlRec],
                             const uint32_t (&fine)[kIlRec], const uint32_t (&mr)[kIlRec],
                             float (&t)[kIlRec]) {
        il_score<NSQ, HALF, kIlRec>(tab, srow, gr, off, fine, mr, inv_scale, t);
    };

    for (uint32_t l = 0; l < p.P && !il_failed; ++l) {
        if (!scan_cluster_begin(p, st, qi, l)) break;  // (its first barrier ends the table)
        const uint32_t r0 = st.r0, r1 = st.r1, i0 = st.i0, ni = st.i1 - st.i0;
        if (r1 - r0 + ni == 0) continue;
        if (tid == 0) st.n_records += r1 - r0 + ni;
        if (l == 0 && pre) {
            // srow from the rows loaded before the table build
            const float cdl = st.cdl;
            float4* s4 = reinterpret_cast<float4*>(srow);
#pragma unroll
            for (int u = 0; u < kPre; ++u) {
                const uint32_t i = tid + u * kIlThreads;
                if (i < (F >> 2)) {
                    const float4 a = pre_st[u], b = pre_fd[u];
                    s4[i] = make_float4(2.0f * __fadd_rn(__fadd_rn(cdl, a.x), b.x),
                                        2.0f * __fadd_rn(__fadd_rn(cdl, a.y), b.y),
                                        2.0f * __fadd_rn(__fadd_rn(cdl, a.z), b.z),
                                        2.0f * __fadd_rn(__fadd_rn(cdl, a.w), b.w));
                }
            }
            __syncthreads();
        } else {
            scan_fill_srow(p, srow, fdk, st.c, st.cdl);
        }
        uint32_t b0 = 0, nblk = 0, rounds = 0;
        if (r1 > r0) {
            b0 = r0 >> 5;
            nblk = ((r1 - 1) >> 5) - b0 + 1;
            rounds = (nblk + kIlBlocksPerRound - 1) / kIlBlocksPerRound;
        }
        // rounds of this cluster already in flight (the first cluster's, primed)
        uint32_t sent = (l == 0 && primed_blocks > 0 && primed_blk0 == b0)
                            ? (primed_blocks + kIlBlocksPerRound - 1) / kIlBlocksPerRound
                            : 0;
        if (tid == 0) {
            for (; sent < rounds && sent < (uint32_t)kIlStages; ++sent)
                issue(g_issued++, (uint64_t)b0 + sent * kIlBlocksPerRound,
                      min(kIlBlocksPerRound, nblk - sent * kIlBlocksPerRound));
        }
        sent = rounds < (uint32_t)kIlStages ? rounds : (uint32_t)kIlStages;
        g_issued = g_done + sent;  // every thread tracks the count thread 0 issued
        const uint32_t blk = tid >> 5, lane = tid & 31;
        for (uint32_t k = 0; k < rounds; ++k) {
            const long long t_round = clock64();
            const uint64_t tau = st.tau;
            // tau as (float, id): key(t, id) < tau iff t < tau_f, or t == tau_f and
            // id < tau_id (float compares treat -0 as +0, as the keys do; a bound
            // whose float part is the key of -0 keeps exactly the t < 0)
            float tau_f = tau == kKeyMax ? __int_as_float(0x7f800000) : key_value(tau);
            uint32_t tau_id = tau == kKeyMax ? 0xFFFFFFFFu : (uint32_t)tau;
            if ((uint32_t)(tau >> 32) == 0x7FFFFFFFu) {
                tau_f = 0.0f;
                tau_id = 0;
            }
            const uint32_t g = g_done;
            if (!il_wait(bar_of(g), (g / kIlStages) & 1u)) {
                if (lane == 0) atomicExch(&il_failed, 1);
            }
            uint2 gr[kIlRec][NG];
            float off[kIlRec], t[kIlRec];
            uint32_t fine[kIlRec], rr[kIlRec];
            bool valid[kIlRec];
#pragma unroll
            for (int j = 0; j < kIlRec; ++j) {
                const uint32_t bl = blk + j * (kIlThreads / 32);  // block of the round
                const uint64_t bk = (uint64_t)b0 + k * kIlBlocksPerRound + bl;
                rr[j] = (uint32_t)(bk * 32 + lane);
                valid[j] = bk < (uint64_t)b0 + nblk && rr[j] >= r0 && rr[j] < r1 && !il_failed;
                // out-of-range slots read stale bytes of the slot and are dropped below
                const unsigned char* rec = ring + (g % kIlStages) * kSlot + bl * kBlk;
#pragma unroll
                for (int q2 = 0; q2 < NG; ++q2)
                    gr[j][q2] = *reinterpret_cast<const uint2*>(rec + q2 * 256 + 8 * lane);
                off[j] = *reinterpret_cast<const float*>(rec + 32 * kG + 4 * lane);
                fine[j] = valid[j] ? *reinterpret_cast<const uint16_t*>(rec + 32 * kG + 128 + 2 * lane)
                                   : 0u;
            }
            score_records(gr, off, fine, rr, t);
#pragma unroll
            for (int j = 0; j < kIlRec; ++j) {
                // key(t, id) < tau by float compares; the key only for kept records
                const bool keep =
                    valid[j] && (t[j] < tau_f || (t[j] == tau_f && rr[j] < tau_id));
                my_eval += valid[j] ? 1 : 0;
                scan_insert(st, keys, keep, keep ? filter_key(t[j], rr[j]) : 0ull, my_pass);
            }
            scan_after_round<kIlThreads>(st, keys, hist, cap, kIlRound, T, tau, t_round);
            if (il_failed) break;  // read after the barrier: the same on every thread
            ++g_done;
            // the slot of round g is free: thread 0 refills it with round k + kIlStages
            const uint32_t kn = k + kIlStages;
            if (kn < rounds) {
                if (tid == 0)
                    issue(g_issued, (uint64_t)b0 + kn * kIlBlocksPerRound,
                          min(kIlBlocksPerRound, nblk - kn * kIlBlocksPerRound));
                ++g_issued;
            }
        }
        // realtime: the cluster's inserted records, read from the interleaved copy
        for (uint32_t v0 = 0; v0 < ni; v0 += kIlRound) {
            const long long t_round = clock64();
            const uint64_t tau = st.tau;
            uint2 gr[kIlRec][NG];
            float off[kIlRec], t[kIlRec];
            uint32_t fine[kIlRec], mr[kIlRec];
            bool valid[kIlRec];
#pragma unroll
            for (int j = 0; j < kIlRec; ++j) {
                const uint32_t v = v0 + tid + j * kIlThreads;
                valid[j] = v < ni;
                mr[j] = valid[j] ? p.ins_cl_ids[i0 + v] : 0u;
#pragma unroll
                for (int q2 = 0; q2 < NG; ++q2)
                    gr[j][q2] = __ldg(reinterpret_cast<const uint2*>(
                        p.codes_il + il_granule_offset(mr[j], q2, NSQ)));
                off[j] = __ldg(reinterpret_cast<const float*>(p.codes_il + il_offset_offset(mr[j], NSQ)));
                fine[j] = __ldg(reinterpret_cast<const uint16_t*>(p.codes_il + il_fine_offset(mr[j], NSQ)));
            }
            score_records(gr, off, fine, mr, t);
#pragma unroll
            for (int j = 0; j < kIlRec; ++j) {
                const uint64_t key = filter_key(t[j], mr[j]);
                const bool keep = valid[j] && key < tau;
                my_eval += valid[j] ? 1 : 0;
                scan_insert(st, keys, keep, key, my_pass);
            }
            scan_after_round<kIlThreads>(st, keys, hist, cap, kIlRound, T, tau, t_round);
        }
    }
    if (il_failed) {
        // a copy did not arrive in time: wait (bounded) for every copy issued, so
        // none lands in shared memory after the block, and report the query as empty
        for (uint32_t g = g_done; g < g_issued; ++g) il_wait(bar_of(g), (g / kIlStages) & 1u);
        __syncthreads();
        if (tid == 0) {
            p.hcnt[qi] = 0;
            atomicExch(p.err, 1);
        }
        return;
    }
    scan_finish<kIlThreads>(p, st, keys, hist, qi, my_eval, my_eval, my_pass, t_start, t_pro);
}

// Launch order of the scan's blocks. A block's time follows the records of the
// clusters its query probes, and blocks start in index order: queries sorted by
// descending record count start the longest scans first and end the grid with the
// shortest, so fewer SMs sit idle at the tail. The sort is by bucket (4 steps per
// octave of the count), which is all the ordering needs; the results do not depend
// on it.
constexpr uint32_t kOrderBuckets = 132;
constexpr int kOrderThreads = 1024;

__device__ __forceinline__ uint32_t work_bucket(uint32_t w) {
    if (w == 0) return kOrderBuckets - 1;  // nothing to scan: last
    const int e = 31 - __clz(w);
    const uint32_t frac = e >= 2 ? (w >> (e - 2)) & 3u : (w << (2 - e)) & 3u;
    return (kOrderBuckets - 2) - ((uint32_t)e * 4 + frac);  // more records: earlier
}

// One thread per query: its record count over the probed clusters, as a bucket.
__global__ void k_scan_work(const uint32_t* __restrict__ ctag, const int32_t* __restrict__ status,
                            const uint32_t* __restrict__ cell_start,
                            const uint32_t* __restrict__ ins_cl_start, uint32_t n, uint32_t P,
                            uint32_t C, uint32_t F, uint8_t* __restrict__ wbucket) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t w = 0;
    if (status[q] == 0) {
        for (uint32_t l = 0; l < P; ++l) {
            const uint32_t c = ctag[(uint64_t)q * P + l];
            if (c >= C) break;  // the probed clusters fill a prefix of the slots
            w += cell_start[(uint64_t)c * F + F] - cell_start[(uint64_t)c * F];
            if (ins_cl_start) w += ins_cl_start[c + 1] - ins_cl_start[c];
        }
    }
    wbucket[q] = (uint8_t)work_bucket(w);
}

// One block: counting sort of the queries by bucket (order within a bucket is free).
__global__ __launch_bounds__(kOrderThreads) void k_scan_order(const uint8_t* __restrict__ wbucket,
                                                              uint32_t n, uint32_t* __restrict__ order) {
    __shared__ uint32_t hist[kOrderBuckets];
    for (uint32_t i = threadIdx.x; i < kOrderBuckets; i += kOrderThreads) hist[i] = 0;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < n; q += kOrderThreads) atomicAdd(&hist[wbucket[q]], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t i = 0; i < kOrderBuckets; ++i) {
            const uint32_t c = hist[i];
            hist[i] = run;
            run += c;
        }
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < n; q += kOrderThreads)
        order[atomicAdd(&hist[wbucket[q]], 1u)] = q;
}

// ------------------------------------------------------------ split scan
// The interleaved layout's scan when the per-pass scratch holds the distance of every
// record the batch scans (Scratch::tbuf); queries that do not fit, or whose cut bin
// holds too many records, stay with k_scan_il. One block per query (k_scan_score):
//   1. the table (il_build_table), then, per probed cluster, the cell terms;
//   2. the histogram's range from one record per thread at evenly spaced positions of
//      the first probed cluster;
//   3. records, with no barrier: each warp streams its own record blocks straight
//      from the interleaved copy (coalesced 8-byte loads, the next step's loads in
//      flight while the current one is scored), writes each record's t (the same
//      il_score arithmetic as k_scan_il) to tbuf, query q's records at qoff[q] cluster
//      by cluster (base records, then inserted ones), and counts it in a
//      kSplitBins-bin histogram linear in t;
//   4. the cut: the bin where the running count reaches T; every record of a higher
//      bin has T records strictly below it;
//   5. the pick: the block reads its own distances back (mostly from L2), keeps those
//      at or below the cut bin as (t, position) keys in the table's place, maps
//      positions to memory ids and writes the exact T smallest (t, id), unordered:
//      the same set as k_scan_il's.
// Without k_scan_il's key buffer and its cut-backs, a block holds the table, the cell
// terms and the histogram: two blocks per SM, so one block's table build and pick
// overlap the other's records. The FP16 table (precision form) keeps one entry per
// 4-byte slot, the FP32 table's addresses: a lookup is the same PRMT, load and add
// (the compact 2-byte layout costs a shift per lookup, and its smaller footprint buys
// nothing here).
// record blocks per warp and step (FP32 table, FP16 table)
#ifndef PGPU_SPLIT_RB32
#define PGPU_SPLIT_RB32 4
#endif
#ifndef PGPU_SPLIT_RB16
#define PGPU_SPLIT_RB16 4
#endif
constexpr int kSplitThreads = 256;
constexpr int kSplitWarps = kSplitThreads / 32;
constexpr uint32_t kSplitBins = 4096;
constexpr uint32_t kSplitMaxSlots = 512;   // probed clusters a split query may have
constexpr uint32_t kSplitNo = 0xFFFFFFFFu; // count of a query left to k_scan_il
#ifndef PGPU_SPLIT_AHEAD
#define PGPU_SPLIT_AHEAD 2
#endif
constexpr int kSplitAhead = PGPU_SPLIT_AHEAD;  // L2 prefetch distance in record steps (-1: none)
// candidates the pick phase holds (in the table's place): 8192
__host__ __device__ constexpr uint32_t split_max_keys(bool) { return il_table_bytes(false) / 8; }

struct SplitParams {
    const uint32_t* ctag;
    const float* cdist;
    const int32_t* status;
    const uint32_t* cell_start;
    const uint32_t* ins_cl_start;  // realtime: [C+1], or null
    const uint32_t* ins_cl_ids;
    const float* stationary;
    const float* fd_by_fine;
    const float* q;
    const float* qnorm;
    const float* codebook;
    const uint8_t* codes_il;
    const uint32_t* order;
    uint32_t* qcnt;
    uint32_t* qoff;
    uint32_t* qflag;
    SplitCut* cut;
    float* tbuf;
    float* hdist;
    uint32_t* htag;
    uint32_t* hcnt;
    unsigned long long* counters;
    uint64_t tcap;  // floats tbuf holds
    uint32_t n, d, C, F, lsq, P, T;
    float codebook_max;
};

// bin(t) = clamp(trunc((t - lo) * scale), 0, kSplitBins - 1): non-decreasing in t
// (each step rounds monotonically; a NaN product, 0 * inf at t = lo, converts to 0).
__device__ __forceinline__ uint32_t split_bin(float t, float lo, float scale) {
    const int b = __float2int_rz(__fmul_rn(__fsub_rn(t, lo), scale));
    return (uint32_t)min(max(b, 0), (int)kSplitBins - 1);
}

// One thread per query: records over its probed clusters (kSplitNo: not split).
__global__ void k_split_counts(SplitParams sp) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= sp.n) return;
    uint32_t w = kSplitNo;
    if (sp.status[q] == 0) {
        w = 0;
        for (uint32_t l = 0; l < sp.P; ++l) {
            const uint32_t c = sp.ctag[(uint64_t)q * sp.P + l];
            if (c >= sp.C) break;  // the probed clusters fill a prefix of the slots
            if (l >= kSplitMaxSlots) {
                w = kSplitNo;
                break;
            }
            w += sp.cell_start[(uint64_t)c * sp.F + sp.F] - sp.cell_start[(uint64_t)c * sp.F];
            if (sp.ins_cl_start) w += sp.ins_cl_start[c + 1] - sp.ins_cl_start[c];
        }
    }
    sp.qcnt[q] = w;
}

// One block: each query's place in tbuf (its records rounded up to 4 floats, so
// every query starts 16-byte aligned), in query order; a query fits when its records
// end within tcap, and only fitting queries are flagged for the split scan.
__global__ __launch_bounds__(1024) void k_split_offsets(SplitParams sp) {
    __shared__ unsigned long long wsum[32];
    __shared__ unsigned long long base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (uint32_t q0 = 0; q0 < sp.n; q0 += 1024) {
        const uint32_t q = q0 + threadIdx.x;
        const uint32_t w = q < sp.n ? sp.qcnt[q] : kSplitNo;
        const unsigned long long v = w == kSplitNo ? 0ull : ((unsigned long long)w + 3) & ~3ull;
        const unsigned long long b0 = base;
        unsigned long long x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long z = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z;
        }
        __syncthreads();
        const unsigned long long excl = b0 + (warp ? wsum[warp - 1] : 0ull) + x - v;
        if (q < sp.n) {
            const bool fits = w != kSplitNo && excl + v <= sp.tcap;
            sp.qoff[q] = fits ? (uint32_t)excl : 0u;
            sp.qflag[q] = fits ? 1u : 0u;
        }
        __syncthreads();
        if (threadIdx.x == 0) base = b0 + wsum[31];
        __syncthreads();
    }
}

template <int NSQ, bool HALF>
#ifndef PGPU_SPLIT_MINB16
#define PGPU_SPLIT_MINB16 2
#endif
__global__ __launch_bounds__(kSplitThreads, HALF ? PGPU_SPLIT_MINB16 : 2) void k_scan_score(SplitParams sp) {
    constexpr int NG = (NSQ + 7) / 8;  // 8-byte code granules per record
    constexpr uint32_t kG = NG * 8;
    constexpr uint32_t kBlk = 32 * kG + 192;  // il_block_bytes
    constexpr int NW = kSplitWarps, RB = HALF ? PGPU_SPLIT_RB16 : PGPU_SPLIT_RB32;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint32_t s_c, s_r0, s_r1, s_i0, s_i1;
    __shared__ float s_cdl;
    __shared__ float s_lo[NW], s_hi[NW];
    __shared__ uint32_t s_red[NW], s_bin;
    // the pick phase's select scratch (block_kth_hist) and counters
    __shared__ uint32_t k_red[2 * NW + 2], k_hist256[256], k_cnt, k_count, k_slots, k_out;
    __shared__ uint64_t k_sel[4];
    const uint32_t qi = sp.order[blockIdx.x];
    if (!sp.qflag[qi]) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t F = sp.F, T = sp.T;
    unsigned char* tab = smem;
    // the FP16 table takes one 4-byte slot per entry (the FP32 table's addresses and size)
    float* qv = reinterpret_cast<float*>(smem + il_table_bytes(false));
    unsigned char* rest = smem + il_table_bytes(false) + il_query_bytes(sp.d);
    float* stage = reinterpret_cast<float*>(rest);  // [NSQ][257] while the table is built
    float* srow = reinterpret_cast<float*>(rest);   // [F] afterwards
    uint32_t* hist = reinterpret_cast<uint32_t*>(rest + il_srow_bytes(F));  // [kSplitBins]
    // the probed clusters' record positions: start, base records, first memory id,
    // first inserted slot
    uint32_t* sl_start = hist + kSplitBins;  // [kSplitMaxSlots + 1]
    uint32_t* sl_nb = sl_start + kSplitMaxSlots + 1;
    uint32_t* sl_r0 = sl_nb + kSplitMaxSlots;
    uint32_t* sl_i0 = sl_r0 + kSplitMaxSlots;
    for (uint32_t i = tid; i < sp.d; i += kSplitThreads) qv[i] = sp.q[(uint64_t)qi * sp.d + i];
    const int lut_e = HALF ? half_lut_exponent(sp.qnorm[qi], sp.codebook_max) : 0;
    const float inv_scale = HALF ? ldexpf(1.0f, -lut_e) : 1.0f;
    __syncthreads();
    il_build_table<NSQ, HALF, kSplitThreads, true>(tab, stage, qv, sp.codebook, sp.lsq, lut_e);
    __syncthreads();  // stage (under srow and hist) is read to the end of the expansion
    for (uint32_t b = tid; b < kSplitBins; b += kSplitThreads) hist[b] = 0;
    // slot table: records per probed cluster, then an exclusive scan (PS slots per thread)
    const uint32_t maxl = sp.P < kSplitMaxSlots ? sp.P : kSplitMaxSlots;
    if (tid == 0) {
        k_count = 0;
        k_out = 0;
        k_slots = maxl;
    }
    __syncthreads();
    for (uint32_t l = tid; l < maxl; l += kSplitThreads)
        if (sp.ctag[(uint64_t)qi * sp.P + l] >= sp.C) atomicMin(&k_slots, l);
    __syncthreads();
    const uint32_t L = k_slots;
    {
        constexpr int PS = kSplitMaxSlots / kSplitThreads;
        uint32_t len[PS], run = 0;
#pragma unroll
        for (int j = 0; j < PS; ++j) {
            const uint32_t l = tid * PS + j;
            len[j] = 0;
            if (l < L) {
                const uint32_t c = sp.ctag[(uint64_t)qi * sp.P + l];
                const uint32_t r0 = sp.cell_start[(uint64_t)c * F], r1 = sp.cell_start[(uint64_t)c * F + F];
                uint32_t i0 = 0, i1 = 0;
                if (sp.ins_cl_start) {
                    i0 = sp.ins_cl_start[c];
                    i1 = sp.ins_cl_start[c + 1];
                }
                sl_nb[l] = r1 - r0;
                sl_r0[l] = r0;
                sl_i0[l] = i0;
                len[j] = (r1 - r0) + (i1 - i0);
            }
            run += len[j];
        }
        uint32_t incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_red[warp] = incl;
        __syncthreads();
        uint32_t st0 = incl - run;
        for (int w = 0; w < warp; ++w) st0 += s_red[w];
#pragma unroll
        for (int j = 0; j < PS; ++j) {
            const uint32_t l = tid * PS + j;
            if (l < L) sl_start[l] = st0;
            st0 += len[j];
        }
        if (tid == kSplitThreads - 1) sl_start[L] = st0;  // the total
    }
    __syncthreads();
    const uint32_t N = sl_start[L];  // records of all probed clusters
    // slot of record position ps (the last slot starting at or before it)
    auto slot_of = [&](uint32_t ps) {
        uint32_t a = 0, b = L;
        while (b - a > 1) {
            const uint32_t mid = (a + b) >> 1;
            if (sl_start[mid] <= ps) a = mid;
            else b = mid;
        }
        return a;
    };
    float* out = sp.tbuf + sp.qoff[qi];
    const float* fdk = sp.fd_by_fine + (uint64_t)qi * F;
    uint32_t pos = 0;  // records written (the same on every thread)
    float lo = 0.0f, scale = 0.0f;
    // the histogram's range: the smallest and largest of one t per thread (ok: the
    // thread has one). All threads; barrier inside.
    auto set_range = [&](float t1, bool ok) {
        float mn = ok ? t1 : __int_as_float(0x7f800000), mx = ok ? t1 : __int_as_float(0xff800000);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) {
            s_lo[warp] = mn;
            s_hi[warp] = mx;
        }
        __syncthreads();
        mn = s_lo[0];
        mx = s_hi[0];
#pragma unroll
        for (int w = 1; w < NW; ++w) {
            mn = fminf(mn, s_lo[w]);
            mx = fmaxf(mx, s_hi[w]);
        }
        if (mx > mn) {
            lo = mn;
            scale = __fdiv_rn((float)(kSplitBins - 1), __fsub_rn(mx, mn));
        } else {
            lo = mn > -3.0e38f && mn < 3.0e38f ? mn : 0.0f;
            scale = 0.0f;
        }
    };
    {
        // the histogram's range: t of one record per thread at evenly spaced positions
        // of all probed clusters (its cell term read from global memory; the range only
        // has to be the same for every record, not exact)
        const bool ok = N > 0;
        const uint32_t ps = ok ? (uint32_t)(((uint64_t)tid * N) / kSplitThreads) : 0u;
        const uint32_t a = ok ? slot_of(ps) : 0u;
        const uint32_t local = ps - sl_start[a];
        uint32_t m1[1];
        m1[0] = !ok ? 0u : local < sl_nb[a] ? sl_r0[a] + local : sp.ins_cl_ids[sl_i0[a] + (local - sl_nb[a])];
        uint2 g1[1][NG];
        float o1[1], t1[1];
        uint32_t f1[1] = {0u};
#pragma unroll
        for (int q2 = 0; q2 < NG; ++q2)
            g1[0][q2] = __ldg(reinterpret_cast<const uint2*>(sp.codes_il + il_granule_offset(m1[0], q2, NSQ)));
        o1[0] = __ldg(reinterpret_cast<const float*>(sp.codes_il + il_offset_offset(m1[0], NSQ)));
        const uint32_t fi = __ldg(reinterpret_cast<const uint16_t*>(sp.codes_il + il_fine_offset(m1[0], NSQ)));
        float cterm[1] = {0.0f};
        if (ok) {
            const uint32_t c = sp.ctag[(uint64_t)qi * sp.P + a];
            const float cd = sp.cdist[(uint64_t)qi * sp.P + a];
            cterm[0] = 2.0f * __fadd_rn(__fadd_rn(cd, __ldg(sp.stationary + (uint64_t)c * F + fi)), __ldg(fdk + fi));
        }
        il_score<NSQ, HALF, 1, true>(tab, cterm, g1, o1, f1, m1, inv_scale, t1);
        set_range(t1[0], ok);
    }
    for (uint32_t l = 0; l < L; ++l) {
        __syncthreads();  // the previous cluster's cell terms are no longer read
        if (tid == 0) {
            const uint32_t c = sp.ctag[(uint64_t)qi * sp.P + l];
            s_c = c;
            s_cdl = sp.cdist[(uint64_t)qi * sp.P + l];
            s_r0 = s_r1 = s_i0 = s_i1 = 0;
            if (c < sp.C) {
                s_r0 = sp.cell_start[(uint64_t)c * F];
                s_r1 = sp.cell_start[(uint64_t)c * F + F];
                if (sp.ins_cl_start) {
                    s_i0 = sp.ins_cl_start[c];
                    s_i1 = sp.ins_cl_start[c + 1];
                }
            }
        }
        __syncthreads();
        const uint32_t c = s_c;
        if (c >= sp.C) break;  // the probed clusters fill a prefix of the slots
        const uint32_t r0 = s_r0, r1 = s_r1, i0 = s_i0, ni = s_i1 - s_i0, nrec = r1 - r0;
        if (nrec + ni == 0) continue;
        // srow[f] = 2 * cell_dist of cell f, cell_dist = (cd + stationary) + fd
        // (puck_index.cpp:539-540)
        const float cdl = s_cdl;
        if ((F & 3u) == 0) {
            const float4* st4 = reinterpret_cast<const float4*>(sp.stationary + (uint64_t)c * F);
            const float4* fd4 = reinterpret_cast<const float4*>(fdk);
            float4* s4 = reinterpret_cast<float4*>(srow);
            for (uint32_t i = tid; i < (F >> 2); i += kSplitThreads) {
                const float4 a = __ldg(st4 + i), b = __ldg(fd4 + i);
                s4[i] = make_float4(2.0f * __fadd_rn(__fadd_rn(cdl, a.x), b.x),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.y), b.y),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.z), b.z),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.w), b.w));
            }
        } else {
            for (uint32_t i = tid; i < F; i += kSplitThreads)
                srow[i] = 2.0f * __fadd_rn(__fadd_rn(cdl, sp.stationary[(uint64_t)c * F + i]), fdk[i]);
        }
        __syncthreads();
        if (nrec > 0) {
            const uint32_t b0 = r0 >> 5, nblk = ((r1 - 1) >> 5) - b0 + 1;
            const uint32_t steps = (nblk + NW * RB - 1) / (NW * RB);
            // step j: warp w takes record blocks j * NW * RB + r * NW + w of the cluster
            auto load = [&](uint32_t j, uint2 (&g)[RB][NG], float (&o)[RB], uint32_t (&f)[RB],
                            uint32_t (&m)[RB], bool (&v)[RB]) {
#pragma unroll
                for (int r = 0; r < RB; ++r) {
                    const uint32_t bi = j * (NW * RB) + r * NW + warp;
                    m[r] = (b0 + bi) * 32u + lane;
                    v[r] = bi < nblk && m[r] - r0 < nrec;
                    if (bi < nblk) {
                        const unsigned char* rec = sp.codes_il + (uint64_t)(b0 + bi) * kBlk;
#pragma unroll
                        for (int q2 = 0; q2 < NG; ++q2)
                            g[r][q2] = __ldg(reinterpret_cast<const uint2*>(rec + q2 * 256 + 8 * lane));
                        o[r] = __ldg(reinterpret_cast<const float*>(rec + 32 * kG + 4 * lane));
                        f[r] = v[r] ? __ldg(reinterpret_cast<const uint16_t*>(rec + 32 * kG + 128 + 2 * lane))
                                    : 0u;
                    } else {
#pragma unroll
                        for (int q2 = 0; q2 < NG; ++q2) g[r][q2] = make_uint2(0u, 0u);
                        o[r] = 0.0f;
                        f[r] = 0u;
                    }
                }
            };
            // bulk L2 prefetch of step j's record blocks (one copy engine request by
            // thread 0), kSplitAhead + 1 steps before their loads are issued
            auto prefetch = [&](uint32_t j) {
                if (kSplitAhead >= 0 && tid == 0 && j < steps) {
                    const uint32_t first = j * (NW * RB);
                    const uint32_t cnt = min((uint32_t)(NW * RB), nblk - first);
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(
                                     sp.codes_il + (uint64_t)(b0 + first) * kBlk),
                                 "r"(cnt * kBlk)
                                 : "memory");
                }
            };
            for (int j = 1; j <= kSplitAhead; ++j) prefetch((uint32_t)j);
            // two register sets, A and B, in turn: step j + 1's loads go into one set
            // while step j is scored from the other (no copies between steps)
            uint2 ga[RB][NG], gb[RB][NG];
            float oa[RB], ob[RB];
            uint32_t fa[RB], fb[RB], ma[RB], mb[RB];
            bool va[RB], vb[RB];
            auto emit = [&](const uint2 (&g)[RB][NG], const float (&o)[RB], const uint32_t (&f)[RB],
                            const uint32_t (&m)[RB], const bool (&v)[RB]) {
                float t[RB];
                il_score<NSQ, HALF, RB, true>(tab, srow, g, o, f, m, inv_scale, t);
#pragma unroll
                for (int r = 0; r < RB; ++r)
                    if (v[r]) {
                        out[pos + (m[r] - r0)] = t[r];
                        atomicAdd(&hist[split_bin(t[r], lo, scale)], 1u);
                    }
            };
            load(0, ga, oa, fa, ma, va);
            for (uint32_t j = 0; j < steps; j += 2) {
                prefetch(j + kSplitAhead + 1);
                if (j + 1 < steps) load(j + 1, gb, ob, fb, mb, vb);
                emit(ga, oa, fa, ma, va);
                if (j + 1 < steps) {
                    prefetch(j + kSplitAhead + 2);
                    if (j + 2 < steps) load(j + 2, ga, oa, fa, ma, va);
                    emit(gb, ob, fb, mb, vb);
                }
            }
            pos += nrec;
        }
        // realtime: the cluster's inserted records (gathered from the interleaved copy)
        for (uint32_t v0 = 0; v0 < ni; v0 += kSplitThreads * RB) {
            uint2 g[RB][NG];
            float o[RB], t[RB];
            uint32_t f[RB], m[RB];
            bool v[RB];
#pragma unroll
            for (int r = 0; r < RB; ++r) {
                const uint32_t vi = v0 + r * kSplitThreads + tid;
                v[r] = vi < ni;
                m[r] = v[r] ? sp.ins_cl_ids[i0 + vi] : 0u;
#pragma unroll
                for (int q2 = 0; q2 < NG; ++q2)
                    g[r][q2] = __ldg(reinterpret_cast<const uint2*>(sp.codes_il + il_granule_offset(m[r], q2, NSQ)));
                o[r] = __ldg(reinterpret_cast<const float*>(sp.codes_il + il_offset_offset(m[r], NSQ)));
                f[r] = v[r] ? __ldg(reinterpret_cast<const uint16_t*>(sp.codes_il + il_fine_offset(m[r], NSQ)))
                            : 0u;
            }
            il_score<NSQ, HALF, RB, true>(tab, srow, g, o, f, m, inv_scale, t);
#pragma unroll
            for (int r = 0; r < RB; ++r)
                if (v[r]) {
                    out[pos + v0 + r * kSplitThreads + tid] = t[r];
                    atomicAdd(&hist[split_bin(t[r], lo, scale)], 1u);
                }
        }
        pos += ni;
    }
    __syncthreads();
    // the cut: the first bin at which the running count reaches T (every bin when
    // the query has no more than T records)
    uint32_t bstar = kSplitBins - 1;
    if (pos > T) {
        constexpr int PB = kSplitBins / kSplitThreads;
        uint32_t cb[PB], run = 0;
#pragma unroll
        for (int j = 0; j < PB; ++j) {
            cb[j] = hist[tid * PB + j];
            run += cb[j];
        }
        uint32_t incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_red[warp] = incl;
        __syncthreads();
        uint32_t below = incl - run;
        for (int w = 0; w < warp; ++w) below += s_red[w];
        if (below < T && T <= below + run) {
#pragma unroll
            for (int j = 0; j < PB; ++j) {
                if (below < T && T <= below + cb[j]) s_bin = tid * PB + j;
                below += cb[j];
            }
        }
        __syncthreads();
        bstar = s_bin;
    }
    // ---- pick: the records at or below the cut bin, read back from this block's own
    // distances (recently written, mostly still in L2), as (t bits, position) keys in
    // the table's place; positions to memory ids; the exact T smallest (t, id) out.
    __syncthreads();  // the table, the cell terms and the histogram are no longer read
    constexpr uint32_t kKeys = split_max_keys(false);
    uint64_t* keys = reinterpret_cast<uint64_t*>(tab);
    uint32_t* khist = hist;  // [kHistBins] block_kth_hist scratch
    // candidates: each thread marks its 16 values of a step, a warp scan of the marks
    // gives each thread its first slot (one shared atomic per warp and step)
    const float4* tb4 = reinterpret_cast<const float4*>(out);  // out is 16-byte aligned
    const uint32_t n4 = (N + 3) / 4;
    for (uint32_t i0 = 0; i0 < n4; i0 += kSplitThreads * 4) {
        float4 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t i = i0 + u * kSplitThreads + tid;
            x[u] = i < n4 ? __ldcg(tb4 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        uint32_t mask = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t i = i0 + u * kSplitThreads + tid;
            const float tv[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const bool keep = i < n4 && i * 4 + e < N && split_bin(tv[e], lo, scale) <= bstar;
                mask |= keep ? 1u << (u * 4 + e) : 0u;
            }
        }
        const uint32_t c = __popc(mask);
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        uint32_t base = 0;
        if (lane == 31 && incl) base = atomicAdd(&k_count, incl);
        base = __shfl_sync(0xffffffffu, base, 31);
        uint32_t slot = base + incl - c;
        while (mask) {
            const int b = __ffs(mask) - 1;
            mask &= mask - 1;
            const int u = b >> 2, e = b & 3;
            const uint32_t ps = (i0 + u * kSplitThreads + tid) * 4 + e;
            float tv = 0.0f;  // x[u] element e, by selects (no local-memory array)
#pragma unroll
            for (int uu = 0; uu < 4; ++uu)
                if (uu == u) tv = e == 0 ? x[uu].x : e == 1 ? x[uu].y : e == 2 ? x[uu].z : x[uu].w;
            if (slot < kKeys) keys[slot] = ((uint64_t)__float_as_uint(tv) << 32) | ps;
            ++slot;
        }
    }
    __syncthreads();
    const uint32_t m = k_count;
    if (m > kKeys) {  // too many records in the cut bin: k_scan_il takes the query
        if (tid == 0) sp.qflag[qi] = 0;
        return;
    }
    // positions to memory ids: the slot holding the position (binary search), then the
    // base record or the inserted one
    for (uint32_t i = tid; i < m; i += kSplitThreads) {
        const uint64_t k = keys[i];
        const uint32_t ps = (uint32_t)k;
        const uint32_t a = slot_of(ps);
        const uint32_t local = ps - sl_start[a];
        const uint32_t id =
            local < sl_nb[a] ? sl_r0[a] + local : sp.ins_cl_ids[sl_i0[a] + (local - sl_nb[a])];
        keys[i] = filter_key(__uint_as_float((uint32_t)(k >> 32)), id);
    }
    __syncthreads();
    // the exact T smallest: the keys up to the T-th (all of them when m <= T), written
    // unordered like k_scan_il's
    const uint64_t bound =
        m > T ? block_kth_hist<kSplitThreads>(keys, m, T, khist, k_red, &k_cnt, k_hist256, k_sel) + 1
              : kKeyMax;
    for (uint32_t i0 = 0; i0 < m; i0 += kSplitThreads) {
        const uint32_t i = i0 + tid;
        const uint64_t k = i < m ? keys[i] : kKeyMax;
        const bool keep = k < bound;
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if (b) {
            uint32_t base = 0;
            if (lane == __ffs(b) - 1) base = atomicAdd(&k_out, (uint32_t)__popc(b));
            base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
            if (keep) {
                const uint32_t slot = base + __popc(b & ((1u << lane) - 1));
                sp.hdist[(uint64_t)qi * T + slot] = key_value(k);
                sp.htag[(uint64_t)qi * T + slot] = (uint32_t)k;
            }
        }
    }
    __syncthreads();
    const uint32_t outn = k_out;  // min(m, T)
    for (uint32_t i = outn + tid; i < T; i += kSplitThreads) {
        sp.hdist[(uint64_t)qi * T + i] = sentinel_f();
        sp.htag[(uint64_t)qi * T + i] = kNoLabel;
    }
    if (tid == 0) {
        sp.hcnt[qi] = outn;
        if (sp.counters) {
            atomicAdd(sp.counters + kScRecords, (unsigned long long)N);
            atomicAdd(sp.counters + kScKept, (unsigned long long)m);
        }
    }
}

}  // namespace

// Shared memory of the interleaved kernel (il_applies(nsq)) for filter_topk T.
static size_t il_smem_bytes(const DeviceIndex& ix, uint32_t T, bool half) {
    const size_t stage = sizeof(float) * ix.nsq * 257;
    const size_t work = il_srow_bytes(ix.F) +
                        sizeof(uint64_t) * (half ? il_cap<true>(T) : il_cap<false>(T)) +
                        sizeof(uint32_t) * kHistBins;
    const size_t ring = half ? (size_t)IlShape<true>::kStages * il_slot_bytes<true>(ix.nsq)
                             : (size_t)IlShape<false>::kStages * il_slot_bytes<false>(ix.nsq);
    return il_table_bytes(half) + il_query_bytes(ix.d) + ring +
           (stage > work ? stage : work);
}

size_t scan_smem_bytes(const DeviceIndex& ix, uint32_t T) {
    if (il_applies(ix.nsq)) return il_smem_bytes(ix, T, false);
    return sizeof(uint64_t) * scan_cap(T) + sizeof(uint32_t) * kHistBins +
           sizeof(float) * ix.nsq * 256 + sizeof(float) * ix.F + sizeof(float) * ix.d;
}

size_t scan_smem_bytes_half(const DeviceIndex& ix, uint32_t T) {
    if (il_applies(ix.nsq)) return il_smem_bytes(ix, T, true);
    return sizeof(uint64_t) * scan_cap(T) + sizeof(uint32_t) * kHistBins +
           sizeof(__half) * ix.nsq * 256 + sizeof(float) * ix.F + sizeof(float) * ix.d;
}

// The buffer takes T + a round + at least 1024 more keys between cuts.
uint32_t scan_max_filter_topk() { return kMaxCap - kRound - 1024; }

cudaError_t launch_scan_order(const DeviceIndex& ix, uint32_t n, Scratch& s, cudaStream_t stream) {
    if (s.order == nullptr || s.wbucket == nullptr) return cudaErrorInvalidValue;
    k_scan_work<<<(n + 255) / 256, 256, 0, stream>>>(s.ctag, s.status, ix.cell_start,
                                                     ix.ins_n ? ix.ins_cl_start : nullptr, n, s.P,
                                                     ix.C, ix.F, s.wbucket);
    k_scan_order<<<1, kOrderThreads, 0, stream>>>(s.wbucket, n, s.order);
    return cudaGetLastError();
}

// Shared memory of k_scan_score: the table, the query, then the compact table being
// built or the cell terms and the histogram.
static size_t split_score_smem(const DeviceIndex& ix, bool half) {
    (void)half;  // the FP16 table takes the FP32 table's slots
    const size_t stage = sizeof(float) * ix.nsq * 257;
    const size_t work = il_srow_bytes(ix.F) + sizeof(uint32_t) * (kSplitBins + 4 * kSplitMaxSlots + 1);
    return il_table_bytes(false) + il_query_bytes(ix.d) + (stage > work ? stage : work);
}

bool scan_split_possible(const DeviceIndex& ix, uint32_t T) {
    return il_applies(ix.nsq) && split_score_smem(ix, false) <= 220 * 1024 &&
           T < split_max_keys(false);
}

bool scan_split_applies(const DeviceIndex& ix, const Scratch& s) {
    return ix.codes_il != nullptr && s.tbuf != nullptr && s.tcap > 0 && scan_split_possible(ix, s.T);
}

static SplitParams split_params(const DeviceIndex& ix, uint32_t n, Scratch& s) {
    SplitParams sp;
    sp.ctag = s.ctag;
    sp.cdist = s.cdist;
    sp.status = s.status;
    sp.cell_start = ix.cell_start;
    sp.ins_cl_start = ix.ins_n ? ix.ins_cl_start : nullptr;
    sp.ins_cl_ids = ix.ins_cl_ids;
    sp.stationary = ix.stationary;
    sp.fd_by_fine = s.dots;
    sp.q = s.q;
    sp.qnorm = s.qnorm;
    sp.codebook = ix.codebook;
    sp.codes_il = ix.codes_il;
    sp.order = s.order;
    sp.qcnt = s.qcnt;
    sp.qoff = s.qoff;
    sp.qflag = s.qflag;
    sp.cut = s.cut;
    sp.tbuf = s.tbuf;
    sp.hdist = s.hdist;
    sp.htag = s.htag;
    sp.hcnt = s.hcnt;
    sp.counters = s.counters;
    sp.tcap = s.tcap;
    sp.n = n;
    sp.d = ix.d;
    sp.C = ix.C;
    sp.F = ix.F;
    sp.lsq = ix.lsq;
    sp.P = s.P;
    sp.T = s.T;
    sp.codebook_max = ix.codebook_max;
    return sp;
}

static cudaError_t launch_fused(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                                const uint32_t* done, cudaStream_t stream) {
    ScanParams p;
    p.q = s.q;
    p.qnorm = s.qnorm;
    p.status = s.status;
    p.cdist = s.cdist;
    p.ctag = s.ctag;
    p.fd_by_fine = s.dots;
    p.hdist = s.hdist;
    p.htag = s.htag;
    p.hcnt = s.hcnt;
    p.stationary = ix.stationary;
    p.cell_start = ix.cell_start;
    p.rec_fine = ix.rec_fine;
    p.offsets = ix.offsets;
    p.codes = ix.codes;
    p.codes_il = ix.codes_il;
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
    p.cap = scan_cap(s.T);
    p.codebook_max = ix.codebook_max;
    if (s.order == nullptr || s.T > scan_max_filter_topk()) return cudaErrorInvalidValue;
    p.order = s.order;
    p.err = s.tc_err;
    p.ins_cl_start = ix.ins_n ? ix.ins_cl_start : nullptr;
    p.ins_cl_ids = ix.ins_cl_ids;
    p.done = done;
    const size_t smem = half_lut ? scan_smem_bytes_half(ix, s.T) : scan_smem_bytes(ix, s.T);
    const uint32_t nw = ix.code_stride / 4;
    auto launch = [&](void (*kernel)(ScanParams), int threads) {
        ensure_max_dynamic_smem(kernel, 220 * 1024);
        kernel<<<n, threads, smem, stream>>>(p);
    };
    if (il_applies(ix.nsq)) {
        if (ix.codes_il == nullptr) return cudaErrorInvalidValue;
        p.cap = half_lut ? il_cap<true>(s.T) : il_cap<false>(s.T);
        switch (ix.nsq) {
#define PGPU_IL(N) \
    case N:                                                                                \
        if (half_lut) launch(k_scan_il<N, true>, IlShape<true>::kThreads);                   \
        else launch(k_scan_il<N, false>, IlShape<false>::kThreads);                          \
        break;
            PGPU_IL(4) PGPU_IL(8) PGPU_IL(12) PGPU_IL(16) PGPU_IL(20) PGPU_IL(24) PGPU_IL(28)
            PGPU_IL(32)
#undef PGPU_IL
            default: return cudaErrorInvalidValue;
        }
    } else if (half_lut) {
        if (nw <= 2) launch(k_scan_select<2, kTabF16>, kThreads);
        else if (nw <= 4) launch(k_scan_select<4, kTabF16>, kThreads);
        else if (nw <= 6) launch(k_scan_select<6, kTabF16>, kThreads);
        else if (nw <= 8) launch(k_scan_select<8, kTabF16>, kThreads);
        else launch(k_scan_select<16, kTabF16>, kThreads);
    } else {
        if (nw <= 2) launch(k_scan_select<2, kTabF32>, kThreads);
        else if (nw <= 4) launch(k_scan_select<4, kTabF32>, kThreads);
        else if (nw <= 6) launch(k_scan_select<6, kTabF32>, kThreads);
        else if (nw <= 8) launch(k_scan_select<8, kTabF32>, kThreads);
        else launch(k_scan_select<16, kTabF32>, kThreads);
    }
    return cudaGetLastError();
}

cudaError_t launch_scan_prepare(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                                cudaStream_t stream) {
    if (!scan_split_applies(ix, s)) return cudaSuccess;
    (void)half_lut;
    const SplitParams sp = split_params(ix, n, s);
    k_split_counts<<<(n + 255) / 256, 256, 0, stream>>>(sp);
    k_split_offsets<<<1, 1024, 0, stream>>>(sp);
    return cudaGetLastError();
}

cudaError_t launch_scan_records(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                                cudaStream_t stream) {
    if (!scan_split_applies(ix, s)) return launch_fused(ix, n, s, half_lut, nullptr, stream);
    const SplitParams sp = split_params(ix, n, s);
    const size_t smem = split_score_smem(ix, half_lut);
    auto score = [&](void (*kernel)(SplitParams)) {
        ensure_max_dynamic_smem(reinterpret_cast<const void*>(kernel), 220 * 1024);
        kernel<<<n, kSplitThreads, smem, stream>>>(sp);
    };
    switch (ix.nsq) {
#define PGPU_SPLIT(N)                           \
    case N:                                     \
        if (half_lut) score(k_scan_score<N, true>); \
        else score(k_scan_score<N, false>);     \
        break;
        PGPU_SPLIT(4) PGPU_SPLIT(8) PGPU_SPLIT(12) PGPU_SPLIT(16) PGPU_SPLIT(20) PGPU_SPLIT(24)
        PGPU_SPLIT(28) PGPU_SPLIT(32)
#undef PGPU_SPLIT
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_scan_finish(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                               cudaStream_t stream) {
    if (!scan_split_applies(ix, s)) return cudaSuccess;
    // the fused kernel takes the queries the split scan did not answer (its blocks for
    // answered queries return at once)
    return launch_fused(ix, n, s, half_lut, s.qflag, stream);
}

}  // namespace pgpu
