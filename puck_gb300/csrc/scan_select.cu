// k_scan_select: throughput-mode filter stage. For one query it streams every
// filter record of its probed coarse clusters (each cluster is one contiguous
// range in memory order) and keeps the filter_topk smallest ADC distances.
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
// Selection: a buffer of (t, id) keys in shared memory with a running threshold
// tau, a key with at least filter_topk kept keys at or below it; records whose
// (2*cell_dist + offset, id) key is not below tau are dropped before the table
// lookups (t can only grow). When the buffer could not take another round, an
// MSB radix select (two digit passes) finds a new bound and the keys above it are
// dropped. A last exact select leaves the set of the filter_topk smallest (t, id)
// keys, unordered.
//
// Blocks start in launch order longest scan first (k_scan_work, k_scan_order),
// one block per query.
//
// Precision form (HALF): the table is stored in FP16, scaled per query by a
// power of two 2^e chosen from the bound (|q| + max |codeword|)^2 >= every entry
// so that all entries stay below 32768; lookups are accumulated in FP32 and the
// sum is multiplied by 2^-e. Entries are non-negative, so t >= t0 still holds and
// the threshold test before the lookups stays valid.
#include <cuda_fp16.h>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

// Block shape of the scan (compile-time; -D overrides for tuning sweeps).
#ifndef PGPU_SCAN_THREADS
#define PGPU_SCAN_THREADS 128
#endif
#ifndef PGPU_SCAN_RECORDS
#define PGPU_SCAN_RECORDS 4
#endif
#ifndef PGPU_SCAN_CAP
#define PGPU_SCAN_CAP 1792
#endif
#ifndef PGPU_SCAN_MIN_BLOCKS
#define PGPU_SCAN_MIN_BLOCKS 8
#endif
constexpr int kThreads = PGPU_SCAN_THREADS;
constexpr int kRecPerThread = PGPU_SCAN_RECORDS;
constexpr int kRound = kThreads * kRecPerThread;  // records per round
constexpr uint32_t kCandCap = PGPU_SCAN_CAP;      // candidate buffer (keys)
static_assert(kCandCap % kThreads == 0 && kCandCap > (uint32_t)kRound,
              "the buffer holds a round beyond the kept keys");

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
    const float* codebook;
    unsigned long long* counters;
    const unsigned char* luts;  // [B][lut_bytes] tables from k_build_luts
    const uint32_t* order;      // [B] query of each block
    int* err;                   // set when the table copy did not arrive in time
    uint32_t d, C, F, nsq, lsq, code_stride, P, T, lut_bytes;
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

// get_dist_table (quantization.cpp:260-270) for a batch: kLutQueries queries per
// block, thread j computes codeword j of every subspace for each of them (coalesced
// 16-byte codebook loads, 8 subspaces in flight, each codeword loaded once for the
// block's queries), in the reference's lane order (l2sqr_sse).
constexpr uint32_t kLutQueries = 8;
template <bool HALF>
__global__ __launch_bounds__(256) void k_build_luts(const float* __restrict__ q,
                                                    const float* __restrict__ qnorm,
                                                    const int32_t* __restrict__ status,
                                                    const float* __restrict__ cb, uint32_t n,
                                                    uint32_t d, uint32_t nsq, uint32_t lsq,
                                                    float codebook_max,
                                                    unsigned char* __restrict__ luts) {
    __shared__ float qs[kLutQueries][kMaxDim];
    __shared__ float qscale[kLutQueries];
    __shared__ int qok[kLutQueries];
    const uint32_t q0 = blockIdx.x * kLutQueries, j = threadIdx.x;
    const uint32_t nq = n - q0 < kLutQueries ? n - q0 : kLutQueries;
    for (uint32_t t = j; t < nq * d; t += 256) qs[t / d][t % d] = q[(uint64_t)q0 * d + t];
    if (j < nq) {
        qok[j] = status[q0 + j] == 0;
        qscale[j] = HALF ? ldexpf(1.0f, half_lut_exponent(qnorm[q0 + j], codebook_max)) : 1.0f;
    }
    __syncthreads();
    auto store = [&](uint32_t u, uint32_t m, float v) {
        const uint64_t at = (uint64_t)(q0 + u) * nsq * 256 + m * 256 + j;
        if (HALF) reinterpret_cast<__half*>(luts)[at] = __float2half_rn(v * qscale[u]);
        else reinterpret_cast<float*>(luts)[at] = v;
    };
    if (lsq == 4) {
        const float4* cb4 = reinterpret_cast<const float4*>(cb);
        for (uint32_t m0 = 0; m0 < nsq; m0 += 8) {
            float4 y[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (m0 + u < nsq) y[u] = __ldg(cb4 + (uint64_t)(m0 + u) * 256 + j);
            for (uint32_t qq = 0; qq < nq; ++qq) {
                if (!qok[qq]) continue;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const uint32_t m = m0 + u;
                    if (m >= nsq) break;
                    const float* x = qs[qq] + m * 4;
                    const float t0 = __fsub_rn(x[0], y[u].x), t1 = __fsub_rn(x[1], y[u].y);
                    const float t2 = __fsub_rn(x[2], y[u].z), t3 = __fsub_rn(x[3], y[u].w);
                    store(qq, m, __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)),
                                           __fadd_rn(__fmul_rn(t2, t2), __fmul_rn(t3, t3))));
                }
            }
        }
    } else {
        for (uint32_t m = 0; m < nsq; ++m)
            for (uint32_t qq = 0; qq < nq; ++qq)
                if (qok[qq])
                    store(qq, m, l2sqr_sse(qs[qq] + m * lsq, cb + ((uint64_t)m * 256 + j) * lsq, lsq));
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
__device__ uint64_t block_select_kth(const uint64_t* keys, uint32_t count, uint32_t K,
                                     uint32_t* hist, uint64_t* sel, int max_digits = 0) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the leading bits every key shares need no pass: start at the digit where the
    // smallest and the largest key first differ
    uint64_t lo = ~0ull, hi = 0;
    for (uint32_t i = tid; i < count; i += kThreads) {
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
    __shared__ uint64_t red_lo[kThreads / 32], red_hi[kThreads / 32];
    if (lane == 0) {
        red_lo[warp] = lo;
        red_hi[warp] = hi;
    }
    __syncthreads();
    lo = red_lo[0];
    hi = red_hi[0];
    for (int w = 1; w < kThreads / 32; ++w) {
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
        for (int i = tid; i < 256; i += kThreads) hist[i] = 0;
        __syncthreads();
        for (uint32_t i0 = 0; i0 < count; i0 += kThreads) {
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
            for (uint32_t i = tid; i < count; i += kThreads)
                if ((keys[i] & mask) == prefix) sel[3] = keys[i];
            __syncthreads();
            const uint64_t r = sel[3];
            __syncthreads();
            return r;
        }
    }
    return prefix;
}

// Keeps the keys <= kth (exactly K of them, in arbitrary order) at the front;
// returns nothing, every thread must call it. `cnt` is a shared counter.
template <int PER>
__device__ void block_compact_le(uint64_t* keys, uint32_t count, uint64_t kth, uint32_t* cnt) {
    const int tid = threadIdx.x, lane = tid & 31;
    uint64_t mine[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const uint32_t i = tid + j * kThreads;
        mine[j] = i < count ? keys[i] : ~0ull;
    }
    if (tid == 0) *cnt = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        const bool keep = mine[j] <= kth;
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        uint32_t base = 0;
        if (b) {
            if (lane == __ffs(b) - 1) base = atomicAdd(cnt, (uint32_t)__popc(b));
            base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);
        }
        if (keep) keys[base + __popc(b & ((1u << lane) - 1))] = mine[j];
    }
    __syncthreads();
}

// Diagnostic counters (pgpu_walk_counters slots, summed per launch): 0 records
// evaluated, 1 records past the cell-distance test (table lookups), 2 records kept, 3 compactions, 5 max records of one query, and
// thread-0 clock cycles: 6 prologue (LUT, fine terms), 7 whole block, 8 record
// rounds, 9 compaction sorts, 10 final sort + output.
enum { kScRecords = 0, kScLookups = 1, kScKept = 2, kScCompactions = 3, kScMaxRecords = 5, kScCycPrologue = 6,
       kScCycTotal = 7, kScCycRounds = 8, kScCycCompact = 9, kScCycFinal = 10 };

struct ScanState {
    uint64_t tau;
    uint64_t sel[4];
    uint64_t lut_bar;
    uint32_t hist[256];
    uint32_t ccount;
    uint32_t count;
    uint32_t c;
    float cdl;
    uint32_t r0, r1;
    unsigned long long evaluated, looked, passed;
    unsigned long long cyc_rounds, cyc_compact, n_compact, n_records;
};

// NW = code words per record (code_stride / 4); HALF = FP16 table.
template <int NW, bool HALF>
__global__ __launch_bounds__(kThreads, PGPU_SCAN_MIN_BLOCKS) void k_scan_select(ScanParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ScanState st;
    const uint32_t qi = p.order[blockIdx.x];
    const int tid = threadIdx.x;
    const uint32_t nsq = p.nsq, F = p.F, T = p.T;
    float* lut = reinterpret_cast<float*>(smem + sizeof(uint64_t) * kCandCap);
    __half* luth = reinterpret_cast<__half*>(lut);
    float* srow = HALF ? reinterpret_cast<float*>(luth + nsq * 256)
                       : lut + nsq * 256;  // [F] 2 * cell_dist of the current cluster's cells
    uint64_t* keys = reinterpret_cast<uint64_t*>(smem);  // [kCandCap], first (8-byte aligned)
    float* qv = srow + F;                  // [d]

    if (p.status[qi] != 0) {
        if (tid == 0) p.hcnt[qi] = 0;
        return;
    }
    const long long t_start = clock64();
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&st.lut_bar);
    if (tid == 0) {
        // the query's table (from k_build_luts): one bulk async copy global -> shared
        // (TMA), counted in bytes on an mbarrier; it lands while the block sets up
        // its first cluster
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1u));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "r"(p.lut_bytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"((uint32_t)__cvta_generic_to_shared(lut)),
            "l"(p.luts + (uint64_t)qi * p.lut_bytes), "r"(p.lut_bytes), "r"(bar)
            : "memory");
    }
    bool lut_ready = false;
    // Waits (bounded) for the table; on expiry flags the pass and builds the same
    // table here. Every thread calls it.
    auto wait_lut = [&]() {
        uint32_t done = 0;
        for (uint32_t it = 0; it < (1u << 22) && !done; ++it) {
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                "selp.b32 %0, 1, 0, p;\n}"
                : "=r"(done)
                : "r"(bar), "r"(0u)
                : "memory");
        }
        if (!__syncthreads_and(done != 0)) {
            if (tid == 0) atomicExch(p.err, 2);
            if (HALF) {
                const float scale =
                    ldexpf(1.0f, half_lut_exponent(p.qnorm[qi], p.codebook_max));
                for (uint32_t e = tid; e < nsq * 256; e += kThreads)
                    luth[e] = __float2half_rn(
                        l2sqr_sse(qv + (e >> 8) * p.lsq, p.codebook + (uint64_t)e * p.lsq, p.lsq) *
                        scale);
            } else {
                build_lut(lut, qv, p.codebook, nsq, p.lsq, kThreads);
            }
            __syncthreads();
        }
        lut_ready = true;
    };
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
    __syncthreads();
    const float inv_scale = HALF ? ldexpf(1.0f, -half_lut_exponent(p.qnorm[qi], p.codebook_max)) : 1.0f;
    unsigned long long my_eval = 0, my_look = 0, my_pass = 0;
    __syncthreads();
    const long long t_pro = clock64();
    for (uint32_t l = 0; l < p.P; ++l) {
        __syncthreads();
        if (tid == 0) {
            const uint32_t c = p.ctag[(uint64_t)qi * p.P + l];
            st.c = c;
            st.cdl = p.cdist[(uint64_t)qi * p.P + l];
            if (c < p.C) {
                st.r0 = p.cell_start[(uint64_t)c * F];
                st.r1 = p.cell_start[(uint64_t)c * F + F];
            } else {
                st.r0 = st.r1 = 0;  // never taken for finite queries
            }
        }
        __syncthreads();
        const uint32_t c = st.c, r0 = st.r0, r1 = st.r1;
        const float cdl = st.cdl;
        if (r0 >= r1) continue;
        // per fine id of this cluster: 2 * cell_dist, cell_dist = (cd + stationary) + fd
        if ((F & 3u) == 0) {
            // 16-byte rows (F % 4 == 0): one float4 of each row per step
            const float4* st4 = reinterpret_cast<const float4*>(p.stationary + (uint64_t)c * F);
            const float4* fd4 = reinterpret_cast<const float4*>(fdk);
            float4* s4 = reinterpret_cast<float4*>(srow);
            for (uint32_t i = tid; i < (F >> 2); i += kThreads) {
                const float4 a = __ldg(st4 + i), b = __ldg(fd4 + i);
                s4[i] = make_float4(2.0f * __fadd_rn(__fadd_rn(cdl, a.x), b.x),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.y), b.y),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.z), b.z),
                                    2.0f * __fadd_rn(__fadd_rn(cdl, a.w), b.w));
            }
        } else {
            for (uint32_t i = tid; i < F; i += kThreads)
                srow[i] = 2.0f * __fadd_rn(__fadd_rn(cdl, p.stationary[(uint64_t)c * F + i]), fdk[i]);
        }
        if (!lut_ready) wait_lut();
        __syncthreads();
        if (tid == 0) st.n_records += r1 - r0;
        for (uint32_t base = r0; base < r1; base += kRound) {
            const long long t_round = clock64();
            const uint64_t tau = st.tau;
            // all loads of the thread's records first, so their latencies overlap
            uint32_t fine_id[kRecPerThread];
            float off[kRecPerThread];
            uint32_t words[kRecPerThread][NW];
#pragma unroll
            for (int j = 0; j < kRecPerThread; ++j) {
                const uint32_t mi = base + tid + j * kThreads;
                const uint32_t mr = mi < r1 ? mi : r0;
                fine_id[j] = p.rec_fine[mr];
                off[j] = p.offsets[mr];
                const uint32_t* cw = reinterpret_cast<const uint32_t*>(p.codes + (uint64_t)mr * p.code_stride);
#pragma unroll
                for (int i = 0; i < NW; ++i) words[j][i] = __ldg(cw + i);
            }
            // one shared atomic per warp for the kept records
            auto insert = [&](bool keep, uint64_t key) {
                const unsigned ballot = __ballot_sync(0xffffffffu, keep);
                if (ballot) {
                    const int lane = tid & 31;
                    uint32_t base_slot = 0;
                    if (lane == __ffs(ballot) - 1) base_slot = atomicAdd(&st.count, (uint32_t)__popc(ballot));
                    base_slot = __shfl_sync(0xffffffffu, base_slot, __ffs(ballot) - 1);
                    if (keep) {
                        // capacity is kept >= count + kRound by the compaction below
                        keys[base_slot + __popc(ballot & ((1u << lane) - 1))] = key;
                        ++my_pass;
                    }
                }
            };
#pragma unroll
            for (int j = 0; j < kRecPerThread; ++j) {
                const uint32_t mi = base + tid + j * kThreads;
                bool keep = false;
                uint64_t key = 0;
                if (mi < r1) {
                    // (float)(2.0 * cell_dist + offset): one float add of the exact
                    // 2 * cell_dist (see adc_base)
                    const float t0 = __fadd_rn(srow[fine_id[j]], off[j]);
                    ++my_eval;
                    if (filter_key(t0, mi) < tau) {  // t can only grow past t0
                        ++my_look;
                        const float t =
                            HALF ? t0 + lut_sum_words_half<NW>(words[j], luth, nsq) * inv_scale
                                 : __fadd_rn(t0, lut_sum_words<NW>(words[j], lut, nsq));
                        key = filter_key(t, mi);
                        keep = key < tau;
                    }
                }
                insert(keep, key);
            }
            __syncthreads();
            const long long t_round_end = clock64();
            if (tid == 0) st.cyc_rounds += (unsigned long long)(t_round_end - t_round);
            // cut back when the buffer could not take another round
            if (st.count > kCandCap - kRound) {
                // cut back to a bound with at least T keys below it (two digit passes;
                // the final select below is exact); tau = that bound. If the bound's
                // bucket kept too many to take another round, cut exactly to T.
                const uint32_t cnt = st.count;
                uint64_t kth = block_select_kth(keys, cnt, T, st.hist, st.sel, 2);
                block_compact_le<kCandCap / kThreads>(keys, cnt, kth, &st.ccount);
                const uint32_t kept = st.ccount;
                if (kept > kCandCap - kRound) {
                    kth = block_select_kth(keys, kept, T, st.hist, st.sel);
                    block_compact_le<kCandCap / kThreads>(keys, kept, kth, &st.ccount);
                }
                if (tid == 0) {
                    st.count = st.ccount;
                    st.tau = kth;
                    st.n_compact += 1;
                    st.cyc_compact += (unsigned long long)(clock64() - t_round_end);
                }
                __syncthreads();
            }
        }
    }
    if (!lut_ready) wait_lut();  // no copy may be in flight when the block exits
    __syncthreads();
    const long long t_final = clock64();
    uint32_t count = st.count;
    if (count > T) {
        const uint64_t kth = block_select_kth(keys, count, T, st.hist, st.sel);
        block_compact_le<kCandCap / kThreads>(keys, count, kth, &st.ccount);
        count = T;
    }
    // the T survivors leave unordered: only the rerank's tie path needs their
    // (t, id) order, and it sorts them itself
    const uint32_t out = count < T ? count : T;
    for (uint32_t i = tid; i < T; i += kThreads) {
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
                            const uint32_t* __restrict__ cell_start, uint32_t n, uint32_t P,
                            uint32_t C, uint32_t F, uint8_t* __restrict__ wbucket) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    uint32_t w = 0;
    if (status[q] == 0) {
        for (uint32_t l = 0; l < P; ++l) {
            const uint32_t c = ctag[(uint64_t)q * P + l];
            if (c < C) w += cell_start[(uint64_t)c * F + F] - cell_start[(uint64_t)c * F];
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

}  // namespace

size_t scan_smem_bytes(const DeviceIndex& ix) {
    return sizeof(uint64_t) * kCandCap + sizeof(float) * ix.nsq * 256 + sizeof(float) * ix.F +
           sizeof(float) * ix.d;
}

size_t scan_smem_bytes_half(const DeviceIndex& ix) {
    return sizeof(uint64_t) * kCandCap + sizeof(__half) * ix.nsq * 256 + sizeof(float) * ix.F +
           sizeof(float) * ix.d;
}

uint32_t scan_max_filter_topk() { return kCandCap - kRound; }

cudaError_t launch_scan_select(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                               cudaStream_t stream) {
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
    p.codebook_max = ix.codebook_max;
    p.luts = reinterpret_cast<const unsigned char*>(s.luts);
    p.lut_bytes = ix.nsq * 256 * (half_lut ? 2 : 4);
    p.err = s.tc_err;
    if (s.luts == nullptr || s.order == nullptr || s.wbucket == nullptr) return cudaErrorInvalidValue;
    k_scan_work<<<(n + 255) / 256, 256, 0, stream>>>(s.ctag, s.status, ix.cell_start, n, s.P, ix.C,
                                                     ix.F, s.wbucket);
    k_scan_order<<<1, kOrderThreads, 0, stream>>>(s.wbucket, n, s.order);
    p.order = s.order;
    {
        const dim3 g((n + kLutQueries - 1) / kLutQueries);
        if (half_lut)
            k_build_luts<true><<<g, 256, 0, stream>>>(s.q, s.qnorm, s.status, ix.codebook, n, ix.d,
                                                      ix.nsq, ix.lsq, ix.codebook_max, s.luts);
        else
            k_build_luts<false><<<g, 256, 0, stream>>>(s.q, s.qnorm, s.status, ix.codebook, n, ix.d,
                                                       ix.nsq, ix.lsq, ix.codebook_max, s.luts);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const size_t smem = half_lut ? scan_smem_bytes_half(ix) : scan_smem_bytes(ix);
    const uint32_t nw = ix.code_stride / 4;
    auto launch = [&](void (*kernel)(ScanParams), int) {
        ensure_max_dynamic_smem(kernel, 220 * 1024);
        kernel<<<n, kThreads, smem, stream>>>(p);
    };
    if (half_lut) {
        if (nw <= 2) launch(k_scan_select<2, true>, 5);
        else if (nw <= 4) launch(k_scan_select<4, true>, 6);
        else if (nw <= 6) launch(k_scan_select<6, true>, 7);
        else if (nw <= 8) launch(k_scan_select<8, true>, 8);
        else launch(k_scan_select<16, true>, 9);
    } else {
        if (nw <= 2) launch(k_scan_select<2, false>, 0);
        else if (nw <= 4) launch(k_scan_select<4, false>, 1);
        else if (nw <= 6) launch(k_scan_select<6, false>, 2);
        else if (nw <= 8) launch(k_scan_select<8, false>, 3);
        else launch(k_scan_select<16, false>, 4);
    }
    return cudaGetLastError();
}

}  // namespace pgpu
