// k_rerank: rank_topN_points, Puck-Flat branch (puck/puck/puck_index.cpp:428-457):
// the exact FP32 squared L2 of every filter survivor against its original vector,
// then MaxHeap(topk) fed in the order the survivors are given, then reorder().
//
// One block per query. Each warp computes one candidate at a time with coalesced
// row loads; the sum follows the AVX build of L2Sqr16Ext / L2SqrExt
// (puck/tinker/method/hnsw_distfunc_opt_impl_inline.h:41-122): per 16-dim chunk,
// lane i<8 holds d_i^2 + d_{i+8}^2, the 8 lanes are added left to right, chunks
// are added to the running total in order; a tail under 16 dims uses 4 lane
// accumulators, ((l0+l1)+l2)+l3, then a scalar loop. The early abandon of the
// reference only ever rejects candidates the heap would reject, so full sums give
// the same result.
//
// Selection: when no two of the topk+1 smallest distances are equal the heap's
// output is just the ascending order, found by a bitonic sort of
// (distance, position); otherwise thread 0 replays the heap exactly.
//
// k_rerank_screen (precision form): the same result from fewer bytes. Each
// candidate is first measured on a BF16 copy of its vector; with |x~ - x| <=
// 2^-8 |x| per row and both sums in FP32, |d~ - d| <= E (see screen_bound), so
// every candidate whose exact distance can reach the topk-th lies in
// W = { j : d~_j - E_j <= U }, U = the topk-th smallest d~_j + E_j. Only W is
// recomputed with the exact FP32 order above, sorted and tie-checked like
// k_rerank; a tie sends the block to the full exact heap replay.
#include <cuda_bf16.h>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

// Block shapes (compile-time; -D overrides for tuning sweeps). The exact FP32
// rerank runs 256 threads per query. The screen runs 128 with eight blocks per SM,
// so one block's select and sort overlap other blocks' row gathers.
#ifndef PGPU_RERANK_THREADS
#define PGPU_RERANK_THREADS 256
#endif
#ifndef PGPU_RERANK_SCREEN_THREADS
#define PGPU_RERANK_SCREEN_THREADS 128
#endif
#ifndef PGPU_RERANK_SCREEN_MIN_BLOCKS
#define PGPU_RERANK_SCREEN_MIN_BLOCKS 8
#endif
constexpr int kThreads = PGPU_RERANK_THREADS;
constexpr int kWarps = kThreads / 32;
constexpr int kScreenThreads = PGPU_RERANK_SCREEN_THREADS;
constexpr int kScreenWarps = kScreenThreads / 32;
constexpr int kRows = 8;  // candidate rows per warp in flight (rows8_l2_exact)

struct RerankParams {
    const float* q;
    const float* qnorm;
    const int32_t* status;
    const float* hdist;
    int sort_ties;  // scan mode: replay ties in the filter's (t, memory id) order
    const uint32_t* htag;
    const uint32_t* hcnt;
    const float* feat;
    const uint32_t* mem2local;
    float* out_dist;
    uint32_t* out_ids;
    int32_t* out_status;
    uint32_t d, T, Tp, topk;
    // second-level PQ (whether_pq)
    const float* pq_codebook;
    const float* pq_offsets;
    const uint8_t* pq_codes;
    uint32_t pq_nsq, pq_lsq, pq_code_stride;
    // a realtime index (RealtimeInsertPuckIndex) sums the PQ table subspace by
    // subspace in order (realtime_insert_puck_index.cpp:466-499), not in
    // lookup_dist_table's four partials
    int pq_sequential;
};

// Exact-order squared L2 of G rows against q (shared memory), computed by one
// warp with the G rows' loads in flight together; results on every lane.
template <int G>
__device__ __forceinline__ void warp_l2_exact(const float* const* rows, const float* q, uint32_t d,
                                              int lane, float* out) {
    const uint32_t d16 = d & ~15u;
    float t[G];
#pragma unroll
    for (int u = 0; u < G; ++u) t[u] = 0.0f;
    const int grp = lane & 16;
    for (uint32_t base = 0; base < d16; base += 32) {
        const uint32_t e = base + lane;
        float sq[G];
#pragma unroll
        for (int u = 0; u < G; ++u) {
            sq[u] = 0.0f;
            if (e < d16) {
                const float a = __fsub_rn(__ldg(rows[u] + e), q[e]);
                sq[u] = __fmul_rn(a, a);
            }
        }
#pragma unroll
        for (int u = 0; u < G; ++u) {
            // lanes 0-7 (chunk at base) and 16-23 (chunk at base+16): d_i^2 + d_{i+8}^2
            const float s = __fadd_rn(sq[u], __shfl_down_sync(0xffffffffu, sq[u], 8));
            float acc = __shfl_sync(0xffffffffu, s, grp);
#pragma unroll
            for (int i = 1; i < 8; ++i) acc = __fadd_rn(acc, __shfl_sync(0xffffffffu, s, grp + i));
            const float acc_b = __shfl_sync(0xffffffffu, acc, 16);
            float tu = __fadd_rn(t[u], acc);               // chunk at base (lane 0's acc)
            tu = __shfl_sync(0xffffffffu, tu, 0);
            if (base + 16 < d16) tu = __fadd_rn(tu, acc_b);  // chunk at base + 16
            t[u] = tu;
        }
    }
    if (d16 < d) {  // L2SqrExt on the last d - d16 < 16 dims, serially
        const uint32_t qty = d - d16;
#pragma unroll
        for (int u = 0; u < G; ++u) {
            const float* x = rows[u] + d16;
            const float* qq = q + d16;
            float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f, l3 = 0.0f;
            uint32_t i = 0;
            for (; i + 4 <= qty; i += 4) {
                const float a0 = __fsub_rn(__ldg(x + i), qq[i]);
                const float a1 = __fsub_rn(__ldg(x + i + 1), qq[i + 1]);
                const float a2 = __fsub_rn(__ldg(x + i + 2), qq[i + 2]);
                const float a3 = __fsub_rn(__ldg(x + i + 3), qq[i + 3]);
                l0 = __fadd_rn(l0, __fmul_rn(a0, a0));
                l1 = __fadd_rn(l1, __fmul_rn(a1, a1));
                l2 = __fadd_rn(l2, __fmul_rn(a2, a2));
                l3 = __fadd_rn(l3, __fmul_rn(a3, a3));
            }
            float sum = __fadd_rn(__fadd_rn(__fadd_rn(l0, l1), l2), l3);
            for (; i < qty; ++i) {
                const float a = __fsub_rn(__ldg(x + i), qq[i]);
                sum = __fadd_rn(sum, __fmul_rn(a, a));
            }
            t[u] = __fadd_rn(t[u], sum);
        }
    }
#pragma unroll
    for (int u = 0; u < G; ++u) out[u] = t[u];
}

// The same sums as warp_l2_exact for G = 8 rows, d % 4 == 0 and 16-byte aligned
// rows and q: each group of 8 lanes measures two rows with 16-byte loads (lane l
// holds the float4s l, l + 8, ...), so a warp load instruction covers four whole
// 128-byte row segments. In one 16-dim chunk the four lanes holding float4s
// 0..3 pair dims i and i + 8 by one exchange (lane u <-> u + 2), lane 0 sums
// s0..s3 left to right and lane 1 continues with s4..s7 after one more
// exchange, so each chunk sum keeps the L2Sqr16Ext order; the running total is
// kept on lane 1 of the group, chunk by chunk in order. Results on every lane.
__device__ __forceinline__ void warp_l2_exact_vec(const float* const* rows, const float* q,
                                                  uint32_t d, int lane, float* out) {
    constexpr int R = 2;  // rows per group of 8 lanes
    const int g = lane >> 3, l = lane & 7;
    const uint32_t d16 = d & ~15u;
    const uint32_t nf4 = d16 >> 2;
    const float4* q4 = reinterpret_cast<const float4*>(q);
    // this group's rows g and g + 4 (selects on constant indices keep them in registers)
    const float* mine[R];
#pragma unroll
    for (int r = 0; r < R; ++r)
        mine[r] = g == 0 ? rows[4 * r] : g == 1 ? rows[4 * r + 1] : g == 2 ? rows[4 * r + 2] : rows[4 * r + 3];
    float t[R];
#pragma unroll
    for (int r = 0; r < R; ++r) t[r] = 0.0f;
    for (uint32_t f0 = 0; f0 < nf4; f0 += 8) {
        const uint32_t f = f0 + l;
        const bool in = f < nf4;
        float4 x[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
            x[r] = in ? __ldg(reinterpret_cast<const float4*>(mine[r]) + f)
                      : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 qq = in ? q4[f] : make_float4(0.f, 0.f, 0.f, 0.f);
        const bool second = f0 + 4 < nf4;  // this step holds two chunks
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float a0 = __fsub_rn(x[r].x, qq.x), a1 = __fsub_rn(x[r].y, qq.y);
            const float a2 = __fsub_rn(x[r].z, qq.z), a3 = __fsub_rn(x[r].w, qq.w);
            const float q0 = __fmul_rn(a0, a0), q1 = __fmul_rn(a1, a1);
            const float q2 = __fmul_rn(a2, a2), q3 = __fmul_rn(a3, a3);
            // lanes u = 0, 1 of a chunk: d_i^2 + d_{i+8}^2 with the partner u + 2
            const float s0 = __fadd_rn(q0, __shfl_xor_sync(0xffffffffu, q0, 2));
            const float s1 = __fadd_rn(q1, __shfl_xor_sync(0xffffffffu, q1, 2));
            const float s2 = __fadd_rn(q2, __shfl_xor_sync(0xffffffffu, q2, 2));
            const float s3 = __fadd_rn(q3, __shfl_xor_sync(0xffffffffu, q3, 2));
            const float a = __fadd_rn(__fadd_rn(__fadd_rn(s0, s1), s2), s3);   // lane u = 0
            const float b = __shfl_xor_sync(0xffffffffu, a, 1);                 // to lane u = 1
            const float chunk = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(b, s0), s1), s2), s3);
            const float hi = __shfl_down_sync(0xffffffffu, chunk, 4);           // lane 5 -> 1
            float tr = __fadd_rn(t[r], chunk);
            if (second) tr = __fadd_rn(tr, hi);
            t[r] = tr;
        }
    }
    if (d16 < d && l == 1) {  // L2SqrExt on the last d - d16 (a multiple of 4) dims
        const uint32_t qty = d - d16;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float* xr = mine[r] + d16;
            const float* qr = q + d16;
            float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f, l3 = 0.0f;
            for (uint32_t i = 0; i + 4 <= qty; i += 4) {
                const float a0 = __fsub_rn(__ldg(xr + i), qr[i]);
                const float a1 = __fsub_rn(__ldg(xr + i + 1), qr[i + 1]);
                const float a2 = __fsub_rn(__ldg(xr + i + 2), qr[i + 2]);
                const float a3 = __fsub_rn(__ldg(xr + i + 3), qr[i + 3]);
                l0 = __fadd_rn(l0, __fmul_rn(a0, a0));
                l1 = __fadd_rn(l1, __fmul_rn(a1, a1));
                l2 = __fadd_rn(l2, __fmul_rn(a2, a2));
                l3 = __fadd_rn(l3, __fmul_rn(a3, a3));
            }
            t[r] = __fadd_rn(t[r], __fadd_rn(__fadd_rn(__fadd_rn(l0, l1), l2), l3));
        }
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) out[u] = __shfl_sync(0xffffffffu, t[u >> 2], 8 * (u & 3) + 1);
}

// Dispatch: the vector form when d % 4 == 0 and q is 16-byte aligned (rows then
// are: the vectors start 256-byte aligned with d * 4 bytes per row).
__device__ __forceinline__ void rows8_l2_exact(const float* const* rows, const float* q, uint32_t d,
                                               int lane, float* out) {
    if ((d & 3u) == 0 && (reinterpret_cast<uintptr_t>(q) & 15u) == 0)
        warp_l2_exact_vec(rows, q, d, lane, out);
    else
        warp_l2_exact<8>(rows, q, d, lane, out);
}

// PQ: the second-level PQ branch of rank_topN_points (puck_index.cpp:402-427): per
// candidate (filter distance - |q|^2) + pq offset, then + lookup_dist_table over
// the PQ table (get_dist_table, quantization.cpp:260-270), in the reference's
// float order; the same heap semantics as the Puck-Flat branch.
template <bool PQ>
__global__ __launch_bounds__(kThreads) void k_rerank(RerankParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* okey = reinterpret_cast<unsigned long long*>(smem);  // [Tp]
    float* qv = reinterpret_cast<float*>(okey + p.Tp);
    float* dist = qv + p.d;                                   // [T]
    float* sv = dist + p.T;                                   // [Tp]
    uint32_t* si = reinterpret_cast<uint32_t*>(sv + p.Tp);    // [Tp]
    uint32_t* opos = si + p.Tp;                               // [Tp]
    float* pq_lut = reinterpret_cast<float*>(opos + p.Tp);    // [pq_nsq * 256] (PQ)
    __shared__ uint32_t sel_hist[256];
    __shared__ uint32_t sel_state[2];
    __shared__ uint32_t sel_count;
    const uint32_t qi = blockIdx.x, topk = p.topk;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* od = p.out_dist + (uint64_t)qi * topk;
    uint32_t* oi = p.out_ids + (uint64_t)qi * topk;
    const int32_t stq = p.status[qi];
    if (p.out_status && tid == 0) p.out_status[qi] = stq;
    if (stq != 0) {
        for (uint32_t i = tid; i < topk; i += kThreads) {
            od[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    const uint32_t cnt = p.hcnt[qi];
    const uint32_t* tags = p.htag + (uint64_t)qi * p.T;
    for (uint32_t i = tid; i < p.d; i += kThreads) qv[i] = p.q[(uint64_t)qi * p.d + i];
    {
        // the candidates' memory ids in shared memory (one coalesced load)
        uint32_t* stag = reinterpret_cast<uint32_t*>(pq_lut + (p.pq_lsq > 1 ? p.pq_nsq * 256 : 0));
        for (uint32_t i = tid; i < cnt; i += kThreads) stag[i] = tags[i];
        tags = stag;
    }
    __syncthreads();
    if (PQ) {
        const float qn = p.qnorm[qi];
        const float* hd = p.hdist + (uint64_t)qi * p.T;
        if (p.pq_lsq == 1) {
            // one-dimensional subspaces: each table entry (q_m - c)^2 is formed when
            // it is looked up (one subtraction, one product: the same bits as the
            // table), summed in lookup_dist_table's lane order
            for (uint32_t j = tid; j < cnt; j += kThreads) {
                const uint32_t mi = tags[j];
                const uint32_t* w = reinterpret_cast<const uint32_t*>(
                    p.pq_codes + (uint64_t)mi * p.pq_code_stride);
                float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                float t = __fadd_rn(__fsub_rn(hd[j], qn), p.pq_offsets[mi]);
                for (uint32_t m0 = 0; m0 < p.pq_nsq; m0 += 4) {
                    const uint32_t c4 = __ldg(w + (m0 >> 2));
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t m = m0 + k;
                        if (m < p.pq_nsq) {
                            const float y = __ldg(p.pq_codebook + (uint64_t)m * 256 + ((c4 >> (8 * k)) & 255u));
                            const float df = __fsub_rn(qv[m], y);
                            if (p.pq_sequential) t = __fadd_rn(t, __fmul_rn(df, df));
                            else a[k] = __fadd_rn(a[k], __fmul_rn(df, df));
                        }
                    }
                }
                if (!p.pq_sequential)
                    t = __fadd_rn(t, __fadd_rn(__fadd_rn(a[0], a[1]), __fadd_rn(a[2], a[3])));
                dist[j] = t;
            }
        } else {
            for (uint32_t e = tid; e < p.pq_nsq * 256; e += kThreads)
                pq_lut[e] = l2sqr_sse(qv + (e >> 8) * p.pq_lsq,
                                      p.pq_codebook + (uint64_t)e * p.pq_lsq, p.pq_lsq);
            __syncthreads();
            for (uint32_t j = tid; j < cnt; j += kThreads) {
                const uint32_t mi = tags[j];
                float t = __fsub_rn(hd[j], qn);
                t = __fadd_rn(t, p.pq_offsets[mi]);
                const uint8_t* code = p.pq_codes + (uint64_t)mi * p.pq_code_stride;
                if (p.pq_sequential) {
                    for (uint32_t m = 0; m < p.pq_nsq; ++m)
                        t = __fadd_rn(t, pq_lut[m * 256 + code[m]]);
                } else {
                    t = __fadd_rn(t, lut_sum(code, pq_lut, p.pq_nsq));
                }
                dist[j] = t;
            }
        }
    }
    // kRows rows per warp with their loads in flight together
    for (uint32_t j0 = warp * kRows; !PQ && j0 < cnt; j0 += kWarps * kRows) {
        const float* rows[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const uint32_t j = j0 + u;
            rows[u] = p.feat + (uint64_t)tags[j < cnt ? j : j0] * p.d;
        }
        float v[kRows];
        rows8_l2_exact(rows, qv, p.d, lane, v);
        if (lane == 0) {
#pragma unroll
            for (int u = 0; u < kRows; ++u)
                if (j0 + u < cnt) dist[j0 + u] = v[u];
        }
    }
    __syncthreads();
    // (distance, position) pairs, ascending. Only the topk+1 smallest matter (result
    // and tie check): with more candidates, keep every one at or below the
    // (topk+1)-th smallest distance (ties included) and sort just those.
    uint32_t m2 = p.Tp;
    if (cnt > topk + 1) {
        const float U = key_to_float(block_kth_key<kThreads>(dist, cnt, topk + 1, sel_hist, sel_state));
        if (tid == 0) sel_count = 0;
        __syncthreads();
        for (uint32_t i = tid; i < cnt; i += kThreads)
            if (dist[i] <= U) {
                const uint32_t pos = atomicAdd(&sel_count, 1u);
                sv[pos] = dist[i];
                si[pos] = i;
            }
        __syncthreads();
        const uint32_t m = sel_count;
        m2 = 2;
        while (m2 < m) m2 <<= 1;
        for (uint32_t i = m + tid; i < m2; i += kThreads) {
            sv[i] = __int_as_float(0x7f800000);
            si[i] = 0xFFFFFFFFu;
        }
    } else {
        for (uint32_t i = tid; i < p.Tp; i += kThreads) {
            sv[i] = i < cnt ? dist[i] : __int_as_float(0x7f800000);
            si[i] = i < cnt ? i : 0xFFFFFFFFu;
        }
    }
    __syncthreads();
    for (uint32_t size = 2; size <= m2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = tid; t < m2 / 2; t += kThreads) {
                const uint32_t lo = 2 * t - (t & (stride - 1));
                const uint32_t hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const float a = sv[lo], b = sv[hi];
                const uint32_t ia = si[lo], ib = si[hi];
                const bool gt = (a > b) || (a == b && ia > ib);
                if (gt == asc) {
                    sv[lo] = b;
                    sv[hi] = a;
                    si[lo] = ib;
                    si[hi] = ia;
                }
            }
            __syncthreads();
        }
    }
    const uint32_t keep = cnt < topk ? cnt : topk;
    // ties that the heap could resolve differently: among the topk+1 smallest, or
    // anywhere among the results when there are no more candidates than topk
    const uint32_t check = cnt <= topk ? (cnt > 0 ? cnt - 1 : 0) : topk;
    int tie = 0;
    for (uint32_t i = tid; i < check; i += kThreads)
        if (sv[i] == sv[i + 1]) tie = 1;
    tie = __syncthreads_or(tie);
    if (!tie) {
        for (uint32_t i = tid; i < topk; i += kThreads) {
            od[i] = i < keep ? sv[i] : sentinel_f();
            oi[i] = i < keep ? p.mem2local[tags[si[i]]] : kNoLabel;
        }
        return;
    }
    __syncthreads();
    if (p.sort_ties)
        order_by_filter_key<kThreads>(p.hdist + (uint64_t)qi * p.T, tags, cnt, p.Tp, okey, opos);
    if (tid == 0) {
        // exact MaxHeap(topk) replay in candidate order, then reorder()
        float* hv = sv - 1;
        uint32_t* ht = si - 1;
        for (uint32_t i = 1; i <= topk; ++i) hv[i] = sentinel_f();
        uint32_t dpc = topk;
        for (uint32_t r = 0; r < cnt; ++r) {
            const uint32_t j = p.sort_ties ? opos[r] : r;
            const float v = dist[j];
            if (v < hv[1]) heap_update(hv, ht, topk, dpc, v, p.mem2local[tags[j]]);
        }
        heap_reorder(hv, ht, topk);
        const uint32_t rn = topk - dpc;
        for (uint32_t i = 0; i < topk; ++i) {
            od[i] = hv[i + 1];
            oi[i] = i < rn ? ht[i + 1] : kNoLabel;
        }
    }
}

// Bound on |d~ - d| for a row with |x| <= xabs and screened distance d~ (d dims).
__device__ __forceinline__ float screen_bound(float dt, float xabs, uint32_t d) {
    const float ta = sqrtf(fmaxf(dt, 0.0f)) * 1.0009765625f + 1e-20f;
    const float dx = 0.00390625f * xabs * 1.0009765625f;
    const float tb = ta + dx;
    return dx * (2.0f * ta + dx) + (float)(3 * d + 8) * 1.1920928955078125e-07f * tb * tb + 1e-30f;
}

struct ScreenParams {
    const float* q;
    const int32_t* status;
    const float* hdist;
    const uint32_t* htag;
    const uint32_t* hcnt;
    const float* feat;
    const uint16_t* feat_bf16;
    const float* feat_abs;
    const uint32_t* mem2local;
    float* out_dist;
    uint32_t* out_ids;
    int32_t* out_status;
    uint32_t d, T, Tp, topk;
};

__global__ __launch_bounds__(kScreenThreads, PGPU_RERANK_SCREEN_MIN_BLOCKS) void k_rerank_screen(ScreenParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(smem);  // [Tp]
    float* qv = reinterpret_cast<float*>(keys + p.Tp);                       // [d]
    float* approx = qv + p.d;                                                // [T]
    float* hi = approx + p.T;                                                // [T] d~ + E, then exact
    float* bnd = hi + p.T;                                                   // [T]
    float* hv = bnd + p.T;                                                   // [topk + 1]
    uint32_t* ht = reinterpret_cast<uint32_t*>(hv + p.topk + 1);             // [topk + 1]
    uint32_t* opos = ht + p.topk + 1;                                        // [Tp]
    __shared__ uint32_t hist[256];
    __shared__ uint32_t state[2];
    __shared__ uint32_t wcount;
    const uint32_t qi = blockIdx.x, topk = p.topk, d = p.d;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* od = p.out_dist + (uint64_t)qi * topk;
    uint32_t* oi = p.out_ids + (uint64_t)qi * topk;
    const int32_t stq = p.status[qi];
    if (p.out_status && tid == 0) p.out_status[qi] = stq;
    if (stq != 0) {
        for (uint32_t i = tid; i < topk; i += kScreenThreads) {
            od[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    const uint32_t cnt = p.hcnt[qi];
    const uint32_t* tags = p.htag + (uint64_t)qi * p.T;
    for (uint32_t i = tid; i < d; i += kScreenThreads) qv[i] = p.q[(uint64_t)qi * d + i];
    // the candidates' memory ids in shared memory: one coalesced load, then every row
    // gather below starts from a shared-memory read
    uint32_t* stag = opos + p.Tp;  // [T]
    for (uint32_t i = tid; i < cnt; i += kScreenThreads) stag[i] = tags[i];
    tags = stag;
    if (tid == 0) wcount = 0;
    __syncthreads();
    bool full = cnt <= topk;
    if (!full) {
        if ((d & 7u) == 0 && d <= 128) {
            // screen, vector form: a half warp per row, 8 dimensions (one 16-byte
            // load) per lane, kRows rows per half warp in flight
            const int half = lane >> 4, hl = lane & 15;
            const bool active = (uint32_t)hl * 8 < d;
            float qr[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) qr[t] = active ? qv[hl * 8 + t] : 0.0f;
            // the loop runs the same iterations on both half warps (the shuffles below
            // take the full mask): a warp owns 2 * kRows rows per iteration
            for (uint32_t jw = warp * 2 * kRows; jw < cnt; jw += kScreenWarps * 2 * kRows) {
                const uint32_t j0 = jw + half * kRows;
                uint4 x[kRows];
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const uint32_t j = j0 + u < cnt ? j0 + u : jw;
                    x[u] = active ? __ldg(reinterpret_cast<const uint4*>(
                                        p.feat_bf16 + (uint64_t)tags[j] * d) + hl)
                                  : make_uint4(0, 0, 0, 0);
                }
                float acc[kRows];
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const uint32_t w[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
                    float a = 0.0f;
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const float lo = __uint_as_float(w[t] << 16);
                        const float hi2 = __uint_as_float(w[t] & 0xFFFF0000u);
                        const float d0 = qr[2 * t] - lo, d1 = qr[2 * t + 1] - hi2;
                        a += d0 * d0 + d1 * d1;
                    }
                    acc[u] = active ? a : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < kRows; ++u)
#pragma unroll
                    for (int o = 8; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
                if (hl < kRows) {
                    float mine = acc[0];
#pragma unroll
                    for (int u = 1; u < kRows; ++u)
                        if (hl == u) mine = acc[u];
                    const uint32_t j = j0 + hl;
                    if (j < cnt) {
                        const float e = screen_bound(mine, p.feat_abs[tags[j]], d);
                        approx[j] = mine;
                        bnd[j] = e;
                        hi[j] = mine + e;
                    }
                }
            }
        } else {
        // screen: kRows BF16 rows per warp in flight
        for (uint32_t j0 = warp * kRows; j0 < cnt; j0 += kScreenWarps * kRows) {
            float acc[kRows];
            const uint16_t* rows[kRows];
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const uint32_t j = j0 + u;
                rows[u] = p.feat_bf16 + (uint64_t)tags[j < cnt ? j : j0] * d;
                acc[u] = 0.0f;
            }
            for (uint32_t k = lane; k < d; k += 32) {
                const float qk = qv[k];
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const float x = __bfloat162float(__ushort_as_bfloat16(__ldg(rows[u] + k)));
                    const float df = qk - x;
                    acc[u] += df * df;
                }
            }
#pragma unroll
            for (int u = 0; u < kRows; ++u)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
            if (lane < kRows) {
                float mine = acc[0];
#pragma unroll
                for (int u = 1; u < kRows; ++u)
                    if (lane == u) mine = acc[u];
                const uint32_t j = j0 + lane;
                if (j < cnt) {
                    const float e = screen_bound(mine, p.feat_abs[tags[j]], d);
                    approx[j] = mine;
                    bnd[j] = e;
                    hi[j] = mine + e;
                }
            }
        }
        }
        __syncthreads();
        const float U = key_to_float(block_kth_key<kScreenThreads>(hi, cnt, topk, hist, state));
        for (uint32_t j = tid; j < cnt; j += kScreenThreads)
            if (approx[j] - bnd[j] <= U) keys[atomicAdd(&wcount, 1u)] = j;
        __syncthreads();
        const uint32_t m = wcount;
        // exact FP32 distances of the window, in the reference's order
        for (uint32_t i0 = warp * kRows; i0 < m; i0 += kScreenWarps * kRows) {
            const float* rows[kRows];
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
                const uint32_t i = i0 + u;
                rows[u] = p.feat + (uint64_t)tags[(uint32_t)keys[i < m ? i : i0]] * d;
            }
            float v[kRows];
            rows8_l2_exact(rows, qv, d, lane, v);
            __syncwarp();
            if (lane == 0) {
#pragma unroll
                for (int u = 0; u < kRows; ++u) {
                    const uint32_t i = i0 + u;
                    if (i < m) {
                        const uint32_t j = (uint32_t)keys[i];
                        keys[i] = ((unsigned long long)ordered_key(v[u]) << 32) | j;
                    }
                }
            }
        }
        __syncthreads();
        uint32_t mp = 2;
        while (mp < m) mp <<= 1;
        for (uint32_t i = m + tid; i < mp; i += kScreenThreads) keys[i] = ~0ull;
        __syncthreads();
        bitonic_sort_u64<kScreenThreads>(keys, mp);
        const uint32_t check = m - 1 < topk ? m - 1 : topk;
        int tie = 0;
        for (uint32_t i = tid; i < check; i += kScreenThreads)
            if ((uint32_t)(keys[i] >> 32) == (uint32_t)(keys[i + 1] >> 32)) tie = 1;
        tie = __syncthreads_or(tie);
        if (!tie) {
            for (uint32_t i = tid; i < topk; i += kScreenThreads) {
                od[i] = key_to_float((uint32_t)(keys[i] >> 32));
                oi[i] = p.mem2local[tags[(uint32_t)keys[i]]];
            }
            return;
        }
        full = true;
    }
    // every candidate exactly, then MaxHeap(topk) in candidate order and reorder()
    for (uint32_t j0 = warp * kRows; j0 < cnt; j0 += kScreenWarps * kRows) {
        const float* rows[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const uint32_t j = j0 + u;
            rows[u] = p.feat + (uint64_t)tags[j < cnt ? j : j0] * d;
        }
        float v[kRows];
        rows8_l2_exact(rows, qv, d, lane, v);
        if (lane == 0) {
#pragma unroll
            for (int u = 0; u < kRows; ++u)
                if (j0 + u < cnt) hi[j0 + u] = v[u];
        }
    }
    __syncthreads();
    // the heap is fed in the filter's (t, memory id) order
    order_by_filter_key<kScreenThreads>(p.hdist + (uint64_t)qi * p.T, tags, cnt, p.Tp, keys, opos);
    if (tid == 0) {
        float* h1 = hv;  // 1-based: slots 1..topk
        for (uint32_t i = 1; i <= topk; ++i) h1[i] = sentinel_f();
        uint32_t dpc = topk;
        for (uint32_t r = 0; r < cnt; ++r) {
            const uint32_t j = opos[r];
            const float v = hi[j];
            if (v < h1[1]) heap_update(h1, ht, topk, dpc, v, p.mem2local[tags[j]]);
        }
        heap_reorder(h1, ht, topk);
        const uint32_t rn = topk - dpc;
        for (uint32_t i = 0; i < topk; ++i) {
            od[i] = h1[i + 1];
            oi[i] = i < rn ? ht[i + 1] : kNoLabel;
        }
    }
}

uint32_t pow2_at_least(uint32_t v) {
    uint32_t p = 2;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace

size_t rerank_smem_bytes(const DeviceIndex& ix, uint32_t T, uint32_t topk) {
    const uint32_t Tp = pow2_at_least(T > topk ? T : topk);
    // the PQ table is only held for subspaces of more than one dimension
    const size_t pq_table = ix.pq_lsq > 1 ? sizeof(float) * ix.pq_nsq * 256 : 0;
    return sizeof(float) * (ix.d + T) + (sizeof(float) + 2 * sizeof(uint32_t) + 8) * Tp + pq_table +
           sizeof(uint32_t) * T;
}

cudaError_t launch_rerank(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t n,
                          uint32_t topk, const Scratch& s, float* out_dist, uint32_t* out_ids,
                          int32_t* out_status, cudaStream_t stream) {
    RerankParams p;
    p.q = s.q;
    p.qnorm = s.qnorm;
    p.status = s.status;
    p.hdist = s.hdist;
    p.sort_ties = cfg.mode == PGPU_MODE_SCAN ? 1 : 0;
    p.pq_codebook = ix.pq_codebook;
    p.pq_offsets = ix.pq_offsets;
    p.pq_codes = ix.pq_codes;
    p.pq_nsq = ix.pq_nsq;
    p.pq_lsq = ix.pq_lsq;
    p.pq_code_stride = ix.pq_code_stride;
    p.pq_sequential = ix.ins_cap > 0 ? 1 : 0;
    p.htag = s.htag;
    p.hcnt = s.hcnt;
    p.feat = ix.feat;
    p.mem2local = ix.mem2local;
    p.out_dist = out_dist;
    p.out_ids = out_ids;
    p.out_status = out_status;
    p.d = ix.d;
    p.T = s.T;
    p.Tp = pow2_at_least(s.T > topk ? s.T : topk);
    p.topk = topk;
    const size_t smem = rerank_smem_bytes(ix, s.T, topk);
    if (ix.pq_nsq) {
        ensure_max_dynamic_smem(k_rerank<true>, 220 * 1024);
        k_rerank<true><<<n, kThreads, smem, stream>>>(p);
    } else {
        ensure_max_dynamic_smem(k_rerank<false>, 220 * 1024);
        k_rerank<false><<<n, kThreads, smem, stream>>>(p);
    }
    return cudaGetLastError();
}

size_t rerank_screen_smem_bytes(const DeviceIndex& ix, uint32_t T, uint32_t topk) {
    const uint32_t Tp = pow2_at_least(T);
    return sizeof(unsigned long long) * Tp + sizeof(float) * (ix.d + 3ull * T) +
           (sizeof(float) + sizeof(uint32_t)) * (topk + 1ull) + sizeof(uint32_t) * (Tp + T);
}

cudaError_t launch_rerank_screen(const DeviceIndex& ix, uint32_t n, uint32_t topk, const Scratch& s,
                                 float* out_dist, uint32_t* out_ids, int32_t* out_status,
                                 cudaStream_t stream) {
    if (ix.feat_bf16 == nullptr || ix.feat_abs == nullptr) return cudaErrorInvalidValue;
    ScreenParams p;
    p.q = s.q;
    p.status = s.status;
    p.hdist = s.hdist;
    p.htag = s.htag;
    p.hcnt = s.hcnt;
    p.feat = ix.feat;
    p.feat_bf16 = ix.feat_bf16;
    p.feat_abs = ix.feat_abs;
    p.mem2local = ix.mem2local;
    p.out_dist = out_dist;
    p.out_ids = out_ids;
    p.out_status = out_status;
    p.d = ix.d;
    p.T = s.T;
    p.Tp = pow2_at_least(s.T);
    p.topk = topk;
    const size_t smem = rerank_screen_smem_bytes(ix, s.T, topk);
    ensure_max_dynamic_smem(k_rerank_screen, 220 * 1024);
    k_rerank_screen<<<n, kScreenThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace pgpu
