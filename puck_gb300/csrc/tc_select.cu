// Exact selections on top of the BF16 tensor-core contraction.
//
// The tensor core gives s^_j ~ s_j for every centroid j, where s_j is the FP32
// value the reference computes (bias_j - q.c_j summed sequentially). With q and
// c_j rounded to BF16 (unit roundoff 2^-8) and any FP32 accumulation order,
//
//   |s^_j - s_j| <= E_j = eps * |q| |c_j| + 2^-20 (|bias_j| + |s^_j|),
//   eps = 2^-7 + 2^-15 + (d + 8) * 2^-21,
//
// (the 2^-7 term bounds the two BF16 roundings of each product, the d term the
// FP32 accumulation of both sides, the last term the final subtractions).
// Let U be the P-th smallest s^_j + E_j. Then every j with s_j <= s_(P) (the
// P-th smallest exact value) has s^_j - E_j <= s_j <= s_(P) <= U, so the window
// W = { j : s^_j - E_j <= U } holds the exact top P and every value tied with
// the P-th. Only W is recomputed in exact FP32 (the reference's operation
// order), sorted by (value, id) and checked for ties among the first P+1
// exactly as k_topsort does; with a tie, or with W beyond its buffer, or when
// the contraction reported a failure, the block recomputes every s_j and
// replays Puck's MaxHeap, so the result is always the reference's.
#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr int kWinThreads = 256;
constexpr uint32_t kWinCap = 1024;

__device__ __forceinline__ float window_eps(uint32_t d) {
    return 0.0078125f + 3.0517578125e-05f + (float)(d + 8) * 4.76837158203125e-07f;
}

// Exact top-P of bias_j - q.c_j per row (k_topsort's output and tie rule).
__global__ __launch_bounds__(kWinThreads) void k_window_topk(
    const float* __restrict__ approx, uint32_t ld, const float* __restrict__ Q, uint32_t d,
    const float* __restrict__ qnorm, const float* __restrict__ cents,
    const float* __restrict__ bias, const float* __restrict__ cabs, uint32_t C, uint32_t P,
    uint32_t ld_out, float* __restrict__ out_val, uint32_t* __restrict__ out_idx,
    const int32_t* __restrict__ status,
    const int* __restrict__ tc_err, unsigned long long* __restrict__ fallbacks,
    const int32_t* __restrict__ skip, const uint32_t* __restrict__ qidx,
    const uint32_t* __restrict__ nrows_dev) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* shi = reinterpret_cast<float*>(smem);                 // [C]   s^ + E, later exact s
    float* slo = shi + C;                                        // [C+1] s^ - E, later heap values
    uint32_t* stag = reinterpret_cast<uint32_t*>(slo + C + 1);   // [C+1] heap tags
    float* sq = reinterpret_cast<float*>(stag + C + 1);          // [d]
    unsigned long long* ckey = reinterpret_cast<unsigned long long*>(
        (reinterpret_cast<uintptr_t>(sq + d) + 7) & ~uintptr_t(7));  // [kWinCap]
    __shared__ uint32_t hist[256];
    __shared__ uint32_t state[2];
    __shared__ uint32_t ncand;
    // screen row rc; the query it belongs to (a compacted list when a probe answered
    // the others)
    const uint32_t rc = blockIdx.x;
    if (nrows_dev != nullptr && rc >= *nrows_dev) return;
    const uint32_t row = qidx ? qidx[rc] : rc;
    const int tid = threadIdx.x;
    if (skip != nullptr && skip[row]) return;  // the learned probe answered this query
    float* ov = out_val + (uint64_t)row * ld_out;
    uint32_t* oi = out_idx + (uint64_t)row * ld_out;
    // slots past P (a probe's wider cap): unused
    for (uint32_t i = P + tid; i < ld_out; i += kWinThreads) {
        ov[i] = sentinel_f();
        oi[i] = kNoLabel;
    }
    if (status != nullptr && status[row] != 0) {
        for (uint32_t i = tid; i < P; i += kWinThreads) {
            ov[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    const float* q = Q + (uint64_t)row * d;
    for (uint32_t k = tid; k < d; k += kWinThreads) sq[k] = q[k];
    if (tid == 0) ncand = 0;
    bool exact_all = (*tc_err != 0);
    if (!exact_all) {
        const float eps = window_eps(d);
        const float qa = sqrtf(qnorm[row]);
        const float* a = approx + (uint64_t)rc * ld;
        for (uint32_t j = tid; j < C; j += kWinThreads) {
            const float s = a[j];
            const float e = eps * qa * cabs[j] + 9.5367431640625e-07f * (fabsf(bias[j]) + fabsf(s)) +
                            1e-30f;
            shi[j] = s + e;
            slo[j] = s - e;
        }
        __syncthreads();
        const float U = key_to_float(block_kth_key<kWinThreads>(shi, C, P, hist, state));
        for (uint32_t j = tid; j < C; j += kWinThreads) {
            if (slo[j] <= U) {
                const uint32_t pos = atomicAdd(&ncand, 1u);
                if (pos < kWinCap) ckey[pos] = j;
            }
        }
        __syncthreads();
        const uint32_t m = ncand;
        if (m > kWinCap) {
            exact_all = true;
        } else {
            uint32_t mp = 1;
            while (mp < m) mp <<= 1;
            for (uint32_t t = tid; t < mp; t += kWinThreads) {
                if (t < m) {
                    const uint32_t j = (uint32_t)ckey[t];
                    const float v =
                        __fsub_rn(bias[j], dot_seq(sq, cents + (uint64_t)j * d, d));
                    ckey[t] = ((unsigned long long)ordered_key(v) << 32) | j;
                } else {
                    ckey[t] = ~0ull;
                }
            }
            __syncthreads();
            bitonic_sort_u64<kWinThreads>(ckey, mp);
            int tie = 0;
            const uint32_t last = P < m ? P : m - 1;
            for (uint32_t i = tid; i < last; i += kWinThreads)
                if ((uint32_t)(ckey[i] >> 32) == (uint32_t)(ckey[i + 1] >> 32)) tie = 1;
            tie = __syncthreads_or(tie);
            if (!tie) {
                for (uint32_t i = tid; i < P; i += kWinThreads) {
                    ov[i] = key_to_float((uint32_t)(ckey[i] >> 32));
                    oi[i] = (uint32_t)ckey[i];
                }
                return;
            }
            exact_all = true;
        }
    }
    // Reference path: every exact value, then MaxHeap(P) fed in index order.
    __syncthreads();
    for (uint32_t j = tid; j < C; j += kWinThreads)
        shi[j] = __fsub_rn(bias[j], dot_seq(sq, cents + (uint64_t)j * d, d));
    __syncthreads();
    if (tid == 0) {
        atomicAdd(fallbacks, 1ull);
        for (uint32_t i = 1; i <= P; ++i) slo[i] = sentinel_f();
        uint32_t dpc = P;
        for (uint32_t j = 0; j < C; ++j) heap_update(slo, stag, P, dpc, shi[j], j);
        heap_reorder(slo, stag, P);
    }
    __syncthreads();
    for (uint32_t i = tid; i < P; i += kWinThreads) {
        ov[i] = slo[i + 1];
        oi[i] = stag[i + 1];
    }
}

// The same selection for small P (P <= kSmallP), one warp per query row: the P-th
// smallest s^ + E by P rounds of warp minima over (value, id), the window's exact
// values recomputed one per lane, a warp bitonic sort of at most 64 candidates,
// and the tie check. With a tie or a wider window the warp feeds every exact
// value, 32 at a time in index order, to lane 0's MaxHeap(P).
constexpr uint32_t kSmallP = 16;
constexpr uint32_t kSmallCap = 64;
// PMAX: compile-time bound on P (1, 4 or 16) for the per-lane sorted lists.
template <uint32_t PMAX>
__global__ __launch_bounds__(256) void k_window_small(
    const float* __restrict__ approx, uint32_t ld, const float* __restrict__ Q, uint32_t d,
    const float* __restrict__ qnorm, const float* __restrict__ cents,
    const float* __restrict__ bias, const float* __restrict__ cabs, uint32_t C, uint32_t P,
    uint32_t ld_out, uint32_t nrows, float* __restrict__ out_val, uint32_t* __restrict__ out_idx,
    const int32_t* __restrict__ status, const int* __restrict__ tc_err,
    unsigned long long* __restrict__ fallbacks, const int32_t* __restrict__ skip,
    const uint32_t* __restrict__ qidx, const uint32_t* __restrict__ nrows_dev) {
    __shared__ unsigned long long wkey[8][kSmallCap];
    __shared__ float hv_s[8][kSmallP + 1];
    __shared__ uint32_t ht_s[8][kSmallP + 1];
    __shared__ float chunk[8][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rc = blockIdx.x * 8 + warp;  // screen row; its query below
    if (rc >= nrows || (nrows_dev != nullptr && rc >= *nrows_dev)) return;
    const uint32_t row = qidx ? qidx[rc] : rc;
    if (skip != nullptr && skip[row]) return;  // the learned probe answered this query
    float* ov = out_val + (uint64_t)row * ld_out;
    uint32_t* oi = out_idx + (uint64_t)row * ld_out;
    for (uint32_t i = P + lane; i < ld_out; i += 32) {
        ov[i] = sentinel_f();
        oi[i] = kNoLabel;
    }
    if (status != nullptr && status[row] != 0) {
        for (uint32_t i = lane; i < P; i += 32) {
            ov[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    const float* q = Q + (uint64_t)row * d;
    const float* a = approx + (uint64_t)rc * ld;
    unsigned long long* keys = wkey[warp];
    bool exact_all = (*tc_err != 0);
    if (!exact_all) {
        const float eps = window_eps(d);
        const float qa = sqrtf(qnorm[row]);
        // P-th smallest (hi, id): each lane keeps its P smallest in ascending order
        // (one pass), then P rounds of warp minima over the lanes' heads
        float tv[PMAX];
        uint32_t ti[PMAX];
#pragma unroll
        for (uint32_t r = 0; r < PMAX; ++r) {
            tv[r] = FLT_MAX;
            ti[r] = 0xFFFFFFFFu;
        }
        float worst = FLT_MAX;  // tv[P - 1]
        for (uint32_t j = lane; j < C; j += 32) {
            const float sv = a[j];
            const float hi = sv + (eps * qa * cabs[j] +
                                   9.5367431640625e-07f * (fabsf(bias[j]) + fabsf(sv)) + 1e-30f);
            if (hi < worst) {  // ids ascend within a lane: equal values keep the earlier
                float v = hi;
                uint32_t id = j;
#pragma unroll
                for (uint32_t r = 0; r < PMAX; ++r) {
                    if (r < P && v < tv[r]) {
                        const float t1 = tv[r];
                        const uint32_t t2 = ti[r];
                        tv[r] = v;
                        ti[r] = id;
                        v = t1;
                        id = t2;
                    }
                    if (r + 1 == P) worst = tv[r];
                }
            }
        }
        uint32_t head = 0;
        float lv = FLT_MAX;
        for (uint32_t r = 0; r < P; ++r) {
            float hv = FLT_MAX;
            uint32_t hid = 0xFFFFFFFFu;
#pragma unroll
            for (uint32_t t = 0; t < PMAX; ++t)
                if (t == head) {
                    hv = tv[t];
                    hid = ti[t];
                }
            float bv = hv;
            uint32_t bi = hid;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ov2 = __shfl_xor_sync(0xffffffffu, bv, o);
                const uint32_t oi2 = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov2 < bv || (ov2 == bv && oi2 < bi)) {
                    bv = ov2;
                    bi = oi2;
                }
            }
            if (hid == bi && hv == bv && bi != 0xFFFFFFFFu) ++head;
            lv = bv;
        }
        const float U = lv;
        // window: lo <= U, exact value per candidate
        uint32_t m = 0;
        for (uint32_t j0 = 0; j0 < C; j0 += 32) {
            const uint32_t j = j0 + lane;
            bool in = false;
            if (j < C) {
                const float sv = a[j];
                const float e = eps * qa * cabs[j] + 9.5367431640625e-07f * (fabsf(bias[j]) + fabsf(sv)) +
                                1e-30f;
                in = (sv - e) <= U;
            }
            const unsigned b = __ballot_sync(0xffffffffu, in);
            if (m + __popc(b) > kSmallCap) {
                m = kSmallCap + 1;
                break;
            }
            if (in) keys[m + __popc(b & ((1u << lane) - 1))] = j;
            m += __popc(b);
        }
        __syncwarp();
        if (m <= kSmallCap) {
            // the members' exact values, one member per lane: every dot's loads in flight
            // together instead of one chunk of the screen at a time
            for (uint32_t i = lane; i < m; i += 32) {
                const uint32_t j = (uint32_t)keys[i];
                const float v = __fsub_rn(bias[j], dot_seq(q, cents + (uint64_t)j * d, d));
                keys[i] = ((unsigned long long)ordered_key(v) << 32) | j;
            }
            __syncwarp();
        }
        if (m > kSmallCap) {
            exact_all = true;
        } else {
            for (uint32_t i = m + lane; i < kSmallCap; i += 32) keys[i] = ~0ull;
            __syncwarp();
            // bitonic sort of 64 keys, two compare-exchanges per lane and step
            for (uint32_t size = 2; size <= kSmallCap; size <<= 1) {
                for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                    const uint32_t t = lane;
                    const uint32_t lo = 2 * t - (t & (stride - 1));
                    const uint32_t hi = lo + stride;
                    const unsigned long long x = keys[lo], y = keys[hi];
                    if ((x > y) == ((lo & size) == 0)) {
                        keys[lo] = y;
                        keys[hi] = x;
                    }
                    __syncwarp();
                }
            }
            bool tie = false;
            const uint32_t last = P < m ? P : m - 1;
            for (uint32_t i = lane; i < last; i += 32)
                tie |= (uint32_t)(keys[i] >> 32) == (uint32_t)(keys[i + 1] >> 32);
            if (!__any_sync(0xffffffffu, tie)) {
                for (uint32_t i = lane; i < P; i += 32) {
                    ov[i] = key_to_float((uint32_t)(keys[i] >> 32));
                    oi[i] = (uint32_t)keys[i];
                }
                return;
            }
            exact_all = true;
        }
    }
    // Reference path: every exact value, in index order, into MaxHeap(P).
    float* hv = hv_s[warp];
    uint32_t* ht = ht_s[warp];
    uint32_t dpc = P;
    if (lane == 0) {
        atomicAdd(fallbacks, 1ull);
        for (uint32_t i = 1; i <= P; ++i) hv[i] = sentinel_f();
    }
    for (uint32_t j0 = 0; j0 < C; j0 += 32) {
        const uint32_t j = j0 + lane;
        if (j < C) chunk[warp][lane] = __fsub_rn(bias[j], dot_seq(q, cents + (uint64_t)j * d, d));
        __syncwarp();
        if (lane == 0) {
            const uint32_t cnt = C - j0 < 32 ? C - j0 : 32;
            for (uint32_t t = 0; t < cnt; ++t) heap_update(hv, ht, P, dpc, chunk[warp][t], j0 + t);
        }
        __syncwarp();
    }
    if (lane == 0) {
        heap_reorder(hv, ht, P);
        for (uint32_t i = 0; i < P; ++i) {
            ov[i] = hv[i + 1];
            oi[i] = ht[i + 1];
        }
    }
}

// nearest_center (kmeans.cpp:221-258) from a tensor-core screen: one warp per
// point. s^_j ~ 0.5|c_j|^2 - x.c_j orders the centroids like the reference's
// cur_j = (|x|^2 + |c_j|^2) - 2 x.c_j; the window around the screened minimum
// is recomputed exactly and the smallest cur_j with the lowest id wins, as in
// the reference's strict-< scan.
__global__ __launch_bounds__(256) void k_window_argmin(
    const float* __restrict__ approx, uint32_t ld, const float* __restrict__ X, uint64_t row0,
    uint32_t rows, uint32_t d, const float* __restrict__ cents, const float* __restrict__ cnorm,
    uint32_t K, const int* __restrict__ tc_err, int32_t* __restrict__ assign,
    float* __restrict__ dis) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= rows) return;
    const uint64_t p = row0 + w;
    const float* x = X + p * d;
    float xn = 0.0f;
    if (lane == 0) xn = dot_seq(x, x, d);
    xn = __shfl_sync(0xffffffffu, xn, 0);
    const bool screen = (*tc_err == 0);
    float U = FLT_MAX;
    const float* a = approx + (uint64_t)w * ld;
    const float eps = window_eps(d);
    const float xa = sqrtf(xn);
    if (screen) {
        for (uint32_t j = lane; j < K; j += 32) {
            const float s = a[j];
            const float cn = cnorm[j];
            const float e = eps * xa * sqrtf(cn) + 4.76837158203125e-07f * (xn + cn) +
                            9.5367431640625e-07f * fabsf(s) + 1e-30f;
            U = fminf(U, s + e);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) U = fminf(U, __shfl_xor_sync(0xffffffffu, U, o));
    }
    // the reference's scan: min starts at FLT_MAX, strict < in ascending id order
    float best = FLT_MAX;
    uint32_t bidx = 0xFFFFFFFFu;
    for (uint32_t j = lane; j < K; j += 32) {
        if (screen) {
            const float s = a[j];
            const float cn = cnorm[j];
            const float e = eps * xa * sqrtf(cn) + 4.76837158203125e-07f * (xn + cn) +
                            9.5367431640625e-07f * fabsf(s) + 1e-30f;
            if (s - e > U) continue;
        }
        const float cur =
            __fsub_rn(__fadd_rn(xn, cnorm[j]), 2.0f * dot_seq(x, cents + (uint64_t)j * d, d));
        if (cur < best) {  // j ascends within a lane
            best = cur;
            bidx = j;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, best, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ov < best || (ov == best && oi < bidx)) {
            best = ov;
            bidx = oi;
        }
    }
    if (lane == 0) {
        if (bidx == 0xFFFFFFFFu) {  // nothing below FLT_MAX: the reference keeps id 0
            best = FLT_MAX;
            bidx = 0;
        }
        assign[p] = (int32_t)bidx;
        dis[p] = best;
    }
}

__global__ void k_sqrt_norms(const float* __restrict__ half_norms, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sqrtf(2.0f * half_norms[i]) * 1.0000005f;
}

__global__ void k_halve(const float* __restrict__ x, uint64_t n, float* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = 0.5f * x[i];
}

__global__ void k_norms_seq(const float* __restrict__ X, uint64_t rows, uint32_t d,
                            float* __restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) out[r] = dot_seq(X + r * d, X + r * d, d);
}

}  // namespace

size_t window_smem_bytes(uint32_t C, uint32_t d) {
    return (size_t)C * 4 + (size_t)(C + 1) * 8 + (size_t)d * 4 + 16 + (size_t)kWinCap * 8;
}

cudaError_t launch_abs_from_half_norms(const float* half_norms, uint32_t n, float* out,
                                       cudaStream_t stream) {
    k_sqrt_norms<<<(n + 255) / 256, 256, 0, stream>>>(half_norms, n, out);
    return cudaGetLastError();
}

cudaError_t launch_coarse_tc(const DeviceIndex& ix, uint32_t n, Scratch& s, cudaStream_t stream) {
    // with a probe, only the queries it left (s.ulist, their count s.ucount on the device)
    TcOperand A{nullptr, ix.d, 1, n, s.qb, s.ulist, s.ucount};
    TcOperand B{nullptr, ix.d, 1, ix.C, ix.coarse_bf16};
    TcEpilogue ep{};
    ep.mode = TC_EPI_SCORE;
    ep.out = s.dots;
    ep.ld = ix.C;
    ep.bias = ix.coarse_norms;
    return launch_tc_gemm(A, B, ix.d, ep, s.tc_err, stream);
}

cudaError_t launch_coarse_window(const DeviceIndex& ix, uint32_t n, Scratch& s,
                                 cudaStream_t stream) {
    if (s.Pfix <= kSmallP) {
        auto kern = s.Pfix == 1 ? k_window_small<1> : s.Pfix <= 4 ? k_window_small<4>
                                                                   : k_window_small<16>;
        kern<<<(n + 7) / 8, 256, 0, stream>>>(
            s.dots, ix.C, s.q, ix.d, s.qnorm, ix.coarse, ix.coarse_norms, ix.coarse_abs, ix.C,
            s.Pfix, s.P, n, s.cdist, s.ctag, s.status, s.tc_err, s.counters + kCounterWindowFallbacks,
            s.pconf, s.ulist, s.ucount);
        return cudaGetLastError();
    }
    const size_t smem = window_smem_bytes(ix.C, ix.d);
    ensure_max_dynamic_smem(k_window_topk, 200 * 1024);
    k_window_topk<<<n, kWinThreads, smem, stream>>>(s.dots, ix.C, s.q, ix.d, s.qnorm, ix.coarse,
                                                    ix.coarse_norms, ix.coarse_abs, ix.C, s.Pfix,
                                                    s.P, s.cdist, s.ctag, s.status, s.tc_err,
                                                    s.counters + kCounterWindowFallbacks, s.pconf,
                                                    s.ulist, s.ucount);
    return cudaGetLastError();
}

cudaError_t launch_nearest_center_tc(uint32_t dim, const float* cents, uint64_t k, const float* x,
                                     uint64_t n, int32_t* assign, float* dis, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    // screen buffer of at most 256 MiB: rows per chunk, a multiple of 128
    uint64_t chunk = (256ull << 20) / (4 * (k ? k : 1));
    chunk = chunk < 128 ? 128 : (chunk / 128) * 128;
    // the contraction's grid.y (row tiles of 128) is at most 65535
    if (chunk > 65535ull * 128) chunk = 65535ull * 128;
    if (chunk > n) chunk = n;
    float* cnorm = nullptr;
    float* half = nullptr;
    float* screen = nullptr;
    int* err = nullptr;
    cudaError_t e = cudaMallocAsync(&cnorm, sizeof(float) * k, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&half, sizeof(float) * k, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&screen, sizeof(float) * chunk * k, stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&err, sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), stream);
    if (e == cudaSuccess) {
        k_norms_seq<<<(unsigned)((k + 255) / 256), 256, 0, stream>>>(cents, k, dim, cnorm);
        k_halve<<<(unsigned)((k + 255) / 256), 256, 0, stream>>>(cnorm, k, half);
        e = cudaGetLastError();
    }
    for (uint64_t r0 = 0; e == cudaSuccess && r0 < n; r0 += chunk) {
        const uint32_t rows = (uint32_t)(n - r0 < chunk ? n - r0 : chunk);
        TcOperand A{x + r0 * dim, dim, 1, rows};
        TcOperand B{cents, dim, 1, (uint32_t)k};
        TcEpilogue ep{};
        ep.mode = TC_EPI_SCORE;
        ep.out = screen;
        ep.ld = k;
        ep.bias = half;
        e = launch_tc_gemm(A, B, dim, ep, err, stream);
        if (e != cudaSuccess) break;
        k_window_argmin<<<(rows + 7) / 8, 256, 0, stream>>>(screen, (uint32_t)k, x, r0, rows, dim,
                                                           cents, cnorm, (uint32_t)k, err, assign,
                                                           dis);
        e = cudaGetLastError();
    }
    if (cnorm) cudaFreeAsync(cnorm, stream);
    if (half) cudaFreeAsync(half, stream);
    if (screen) cudaFreeAsync(screen, stream);
    if (err) cudaFreeAsync(err, stream);
    return e;
}

}  // namespace pgpu
