// Device helpers shared by the search kernels: Puck's MaxHeap, the reference's
// float operation orders (BLAS dot, SSE LUT build and lookup), block scans.
#pragma once
#include <cfloat>
#include <cstdint>

#include "pgpu_internal.h"

namespace pgpu {

__device__ __forceinline__ float sentinel_f() { return __uint_as_float(kHeapSentinelBits); }

// Sequential dot product, each product and partial sum rounded (BLAS order of
// the oracle build: s = 0; s += x[i]*y[i]).
__device__ __forceinline__ float dot_seq(const float* x, const float* y, uint32_t n) {
    float s = 0.0f;
    for (uint32_t i = 0; i < n; ++i) s = __fadd_rn(s, __fmul_rn(x[i], y[i]));
    return s;
}

// ------------------------------------------------------------------ MaxHeap
// Puck's bounded max-heap (puck/hierarchical_cluster/max_heap.cpp:28-102) on
// 1-based arrays: reject v >= top; the first `size` inserts sift down from the
// last unfilled slot; reorder() heap-sorts to ascending order. Single thread.
__device__ __forceinline__ void heap_insert(float* hv, uint32_t* ht, uint32_t heap_size,
                                            uint32_t father, float v, uint32_t t) {
    for (;;) {
        uint32_t left = father << 1;
        if (left > heap_size) break;
        uint32_t right = left + 1;
        float lv = hv[left];
        if (right > heap_size || lv > hv[right]) {
            if (lv < v) break;
            hv[father] = lv;
            ht[father] = ht[left];
            father = left;
        } else {
            float rv = hv[right];
            if (rv < v) break;
            hv[father] = rv;
            ht[father] = ht[right];
            father = right;
        }
    }
    hv[father] = v;
    ht[father] = t;
}

__device__ __forceinline__ bool heap_update(float* hv, uint32_t* ht, uint32_t size,
                                            uint32_t& dpc, float v, uint32_t t) {
    if (v >= hv[1]) return false;
    uint32_t father = 1;
    if (dpc > 0) father = dpc--;
    heap_insert(hv, ht, size, father, v, t);
    return true;
}

__device__ __forceinline__ void heap_reorder(float* hv, uint32_t* ht, uint32_t size) {
    for (uint32_t i = 0; i < size; ++i) {
        float vb = hv[1];
        uint32_t tb = ht[1];
        uint32_t hs = size - i;
        heap_insert(hv, ht, hs - 1, 1, hv[hs], ht[hs]);
        hv[hs] = vb;
        ht[hs] = tb;
    }
}

// ------------------------------------------------------------- block scans
// Inclusive scan over a block of NW warps; `warp_tot` needs NW slots.
template <int NW>
__device__ __forceinline__ uint32_t block_scan_incl(uint32_t v, uint32_t* warp_tot,
                                                   uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    uint32_t add = 0;
    for (int w = 0; w < warp; ++w) add += warp_tot[w];
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) t += warp_tot[w];
    *total = t;
    __syncthreads();
    return v + add;
}

// fvec_L2sqr, SSE order (puck/puck/distances_simd.cpp:120-133, 210-236).
__device__ __forceinline__ float l2sqr_sse(const float* x, const float* y, uint32_t d) {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    uint32_t i = 0;
    for (; i + 4 <= d; i += 4) {
        float t0 = __fsub_rn(x[i], y[i]), t1 = __fsub_rn(x[i + 1], y[i + 1]);
        float t2 = __fsub_rn(x[i + 2], y[i + 2]), t3 = __fsub_rn(x[i + 3], y[i + 3]);
        a0 = __fadd_rn(a0, __fmul_rn(t0, t0));
        a1 = __fadd_rn(a1, __fmul_rn(t1, t1));
        a2 = __fadd_rn(a2, __fmul_rn(t2, t2));
        a3 = __fadd_rn(a3, __fmul_rn(t3, t3));
    }
    if (i < d) {
        float t0 = __fsub_rn(x[i], y[i]);
        float t1 = (i + 1 < d) ? __fsub_rn(x[i + 1], y[i + 1]) : 0.0f;
        float t2 = (i + 2 < d) ? __fsub_rn(x[i + 2], y[i + 2]) : 0.0f;
        a0 = __fadd_rn(a0, __fmul_rn(t0, t0));
        a1 = __fadd_rn(a1, __fmul_rn(t1, t1));
        a2 = __fadd_rn(a2, __fmul_rn(t2, t2));
        a3 = __fadd_rn(a3, 0.0f);
    }
    return __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
}

// lookup_dist_table (puck_index.cpp:75-113): lane m%4 accumulates subspace m in
// increasing m, then (l0+l1)+(l2+l3). `code` is 4-byte aligned.
__device__ __forceinline__ float lut_sum(const uint8_t* __restrict__ code, const float* lut,
                                         uint32_t nsq) {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    const uint32_t* w = reinterpret_cast<const uint32_t*>(code);
    uint32_t m = 0;
    for (; m + 4 <= nsq; m += 4) {
        const uint32_t c = __ldg(w + (m >> 2));
        a0 = __fadd_rn(a0, lut[(m + 0) * 256 + (c & 0xff)]);
        a1 = __fadd_rn(a1, lut[(m + 1) * 256 + ((c >> 8) & 0xff)]);
        a2 = __fadd_rn(a2, lut[(m + 2) * 256 + ((c >> 16) & 0xff)]);
        a3 = __fadd_rn(a3, lut[(m + 3) * 256 + (c >> 24)]);
    }
    if (m < nsq) {
        const uint32_t c = __ldg(w + (m >> 2));
        a0 = __fadd_rn(a0, lut[m * 256 + (c & 0xff)]);
        if (m + 1 < nsq) a1 = __fadd_rn(a1, lut[(m + 1) * 256 + ((c >> 8) & 0xff)]);
        if (m + 2 < nsq) a2 = __fadd_rn(a2, lut[(m + 2) * 256 + ((c >> 16) & 0xff)]);
    }
    return __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
}

// get_dist_table (quantization.cpp:260-270) for one query into shared memory,
// by all threads of the block (nthreads). lsq = 4 takes one 16-byte codebook load
// per entry, four entries per thread in flight; other lsq use l2sqr_sse.
__device__ __forceinline__ void build_lut(float* lut, const float* qv, const float* __restrict__ cb,
                                          uint32_t nsq, uint32_t lsq, int nthreads) {
    const uint32_t total = nsq * 256;
    const int tid = threadIdx.x;
    if (lsq == 4) {
        const float4* cb4 = reinterpret_cast<const float4*>(cb);
        for (uint32_t e0 = 4 * tid; e0 < total; e0 += 4 * nthreads) {
            float4 y[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) y[u] = __ldg(cb4 + (e0 + u < total ? e0 + u : e0));
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t e = e0 + u;
                if (e >= total) break;
                const float* x = qv + (e >> 8) * 4;
                const float t0 = __fsub_rn(x[0], y[u].x), t1 = __fsub_rn(x[1], y[u].y);
                const float t2 = __fsub_rn(x[2], y[u].z), t3 = __fsub_rn(x[3], y[u].w);
                lut[e] = __fadd_rn(__fadd_rn(__fmul_rn(t0, t0), __fmul_rn(t1, t1)),
                                   __fadd_rn(__fmul_rn(t2, t2), __fmul_rn(t3, t3)));
            }
        }
    } else {
        for (uint32_t e = tid; e < total; e += nthreads) {
            const uint32_t m = e >> 8, j = e & 255;
            lut[e] = l2sqr_sse(qv + m * lsq, cb + ((uint64_t)m * 256 + j) * lsq, lsq);
        }
    }
}

// lookup_dist_table over codes already in registers: NW 32-bit words holding the
// record's nsq codes (4 per word, little-endian); same order as lut_sum.
template <int NW>
__device__ __forceinline__ float lut_sum_words(const uint32_t (&w)[NW], const float* lut,
                                               uint32_t nsq) {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        const uint32_t m = 4u * i;
        if (m >= nsq) break;
        const uint32_t c = w[i];
        a0 = __fadd_rn(a0, lut[(m + 0) * 256 + (c & 0xff)]);
        if (m + 1 < nsq) a1 = __fadd_rn(a1, lut[(m + 1) * 256 + ((c >> 8) & 0xff)]);
        if (m + 2 < nsq) a2 = __fadd_rn(a2, lut[(m + 2) * 256 + ((c >> 16) & 0xff)]);
        if (m + 3 < nsq) a3 = __fadd_rn(a3, lut[(m + 3) * 256 + (c >> 24)]);
    }
    return __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
}

// First half of compute_quantized_distance's per-point value
// (float)(2.0 * cell_dist + offset) (puck_index.cpp:360). The reference adds in
// double and rounds to float; for float operands double rounding of a sum is
// innocuous (53 >= 2*24 + 2), so one float add of the exact 2*cell_dist gives
// the same bits whenever 2*cell_dist is finite.
__device__ __forceinline__ float adc_base(float cell_dist, float offset) {
    return __fadd_rn(2.0f * cell_dist, offset);
}

__device__ __forceinline__ float pivot_of(float top, float qn, double rr) {
    // (top - query_norm) / radius_rate / 2.0 (puck_index.cpp:517, 544)
    return __double2float_rn((double)__fsub_rn(top, qn) / rr / 2.0);
}

// ------------------------------------------------------- radix selection
// Monotone 32-bit key of a float (total order of non-NaN values; -0 < +0).
__device__ __forceinline__ uint32_t ordered_key(float v) {
    const uint32_t b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_to_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// K-th smallest (1-based) ordered key of vals[0..L) by a 4-pass 8-bit radix
// select over NT threads; `hist` has 256 slots, `state` 2. Every thread returns it.
template <int NT>
__device__ uint32_t block_kth_key(const float* vals, uint32_t L, uint32_t K, uint32_t* hist,
                                  uint32_t* state) {
    uint32_t prefix = 0, mask = 0, kth = K;
    const int tid = threadIdx.x;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = tid; b < 256; b += NT) hist[b] = 0;
        __syncthreads();
        for (uint32_t j = tid; j < L; j += NT) {
            const uint32_t key = ordered_key(vals[j]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid < 32) {
            // lane l owns bins 8l .. 8l+7
            uint32_t cnt[8], tot = 0;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                cnt[t] = hist[tid * 8 + t];
                tot += cnt[t];
            }
            uint32_t incl = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += u;
            }
            const uint32_t excl = incl - tot;
            if (excl < kth && kth <= incl) {
                uint32_t run = excl;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    if (run < kth && kth <= run + cnt[t]) {
                        state[0] = prefix | ((uint32_t)(tid * 8 + t) << shift);
                        state[1] = kth - run;
                    }
                    run += cnt[t];
                }
            }
        }
        __syncthreads();
        prefix = state[0];
        kth = state[1];
        mask |= 255u << shift;
        __syncthreads();
    }
    return prefix;
}

// Ascending bitonic sort of n (a power of two) 64-bit keys by NT threads.
template <int NT>
__device__ void bitonic_sort_u64(unsigned long long* keys, uint32_t n) {
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = threadIdx.x; t < n / 2; t += NT) {
                const uint32_t lo = 2 * t - (t & (stride - 1));
                const uint32_t hi = lo + stride;
                const unsigned long long a = keys[lo], b = keys[hi];
                if ((a > b) == ((lo & size) == 0)) {
                    keys[lo] = b;
                    keys[hi] = a;
                }
            }
            __syncthreads();
        }
    }
}

// (t, memory id) of a filter candidate as one 64-bit key whose unsigned order is
// the lexicographic order of (t as a float, id); -0 is folded onto +0 so that
// equal floats compare equal.
__device__ __forceinline__ uint64_t filter_key(float t, uint32_t id) {
    uint32_t b = __float_as_uint(t == 0.0f ? 0.0f : t);
    b = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return ((uint64_t)b << 32) | id;
}

// Ascending bitonic sort of n (a power of two) keys with companion values.
template <int NT>
__device__ void bitonic_sort_pairs(unsigned long long* keys, uint32_t* vals, uint32_t n) {
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = threadIdx.x; t < n / 2; t += NT) {
                const uint32_t lo = 2 * t - (t & (stride - 1));
                const uint32_t hi = lo + stride;
                const unsigned long long a = keys[lo], b = keys[hi];
                if ((a > b) == ((lo & size) == 0)) {
                    keys[lo] = b;
                    keys[hi] = a;
                    const uint32_t va = vals[lo];
                    vals[lo] = vals[hi];
                    vals[hi] = va;
                }
            }
            __syncthreads();
        }
    }
}

// Positions 0..cnt of scan-mode candidates in the filter's (t, memory id) order
// (the order in which the reference's heap would have been fed); n2 >= cnt is a
// power of two. All NT threads call it.
template <int NT>
__device__ void order_by_filter_key(const float* t, const uint32_t* mem_id, uint32_t cnt,
                                    uint32_t n2, unsigned long long* keys, uint32_t* pos) {
    for (uint32_t i = threadIdx.x; i < n2; i += NT) {
        keys[i] = i < cnt ? filter_key(t[i], mem_id[i]) : ~0ull;
        pos[i] = i;
    }
    __syncthreads();
    bitonic_sort_pairs<NT>(keys, pos, n2);
}

}  // namespace pgpu
