// Exact-mode search kernels for Puck-Flat indexes on sm_103a.
//
// Float semantics: every product and sum is rounded separately (__fmul_rn,
// __fadd_rn: no FMA contraction) and every reduction runs in the order the
// reference's code (built without FMA contraction, with a sequential BLAS)
// uses, so distances, heap contents and tie resolution are bit-identical to
// PuckIndex::search (puck/puck/puck_index.cpp:559-600).
//
// Pipeline per pass of B queries (one stream):
//   k_prep_queries     normalisation + |q|^2          hierarchical_cluster_index.cpp:1513-1536
//   k_centroid_scores  0.5|c|^2 - q.c  /  -q.f        hierarchical_cluster_index.cpp:700-727,
//                                                     puck_index.cpp:494-501
//   k_topsort          top-P coarse / full fine order max_heap.cpp (exact heap on ties)
//   k_walk_scan        cell walk + filter-PQ ADC      puck_index.cpp:346-390, 485-557
//   k_rerank           exact L2 of the survivors      puck_index.cpp:392-457
#include <cuda_bf16.h>

#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

// ---------------------------------------------------------------- kernels

// One warp per query (kPrepWarps per block): the row is read coalesced into shared
// memory; the two sums that fix the result bits (the norm, |q|^2) run sequentially in
// lane 0 in the reference's order, every other pass is spread over the lanes.
// q_in rows hold qdim floats: d, or d - 1 on an ip2cos index.
constexpr int kPrepWarps = 8;
__global__ __launch_bounds__(kPrepWarps * 32) void k_prep_queries(
    const float* __restrict__ q_in, float* __restrict__ q_out, uint16_t* __restrict__ q_bf16,
    float* __restrict__ qnorm, int32_t* __restrict__ status, uint32_t n, uint32_t d,
    uint32_t qdim, int whether_norm, int ip2cos) {
    extern __shared__ float prep_rows[];  // [kPrepWarps][d]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * kPrepWarps + warp;
    if (i >= n) return;  // whole warps only; no block barrier follows
    float* y = prep_rows + (uint64_t)warp * d;
    const float* x = q_in + (uint64_t)i * qdim;
    // Non-finite input has no defined result in the reference; it is rejected so
    // that no NaN reaches the sorts and the walk.
    int bad = 0;
    for (uint32_t k = lane; k < qdim; k += 32) {
        const float v = x[k];
        bad |= !isfinite(v);
        y[k] = v;
    }
    // ip2cos: the caller's d - 1 values and a 0, not normalised (hierarchical_cluster_index.cpp:
    // 1516-1520; the reference's memset there counts bytes and leaves the last float as it
    // was, the transform means it to be 0)
    for (uint32_t k = qdim + lane; k < d; k += 32) y[k] = 0.0f;
    int32_t st = __any_sync(0xffffffffu, bad) ? PGPU_E_INVALID : 0;
    __syncwarp();
    bool scale = false;
    float alpha = 1.0f;
    if (st == 0 && whether_norm && !ip2cos) {
        // cblas_snrm2 then cblas_sscal(1.0 / norm) (hierarchical_cluster_index.cpp:1524-1531)
        float s = 0.0f;
        if (lane == 0) s = dot_seq(y, y, d);
        const float norm = __fsqrt_rn(__shfl_sync(0xffffffffu, s, 0));
        if ((double)norm < 1e-6) {
            st = PGPU_E_ZERO_NORM;
        } else {
            alpha = __double2float_rn(1.0 / (double)norm);
            scale = true;
        }
    }
    float* yo = q_out + (uint64_t)i * d;
    uint16_t* yb = q_bf16 + (uint64_t)i * d;
    for (uint32_t k = lane; k < d; k += 32) {
        const float v = st != 0 ? 0.0f : (scale ? __fmul_rn(alpha, y[k]) : y[k]);
        y[k] = v;
        yo[k] = v;
        yb[k] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
    __syncwarp();
    if (lane == 0) {
        const float qn = dot_seq(y, y, d);
        qnorm[i] = qn;
        if (st == 0 && !isfinite(qn)) st = PGPU_E_INVALID;
        status[i] = st;
    }
}

// out[i][j] = bias[j] - a_i.b_j (MODE 0), -(a_i.b_j) (MODE 1), bias[j] + a_i.b_j (MODE 2).
// 128x128 output tile per block, 8x8 per thread (rows ty + 16i, columns tx + 16j);
// the k loop runs in order for every output, so each dot product is summed
// sequentially (a product, then an add, no contraction).
constexpr int kTile = 128, kTileK = 16;
template <int MODE>
__global__ __launch_bounds__(256) void k_centroid_scores(const float* __restrict__ A, uint32_t na,
                                                         const float* __restrict__ B, uint32_t nb,
                                                         uint32_t d, const float* __restrict__ bias,
                                                         float* __restrict__ out, uint32_t ld_out) {
    __shared__ float As[kTileK][kTile + 4];
    __shared__ float Bs[kTileK][kTile + 4];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const uint32_t a0 = blockIdx.y * kTile, b0 = blockIdx.x * kTile;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    for (uint32_t k0 = 0; k0 < d; k0 += kTileK) {
        // 16 consecutive threads read 16 consecutive k of one row
        for (int e = threadIdx.x; e < kTile * kTileK; e += 256) {
            const int r = e / kTileK, kk = e % kTileK;
            const uint32_t k = k0 + kk;
            As[kk][r] = (a0 + r < na && k < d) ? __ldg(A + (uint64_t)(a0 + r) * d + k) : 0.0f;
            Bs[kk][r] = (b0 + r < nb && k < d) ? __ldg(B + (uint64_t)(b0 + r) * d + k) : 0.0f;
        }
        __syncthreads();
        const uint32_t kmax = min((uint32_t)kTileK, d - k0);
        for (uint32_t kk = 0; kk < kmax; ++kk) {
            float av[8], bv[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 8; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = __fadd_rn(acc[i][j], __fmul_rn(av[i], bv[j]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t a = a0 + ty + 16 * i;
        if (a >= na) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t b = b0 + tx + 16 * j;
            if (b >= nb) continue;
            float v;
            if (MODE == 0) v = __fsub_rn(bias[b], acc[i][j]);
            else if (MODE == 1) v = -acc[i][j];
            else v = __fadd_rn(bias[b], acc[i][j]);
            out[(uint64_t)a * ld_out + b] = v;
        }
    }
}

__global__ void k_half_norms(const float* __restrict__ X, uint32_t rows, uint32_t d,
                             float* __restrict__ out) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float* x = X + (uint64_t)r * d;
    out[r] = dot_seq(x, x, d) / 2.0f;
}

// Empty cells get stationary = sqrt(FLT_MAX); min_dist_offset[c] = min over the
// coarse cluster's cells (puck_index.cpp:284-305).
__global__ void k_cell_constants(float* __restrict__ stationary, const uint32_t* __restrict__ cell_start,
                                 float* __restrict__ mdo, uint32_t C, uint32_t F, float empty_value) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    float m = FLT_MAX;
    for (uint32_t f = 0; f < F; ++f) {
        const uint64_t cell = (uint64_t)c * F + f;
        float s = stationary[cell];
        if (cell_start[cell] == cell_start[cell + 1]) {
            s = empty_value;
            stationary[cell] = s;
        }
        if (s < m) m = s;
    }
    mdo[c] = m;
}

// Per row: ascending order of L values by (value, index); the first K are
// written out. Equal to Puck's heap + reorder() whenever no two values among the
// first K+1 are equal; otherwise one thread replays the heap exactly.
__global__ void k_topsort(const float* __restrict__ vals, uint32_t L, uint32_t Lp, uint32_t ld,
                          uint32_t K, float* __restrict__ out_val, uint32_t* __restrict__ out_idx,
                          const int32_t* __restrict__ status) {
    extern __shared__ unsigned char smem[];
    float* sv = reinterpret_cast<float*>(smem);
    uint32_t* si = reinterpret_cast<uint32_t*>(sv + Lp);
    const uint32_t row = blockIdx.x;
    const float* v = vals + (uint64_t)row * ld;
    float* ov = out_val + (uint64_t)row * K;
    uint32_t* oi = out_idx + (uint64_t)row * K;
    if (status != nullptr && status[row] != 0) {
        for (uint32_t i = threadIdx.x; i < K; i += blockDim.x) {
            ov[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    for (uint32_t i = threadIdx.x; i < Lp; i += blockDim.x) {
        sv[i] = i < L ? v[i] : __int_as_float(0x7f800000);
        si[i] = i < L ? i : 0xFFFFFFFFu;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= Lp; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = threadIdx.x; t < Lp / 2; t += blockDim.x) {
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
    int tie = 0;
    const uint32_t last = K < L ? K : L - 1;
    for (uint32_t i = threadIdx.x; i < last; i += blockDim.x)
        if (sv[i] == sv[i + 1]) tie = 1;
    tie = __syncthreads_or(tie);
    if (!tie) {
        for (uint32_t i = threadIdx.x; i < K; i += blockDim.x) {
            ov[i] = sv[i];
            oi[i] = si[i];
        }
        return;
    }
    if (threadIdx.x == 0) {
        // Exact replay of MaxHeap(K) fed in index order, then reorder().
        float* hv = sv - 1;
        uint32_t* ht = si - 1;
        for (uint32_t i = 1; i <= K; ++i) hv[i] = sentinel_f();
        uint32_t dpc = K;
        for (uint32_t i = 0; i < L; ++i) heap_update(hv, ht, K, dpc, v[i], i);
        heap_reorder(hv, ht, K);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < K; i += blockDim.x) {
        ov[i] = sv[i];
        oi[i] = si[i];
    }
}

// Top-K of a row for small K (K + 1 <= 32): K + 1 passes, each taking the smallest
// (value, index) key above the previous one with a block-wide min. Same output
// and tie rule as k_topsort: when no two of the K+1 smallest values are equal the
// ascending order is what MaxHeap(K) + reorder() gives; otherwise thread 0
// replays the heap exactly.
constexpr int kSelThreads = 128;
__global__ __launch_bounds__(kSelThreads) void k_topsel_small(
    const float* __restrict__ vals, uint32_t L, uint32_t ld, uint32_t K, float* __restrict__ out_val,
    uint32_t* __restrict__ out_idx, const int32_t* __restrict__ status) {
    extern __shared__ float sval[];  // [L]
    __shared__ float red_v[kSelThreads / 32];
    __shared__ uint32_t red_i[kSelThreads / 32];
    __shared__ float sel_v[33];
    __shared__ uint32_t sel_i[33];
    __shared__ float heap_v[33];
    __shared__ uint32_t heap_t[33];
    const uint32_t row = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* ov = out_val + (uint64_t)row * K;
    uint32_t* oi = out_idx + (uint64_t)row * K;
    if (status != nullptr && status[row] != 0) {
        for (uint32_t i = tid; i < K; i += kSelThreads) {
            ov[i] = sentinel_f();
            oi[i] = kNoLabel;
        }
        return;
    }
    const float* v = vals + (uint64_t)row * ld;
    for (uint32_t i = tid; i < L; i += kSelThreads) sval[i] = v[i];
    __syncthreads();
    const uint32_t picks = K + 1 < L ? K + 1 : L;
    float lv = __int_as_float(0xff800000);  // -inf
    uint32_t li = 0;
    bool first = true;
    for (uint32_t r = 0; r < picks; ++r) {
        float bv = __int_as_float(0x7f800000);
        uint32_t bi = 0xFFFFFFFFu;
        for (uint32_t i = tid; i < L; i += kSelThreads) {
            const float x = sval[i];
            const bool above = first || x > lv || (x == lv && i > li);
            if (above && (x < bv || (x == bv && i < bi))) {
                bv = x;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov2 = __shfl_down_sync(0xffffffffu, bv, o);
            const uint32_t oi2 = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov2 < bv || (ov2 == bv && oi2 < bi)) {
                bv = ov2;
                bi = oi2;
            }
        }
        if (lane == 0) {
            red_v[warp] = bv;
            red_i[warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            float fv = red_v[0];
            uint32_t fi = red_i[0];
            for (int w = 1; w < kSelThreads / 32; ++w)
                if (red_v[w] < fv || (red_v[w] == fv && red_i[w] < fi)) {
                    fv = red_v[w];
                    fi = red_i[w];
                }
            sel_v[r] = fv;
            sel_i[r] = fi;
        }
        __syncthreads();
        lv = sel_v[r];
        li = sel_i[r];
        first = false;
    }
    bool tie = false;
    for (uint32_t r = 0; r + 1 < picks; ++r) tie |= (sel_v[r] == sel_v[r + 1]);
    if (!tie) {
        for (uint32_t i = tid; i < K; i += kSelThreads) {
            ov[i] = sel_v[i];
            oi[i] = sel_i[i];
        }
        return;
    }
    if (tid == 0) {
        // heap arrays are 1-based: slots 1..K of 33
        for (uint32_t i = 1; i <= K; ++i) heap_v[i] = sentinel_f();
        uint32_t dpc = K;
        for (uint32_t i = 0; i < L; ++i) heap_update(heap_v, heap_t, K, dpc, sval[i], i);
        heap_reorder(heap_v, heap_t, K);
        for (uint32_t i = 0; i < K; ++i) {
            ov[i] = heap_v[i + 1];
            oi[i] = heap_t[i + 1];
        }
    }
}

// Tile of k_nearest_center: 64 points x 64 centroids per step, 4x4 per thread.
constexpr int kNcTile = 64, kNcTileK = 32;
// nearest_center (kmeans.cpp:221-258): argmin_c (|x|^2 + |c|^2) - 2 x.c, with the
// double-precision subtraction of the reference done as one float subtraction
// (exact 2*dot, innocuous double rounding), first centroid wins ties.
__global__ __launch_bounds__(256) void k_nearest_center(const float* __restrict__ X, uint64_t n,
                                                        const float* __restrict__ Cn, uint64_t k,
                                                        uint32_t d, const float* __restrict__ xnorm,
                                                        const float* __restrict__ cnorm,
                                                        int32_t* __restrict__ assign,
                                                        float* __restrict__ dis) {
    __shared__ float As[kNcTileK][kNcTile + 1];
    __shared__ float Bs[kNcTileK][kNcTile + 1];
    __shared__ float red_v[16][kNcTile];
    __shared__ uint32_t red_i[16][kNcTile];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const uint64_t a0 = (uint64_t)blockIdx.x * kNcTile;
    float best[4];
    uint32_t bidx[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        best[i] = FLT_MAX;
        bidx[i] = 0;
    }
    for (uint64_t b0 = 0; b0 < k; b0 += kNcTile) {
        float acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
        for (uint32_t k0 = 0; k0 < d; k0 += kNcTileK) {
            for (int e = threadIdx.x; e < kNcTile * kNcTileK; e += 256) {
                const int r = e / kNcTileK, kk = e % kNcTileK;
                const uint32_t kd = k0 + kk;
                As[kk][r] = (a0 + r < n && kd < d) ? X[(a0 + r) * d + kd] : 0.0f;
                Bs[kk][r] = (b0 + r < k && kd < d) ? Cn[(b0 + r) * d + kd] : 0.0f;
            }
            __syncthreads();
            const uint32_t kmax = min((uint32_t)kNcTileK, d - k0);
            for (uint32_t kk = 0; kk < kmax; ++kk) {
                float av[4], bv[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        acc[i][j] = __fadd_rn(acc[i][j], __fmul_rn(av[i], bv[j]));
            }
            __syncthreads();
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint64_t a = a0 + ty + 16 * i;
            if (a >= n) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint64_t b = b0 + tx + 16 * j;
                if (b >= k) continue;
                const float s = __fadd_rn(xnorm[a], cnorm[b]);
                const float cur = __fsub_rn(s, 2.0f * acc[i][j]);
                if (cur < best[i]) {  // j ascends within a thread, tiles ascend: first wins
                    best[i] = cur;
                    bidx[i] = (uint32_t)b;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        red_v[tx][ty + 16 * i] = best[i];
        red_i[tx][ty + 16 * i] = bidx[i];
    }
    __syncthreads();
    if (threadIdx.x < kNcTile) {
        const int r = threadIdx.x;
        // Per-thread results are either a strict improvement on FLT_MAX or
        // (FLT_MAX, 0) for "none"; merge to the smallest value, lowest id.
        float bv = FLT_MAX;
        uint32_t bi = 0;
        for (int t = 0; t < 16; ++t) {
            const float v = red_v[t][r];
            const uint32_t id = red_i[t][r];
            if (v < bv || (v == bv && v < FLT_MAX && id < bi)) {
                bv = v;
                bi = id;
            }
        }
        const uint64_t a = a0 + r;
        if (a < n) {
            assign[a] = (int32_t)bi;
            dis[a] = bv;
        }
    }
}

__global__ void k_to_bf16_rows(const float* __restrict__ x, uint64_t n, uint16_t* __restrict__ y) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __bfloat16_as_ushort(__float2bfloat16_rn(x[i]));
}

__global__ void k_gather_u32(const uint32_t* __restrict__ idx, uint64_t n,
                             const uint32_t* __restrict__ table, uint32_t* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = idx[i] == kNoLabel ? kNoLabel : table[idx[i]];
}

__global__ void k_norms_full(const float* __restrict__ X, uint64_t rows, uint32_t d,
                             float* __restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    out[r] = dot_seq(X + r * d, X + r * d, d);
}

}  // namespace

// ----------------------------------------------------------------- launchers

cudaError_t launch_prep_queries(const DeviceIndex& ix, const float* q_in, uint32_t n, Scratch& s,
                                cudaStream_t stream) {
    const size_t smem = sizeof(float) * kPrepWarps * ix.d;  // <= 32 KB (d <= kMaxDim)
    k_prep_queries<<<(n + kPrepWarps - 1) / kPrepWarps, kPrepWarps * 32, smem, stream>>>(
        q_in, s.q, s.qb, s.qnorm, s.status, n, ix.d, ix.qdim, ix.whether_norm, ix.ip2cos);
    return cudaGetLastError();
}

cudaError_t launch_centroid_scores(const float* queries, uint32_t nq, const float* cents,
                                   uint32_t nc, uint32_t d, const float* bias, bool negate,
                                   float* out, uint32_t ld_out, cudaStream_t stream) {
    dim3 grid((nc + kTile - 1) / kTile, (nq + kTile - 1) / kTile);
    if (negate) {
        k_centroid_scores<1><<<grid, 256, 0, stream>>>(queries, nq, cents, nc, d, bias, out, ld_out);
    } else {
        k_centroid_scores<0><<<grid, 256, 0, stream>>>(queries, nq, cents, nc, d, bias, out, ld_out);
    }
    return cudaGetLastError();
}

cudaError_t launch_stationary(const float* coarse, uint32_t C, const float* fine, uint32_t F,
                              uint32_t d, const float* fine_half_norms, float* stationary,
                              cudaStream_t stream) {
    // stationary[c][f] = 0.5|f|^2 + f.c (hierarchical_cluster_index.cpp:302-320)
    dim3 grid((F + kTile - 1) / kTile, (C + kTile - 1) / kTile);
    k_centroid_scores<2><<<grid, 256, 0, stream>>>(coarse, C, fine, F, d, fine_half_norms,
                                                   stationary, F);
    return cudaGetLastError();
}

cudaError_t launch_half_norms(const float* X, uint32_t rows, uint32_t d, float* out,
                              cudaStream_t stream) {
    k_half_norms<<<(rows + 127) / 128, 128, 0, stream>>>(X, rows, d, out);
    return cudaGetLastError();
}

cudaError_t launch_cell_constants(float* stationary, const uint32_t* cell_start, float* mdo,
                                  uint32_t C, uint32_t F, float empty_value, cudaStream_t stream) {
    k_cell_constants<<<(C + 127) / 128, 128, 0, stream>>>(stationary, cell_start, mdo, C, F,
                                                         empty_value);
    return cudaGetLastError();
}

static uint32_t next_pow2(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

cudaError_t launch_topsort_status(const float* vals, uint32_t nrows, uint32_t L, uint32_t ld_vals,
                                  uint32_t K, float* out_val, uint32_t* out_idx,
                                  const int32_t* status, cudaStream_t stream) {
    if (K < L && K + 1 <= 32) {
        ensure_max_dynamic_smem(k_topsel_small, 220 * 1024);
        k_topsel_small<<<nrows, kSelThreads, (size_t)L * sizeof(float), stream>>>(
            vals, L, ld_vals, K, out_val, out_idx, status);
        return cudaGetLastError();
    }
    const uint32_t Lp = next_pow2(L < 2 ? 2 : L);
    const size_t smem = (size_t)Lp * 8;
    ensure_max_dynamic_smem(k_topsort, 220 * 1024);
    k_topsort<<<nrows, 512, smem, stream>>>(vals, L, Lp, ld_vals, K, out_val, out_idx, status);
    return cudaGetLastError();
}

cudaError_t launch_topsort(const float* vals, uint32_t nrows, uint32_t L, uint32_t ld_vals,
                           uint32_t K, float* out_val, uint32_t* out_idx, cudaStream_t stream) {
    return launch_topsort_status(vals, nrows, L, ld_vals, K, out_val, out_idx, nullptr, stream);
}

cudaError_t launch_nearest_center(uint32_t dim, const float* cents, uint64_t k, const float* x,
                                  uint64_t n, int32_t* assign, float* dis, cudaStream_t stream) {
    float* xnorm = nullptr;
    float* cnorm = nullptr;
    cudaError_t e = cudaMallocAsync(&xnorm, sizeof(float) * (n ? n : 1), stream);
    if (e != cudaSuccess) return e;
    e = cudaMallocAsync(&cnorm, sizeof(float) * (k ? k : 1), stream);
    if (e != cudaSuccess) {
        cudaFreeAsync(xnorm, stream);
        return e;
    }
    k_norms_full<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(x, n, dim, xnorm);
    k_norms_full<<<(unsigned)((k + 255) / 256), 256, 0, stream>>>(cents, k, dim, cnorm);
    k_nearest_center<<<(unsigned)((n + kNcTile - 1) / kNcTile), 256, 0, stream>>>(x, n, cents, k, dim,
                                                                             xnorm, cnorm, assign,
                                                                             dis);
    e = cudaGetLastError();
    cudaFreeAsync(xnorm, stream);
    cudaFreeAsync(cnorm, stream);
    return e;
}

cudaError_t launch_nearest_center_scratch(uint32_t dim, const float* cents, uint64_t k,
                                          const float* x, uint64_t n, int32_t* assign, float* dis,
                                          float* xnorm, float* cnorm, cudaStream_t stream) {
    k_norms_full<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(x, n, dim, xnorm);
    k_norms_full<<<(unsigned)((k + 255) / 256), 256, 0, stream>>>(cents, k, dim, cnorm);
    k_nearest_center<<<(unsigned)((n + kNcTile - 1) / kNcTile), 256, 0, stream>>>(x, n, cents, k, dim,
                                                                             xnorm, cnorm, assign,
                                                                             dis);
    return cudaGetLastError();
}

cudaError_t launch_gather_u32(const uint32_t* idx, uint64_t n, const uint32_t* table,
                              uint32_t* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_gather_u32<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(idx, n, table, out);
    return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* x, uint64_t n, uint16_t* y, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_to_bf16_rows<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(x, n, y);
    return cudaGetLastError();
}

}  // namespace pgpu
