// Brute-force k nearest neighbours (squared L2) of a query batch over a base
// set, on the GPU: the training labels of the learned probe.
//
// Every (query, base) pair is screened on the tensor cores: s = 0.5|x|^2 - q.x
// (BF16 operands, FP32 accumulation), which orders the base like |q - x|^2. Per
// query the 64 smallest screened values are kept across base chunks (one warp
// per query row, threshold test then a merge of 64 + 64 candidates in shared
// memory), then rescored in FP32 and the k best returned in ascending order.
// Candidates are exact as long as the true k-th neighbour's screened value is
// among the 64 smallest, i.e. except where more than 64 - k points lie within
// the screen's error of it.
#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr uint32_t kKC = 64;          // candidates per query
constexpr int kWarpsPerBlock = 8;

__global__ void k_half_sq_norms(const float* __restrict__ X, uint64_t rows, uint32_t d,
                                float* __restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const float* x = X + r * d;
    float s = 0.0f;
    for (uint32_t k = 0; k < d; ++k) s += x[k] * x[k];
    out[r] = 0.5f * s;
}

__global__ void k_knn_reset(float* __restrict__ cs, uint32_t* __restrict__ ci,
                            float* __restrict__ thr, uint32_t nq) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint64_t)nq * kKC) {
        cs[i] = FLT_MAX;
        ci[i] = kNoLabel;
    }
    if (i < nq) thr[i] = FLT_MAX;
}

// Sorts a warp's 128 (value, id) pairs ascending (4 per lane, bitonic over shared memory).
__device__ void warp_sort128(float* v, uint32_t* id) {
    const int lane = threadIdx.x & 31;
    for (uint32_t size = 2; size <= 128; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const uint32_t t = lane + 32 * u;  // 64 compare-exchanges
                const uint32_t lo = 2 * t - (t & (stride - 1));
                const uint32_t hi = lo + stride;
                const float a = v[lo], b = v[hi];
                const uint32_t ia = id[lo], ib = id[hi];
                const bool gt = a > b || (a == b && ia > ib);
                if (gt == ((lo & size) == 0)) {
                    v[lo] = b;
                    v[hi] = a;
                    id[lo] = ib;
                    id[hi] = ia;
                }
            }
            __syncwarp();
        }
    }
}

// One warp per query row of the screen chunk S [rows][ld] (base ids base0 + j).
__global__ __launch_bounds__(kWarpsPerBlock * 32) void k_knn_merge(
    const float* __restrict__ S, uint32_t ld, uint32_t rows, uint32_t cols, uint32_t base0,
    float* __restrict__ cs, uint32_t* __restrict__ ci, float* __restrict__ thr) {
    __shared__ float bv[kWarpsPerBlock][2 * kKC];
    __shared__ uint32_t bi[kWarpsPerBlock][2 * kKC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t row = blockIdx.x * kWarpsPerBlock + warp;
    if (row >= rows) return;
    float* v = bv[warp];
    uint32_t* id = bi[warp];
    float* rs = cs + (uint64_t)row * kKC;
    uint32_t* ri = ci + (uint64_t)row * kKC;
    for (int u = 0; u < 2; ++u) {
        v[lane + 32 * u] = rs[lane + 32 * u];
        id[lane + 32 * u] = ri[lane + 32 * u];
    }
    float t = thr[row];
    uint32_t nb = 0;  // new candidates in v[64 ..)
    const float* s = S + (uint64_t)row * ld;
    for (uint32_t j0 = 0; j0 < cols; j0 += 32) {
        const uint32_t j = j0 + lane;
        const float x = j < cols ? s[j] : FLT_MAX;
        unsigned b = __ballot_sync(0xffffffffu, x < t);
        if (b == 0) continue;
        if (nb + __popc(b) > kKC) {
            // merge: sort the 64 kept + the nb new ones, keep 64, tighten the threshold
            for (uint32_t e = kKC + nb + lane; e < 2 * kKC; e += 32) {
                v[e] = FLT_MAX;
                id[e] = kNoLabel;
            }
            __syncwarp();
            warp_sort128(v, id);
            t = v[kKC - 1];
            nb = 0;
            b = __ballot_sync(0xffffffffu, x < t);
            if (b == 0) continue;
        }
        if (x < t) {
            const uint32_t pos = kKC + nb + __popc(b & ((1u << lane) - 1));
            v[pos] = x;
            id[pos] = base0 + j;
        }
        nb += __popc(b);
        __syncwarp();
    }
    if (nb > 0) {
        for (uint32_t e = kKC + nb + lane; e < 2 * kKC; e += 32) {
            v[e] = FLT_MAX;
            id[e] = kNoLabel;
        }
        __syncwarp();
        warp_sort128(v, id);
        t = v[kKC - 1];
    }
    for (int u = 0; u < 2; ++u) {
        rs[lane + 32 * u] = v[lane + 32 * u];
        ri[lane + 32 * u] = id[lane + 32 * u];
    }
    if (lane == 0) thr[row] = t;
}

// FP32 rescoring of the 64 candidates, k best ascending (one warp per query).
__global__ __launch_bounds__(kWarpsPerBlock * 32) void k_knn_final(
    const float* __restrict__ base, uint32_t d, const float* __restrict__ Q, uint32_t rows,
    const uint32_t* __restrict__ ci, uint32_t k, uint32_t* __restrict__ out_ids,
    float* __restrict__ out_dist) {
    __shared__ float bv[kWarpsPerBlock][2 * kKC];
    __shared__ uint32_t bi[kWarpsPerBlock][2 * kKC];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t row = blockIdx.x * kWarpsPerBlock + warp;
    if (row >= rows) return;
    float* v = bv[warp];
    uint32_t* id = bi[warp];
    const float* q = Q + (uint64_t)row * d;
    for (int u = 0; u < 4; ++u) {
        const uint32_t e = lane + 32 * u;
        uint32_t c = e < kKC ? ci[(uint64_t)row * kKC + e] : kNoLabel;
        float dist = FLT_MAX;
        if (c != kNoLabel) {
            const float* x = base + (uint64_t)c * d;
            float s = 0.0f;
            for (uint32_t t = 0; t < d; ++t) {
                const float df = q[t] - x[t];
                s += df * df;
            }
            dist = s;
        }
        v[e] = dist;
        id[e] = c;
    }
    __syncwarp();
    warp_sort128(v, id);
    for (uint32_t e = lane; e < k; e += 32) {
        out_ids[(uint64_t)row * k + e] = id[e];
        out_dist[(uint64_t)row * k + e] = v[e];
    }
}

}  // namespace

cudaError_t launch_knn(const float* base, uint64_t n, uint32_t d, const float* Q, uint32_t nq,
                       uint32_t k, uint32_t* ids, float* dist, int* err, cudaStream_t st) {
    if (k == 0 || k > kKC || n == 0 || nq == 0) return cudaErrorInvalidValue;
    constexpr uint32_t kQC = 8192, kBC = 16384;
    float *S = nullptr, *hb = nullptr, *cs = nullptr, *thr = nullptr;
    uint32_t* ci = nullptr;
    cudaError_t e = cudaMallocAsync(&S, sizeof(float) * kQC * kBC, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&hb, sizeof(float) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&cs, sizeof(float) * kQC * kKC, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&ci, sizeof(uint32_t) * kQC * kKC, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&thr, sizeof(float) * kQC, st);
    if (e == cudaSuccess) {
        k_half_sq_norms<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(base, n, d, hb);
        e = cudaGetLastError();
    }
    for (uint32_t q0 = 0; e == cudaSuccess && q0 < nq; q0 += kQC) {
        const uint32_t qr = nq - q0 < kQC ? nq - q0 : kQC;
        k_knn_reset<<<(qr * kKC + 255) / 256, 256, 0, st>>>(cs, ci, thr, qr);
        for (uint64_t b0 = 0; e == cudaSuccess && b0 < n; b0 += kBC) {
            const uint32_t br = (uint32_t)(n - b0 < kBC ? n - b0 : kBC);
            TcEpilogue ep{};
            ep.mode = TC_EPI_SCORE;
            ep.out = S;
            ep.ld = kBC;
            ep.bias = hb + b0;
            e = launch_tc_gemm(TcOperand{Q + (uint64_t)q0 * d, d, 1, qr},
                               TcOperand{base + b0 * d, d, 1, br}, d, ep, err, st);
            if (e != cudaSuccess) break;
            k_knn_merge<<<(qr + kWarpsPerBlock - 1) / kWarpsPerBlock, kWarpsPerBlock * 32, 0, st>>>(
                S, kBC, qr, br, (uint32_t)b0, cs, ci, thr);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        k_knn_final<<<(qr + kWarpsPerBlock - 1) / kWarpsPerBlock, kWarpsPerBlock * 32, 0, st>>>(
            base, d, Q + (uint64_t)q0 * d, qr, ci, k, ids + (uint64_t)q0 * k,
            dist + (uint64_t)q0 * k);
        e = cudaGetLastError();
    }
    if (S) cudaFreeAsync(S, st);
    if (hb) cudaFreeAsync(hb, st);
    if (cs) cudaFreeAsync(cs, st);
    if (ci) cudaFreeAsync(ci, st);
    if (thr) cudaFreeAsync(thr, st);
    return e;
}

}  // namespace pgpu
