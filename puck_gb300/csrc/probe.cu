// Learned probe predictor: a small MLP (query -> coarse-cluster scores) trained
// and evaluated on the GPU with the BF16 tensor-core contraction (tc_gemm.cu).
//
//   H1 = GELU(X W1^T + b1)      X [n][d],  W1 [h][d]
//   H2 = GELU(H1 W2^T + b2)     W2 [h][h]
//   Z  = H2 W3^T + b3           W3 [C][h]  (scores of the C coarse clusters)
//
// Training target of a query: the distribution of the coarse clusters that hold
// its exact top-L neighbours (L ids per query, kNoLabel for none); the loss is
// the softmax cross-entropy against it, mean over the batch; Adam on FP32
// master weights. Every GEMM of the forward and backward passes runs on the
// tensor cores in BF16 with FP32 accumulation; softmax, bias gradients and the
// optimizer are FP32 CUDA kernels.
//
// Search with a probe attached (scan mode): per query the clusters are taken in
// descending predicted probability until their mass reaches `mass` (adaptive
// search_coarse_count); when max_probe clusters do not reach it, the query keeps
// the plain fixed-count coarse selection (confidence fallback). The coarse
// distance of a chosen cluster is the reference's exact FP32 value.
#include <cuda_bf16.h>

#include <cfloat>
#include <cstdint>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr int kProbeThreads = 256;

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// uniform(-a, a) from a counter-based hash: deterministic for a seed
__global__ void k_init_uniform(float* __restrict__ w, uint64_t n, float a, uint64_t seed) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t r = splitmix64(seed * 0x100000001B3ull + i);
    const float u = (float)(r >> 40) * (1.0f / 16777216.0f);  // [0, 1)
    w[i] = (2.0f * u - 1.0f) * a;
}

// Per row: softmax of the scores, the soft target from the row's label ids, the
// row loss, and dZ = (softmax - target) / n.
__global__ __launch_bounds__(kProbeThreads) void k_softmax_xent(
    const float* __restrict__ Z, uint32_t C, const uint32_t* __restrict__ labels, uint32_t L,
    uint32_t n, float* __restrict__ dZ, float* __restrict__ loss_sum) {
    __shared__ float red[kProbeThreads / 32];
    __shared__ float bcast;
    const uint32_t row = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float* z = Z + (uint64_t)row * C;
    float* g = dZ + (uint64_t)row * C;
    float m = -FLT_MAX;
    for (uint32_t c = tid; c < C; c += kProbeThreads) m = fmaxf(m, z[c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red[warp] = m;
    __syncthreads();
    if (tid == 0) {
        float v = red[0];
        for (int w = 1; w < kProbeThreads / 32; ++w) v = fmaxf(v, red[w]);
        bcast = v;
    }
    __syncthreads();
    m = bcast;
    float s = 0.0f;
    for (uint32_t c = tid; c < C; c += kProbeThreads) s += expf(z[c] - m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __syncthreads();
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (tid == 0) {
        float v = 0.0f;
        for (int w = 0; w < kProbeThreads / 32; ++w) v += red[w];
        bcast = v;
    }
    __syncthreads();
    const float lse = m + logf(bcast);
    const uint32_t* lab = labels + (uint64_t)row * L;
    uint32_t valid = 0;
    for (uint32_t t = 0; t < L; ++t) valid += lab[t] < C;
    const float w = valid ? 1.0f / (float)valid : 0.0f;
    const float inv_n = 1.0f / (float)n;
    for (uint32_t c = tid; c < C; c += kProbeThreads) g[c] = expf(z[c] - lse) * inv_n;
    __syncthreads();
    if (tid == 0) {
        float l = 0.0f;
        for (uint32_t t = 0; t < L; ++t) {
            const uint32_t c = lab[t];
            if (c >= C) continue;
            g[c] -= w * inv_n;
            l += w * (lse - z[c]);
        }
        atomicAdd(loss_sum, l * inv_n);
    }
}

// out[j] = sum_i G[i][j] (bias gradients), one thread per column
__global__ void k_colsum(const float* __restrict__ G, uint32_t rows, uint32_t cols,
                         float* __restrict__ out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.0f;
    for (uint32_t i = 0; i < rows; ++i) s += G[(uint64_t)i * cols + j];
    out[j] = s;
}

__global__ void k_to_bf16(const float* __restrict__ x, uint64_t n, uint16_t* __restrict__ y) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __bfloat16_as_ushort(__float2bfloat16_rn(x[i]));
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, uint64_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Adaptive cluster choice from the probe's scores (see the file comment). Rows
// that the probe answers get their clusters in ctag/cdist [n][Pcap] (unused slots
// kNoLabel) and pconf = 1; the others get pconf = 0 and are left to the
// fixed-count selection.
__global__ __launch_bounds__(kProbeThreads) void k_probe_select(
    const float* __restrict__ Z, uint32_t C, const float* __restrict__ Q, uint32_t d,
    const float* __restrict__ cents, const float* __restrict__ bias, const int32_t* __restrict__ status,
    float mass, uint32_t max_probe, uint32_t Pcap, float* __restrict__ cdist,
    uint32_t* __restrict__ ctag, int32_t* __restrict__ pconf,
    unsigned long long* __restrict__ counters, uint32_t* __restrict__ ulist,
    uint32_t* __restrict__ ucount) {
    extern __shared__ float sp[];  // [C] probabilities
    __shared__ float red_v[kProbeThreads / 32];
    __shared__ uint32_t red_i[kProbeThreads / 32];
    __shared__ float sp_top[kProbeThreads / 32];
    __shared__ float bcast;
    __shared__ uint32_t pick[64];
    __shared__ uint32_t npick;
    __shared__ int confident;
    const uint32_t row = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) pconf[row] = 0;
    // a row the probe does not answer goes to the fixed-count selection's list
    auto leave = [&]() {
        if (tid == 0 && ulist != nullptr) ulist[atomicAdd(ucount, 1u)] = row;
    };
    if (status[row] != 0) {
        leave();
        return;
    }
    const float* z = Z + (uint64_t)row * C;
    float m = -FLT_MAX;
    for (uint32_t c = tid; c < C; c += kProbeThreads) m = fmaxf(m, z[c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) red_v[warp] = m;
    __syncthreads();
    if (tid == 0) {
        float v = red_v[0];
        for (int w = 1; w < kProbeThreads / 32; ++w) v = fmaxf(v, red_v[w]);
        bcast = v;
    }
    __syncthreads();
    m = bcast;
    float s = 0.0f;
    float ev = -1.0f;  // the largest exp value, lowest id: the first cluster of the order below
    uint32_t ei = 0xFFFFFFFFu;
    for (uint32_t c = tid; c < C; c += kProbeThreads) {
        const float e = expf(z[c] - m);
        sp[c] = e;
        s += e;
        if (e > ev) {  // c ascends within a thread
            ev = e;
            ei = c;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        const float ov = __shfl_xor_sync(0xffffffffu, ev, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, ei, o);
        if (ov > ev || (ov == ev && oi < ei)) {
            ev = ov;
            ei = oi;
        }
    }
    __syncthreads();
    if (lane == 0) {
        red_v[warp] = s;
        red_i[warp] = ei;
        sp_top[warp] = ev;
    }
    __syncthreads();
    if (tid == 0) {
        float v = 0.0f, bv = -1.0f;
        uint32_t bi = 0xFFFFFFFFu;
        for (int w = 0; w < kProbeThreads / 32; ++w) {
            v += red_v[w];
            if (sp_top[w] > bv || (sp_top[w] == bv && red_i[w] < bi)) {
                bv = sp_top[w];
                bi = red_i[w];
            }
        }
        bcast = v;
        npick = 0;
        confident = 0;
        // one cluster already holds the mass: no ranking rounds
        if (bv * (1.0f / v) >= mass && max_probe >= 1) {
            pick[0] = bi;
            npick = 1;
            confident = 1;
        }
    }
    __syncthreads();
    const float inv = 1.0f / bcast;
    float acc = 0.0f;
    // descending probability, ties to the lower id, until the mass is reached
    for (uint32_t r = 0; !confident && r < max_probe; ++r) {
        float bv = -1.0f;
        uint32_t bi = 0xFFFFFFFFu;
        for (uint32_t c = tid; c < C; c += kProbeThreads) {
            const float v = sp[c];
            if (v > bv || (v == bv && c < bi)) {
                bv = v;
                bi = c;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
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
            for (int w = 1; w < kProbeThreads / 32; ++w)
                if (red_v[w] > fv || (red_v[w] == fv && red_i[w] < fi)) {
                    fv = red_v[w];
                    fi = red_i[w];
                }
            pick[r] = fi;
            npick = r + 1;
            sp[fi] = -1.0f;
            bcast = fv * inv;
        }
        __syncthreads();
        acc += bcast;
        if (acc >= mass) {
            if (tid == 0) confident = 1;
            break;
        }
    }
    __syncthreads();
    if (!confident) {
        if (tid == 0) atomicAdd(counters + kCounterProbeFallbacks, 1ull);
        leave();
        return;  // the fixed-count selection fills this row
    }
    if (tid == 0) pconf[row] = 1;
    const uint32_t np = npick;
    const float* q = Q + (uint64_t)row * d;
    for (uint32_t i = tid; i < Pcap; i += kProbeThreads) {
        if (i < np) {
            const uint32_t c = pick[i];
            cdist[(uint64_t)row * Pcap + i] = __fsub_rn(bias[c], dot_seq(q, cents + (uint64_t)c * d, d));
            ctag[(uint64_t)row * Pcap + i] = c;
        } else {
            cdist[(uint64_t)row * Pcap + i] = sentinel_f();
            ctag[(uint64_t)row * Pcap + i] = kNoLabel;
        }
    }
    if (tid == 0) atomicAdd(counters + kCounterProbeClusters, (unsigned long long)np);
}

}  // namespace

uint64_t ProbeNet::param_count() const {
    return (uint64_t)h * d + h + (uint64_t)h * h + h + (uint64_t)C * h + C;
}

cudaError_t probe_forward(const ProbeNet& net, const float* X, uint32_t n, float* H1, float* Z1,
                          float* H2, float* Z2, float* Z, int* err, cudaStream_t st) {
    TcEpilogue e1{};
    e1.mode = TC_EPI_BIAS_GELU;
    e1.out = H1;
    e1.ld = net.h;
    e1.bias = net.b1;
    e1.out2 = Z1;
    cudaError_t e = launch_tc_gemm(TcOperand{X, net.d, 1, n}, TcOperand{net.W1, net.d, 1, net.h},
                                   net.d, e1, err, st);
    if (e != cudaSuccess) return e;
    TcEpilogue e2{};
    e2.mode = TC_EPI_BIAS_GELU;
    e2.out = H2;
    e2.ld = net.h;
    e2.bias = net.b2;
    e2.out2 = Z2;
    e = launch_tc_gemm(TcOperand{H1, net.h, 1, n}, TcOperand{net.W2, net.h, 1, net.h}, net.h, e2,
                       err, st);
    if (e != cudaSuccess) return e;
    TcEpilogue e3{};
    e3.mode = TC_EPI_BIAS;
    e3.out = Z;
    e3.ld = net.C;
    e3.bias = net.b3;
    return launch_tc_gemm(TcOperand{H2, net.h, 1, n}, TcOperand{net.W3, net.h, 1, net.C}, net.h, e3,
                          err, st);
}

cudaError_t probe_sync_bf16(const ProbeNet& net, cudaStream_t st) {
    const struct {
        const float* w;
        uint16_t* b;
        uint64_t n;
    } mats[] = {{net.W1, net.W1b, (uint64_t)net.h * net.d},
                {net.W2, net.W2b, (uint64_t)net.h * net.h},
                {net.W3, net.W3b, (uint64_t)net.C * net.h}};
    for (const auto& m : mats)
        k_to_bf16<<<(unsigned)((m.n + 255) / 256), 256, 0, st>>>(m.w, m.n, m.b);
    return cudaGetLastError();
}

cudaError_t probe_infer(const ProbeNet& net, const float* X, const uint16_t* Xb, uint32_t n,
                        uint16_t* H1b, uint16_t* H2b, float* Z, int* err, cudaStream_t st) {
    TcEpilogue e1{};
    e1.mode = TC_EPI_BIAS_GELU;
    e1.out_bf16 = H1b;
    e1.ld = net.h;
    e1.bias = net.b1;
    TcOperand w1{nullptr, net.d, 1, net.h, net.W1b};
    cudaError_t e = launch_tc_gemm(TcOperand{X, net.d, 1, n, Xb}, w1, net.d, e1, err, st);
    if (e != cudaSuccess) return e;
    TcEpilogue e2{};
    e2.mode = TC_EPI_BIAS_GELU;
    e2.out_bf16 = H2b;
    e2.ld = net.h;
    e2.bias = net.b2;
    e = launch_tc_gemm(TcOperand{nullptr, net.h, 1, n, H1b},
                       TcOperand{nullptr, net.h, 1, net.h, net.W2b}, net.h, e2, err, st);
    if (e != cudaSuccess) return e;
    TcEpilogue e3{};
    e3.mode = TC_EPI_BIAS;
    e3.out = Z;
    e3.ld = net.C;
    e3.bias = net.b3;
    return launch_tc_gemm(TcOperand{nullptr, net.h, 1, n, H2b},
                          TcOperand{nullptr, net.h, 1, net.C, net.W3b}, net.h, e3, err, st);
}

cudaError_t probe_backward(const ProbeNet& net, const float* X, uint32_t n,
                           const uint32_t* labels, uint32_t L, ProbeWork& w, ProbeNet& grad,
                           float* loss_sum, int* err, cudaStream_t st) {
    cudaError_t e = probe_forward(net, X, n, w.H1, w.Z1, w.H2, w.Z2, w.Z, err, st);
    if (e != cudaSuccess) return e;
    k_softmax_xent<<<n, kProbeThreads, 0, st>>>(w.Z, net.C, labels, L, n, w.dZ, loss_sum);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    TcEpilogue s{};
    s.mode = TC_EPI_STORE;
    s.alpha = 1.0f;
    // dW3 = dZ^T H2                                     [C][h], contraction over the batch
    s.out = grad.W3;
    s.ld = net.h;
    e = launch_tc_gemm(TcOperand{w.dZ, 1, net.C, net.C}, TcOperand{w.H2, 1, net.h, net.h}, n, s,
                       err, st);
    if (e != cudaSuccess) return e;
    k_colsum<<<(net.C + 255) / 256, 256, 0, st>>>(w.dZ, n, net.C, grad.b3);
    // dZ2 = (dZ W3) * GELU'(Z2)                          [n][h], contraction over C
    TcEpilogue gb{};
    gb.mode = TC_EPI_GELU_BWD;
    gb.out = w.dH2;
    gb.ld = net.h;
    gb.aux = w.Z2;
    gb.ld_aux = net.h;
    e = launch_tc_gemm(TcOperand{w.dZ, net.C, 1, n}, TcOperand{net.W3, 1, net.h, net.h}, net.C, gb,
                       err, st);
    if (e != cudaSuccess) return e;
    // dW2 = dZ2^T H1, db2
    s.out = grad.W2;
    s.ld = net.h;
    e = launch_tc_gemm(TcOperand{w.dH2, 1, net.h, net.h}, TcOperand{w.H1, 1, net.h, net.h}, n, s,
                       err, st);
    if (e != cudaSuccess) return e;
    k_colsum<<<(net.h + 255) / 256, 256, 0, st>>>(w.dH2, n, net.h, grad.b2);
    // dZ1 = (dZ2 W2) * GELU'(Z1)
    gb.out = w.dH1;
    gb.aux = w.Z1;
    e = launch_tc_gemm(TcOperand{w.dH2, net.h, 1, n}, TcOperand{net.W2, 1, net.h, net.h}, net.h, gb,
                       err, st);
    if (e != cudaSuccess) return e;
    // dW1 = dZ1^T X, db1
    s.out = grad.W1;
    s.ld = net.d;
    e = launch_tc_gemm(TcOperand{w.dH1, 1, net.h, net.h}, TcOperand{X, 1, net.d, net.d}, n, s, err,
                       st);
    if (e != cudaSuccess) return e;
    k_colsum<<<(net.h + 255) / 256, 256, 0, st>>>(w.dH1, n, net.h, grad.b1);
    return cudaGetLastError();
}

cudaError_t probe_init(ProbeNet& net, uint64_t seed, cudaStream_t st) {
    struct L {
        float* w;
        uint64_t n;
        float a;
    } layers[] = {{net.W1, (uint64_t)net.h * net.d, sqrtf(3.0f / net.d)},
                  {net.W2, (uint64_t)net.h * net.h, sqrtf(3.0f / net.h)},
                  {net.W3, (uint64_t)net.C * net.h, sqrtf(3.0f / net.h)}};
    uint64_t k = 0;
    for (const L& l : layers) {
        k_init_uniform<<<(unsigned)((l.n + 255) / 256), 256, 0, st>>>(l.w, l.n, l.a, seed * 3 + k++);
    }
    cudaMemsetAsync(net.b1, 0, sizeof(float) * net.h, st);
    cudaMemsetAsync(net.b2, 0, sizeof(float) * net.h, st);
    cudaMemsetAsync(net.b3, 0, sizeof(float) * net.C, st);
    return cudaGetLastError();
}

cudaError_t probe_adam(ProbeNet& net, const ProbeNet& grad, ProbeNet& m, ProbeNet& v, float lr,
                       uint64_t step, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    // the parameters are one contiguous block in every ProbeNet
    const uint64_t n = net.param_count();
    k_adam<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(net.W1, grad.W1, m.W1, v.W1, n, lr, b1, b2,
                                                         eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_probe_select(const ProbeNet& net, const DeviceIndex& ix, uint32_t n,
                                const float* Z, float mass, uint32_t max_probe, Scratch& s,
                                cudaStream_t st) {
    ensure_max_dynamic_smem(k_probe_select, 200 * 1024);
    k_probe_select<<<n, kProbeThreads, sizeof(float) * net.C, st>>>(
        Z, net.C, s.q, ix.d, ix.coarse, ix.coarse_norms, s.status, mass, max_probe, s.P, s.cdist,
        s.ctag, s.pconf, s.counters, s.ulist, s.ucount);
    return cudaGetLastError();
}

}  // namespace pgpu
