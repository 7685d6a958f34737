// pgpu_puck_assign: the build's encoder, PuckIndex::puck_assign
// (puck/puck/puck_index.cpp:602-709), for points whose cells are already known.
//
// Per point, in the reference's float order:
//   r = (x - coarse[c]) - fine[f]                     saxpy(-1) twice (:638-643)
//   per filter subspace k: code_k = nearest_center of r's slice over the 256
//     codewords (kmeans.cpp:221-258: (|r_k|^2 + |w|^2) - 2 r_k.w, first minimum
//     wins), then r_k -= w[code_k]                    (:649-679)
//   the second-level PQ (whether_pq) encodes what is left of r the same way
//   offset = 2 * sdot(decode(codes), vocab), vocab = coarse[c] + fine[f], and for
//     the second-level PQ vocab += the filter decode   (set_static_value_of_formula,
//     quantization.cpp:244-258)
// Every dot product sums sequentially from 0, one rounding per product and sum.
// The reference subtracts 2*dot in double after a float sum; that is one
// correctly rounded operation on two floats, so one float subtraction gives the
// same bits.
//
// One warp per point: the residual and the running vocab sit in shared memory,
// the 32 lanes split the 256 codewords of a subspace and reduce (value, index)
// to the smallest value with the lowest index; lane 0 runs the two offset sums.
#include <cuda_runtime.h>

#include <cfloat>
#include <string>

#include "device_common.cuh"
#include "pgpu_internal.h"

namespace {

constexpr int kAssignWarps = 8;

__global__ void k_codeword_norms(const float* __restrict__ cb, uint64_t rows, uint32_t lsq,
                                 float* __restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) out[r] = pgpu::dot_seq(cb + r * lsq, cb + r * lsq, lsq);
}

struct AssignParams {
    const float* base;          // [n][d]
    const uint32_t* cell_assign;
    const float* coarse;        // [C][d]
    const float* fine;          // [F][d]
    const float* fcb;           // [fnsq][256][flsq]
    const float* fcb_norm;      // [fnsq][256]
    const float* pcb;           // [pnsq][256][plsq] (pnsq = 0: none)
    const float* pcb_norm;
    float* f_off;
    uint8_t* f_codes;           // [n][fnsq]
    float* p_off;
    uint8_t* p_codes;           // [n][pnsq]
    int* err;                   // set to 1 for a cell id out of range
    uint64_t n;
    uint32_t d, C, F, fnsq, flsq, pnsq, plsq, stride;  // stride: shared floats per warp
};

// One quantizer's pass over the residual r (shared memory); codes to cs (shared) and out.
__device__ void warp_encode(float* r, const float* __restrict__ cb, const float* __restrict__ cbn,
                            uint32_t nsq, uint32_t lsq, uint8_t* cs, uint8_t* out, int lane) {
    for (uint32_t k = 0; k < nsq; ++k) {
        float* s = r + (uint64_t)k * lsq;
        const float pn = pgpu::dot_seq(s, s, lsq);
        float best = FLT_MAX;
        uint32_t bi = 0;
        for (uint32_t c = lane; c < 256; c += 32) {  // ascending within a lane: first wins
            const float* w = cb + ((uint64_t)k * 256 + c) * lsq;
            float dt = 0.0f;
            for (uint32_t t = 0; t < lsq; ++t) dt = __fadd_rn(dt, __fmul_rn(s[t], __ldg(w + t)));
            const float cur = __fsub_rn(__fadd_rn(pn, __ldg(cbn + (uint64_t)k * 256 + c)), 2.0f * dt);
            if (cur < best) {
                best = cur;
                bi = c;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov < best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            cs[k] = (uint8_t)bi;
            out[k] = (uint8_t)bi;
        }
        const float* w = cb + ((uint64_t)k * 256 + bi) * lsq;
        for (uint32_t t = lane; t < lsq; t += 32) s[t] = __fsub_rn(s[t], __ldg(w + t));
        __syncwarp();
    }
}

// 2 * sum_t decode(codes)[t] * v[t], sequential (lane 0 only).
__device__ float decode_dot(const float* __restrict__ cb, const uint8_t* cs, uint32_t lsq,
                            const float* v, uint32_t d) {
    float s = 0.0f;
    for (uint32_t t = 0; t < d; ++t) {
        const uint32_t k = t / lsq;
        const float dec = __ldg(cb + ((uint64_t)k * 256 + cs[k]) * lsq + (t - k * lsq));
        s = __fadd_rn(s, __fmul_rn(dec, v[t]));
    }
    return 2.0f * s;
}

__global__ __launch_bounds__(kAssignWarps * 32) void k_puck_assign(AssignParams p) {
    extern __shared__ float assign_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t i = (uint64_t)blockIdx.x * kAssignWarps + warp;
    if (i >= p.n) return;  // whole warps only; no block barrier follows
    const uint32_t d = p.d;
    float* r = assign_smem + (uint64_t)warp * p.stride;
    float* v = r + d;
    uint8_t* fcs = reinterpret_cast<uint8_t*>(v + d);
    uint8_t* pcs = fcs + p.fnsq;
    const uint32_t cell = p.cell_assign[i];
    if ((uint64_t)cell >= (uint64_t)p.C * p.F) {
        if (lane == 0) atomicExch(p.err, 1);
        return;
    }
    const uint32_t c = cell / p.F, f = cell % p.F;
    const float* x = p.base + i * d;
    const float* cv = p.coarse + (uint64_t)c * d;
    const float* fv = p.fine + (uint64_t)f * d;
    for (uint32_t t = lane; t < d; t += 32) r[t] = __fsub_rn(__fsub_rn(x[t], cv[t]), fv[t]);
    __syncwarp();
    warp_encode(r, p.fcb, p.fcb_norm, p.fnsq, p.flsq, fcs, p.f_codes + i * p.fnsq, lane);
    if (p.pnsq) warp_encode(r, p.pcb, p.pcb_norm, p.pnsq, p.plsq, pcs, p.p_codes + i * p.pnsq, lane);
    for (uint32_t t = lane; t < d; t += 32) v[t] = __fadd_rn(cv[t], fv[t]);
    __syncwarp();
    if (lane == 0) {
        p.f_off[i] = decode_dot(p.fcb, fcs, p.flsq, v, d);
        if (p.pnsq) {
            for (uint32_t t = 0; t < d; ++t) {
                const uint32_t k = t / p.flsq;
                v[t] = __fadd_rn(v[t], __ldg(p.fcb + ((uint64_t)k * 256 + fcs[k]) * p.flsq +
                                             (t - k * p.flsq)));
            }
            p.p_off[i] = decode_dot(p.pcb, pcs, p.plsq, v, d);
        }
    }
}

}  // namespace

extern "C" int pgpu_puck_assign(uint32_t d, uint64_t n, const float* base,
                                const uint32_t* cell_assign, const float* coarse, uint32_t C,
                                const float* fine, uint32_t F, const float* filter_codebook,
                                uint32_t filter_nsq, const float* pq_codebook, uint32_t pq_nsq,
                                float* filter_offsets, uint8_t* filter_codes, float* pq_offsets,
                                uint8_t* pq_codes, void* stream) {
    if (d == 0 || C == 0 || F == 0 || filter_nsq == 0 || base == nullptr || cell_assign == nullptr ||
        coarse == nullptr || fine == nullptr || filter_codebook == nullptr ||
        filter_offsets == nullptr || filter_codes == nullptr ||
        (pq_nsq > 0 && (pq_codebook == nullptr || pq_offsets == nullptr || pq_codes == nullptr)))
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    if (d % filter_nsq != 0 || (pq_nsq > 0 && d % pq_nsq != 0))
        return pgpu::set_last_error(PGPU_E_UNSUPPORTED, "feature_dim must be a multiple of nsq");
    if (d > pgpu::kMaxDim)
        return pgpu::set_last_error(PGPU_E_LIMIT, "feature_dim above the supported limit");
    if ((uint64_t)C * F > 0xFFFFFFFFull)
        return pgpu::set_last_error(PGPU_E_LIMIT, "more than 2^32-1 cells");
    if (n == 0) return PGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    AssignParams p;
    p.base = base;
    p.cell_assign = cell_assign;
    p.coarse = coarse;
    p.fine = fine;
    p.fcb = filter_codebook;
    p.pcb = pq_codebook;
    p.f_off = filter_offsets;
    p.f_codes = filter_codes;
    p.p_off = pq_offsets;
    p.p_codes = pq_codes;
    p.n = n;
    p.d = d;
    p.C = C;
    p.F = F;
    p.fnsq = filter_nsq;
    p.flsq = d / filter_nsq;
    p.pnsq = pq_nsq;
    p.plsq = pq_nsq ? d / pq_nsq : 0;
    // residual and vocab floats, then the two code rows, rounded up to whole floats
    p.stride = 2 * d + (filter_nsq + pq_nsq + 3) / 4;
    const size_t smem = sizeof(float) * kAssignWarps * p.stride;  // <= 72 KB (d <= kMaxDim)
    const uint64_t nnorm = (uint64_t)(filter_nsq + pq_nsq) * 256;
    float* norms = nullptr;
    int* err = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&norms, sizeof(float) * nnorm + sizeof(int), st);
    if (e != cudaSuccess)
        return pgpu::set_last_error(e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA,
                                    std::string("puck_assign scratch: ") + cudaGetErrorString(e));
    err = reinterpret_cast<int*>(norms + nnorm);
    p.fcb_norm = norms;
    p.pcb_norm = norms + (uint64_t)filter_nsq * 256;
    p.err = err;
    pgpu::ensure_max_dynamic_smem(k_puck_assign, 100 * 1024);
    e = cudaMemsetAsync(err, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        k_codeword_norms<<<(unsigned)((filter_nsq * 256ull + 255) / 256), 256, 0, st>>>(
            filter_codebook, filter_nsq * 256ull, p.flsq, norms);
        if (pq_nsq)
            k_codeword_norms<<<(unsigned)((pq_nsq * 256ull + 255) / 256), 256, 0, st>>>(
                pq_codebook, pq_nsq * 256ull, p.plsq, norms + (uint64_t)filter_nsq * 256);
        k_puck_assign<<<(unsigned)((n + kAssignWarps - 1) / kAssignWarps), kAssignWarps * 32, smem,
                        st>>>(p);
        e = cudaGetLastError();
    }
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(norms, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return pgpu::set_last_error(PGPU_E_CUDA, std::string("puck_assign: ") + cudaGetErrorString(e));
    if (flag) return pgpu::set_last_error(PGPU_E_INVALID, "cell_assign entry out of range");
    return PGPU_OK;
}
