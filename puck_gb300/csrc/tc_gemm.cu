// BF16 tensor-core contraction on sm_103a (tcgen05 + TMEM).
//
//   acc[i][j] = sum_k bf16(A(i,k)) * bf16(B(j,k))          (FP32 accumulation)
//
// A(i,k) = A.p[i*A.rs + k*A.ks], B(j,k) likewise: FP32 operands in any 2-D
// layout (row-major, or transposed for the weight gradients of the probe
// network). They are rounded to BF16 while being staged into shared memory in
// the canonical no-swizzle K-major layout of tcgen05: 8-row x 16-byte core
// matrices, the 16 row groups of a 128-row tile 128 B apart (stride byte offset),
// K groups of 8 elements 2 KiB apart (leading byte offset).
//
// One CTA (4 warps) owns one 128 x 128 output tile. K runs in chunks of 64 over
// two shared-memory stages: all threads stage chunk c+1 while the tensor core
// works on chunk c; thread 0 issues the tcgen05.mma (M=128, N=128, K=16) of a
// chunk into a 128-column TMEM accumulator and commits them to that stage's
// mbarrier, which frees the stage. Each warp then reads its 32 TMEM lanes (= 32
// output rows) with tcgen05.ld and applies the epilogue. Every mbarrier wait is
// bounded: on expiry the kernel sets *err = 1, waits (bounded) for the
// last commit, skips the epilogue and releases its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <mutex>

#include "pgpu_internal.h"

namespace pgpu {
namespace {

constexpr int kTcThreads = 128;
constexpr uint32_t kTileM = 128, kTileN = 128, kChunkK = 64;
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kStageBytes = (kTileM + kTileN) * kChunkK * 2;  // 32 KiB
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading byte offset (between
// core matrices along K), stride byte offset (between 8-row groups), the fixed
// 0b001 at bits 46-48, base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kInstrDesc = (1u << 4) | (1u << 7) | (1u << 10) | ((kTileN >> 3) << 17) |
                                ((kTileM >> 4) << 24);

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
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

// Rows of an operand: op.rows, or fewer when a device count is given; row i of the
// contraction reads source row ridx[i] when a row index is given.
__device__ __forceinline__ uint32_t op_rows(const TcOperand& op) {
    if (op.rows_dev == nullptr) return op.rows;
    const uint32_t r = *op.rows_dev;
    return r < op.rows ? r : op.rows;
}
__device__ __forceinline__ uint32_t src_row(const TcOperand& op, uint32_t i) {
    return op.ridx ? op.ridx[i] : i;
}

// Stages rows [row0, row0+128) x k [k0, k0 + 8*nkg) of an operand into `tile`.
// Thread t owns row t of the tile and writes one 16-byte core-matrix row per K
// group, so a quarter warp stores 128 contiguous bytes (no bank conflict). All of
// a thread's global loads for a group of K groups are issued before any store.
__device__ __forceinline__ void stage_operand(uint8_t* tile, const TcOperand& op, uint32_t row0,
                                              uint32_t k0, uint32_t K, uint32_t nkg, bool vec) {
    const uint32_t r = threadIdx.x;
    const uint32_t crow = row0 + r;
    const bool in = crow < op_rows(op);
    const uint32_t row = in ? src_row(op, crow) : 0u;
    uint8_t* dst = tile + (r >> 3) * 128u + (r & 7u) * 16u;
    if (op.pb != nullptr) {
        const uint16_t* base = op.pb + (uint64_t)row * op.rs;
        uint4 w[8];
#pragma unroll
        for (int kg = 0; kg < 8; ++kg) {
            if ((uint32_t)kg >= nkg) break;
            const uint32_t k = k0 + kg * 8;
            if (in && vec && k + 8 <= K) {
                w[kg] = __ldg(reinterpret_cast<const uint4*>(base + k));
            } else {
                uint32_t h[8];
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    h[t] = (in && k + t < K) ? (uint32_t)__ldg(base + (uint64_t)(k + t) * op.ks) : 0u;
                w[kg] = make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16),
                                   h[6] | (h[7] << 16));
            }
        }
#pragma unroll
        for (int kg = 0; kg < 8; ++kg) {
            if ((uint32_t)kg >= nkg) break;
            *reinterpret_cast<uint4*>(dst + kg * (16u * 128u)) = w[kg];
        }
        return;
    }
    const float* base = op.p + (uint64_t)row * op.rs;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float4 x[4][2];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t kg = half * 4 + u;
            if (kg >= nkg) break;
            const uint32_t k = k0 + kg * 8;
            if (in && vec && k + 8 <= K) {
                x[u][0] = __ldg(reinterpret_cast<const float4*>(base + k));
                x[u][1] = __ldg(reinterpret_cast<const float4*>(base + k + 4));
            } else {
                float e[8];
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    e[t] = (in && k + t < K) ? __ldg(base + (uint64_t)(k + t) * op.ks) : 0.0f;
                x[u][0] = make_float4(e[0], e[1], e[2], e[3]);
                x[u][1] = make_float4(e[4], e[5], e[6], e[7]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t kg = half * 4 + u;
            if (kg >= nkg) break;
            uint4 w;
            w.x = bf16x2(x[u][0].x, x[u][0].y);
            w.y = bf16x2(x[u][0].z, x[u][0].w);
            w.z = bf16x2(x[u][1].x, x[u][1].y);
            w.w = bf16x2(x[u][1].z, x[u][1].w);
            *reinterpret_cast<uint4*>(dst + kg * (16u * 128u)) = w;
        }
    }
}

// Stages rows [row0, row0+128) x k [k0, k0 + 8*nkg) of a BF16 operand whose rows
// are 16-byte aligned with cp.async (global -> shared, no registers), zero-filling
// rows past op.rows and elements past K. Same layout as stage_operand.
__device__ __forceinline__ void stage_operand_async(uint8_t* tile, const TcOperand& op,
                                                    uint32_t row0, uint32_t k0, uint32_t K,
                                                    uint32_t nkg) {
    const uint32_t r = threadIdx.x;
    const uint32_t crow = row0 + r;
    const bool in = crow < op_rows(op);
    const uint16_t* base = op.pb + (uint64_t)(in ? src_row(op, crow) : 0u) * op.rs;
    const uint32_t dst = smem_u32(tile) + (r >> 3) * 128u + (r & 7u) * 16u;
    for (uint32_t kg = 0; kg < nkg; ++kg) {
        const uint32_t k = k0 + kg * 8;
        const uint32_t bytes = (in && k < K) ? (K - k >= 8 ? 16u : 2u * (K - k)) : 0u;
        const uint16_t* src = base + (k < K ? k : 0);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst + kg * (16u * 128u)),
                     "l"(src), "r"(bytes)
                     : "memory");
    }
}

__device__ __forceinline__ float gelu_f(float x) {
    return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad_f(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

template <int EPI>
__device__ __forceinline__ float epilogue(float acc, uint32_t i, uint32_t j, const TcEpilogue& ep) {
    if (EPI == TC_EPI_SCORE) return __fsub_rn(ep.bias[j], acc);
    if (EPI == TC_EPI_NEG) return -acc;
    if (EPI == TC_EPI_STORE) {
        float v = ep.alpha * acc;
        if (ep.beta != 0.0f) v += ep.beta * ep.out[(uint64_t)i * ep.ld + j];
        return v;
    }
    if (EPI == TC_EPI_BIAS) return acc + ep.bias[j];
    if (EPI == TC_EPI_BIAS_GELU) {
        const float pre = acc + ep.bias[j];
        if (ep.out2) ep.out2[(uint64_t)i * ep.ld + j] = pre;
        return gelu_f(pre);
    }
    // TC_EPI_GELU_BWD: upstream gradient times GELU'(pre-activation)
    return acc * gelu_grad_f(ep.aux[(uint64_t)i * ep.ld_aux + j]);
}

// ASYNC: both operands BF16 with 16-byte aligned rows, staged by cp.async through
// kAsyncStages buffers so that the loads of the next chunks overlap the MMAs.
constexpr uint32_t kAsyncStages = 2;

template <int EPI, bool ASYNC>
__global__ __launch_bounds__(kTcThreads) void k_tc_gemm(TcOperand A, TcOperand B, uint32_t K,
                                                         int a_vec, int b_vec, TcEpilogue ep,
                                                         int* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[kAsyncStages];
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    const uint32_t m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileN;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t a_rows = op_rows(A);
    if (m0 >= a_rows) return;  // a device row count below the launch's rows: nothing here

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        failed = 0;
        for (uint32_t i = 0; i < kAsyncStages; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[i])), "r"(1u));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;

    const uint32_t nch = (K + kChunkK - 1) / kChunkK;
    bool ok = true;
    auto issue_mma = [&](uint32_t c, uint8_t* a_tile, uint8_t* b_tile, uint32_t bar) {
        const uint32_t kc = min(kChunkK, K - c * kChunkK);
        const uint32_t nk16 = (kc + 15) / 16;
        const uint32_t lbo = 16u * 128u, sbo = 128u;
        const uint32_t a_addr = smem_u32(a_tile), b_addr = smem_u32(b_tile);
        for (uint32_t s = 0; s < nk16; ++s) {
            const uint64_t ad = smem_desc(a_addr + s * 2u * lbo, lbo, sbo);
            const uint64_t bd = smem_desc(b_addr + s * 2u * lbo, lbo, sbo);
            const uint32_t accum = (c > 0 || s > 0) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(kInstrDesc), "r"(accum)
                : "memory");
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
            : "memory");
    };
    if (ASYNC) {
        constexpr uint32_t S = kAsyncStages;
        auto stage = [&](uint32_t c) {
            uint8_t* a_tile = smem + (c % S) * kStageBytes;
            uint8_t* b_tile = a_tile + kTileM * kChunkK * 2;
            const uint32_t k0 = c * kChunkK;
            const uint32_t nkg = ((min(kChunkK, K - k0) + 15) / 16) * 2;
            stage_operand_async(a_tile, A, m0, k0, K, nkg);
            stage_operand_async(b_tile, B, n0, k0, K, nkg);
        };
        for (uint32_t c = 0; c + 1 < S; ++c) {
            if (c < nch) stage(c);
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        for (uint32_t c = 0; c < nch; ++c) {
            const uint32_t nc = c + S - 1;
            // the buffer of chunk nc held chunk c-1: its MMAs must be done
            if (nc < nch && c >= 1 &&
                !mbar_wait(smem_u32(&mbar[(c - 1) % S]), ((c - 1) / S) & 1u))
                ok = false;
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            if (nc < nch) stage(nc);
            asm volatile("cp.async.commit_group;" ::: "memory");
            asm volatile("cp.async.wait_group %0;" ::"n"(S - 1) : "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;");
            if (tid == 0) {
                uint8_t* a_tile = smem + (c % S) * kStageBytes;
                issue_mma(c, a_tile, a_tile + kTileM * kChunkK * 2, smem_u32(&mbar[c % S]));
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (nch > 0 && ok) {
            const uint32_t L = nch - 1;
            if (!mbar_wait(smem_u32(&mbar[L % S]), (L / S) & 1u)) ok = false;
        }
    }
    for (uint32_t c = 0; !ASYNC && c < nch; ++c) {
        const uint32_t b = c & 1u;
        if (c >= 2 && !mbar_wait(smem_u32(&mbar[b]), ((c - 2) >> 1) & 1u)) ok = false;
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        const uint32_t k0 = c * kChunkK;
        const uint32_t kc = min(kChunkK, K - k0);
        const uint32_t nk16 = (kc + 15) / 16;
        uint8_t* a_tile = smem + b * kStageBytes;
        uint8_t* b_tile = a_tile + kTileM * kChunkK * 2;
        stage_operand(a_tile, A, m0, k0, K, nk16 * 2, a_vec != 0);
        stage_operand(b_tile, B, n0, k0, K, nk16 * 2, b_vec != 0);
        // generic-proxy writes -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) issue_mma(c, a_tile, b_tile, smem_u32(&mbar[b]));
    }
    // The last commit covers every MMA issued before it.
    if (!ASYNC && nch > 0 && ok) {
        const uint32_t L = nch - 1;
        if (!mbar_wait(smem_u32(&mbar[L & 1u]), (L >> 1) & 1u)) ok = false;
    }
    if (!ok && lane == 0) {
        atomicExch(&failed, 1);
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (!failed && nch > 0) {
        const uint32_t row = m0 + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        const bool vec_out = ((ep.ld & 3u) == 0) &&
                             ((reinterpret_cast<uintptr_t>(ep.out) & 15u) == 0);
        const bool vec_out_b = ((ep.ld & 7u) == 0) &&
                               ((reinterpret_cast<uintptr_t>(ep.out_bf16) & 15u) == 0);
#pragma unroll 1
        for (uint32_t c = 0; c < kTileN / 16; ++c) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                "%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(lane_addr + c * 16));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row >= a_rows) continue;
            const uint32_t col0 = n0 + c * 16;
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
                v[j] = (col0 + j < B.rows) ? epilogue<EPI>(__uint_as_float(r[j]), row, col0 + j, ep)
                                           : 0.0f;
            if (ep.out_bf16 != nullptr) {
                uint16_t* orow = ep.out_bf16 + (uint64_t)row * ep.ld;
                if (vec_out_b && col0 + 16 <= B.rows) {
                    uint4 lo, hi;
                    lo.x = bf16x2(v[0], v[1]);
                    lo.y = bf16x2(v[2], v[3]);
                    lo.z = bf16x2(v[4], v[5]);
                    lo.w = bf16x2(v[6], v[7]);
                    hi.x = bf16x2(v[8], v[9]);
                    hi.y = bf16x2(v[10], v[11]);
                    hi.z = bf16x2(v[12], v[13]);
                    hi.w = bf16x2(v[14], v[15]);
                    *reinterpret_cast<uint4*>(orow + col0) = lo;
                    *reinterpret_cast<uint4*>(orow + col0 + 8) = hi;
                } else {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (col0 + j < B.rows)
                            orow[col0 + j] = __bfloat16_as_ushort(__float2bfloat16_rn(v[j]));
                }
                continue;
            }
            float* orow = ep.out + (uint64_t)row * ep.ld;
            if (vec_out && col0 + 16 <= B.rows) {
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *reinterpret_cast<float4*>(orow + col0 + j) =
                        make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (col0 + j < B.rows) orow[col0 + j] = v[j];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

// ------------------------------------------------------------ persistent TMA form
// For BF16 operands with 16-byte aligned rows and no row gather (the probe's
// inference layers, the coarse and fine screens): a persistent, warp-specialised
// kernel, one CTA per SM looping over 128 x NT output tiles (n fastest, so
// neighbouring CTAs share the A tile in L2):
//   warp 0 (one lane): TMA producer. Per K chunk of 64 it loads the A box
//     (64 x 128) and the B box (64 x NT) into a ring of kTmaStages stages, 128-byte
//     swizzled (cp.async.bulk.tensor, completion on the stage's full mbarrier);
//     rows and K past the operands' ends arrive as zeros.
//   warp 1 (one lane): MMA issuer. tcgen05.mma (M = 128, N = NT, K = 16) per 32-byte
//     step of the swizzle atom, into one of two TMEM accumulators (2 x NT columns);
//     each chunk's MMAs commit to the stage's empty mbarrier, each tile's to the
//     accumulator's full mbarrier.
//   warps 2-5: epilogue. Warp w reads TMEM lanes 32 (w % 4) .. +32 (its rows), 32
//     columns at a time, with tcgen05.ld, applies the epilogue, and writes the
//     32 x 32 block through shared memory so that each store covers one row's 32
//     columns (128 contiguous bytes); then it arrives on the accumulator's empty
//     mbarrier, so the next tile's MMAs overlap this tile's epilogue.
// Every wait is bounded: on expiry the kernel sets *err, the roles stop, the
// producer waits (bounded) for its copies in flight and the TMEM is released.
constexpr int kTmaThreads = 192;
constexpr uint32_t kTmaStages = 4;
constexpr uint32_t kTmaK = 64;  // K per chunk: 64 BF16 = one 128-byte swizzle atom row
constexpr uint32_t kTmaABytes = 128u * kTmaK * 2u;

__host__ __device__ constexpr uint32_t tma_stage_bytes(int nt) {
    return kTmaABytes + (uint32_t)nt * kTmaK * 2u;
}

// K-major, 128-byte swizzled operand tile (8-row x 128-byte atoms, 1024 bytes apart):
// start address, leading byte offset 16 (unused within one atom), stride byte offset
// 1024, the fixed 0b001 at bits 46-48, swizzle mode 2 (128 B) at bits 61-63.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) |
           ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ bool tma_wait(uint32_t bar, uint32_t parity, const volatile int* failed) {
    for (uint32_t it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.b32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 1023u) == 1023u && *failed) return false;
    }
    return false;
}

template <int EPI, int NT>
__global__ __launch_bounds__(kTmaThreads, 1) void k_tc_gemm_tma(
    const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
    uint32_t M, uint32_t N, uint32_t K, TcEpilogue ep, int* __restrict__ err) {
    constexpr uint32_t kStage = tma_stage_bytes(NT);
    constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NT >> 3) << 17) |
                                ((128u >> 4) << 24);
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full[kTmaStages], empty[kTmaStages], tfull[2], tempty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // 128-byte swizzled stages start on 1024-byte boundaries
    const uint32_t sbase = (smem_u32(smem_raw) + 1023u) & ~1023u;
    const uint32_t tiles_n = (N + NT - 1) / NT, tiles = ((M + 127) / 128) * tiles_n;
    const uint32_t nch = (K + kTmaK - 1) / kTmaK;
    if (threadIdx.x == 0) {
        failed = 0;
        for (uint32_t i = 0; i < kTmaStages; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[i])), "r"(1u));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&empty[i])), "r"(1u));
        }
        for (uint32_t i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tfull[i])), "r"(1u));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&tempty[i])), "r"(4u));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base)),
                     "r"(2u * NT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    auto fail = [&]() {
        failed = 1;
        atomicExch(err, 1);
    };

    if (warp == 0) {
        if (lane == 0) {
            // producer
            uint32_t it = 0;
            for (uint32_t t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
                const int32_t m0 = (int32_t)((t / tiles_n) * 128u), n0 = (int32_t)((t % tiles_n) * NT);
                for (uint32_t c = 0; c < nch; ++c, ++it) {
                    const uint32_t st = it % kTmaStages;
                    if (it >= kTmaStages &&
                        !tma_wait(smem_u32(&empty[st]), ((it / kTmaStages) & 1u) ^ 1u, &failed)) {
                        fail();
                        break;
                    }
                    const uint32_t bar = smem_u32(&full[st]);
                    const uint32_t dst = sbase + st * kStage;
                    const int32_t k0 = (int32_t)(c * kTmaK);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                                 "r"(kStage)
                                 : "memory");
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
                        "l"(reinterpret_cast<uint64_t>(&tma_a)), "r"(k0), "r"(m0), "r"(bar)
                        : "memory");
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst + kTmaABytes),
                        "l"(reinterpret_cast<uint64_t>(&tma_b)), "r"(k0), "r"(n0), "r"(bar)
                        : "memory");
                }
            }
            // no copy may land after the CTA: wait (bounded) for the last one of each stage
            for (uint32_t st = 0; st < kTmaStages && st < it; ++st) {
                const uint32_t last = it - 1 - ((it - 1 - st) % kTmaStages);  // last use of stage st
                tma_wait(smem_u32(&full[st]), (last / kTmaStages) & 1u, &failed);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            uint32_t it = 0, lt = 0;
            bool any = false;
            for (uint32_t t = blockIdx.x; t < tiles && !failed; t += gridDim.x, ++lt) {
                const uint32_t acc = lt & 1u, use = lt >> 1;
                if (lt >= 2 && !tma_wait(smem_u32(&tempty[acc]), (use - 1) & 1u, &failed)) {
                    fail();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t d_tmem = tmem + acc * NT;
                bool ok = true;
                for (uint32_t c = 0; c < nch; ++c, ++it) {
                    const uint32_t st = it % kTmaStages;
                    if (!tma_wait(smem_u32(&full[st]), (it / kTmaStages) & 1u, &failed)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t a_addr = sbase + st * kStage, b_addr = a_addr + kTmaABytes;
#pragma unroll
                    for (uint32_t k = 0; k < kTmaK / 16; ++k) {
                        const uint64_t ad = sw128_desc(a_addr + k * 32u);
                        const uint64_t bd = sw128_desc(b_addr + k * 32u);
                        const uint32_t accum = (c > 0 || k > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
                            "l"(ad), "l"(bd), "r"(kIdesc), "r"(accum)
                            : "memory");
                    }
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                            smem_u32(&empty[st]))
                        : "memory");
                }
                if (!ok) {
                    fail();
                    break;
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        smem_u32(&tfull[acc]))
                    : "memory");
                any = true;
            }
            // the last commit covers every MMA issued before it
            if (any) {
                const uint32_t lt_last = lt - 1;
                tma_wait(smem_u32(&tfull[lt_last & 1u]), (lt_last >> 1) & 1u, &failed);
            }
        }
    } else {
        // epilogue: warps 2..5 own TMEM lanes 32 * (warp % 4)
        const uint32_t quarter = (uint32_t)(warp & 3);
        float* stage_out = reinterpret_cast<float*>(smem_raw + (sbase - smem_u32(smem_raw)) +
                                                    kTmaStages * kStage);
        uint32_t lt = 0;
        for (uint32_t t = blockIdx.x; t < tiles; t += gridDim.x, ++lt) {
            const uint32_t acc = lt & 1u, use = lt >> 1;
            if (!tma_wait(smem_u32(&tfull[acc]), use & 1u, &failed)) {
                if (lane == 0) fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t m0 = (t / tiles_n) * 128u, n0 = (t % tiles_n) * NT;
            const uint32_t rbase = m0 + quarter * 32;  // this warp's 32 rows
            const uint32_t row = rbase + lane;
            const uint32_t taddr = tmem + acc * NT + ((quarter * 32u) << 16);
            float* buf = stage_out + (warp - 2) * (32 * 33);  // [32 rows][33]
#pragma unroll 1
            for (uint32_t cg = 0; cg < NT / 32; ++cg) {
                // 32 columns of this warp's rows: lane = row, then through shared memory
                // so that each store writes one row's 32 columns (128 contiguous bytes)
                uint32_t r[32];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                    "%13,%14,%15}, [%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                      "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                      "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                    : "r"(taddr + cg * 32));
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                    "%13,%14,%15}, [%16];"
                    : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                      "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                      "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr + cg * 32 + 16));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                const uint32_t col0 = n0 + cg * 32;
                if (rbase >= M || col0 >= N) continue;  // the whole warp: nothing to store
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    buf[lane * 33 + j] = (row < M && col0 + j < N)
                                             ? epilogue<EPI>(__uint_as_float(r[j]), row, col0 + j, ep)
                                             : 0.0f;
                __syncwarp();
                const uint32_t col = col0 + lane;
                const uint32_t nrows = M - rbase < 32 ? M - rbase : 32;
                if (ep.out_bf16 != nullptr) {
                    for (uint32_t rr = 0; rr < nrows; ++rr)
                        if (col < N)
                            ep.out_bf16[(uint64_t)(rbase + rr) * ep.ld + col] =
                                __bfloat16_as_ushort(__float2bfloat16_rn(buf[rr * 33 + lane]));
                } else {
                    for (uint32_t rr = 0; rr < nrows; ++rr)
                        if (col < N) ep.out[(uint64_t)(rbase + rr) * ep.ld + col] = buf[rr * 33 + lane];
                }
                __syncwarp();
            }
            // this accumulator may take the next tile's MMAs
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[acc]))
                             : "memory");
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2u * NT)
                     : "memory");
    }
}

bool operand_vec(const TcOperand& op) {
    if (op.pb != nullptr)
        return op.ks == 1 && (op.rs & 7u) == 0 && (reinterpret_cast<uintptr_t>(op.pb) & 15u) == 0;
    return op.ks == 1 && (op.rs & 3u) == 0 && (reinterpret_cast<uintptr_t>(op.p) & 15u) == 0;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the
// driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 2-D BF16 tensor map of an operand (rows x K, row stride rs elements), box 64 (K)
// x box_rows, 128-byte swizzle, zero fill past the ends.
bool encode_operand(CUtensorMap* map, const TcOperand& op, uint32_t K, uint32_t box_rows) {
    EncodeTiledFn fn = encode_tiled_fn();
    if (fn == nullptr) return false;
    const cuuint64_t dims[2] = {K, op.rows};
    const cuuint64_t strides[1] = {op.rs * 2ull};
    const cuuint32_t box[2] = {kTmaK, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t*>(op.pb), dims, strides,
              box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int sm_count() {
    static std::mutex mu;
    static int counts[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 0 && dev < 64 && counts[dev] == 0)
        cudaDeviceGetAttribute(&counts[dev], cudaDevAttrMultiProcessorCount, dev);
    return dev >= 0 && dev < 64 && counts[dev] > 0 ? counts[dev] : 1;
}

// The persistent TMA form applies: both operands BF16, rows 16-byte aligned, every
// row read in place (no gather, no device row count).
bool tma_applies(const TcOperand& A, const TcOperand& B, uint32_t K) {
    return A.pb != nullptr && B.pb != nullptr && operand_vec(A) && operand_vec(B) &&
           A.ridx == nullptr && A.rows_dev == nullptr && B.ridx == nullptr &&
           B.rows_dev == nullptr && K >= 8 && (uint64_t)A.rows < (1ull << 31) &&
           (uint64_t)B.rows < (1ull << 31);
}

cudaError_t launch_tc_gemm_tma(const TcOperand& A, const TcOperand& B, uint32_t K,
                               const TcEpilogue& ep, int* err, cudaStream_t stream, bool* done) {
    *done = false;
    // 256-column tiles when they give every SM two or more (the ring and the second
    // accumulator then overlap tiles), else 128-column tiles
    const uint64_t tiles_m = (A.rows + 127) / 128;
    const int nt = B.rows >= 256 && tiles_m * ((B.rows + 255) / 256) >= 2ull * (uint64_t)sm_count()
                       ? 256
                       : 128;
    CUtensorMap ma, mb;
    if (!encode_operand(&ma, A, K, 128) || !encode_operand(&mb, B, K, (uint32_t)nt))
        return cudaSuccess;  // not encodable: the cp.async form runs instead
    const uint64_t tiles = tiles_m * ((B.rows + nt - 1) / nt);
    const unsigned grid = (unsigned)(tiles < (uint64_t)sm_count() ? tiles : (uint64_t)sm_count());
    // stages, the epilogue's 4 x [32][33] staging floats, alignment slack
    const size_t smem = kTmaStages * (size_t)tma_stage_bytes(nt) + 4 * 32 * 33 * 4 + 1024;
#define PGPU_TMA_CASE(M)                                                                    \
    case M:                                                                                 \
        if (nt == 256) {                                                                    \
            ensure_max_dynamic_smem(k_tc_gemm_tma<M, 256>, (int)smem);                      \
            k_tc_gemm_tma<M, 256><<<grid, kTmaThreads, smem, stream>>>(ma, mb, A.rows, B.rows, \
                                                                       K, ep, err);        \
        } else {                                                                            \
            ensure_max_dynamic_smem(k_tc_gemm_tma<M, 128>, (int)smem);                      \
            k_tc_gemm_tma<M, 128><<<grid, kTmaThreads, smem, stream>>>(ma, mb, A.rows, B.rows, \
                                                                       K, ep, err);        \
        }                                                                                   \
        break;
    switch (ep.mode) {
        PGPU_TMA_CASE(TC_EPI_SCORE)
        PGPU_TMA_CASE(TC_EPI_NEG)
        PGPU_TMA_CASE(TC_EPI_STORE)
        PGPU_TMA_CASE(TC_EPI_BIAS)
        PGPU_TMA_CASE(TC_EPI_BIAS_GELU)
        PGPU_TMA_CASE(TC_EPI_GELU_BWD)
        default:
            return cudaErrorInvalidValue;
    }
#undef PGPU_TMA_CASE
    *done = true;
    return cudaGetLastError();
}

}  // namespace

size_t tc_gemm_smem_bytes() { return 2 * (size_t)kStageBytes; }
size_t tc_gemm_async_smem_bytes() { return kAsyncStages * (size_t)kStageBytes; }

cudaError_t launch_tc_gemm(const TcOperand& A, const TcOperand& B, uint32_t K,
                           const TcEpilogue& ep, int* err, cudaStream_t stream) {
    if (A.rows == 0 || B.rows == 0) return cudaSuccess;
    if (K == 0 || (A.p == nullptr && A.pb == nullptr) || (B.p == nullptr && B.pb == nullptr) ||
        (ep.out == nullptr && ep.out_bf16 == nullptr) || err == nullptr)
        return cudaErrorInvalidValue;
    if (ep.out == nullptr && ep.mode == TC_EPI_STORE && ep.beta != 0.0f) return cudaErrorInvalidValue;
    if ((ep.mode == TC_EPI_SCORE || ep.mode == TC_EPI_BIAS || ep.mode == TC_EPI_BIAS_GELU) &&
        ep.bias == nullptr)
        return cudaErrorInvalidValue;
    if (ep.mode == TC_EPI_GELU_BWD && ep.aux == nullptr) return cudaErrorInvalidValue;
    if (tma_applies(A, B, K)) {
        bool done = false;
        const cudaError_t e = launch_tc_gemm_tma(A, B, K, ep, err, stream, &done);
        if (e != cudaSuccess || done) return e;
    }
    const dim3 grid((B.rows + kTileN - 1) / kTileN, (A.rows + kTileM - 1) / kTileM);
    if (grid.y > 65535) return cudaErrorInvalidValue;
    const int av = operand_vec(A) ? 1 : 0, bv = operand_vec(B) ? 1 : 0;
    const bool async = A.pb != nullptr && B.pb != nullptr && av && bv;
    const size_t smem = async ? tc_gemm_async_smem_bytes() : tc_gemm_smem_bytes();
#define PGPU_TC_CASE(M)                                                                        \
    case M:                                                                                    \
        if (async) {                                                                           \
            ensure_max_dynamic_smem(k_tc_gemm<M, true>, (int)smem);                            \
            k_tc_gemm<M, true><<<grid, kTcThreads, smem, stream>>>(A, B, K, av, bv, ep, err); \
        } else {                                                                               \
            ensure_max_dynamic_smem(k_tc_gemm<M, false>, (int)smem);                           \
            k_tc_gemm<M, false><<<grid, kTcThreads, smem, stream>>>(A, B, K, av, bv, ep, err);\
        }                                                                                      \
        break;
    switch (ep.mode) {
        PGPU_TC_CASE(TC_EPI_SCORE)
        PGPU_TC_CASE(TC_EPI_NEG)
        PGPU_TC_CASE(TC_EPI_STORE)
        PGPU_TC_CASE(TC_EPI_BIAS)
        PGPU_TC_CASE(TC_EPI_BIAS_GELU)
        PGPU_TC_CASE(TC_EPI_GELU_BWD)
        default:
            return cudaErrorInvalidValue;
    }
#undef PGPU_TC_CASE
    return cudaGetLastError();
}

}  // namespace pgpu
