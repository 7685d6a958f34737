// Device-resident index construction: copies the host layout to HBM, permutes
// the original vectors into memory order on the GPU, and computes the per-cell
// constants of HierarchicalClusterIndex::read_coodbooks
// (puck/hierarchical_cluster/hierarchical_cluster_index.cpp:278-320) and
// PuckIndex::convert_local_to_memory_idx (puck/puck/puck_index.cpp:284-305).
#include <cuda_bf16.h>

#include <cfloat>
#include <cmath>

#include "pgpu_internal.h"

namespace pgpu {
namespace {

__global__ void k_gather_rows(const float* __restrict__ src, const uint32_t* __restrict__ rows,
                              uint64_t n, uint32_t d, float* __restrict__ dst) {
    // one warp per destination row
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const float* s = src + (uint64_t)rows[w] * d;
    float* t = dst + w * d;
    for (uint32_t k = lane; k < d; k += 32) t[k] = s[k];
}

// BF16 copy of each row (round to nearest even) and |x| rounded up.
__global__ void k_bf16_rows(const float* __restrict__ src, uint64_t n, uint32_t d,
                            uint16_t* __restrict__ dst, float* __restrict__ absn) {
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const float* s = src + w * d;
    uint16_t* t = dst + w * d;
    float acc = 0.0f;
    for (uint32_t k = lane; k < d; k += 32) {
        const float x = s[k];
        t[k] = __bfloat16_as_ushort(__float2bfloat16_rn(x));
        acc += x * x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) absn[w] = sqrtf(acc) * (1.0f + 1e-5f) + 1e-30f;
}

template <class T>
cudaError_t dev_copy(T** dst, const T* src, uint64_t count, uint64_t* bytes) {
    const size_t sz = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc((void**)dst, sz);
    if (e != cudaSuccess) return e;
    *bytes += sz;
    if (count) e = cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
    return e;
}

template <class T>
cudaError_t dev_alloc(T** dst, uint64_t count, uint64_t* bytes) {
    const size_t sz = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc((void**)dst, sz);
    if (e == cudaSuccess) *bytes += sz;
    return e;
}

}  // namespace

// base: the original vectors in input order (host).
int upload_index_with_base(const HostIndex& h, const float* base, DeviceIndex* ix,
                           std::string* err) {
    *ix = DeviceIndex();
    ix->d = h.d;
    ix->n = h.n;
    ix->C = h.C;
    ix->F = h.F;
    ix->nsq = h.nsq;
    ix->lsq = h.lsq;
    ix->whether_norm = h.whether_norm;
    ix->ip2cos = h.ip2cos;
    ix->qdim = h.d - (uint32_t)h.ip2cos;
    ix->code_stride = h.code_stride;
    {
        // largest codeword norm: bounds every lookup-table entry (precision form)
        double mx = 0.0;
        for (uint64_t e = 0; e + h.lsq <= h.codebook.size(); e += h.lsq) {
            double s2 = 0.0;
            for (uint32_t t = 0; t < h.lsq; ++t) s2 += (double)h.codebook[e + t] * h.codebook[e + t];
            if (s2 > mx) mx = s2;
        }
        ix->codebook_max = (float)(std::sqrt(mx) * (1.0 + 1e-6));
    }
    uint64_t bytes = 0;
    const uint64_t cells = (uint64_t)h.C * h.F;
    cudaError_t e = cudaSuccess;
    float* fine_half = nullptr;
    float* base_dev = nullptr;
#define PGPU_TRY(x)              \
    do {                         \
        e = (x);                 \
        if (e != cudaSuccess) goto fail; \
    } while (0)
    PGPU_TRY(dev_copy(&ix->coarse, h.coarse.data(), h.coarse.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->fine, h.fine.data(), h.fine.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->codebook, h.codebook.data(), h.codebook.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->cell_start, h.cell_start.data(), h.cell_start.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->mem2local, h.mem2local.data(), h.mem2local.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->rec_fine, h.rec_fine.data(), h.rec_fine.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->offsets, h.offsets_mem.data(), h.offsets_mem.size(), &bytes));
    PGPU_TRY(dev_copy(&ix->codes, h.codes_mem.data(), h.codes_mem.size(), &bytes));
    PGPU_TRY(dev_alloc(&ix->coarse_norms, h.C, &bytes));
    PGPU_TRY(dev_alloc(&ix->coarse_abs, h.C, &bytes));
    PGPU_TRY(dev_alloc(&ix->coarse_bf16, (uint64_t)h.C * h.d, &bytes));
    PGPU_TRY(dev_alloc(&ix->fine_bf16, (uint64_t)h.F * h.d, &bytes));
    PGPU_TRY(dev_alloc(&ix->stationary, cells, &bytes));
    PGPU_TRY(dev_alloc(&ix->stat_sorted, cells, &bytes));
    PGPU_TRY(dev_alloc(&ix->stat_fine, cells, &bytes));
    PGPU_TRY(dev_alloc(&ix->min_dist_offset, h.C, &bytes));
    if (base != nullptr) PGPU_TRY(dev_alloc(&ix->feat, (uint64_t)h.n * h.d, &bytes));
    if (h.pq_nsq) {
        ix->pq_nsq = h.pq_nsq;
        ix->pq_lsq = h.pq_lsq;
        ix->pq_code_stride = h.pq_code_stride;
        PGPU_TRY(dev_copy(&ix->pq_codebook, h.pq_codebook.data(), h.pq_codebook.size(), &bytes));
        PGPU_TRY(dev_copy(&ix->pq_offsets, h.pq_offsets_mem.data(), h.pq_offsets_mem.size(), &bytes));
        PGPU_TRY(dev_copy(&ix->pq_codes, h.pq_codes_mem.data(), h.pq_codes_mem.size(), &bytes));
    }
    PGPU_TRY(cudaMalloc(&fine_half, sizeof(float) * h.F));
    if (base != nullptr) {
        PGPU_TRY(cudaMalloc(&base_dev, sizeof(float) * ((uint64_t)h.n * h.d + 1)));
        if (h.n)
            PGPU_TRY(cudaMemcpy(base_dev, base, sizeof(float) * (uint64_t)h.n * h.d,
                                cudaMemcpyHostToDevice));
    }
    if (h.n && base != nullptr) {
        const uint64_t threads = (uint64_t)h.n * 32;
        k_gather_rows<<<(unsigned)((threads + 255) / 256), 256>>>(base_dev, ix->mem2local, h.n, h.d,
                                                                  ix->feat);
        PGPU_TRY(cudaGetLastError());
    }
    PGPU_TRY(launch_half_norms(ix->coarse, h.C, h.d, ix->coarse_norms, 0));
    PGPU_TRY(launch_abs_from_half_norms(ix->coarse_norms, h.C, ix->coarse_abs, 0));
    PGPU_TRY(launch_to_bf16(ix->coarse, (uint64_t)h.C * h.d, ix->coarse_bf16, 0));
    PGPU_TRY(launch_to_bf16(ix->fine, (uint64_t)h.F * h.d, ix->fine_bf16, 0));
    PGPU_TRY(launch_half_norms(ix->fine, h.F, h.d, fine_half, 0));
    PGPU_TRY(launch_stationary(ix->coarse, h.C, ix->fine, h.F, h.d, fine_half, ix->stationary, 0));
    PGPU_TRY(launch_cell_constants(ix->stationary, ix->cell_start, ix->min_dist_offset, h.C, h.F,
                                   std::sqrt(FLT_MAX), 0));
    // per coarse cluster, its cells in ascending stationary order (after the
    // empty-cell fix-up): the enumeration order of the walk kernel
    PGPU_TRY(launch_topsort(ix->stationary, h.C, h.F, h.F, h.F, ix->stat_sorted, ix->stat_fine, 0));
    PGPU_TRY(cudaDeviceSynchronize());
    cudaFree(fine_half);
    cudaFree(base_dev);
    ix->bytes = bytes;
    return PGPU_OK;
fail:
#undef PGPU_TRY
    if (fine_half) cudaFree(fine_half);
    if (base_dev) cudaFree(base_dev);
    *err = std::string("CUDA error during index upload: ") + cudaGetErrorString(e);
    free_device_index(ix);
    return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
}

cudaError_t launch_bf16_rows(const float* x, uint64_t rows, uint32_t d, uint16_t* out,
                             float* absn, cudaStream_t stream) {
    if (rows == 0) return cudaSuccess;
    const uint64_t threads = rows * 32;
    k_bf16_rows<<<(unsigned)((threads + 255) / 256), 256, 0, stream>>>(x, rows, d, out, absn);
    return cudaGetLastError();
}

int ensure_bf16_features(DeviceIndex* ix, std::string* err) {
    if (ix->feat_bf16 != nullptr) return PGPU_OK;
    uint64_t bytes = 0;
    // rows for the inserted points too (realtime: n + ins_cap)
    const uint64_t rows = (uint64_t)ix->n + ix->ins_cap, used = (uint64_t)ix->n + ix->ins_n;
    cudaError_t e = dev_alloc(&ix->feat_bf16, rows * ix->d, &bytes);
    if (e == cudaSuccess) e = dev_alloc(&ix->feat_abs, rows, &bytes);
    if (e == cudaSuccess) e = launch_bf16_rows(ix->feat, used, ix->d, ix->feat_bf16, ix->feat_abs, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        if (ix->feat_bf16) cudaFree(ix->feat_bf16);
        if (ix->feat_abs) cudaFree(ix->feat_abs);
        ix->feat_bf16 = nullptr;
        ix->feat_abs = nullptr;
        *err = std::string("BF16 feature copy: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
    }
    ix->bytes += bytes;
    return PGPU_OK;
}

// One thread per record: its rotated codes (byte s = code of subspace
// (s + (r & 31)) mod nsq) as 8-byte granules of the interleaved layout, its filter
// offset and its fine id.
__global__ void k_interleave_codes(const uint8_t* __restrict__ codes, uint32_t stride,
                                   const float* __restrict__ offsets,
                                   const uint16_t* __restrict__ rec_fine, uint32_t nsq,
                                   uint64_t r0, uint64_t rows, uint8_t* __restrict__ il) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const uint64_t r = r0 + i;
    const uint32_t rho = (uint32_t)(r & 31) % nsq;
    const uint8_t* src = codes + r * stride;
    const uint32_t ng = il_record_bytes(nsq) / 8;
    for (uint32_t g = 0; g < ng; ++g) {
        unsigned long long v = 0;
        for (uint32_t b = 0; b < 8; ++b) {
            const uint32_t s = g * 8 + b;
            if (s < nsq) {
                const uint32_t m = s + rho < nsq ? s + rho : s + rho - nsq;
                v |= (unsigned long long)src[m] << (8 * b);
            }
        }
        *reinterpret_cast<unsigned long long*>(il + il_granule_offset(r, g, nsq)) = v;
    }
    *reinterpret_cast<float*>(il + il_offset_offset(r, nsq)) = offsets[r];
    *reinterpret_cast<uint16_t*>(il + il_fine_offset(r, nsq)) = rec_fine[r];
}

cudaError_t launch_interleave_codes(const DeviceIndex& ix, uint64_t r0, uint64_t rows,
                                    cudaStream_t stream) {
    if (rows == 0) return cudaSuccess;
    k_interleave_codes<<<(unsigned)((rows + 255) / 256), 256, 0, stream>>>(
        ix.codes, ix.code_stride, ix.offsets, ix.rec_fine, ix.nsq, r0, rows, ix.codes_il);
    return cudaGetLastError();
}

int ensure_interleaved_codes(DeviceIndex* ix, std::string* err) {
    if (ix->codes_il != nullptr || !il_applies(ix->nsq) || ix->n == 0) return PGPU_OK;
    uint64_t bytes = 0;
    // rows for the inserted points too (realtime: n + ins_cap)
    const uint64_t rows = (uint64_t)ix->n + ix->ins_cap, used = (uint64_t)ix->n + ix->ins_n;
    cudaError_t e = dev_alloc(&ix->codes_il, il_bytes(rows, ix->nsq), &bytes);
    if (e == cudaSuccess) e = cudaMemset(ix->codes_il, 0, il_bytes(rows, ix->nsq));
    if (e == cudaSuccess)
        e = launch_interleave_codes(*ix, 0, used, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        if (ix->codes_il) cudaFree(ix->codes_il);
        ix->codes_il = nullptr;
        *err = std::string("interleaved code copy: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PGPU_E_NOMEM : PGPU_E_CUDA;
    }
    ix->bytes += bytes;
    return PGPU_OK;
}

}  // namespace pgpu
