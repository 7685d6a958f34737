// pgpu_nearest_center_noalloc: the k-means assignment step without any device
// allocation, for callers that must not allocate GPU memory.
//
// pgpu_nearest_center allocates two small scratch arrays (the squared norms of
// the points and of the centroids) with cudaMallocAsync on every call. Some
// callers cannot allow that: a process whose device memory is handed out by its
// own pool and must not be fragmented, code that runs where the CUDA allocator
// must not be entered, or a tight build loop that should never touch the
// allocator. This entry point keeps the same scratch in a fixed array that is
// part of the library image on the GPU instead. It runs the exact SIMT kernel
// (k_nearest_center: one sequential FP32 dot per pair, strict-< scan, first
// index wins ties), not the tensor-core screen + exact window of
// pgpu_nearest_center. Both compute every candidate distance in the same FP32
// order with the same tie rule, so the results are the same bit for bit; the
// throughput is not: at its size limit this variant is a SIMT contraction of
// 65,536 centroids by 2^20 points, far slower than the tensor-core path.
//
// Costs and rules of the fixed array:
//   * it holds kMaxPoints + kMaxCentroids floats (4.25 MiB), reserved on every
//     GPU that loads this library, until the process exits;
//   * n above kMaxPoints or k above kMaxCentroids is rejected (PGPU_E_LIMIT);
//   * the device address of the array is looked up once per device, on the
//     first call made with that device current (cudaGetSymbolAddress), so that
//     first call must come before any stream capture on that device;
//   * the looked-up address is kept for the life of the process: the library
//     must not be used on a device across cudaDeviceReset (or any other
//     teardown of the device's primary context), which reloads the module and
//     moves the array;
//   * every call on a device shares the array and its contents outlive the call:
//     calls whose work overlaps on the GPU (different streams, or concurrent
//     host threads) race on it and must be serialised by the caller. Nothing in
//     it needs to start at zero: each call overwrites the norms it reads.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>

#include "pgpu_internal.h"

namespace {

constexpr uint64_t kMaxPoints = 1ull << 20;
constexpr uint64_t kMaxCentroids = 1ull << 16;

// [0, kMaxPoints): point norms; [kMaxPoints, +kMaxCentroids): centroid norms.
static __device__ __align__(256) float g_assign_scratch[kMaxPoints + kMaxCentroids];

std::mutex g_scratch_mu;
std::map<int, float*> g_scratch_ptr;  // device ordinal -> device address of the array

}  // namespace

extern "C" int pgpu_nearest_center_noalloc(uint32_t dim, const float* centroids, uint64_t k,
                                           const float* points, uint64_t n, int32_t* assign,
                                           float* distance, void* stream) {
    if (dim == 0 || k == 0 || centroids == nullptr || points == nullptr || assign == nullptr ||
        distance == nullptr)
        return pgpu::set_last_error(PGPU_E_INVALID, "invalid argument");
    if (n > kMaxPoints || k > kMaxCentroids)
        return pgpu::set_last_error(
            PGPU_E_LIMIT, "pgpu_nearest_center_noalloc takes at most " +
                              std::to_string(kMaxPoints) + " points and " +
                              std::to_string(kMaxCentroids) + " centroids per call; got " +
                              std::to_string(n) + " and " + std::to_string(k));
    if (n == 0) return PGPU_OK;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return pgpu::set_last_error(PGPU_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    float* scratch = nullptr;
    {
        std::lock_guard<std::mutex> g(g_scratch_mu);
        auto it = g_scratch_ptr.find(dev);
        if (it == g_scratch_ptr.end()) {
            // once per device, with that device current
            e = cudaGetSymbolAddress((void**)&scratch, g_assign_scratch);
            if (e != cudaSuccess)
                return pgpu::set_last_error(
                    PGPU_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = scratch;
        } else {
            scratch = it->second;
        }
    }
    e = pgpu::launch_nearest_center_scratch(dim, centroids, k, points, n, assign, distance,
                                            scratch, scratch + kMaxPoints, (cudaStream_t)stream);
    if (e != cudaSuccess)
        return pgpu::set_last_error(PGPU_E_CUDA,
                                    std::string("nearest_center_noalloc: ") + cudaGetErrorString(e));
    return PGPU_OK;
}
