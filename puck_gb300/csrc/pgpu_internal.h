// Internal types shared by the host loader, the C ABI and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/puck_gb300.h"

namespace pgpu {

// 0x7f7f7f7f: the fill value of Puck's MaxHeap (max_heap.cpp:32).
constexpr uint32_t kHeapSentinelBits = 0x7f7f7f7fu;
constexpr uint32_t kNoLabel = 0xFFFFFFFFu;

// Limits of the exact-mode kernels (checked on the host; PGPU_E_LIMIT beyond).
constexpr uint32_t kMaxClusters = 8192;   // coarse or fine count: sorted in shared memory
constexpr uint32_t kMaxFilterNsq = 64;    // LUT of nsq*256 floats in shared memory
constexpr uint32_t kMaxFilterTopk = 4096; // filter heap in shared memory
constexpr uint32_t kMaxDim = 1024;
constexpr uint32_t kMaxPqNsq = 192;       // PQ table of pq_nsq*256 floats in shared memory
constexpr int kNumWalkCounters = 14;  // see the counter enum in walk_scan.cu
// Counter slot 11: queries whose coarse top-P fell back from the tensor-core
// window to the full exact recompute (ties at the cut, or a wide window).
constexpr int kCounterWindowFallbacks = 11;
// Slots 12, 13: queries that kept the fixed-count selection because the probe was
// not confident, and clusters chosen by the probe for the others.
constexpr int kCounterProbeFallbacks = 12;
constexpr int kCounterProbeClusters = 13;

// Probe network parameters: views into one contiguous FP32 block laid out
// W1 [h][d], b1 [h], W2 [h][h], b2 [h], W3 [C][h], b3 [C].
struct ProbeNet {
    uint32_t d = 0, h = 0, C = 0;
    float *W1 = nullptr, *b1 = nullptr, *W2 = nullptr, *b2 = nullptr, *W3 = nullptr, *b3 = nullptr;
    // BF16 copies of the weight matrices for inference (refreshed after every update)
    uint16_t *W1b = nullptr, *W2b = nullptr, *W3b = nullptr;
    uint64_t param_count() const;
    void bind(float* base) {
        W1 = base;
        b1 = W1 + (uint64_t)h * d;
        W2 = b1 + h;
        b2 = W2 + (uint64_t)h * h;
        W3 = b2 + h;
        b3 = W3 + (uint64_t)C * h;
    }
};
// Activations and gradients of one training batch (rows <= cap).
struct ProbeWork {
    uint32_t cap = 0;
    float *H1 = nullptr, *Z1 = nullptr, *H2 = nullptr, *Z2 = nullptr, *Z = nullptr, *dZ = nullptr,
          *dH2 = nullptr, *dH1 = nullptr;
};

// Device-resident index. Point arrays are in Puck's "memory order": sorted by
// (cell id, filter offset, input id), so every coarse cluster is one
// contiguous range and points inside a cell ascend by filter offset
// (puck/puck/puck_index.cpp:248-282).
struct DeviceIndex {
    uint32_t d = 0, n = 0, C = 0, F = 0, nsq = 0, lsq = 0;
    int whether_norm = 0;
    int ip2cos = 0;     // 1: the caller's queries have qdim = d - 1 values, a 0 is appended
    uint32_t qdim = 0;  // floats per caller query
    uint32_t code_stride = 0;     // bytes per code row (nsq rounded up to 4)
    float* coarse = nullptr;      // [C][d]
    float* fine = nullptr;        // [F][d]
    float* coarse_norms = nullptr;// [C]  0.5*|c|^2
    float* coarse_abs = nullptr;  // [C]  |c| rounded up (error bound of the tensor-core screen)
    uint16_t* coarse_bf16 = nullptr;  // [C][d] BF16 copy: operand of the tensor-core screen
    uint16_t* fine_bf16 = nullptr;    // [F][d]
    float* stationary = nullptr;  // [C][F] 0.5*|f|^2 + f.c ; sqrt(FLT_MAX) for empty cells
    float* stat_sorted = nullptr; // [C][F] each coarse row of stationary, ascending
    uint32_t* stat_fine = nullptr;// [C][F] fine id of each stat_sorted entry
    uint32_t* cell_start = nullptr; // [C*F + 1]
    float* min_dist_offset = nullptr; // [C]
    uint32_t* mem2local = nullptr;  // [n]
    uint16_t* rec_fine = nullptr;   // [n] fine id of the cell each record belongs to
    float* offsets = nullptr;       // [n] filter offset per point
    uint8_t* codes = nullptr;       // [n][code_stride]
    uint8_t* codes_il = nullptr;    // scan-mode copy of the records (codes, offset, fine id)
                                    // interleaved by blocks of 32, each record's codes
                                    // rotated by its lane (il_* below; made on first use)
    // realtime inserts (realtime.cu): per-record arrays hold n + ins_cap rows, inserted
    // point i at row (memory id) n + i
    uint32_t ins_cap = 0, ins_n = 0;
    int32_t* ins_head = nullptr;      // [C*F] newest insert id of each cell, -1: none
    int32_t* ins_next = nullptr;      // [ins_cap] next older insert id of the same cell, -1
    uint32_t* ins_cl_start = nullptr; // [C+1] each coarse cluster's range in ins_cl_ids
    uint32_t* ins_cl_ids = nullptr;   // [ins_cap] inserted memory ids grouped by coarse cluster
    float* feat = nullptr;          // [n][d] original vectors
    uint16_t* feat_bf16 = nullptr;  // [n][d] BF16 copy (precision form; made on first use)
    float* feat_abs = nullptr;      // [n] |x| rounded up (error bound of the BF16 screen)
    float codebook_max = 0.0f;      // largest |codeword| (FP16 table scale bound)
    // second-level PQ (whether_pq): the rerank's table and records; feat is null
    uint32_t pq_nsq = 0, pq_lsq = 0, pq_code_stride = 0;
    float* pq_codebook = nullptr;   // [pq_nsq][256][pq_lsq]
    float* pq_offsets = nullptr;    // [n] memory order
    uint8_t* pq_codes = nullptr;    // [n][pq_code_stride] memory order
    float* codebook = nullptr;      // [nsq][256][lsq]
    uint64_t bytes = 0;
};

// Per-pass scratch (sized for max_batch queries).
// Interleaved record copy of the scan (DeviceIndex::codes_il), made when nsq is a
// multiple of 4 and at most 32. Records are grouped in blocks of 32 by memory id
// (block b = r >> 5, lane l = r & 31). A block is il_block_bytes long and holds
//   * the codes, G = il_record_bytes bytes a record as 8-byte granules: granule g
//     of lane l at g * 256 + 8 * l, so one warp reads a block's granule g as one
//     256-byte line;
//   * the 32 filter offsets (float) at 32 * G, and the 32 fine ids (uint16) at
//     32 * G + 128.
// Byte s < nsq of a record's codes is the code of subspace (s + l) mod nsq (bytes
// past nsq are 0): at lookup step s the 32 lanes of a warp read 32 consecutive
// table columns. A block is a multiple of 16 bytes, so a run of blocks is one bulk
// copy.
__host__ __device__ inline bool il_applies(uint32_t nsq) { return nsq % 4 == 0 && nsq <= 32 && nsq > 0; }
__host__ __device__ inline uint32_t il_record_bytes(uint32_t nsq) { return (nsq + 7u) & ~7u; }
__host__ __device__ inline uint32_t il_block_bytes(uint32_t nsq) {
    return 32u * il_record_bytes(nsq) + 128u + 64u;
}
__host__ __device__ inline uint64_t il_bytes(uint64_t rows, uint32_t nsq) {
    return (rows + 31) / 32 * il_block_bytes(nsq);
}
__host__ __device__ inline uint64_t il_granule_offset(uint64_t r, uint32_t g, uint32_t nsq) {
    return (r >> 5) * il_block_bytes(nsq) + g * 256u + 8u * (uint32_t)(r & 31);
}
__host__ __device__ inline uint64_t il_offset_offset(uint64_t r, uint32_t nsq) {
    return (r >> 5) * il_block_bytes(nsq) + 32u * il_record_bytes(nsq) + 4u * (uint32_t)(r & 31);
}
__host__ __device__ inline uint64_t il_fine_offset(uint64_t r, uint32_t nsq) {
    return (r >> 5) * il_block_bytes(nsq) + 32u * il_record_bytes(nsq) + 128u +
           2u * (uint32_t)(r & 31);
}
// Interleaved records of rows [r0, r0 + rows) from the row-major codes, the filter
// offsets and the fine ids.
cudaError_t launch_interleave_codes(const DeviceIndex& ix, uint64_t r0, uint64_t rows,
                                    cudaStream_t stream);

// Split scan: per query, the histogram cut of its records' distances (k_scan_score).
struct SplitCut {
    float lo, scale;  // bin(t) = clamp(trunc((t - lo) * scale), 0, 4095)
    uint32_t bin;     // the highest bin kept: at least filter_topk records lie at or below it
    uint32_t n;       // records written to tbuf
};

struct Scratch {
    uint32_t cap = 0;
    float* q = nullptr;        // [B][d] normalised queries
    uint16_t* qb = nullptr;    // [B][d] the same, BF16 (tensor-core operand)
    float* qnorm = nullptr;    // [B]
    int32_t* status = nullptr; // [B]
    float* dots = nullptr;     // [B][max(C,F)]
    float* cdist = nullptr;    // [B][P]
    uint32_t* ctag = nullptr;  // [B][P]
    float* fdist = nullptr;    // [B][F]
    uint32_t* ftag = nullptr;  // [B][F]
    float* hdist = nullptr;    // [B][T] filter heap values
    uint32_t* htag = nullptr;  // [B][T] filter heap memory ids
    uint32_t* hcnt = nullptr;  // [B]
    unsigned long long* counters = nullptr; // [kNumWalkCounters] walk diagnostics
    int* tc_err = nullptr;     // set by a tensor-core contraction or table copy whose wait expired
    uint16_t* ph1 = nullptr;   // probe hidden activations [B][h], BF16 (with a probe attached)
    uint16_t* ph2 = nullptr;
    int32_t* pconf = nullptr;  // [B] 1 where the probe chose the clusters (null: no probe)
    float* pz = nullptr;       // [B][C] probe scores
    uint32_t* order = nullptr; // scan mode: [B] queries in launch order (longest scans first)
    uint32_t* ulist = nullptr;  // with a probe: [B] queries left to the fixed-count selection
    uint32_t* ucount = nullptr; // their number (device)
    uint8_t* wbucket = nullptr; // scan mode: [B] work bucket of each query
    // split scan (interleaved layout): every scanned record's distance, per query at
    // qoff; qflag 1 where the split scan answers the query
    float* tbuf = nullptr;      // [tcap]
    uint64_t tcap = 0;
    uint32_t* qcnt = nullptr;   // [B] records of each query
    uint32_t* qoff = nullptr;   // [B]
    uint32_t* qflag = nullptr;  // [B]
    SplitCut* cut = nullptr;    // [B]
    uint32_t Pfix = 0;         // fixed coarse count (<= P when a probe widens the slots)
    uint32_t P = 0, T = 0;
    uint64_t bytes = 0;
};

struct SearchConfig {
    uint32_t P = 200, T = 1100, topk_max = 100;
    double radius_rate = 1.0;
    int mode = PGPU_MODE_EXACT;
    int precision = PGPU_PRECISION_FP32;
    uint32_t margin = 0;  // BF16: extra filter candidates
    const ProbeNet* probe = nullptr;  // learned probe (scan mode), not owned
    float probe_mass = 0.9f;
    uint32_t probe_max = 0;
    // coarse slots per query: the fixed count, or the probe's cap when larger
    uint32_t coarse_slots(uint32_t C) const {
        uint32_t p = P < C ? P : C;
        if (probe && probe_max > p) p = probe_max;
        return p;
    }
    // filter candidates kept per query
    uint32_t filter_keep() const { return T + (precision == PGPU_PRECISION_BF16 ? margin : 0); }
};

// Kernel launchers (kernels_search.cu). All enqueue on `stream`.
cudaError_t launch_prep_queries(const DeviceIndex& ix, const float* q_in, uint32_t n, Scratch& s,
                                cudaStream_t stream);
cudaError_t launch_centroid_scores(const float* queries, uint32_t nq, const float* cents,
                                   uint32_t nc, uint32_t d, const float* bias, bool negate,
                                   float* out, uint32_t ld_out, cudaStream_t stream);
cudaError_t launch_topsort(const float* vals, uint32_t nrows, uint32_t L, uint32_t ld_vals,
                           uint32_t K, float* out_val, uint32_t* out_idx, cudaStream_t stream);
cudaError_t launch_walk_scan(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t n,
                             Scratch& s, cudaStream_t stream);
cudaError_t launch_rerank(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t n,
                          uint32_t topk, const Scratch& s, float* out_dist, uint32_t* out_ids,
                          int32_t* out_status, cudaStream_t stream);
cudaError_t launch_nearest_center(uint32_t dim, const float* cents, uint64_t k, const float* x,
                                  uint64_t n, int32_t* assign, float* dis, cudaStream_t stream);
// nearest_center with caller-provided scratch for the point and centroid norms
// (xnorm: n floats, cnorm: k floats); launches the same kernels as launch_nearest_center.
cudaError_t launch_nearest_center_scratch(uint32_t dim, const float* cents, uint64_t k,
                                          const float* x, uint64_t n, int32_t* assign, float* dis,
                                          float* xnorm, float* cnorm, cudaStream_t stream);
// The build's exact nearest-cell assignment (cell_assign.cu). stat: the [C][F]
// stationary terms to use (an index's live ones), or null to compute them.
cudaError_t launch_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C,
                                       const float* fine, uint32_t F, const float* x, uint64_t n,
                                       uint32_t* cell, float* dist, cudaStream_t stream,
                                       const float* stat = nullptr);
// BF16 copy of rows and |x| rounded up (the precision form's screen operand).
cudaError_t launch_bf16_rows(const float* x, uint64_t rows, uint32_t d, uint16_t* out,
                             float* absn, cudaStream_t stream);
// Host mirrors of the realtime lists (realtime.cu).
struct RealtimeHost {
    std::vector<int32_t> head;     // [C*F]
    std::vector<int32_t> next;     // [ins_n]
    std::vector<uint32_t> cluster; // [ins_n] coarse cluster of each insert
    std::vector<uint32_t> cnt;     // [C*F] base + inserted points of each cell
};
// RealtimeInsertPuckIndex::init: room for cap inserted points (synchronous).
int realtime_open(DeviceIndex* ix, RealtimeHost* rh, uint32_t cap, std::string* err);
// Inserts the rows of x (DEVICE, [m][d], normalised as the index wants) whose ok[i]
// (host) is set, in order; ids[i] = n + insert id, or -1. Synchronous.
int realtime_insert(DeviceIndex* ix, RealtimeHost* rh, uint32_t m, const float* x,
                    const int32_t* ok, int64_t* ids, cudaStream_t st, std::string* err);
cudaError_t launch_gather_u32(const uint32_t* idx, uint64_t n, const uint32_t* table,
                              uint32_t* out, cudaStream_t stream);
// Records `msg` as the calling thread's last error (pgpu_last_error) and returns `code`.
int set_last_error(int code, const std::string& msg);

// Raises a kernel's dynamic shared-memory limit to `bytes` on the calling thread's
// current device, once per (kernel, device, bytes). Function attributes belong to a
// device's context, so a process that searches on several GPUs sets them on each one.
// Thread-safe.
void ensure_max_dynamic_smem(const void* kernel, int bytes);
template <class K>
inline void ensure_max_dynamic_smem(K* kernel, int bytes) {
    ensure_max_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}
cudaError_t launch_topsort_status(const float* vals, uint32_t nrows, uint32_t L, uint32_t ld_vals,
                                  uint32_t K, float* out_val, uint32_t* out_idx,
                                  const int32_t* status, cudaStream_t stream);
cudaError_t launch_stationary(const float* coarse, uint32_t C, const float* fine, uint32_t F,
                              uint32_t d, const float* fine_half_norms, float* stationary,
                              cudaStream_t stream);
cudaError_t launch_half_norms(const float* X, uint32_t rows, uint32_t d, float* out,
                              cudaStream_t stream);
cudaError_t launch_to_bf16(const float* x, uint64_t n, uint16_t* y, cudaStream_t stream);
cudaError_t launch_cell_constants(float* stationary, const uint32_t* cell_start, float* mdo,
                                  uint32_t C, uint32_t F, float empty_value, cudaStream_t stream);
size_t walk_smem_bytes(const DeviceIndex& ix, uint32_t T);
size_t scan_smem_bytes(const DeviceIndex& ix, uint32_t T);
uint32_t scan_max_filter_topk();
// Scan mode: the blocks' launch order (longest scans first), then the scan itself.
cudaError_t launch_scan_order(const DeviceIndex& ix, uint32_t n, Scratch& s, cudaStream_t stream);
// The scan (scan mode), in three parts timed as stages 4-6: launch_scan_prepare
// (the split scan's record counts and buffer offsets; nothing otherwise),
// launch_scan_records (k_scan_score, or the fused kernel when the split scan does
// not apply), launch_scan_finish (the fused kernel for the queries the split scan
// left).
cudaError_t launch_scan_prepare(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                                cudaStream_t stream);
cudaError_t launch_scan_records(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                                cudaStream_t stream);
cudaError_t launch_scan_finish(const DeviceIndex& ix, uint32_t n, Scratch& s, bool half_lut,
                               cudaStream_t stream);
size_t scan_smem_bytes_half(const DeviceIndex& ix, uint32_t T);
// The split scan runs (k_split_counts, k_split_offsets, k_scan_score before the fused
// kernel) when the index has the interleaved layout, its block fits shared memory
// (scan_split_possible: the cell terms of F fine clusters, filter_topk below the
// pick's 8192 keys) and the scratch holds its distance buffer; otherwise the fused
// kernel answers every query.
bool scan_split_possible(const DeviceIndex& ix, uint32_t T);
bool scan_split_applies(const DeviceIndex& ix, const Scratch& s);
// BF16 copy of the vectors and their norms (precision form), synchronous.
int ensure_bf16_features(DeviceIndex* ix, std::string* err);
// The precision form's rotated copy of the filter codes (nsq a multiple of 4, at
// most 32; otherwise nothing is made), synchronous.
int ensure_interleaved_codes(DeviceIndex* ix, std::string* err);
size_t rerank_screen_smem_bytes(const DeviceIndex& ix, uint32_t T, uint32_t topk);
cudaError_t launch_rerank_screen(const DeviceIndex& ix, uint32_t n, uint32_t topk, const Scratch& s,
                                 float* out_dist, uint32_t* out_ids, int32_t* out_status,
                                 cudaStream_t stream);
size_t rerank_smem_bytes(const DeviceIndex& ix, uint32_t T, uint32_t topk);

// BF16 tensor-core contraction (tc_gemm.cu): out = epilogue(sum_k A(i,k) B(j,k)).
// A(i,k) = p[i*rs + k*ks] for i < rows; B likewise.
struct TcOperand {
    const float* p;
    uint64_t rs, ks;
    uint32_t rows;
    const uint16_t* pb = nullptr;  // BF16 operand instead of p (same strides, in elements)
    const uint32_t* ridx = nullptr;     // row i reads source row ridx[i] (A only)
    const uint32_t* rows_dev = nullptr; // device count of rows (<= rows) (A only)
};
enum TcEpi {
    TC_EPI_SCORE = 0,     // bias[j] - acc
    TC_EPI_NEG = 1,       // -acc
    TC_EPI_STORE = 2,     // alpha*acc + beta*out
    TC_EPI_BIAS = 3,      // acc + bias[j]
    TC_EPI_BIAS_GELU = 4, // out2 = acc + bias[j]; out = GELU(out2)
    TC_EPI_GELU_BWD = 5,  // acc * GELU'(aux[i][j])
};
struct TcEpilogue {
    int mode;
    float* out;             // FP32 output, or
    uint16_t* out_bf16;     // BF16 output (when set, out is not written)
    uint64_t ld;
    const float* bias;
    const float* aux;
    uint64_t ld_aux;
    float* out2;
    float alpha, beta;
};
size_t tc_gemm_smem_bytes();
cudaError_t launch_tc_gemm(const TcOperand& A, const TcOperand& B, uint32_t K,
                           const TcEpilogue& ep, int* err, cudaStream_t stream);
// Exact selections over a tensor-core screen (tc_select.cu).
size_t window_smem_bytes(uint32_t C, uint32_t d);
cudaError_t launch_abs_from_half_norms(const float* half_norms, uint32_t n, float* out,
                                       cudaStream_t stream);
cudaError_t launch_coarse_tc(const DeviceIndex& ix, uint32_t n, Scratch& s, cudaStream_t stream);
cudaError_t launch_coarse_window(const DeviceIndex& ix, uint32_t n, Scratch& s,
                                 cudaStream_t stream);
cudaError_t launch_nearest_center_tc(uint32_t dim, const float* cents, uint64_t k, const float* x,
                                     uint64_t n, int32_t* assign, float* dis, cudaStream_t stream);

// Learned probe (probe.cu).
cudaError_t probe_forward(const ProbeNet& net, const float* X, uint32_t n, float* H1, float* Z1,
                          float* H2, float* Z2, float* Z, int* err, cudaStream_t st);
cudaError_t probe_backward(const ProbeNet& net, const float* X, uint32_t n,
                           const uint32_t* labels, uint32_t L, ProbeWork& w, ProbeNet& grad,
                           float* loss_sum, int* err, cudaStream_t st);
cudaError_t probe_init(ProbeNet& net, uint64_t seed, cudaStream_t st);
// Refreshes the BF16 weight copies from the FP32 weights.
cudaError_t probe_sync_bf16(const ProbeNet& net, cudaStream_t st);
// Inference: scores Z [n][C] (FP32) with BF16 hidden activations H1b, H2b [n][h].
// X: FP32 queries, or their BF16 copy Xb when not null.
cudaError_t probe_infer(const ProbeNet& net, const float* X, const uint16_t* Xb, uint32_t n,
                        uint16_t* H1b, uint16_t* H2b, float* Z, int* err, cudaStream_t st);
cudaError_t probe_adam(ProbeNet& net, const ProbeNet& grad, ProbeNet& m, ProbeNet& v, float lr,
                       uint64_t step, cudaStream_t st);
cudaError_t launch_probe_select(const ProbeNet& net, const DeviceIndex& ix, uint32_t n,
                                const float* Z, float mass, uint32_t max_probe, Scratch& s,
                                cudaStream_t st);

// Brute-force kNN on the tensor-core screen with FP32 rescoring (knn.cu); k <= 64.
cudaError_t launch_knn(const float* base, uint64_t n, uint32_t d, const float* Q, uint32_t nq,
                       uint32_t k, uint32_t* ids, float* dist, int* err, cudaStream_t st);
const ProbeNet* probe_net(const pgpu_probe* p);
int probe_device(const pgpu_probe* p);

// Pass pipeline (pipeline.cpp).
void free_scratch(Scratch* s);
uint64_t scratch_bytes(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t B);
int alloc_scratch(const DeviceIndex& ix, const SearchConfig& cfg, uint32_t B, Scratch* s,
                  std::string* err);
// Enqueues one pass of n <= s.cap queries (all pointers on the device). `ev`, if not
// null, holds PGPU_NUM_STAGES + 1 events recorded around the stages. On failure
// *what names the step.
cudaError_t run_pipeline(const DeviceIndex& ix, const SearchConfig& cfg, Scratch& s, uint32_t n,
                         const float* d_q, uint32_t topk, float* d_dist, uint32_t* d_ids,
                         int32_t* d_status, cudaStream_t st, cudaEvent_t* ev, int* launched,
                         const char** what);

// Host-side loader (index_host.cpp).
struct HostIndex {
    uint32_t d = 0, n = 0, C = 0, F = 0, nsq = 0, lsq = 0;
    int whether_norm = 0;
    int ip2cos = 0;  // 1: queries carry d - 1 values and get a 0 appended
    std::vector<float> coarse, fine, codebook;
    std::vector<uint32_t> cell_start, mem2local;
    std::vector<uint16_t> rec_fine;   // memory order
    std::vector<float> offsets_mem;   // memory order
    std::vector<uint8_t> codes_mem;   // memory order, code_stride bytes per row
    std::vector<float> feat_mem;      // memory order
    uint32_t code_stride = 0;
    // second-level PQ, memory order (empty without it)
    uint32_t pq_nsq = 0, pq_lsq = 0, pq_code_stride = 0;
    std::vector<float> pq_codebook, pq_offsets_mem;
    std::vector<uint8_t> pq_codes_mem;
};
int read_index_files(const char* dir, pgpu_index_arrays* arrays, std::vector<char>& storage,
                     std::string* err);
int build_host_index(const pgpu_index_arrays& a, HostIndex* h, std::string* err);
// base: original vectors in input order (host); permuted into memory order on the GPU.
int upload_index_with_base(const HostIndex& h, const float* base, DeviceIndex* ix,
                           std::string* err);
void free_device_index(DeviceIndex* ix);

}  // namespace pgpu
