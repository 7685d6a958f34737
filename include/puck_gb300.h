/*
 * puck_gb300 — GB300-native batched search for Puck (Puck-Flat) indexes.
 *
 * C ABI: plain pointers and sizes, no C++ or torch types. Every entry point
 * returns 0 on success and a negative PGPU_E* code on failure; the message of
 * the last failure on the calling thread is available from pgpu_last_error().
 *
 * The index is the reference's on-disk Puck index (index.dat, coarse.dat,
 * fine.dat, cell_assign.dat, filter_codebook.dat, filter_data.dat, and
 * all_data.feat.bin or, with whether_pq = 1, learn_codebooks.dat + pq_data.dat):
 * filter-PQ ADC scan followed by an exact FP32 rerank against the original
 * vectors ("Puck-Flat") or by the second-level PQ rerank. The search runs on one
 * GPU; there is no CPU fallback.
 */
#ifndef PUCK_GB300_H
#define PUCK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGPU_OK 0
#define PGPU_E_INVALID (-1)     /* bad argument: topk > configured topk, null feature, ... */
#define PGPU_E_ZERO_NORM (-2)   /* whether_norm index and a query with norm < 1e-6 */
#define PGPU_E_IO (-3)          /* index file missing, short or inconsistent */
#define PGPU_E_UNSUPPORTED (-4) /* index feature outside the supported set (ip2cos = 2, ks != 256) */
#define PGPU_E_CUDA (-5)        /* CUDA runtime error, or no usable GPU */
#define PGPU_E_NOMEM (-6)       /* device allocation failed */
#define PGPU_E_LIMIT (-7)       /* size beyond a documented limit of a kernel */
#define PGPU_E_TIMEOUT (-8)     /* pgpu_server_wait: the request did not finish in time */

/* Search modes. */
#define PGPU_MODE_EXACT 0      /* reference-exact: the same cells, heap and ties as PuckIndex::search */
#define PGPU_MODE_SCAN 1       /* every record of the probed coarse clusters is scanned (no pivot
                                  pruning); the filter_topk smallest ADC distances, each bit-identical
                                  to the reference's value for that record, go to the exact rerank.
                                  filter_topk (+ filter_margin) <= 2048. */

/* Arithmetic of the search (pgpu_params.precision).
 * FP32: every distance in FP32 in the reference's operation order (the coarse
 *       stage screens on the tensor cores and recomputes a provable window in
 *       FP32, so results do not change).
 * BF16: the precision form, scan mode only. Fine distances come from the BF16
 *       tensor-core contraction (FP32 accumulation), the ADC scan reads an FP16
 *       lookup table (accumulated in FP32) and keeps filter_topk + filter_margin
 *       candidates; the rerank screens them on a BF16 copy of the vectors and
 *       recomputes in FP32 every candidate within the screen's error bound of
 *       the topk-th, so the returned distances are FP32 and the returned ids
 *       are the FP32 rerank's over the same candidates. The BF16 copy (2 bytes
 *       per dimension per point) is made on the first use. */
#define PGPU_PRECISION_FP32 0
#define PGPU_PRECISION_BF16 1

/* Search parameters. Field names and meanings follow Puck's gflags
 * (puck/gflags/puck_gflags.cpp:68-78): search_coarse_count (default 200),
 * topk (default 100, the largest request topk allowed), filter_topk
 * (default 11 * topk, puck/index_conf.cpp:178-180), radius_rate (default 1.0). */
typedef struct {
    uint32_t search_coarse_count;
    uint32_t topk;
    uint32_t filter_topk;
    double radius_rate;
    int32_t device;     /* CUDA device ordinal */
    uint32_t max_batch; /* queries per device pass; sizes the per-pass scratch (scan mode adds a
                           distance buffer of 40960 floats per query, 4 MiB to 4 GiB in all) */
    int32_t mode;       /* PGPU_MODE_* */
    int32_t precision;  /* PGPU_PRECISION_* (default FP32) */
    uint32_t filter_margin; /* BF16 only: extra filter candidates kept for the rerank */
} pgpu_params;

typedef struct pgpu_index pgpu_index;

typedef struct {
    uint32_t feature_dim;
    uint32_t total_point_count;
    uint32_t coarse_cluster_count;
    uint32_t fine_cluster_count;
    uint32_t filter_nsq;
    uint32_t lsq;
    int32_t whether_norm;
    uint64_t device_bytes; /* HBM held by the resident index */
    /* floats per query read by the search entry points: feature_dim, or feature_dim - 1
     * on an ip2cos = 1 index (the caller's vectors; PySearcher::init, py_api_wrapper.cpp:104-106) */
    uint32_t query_dim;
    int32_t ip2cos;
} pgpu_index_info;

/* Host arrays of a Puck-Flat index, in the reference's input ("local") order,
 * i.e. exactly what the index files hold. Used by pgpu_open_arrays. */
typedef struct {
    uint32_t feature_dim, total_point_count, coarse_cluster_count, fine_cluster_count;
    uint32_t filter_nsq;
    int32_t whether_norm;
    const float* coarse;          /* [coarse_cluster_count][feature_dim] */
    const float* fine;            /* [fine_cluster_count][feature_dim] */
    const float* base;            /* [total_point_count][feature_dim] */
    const uint32_t* cell_assign;  /* [total_point_count], coarse * fine_cluster_count + fine */
    const float* filter_codebook; /* [filter_nsq][256][feature_dim / filter_nsq] */
    const float* filter_offsets;  /* [total_point_count] */
    const uint8_t* filter_codes;  /* [total_point_count][filter_nsq] */
    /* second-level PQ (whether_pq = 1, the reference's default): the rerank uses it
     * instead of the original vectors, and base may be NULL */
    int32_t whether_pq;
    uint32_t pq_nsq;              /* PQ subspaces (feature_dim by default, lsq = 1) */
    const float* pq_codebook;     /* [pq_nsq][256][feature_dim / pq_nsq] */
    const float* pq_offsets;      /* [total_point_count] */
    const uint8_t* pq_codes;      /* [total_point_count][pq_nsq] */
    /* ip2cos = 1: the index holds feature_dim = caller dimension + 1 vectors (inner product
     * recast as L2); each query is the caller's feature_dim - 1 values plus a 0, not
     * normalised (hierarchical_cluster_index.cpp:1516-1520). 0: off. */
    int32_t ip2cos;
} pgpu_index_arrays;

/* Fills the reference's flag defaults (search_coarse_count 200, topk 100,
 * filter_topk 1100, radius_rate 1.0, device 0, max_batch 8192, exact mode,
 * FP32, filter_margin 0). */
void pgpu_params_default(pgpu_params* params);

/* Replaces Index::init() (puck/hierarchical_cluster/hierarchical_cluster_index.cpp:220-255,
 * PuckIndex overrides puck/puck/puck_index.cpp:173-344): reads the index files under
 * index_path, builds the memory order (stable by cell, filter offset, input id),
 * the per-cell constants, and uploads the device-resident layout. */
int pgpu_open(const char* index_path, const pgpu_params* params, pgpu_index** out);

/* Same as pgpu_open, from host arrays instead of files. */
int pgpu_open_arrays(const pgpu_index_arrays* arrays, const pgpu_params* params,
                     pgpu_index** out);

/* Replaces the search-parameter part of update_gflag() + init()
 * (pyapi_wrapper/py_api_wrapper.cpp:33-35, 78-108) without reloading the index.
 * feature/structure come from the index; only search_coarse_count, topk,
 * filter_topk, radius_rate, max_batch and mode are taken. */
int pgpu_set_search_params(pgpu_index* index, const pgpu_params* params);

/* Replaces PySearcher::search (pyapi_wrapper/py_api_wrapper.cpp:154-170): n queries
 * of query_dim floats (pgpu_index_info: feature_dim, or feature_dim - 1 on an ip2cos
 * index), row-major, HOST memory; writes n*topk distances
 * (squared L2 in the searched space, ascending) and labels (input-order ids) per
 * query. Slots past a query's result count hold distance 0x7f7f7f7f (3.3961514e38)
 * and label 0xFFFFFFFF. status (optional, n entries) receives each query's
 * PuckIndex::search return code (0, or PGPU_E_INVALID / PGPU_E_ZERO_NORM). */
int pgpu_search_batch(pgpu_index* index, uint32_t n, const float* query, uint32_t topk,
                      float* distance, uint32_t* labels, int32_t* status);

/* Replaces virtual int puck::Index::search(const Request*, Response*)
 * (puck/index.h:46, implemented by puck/puck/puck_index.cpp:559-600) for one query:
 * Request{topk, feature} -> Response{distance, local_idx, result_num}. */
int pgpu_search(pgpu_index* index, const float* feature, uint32_t topk, float* distance,
                uint32_t* local_idx, uint32_t* result_num);

/* Device-memory variant of pgpu_search_batch: query, distance, labels and status
 * are DEVICE pointers on the index's GPU; work is enqueued on `stream`
 * (a cudaStream_t, NULL = the legacy default stream) and the call returns
 * without synchronising. */
int pgpu_search_batch_device(pgpu_index* index, uint32_t n, const float* query, uint32_t topk,
                             float* distance, uint32_t* labels, int32_t* status, void* stream);

int pgpu_index_info_get(const pgpu_index* index, pgpu_index_info* info);

/* Launch statistics of the last search call on this index: kernels launched and
 * the number of filter records the ADC scan evaluated. */
int pgpu_last_stats(const pgpu_index* index, uint64_t* kernels_launched,
                    uint64_t* records_scanned, uint64_t* cells_scanned);

/* Per-stage device timing (CUDA events recorded on the launching stream around
 * each kernel). With profiling enabled, pgpu_stage_times returns, for the last
 * search call, the milliseconds spent in each stage, summed over its passes:
 * 0 query prep, 1 coarse scores (+ the learned probe, which runs first and leaves the coarse
 * screen only the queries it does not answer), 2 coarse select, 3 fine scores, 4 fine order
 * (exact mode) or the scan's block launch order and record offsets (scan mode), 5 cell walk
 * (exact mode) or the filter scan (scan mode: k_scan_score, which scores the probed records and
 * selects the top filter_topk, or the fused k_scan_il when the split scan does not apply), 6 the
 * fused scan for the queries the split scan left (scan mode; nothing in exact mode), 7 rerank.
 * It waits for the call's work to finish. */
#define PGPU_NUM_STAGES 8
int pgpu_set_profiling(pgpu_index* index, int enable);
int pgpu_stage_times(pgpu_index* index, float* ms, uint32_t n_stages);

/* Diagnostic counters of the filter stage for the last pgpu_search_batch call,
 * summed over queries. Exact mode: 0 filter records scanned, 1 cells scanned,
 * 2 fine-order chunks, 3 stationary-order enumerations, 4 coarse clusters walked in
 * fine order, 5 heap inserts, then thread-0 clock cycles: 6 replay, 7 whole walk,
 * 8 prologue (LUT), 9 candidate generation, 10 speculative ADC. Scan mode:
 * 0 records evaluated, 1 records past the cell-distance test, 2 records kept,
 * 3 buffer compactions, 5 most records of one
 * query, then cycles: 6 prologue, 7 whole block, 8 record rounds, 9 compactions,
 * 10 final sort. Both modes: 11 queries whose coarse top-P was recomputed in full
 * (exact ties at the cut of the tensor-core window); with a learned probe, 12
 * queries that kept the fixed count and 13 clusters the probe chose for the
 * others. Fills min(n, 14) values. */
int pgpu_walk_counters(const pgpu_index* index, uint64_t* out, uint32_t n);

/* Diagnostic of the scan-mode filter stage: runs one pass of n <= max_batch HOST
 * queries and returns, per query, the candidates handed to the rerank: labels
 * (input-order ids) and filter distances, filter_topk (+ filter_margin in BF16)
 * slots per query (the set of the smallest filter distances, unordered), and
 * count[i] of them filled. */
int pgpu_filter_candidates(pgpu_index* index, uint32_t n, const float* query, uint32_t* labels,
                           float* distance, uint32_t* count);

/* ------------------------------------------------------------ realtime insert
 * RealtimeInsertPuckIndex (puck/puck/realtime_insert_puck_index.h:32-107) on the
 * device. pgpu_realtime_open replaces its init() (realtime_insert_puck_index.cpp:
 * 225-272): it reserves room for `capacity` inserted points on the index's GPU
 * (the per-record arrays are widened once, so call it before any server is created
 * on the index). pgpu_insert replaces insert(const InsertRequest*) (:273-337) for n
 * HOST features ([n][query_dim], labels stay with the caller): each is normalised
 * when the index normalises, assigned to its nearest cell on the index's live
 * stationary terms, encoded like the build, and then found by every search in both
 * modes, exactly as the reference scans a cell's inserted points after its base
 * records. local_idx[i] = the point's local id (point count + insert id), or -1
 * (a non-finite or zero-norm feature). Inserts take the index's lock; they must not
 * overlap a server running on the same index. PGPU_E_LIMIT beyond the capacity,
 * PGPU_E_UNSUPPORTED on an ip2cos index. */
int pgpu_realtime_open(pgpu_index* index, uint32_t capacity);
int pgpu_insert(pgpu_index* index, uint32_t n, const float* feature, int64_t* local_idx);

int pgpu_close(pgpu_index* index);

/* ------------------------------------------------------------------ serving
 * Continuous batching of search requests on one resident index. No counterpart in
 * the reference, whose callers fan single searches out over threads
 * (pyapi_wrapper/py_api_wrapper.cpp:110-170); here a scheduler thread fills device
 * batches from all pending requests.
 *
 * The server owns S slots (S = min(max_slots, scratch_budget_bytes / slot size)),
 * each with its own scratch, stream, pinned staging and one CUDA graph per
 * (batch-size bucket, topk) holding the whole pass (query upload, the search
 * kernels of the index's current mode, result download), captured on first use.
 * A free slot takes requests from the head of the queue with the same topk, up to
 * max_batch queries, padded to the next bucket (32, 64, ..., max_batch); slots run
 * concurrently on separate streams. A request's results are bit-identical to
 * pgpu_search_batch on the same queries. The index's search parameters must not
 * change while a server is attached. Query, distance, labels and status buffers
 * belong to the caller and must stay valid until pgpu_server_wait returns. */
typedef struct pgpu_server pgpu_server;

typedef struct {
    uint32_t max_batch;            /* queries per device batch (and per request) */
    uint64_t scratch_budget_bytes; /* device + pinned memory the slots may use */
    uint32_t max_slots;
} pgpu_server_params;

typedef struct {
    uint64_t requests_submitted, requests_done, queries_done;
    uint64_t batches, graph_launches, graphs_captured, padded_queries;
    double latency_us_sum; /* submit -> results delivered, summed over done requests */
    uint32_t slots;
    uint64_t slot_bytes;
} pgpu_server_stats;

/* max_batch 1024, scratch budget 1 GiB, 4 slots. */
void pgpu_server_params_default(pgpu_server_params* params);
int pgpu_server_create(pgpu_index* index, const pgpu_server_params* params, pgpu_server** out);
/* Queues n (1..max_batch) host queries (query_dim floats each) with their own topk;
 * returns a ticket. */
int pgpu_server_submit(pgpu_server* server, uint32_t n, const float* query, uint32_t topk,
                       float* distance, uint32_t* labels, int32_t* status, uint64_t* ticket);
/* Waits for a ticket (timeout_ms < 0: no limit); latency_us (optional) receives
 * the time from submit to results delivered. A ticket can be waited for once. */
int pgpu_server_wait(pgpu_server* server, uint64_t ticket, int32_t timeout_ms, double* latency_us);
int pgpu_server_stats_get(pgpu_server* server, pgpu_server_stats* out);
/* Finishes queued and running requests, then frees the server. */
int pgpu_server_destroy(pgpu_server* server);

/* k-means assignment step used by train (kmeans.cpp:221-258 nearest_center):
 * for each of n points (DEVICE pointer, [n][dim]) the id of the nearest of k
 * centroids (DEVICE pointer, [k][dim]) and its distance
 * |x|^2 + |c|^2 - 2 x.c, first centroid wins ties. A BF16 tensor-core screen
 * of every (point, centroid) pair bounds the window that is recomputed in the
 * reference's FP32 order, so the result is the exact one. Enqueued on `stream`. */
int pgpu_nearest_center(uint32_t dim, const float* centroids, uint64_t k, const float* points,
                        uint64_t n, int32_t* assign, float* distance, void* stream);

/* The build's cell assignment (hierarchical_cluster_index.cpp:1042-1138,
 * HierarchicalClusterIndex::nearest_cell_assign driven by assign): for each of n
 * points (DEVICE pointer, [n][dim]) the cell c * F + f minimising
 * ((0.5|c|^2 - x.c) + 0.5|x|^2 - x.f) + (0.5|f|^2 + f.c) over the C coarse and F
 * fine centroids (DEVICE pointers; the fine ones in the index's order, descending
 * norm), walked like the reference (coarse clusters by ascending term, fine ids in
 * order, its triangle-inequality break, first minimum wins), in the reference's
 * FP32 order: the same cells and distances bit for bit. cell: [n] u32, distance:
 * [n] floats (DEVICE). Enqueued on `stream`; returns after it finished. */
int pgpu_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C, const float* fine,
                             uint32_t F, const float* points, uint64_t n, uint32_t* cell,
                             float* distance, void* stream);

/* Replaces PuckIndex::puck_assign (puck/puck/puck_index.cpp:602-709), the build's
 * encoder, for n points whose cells are known (cell_assign = coarse * F + fine): the
 * filter-PQ offset and codes of each point (filter_data.dat records) and, with
 * pq_nsq > 0, the second-level PQ's (pq_data.dat), bit-identical to the reference.
 * base [n][d], coarse [C][d], fine [F][d], filter_codebook [filter_nsq][256][d/filter_nsq],
 * pq_codebook [pq_nsq][256][d/pq_nsq]; outputs offsets [n] and codes [n][nsq]. All
 * pointers DEVICE on the calling thread's current device; work runs on `stream` and
 * the call returns when it is done. PGPU_E_INVALID for a cell id >= C * F. */
int pgpu_puck_assign(uint32_t d, uint64_t n, const float* base, const uint32_t* cell_assign,
                     const float* coarse, uint32_t C, const float* fine, uint32_t F,
                     const float* filter_codebook, uint32_t filter_nsq, const float* pq_codebook,
                     uint32_t pq_nsq, float* filter_offsets, uint8_t* filter_codes,
                     float* pq_offsets, uint8_t* pq_codes, void* stream);

/* The k-means assignment step of pgpu_nearest_center, allocating no device
 * memory, on the exact SIMT kernel (same results bit for bit as the tensor-core
 * screen + exact window of pgpu_nearest_center, lower throughput). No counterpart in the reference: it exists for callers that must not
 * allocate GPU memory (a process that hands out device memory from its own pool,
 * or code that must not enter the CUDA allocator). pgpu_nearest_center allocates
 * its norm scratch on every call; this variant keeps it in a fixed array inside
 * the library instead (4.25 MiB held on each GPU that loads the library, until
 * exit), so it takes at most 1048576 points and 65536 centroids per call
 * (PGPU_E_LIMIT beyond). It runs on the calling thread's current device; its
 * first call on a device looks up the array's device address and should come
 * before any stream capture; the address is kept for the life of the process, so
 * the library must not be used on a device across cudaDeviceReset. All calls on
 * a device share the array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller. Results are identical to pgpu_nearest_center's. */
int pgpu_nearest_center_noalloc(uint32_t dim, const float* centroids, uint64_t k,
                                const float* points, uint64_t n, int32_t* assign,
                                float* distance, void* stream);

/* BF16 tensor-core contraction (tcgen05.mma, FP32 accumulation in tensor memory)
 * on DEVICE pointers of the calling thread's current device:
 *   acc(i,j) = sum_{t<k} bf16(a[i*a_rs + t*a_ks]) * bf16(b[j*b_rs + t*b_ks]),
 *   i < na, j < nb, and out[i*ld_out + j] = f(acc) with f by mode:
 *   SCORE bias[j] - acc; NEG -acc; STORE alpha*acc + beta*out; BIAS acc + bias[j];
 *   BIAS_GELU out2[i*ld_out + j] = acc + bias[j], out = GELU(out2) (erf form);
 *   GELU_BWD acc * GELU'(aux[i*ld_aux + j]).
 * The engine behind the coarse screen, nearest_center and the probe network;
 * exported for tests and tools. Enqueued on `stream`; returns after it finished. */
#define PGPU_CONTRACT_SCORE 0
#define PGPU_CONTRACT_NEG 1
#define PGPU_CONTRACT_STORE 2
#define PGPU_CONTRACT_BIAS 3
#define PGPU_CONTRACT_BIAS_GELU 4
#define PGPU_CONTRACT_GELU_BWD 5
int pgpu_contract_bf16(int32_t mode, uint32_t na, uint32_t nb, uint32_t k, const float* a,
                       uint64_t a_rs, uint64_t a_ks, const float* b, uint64_t b_rs, uint64_t b_ks,
                       const float* bias, const float* aux, uint64_t ld_aux, float* out,
                       uint64_t ld_out, float* out2, float alpha, float beta, void* stream);
/* The same contraction on BF16 operands already in memory, row-major (row i of a at
 * a + i*a_rs elements, k contiguous values). With 16-byte aligned rows (a_rs and b_rs
 * multiples of 8, 16-byte aligned pointers) it runs the persistent, warp-specialised
 * kernel (TMA-loaded, 128-byte swizzled operands, double-buffered TMEM accumulators):
 * the form the search's screens and the probe's inference use; otherwise the
 * cp.async kernel. Same modes and outputs as pgpu_contract_bf16. No counterpart in
 * the reference; exported for tests and tools. */
int pgpu_contract_bf16_rows(int32_t mode, uint32_t na, uint32_t nb, uint32_t k,
                            const uint16_t* a, uint64_t a_rs, const uint16_t* b, uint64_t b_rs,
                            const float* bias, const float* aux, uint64_t ld_aux, float* out,
                            uint64_t ld_out, float* out2, float alpha, float beta, void* stream);

/* ------------------------------------------------------------ learned probe
 * A small MLP (query -> coarse-cluster scores, GELU, 2 hidden layers) trained and
 * evaluated on the GPU with the BF16 tensor-core contraction (FP32 accumulation,
 * FP32 master weights, Adam). No counterpart in the reference: it replaces the
 * fixed search_coarse_count by a per-query count in scan mode.
 * Parameter layout (pgpu_probe_get/set_params, pgpu_probe_gradients):
 *   W1 [hidden][dim], b1 [hidden], W2 [hidden][hidden], b2 [hidden],
 *   W3 [clusters][hidden], b3 [clusters]. */
typedef struct pgpu_probe pgpu_probe;
int pgpu_probe_create(uint32_t dim, uint32_t hidden, uint32_t clusters, uint64_t seed,
                      int32_t device, pgpu_probe** out);
int pgpu_probe_destroy(pgpu_probe* probe);
int pgpu_probe_info(const pgpu_probe* probe, uint32_t* dim, uint32_t* hidden, uint32_t* clusters,
                    uint64_t* params);
/* One Adam step on a batch. queries [n][dim] (normalised as the index normalises
 * them) and labels [n][L] (coarse cluster ids of each query's nearest points,
 * 0xFFFFFFFF = none; the target is their distribution) are DEVICE pointers whose
 * contents are complete when the call is made. loss (optional, host) receives
 * the batch's mean softmax cross-entropy before the step. */
int pgpu_probe_train_step(pgpu_probe* probe, const float* queries, const uint32_t* labels,
                          uint32_t n, uint32_t L, float lr, float* loss);
/* Loss and gradients of a batch without an update; grads is a HOST buffer of
 * the parameter count, in the parameter layout. */
int pgpu_probe_gradients(pgpu_probe* probe, const float* queries, const uint32_t* labels,
                         uint32_t n, uint32_t L, float* loss, float* grads);
/* Scores [n][clusters] (DEVICE) of n DEVICE queries. */
int pgpu_probe_forward(pgpu_probe* probe, const float* queries, uint32_t n, float* scores);
int pgpu_probe_get_params(const pgpu_probe* probe, float* params, uint64_t count);
int pgpu_probe_set_params(pgpu_probe* probe, const float* params, uint64_t count);
/* Attaches a probe to a scan-mode index (NULL detaches; the probe must outlive
 * the attachment). Per query the clusters are taken in descending predicted
 * probability until their mass reaches `mass` (at most max_probe <= 64
 * clusters); a query whose max_probe best clusters stay below `mass` keeps the
 * fixed search_coarse_count selection. Walk counters 12 and 13 report the
 * fallbacks and the clusters the probe chose. */
int pgpu_set_probe(pgpu_index* index, pgpu_probe* probe, float mass, uint32_t max_probe);

/* Brute-force k nearest neighbours (k <= 64) by squared L2 of nq DEVICE queries
 * over n DEVICE base vectors: a BF16 tensor-core screen of every pair keeps 64
 * candidates per query, which are rescored in FP32; labels and distances
 * ([nq][k], DEVICE) ascend. The labels of the learned probe's training set.
 * Enqueued on `stream`; returns after it finished. */
int pgpu_knn(const float* base, uint64_t n, uint32_t dim, const float* queries, uint32_t nq,
             uint32_t k, uint32_t* labels, float* distance, void* stream);

const char* pgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
