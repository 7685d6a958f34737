/*
 * ORACLE — test infrastructure, not the product.
 *
 * A plain-C restatement of Puck's batched search path (index load,
 * normalisation, coarse/fine stage, filter-PQ ADC walk, exact rerank or the
 * second-level PQ rerank of whether_pq indexes) and of
 * the k-means assignment step, following the reference's float operation order
 * exactly (every product and sum rounded separately, BLAS dot products summed
 * sequentially). Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it, and only as the checker. Pinned against golden
 * vectors produced by the reference itself (tests/golden/make_golden.py).
 */
#ifndef PUCK_ORACLE_H
#define PUCK_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct po_index po_index;

typedef struct {
    uint32_t search_coarse_count; /* clamped to the index's coarse_cluster_count */
    uint32_t filter_topk;
    uint32_t topk;                /* the configured maximum top-k (FLAGS_topk) */
    double radius_rate;
} po_params;

/* Per-query intermediates, all optional (NULL = not wanted). */
typedef struct {
    uint32_t* coarse_tag; /* [search_coarse_count] */
    float* coarse_dist;   /* [search_coarse_count] */
    uint32_t* filter_tag; /* [filter_topk] memory idx, heap layout as the reference leaves it */
    float* filter_dist;   /* [filter_topk] */
    uint32_t filter_cnt;
    float* lut;           /* [filter_nsq * 256] */
    uint64_t scanned_points;
    uint64_t scanned_cells;
    uint64_t visited_cells;   /* fine-cell iterations of the walk before each break */
    uint64_t low_stat_cells;  /* cells with stationary below each coarse cluster's initial bound */
} po_trace;

po_index* po_load(const char* index_dir, int* err);
/* Same index from in-memory arrays in input order (the contents of the files). */
po_index* po_load_arrays(uint32_t d, uint32_t n, uint32_t C, uint32_t F, uint32_t nsq,
                         int whether_norm, const float* coarse, const float* fine,
                         const float* base, const uint32_t* cell_assign, const float* codebook,
                         const float* offsets_local, const uint8_t* codes_local, int* err);
/* The same with the second-level PQ (whether_pq): pq_nsq subspaces, its codebook
 * [pq_nsq][256][d/pq_nsq] and per-point offsets and codes in input order; base may
 * then be NULL. pq_nsq = 0 is po_load_arrays. */
po_index* po_load_arrays_pq(uint32_t d, uint32_t n, uint32_t C, uint32_t F, uint32_t nsq,
                            int whether_norm, const float* coarse, const float* fine,
                            const float* base, const uint32_t* cell_assign, const float* codebook,
                            const float* offsets_local, const uint8_t* codes_local,
                            uint32_t pq_nsq, const float* pq_codebook,
                            const float* pq_offsets_local, const uint8_t* pq_codes_local,
                            int* err);
void po_free(po_index* ix);
/* ip2cos = 1: queries carry d - 1 values and get a 0 appended, no normalisation
 * (hierarchical_cluster_index.cpp:1516-1520). Returns 0, or -1 for other values. */
int po_set_ip2cos(po_index* ix, int ip2cos);
int po_info(const po_index* ix, uint32_t* d, uint32_t* n, uint32_t* coarse, uint32_t* fine,
            uint32_t* filter_nsq, uint32_t* lsq, int* whether_norm);
/* Memory-order arrays built at load (memory_to_local, stationary, cell starts). */
const uint32_t* po_memory_to_local(const po_index* ix);
const float* po_stationary(const po_index* ix);
const uint32_t* po_cell_start(const po_index* ix);

/* One query, PuckIndex::search semantics. Returns 0, or <0 on error. */
int po_search(const po_index* ix, const po_params* p, const float* q, uint32_t topk, float* dist,
              uint32_t* ids, uint32_t* result_num, po_trace* trace);

/* PySearcher::search semantics: queries fanned out over nthreads threads. */
int po_search_batch(const po_index* ix, const po_params* p, uint32_t n, const float* q,
                    uint32_t topk, float* dist, uint32_t* ids, int32_t* status, int nthreads);

/* The library's scan mode: every record of the probed coarse clusters, exact
 * top-filter_topk by (distance, memory id), exact rerank. */
int po_search_scan(const po_index* ix, const po_params* p, const float* q, uint32_t topk,
                   float* dist, uint32_t* ids, uint32_t* result_num, po_trace* trace);
int po_search_scan_batch(const po_index* ix, const po_params* p, uint32_t n, const float* q,
                         uint32_t topk, float* dist, uint32_t* ids, int32_t* status,
                         int nthreads);

/* puck_assign (puck_index.cpp:602-709) for points whose cells are known: filter-PQ
 * codes and offsets, and with pnsq > 0 the second-level PQ's, in input order.
 * fcb [fnsq][256][d/fnsq], pcb [pnsq][256][d/pnsq]; d a multiple of both nsq. */
void po_puck_assign(uint32_t d, uint64_t n, const float* base, const uint32_t* cell_assign,
                    const float* coarse, const float* fine, uint32_t F, const float* fcb,
                    uint32_t fnsq, const float* pcb, uint32_t pnsq, float* f_off,
                    uint8_t* f_codes, float* p_off, uint8_t* p_codes);

/* RealtimeInsertPuckIndex (realtime_insert_puck_index.cpp) on a loaded index:
 * po_realtime_open switches the index to the realtime index's search (inserted points
 * scanned per cell after its records; the second-level PQ rerank summed subspace by
 * subspace), po_insert adds one point of d floats and returns its local id (n + insert
 * id) or -1, po_inserted_records copies out the inserted records. Not thread-safe
 * against concurrent searches. */
int po_realtime_open(po_index* ix);
int64_t po_insert(po_index* ix, const float* feature);
uint32_t po_inserted_records(const po_index* ix, uint32_t* cell, float* off, uint8_t* codes,
                             float* pq_off, uint8_t* pq_codes);

/* k-means assignment step: nearest_center (kmeans.cpp:221-258). */
void po_nearest_center(uint32_t dim, const float* centroids, uint64_t k, const float* x,
                       uint64_t n, int32_t* assign, float* dis);

/* Exact nearest-cell assignment of build (hierarchical_cluster_index.cpp:1042-1138),
 * given coarse/fine vocab with fine rows already in the trained (norm-sorted) order. */
void po_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C, const float* fine,
                            uint32_t F, const float* x, uint64_t n, uint32_t* cell,
                            float* cell_dist);

#ifdef __cplusplus
}
#endif
#endif
