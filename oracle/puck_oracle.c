/*
 * ORACLE — test infrastructure, not the product. See puck_oracle.h.
 *
 * Restates, in plain C and in the reference's float operation order:
 *   load    : HierarchicalClusterIndex::read_coodbooks
 *             (puck/hierarchical_cluster/hierarchical_cluster_index.cpp:257-324),
 *             PuckIndex::convert_local_to_memory_idx (puck/puck/puck_index.cpp:229-309),
 *             read_feature_index (puck_index.cpp:198-227, hierarchical_cluster_index.cpp:367-406)
 *   search  : PuckIndex::search (puck_index.cpp:559-600) and the stages it calls
 *   assign  : nearest_center (puck/hierarchical_cluster/kmeans.cpp:221-258),
 *             nearest_cell_assign (hierarchical_cluster_index.cpp:1042-1085)
 * Build with -O2 -ffp-contract=off (no FMA contraction, no fast-math).
 */
#include "puck_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct po_index {
    uint32_t d, n, C, F, nsq, lsq;
    int whether_norm, ip2cos;
    float* coarse;          /* C*d */
    float* fine;            /* F*d */
    float* coarse_norms;    /* C: 0.5*|c|^2 */
    float* stationary;      /* C*F: 0.5*|f|^2 + f.c, sqrt(FLT_MAX) for empty cells */
    uint32_t* cell_start;   /* C*F + 1 */
    float* min_dist_offset; /* C */
    uint32_t* mem2local;    /* n */
    float* offsets;         /* n, memory order */
    uint8_t* codes;         /* n*nsq, memory order */
    float* feat;            /* n*d, memory order (NULL with the second-level PQ) */
    float* codebook;        /* nsq*256*lsq */
    /* second-level PQ (whether_pq, puck_index.cpp:402-427) */
    uint32_t pq_nsq, pq_lsq;
    float* pq_offsets;      /* n, memory order */
    uint8_t* pq_codes;      /* n*pq_nsq, memory order */
    float* pq_codebook;     /* pq_nsq*256*pq_lsq */
    /* RealtimeInsertPuckIndex (realtime_insert_puck_index.cpp); realtime = 0: PuckIndex */
    int realtime;
    uint32_t ins_n, ins_cap;
    uint32_t* ins_cell;     /* [ins_n] cell of each inserted point */
    float* ins_off;         /* [ins_n] filter offsets */
    uint8_t* ins_codes;     /* [ins_n][nsq] */
    float* ins_pq_off;      /* [ins_n] (second-level PQ) */
    uint8_t* ins_pq_codes;  /* [ins_n][pq_nsq] */
    float* ins_feat;        /* [ins_n][d] (without the second-level PQ) */
    int32_t* ins_head;      /* [C*F] newest insert of each cell, -1: none */
    int32_t* ins_next;      /* [ins_n] next older insert of the same cell */
    uint32_t* cell_cnt;     /* [C*F] base + inserted points (InsertFineCluster::point_cnt) */
};

/* ---------------------------------------------------------------- BLAS order */

/* Sequential dot product: the deterministic BLAS the oracle build of the
 * reference links (oracle/ref/shim_blas.c). */
static float dotf(const float* x, const float* y, uint32_t n) {
    float s = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        float p = x[i] * y[i];
        s = s + p;
    }
    return s;
}

/* ------------------------------------------------------------------ MaxHeap */
/* Bounded max-heap of puck/hierarchical_cluster/max_heap.cpp:28-102: 1-based
 * arrays, 0x7f7f7f7f sentinel fill, a new value is rejected if >= top, the
 * first `size` inserts sift down from the last empty slot, reorder() is an
 * in-place heap sort to ascending order. */
typedef struct {
    float* val; /* 1-based view */
    uint32_t* tag;
    uint32_t size;
    uint32_t dpc; /* slots not yet filled */
} po_heap;

static void heap_init(po_heap* h, uint32_t size, float* val, uint32_t* tag) {
    memset(val, 0x7f, sizeof(float) * size);
    h->val = val - 1;
    h->tag = tag - 1;
    h->size = size;
    h->dpc = size;
}

static void heap_insert(po_heap* h, uint32_t heap_size, uint32_t father, float v, uint32_t t) {
    for (;;) {
        uint32_t left = father << 1;
        if (left > heap_size) break;
        uint32_t right = left + 1;
        if (right > heap_size || h->val[left] > h->val[right]) {
            if (h->val[left] < v) break;
            h->val[father] = h->val[left];
            h->tag[father] = h->tag[left];
            father = left;
        } else {
            if (h->val[right] < v) break;
            h->val[father] = h->val[right];
            h->tag[father] = h->tag[right];
            father = right;
        }
    }
    h->val[father] = v;
    h->tag[father] = t;
}

static int heap_update(po_heap* h, float v, uint32_t t) {
    uint32_t father = 1;
    if (v >= h->val[1]) return 0;
    if (h->dpc > 0) father = h->dpc--;
    heap_insert(h, h->size, father, v, t);
    return 1;
}

static void heap_reorder(po_heap* h) {
    for (uint32_t i = 0; i < h->size; ++i) {
        float vb = h->val[1];
        uint32_t tb = h->tag[1];
        uint32_t hs = h->size - i;
        heap_insert(h, hs - 1, 1, h->val[hs], h->tag[hs]);
        h->val[hs] = vb;
        h->tag[hs] = tb;
    }
}

static uint32_t heap_count(const po_heap* h) { return h->size - h->dpc; }

/* --------------------------------------------------------------- file input */

static int read_file(const char* dir, const char* name, void** out, size_t* len) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    void* buf = malloc(sz > 0 ? (size_t)sz : 1);
    if (!buf || (sz > 0 && fread(buf, 1, (size_t)sz, f) != (size_t)sz)) {
        fclose(f);
        free(buf);
        return -1;
    }
    fclose(f);
    *out = buf;
    *len = (size_t)sz;
    return 0;
}

/* fvecs: per row an int32 dim then dim floats. */
static float* read_fvecs(const char* dir, const char* name, uint32_t dim, uint64_t rows) {
    void* raw;
    size_t len;
    if (read_file(dir, name, &raw, &len) != 0) return NULL;
    if (len != rows * (4 + 4ull * dim)) {
        free(raw);
        return NULL;
    }
    float* out = (float*)malloc(sizeof(float) * dim * rows + 4);
    const uint8_t* p = (const uint8_t*)raw;
    for (uint64_t i = 0; i < rows; ++i) {
        int32_t dd;
        memcpy(&dd, p, 4);
        if ((uint32_t)dd != dim) {
            free(raw);
            free(out);
            return NULL;
        }
        memcpy(out + i * dim, p + 4, 4ull * dim);
        p += 4 + 4ull * dim;
    }
    free(raw);
    return out;
}

typedef struct {
    uint32_t cell;
    float offset;
    uint32_t local;
} mem_order;

/* std::pair<uint32_t, std::pair<float, uint32_t>> ordering (puck_index.cpp:248-268);
 * the local id makes the key unique, so any sort reproduces std::stable_sort. */
static int cmp_mem_order(const void* a, const void* b) {
    const mem_order* x = (const mem_order*)a;
    const mem_order* y = (const mem_order*)b;
    if (x->cell != y->cell) return x->cell < y->cell ? -1 : 1;
    if (x->offset < y->offset) return -1;
    if (y->offset < x->offset) return 1;
    if (x->local != y->local) return x->local < y->local ? -1 : 1;
    return 0;
}

void po_free(po_index* ix) {
    if (!ix) return;
    free(ix->coarse);
    free(ix->fine);
    free(ix->coarse_norms);
    free(ix->stationary);
    free(ix->cell_start);
    free(ix->min_dist_offset);
    free(ix->mem2local);
    free(ix->offsets);
    free(ix->codes);
    free(ix->feat);
    free(ix->codebook);
    free(ix->pq_offsets);
    free(ix->pq_codes);
    free(ix->pq_codebook);
    free(ix->ins_cell);
    free(ix->ins_off);
    free(ix->ins_codes);
    free(ix->ins_pq_off);
    free(ix->ins_pq_codes);
    free(ix->ins_feat);
    free(ix->ins_head);
    free(ix->ins_next);
    free(ix->cell_cnt);
    free(ix);
}

po_index* po_load_arrays_pq(uint32_t d, uint32_t n, uint32_t C, uint32_t F, uint32_t nsq,
                            int whether_norm, const float* coarse, const float* fine,
                            const float* base, const uint32_t* cell_assign, const float* codebook,
                            const float* offsets_local, const uint8_t* codes_local,
                            uint32_t pq_nsq, const float* pq_codebook,
                            const float* pq_offsets_local, const uint8_t* pq_codes_local,
                            int* err) {
    int e = 0;
    mem_order* order = NULL;
    po_index* ix = (po_index*)calloc(1, sizeof(po_index));
    ix->d = d;
    ix->n = n;
    ix->C = C;
    ix->F = F;
    ix->nsq = nsq;
    ix->whether_norm = whether_norm;
    if (nsq == 0 || nsq > d || d % nsq != 0 || C == 0 || F == 0) { e = -7; goto fail; }
    ix->lsq = d / nsq;
    const uint64_t cells = (uint64_t)C * F;
    ix->coarse = (float*)malloc(sizeof(float) * (uint64_t)C * d);
    ix->fine = (float*)malloc(sizeof(float) * (uint64_t)F * d);
    memcpy(ix->coarse, coarse, sizeof(float) * (uint64_t)C * d);
    memcpy(ix->fine, fine, sizeof(float) * (uint64_t)F * d);

    /* read_coodbooks: coarse norms, fine norms, F x C products (sgemm "TN"). */
    ix->coarse_norms = (float*)malloc(sizeof(float) * C);
    for (uint32_t c = 0; c < C; ++c)
        ix->coarse_norms[c] = dotf(ix->coarse + (uint64_t)c * d, ix->coarse + (uint64_t)c * d, d) / 2;
    float* fine_norms = (float*)malloc(sizeof(float) * F);
    for (uint32_t f = 0; f < F; ++f)
        fine_norms[f] = dotf(ix->fine + (uint64_t)f * d, ix->fine + (uint64_t)f * d, d) / 2;
    ix->stationary = (float*)malloc(sizeof(float) * cells);
    for (uint32_t c = 0; c < C; ++c)
        for (uint32_t f = 0; f < F; ++f) {
            float prod = dotf(ix->fine + (uint64_t)f * d, ix->coarse + (uint64_t)c * d, d);
            ix->stationary[(uint64_t)c * F + f] = fine_norms[f] + prod;
        }
    free(fine_norms);

    /* convert_local_to_memory_idx */
    order = (mem_order*)malloc(sizeof(mem_order) * (n ? n : 1));
    for (uint32_t i = 0; i < n; ++i) {
        if (cell_assign[i] >= cells) { e = -11; goto fail; }
        order[i].cell = cell_assign[i];
        order[i].offset = offsets_local[i];
        order[i].local = i;
    }
    qsort(order, n, sizeof(mem_order), cmp_mem_order);
    ix->cell_start = (uint32_t*)malloc(sizeof(uint32_t) * (cells + 1));
    for (uint64_t i = 0; i <= cells; ++i) ix->cell_start[i] = n;
    ix->mem2local = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    {
        uint32_t cellcount = 0;
        ix->cell_start[0] = 0;
        for (uint32_t i = 0; i < n; ++i) {
            ix->mem2local[i] = order[i].local;
            while (cellcount + 1 <= order[i].cell) {
                ++cellcount;
                ix->cell_start[cellcount] = i;
            }
        }
    }
    ix->min_dist_offset = (float*)malloc(sizeof(float) * C);
    for (uint32_t c = 0; c < C; ++c) ix->min_dist_offset[c] = FLT_MAX;
    for (uint64_t i = 0; i < cells; ++i) {
        uint32_t s = ix->cell_start[i], t = ix->cell_start[i + 1];
        uint32_t c = (uint32_t)(i / F);
        if (s > t) { e = -12; goto fail; }
        if (s == t) ix->stationary[i] = sqrtf(FLT_MAX);
        float st = ix->stationary[i];
        if (st < ix->min_dist_offset[c]) ix->min_dist_offset[c] = st;
    }

    /* read_feature_index: filter records and the original vectors (or, with the
     * second-level PQ, its records) in memory order. */
    if (pq_nsq) {
        if (pq_nsq > d || d % pq_nsq != 0 || !pq_codebook || !pq_offsets_local || !pq_codes_local) {
            e = -13;
            goto fail;
        }
        ix->pq_nsq = pq_nsq;
        ix->pq_lsq = d / pq_nsq;
    } else if (!base) {
        e = -14;
        goto fail;
    }
    ix->offsets = (float*)malloc(sizeof(float) * (n ? n : 1));
    ix->codes = (uint8_t*)malloc((uint64_t)nsq * (n ? n : 1));
    if (pq_nsq) {
        ix->pq_offsets = (float*)malloc(sizeof(float) * (n ? n : 1));
        ix->pq_codes = (uint8_t*)malloc((uint64_t)pq_nsq * (n ? n : 1));
        ix->pq_codebook = (float*)malloc(sizeof(float) * (uint64_t)pq_nsq * 256 * ix->pq_lsq);
        memcpy(ix->pq_codebook, pq_codebook, sizeof(float) * (uint64_t)pq_nsq * 256 * ix->pq_lsq);
    } else {
        ix->feat = (float*)malloc(sizeof(float) * (uint64_t)d * (n ? n : 1));
    }
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t l = ix->mem2local[i];
        ix->offsets[i] = offsets_local[l];
        memcpy(ix->codes + (uint64_t)i * nsq, codes_local + (uint64_t)l * nsq, nsq);
        if (pq_nsq) {
            ix->pq_offsets[i] = pq_offsets_local[l];
            memcpy(ix->pq_codes + (uint64_t)i * pq_nsq, pq_codes_local + (uint64_t)l * pq_nsq, pq_nsq);
        } else {
            memcpy(ix->feat + (uint64_t)i * d, base + (uint64_t)l * d, 4ull * d);
        }
    }
    ix->codebook = (float*)malloc(sizeof(float) * (uint64_t)nsq * 256 * ix->lsq);
    memcpy(ix->codebook, codebook, sizeof(float) * (uint64_t)nsq * 256 * ix->lsq);
    free(order);
    if (err) *err = 0;
    return ix;
fail:
    free(order);
    po_free(ix);
    if (err) *err = e;
    return NULL;
}

po_index* po_load_arrays(uint32_t d, uint32_t n, uint32_t C, uint32_t F, uint32_t nsq,
                         int whether_norm, const float* coarse, const float* fine,
                         const float* base, const uint32_t* cell_assign, const float* codebook,
                         const float* offsets_local, const uint8_t* codes_local, int* err) {
    return po_load_arrays_pq(d, n, C, F, nsq, whether_norm, coarse, fine, base, cell_assign,
                             codebook, offsets_local, codes_local, 0, NULL, NULL, NULL, err);
}

po_index* po_load(const char* dir, int* err) {
    int e = 0;
    void* raw = NULL;
    size_t len = 0;
    uint32_t* cell_assign = NULL;
    uint8_t* rec = NULL;
    float *coarse = NULL, *fine = NULL, *feat = NULL, *codebook = NULL, *offsets = NULL;
    float *pq_cb = NULL, *pq_off = NULL;
    uint8_t *codes = NULL, *pq_rec = NULL, *pq_codes = NULL;
    po_index* ix = NULL;
    uint32_t d, n, C, F, nsq, pq_nsq = 0, ip2cos = 0;
    int whether_norm;

    /* index.dat: size_t length + packed config (hierarchical_cluster_index.cpp:551-567) */
    if (read_file(dir, "index.dat", &raw, &len) != 0 || len < 8 + 43) { e = -1; goto done; }
    {
        const uint8_t* p = (const uint8_t*)raw + 8;
        int32_t itype;
        uint32_t u;
        memcpy(&itype, p, 4); p += 4;
        if (itype != 1) { e = -2; goto done; } /* PUCK */
        memcpy(&d, p, 4); p += 4;
        whether_norm = *p; p += 1;
        memcpy(&n, p, 4); p += 4;
        uint8_t whether_filter = *p; p += 1;
        memcpy(&nsq, p, 4); p += 4;
        memcpy(&u, p, 4); p += 4; /* ks */
        if (u != 256 || !whether_filter) { e = -3; goto done; }
        uint8_t whether_pq = *p; p += 1;
        memcpy(&u, p, 4); p += 4; /* nsq of the second-level PQ */
        if (whether_pq) pq_nsq = u;
        memcpy(&u, p, 4); p += 4; /* its ks */
        if (whether_pq && u != 256) { e = -4; goto done; }
        memcpy(&u, p, 4); p += 4;
        /* ip2cos: 1 is searchable; 2 is not (PySearcher passes feature_dim - 1 values while
           normalization widens only for 1, py_api_wrapper.cpp:104-106) */
        if (u > 1) { e = -5; goto done; }
        ip2cos = u;
        memcpy(&C, p, 4); p += 4;
        memcpy(&F, p, 4); p += 4;
    }
    free(raw);
    raw = NULL;
    if (nsq == 0 || nsq > d || d % nsq != 0) { e = -7; goto done; } /* reference reads past d otherwise */
    {
        const uint32_t lsq = d / nsq;
        coarse = read_fvecs(dir, "coarse.dat", d, C);
        fine = read_fvecs(dir, "fine.dat", d, F);
        if (!pq_nsq) feat = read_fvecs(dir, "all_data.feat.bin", d, n);
        codebook = read_fvecs(dir, "filter_codebook.dat", lsq, (uint64_t)nsq * 256);
        if (!coarse || !fine || (!feat && !pq_nsq) || !codebook) { e = -8; goto done; }
        if (pq_nsq) {
            if (pq_nsq > d || d % pq_nsq != 0) { e = -7; goto done; }
            /* learn_codebooks.dat / pq_data.dat (puck/gflags/puck_gflags.cpp defaults) */
            pq_cb = read_fvecs(dir, "learn_codebooks.dat", d / pq_nsq, (uint64_t)pq_nsq * 256);
            const uint32_t prb = 4 + pq_nsq;
            if (!pq_cb || read_file(dir, "pq_data.dat", &raw, &len) != 0 || len != (uint64_t)prb * n) {
                e = -15;
                goto done;
            }
            pq_rec = (uint8_t*)raw;
            raw = NULL;
            pq_off = (float*)malloc(sizeof(float) * (n ? n : 1));
            pq_codes = (uint8_t*)malloc((uint64_t)pq_nsq * (n ? n : 1));
            for (uint32_t i = 0; i < n; ++i) {
                memcpy(&pq_off[i], pq_rec + (uint64_t)i * prb, 4);
                memcpy(pq_codes + (uint64_t)i * pq_nsq, pq_rec + (uint64_t)i * prb + 4, pq_nsq);
            }
        }
        if (read_file(dir, "cell_assign.dat", &raw, &len) != 0 || len != 4ull * n) { e = -9; goto done; }
        cell_assign = (uint32_t*)raw;
        raw = NULL;
        const uint32_t rb = 4 + nsq;
        if (read_file(dir, "filter_data.dat", &raw, &len) != 0 || len != (uint64_t)rb * n) { e = -10; goto done; }
        rec = (uint8_t*)raw;
        raw = NULL;
        offsets = (float*)malloc(sizeof(float) * (n ? n : 1));
        codes = (uint8_t*)malloc((uint64_t)nsq * (n ? n : 1));
        for (uint32_t i = 0; i < n; ++i) {
            memcpy(&offsets[i], rec + (uint64_t)i * rb, 4);
            memcpy(codes + (uint64_t)i * nsq, rec + (uint64_t)i * rb + 4, nsq);
        }
        ix = po_load_arrays_pq(d, n, C, F, nsq, whether_norm, coarse, fine, feat, cell_assign,
                               codebook, offsets, codes, pq_nsq, pq_cb, pq_off, pq_codes, &e);
        if (ix != NULL && po_set_ip2cos(ix, (int)ip2cos) != 0) {
            po_free(ix);
            ix = NULL;
            e = -5;
        }
    }
done:
    free(raw);
    free(cell_assign);
    free(rec);
    free(coarse);
    free(fine);
    free(feat);
    free(codebook);
    free(offsets);
    free(codes);
    free(pq_cb);
    free(pq_off);
    free(pq_rec);
    free(pq_codes);
    if (err) *err = e;
    return ix;
}

int po_set_ip2cos(po_index* ix, int ip2cos) {
    if (ix == NULL || ip2cos < 0 || ip2cos > 1 || (ip2cos == 1 && ix->d < 2)) return -1;
    ix->ip2cos = ip2cos;
    return 0;
}

int po_info(const po_index* ix, uint32_t* d, uint32_t* n, uint32_t* coarse, uint32_t* fine,
            uint32_t* filter_nsq, uint32_t* lsq, int* whether_norm) {
    *d = ix->d;
    *n = ix->n;
    *coarse = ix->C;
    *fine = ix->F;
    *filter_nsq = ix->nsq;
    *lsq = ix->lsq;
    *whether_norm = ix->whether_norm;
    return 0;
}

const uint32_t* po_memory_to_local(const po_index* ix) { return ix->mem2local; }
const float* po_stationary(const po_index* ix) { return ix->stationary; }
const uint32_t* po_cell_start(const po_index* ix) { return ix->cell_start; }

/* ------------------------------------------------------------ distance kernels */

/* fvec_L2sqr SSE order (puck/puck/distances_simd.cpp:120-133, 210-236): four lane
 * accumulators over chunks of 4 (masked zero tail), then (l0+l1)+(l2+l3). */
static float l2sqr_sse(const float* x, const float* y, uint32_t d) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t i = 0;
    for (; i + 4 <= d; i += 4)
        for (int j = 0; j < 4; ++j) {
            float t = x[i + j] - y[i + j];
            float sq = t * t;
            acc[j] = acc[j] + sq;
        }
    if (i < d) {
        for (int j = 0; j < 4; ++j) {
            float t = (i + j < d) ? x[i + j] - y[i + j] : 0.0f;
            float sq = t * t;
            acc[j] = acc[j] + sq;
        }
    }
    float h0 = acc[0] + acc[1];
    float h1 = acc[2] + acc[3];
    return h0 + h1;
}

/* lookup_dist_table (puck_index.cpp:75-113): lane j sums subspaces m = j mod 4 in
 * increasing m; final (l0+l1)+(l2+l3). */
static float lookup_lut(const uint8_t* code, const float* lut, uint32_t nsq) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t m = 0; m < nsq; ++m) {
        float v = lut[(uint64_t)m * 256 + code[m]];
        acc[m & 3] = acc[m & 3] + v;
    }
    float h0 = acc[0] + acc[1];
    float h1 = acc[2] + acc[3];
    return h0 + h1;
}

/* Scan mode's sum for nsq a multiple of 4 up to 32 (the library's interleaved
 * scan, puck_gb300/csrc/scan_select.cu): step s looks up subspace (s + lane) mod
 * nsq, lane = memory id & 31, into partial s mod 4; then (p0 + p1) + (p2 + p3). */
static int scan_rotated(uint32_t nsq) { return nsq > 0 && nsq % 4 == 0 && nsq <= 32; }

static float lookup_lut_rotated(const uint8_t* code, const float* lut, uint32_t nsq, uint32_t mi) {
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const uint32_t lane = mi & 31u;
    for (uint32_t s = 0; s < nsq; ++s) {
        const uint32_t m = (s + lane) % nsq;
        acc[s & 3] = acc[s & 3] + lut[(uint64_t)m * 256 + code[m]];
    }
    float h0 = acc[0] + acc[1];
    float h1 = acc[2] + acc[3];
    return h0 + h1;
}

/* L2Sqr16Ext, AVX build (puck/tinker/method/hnsw_distfunc_opt_impl_inline.h:41-69):
 * lanes i<8 hold d_i^2 + d_{i+8}^2; lanes summed left to right. */
static float l2sqr16(const float* x, const float* q) {
    float lane[8];
    for (int i = 0; i < 8; ++i) {
        float a = x[i] - q[i];
        float b = x[i + 8] - q[i + 8];
        float a2 = a * a, b2 = b * b;
        lane[i] = a2 + b2;
    }
    float s = lane[0];
    for (int i = 1; i < 8; ++i) s = s + lane[i];
    return s;
}

/* L2SqrExt with fewer than 16 dims (hnsw_distfunc_opt_impl_inline.h:71-122): 4-lane
 * chunks, lanes summed left to right, then a scalar tail. */
static float l2sqr_ext(const float* x, const float* q, uint32_t qty) {
    float lane[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t i = 0;
    for (; i + 4 <= qty; i += 4)
        for (int j = 0; j < 4; ++j) {
            float t = x[i + j] - q[i + j];
            float sq = t * t;
            lane[j] = lane[j] + sq;
        }
    float s = ((lane[0] + lane[1]) + lane[2]) + lane[3];
    for (; i < qty; ++i) {
        float t = x[i] - q[i];
        float sq = t * t;
        s = s + sq;
    }
    return s;
}

/* rank_topN_points, second-level PQ branch (puck_index.cpp:402-427): candidates in
 * the given order, temp = (filter distance - |q|^2) + pq offset, then
 * += lookup_dist_table over the PQ table, into MaxHeap(topk). */
static void rerank_pq(const po_index* ix, const float* q, const uint32_t* tags, const float* fdist,
                      uint32_t stride, uint32_t cnt, po_heap* fin) {
    const uint32_t pq_nsq = ix->pq_nsq, lsq = ix->pq_lsq;
    float* lut = (float*)malloc(sizeof(float) * (uint64_t)pq_nsq * 256);
    for (uint32_t m = 0; m < pq_nsq; ++m)
        for (uint32_t j = 0; j < 256; ++j)
            lut[m * 256 + j] = l2sqr_sse(q + (uint64_t)m * lsq,
                                         ix->pq_codebook + ((uint64_t)m * 256 + j) * lsq, lsq);
    const float qn = dotf(q, q, ix->d);
    for (uint32_t idx = 0; idx < cnt; ++idx) {
        const uint32_t mi = tags[(uint64_t)idx * stride];
        float t = fdist[(uint64_t)idx * stride] - qn;
        if (ix->realtime) {
            /* realtime_insert_puck_index.cpp:466-499: inserted records by insert id, and
               the table summed subspace by subspace while below the top */
            const int ins = mi >= ix->n;
            const uint32_t id = mi - ix->n;
            t = t + (ins ? ix->ins_pq_off[id] : ix->pq_offsets[mi]);
            const uint8_t* code = ins ? ix->ins_pq_codes + (uint64_t)id * pq_nsq
                                      : ix->pq_codes + (uint64_t)mi * pq_nsq;
            for (uint32_t m = 0; m < pq_nsq && t < fin->val[1]; ++m) t = t + lut[m * 256 + code[m]];
            if (t < fin->val[1]) heap_update(fin, t, ins ? mi : ix->mem2local[mi]);
            continue;
        }
        t = t + ix->pq_offsets[mi];
        t = t + lookup_lut(ix->pq_codes + (uint64_t)mi * pq_nsq, lut, pq_nsq);
        if (t < fin->val[1]) heap_update(fin, t, ix->mem2local[mi]);
    }
    free(lut);
}

/* -------------------------------------------------------------------- search */

typedef struct {
    float* q;
    float* ip;
    float* cd;
    uint32_t* ctag;
    float* fd;
    uint32_t* ftag;
    float* lut;
    float* rdist;
    uint32_t* rtag;
} po_scratch;

static void scratch_alloc(po_scratch* s, const po_index* ix, const po_params* p) {
    uint32_t cmax = ix->C > ix->F ? ix->C : ix->F;
    s->q = (float*)malloc(sizeof(float) * ix->d);
    s->ip = (float*)malloc(sizeof(float) * cmax);
    s->cd = (float*)malloc(sizeof(float) * (p->search_coarse_count + 1));
    s->ctag = (uint32_t*)malloc(sizeof(uint32_t) * (p->search_coarse_count + 1));
    s->fd = (float*)malloc(sizeof(float) * ix->F);
    s->ftag = (uint32_t*)malloc(sizeof(uint32_t) * ix->F);
    s->lut = (float*)malloc(sizeof(float) * ix->nsq * 256);
    s->rdist = (float*)malloc(sizeof(float) * (p->filter_topk + 1));
    s->rtag = (uint32_t*)malloc(sizeof(uint32_t) * (p->filter_topk + 1));
}

static void scratch_free(po_scratch* s) {
    free(s->q);
    free(s->ip);
    free(s->cd);
    free(s->ctag);
    free(s->fd);
    free(s->ftag);
    free(s->lut);
    free(s->rdist);
    free(s->rtag);
}

/* compute_quantized_distance (puck_index.cpp:346-390); on a realtime index then the
 * cell's inserted points, newest first, none skipped, with memory id n + insert id
 * (realtime_insert_puck_index.cpp:398-453). The realtime count adds one per inserted
 * point, which only makes the walk recompute an unchanged pivot. */
static uint32_t scan_cell(const po_index* ix, uint64_t cell, float cell_dist, const float* lut,
                          po_heap* heap, uint64_t* scanned) {
    uint32_t start = ix->cell_start[cell];
    uint32_t cnt = ix->cell_start[cell + 1] - start;
    uint32_t updated = 0;
    for (uint32_t i = 0; i < cnt; ++i) {
        uint32_t mi = start + i;
        float t = (float)(2.0 * (double)cell_dist + (double)ix->offsets[mi]);
        if (t >= heap->val[1]) break;
        ++*scanned;
        t = t + lookup_lut(ix->codes + (uint64_t)mi * ix->nsq, lut, ix->nsq);
        if (t < heap->val[1]) {
            heap_update(heap, t, mi);
            ++updated;
        }
    }
    if (ix->realtime) {
        for (int32_t id = ix->ins_head[cell]; id >= 0; id = ix->ins_next[id]) {
            ++updated;
            ++*scanned;
            float t = (float)(2.0 * (double)cell_dist + (double)ix->ins_off[id]);
            t = t + lookup_lut(ix->ins_codes + (uint64_t)id * ix->nsq, lut, ix->nsq);
            if (t < heap->val[1]) heap_update(heap, t, ix->n + (uint32_t)id);
        }
    }
    return updated;
}

/* normalization (hierarchical_cluster_index.cpp:1513-1536). ip2cos = 1: the caller's
 * d - 1 values and a 0, not normalised (:1516-1520; the reference's memset there counts
 * bytes, so it never clears the last float, which the transform means to be 0).
 * Returns -2 for a zero-norm query of a whether_norm index (the reference dereferences
 * nullptr there). */
static int prep_query(const po_index* ix, po_scratch* s, const float* query) {
    const uint32_t d = ix->d;
    if (ix->ip2cos) {
        memcpy(s->q, query, sizeof(float) * (d - 1));
        s->q[d - 1] = 0.0f;
        return 0;
    }
    memcpy(s->q, query, sizeof(float) * d);
    if (ix->whether_norm) {
        float norm = sqrtf(dotf(s->q, s->q, d));
        if ((double)norm < 1e-6) return -2;
        float alpha = (float)(1.0 / (double)norm);
        for (uint32_t i = 0; i < d; ++i) s->q[i] = alpha * s->q[i];
    }
    return 0;
}

static int search_one(const po_index* ix, const po_params* p, po_scratch* s, const float* query,
                      uint32_t topk, float* dist, uint32_t* ids, uint32_t* result_num,
                      po_trace* trace) {
    const uint32_t d = ix->d, C = ix->C, F = ix->F, nsq = ix->nsq;
    uint32_t P = p->search_coarse_count < C ? p->search_coarse_count : C;
    const uint32_t T = p->filter_topk;
    if (topk > p->topk || query == NULL || P == 0 || T == 0 || topk == 0) return -1;

    /* normalization (hierarchical_cluster_index.cpp:1513-1536) */
    if (prep_query(ix, s, query) != 0) return -2;
    const float* q = s->q;

    /* search_nearest_coarse_cluster (hierarchical_cluster_index.cpp:700-727) */
    po_heap ch;
    heap_init(&ch, P, s->cd, s->ctag);
    for (uint32_t c = 0; c < C; ++c) {
        float ipc = dotf(ix->coarse + (uint64_t)c * d, q, d);
        float cdv = ix->coarse_norms[c] - ipc;
        if (cdv < ch.val[1]) heap_update(&ch, cdv, c);
    }
    heap_reorder(&ch);

    /* pre_filter_search -> get_dist_table (quantization.cpp:260-270) */
    for (uint32_t m = 0; m < nsq; ++m)
        for (uint32_t j = 0; j < 256; ++j)
            s->lut[m * 256 + j] = l2sqr_sse(q + (uint64_t)m * ix->lsq,
                                            ix->codebook + ((uint64_t)m * 256 + j) * ix->lsq, ix->lsq);

    /* fine stage (puck_index.cpp:494-504): full heap sort of -q.f */
    po_heap fh;
    heap_init(&fh, F, s->fd, s->ftag);
    for (uint32_t f = 0; f < F; ++f) {
        float ipf = dotf(ix->fine + (uint64_t)f * d, q, d);
        heap_update(&fh, -ipf, f);
    }
    heap_reorder(&fh);

    /* walk (puck_index.cpp:513-556) */
    po_heap rh;
    heap_init(&rh, T, s->rdist, s->rtag);
    const float qnorm = dotf(q, q, d);
    const double rr = p->radius_rate;
    float pivot = (float)((double)(rh.val[1] - qnorm) / rr / 2.0);
    uint64_t scanned = 0, cells_scanned = 0, visited = 0, low_stat = 0;
    for (uint32_t l = 0; l < P; ++l) {
        const uint32_t c = s->ctag[l];
        const float cdl = s->cd[l];
        const float* stat = ix->stationary + (uint64_t)c * F;
        const float min_dist = ix->min_dist_offset[c] + cdl;
        float max_stat = (pivot - cdl) - s->fd[0];
        if (trace)
            for (uint32_t f = 0; f < F; ++f) low_stat += stat[f] < max_stat;
        for (uint32_t idx = 0; idx < F; ++idx) {
            if (s->fd[idx] + min_dist >= pivot) break;
            ++visited;
            const uint32_t k = s->ftag[idx];
            if (stat[k] >= max_stat) continue;
            const float cell_dist = (cdl + stat[k]) + s->fd[idx];
            ++cells_scanned;
            uint32_t upd = scan_cell(ix, (uint64_t)c * F + k, cell_dist, s->lut, &rh, &scanned);
            if (upd > 0) pivot = (float)((double)(rh.val[1] - qnorm) / rr / 2.0);
            float cand = (pivot - cdl) - s->fd[idx];
            if (cand < max_stat) max_stat = cand;
        }
    }
    if (heap_count(&rh) < T) heap_reorder(&rh);
    const uint32_t cnt = heap_count(&rh);

    if (trace) {
        if (trace->coarse_tag) memcpy(trace->coarse_tag, s->ctag, sizeof(uint32_t) * P);
        if (trace->coarse_dist) memcpy(trace->coarse_dist, s->cd, sizeof(float) * P);
        if (trace->filter_tag) memcpy(trace->filter_tag, s->rtag, sizeof(uint32_t) * T);
        if (trace->filter_dist) memcpy(trace->filter_dist, s->rdist, sizeof(float) * T);
        if (trace->lut) memcpy(trace->lut, s->lut, sizeof(float) * nsq * 256);
        trace->filter_cnt = cnt;
        trace->scanned_points = scanned;
        trace->scanned_cells = cells_scanned;
        trace->visited_cells = visited;
        trace->low_stat_cells = low_stat;
    }

    /* rank_topN_points, Puck-Flat branch (puck_index.cpp:428-457) */
    po_heap fin;
    heap_init(&fin, topk, dist, ids);
    if (ix->pq_nsq) {
        rerank_pq(ix, q, s->rtag, s->rdist, 1, cnt, &fin);
        heap_reorder(&fin);
        *result_num = heap_count(&fin);
        return 0;
    }
    for (uint32_t idx = 0; idx < cnt; ++idx) {
        const uint32_t mi = s->rtag[idx];
        const int ins = mi >= ix->n;  /* realtime: an inserted point's kept vector */
        const float* x = ins ? ix->ins_feat + (uint64_t)(mi - ix->n) * d : ix->feat + (uint64_t)mi * d;
        float t = 0.0f;
        uint32_t m = 0;
        for (; m + 16 <= d && t < fin.val[1]; m += 16) t = t + l2sqr16(x + m, q + m);
        if (t < fin.val[1]) {
            if (d - m > 0) t = t + l2sqr_ext(x + m, q + m, d - m);
            heap_update(&fin, t, ins ? mi : ix->mem2local[mi]);
        }
    }
    heap_reorder(&fin);
    *result_num = heap_count(&fin);
    return 0;
}

/* ---------------------------------------------------------------- scan mode */
/* Definition of the library's scan mode (test infrastructure): the reference's
 * normalisation, coarse heap and LUT, then EVERY record of the probed coarse
 * clusters gets the reference's per-point distance
 *   t = (float)(2.0 * ((cd + stationary) + fd) + offset) + lookup_dist_table
 * (puck_index.cpp:360-368, 539-540), the table sum in the reference's order, or in
 * the rotated order of lookup_lut_rotated where the library's interleaved scan
 * applies (nsq a multiple of 4 up to 32); the filter_topk smallest by (t, memory id),
 * ascending, are reranked exactly as rank_topN_points does (puck_index.cpp:428-457). */
typedef struct {
    float t;
    uint32_t mi;
} po_cand;

static int cmp_cand(const void* a, const void* b) {
    const po_cand* x = (const po_cand*)a;
    const po_cand* y = (const po_cand*)b;
    if (x->t < y->t) return -1;
    if (y->t < x->t) return 1;
    return (x->mi > y->mi) - (x->mi < y->mi);
}

static int search_scan_one(const po_index* ix, const po_params* p, po_scratch* s,
                           const float* query, uint32_t topk, float* dist, uint32_t* ids,
                           uint32_t* result_num, po_trace* trace) {
    const uint32_t d = ix->d, C = ix->C, F = ix->F, nsq = ix->nsq;
    uint32_t P = p->search_coarse_count < C ? p->search_coarse_count : C;
    const uint32_t T = p->filter_topk;
    if (topk > p->topk || query == NULL || P == 0 || T == 0 || topk == 0) return -1;
    if (prep_query(ix, s, query) != 0) return -2;
    const float* q = s->q;
    po_heap ch;
    heap_init(&ch, P, s->cd, s->ctag);
    for (uint32_t c = 0; c < C; ++c) {
        float ipc = dotf(ix->coarse + (uint64_t)c * d, q, d);
        float cdv = ix->coarse_norms[c] - ipc;
        if (cdv < ch.val[1]) heap_update(&ch, cdv, c);
    }
    heap_reorder(&ch);
    for (uint32_t m = 0; m < nsq; ++m)
        for (uint32_t j = 0; j < 256; ++j)
            s->lut[m * 256 + j] = l2sqr_sse(q + (uint64_t)m * ix->lsq,
                                            ix->codebook + ((uint64_t)m * 256 + j) * ix->lsq, ix->lsq);
    for (uint32_t f = 0; f < F; ++f) s->fd[f] = -dotf(ix->fine + (uint64_t)f * d, q, d);
    uint64_t total = 0;
    for (uint32_t l = 0; l < P; ++l) {
        const uint32_t c = s->ctag[l];
        total += ix->cell_start[(uint64_t)c * F + F] - ix->cell_start[(uint64_t)c * F];
        if (ix->realtime)
            for (uint32_t f = 0; f < F; ++f) {
                const uint64_t cell = (uint64_t)c * F + f;
                total += ix->cell_cnt[cell] - (ix->cell_start[cell + 1] - ix->cell_start[cell]);
            }
    }
    po_cand* cand = (po_cand*)malloc(sizeof(po_cand) * (total ? total : 1));
    uint64_t nc = 0;
    const int rot = scan_rotated(nsq);
    for (uint32_t l = 0; l < P; ++l) {
        const uint32_t c = s->ctag[l];
        const float cdl = s->cd[l];
        for (uint32_t f = 0; f < F; ++f) {
            const uint64_t cell = (uint64_t)c * F + f;
            const float cell_dist = (cdl + ix->stationary[cell]) + s->fd[f];
            for (uint32_t mi = ix->cell_start[cell]; mi < ix->cell_start[cell + 1]; ++mi) {
                float t = (float)(2.0 * (double)cell_dist + (double)ix->offsets[mi]);
                t = t + (rot ? lookup_lut_rotated(ix->codes + (uint64_t)mi * nsq, s->lut, nsq, mi)
                             : lookup_lut(ix->codes + (uint64_t)mi * nsq, s->lut, nsq));
                cand[nc].t = t;
                cand[nc].mi = mi;
                ++nc;
            }
            /* realtime: the cell's inserted points, memory id n + insert id */
            for (int32_t id = ix->realtime ? ix->ins_head[cell] : -1; id >= 0; id = ix->ins_next[id]) {
                const uint32_t mi = ix->n + (uint32_t)id;
                float t = (float)(2.0 * (double)cell_dist + (double)ix->ins_off[id]);
                const uint8_t* code = ix->ins_codes + (uint64_t)id * nsq;
                t = t + (rot ? lookup_lut_rotated(code, s->lut, nsq, mi) : lookup_lut(code, s->lut, nsq));
                cand[nc].t = t;
                cand[nc].mi = mi;
                ++nc;
            }
        }
    }
    qsort(cand, nc, sizeof(po_cand), cmp_cand);
    const uint32_t cnt = nc < T ? (uint32_t)nc : T;
    if (trace) {
        if (trace->coarse_tag) memcpy(trace->coarse_tag, s->ctag, sizeof(uint32_t) * P);
        if (trace->coarse_dist) memcpy(trace->coarse_dist, s->cd, sizeof(float) * P);
        for (uint32_t i = 0; i < T; ++i) {
            if (trace->filter_tag) trace->filter_tag[i] = i < cnt ? cand[i].mi : 0xFFFFFFFFu;
            if (trace->filter_dist) trace->filter_dist[i] = i < cnt ? cand[i].t : 0.0f;
        }
        if (trace->lut) memcpy(trace->lut, s->lut, sizeof(float) * nsq * 256);
        trace->filter_cnt = cnt;
        trace->scanned_points = nc;
    }
    po_heap fin;
    heap_init(&fin, topk, dist, ids);
    if (ix->pq_nsq) {
        rerank_pq(ix, q, &cand[0].mi, &cand[0].t, sizeof(po_cand) / sizeof(float), cnt, &fin);
        heap_reorder(&fin);
        *result_num = heap_count(&fin);
        free(cand);
        return 0;
    }
    for (uint32_t idx = 0; idx < cnt; ++idx) {
        const uint32_t mi = cand[idx].mi;
        const int ins = mi >= ix->n;
        const float* x = ins ? ix->ins_feat + (uint64_t)(mi - ix->n) * d : ix->feat + (uint64_t)mi * d;
        float t = 0.0f;
        uint32_t m = 0;
        for (; m + 16 <= d && t < fin.val[1]; m += 16) t = t + l2sqr16(x + m, q + m);
        if (t < fin.val[1]) {
            if (d - m > 0) t = t + l2sqr_ext(x + m, q + m, d - m);
            heap_update(&fin, t, ins ? mi : ix->mem2local[mi]);
        }
    }
    heap_reorder(&fin);
    *result_num = heap_count(&fin);
    free(cand);
    return 0;
}

int po_search_scan(const po_index* ix, const po_params* p, const float* q, uint32_t topk,
                   float* dist, uint32_t* ids, uint32_t* result_num, po_trace* trace) {
    po_scratch s;
    scratch_alloc(&s, ix, p);
    int rc = search_scan_one(ix, p, &s, q, topk, dist, ids, result_num, trace);
    scratch_free(&s);
    return rc;
}

int po_search(const po_index* ix, const po_params* p, const float* q, uint32_t topk, float* dist,
              uint32_t* ids, uint32_t* result_num, po_trace* trace) {
    po_scratch s;
    scratch_alloc(&s, ix, p);
    int rc = search_one(ix, p, &s, q, topk, dist, ids, result_num, trace);
    scratch_free(&s);
    return rc;
}

typedef struct {
    const po_index* ix;
    const po_params* p;
    uint32_t n, topk;
    const float* q;
    float* dist;
    uint32_t* ids;
    int32_t* status;
    int scan;
    atomic_uint_fast64_t next;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* job = (batch_job*)arg;
    po_scratch s;
    scratch_alloc(&s, job->ix, job->p);
    for (;;) {
        uint64_t i = atomic_fetch_add(&job->next, 1);
        if (i >= job->n) break;
        uint32_t rn = 0;
        int rc = job->scan
                     ? search_scan_one(job->ix, job->p, &s, job->q + i * (job->ix->d - (uint32_t)job->ix->ip2cos), job->topk,
                                       job->dist + i * job->topk, job->ids + i * job->topk, &rn,
                                       NULL)
                     : search_one(job->ix, job->p, &s, job->q + i * (job->ix->d - (uint32_t)job->ix->ip2cos), job->topk,
                                  job->dist + i * job->topk, job->ids + i * job->topk, &rn, NULL);
        if (job->status) job->status[i] = rc;
    }
    scratch_free(&s);
    return NULL;
}

static int batch_run(const po_index* ix, const po_params* p, uint32_t n, const float* q,
                     uint32_t topk, float* dist, uint32_t* ids, int32_t* status, int nthreads,
                     int scan) {
    batch_job job;
    job.scan = scan;
    job.ix = ix;
    job.p = p;
    job.n = n;
    job.topk = topk;
    job.q = q;
    job.dist = dist;
    job.ids = ids;
    job.status = status;
    atomic_init(&job.next, 0);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &job);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    return 0;
}

int po_search_batch(const po_index* ix, const po_params* p, uint32_t n, const float* q,
                    uint32_t topk, float* dist, uint32_t* ids, int32_t* status, int nthreads) {
    return batch_run(ix, p, n, q, topk, dist, ids, status, nthreads, 0);
}

int po_search_scan_batch(const po_index* ix, const po_params* p, uint32_t n, const float* q,
                         uint32_t topk, float* dist, uint32_t* ids, int32_t* status,
                         int nthreads) {
    return batch_run(ix, p, n, q, topk, dist, ids, status, nthreads, 1);
}

/* ------------------------------------------------------------------ assign */

/* One quantizer's pass of puck_assign (puck_index.cpp:644-679): per subspace k, the
 * nearest codeword of r's slice by nearest_center (kmeans.cpp:221-258) over the ks = 256
 * codewords, then saxpy(-1) of that codeword from the slice. cbn: codeword norms. */
static void assign_encode(float* r, const float* cb, const float* cbn, uint32_t nsq, uint32_t lsq,
                          uint8_t* codes) {
    for (uint32_t k = 0; k < nsq; ++k) {
        float* s = r + (uint64_t)k * lsq;
        const float pn = dotf(s, s, lsq);
        float best = FLT_MAX;
        uint32_t bi = 0;
        for (uint32_t c = 0; c < 256; ++c) {
            const float* cw = cb + ((uint64_t)k * 256 + c) * lsq;
            const float t = pn + cbn[(uint64_t)k * 256 + c];
            const float cur = (float)((double)t - 2.0 * (double)dotf(s, cw, lsq));
            if (cur < best) {
                best = cur;
                bi = c;
            }
        }
        codes[k] = (uint8_t)bi;
        const float* cw = cb + ((uint64_t)k * 256 + bi) * lsq;
        for (uint32_t t = 0; t < lsq; ++t) s[t] = s[t] + -1.0f * cw[t];
    }
}

/* Quantization::decode (quantization.cpp:228-242) then set_static_value_of_formula
 * (:244-258): 2 * sdot(decoded residual, vocab), then vocab += decoded residual. */
static float assign_offset(float* vocab, float* dec, const float* cb, const uint8_t* codes,
                           uint32_t nsq, uint32_t lsq) {
    for (uint32_t k = 0; k < nsq; ++k)
        memcpy(dec + (uint64_t)k * lsq, cb + ((uint64_t)k * 256 + codes[k]) * lsq,
               sizeof(float) * lsq);
    const uint32_t d = nsq * lsq;
    const float off = 2 * dotf(dec, vocab, d);
    for (uint32_t t = 0; t < d; ++t) vocab[t] += dec[t];
    return off;
}

static float* codeword_norms(const float* cb, uint32_t nsq, uint32_t lsq) {
    float* out = (float*)malloc(sizeof(float) * (uint64_t)nsq * 256);
    for (uint64_t e = 0; e < (uint64_t)nsq * 256; ++e) out[e] = dotf(cb + e * lsq, cb + e * lsq, lsq);
    return out;
}

void po_puck_assign(uint32_t d, uint64_t n, const float* base, const uint32_t* cell_assign,
                    const float* coarse, const float* fine, uint32_t F, const float* fcb,
                    uint32_t fnsq, const float* pcb, uint32_t pnsq, float* f_off,
                    uint8_t* f_codes, float* p_off, uint8_t* p_codes) {
    const uint32_t flsq = d / fnsq, plsq = pnsq ? d / pnsq : 0;
    float* fn = codeword_norms(fcb, fnsq, flsq);
    float* pn = pnsq ? codeword_norms(pcb, pnsq, plsq) : NULL;
    float* r = (float*)malloc(sizeof(float) * d);
    float* v = (float*)malloc(sizeof(float) * d);
    float* dec = (float*)malloc(sizeof(float) * d);
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t cell = cell_assign[i], c = cell / F, f = cell % F;
        const float* x = base + i * d;
        /* residual: saxpy(-1, coarse) then saxpy(-1, fine) (puck_index.cpp:638-643) */
        for (uint32_t t = 0; t < d; ++t) {
            r[t] = x[t] + -1.0f * coarse[(uint64_t)c * d + t];
            r[t] = r[t] + -1.0f * fine[(uint64_t)f * d + t];
        }
        assign_encode(r, fcb, fn, fnsq, flsq, f_codes + i * fnsq);
        if (pnsq) assign_encode(r, pcb, pn, pnsq, plsq, p_codes + i * pnsq);
        /* offsets: vocab = coarse, saxpy(1, fine) (puck_index.cpp:682-694) */
        for (uint32_t t = 0; t < d; ++t)
            v[t] = coarse[(uint64_t)c * d + t] + 1.0f * fine[(uint64_t)f * d + t];
        f_off[i] = assign_offset(v, dec, fcb, f_codes + i * fnsq, fnsq, flsq);
        if (pnsq) p_off[i] = assign_offset(v, dec, pcb, p_codes + i * pnsq, pnsq, plsq);
    }
    free(fn);
    free(pn);
    free(r);
    free(v);
    free(dec);
}

void po_nearest_center(uint32_t dim, const float* centroids, uint64_t k, const float* x,
                       uint64_t n, int32_t* assign, float* dis) {
    float* cn = (float*)malloc(sizeof(float) * (k ? k : 1));
    for (uint64_t c = 0; c < k; ++c) cn[c] = dotf(centroids + c * dim, centroids + c * dim, dim);
    for (uint64_t j = 0; j < n; ++j) {
        const float* xj = x + j * dim;
        float pn = dotf(xj, xj, dim);
        float best = FLT_MAX;
        uint32_t bi = 0;
        for (uint64_t c = 0; c < k; ++c) {
            float s = pn + cn[c];
            float cur = (float)((double)s - 2.0 * (double)dotf(xj, centroids + c * dim, dim));
            if (cur < best) {
                best = cur;
                bi = (uint32_t)c;
            }
        }
        assign[j] = (int32_t)bi;
        dis[j] = best;
    }
    free(cn);
}

typedef struct {
    float v;
    int32_t id;
} pair_fi;

static int cmp_pair_fi(const void* a, const void* b) {
    const pair_fi* x = (const pair_fi*)a;
    const pair_fi* y = (const pair_fi*)b;
    if (x->v < y->v) return -1;
    if (y->v < x->v) return 1;
    return (x->id > y->id) - (x->id < y->id);
}

void po_nearest_cell_assign(uint32_t dim, const float* coarse, uint32_t C, const float* fine,
                            uint32_t F, const float* x, uint64_t n, uint32_t* cell,
                            float* cell_dist) {
    float* cnorm = (float*)malloc(sizeof(float) * C);
    float* fneg = (float*)malloc(sizeof(float) * F);
    float* fn = (float*)malloc(sizeof(float) * F);
    float* stat = (float*)malloc(sizeof(float) * (uint64_t)C * F);
    float* fip = (float*)malloc(sizeof(float) * F);
    pair_fi* list = (pair_fi*)malloc(sizeof(pair_fi) * C);
    for (uint32_t c = 0; c < C; ++c) cnorm[c] = dotf(coarse + (uint64_t)c * dim, coarse + (uint64_t)c * dim, dim) / 2;
    for (uint32_t f = 0; f < F; ++f) {
        fn[f] = dotf(fine + (uint64_t)f * dim, fine + (uint64_t)f * dim, dim) / 2;
        fneg[f] = 0 - sqrtf(fn[f]);
    }
    for (uint32_t c = 0; c < C; ++c)
        for (uint32_t f = 0; f < F; ++f)
            stat[(uint64_t)c * F + f] =
                fn[f] + dotf(fine + (uint64_t)f * dim, coarse + (uint64_t)c * dim, dim);
    for (uint64_t j = 0; j < n; ++j) {
        const float* xj = x + j * dim;
        float qn = dotf(xj, xj, dim) / 2;
        for (uint32_t c = 0; c < C; ++c) {
            float ipc = dotf(coarse + (uint64_t)c * dim, xj, dim);
            list[c].id = (int32_t)c;
            list[c].v = (cnorm[c] - ipc) + qn;
        }
        for (uint32_t f = 0; f < F; ++f) fip[f] = dotf(fine + (uint64_t)f * dim, xj, dim);
        qsort(list, C, sizeof(pair_fi), cmp_pair_fi);
        float best = FLT_MAX;
        int32_t best_id = -1;
        for (uint32_t i = 0; i < C; ++i) {
            const int32_t cc = list[i].id;
            const float term = list[i].v;
            for (uint32_t f = 0; f < F; ++f) {
                if (sqrtf(best) - fneg[f] < sqrtf(term)) break;
                float score = (term - fip[f]) + stat[(uint64_t)cc * F + f];
                if (score < best) {
                    best = score;
                    best_id = cc * (int32_t)F + (int32_t)f;
                }
            }
        }
        cell[j] = (uint32_t)best_id;
        cell_dist[j] = best;
    }
    free(cnorm);
    free(fneg);
    free(fn);
    free(stat);
    free(fip);
    free(list);
}

/* ------------------------------------------------------------- realtime insert */

/* RealtimeInsertPuckIndex::init (realtime_insert_puck_index.cpp:225-272) over a loaded
 * index: every cell's insert count starts at its base count, no inserted points. */
int po_realtime_open(po_index* ix) {
    if (ix == NULL) return -1;
    if (ix->realtime) return 0;
    const uint64_t cells = (uint64_t)ix->C * ix->F;
    ix->ins_head = (int32_t*)malloc(sizeof(int32_t) * cells);
    ix->cell_cnt = (uint32_t*)malloc(sizeof(uint32_t) * cells);
    for (uint64_t i = 0; i < cells; ++i) {
        ix->ins_head[i] = -1;
        ix->cell_cnt[i] = ix->cell_start[i + 1] - ix->cell_start[i];
    }
    ix->realtime = 1;
    return 0;
}

static void ins_reserve(po_index* ix) {
    if (ix->ins_n < ix->ins_cap) return;
    const uint32_t cap = ix->ins_cap ? 2 * ix->ins_cap : 64;
    ix->ins_cell = (uint32_t*)realloc(ix->ins_cell, sizeof(uint32_t) * cap);
    ix->ins_next = (int32_t*)realloc(ix->ins_next, sizeof(int32_t) * cap);
    ix->ins_off = (float*)realloc(ix->ins_off, sizeof(float) * cap);
    ix->ins_codes = (uint8_t*)realloc(ix->ins_codes, (uint64_t)ix->nsq * cap);
    if (ix->pq_nsq) {
        ix->ins_pq_off = (float*)realloc(ix->ins_pq_off, sizeof(float) * cap);
        ix->ins_pq_codes = (uint8_t*)realloc(ix->ins_pq_codes, (uint64_t)ix->pq_nsq * cap);
    } else {
        ix->ins_feat = (float*)realloc(ix->ins_feat, sizeof(float) * (uint64_t)ix->d * cap);
    }
    ix->ins_cap = cap;
}

/* RealtimeInsertPuckIndex::insert (realtime_insert_puck_index.cpp:273-337):
 *   single_build (hierarchical_cluster_index.cpp:1455-1494): normalisation, then
 *     nearest_cell_assign (:1042-1085) on the index's live stationary terms (a cell
 *     empty in the base keeps sqrt(FLT_MAX) there, so it is never chosen);
 *   puck_single_assign (puck_index.cpp:938-988): the encode of puck_assign;
 *   the point goes to the head of its cell's list; a cell whose count becomes 1 gets
 *   the stationary term c.f - f.f.
 * Returns the inserted point's local id (n + insert id), or -1. */
int64_t po_insert(po_index* ix, const float* feature) {
    if (ix == NULL || !ix->realtime || feature == NULL) return -1;
    const uint32_t d = ix->d, C = ix->C, F = ix->F;
    float* x = (float*)malloc(sizeof(float) * d);
    memcpy(x, feature, sizeof(float) * d);
    if (ix->whether_norm) {
        const float norm = sqrtf(dotf(x, x, d));
        if (norm < 1e-6) {
            free(x);
            return -1;
        }
        const float alpha = (float)(1.0 / (double)norm);
        for (uint32_t i = 0; i < d; ++i) x[i] = alpha * x[i];
    }
    pair_fi* list = (pair_fi*)malloc(sizeof(pair_fi) * C);
    float* fip = (float*)malloc(sizeof(float) * F);
    const float qn = dotf(x, x, d) / 2;
    for (uint32_t c = 0; c < C; ++c) {
        list[c].id = (int32_t)c;
        list[c].v = (ix->coarse_norms[c] - dotf(ix->coarse + (uint64_t)c * d, x, d)) + qn;
    }
    for (uint32_t f = 0; f < F; ++f) fip[f] = dotf(ix->fine + (uint64_t)f * d, x, d);
    qsort(list, C, sizeof(pair_fi), cmp_pair_fi);
    float best = FLT_MAX;
    int32_t best_id = -1;
    for (uint32_t i = 0; i < C; ++i) {
        const int32_t cc = list[i].id;
        const float term = list[i].v;
        for (uint32_t f = 0; f < F; ++f) {
            const float* fv = ix->fine + (uint64_t)f * d;
            const float fneg = 0 - sqrtf(dotf(fv, fv, d) / 2);
            if (sqrtf(best) - fneg < sqrtf(term)) break;
            const float score = (term - fip[f]) + ix->stationary[(uint64_t)cc * F + f];
            if (score < best) {
                best = score;
                best_id = cc * (int32_t)F + (int32_t)f;
            }
        }
    }
    free(list);
    free(fip);
    if (best_id < 0) {
        free(x);
        return -1;
    }
    ins_reserve(ix);
    const uint32_t id = ix->ins_n;
    const uint32_t cell = (uint32_t)best_id;
    po_puck_assign(d, 1, x, &cell, ix->coarse, ix->fine, F, ix->codebook, ix->nsq,
                   ix->pq_nsq ? ix->pq_codebook : NULL, ix->pq_nsq, ix->ins_off + id,
                   ix->ins_codes + (uint64_t)id * ix->nsq, ix->pq_nsq ? ix->ins_pq_off + id : NULL,
                   ix->pq_nsq ? ix->ins_pq_codes + (uint64_t)id * ix->pq_nsq : NULL);
    if (!ix->pq_nsq) memcpy(ix->ins_feat + (uint64_t)id * d, x, sizeof(float) * d);
    ix->ins_cell[id] = cell;
    ix->ins_next[id] = ix->ins_head[cell];
    ix->ins_head[cell] = (int32_t)id;
    ix->ins_n = id + 1;
    if (++ix->cell_cnt[cell] == 1) {
        const float* cv = ix->coarse + (uint64_t)(cell / F) * d;
        const float* fv = ix->fine + (uint64_t)(cell % F) * d;
        float st = dotf(cv, fv, d);
        st -= dotf(fv, fv, d);
        ix->stationary[cell] = st;
    }
    free(x);
    return (int64_t)ix->n + id;
}

/* The inserted points' records: cell, filter offset and codes, second-level PQ offset
 * and codes (NULL outputs are skipped). Returns the number of inserted points. */
uint32_t po_inserted_records(const po_index* ix, uint32_t* cell, float* off, uint8_t* codes,
                             float* pq_off, uint8_t* pq_codes) {
    const uint32_t m = ix->ins_n;
    if (cell) memcpy(cell, ix->ins_cell, sizeof(uint32_t) * m);
    if (off) memcpy(off, ix->ins_off, sizeof(float) * m);
    if (codes) memcpy(codes, ix->ins_codes, (uint64_t)ix->nsq * m);
    if (pq_off && ix->pq_nsq) memcpy(pq_off, ix->ins_pq_off, sizeof(float) * m);
    if (pq_codes && ix->pq_nsq) memcpy(pq_codes, ix->ins_pq_codes, (uint64_t)ix->pq_nsq * m);
    return m;
}

