// Host side of Index::init() for Puck-Flat indexes: reads the reference's index
// files, builds Puck's memory order and uploads the device-resident layout.
//
//   read_index_files  HierarchicalClusterIndex::read_model_file / read_coodbooks /
//                     load_cell_assign / read_feature_index
//                     (puck/hierarchical_cluster/hierarchical_cluster_index.cpp:220-514,
//                     635-676) and Quantization::load (puck/puck/quantization.cpp:152-226)
//   build_host_index  PuckIndex::convert_local_to_memory_idx (puck/puck/puck_index.cpp:229-309)
//   upload_index      device copies; norms, stationary = 0.5|f|^2 + f.c and the
//                     empty-cell / min_dist_offset fix-up are computed on the GPU with
//                     the same float order as the reference
#include <sys/stat.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>

#include "pgpu_internal.h"

namespace pgpu {
namespace {

bool file_size(const std::string& path, uint64_t* size) {
    struct stat stt;
    if (::stat(path.c_str(), &stt) != 0) return false;
    *size = (uint64_t)stt.st_size;
    return true;
}

bool read_all(const std::string& path, char* dst, uint64_t len) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    uint64_t got = 0;
    while (got < len) {
        size_t r = std::fread(dst + got, 1, (size_t)std::min<uint64_t>(len - got, 1ull << 30), f);
        if (r == 0) break;
        got += r;
    }
    std::fclose(f);
    return got == len;
}

// fvecs with exactly `rows` rows of `dim` floats (check_file_length_info +
// read_fvec_format); the dimension prefixes are stripped in place.
bool read_fvecs(const std::string& path, uint32_t dim, uint64_t rows, float* out, std::string* err) {
    uint64_t sz = 0;
    const uint64_t rb = 4ull + 4ull * dim;
    if (!file_size(path, &sz) || sz != rows * rb) {
        *err = "file length check failed: " + path;
        return false;
    }
    // Read in blocks of rows into a bounce buffer, copy the payloads out.
    const uint64_t block_rows = std::max<uint64_t>(1, (64ull << 20) / rb);
    std::vector<char> buf((size_t)std::min<uint64_t>(rows, block_rows) * rb + 1);
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        *err = "cannot open " + path;
        return false;
    }
    for (uint64_t r0 = 0; r0 < rows; r0 += block_rows) {
        const uint64_t nr = std::min(block_rows, rows - r0);
        if (std::fread(buf.data(), 1, (size_t)(nr * rb), f) != nr * rb) {
            std::fclose(f);
            *err = "short read: " + path;
            return false;
        }
        for (uint64_t i = 0; i < nr; ++i) {
            int32_t dd;
            std::memcpy(&dd, buf.data() + i * rb, 4);
            if ((uint32_t)dd != dim) {
                std::fclose(f);
                *err = "fvecs dimension mismatch: " + path;
                return false;
            }
            std::memcpy(out + (r0 + i) * dim, buf.data() + i * rb + 4, 4ull * dim);
        }
    }
    std::fclose(f);
    return true;
}

template <class Fn>
void parallel_for(uint64_t n, Fn fn) {
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096) nt = 1;
    std::vector<std::thread> th;
    const uint64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=] { fn(b, e); });
    }
    for (auto& x : th) x.join();
}

}  // namespace

int read_index_files(const char* dir, pgpu_index_arrays* a, std::vector<char>& storage,
                     std::string* err) {
    const std::string base(dir ? dir : "");
    // index.dat: size_t length, then the packed structural config
    // (hierarchical_cluster_index.cpp:522-567).
    uint64_t sz = 0;
    const std::string conf_path = base + "/index.dat";
    if (!file_size(conf_path, &sz) || sz < 8 + 43) {
        *err = "cannot read " + conf_path;
        return PGPU_E_IO;
    }
    std::vector<char> conf(sz);
    if (!read_all(conf_path, conf.data(), sz)) {
        *err = "cannot read " + conf_path;
        return PGPU_E_IO;
    }
    const char* p = conf.data() + 8;
    int32_t index_type;
    uint32_t d, n, filter_nsq, ks, nsq, ks2, ip2cos, C, F;
    uint8_t whether_norm, whether_filter, whether_pq;
    std::memcpy(&index_type, p, 4); p += 4;
    std::memcpy(&d, p, 4); p += 4;
    whether_norm = (uint8_t)*p; p += 1;
    std::memcpy(&n, p, 4); p += 4;
    whether_filter = (uint8_t)*p; p += 1;
    std::memcpy(&filter_nsq, p, 4); p += 4;
    std::memcpy(&ks, p, 4); p += 4;
    whether_pq = (uint8_t)*p; p += 1;
    std::memcpy(&nsq, p, 4); p += 4;
    std::memcpy(&ks2, p, 4); p += 4;
    std::memcpy(&ip2cos, p, 4); p += 4;
    std::memcpy(&C, p, 4); p += 4;
    std::memcpy(&F, p, 4); p += 4;
    (void)ks2;
    if (index_type != 1) {
        *err = "index_type is not PUCK";
        return PGPU_E_UNSUPPORTED;
    }
    // ip2cos = 2 is not searchable as the reference has it: PySearcher takes feature_dim - 1
    // values per query (py_api_wrapper.cpp:104-106) while normalization() widens only for
    // ip2cos = 1 (hierarchical_cluster_index.cpp:1516), so the search reads past the query
    if (!whether_filter || ks != 256 || ip2cos > 1 || (whether_pq && ks2 != 256)) {
        *err = "unsupported index (needs whether_filter, ks=256, ip2cos 0 or 1)";
        return PGPU_E_UNSUPPORTED;
    }
    if (ip2cos == 1 && d < 2) {
        *err = "ip2cos index needs feature_dim >= 2";
        return PGPU_E_UNSUPPORTED;
    }
    if (whether_pq && (nsq == 0 || nsq > d || d % nsq != 0)) {
        *err = "inconsistent PQ config (feature_dim must be a multiple of nsq)";
        return PGPU_E_UNSUPPORTED;
    }
    if (d == 0 || filter_nsq == 0 || filter_nsq > d || d % filter_nsq != 0 || C == 0 || F == 0) {
        *err = "inconsistent index config (feature_dim must be a multiple of filter_nsq)";
        return PGPU_E_UNSUPPORTED;
    }
    const uint32_t lsq = d / filter_nsq;
    const uint64_t fl_coarse = (uint64_t)C * d, fl_fine = (uint64_t)F * d;
    const uint64_t fl_base = whether_pq ? 0 : (uint64_t)n * d;
    const uint64_t fl_cb = (uint64_t)filter_nsq * 256 * lsq;
    const uint32_t pq_nsq = whether_pq ? nsq : 0;
    const uint64_t fl_pq = whether_pq ? (uint64_t)pq_nsq * 256 * (d / pq_nsq) + n : 0;
    const uint64_t floats = fl_coarse + fl_fine + fl_base + fl_cb + (uint64_t)n + fl_pq;
    const uint64_t bytes = floats * 4 + (uint64_t)n * 4 + (uint64_t)n * filter_nsq +
                           (uint64_t)n * pq_nsq + 64;
    try {
        storage.assign((size_t)bytes, 0);
    } catch (...) {
        *err = "host allocation failed";
        return PGPU_E_NOMEM;
    }
    float* coarse = reinterpret_cast<float*>(storage.data());
    float* fine = coarse + fl_coarse;
    float* basev = fine + fl_fine;
    float* cb = basev + fl_base;
    float* offsets = cb + fl_cb;
    float* pq_cb = offsets + n;                     // [pq_nsq][256][lsq_pq]
    float* pq_off = pq_cb + (whether_pq ? (uint64_t)pq_nsq * 256 * (d / pq_nsq) : 0);
    uint32_t* cell_assign = reinterpret_cast<uint32_t*>(pq_off + (whether_pq ? n : 0));
    uint8_t* codes = reinterpret_cast<uint8_t*>(cell_assign + n);
    uint8_t* pq_codes = codes + (uint64_t)n * filter_nsq;
    if (!read_fvecs(base + "/coarse.dat", d, C, coarse, err)) return PGPU_E_IO;
    if (!read_fvecs(base + "/fine.dat", d, F, fine, err)) return PGPU_E_IO;
    if (!read_fvecs(base + "/filter_codebook.dat", lsq, (uint64_t)filter_nsq * 256, cb, err))
        return PGPU_E_IO;
    if (!whether_pq && !read_fvecs(base + "/all_data.feat.bin", d, n, basev, err)) return PGPU_E_IO;
    if (whether_pq &&
        !read_fvecs(base + "/learn_codebooks.dat", d / pq_nsq, (uint64_t)pq_nsq * 256, pq_cb, err))
        return PGPU_E_IO;
    // cell_assign.dat: n uint32
    const std::string ca = base + "/cell_assign.dat";
    if (!file_size(ca, &sz) || sz != 4ull * n || !read_all(ca, (char*)cell_assign, sz)) {
        *err = "file length check failed: " + ca;
        return PGPU_E_IO;
    }
    // filter_data.dat: n records of [f32 offset][filter_nsq u8]
    const std::string fd = base + "/filter_data.dat";
    const uint64_t rb = 4ull + filter_nsq;
    if (!file_size(fd, &sz) || sz != rb * n) {
        *err = "file length check failed: " + fd;
        return PGPU_E_IO;
    }
    {
        std::vector<char> rec((size_t)std::min<uint64_t>(sz, 1ull << 26) + 1);
        FILE* f = std::fopen(fd.c_str(), "rb");
        if (!f) {
            *err = "cannot open " + fd;
            return PGPU_E_IO;
        }
        const uint64_t block = std::max<uint64_t>(1, (1ull << 26) / rb);
        for (uint64_t r0 = 0; r0 < n; r0 += block) {
            const uint64_t nr = std::min<uint64_t>(block, n - r0);
            if (std::fread(rec.data(), 1, (size_t)(nr * rb), f) != nr * rb) {
                std::fclose(f);
                *err = "short read: " + fd;
                return PGPU_E_IO;
            }
            for (uint64_t i = 0; i < nr; ++i) {
                std::memcpy(offsets + r0 + i, rec.data() + i * rb, 4);
                std::memcpy(codes + (r0 + i) * filter_nsq, rec.data() + i * rb + 4, filter_nsq);
            }
        }
        std::fclose(f);
    }
    if (whether_pq) {
        // pq_data.dat: n records of [f32 offset][pq_nsq u8]
        const std::string pd = base + "/pq_data.dat";
        const uint64_t prb = 4ull + pq_nsq;
        if (!file_size(pd, &sz) || sz != prb * n) {
            *err = "file length check failed: " + pd;
            return PGPU_E_IO;
        }
        std::vector<char> rec((size_t)std::min<uint64_t>(sz, 1ull << 26) + 1);
        FILE* f = std::fopen(pd.c_str(), "rb");
        if (!f) {
            *err = "cannot open " + pd;
            return PGPU_E_IO;
        }
        const uint64_t block = std::max<uint64_t>(1, (1ull << 26) / prb);
        for (uint64_t r0 = 0; r0 < n; r0 += block) {
            const uint64_t nr = std::min<uint64_t>(block, n - r0);
            if (std::fread(rec.data(), 1, (size_t)(nr * prb), f) != nr * prb) {
                std::fclose(f);
                *err = "short read: " + pd;
                return PGPU_E_IO;
            }
            for (uint64_t i = 0; i < nr; ++i) {
                std::memcpy(pq_off + r0 + i, rec.data() + i * prb, 4);
                std::memcpy(pq_codes + (r0 + i) * pq_nsq, rec.data() + i * prb + 4, pq_nsq);
            }
        }
        std::fclose(f);
    }
    a->whether_pq = whether_pq ? 1 : 0;
    a->pq_nsq = pq_nsq;
    a->pq_codebook = whether_pq ? pq_cb : nullptr;
    a->pq_offsets = whether_pq ? pq_off : nullptr;
    a->pq_codes = whether_pq ? pq_codes : nullptr;
    a->feature_dim = d;
    a->total_point_count = n;
    a->coarse_cluster_count = C;
    a->fine_cluster_count = F;
    a->filter_nsq = filter_nsq;
    a->whether_norm = whether_norm ? 1 : 0;
    a->ip2cos = (int32_t)ip2cos;
    a->coarse = coarse;
    a->fine = fine;
    a->base = whether_pq ? nullptr : basev;
    a->cell_assign = cell_assign;
    a->filter_codebook = cb;
    a->filter_offsets = offsets;
    a->filter_codes = codes;
    return PGPU_OK;
}

// Memory order: points sorted by (cell id, filter offset, input id) — the
// std::stable_sort of convert_local_to_memory_idx (puck_index.cpp:248-282).
// A counting scatter by cell keeps input order inside each cell; a stable sort
// by offset (operator<, so -0 == +0 keep input order) then gives the same order.
int build_host_index(const pgpu_index_arrays& a, HostIndex* h, std::string* err) {
    h->d = a.feature_dim;
    h->n = a.total_point_count;
    h->C = a.coarse_cluster_count;
    h->F = a.fine_cluster_count;
    h->nsq = a.filter_nsq;
    h->whether_norm = a.whether_norm;
    h->ip2cos = a.ip2cos;
    if (a.ip2cos < 0 || a.ip2cos > 1 || (a.ip2cos == 1 && h->d < 2)) {
        *err = "ip2cos must be 0 or 1 (1 needs feature_dim >= 2)";
        return PGPU_E_UNSUPPORTED;
    }
    if (h->d == 0 || h->nsq == 0 || h->d % h->nsq != 0 || h->C == 0 || h->F == 0) {
        *err = "inconsistent index shape (feature_dim must be a multiple of filter_nsq)";
        return PGPU_E_UNSUPPORTED;
    }
    if (h->d > kMaxDim || h->nsq > kMaxFilterNsq || h->C > kMaxClusters || h->F > kMaxClusters) {
        *err = "index shape beyond the search kernels' limits";
        return PGPU_E_LIMIT;
    }
    h->lsq = h->d / h->nsq;
    const uint64_t cells = (uint64_t)h->C * h->F;
    const uint32_t n = h->n;
    std::vector<uint32_t> count(cells + 1, 0);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t c = a.cell_assign[i];
        if (c >= cells) {
            *err = "cell_assign entry out of range";
            return PGPU_E_IO;
        }
        ++count[c];
    }
    h->cell_start.assign(cells + 1, 0);
    uint64_t acc = 0;
    for (uint64_t c = 0; c < cells; ++c) {
        h->cell_start[c] = (uint32_t)acc;
        acc += count[c];
    }
    h->cell_start[cells] = (uint32_t)acc;
    h->mem2local.assign(n, 0);
    {
        std::vector<uint32_t> pos(h->cell_start.begin(), h->cell_start.end() - 1);
        for (uint32_t i = 0; i < n; ++i) h->mem2local[pos[a.cell_assign[i]]++] = i;
    }
    const float* off = a.filter_offsets;
    uint32_t* m2l = h->mem2local.data();
    const uint32_t* cs = h->cell_start.data();
    parallel_for(cells, [&](uint64_t b, uint64_t e) {
        for (uint64_t c = b; c < e; ++c) {
            const uint32_t s = cs[c], t = cs[c + 1];
            if (t - s > 1)
                std::stable_sort(m2l + s, m2l + t,
                                 [off](uint32_t x, uint32_t y) { return off[x] < off[y]; });
        }
    });
    h->rec_fine.assign(n, 0);
    {
        uint16_t* rf = h->rec_fine.data();
        const uint32_t F = h->F;
        parallel_for(cells, [&](uint64_t b, uint64_t e) {
            for (uint64_t c = b; c < e; ++c)
                for (uint32_t i = cs[c]; i < cs[c + 1]; ++i) rf[i] = (uint16_t)(c % F);
        });
    }
    h->code_stride = (h->nsq + 3) / 4 * 4;
    h->offsets_mem.assign(n, 0.0f);
    h->codes_mem.assign((uint64_t)n * h->code_stride, 0);
    const uint32_t nsq = h->nsq, stride = h->code_stride;
    float* om = h->offsets_mem.data();
    uint8_t* cm = h->codes_mem.data();
    parallel_for(n, [&](uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; ++i) {
            const uint32_t l = m2l[i];
            om[i] = off[l];
            std::memcpy(cm + i * stride, a.filter_codes + (uint64_t)l * nsq, nsq);
        }
    });
    h->coarse.assign(a.coarse, a.coarse + (uint64_t)h->C * h->d);
    h->fine.assign(a.fine, a.fine + (uint64_t)h->F * h->d);
    h->codebook.assign(a.filter_codebook, a.filter_codebook + (uint64_t)nsq * 256 * h->lsq);
    if (a.whether_pq) {
        const uint32_t pn = a.pq_nsq;
        if (pn == 0 || pn > h->d || h->d % pn != 0 || pn > kMaxPqNsq || !a.pq_codebook ||
            !a.pq_offsets || !a.pq_codes) {
            *err = "inconsistent second-level PQ arrays";
            return PGPU_E_INVALID;
        }
        h->pq_nsq = pn;
        h->pq_lsq = h->d / pn;
        h->pq_code_stride = (pn + 3) / 4 * 4;
        h->pq_codebook.assign(a.pq_codebook, a.pq_codebook + (uint64_t)pn * 256 * h->pq_lsq);
        h->pq_offsets_mem.assign(n, 0.0f);
        h->pq_codes_mem.assign((uint64_t)n * h->pq_code_stride, 0);
        float* po = h->pq_offsets_mem.data();
        uint8_t* pc = h->pq_codes_mem.data();
        const uint32_t ps = h->pq_code_stride;
        parallel_for(n, [&](uint64_t b, uint64_t e) {
            for (uint64_t i = b; i < e; ++i) {
                const uint32_t l = m2l[i];
                po[i] = a.pq_offsets[l];
                std::memcpy(pc + i * ps, a.pq_codes + (uint64_t)l * pn, pn);
            }
        });
    } else if (a.base == nullptr) {
        *err = "base vectors are required without the second-level PQ";
        return PGPU_E_INVALID;
    }
    return PGPU_OK;
}

void free_device_index(DeviceIndex* ix) {
    void* ptrs[] = {ix->coarse, ix->fine, ix->coarse_norms, ix->coarse_abs, ix->coarse_bf16,
                    ix->fine_bf16, ix->feat_bf16,
                    ix->feat_abs, ix->stationary, ix->stat_sorted, ix->stat_fine, ix->rec_fine,
                    ix->cell_start,
                    ix->min_dist_offset, ix->mem2local, ix->offsets, ix->codes, ix->codes_il, ix->feat,
                    ix->codebook, ix->pq_codebook, ix->pq_offsets, ix->pq_codes,
                    ix->ins_head, ix->ins_next, ix->ins_cl_start, ix->ins_cl_ids};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    *ix = DeviceIndex();
}

}  // namespace pgpu
