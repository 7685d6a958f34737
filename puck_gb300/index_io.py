"""Readers and writers for Puck's on-disk index files (Puck-Flat layout).

The GPU search path loads the reference's files unchanged. The formats:

* ``index.dat``: ``size_t`` length, then the packed structural config written by
  ``HierarchicalClusterIndex::save_model_config``
  (puck/hierarchical_cluster/hierarchical_cluster_index.cpp:522-543): IndexType
  (int32), feature_dim u32, whether_norm bool, total_point_count u32,
  whether_filter bool, filter_nsq u32, ks u32, whether_pq bool, nsq u32, ks u32,
  ip2cos u32, coarse_cluster_count u32, fine_cluster_count u32 (43 bytes).
* ``coarse.dat`` / ``fine.dat`` / ``all_data.feat.bin`` / ``filter_codebook.dat``:
  fvecs, i.e. per row an int32 dimension followed by that many float32
  (``write_fvec_format``, hierarchical_cluster_index.cpp:109-137).
* ``cell_assign.dat``: raw uint32 cell id per point, input order
  (hierarchical_cluster_index.cpp:1019-1039).
* ``filter_data.dat``: per point, input order, a record of a float32 offset then
  ``filter_nsq`` uint8 codes (puck/puck/quantization.cpp:42-60, 276-294).

File names are the reference's flag defaults (puck/gflags/puck_gflags.cpp:31-58).
"""
import os
import struct

import numpy as np

INDEX_FILE = "index.dat"
COARSE_FILE = "coarse.dat"
FINE_FILE = "fine.dat"
FEATURE_FILE = "all_data.feat.bin"
CELL_ASSIGN_FILE = "cell_assign.dat"
FILTER_CODEBOOK_FILE = "filter_codebook.dat"
FILTER_DATA_FILE = "filter_data.dat"
# second-level PQ (puck/gflags/puck_gflags.cpp defaults of pq_codebook_file_name, pq_data_file_name)
PQ_CODEBOOK_FILE = "learn_codebooks.dat"
PQ_DATA_FILE = "pq_data.dat"

_CONF_FMT = "<iI?I?II?IIIII"
_CONF_FIELDS = ("index_type", "feature_dim", "whether_norm", "total_point_count",
                "whether_filter", "filter_nsq", "ks", "whether_pq", "nsq", "ks2", "ip2cos",
                "coarse_cluster_count", "fine_cluster_count")
CONF_BYTES = struct.calcsize(_CONF_FMT)
assert CONF_BYTES == 43


def read_index_conf(path):
    with open(path, "rb") as f:
        raw = f.read()
    (size,) = struct.unpack_from("<Q", raw, 0)
    if size < CONF_BYTES or len(raw) < 8 + CONF_BYTES:
        raise ValueError(f"{path}: index config too short ({size} bytes)")
    vals = struct.unpack_from(_CONF_FMT, raw, 8)
    return dict(zip(_CONF_FIELDS, vals))


def write_index_conf(path, *, feature_dim, total_point_count, coarse_cluster_count,
                     fine_cluster_count, filter_nsq, whether_norm, index_type=1,
                     whether_filter=True, ks=256, whether_pq=False, nsq=None, ip2cos=0):
    nsq = feature_dim if nsq is None else nsq
    body = struct.pack(_CONF_FMT, index_type, feature_dim, bool(whether_norm), total_point_count,
                       bool(whether_filter), filter_nsq, ks, bool(whether_pq), nsq, ks, ip2cos,
                       coarse_cluster_count, fine_cluster_count)
    with open(path, "wb") as f:
        f.write(struct.pack("<Q", len(body)))
        f.write(body)


def write_fvecs(path, x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    rec = np.empty((n, d + 1), dtype=np.float32)
    rec.view(np.int32)[:, 0] = d
    rec[:, 1:] = x
    rec.tofile(path)


def read_fvecs(path, d=None):
    raw = np.fromfile(path, dtype=np.int32)
    if raw.size == 0:
        return np.zeros((0, d or 0), np.float32)
    dim = int(raw[0])
    if d is not None and dim != d:
        raise ValueError(f"{path}: dimension {dim} != expected {d}")
    if raw.size % (dim + 1):
        raise ValueError(f"{path}: length is not a multiple of the row size")
    rows = raw.reshape(-1, dim + 1)
    if not np.all(rows[:, 0] == dim):
        raise ValueError(f"{path}: inconsistent row dimensions")
    return rows[:, 1:].view(np.float32).copy()


def filter_record_bytes(filter_nsq):
    return 4 + filter_nsq


def write_filter_data(path, offsets, codes):
    n, nsq = codes.shape
    rec = np.empty((n, filter_record_bytes(nsq)), np.uint8)
    rec[:, :4] = np.ascontiguousarray(offsets, np.float32).view(np.uint8).reshape(n, 4)
    rec[:, 4:] = codes
    rec.tofile(path)


def read_filter_data(path, n, filter_nsq):
    raw = np.fromfile(path, dtype=np.uint8)
    rb = filter_record_bytes(filter_nsq)
    if raw.size != n * rb:
        raise ValueError(f"{path}: {raw.size} bytes, expected {n * rb}")
    rec = raw.reshape(n, rb)
    offsets = rec[:, :4].copy().view(np.float32).reshape(n)
    codes = rec[:, 4:].copy()
    return offsets, codes


def write_index(dirpath, *, base, coarse, fine, cell_assign, filter_codebook, filter_offsets,
                filter_codes, whether_norm, pq_codebook=None, pq_offsets=None, pq_codes=None,
                ip2cos=0):
    """Write a complete Puck index directory in the reference's formats: Puck-Flat,
    or with the second-level PQ when pq_codebook/pq_offsets/pq_codes are given
    (base, the build's input vectors, is then optional). ip2cos=1 marks vectors that
    carry one dimension more than the caller's queries."""
    os.makedirs(dirpath, exist_ok=True)
    d = np.asarray(coarse).shape[1]
    n = np.asarray(cell_assign).shape[0]
    nsq = filter_codes.shape[1]
    pq = pq_codes is not None
    write_index_conf(os.path.join(dirpath, INDEX_FILE), feature_dim=d, total_point_count=n,
                     coarse_cluster_count=coarse.shape[0], fine_cluster_count=fine.shape[0],
                     filter_nsq=nsq, whether_norm=whether_norm, whether_pq=pq,
                     nsq=pq_codes.shape[1] if pq else None, ip2cos=ip2cos)
    write_fvecs(os.path.join(dirpath, COARSE_FILE), coarse)
    write_fvecs(os.path.join(dirpath, FINE_FILE), fine)
    if base is not None:
        write_fvecs(os.path.join(dirpath, FEATURE_FILE), base)
    if pq:
        plsq = pq_codebook.shape[-1]
        write_fvecs(os.path.join(dirpath, PQ_CODEBOOK_FILE), pq_codebook.reshape(-1, plsq))
        write_filter_data(os.path.join(dirpath, PQ_DATA_FILE), pq_offsets, pq_codes)
    np.ascontiguousarray(cell_assign, np.uint32).tofile(os.path.join(dirpath, CELL_ASSIGN_FILE))
    lsq = filter_codebook.shape[-1]
    write_fvecs(os.path.join(dirpath, FILTER_CODEBOOK_FILE), filter_codebook.reshape(-1, lsq))
    write_filter_data(os.path.join(dirpath, FILTER_DATA_FILE), filter_offsets, filter_codes)


def read_index(dirpath):
    """Read every index file into numpy arrays (input/local order); with the
    second-level PQ also pq_codebook [pq_nsq, 256, lsq], pq_offsets, pq_codes."""
    conf = read_index_conf(os.path.join(dirpath, INDEX_FILE))
    d, n = conf["feature_dim"], conf["total_point_count"]
    nsq = conf["filter_nsq"]
    lsq = -(-d // nsq)
    out = dict(conf=conf, whether_norm=bool(conf["whether_norm"]), ip2cos=conf["ip2cos"])
    out["coarse"] = read_fvecs(os.path.join(dirpath, COARSE_FILE), d)
    out["fine"] = read_fvecs(os.path.join(dirpath, FINE_FILE), d)
    fp = os.path.join(dirpath, FEATURE_FILE)
    out["base"] = read_fvecs(fp, d) if os.path.exists(fp) or not conf["whether_pq"] else None
    out["cell_assign"] = np.fromfile(os.path.join(dirpath, CELL_ASSIGN_FILE), np.uint32)
    out["filter_codebook"] = read_fvecs(os.path.join(dirpath, FILTER_CODEBOOK_FILE),
                                        lsq).reshape(nsq, 256, lsq)
    out["filter_offsets"], out["filter_codes"] = read_filter_data(
        os.path.join(dirpath, FILTER_DATA_FILE), n, nsq)
    if conf["whether_pq"]:
        pn = conf["nsq"]
        plsq = d // pn
        out["pq_codebook"] = read_fvecs(os.path.join(dirpath, PQ_CODEBOOK_FILE),
                                        plsq).reshape(pn, 256, plsq)
        out["pq_offsets"], out["pq_codes"] = read_filter_data(
            os.path.join(dirpath, PQ_DATA_FILE), n, pn)
    return out


def materialize_npz_index(npz, dirpath):
    """Write the ``file:<name>`` members of a golden fixture back to a directory."""
    os.makedirs(dirpath, exist_ok=True)
    for key in npz.files:
        if key.startswith("file:"):
            with open(os.path.join(dirpath, key[5:]), "wb") as f:
                f.write(npz[key].tobytes())
    return dirpath
