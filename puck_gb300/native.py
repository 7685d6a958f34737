"""ctypes binding of libpuck_gb300.so (the C ABI in include/puck_gb300.h).

The library is built in-tree by ``puck_gb300.build.build()``. There is no CPU
fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

PGPU_OK = 0
PGPU_E_INVALID = -1
PGPU_E_ZERO_NORM = -2
PGPU_E_IO = -3
PGPU_E_UNSUPPORTED = -4
PGPU_E_CUDA = -5
PGPU_E_NOMEM = -6
PGPU_E_LIMIT = -7
PGPU_E_TIMEOUT = -8
PGPU_MODE_EXACT = 0
PGPU_MODE_SCAN = 1
PGPU_PRECISION_FP32 = 0
PGPU_PRECISION_BF16 = 1

HEAP_SENTINEL = np.uint32(0x7F7F7F7F).view(np.float32)
NO_LABEL = 0xFFFFFFFF

EXPORTED_SYMBOLS = (
    "pgpu_params_default", "pgpu_open", "pgpu_open_arrays", "pgpu_set_search_params",
    "pgpu_search_batch", "pgpu_search", "pgpu_search_batch_device", "pgpu_index_info_get",
    "pgpu_last_stats", "pgpu_close", "pgpu_nearest_center", "pgpu_last_error",
    "pgpu_set_profiling", "pgpu_stage_times", "pgpu_walk_counters",
    "pgpu_nearest_center_noalloc", "pgpu_nearest_cell_assign", "pgpu_server_params_default", "pgpu_server_create",
    "pgpu_server_submit", "pgpu_server_wait", "pgpu_server_stats_get", "pgpu_server_destroy",
    "pgpu_contract_bf16", "pgpu_contract_bf16_rows", "pgpu_filter_candidates", "pgpu_probe_create",
    "pgpu_probe_destroy",
    "pgpu_probe_info", "pgpu_probe_train_step", "pgpu_probe_gradients", "pgpu_probe_forward",
    "pgpu_probe_get_params", "pgpu_probe_set_params", "pgpu_set_probe", "pgpu_knn",
    "pgpu_puck_assign", "pgpu_realtime_open", "pgpu_insert",
)
NOALLOC_MAX_POINTS = 1 << 20
NOALLOC_MAX_CENTROIDS = 1 << 16
WALK_COUNTERS = ("records", "cells", "fd_order_chunks", "enumerations", "fd_order_clusters",
                 "heap_inserts", "cyc_replay", "cyc_total", "cyc_prologue", "cyc_candidates",
                 "cyc_adc", "coarse_window_fallbacks", "probe_fallbacks", "probe_clusters")
STAGES = ("prep", "coarse_scores", "coarse_select", "fine_scores", "fine_order", "walk_scan",
          "filter_select", "rerank")


class PuckGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"puck_gb300 error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("search_coarse_count", ctypes.c_uint32), ("topk", ctypes.c_uint32),
                ("filter_topk", ctypes.c_uint32), ("radius_rate", ctypes.c_double),
                ("device", ctypes.c_int32), ("max_batch", ctypes.c_uint32),
                ("mode", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("filter_margin", ctypes.c_uint32)]


class IndexInfo(ctypes.Structure):
    _fields_ = [("feature_dim", ctypes.c_uint32), ("total_point_count", ctypes.c_uint32),
                ("coarse_cluster_count", ctypes.c_uint32), ("fine_cluster_count", ctypes.c_uint32),
                ("filter_nsq", ctypes.c_uint32), ("lsq", ctypes.c_uint32),
                ("whether_norm", ctypes.c_int32), ("device_bytes", ctypes.c_uint64),
                ("query_dim", ctypes.c_uint32), ("ip2cos", ctypes.c_int32)]


class ServerParams(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_uint32), ("scratch_budget_bytes", ctypes.c_uint64),
                ("max_slots", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("requests_submitted", ctypes.c_uint64), ("requests_done", ctypes.c_uint64),
                ("queries_done", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("graph_launches", ctypes.c_uint64), ("graphs_captured", ctypes.c_uint64),
                ("padded_queries", ctypes.c_uint64), ("latency_us_sum", ctypes.c_double),
                ("slots", ctypes.c_uint32), ("slot_bytes", ctypes.c_uint64)]


class IndexArrays(ctypes.Structure):
    _fields_ = [("feature_dim", ctypes.c_uint32), ("total_point_count", ctypes.c_uint32),
                ("coarse_cluster_count", ctypes.c_uint32), ("fine_cluster_count", ctypes.c_uint32),
                ("filter_nsq", ctypes.c_uint32), ("whether_norm", ctypes.c_int32),
                ("coarse", ctypes.c_void_p), ("fine", ctypes.c_void_p), ("base", ctypes.c_void_p),
                ("cell_assign", ctypes.c_void_p), ("filter_codebook", ctypes.c_void_p),
                ("filter_offsets", ctypes.c_void_p), ("filter_codes", ctypes.c_void_p),
                ("whether_pq", ctypes.c_int32), ("pq_nsq", ctypes.c_uint32),
                ("pq_codebook", ctypes.c_void_p), ("pq_offsets", ctypes.c_void_p),
                ("pq_codes", ctypes.c_void_p), ("ip2cos", ctypes.c_int32)]


_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load the shared library (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(f"{path} is not built; run puck_gb300.build.build() "
                              "(there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
    lib.pgpu_params_default.argtypes = [ctypes.POINTER(Params)]
    lib.pgpu_params_default.restype = None
    lib.pgpu_open.argtypes = [ctypes.c_char_p, ctypes.POINTER(Params), ctypes.POINTER(vp)]
    lib.pgpu_open_arrays.argtypes = [ctypes.POINTER(IndexArrays), ctypes.POINTER(Params),
                                     ctypes.POINTER(vp)]
    lib.pgpu_set_search_params.argtypes = [vp, ctypes.POINTER(Params)]
    lib.pgpu_search_batch.argtypes = [vp, u32, vp, u32, vp, vp, vp]
    lib.pgpu_search.argtypes = [vp, vp, u32, vp, vp, ctypes.POINTER(u32)]
    lib.pgpu_search_batch_device.argtypes = [vp, u32, vp, u32, vp, vp, vp, vp]
    lib.pgpu_index_info_get.argtypes = [vp, ctypes.POINTER(IndexInfo)]
    lib.pgpu_last_stats.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                    ctypes.POINTER(u64)]
    lib.pgpu_close.argtypes = [vp]
    lib.pgpu_nearest_center.argtypes = [u32, vp, u64, vp, u64, vp, vp, vp]
    lib.pgpu_nearest_center_noalloc.argtypes = [u32, vp, u64, vp, u64, vp, vp, vp]
    lib.pgpu_nearest_cell_assign.argtypes = [u32, vp, u32, vp, u32, vp, u64, vp, vp, vp]
    lib.pgpu_realtime_open.argtypes = [vp, u32]
    lib.pgpu_insert.argtypes = [vp, u32, vp, vp]
    lib.pgpu_puck_assign.argtypes = [u32, u64, vp, vp, vp, u32, vp, u32, vp, u32, vp, u32, vp, vp,
                                     vp, vp, vp]
    lib.pgpu_set_profiling.argtypes = [vp, ctypes.c_int]
    lib.pgpu_stage_times.argtypes = [vp, ctypes.POINTER(ctypes.c_float), u32]
    lib.pgpu_walk_counters.argtypes = [vp, ctypes.POINTER(u64), u32]
    lib.pgpu_server_params_default.argtypes = [ctypes.POINTER(ServerParams)]
    lib.pgpu_server_params_default.restype = None
    lib.pgpu_server_create.argtypes = [vp, ctypes.POINTER(ServerParams), ctypes.POINTER(vp)]
    lib.pgpu_server_submit.argtypes = [vp, u32, vp, u32, vp, vp, vp, ctypes.POINTER(u64)]
    lib.pgpu_server_wait.argtypes = [vp, u64, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]
    lib.pgpu_server_stats_get.argtypes = [vp, ctypes.POINTER(ServerStats)]
    lib.pgpu_server_destroy.argtypes = [vp]
    f32 = ctypes.c_float
    lib.pgpu_filter_candidates.argtypes = [vp, u32, vp, vp, vp, vp]
    lib.pgpu_probe_create.argtypes = [u32, u32, u32, u64, ctypes.c_int32, ctypes.POINTER(vp)]
    lib.pgpu_probe_destroy.argtypes = [vp]
    lib.pgpu_probe_info.argtypes = [vp, ctypes.POINTER(u32), ctypes.POINTER(u32),
                                    ctypes.POINTER(u32), ctypes.POINTER(u64)]
    lib.pgpu_probe_train_step.argtypes = [vp, vp, vp, u32, u32, f32, ctypes.POINTER(f32)]
    lib.pgpu_probe_gradients.argtypes = [vp, vp, vp, u32, u32, ctypes.POINTER(f32), vp]
    lib.pgpu_probe_forward.argtypes = [vp, vp, u32, vp]
    lib.pgpu_probe_get_params.argtypes = [vp, vp, u64]
    lib.pgpu_probe_set_params.argtypes = [vp, vp, u64]
    lib.pgpu_set_probe.argtypes = [vp, vp, f32, u32]
    lib.pgpu_knn.argtypes = [vp, u64, u32, vp, u32, u32, vp, vp, vp]
    lib.pgpu_contract_bf16.argtypes = [ctypes.c_int32, u32, u32, u32, vp, u64, u64, vp, u64, u64,
                                       vp, vp, u64, vp, u64, vp, f32, f32, vp]
    lib.pgpu_contract_bf16_rows.argtypes = [ctypes.c_int32, u32, u32, u32, vp, u64, vp, u64, vp,
                                            vp, u64, vp, u64, vp, f32, f32, vp]
    lib.pgpu_last_error.restype = ctypes.c_char_p
    lib.pgpu_last_error.argtypes = []
    for name in EXPORTED_SYMBOLS:
        getattr(lib, name)
    _lib = lib
    return lib


def check(rc):
    if rc != PGPU_OK:
        raise PuckGpuError(rc, load().pgpu_last_error().decode(errors="replace"))
    return rc


def default_params(**overrides):
    p = Params()
    load().pgpu_params_default(ctypes.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def _ptr(x):
    """Data pointer of a numpy array, a torch tensor, or an int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"cannot take a data pointer of {type(x)}")


class GpuIndex:
    """A Puck-Flat index resident on one GPU."""

    def __init__(self, index_path=None, arrays=None, **params):
        lib = load()
        self._h = ctypes.c_void_p()
        p = default_params(**params)
        self._keep = None
        if index_path is not None:
            check(lib.pgpu_open(os.fsencode(index_path), ctypes.byref(p), ctypes.byref(self._h)))
        elif arrays is not None:
            a, keep = _arrays_struct(arrays)
            self._keep = keep
            check(lib.pgpu_open_arrays(ctypes.byref(a), ctypes.byref(p), ctypes.byref(self._h)))
            self._keep = None
        else:
            raise ValueError("index_path or arrays is required")
        self.params = p
        info = IndexInfo()
        check(lib.pgpu_index_info_get(self._h, ctypes.byref(info)))
        self.info = info
        self.d = info.query_dim  # floats per query (feature_dim - 1 on an ip2cos index)
        self.feature_dim = info.feature_dim

    def set_probe(self, probe, mass=0.9, max_probe=8):
        """Attach a learned Probe (None detaches); scan mode only."""
        check(load().pgpu_set_probe(self._h, probe._h if probe is not None else None, mass,
                                    max_probe))
        self._probe = probe

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().pgpu_close(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_search_params(self, **params):
        p = Params.from_buffer_copy(self.params)
        for k, v in params.items():
            setattr(p, k, v)
        check(load().pgpu_set_search_params(self._h, ctypes.byref(p)))
        self.params = p

    def search(self, queries, topk, return_status=False):
        """Host-buffer batch search (PySearcher::search semantics)."""
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.d)
        n = q.shape[0]
        dist = np.empty((n, topk), np.float32)
        ids = np.empty((n, topk), np.uint32)
        status = np.empty(n, np.int32)
        check(load().pgpu_search_batch(self._h, n, q.ctypes.data, topk, dist.ctypes.data,
                                       ids.ctypes.data, status.ctypes.data))
        return (dist, ids, status) if return_status else (dist, ids)

    def search_into(self, n, query_ptr, topk, dist_ptr, ids_ptr, status_ptr=None):
        return check(load().pgpu_search_batch(self._h, n, _ptr(query_ptr), topk, _ptr(dist_ptr),
                                              _ptr(ids_ptr), _ptr(status_ptr)))

    def search_device(self, n, query, topk, dist, ids, status=None, stream=None):
        """Device-buffer batch search; enqueued on `stream` (int handle or torch stream)."""
        s = stream
        if s is not None and not isinstance(s, int):
            s = s.cuda_stream
        return check(load().pgpu_search_batch_device(self._h, n, _ptr(query), topk, _ptr(dist),
                                                     _ptr(ids), _ptr(status), s))

    def search_one(self, feature, topk):
        """Index::search semantics: one query -> (distance, local_idx, result_num)."""
        q = np.ascontiguousarray(feature, np.float32)
        dist = np.empty(topk, np.float32)
        ids = np.empty(topk, np.uint32)
        rn = ctypes.c_uint32(0)
        check(load().pgpu_search(self._h, q.ctypes.data, topk, dist.ctypes.data, ids.ctypes.data,
                                 ctypes.byref(rn)))
        return dist, ids, rn.value

    def realtime_open(self, capacity):
        """Reserve room for `capacity` inserted points (RealtimeInsertPuckIndex::init)."""
        check(load().pgpu_realtime_open(self._h, capacity))

    def insert(self, features):
        """Insert host features [n, query_dim]; returns their local ids (int64, -1 where
        a feature was not inserted)."""
        x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, self.d)
        ids = np.empty(x.shape[0], np.int64)
        check(load().pgpu_insert(self._h, x.shape[0], x.ctypes.data, ids.ctypes.data))
        return ids

    def set_profiling(self, enable=True):
        check(load().pgpu_set_profiling(self._h, int(bool(enable))))

    def stage_times(self):
        """Milliseconds per stage of the last search call (profiling must be on)."""
        arr = (ctypes.c_float * len(STAGES))()
        check(load().pgpu_stage_times(self._h, arr, len(STAGES)))
        return dict(zip(STAGES, list(arr)))

    def walk_counters(self):
        arr = (ctypes.c_uint64 * len(WALK_COUNTERS))()
        check(load().pgpu_walk_counters(self._h, arr, len(WALK_COUNTERS)))
        return dict(zip(WALK_COUNTERS, list(arr)))

    def filter_candidates(self, queries):
        """Scan-mode filter candidates of one pass: (labels [n, keep], filter
        distances [n, keep], counts [n]), keep = filter_topk (+ filter_margin in BF16)."""
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, self.d)
        n = q.shape[0]
        p = self.params
        keep = p.filter_topk + (p.filter_margin if p.precision == PGPU_PRECISION_BF16 else 0)
        labels = np.empty((n, keep), np.uint32)
        dist = np.empty((n, keep), np.float32)
        cnt = np.empty(n, np.uint32)
        check(load().pgpu_filter_candidates(self._h, n, q.ctypes.data, labels.ctypes.data,
                                            dist.ctypes.data, cnt.ctypes.data))
        return labels, dist, cnt

    def last_stats(self):
        k, r, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(load().pgpu_last_stats(self._h, ctypes.byref(k), ctypes.byref(r), ctypes.byref(c)))
        return dict(kernels=k.value, records_scanned=r.value, cells_scanned=c.value)


def _arrays_struct(arr):
    keep = {}

    def c(name, dtype):
        a = np.ascontiguousarray(arr[name], dtype=dtype)
        keep[name] = a
        return a.ctypes.data

    coarse = np.asarray(arr["coarse"])
    codes = np.asarray(arr["filter_codes"])
    s = IndexArrays()
    s.feature_dim = coarse.shape[1]
    s.total_point_count = np.asarray(arr["cell_assign"]).shape[0]
    s.coarse_cluster_count = coarse.shape[0]
    s.fine_cluster_count = np.asarray(arr["fine"]).shape[0]
    s.filter_nsq = codes.shape[1]
    s.whether_norm = int(bool(arr.get("whether_norm", False)))
    s.ip2cos = int(arr.get("ip2cos", 0) or 0)
    s.coarse = c("coarse", np.float32)
    s.fine = c("fine", np.float32)
    pq = arr.get("pq_codes") is not None
    s.base = c("base", np.float32) if not pq else None
    s.cell_assign = c("cell_assign", np.uint32)
    s.filter_codebook = c("filter_codebook", np.float32)
    s.filter_offsets = c("filter_offsets", np.float32)
    s.filter_codes = c("filter_codes", np.uint8)
    if pq:
        s.whether_pq = 1
        s.pq_nsq = np.asarray(arr["pq_codes"]).shape[1]
        s.pq_codebook = c("pq_codebook", np.float32)
        s.pq_offsets = c("pq_offsets", np.float32)
        s.pq_codes = c("pq_codes", np.uint8)
    return s, keep


def nearest_center(centroids, points, assign, distance, stream=None):
    """k-means assignment on device tensors (torch CUDA tensors or raw pointers)."""
    k, dim = centroids.shape
    n = points.shape[0]
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    return check(load().pgpu_nearest_center(dim, _ptr(centroids), k, _ptr(points), n,
                                            _ptr(assign), _ptr(distance), s))


def nearest_cell_assign(coarse, fine, points, cell, distance, stream=None):
    """The build's exact cell assignment (pgpu_nearest_cell_assign) on CUDA tensors:
    coarse [C, d], fine [F, d] (index order), points [n, d] float32; cell [n]
    (int32 or uint32 bits) and distance [n] float32 outputs."""
    C, dim = coarse.shape
    F = fine.shape[0]
    n = points.shape[0]
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    return check(load().pgpu_nearest_cell_assign(dim, _ptr(coarse), C, _ptr(fine), F,
                                                 _ptr(points), n, _ptr(cell), _ptr(distance), s))


def puck_assign(base, cell_assign, coarse, fine, filter_codebook, pq_codebook=None, stream=None):
    """The build's encoder (pgpu_puck_assign) on CUDA tensors: base [n, d] float32,
    cell_assign [n] (int32 or uint32 bits), coarse [C, d], fine [F, d], filter_codebook
    [fnsq, 256, d/fnsq] and optionally pq_codebook [pnsq, 256, d/pnsq]. Returns
    (filter_offsets, filter_codes, pq_offsets, pq_codes) as CUDA tensors (the PQ pair
    None without a PQ codebook)."""
    import torch
    n, d = base.shape
    dev = base.device
    fnsq = filter_codebook.shape[0]
    pnsq = 0 if pq_codebook is None else pq_codebook.shape[0]
    f_off = torch.empty(n, dtype=torch.float32, device=dev)
    f_codes = torch.empty((n, fnsq), dtype=torch.uint8, device=dev)
    p_off = torch.empty(n, dtype=torch.float32, device=dev) if pnsq else None
    p_codes = torch.empty((n, pnsq), dtype=torch.uint8, device=dev) if pnsq else None
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    check(load().pgpu_puck_assign(d, n, _ptr(base.contiguous()), _ptr(cell_assign.contiguous()),
                                  _ptr(coarse.contiguous()), coarse.shape[0],
                                  _ptr(fine.contiguous()), fine.shape[0],
                                  _ptr(filter_codebook.contiguous()), fnsq,
                                  _ptr(pq_codebook.contiguous()) if pnsq else None, pnsq,
                                  _ptr(f_off), _ptr(f_codes), _ptr(p_off), _ptr(p_codes), s))
    return f_off, f_codes, p_off, p_codes


CONTRACT_MODES = {"score": 0, "neg": 1, "store": 2, "bias": 3, "bias_gelu": 4, "gelu_bwd": 5}


def contract_bf16(mode, a, b, out, bias=None, aux=None, out2=None, alpha=1.0, beta=0.0,
                  stream=None):
    """out = f(bf16(a) @ bf16(b).T) on the tensor cores (pgpu_contract_bf16).

    a [na, k] and b [nb, k] are 2-D float32 CUDA tensors in any strides (a
    transposed view is read in place); out is [na, >= nb] with unit column stride."""
    na, k = a.shape
    nb, kb = b.shape
    assert k == kb and out.stride(1) == 1
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    ld_aux = aux.stride(0) if aux is not None else 0
    return check(load().pgpu_contract_bf16(
        CONTRACT_MODES[mode], na, nb, k, _ptr(a), a.stride(0), a.stride(1), _ptr(b),
        b.stride(0), b.stride(1), _ptr(bias) if bias is not None else None,
        _ptr(aux) if aux is not None else None, ld_aux, _ptr(out), out.stride(0),
        _ptr(out2) if out2 is not None else None, alpha, beta, s))


def contract_bf16_rows(mode, a, b, out, bias=None, aux=None, out2=None, alpha=1.0, beta=0.0,
                       stream=None):
    """out = f(a @ b.T) on the tensor cores for BF16 operands already in memory
    (pgpu_contract_bf16_rows): a [na, k] and b [nb, k] are 2-D torch.bfloat16 CUDA
    tensors with unit column stride (rows may be padded); out is float32 [na, >= nb]."""
    import torch
    na, k = a.shape
    nb, kb = b.shape
    assert k == kb and a.dtype == torch.bfloat16 and b.dtype == torch.bfloat16
    assert a.stride(1) == 1 and b.stride(1) == 1 and out.stride(1) == 1
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    ld_aux = aux.stride(0) if aux is not None else 0
    return check(load().pgpu_contract_bf16_rows(
        CONTRACT_MODES[mode], na, nb, k, _ptr(a), a.stride(0), _ptr(b), b.stride(0),
        _ptr(bias) if bias is not None else None, _ptr(aux) if aux is not None else None,
        ld_aux, _ptr(out), out.stride(0), _ptr(out2) if out2 is not None else None, alpha, beta,
        s))


def nearest_center_noalloc(centroids, points, assign, distance, stream=None):
    """Same as nearest_center, without any device allocation inside the library
    (at most NOALLOC_MAX_POINTS points and NOALLOC_MAX_CENTROIDS centroids)."""
    k, dim = centroids.shape
    n = points.shape[0]
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    return check(load().pgpu_nearest_center_noalloc(dim, _ptr(centroids), k, _ptr(points), n,
                                                    _ptr(assign), _ptr(distance), s))


def knn(base, queries, k, labels, distance, stream=None):
    """Brute-force top-k (squared L2) on device tensors (pgpu_knn)."""
    n, d = base.shape
    nq = queries.shape[0]
    s = stream
    if s is not None and not isinstance(s, int):
        s = s.cuda_stream
    return check(load().pgpu_knn(_ptr(base), n, d, _ptr(queries), nq, k, _ptr(labels),
                                 _ptr(distance), s))


class Probe:
    """Learned probe network (pgpu_probe_*): queries -> coarse-cluster scores."""

    def __init__(self, dim, hidden, clusters, seed=0, device=0):
        lib = load()
        self._h = ctypes.c_void_p()
        check(lib.pgpu_probe_create(dim, hidden, clusters, seed, device, ctypes.byref(self._h)))
        self.dim, self.hidden, self.clusters = dim, hidden, clusters
        pc = ctypes.c_uint64()
        check(lib.pgpu_probe_info(self._h, None, None, None, ctypes.byref(pc)))
        self.param_count = pc.value

    def train_step(self, queries, labels, lr):
        """queries [n, dim] float32 and labels [n, L] int32/uint32 CUDA tensors."""
        loss = ctypes.c_float()
        n, L = labels.shape
        check(load().pgpu_probe_train_step(self._h, _ptr(queries), _ptr(labels), n, L, lr,
                                           ctypes.byref(loss)))
        return loss.value

    def gradients(self, queries, labels):
        n, L = labels.shape
        g = np.empty(self.param_count, np.float32)
        loss = ctypes.c_float()
        check(load().pgpu_probe_gradients(self._h, _ptr(queries), _ptr(labels), n, L,
                                          ctypes.byref(loss), g.ctypes.data))
        return loss.value, g

    def forward(self, queries, scores):
        check(load().pgpu_probe_forward(self._h, _ptr(queries), queries.shape[0], _ptr(scores)))

    def get_params(self):
        p = np.empty(self.param_count, np.float32)
        check(load().pgpu_probe_get_params(self._h, p.ctypes.data, self.param_count))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(load().pgpu_probe_set_params(self._h, p.ctypes.data, self.param_count))

    def split(self, flat):
        """Views W1, b1, W2, b2, W3, b3 of a flat parameter (or gradient) vector."""
        d, h, C = self.dim, self.hidden, self.clusters
        sizes = [(h, d), (h,), (h, h), (h,), (C, h), (C,)]
        out, o = [], 0
        for sh in sizes:
            m = int(np.prod(sh))
            out.append(flat[o:o + m].reshape(sh))
            o += m
        return out

    def close(self):
        if self._h:
            load().pgpu_probe_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server over a GpuIndex (pgpu_server_*).

    submit() takes host numpy arrays that must stay alive until wait() returns;
    the Server keeps references to them."""

    def __init__(self, index, max_batch=1024, scratch_budget_bytes=1 << 30, max_slots=4):
        lib = load()
        p = ServerParams()
        lib.pgpu_server_params_default(ctypes.byref(p))
        p.max_batch, p.scratch_budget_bytes, p.max_slots = max_batch, scratch_budget_bytes, max_slots
        self._h = ctypes.c_void_p()
        check(lib.pgpu_server_create(index._h, ctypes.byref(p), ctypes.byref(self._h)))
        self.index = index
        self._live = {}

    def submit(self, queries, topk):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, self.index.d)
        n = q.shape[0]
        dist = np.empty((n, topk), np.float32)
        ids = np.empty((n, topk), np.uint32)
        status = np.empty(n, np.int32)
        t = ctypes.c_uint64()
        check(load().pgpu_server_submit(self._h, n, q.ctypes.data, topk, dist.ctypes.data,
                                        ids.ctypes.data, status.ctypes.data, ctypes.byref(t)))
        self._live[t.value] = (q, dist, ids, status)
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        """Returns (dist, ids, status, latency_us)."""
        lat = ctypes.c_double()
        rc = load().pgpu_server_wait(self._h, ticket, timeout_ms, ctypes.byref(lat))
        q, dist, ids, status = self._live.pop(ticket) if rc == PGPU_OK else self._live[ticket]
        check(rc)
        return dist, ids, status, lat.value

    def stats(self):
        st = ServerStats()
        check(load().pgpu_server_stats_get(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().pgpu_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
