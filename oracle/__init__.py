"""ORACLE — test infrastructure, not the product.

ctypes bindings for the plain-C restatement of Puck's Puck-Flat search path
(oracle/puck_oracle.c) and, where it has been built, for the reference's own
code compiled from its sources (oracle/_ref/, see oracle/ref/Makefile).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, and only as the checker or the timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpuck_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libpuckref.so")
REF_NATIVE_LIB_PATH = os.path.join(HERE, "_ref", "libpuckref_native.so")


def build_oracle(force=False):
    """Compile the C restatement (seconds). No FMA contraction, no fast-math."""
    src = os.path.join(HERE, "puck_oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                           "-fno-fast-math", "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_dir():
    """Where the reference's sources are: the PUCK_REFERENCE_DIR environment
    variable (None when it is unset or not a directory)."""
    ref = os.environ.get("PUCK_REFERENCE_DIR", "")
    return ref if ref and os.path.isdir(ref) else None


def build_reference(native=False, ref=None):
    """Compile the reference's own sources (x86 only) from `ref`, by default the
    PUCK_REFERENCE_DIR environment variable; returns None when neither names a
    directory."""
    ref = ref or reference_dir()
    if ref is None or not os.path.isdir(ref):
        return None
    target = "native" if native else "all"
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref}", "-j8",
                           target])
    return REF_NATIVE_LIB_PATH if native else REF_LIB_PATH


class _Params(ctypes.Structure):
    _fields_ = [("search_coarse_count", ctypes.c_uint32), ("filter_topk", ctypes.c_uint32),
                ("topk", ctypes.c_uint32), ("radius_rate", ctypes.c_double)]


class _Trace(ctypes.Structure):
    _fields_ = [("coarse_tag", ctypes.c_void_p), ("coarse_dist", ctypes.c_void_p),
                ("filter_tag", ctypes.c_void_p), ("filter_dist", ctypes.c_void_p),
                ("filter_cnt", ctypes.c_uint32), ("lut", ctypes.c_void_p),
                ("scanned_points", ctypes.c_uint64), ("scanned_cells", ctypes.c_uint64),
                ("visited_cells", ctypes.c_uint64), ("low_stat_cells", ctypes.c_uint64)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build_oracle())
        lib.po_load.restype = ctypes.c_void_p
        lib.po_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        lib.po_free.argtypes = [ctypes.c_void_p]
        lib.po_set_ip2cos.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.po_realtime_open.argtypes = [ctypes.c_void_p]
        lib.po_insert.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.po_insert.restype = ctypes.c_int64
        lib.po_inserted_records.argtypes = [ctypes.c_void_p] * 6
        lib.po_inserted_records.restype = ctypes.c_uint32
        lib.po_load_arrays_pq.restype = ctypes.c_void_p
        lib.po_load_arrays_pq.argtypes = [ctypes.c_uint32] * 5 + [ctypes.c_int] + [ctypes.c_void_p] * 7 + [
            ctypes.c_uint32] + [ctypes.c_void_p] * 3 + [ctypes.POINTER(ctypes.c_int)]
        lib.po_load_arrays.restype = ctypes.c_void_p
        lib.po_load_arrays.argtypes = [ctypes.c_uint32] * 5 + [ctypes.c_int] + [ctypes.c_void_p] * 7 + [
            ctypes.POINTER(ctypes.c_int)]
        lib.po_info.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_uint32)] * 6 + [
            ctypes.POINTER(ctypes.c_int)]
        lib.po_memory_to_local.restype = ctypes.c_void_p
        lib.po_memory_to_local.argtypes = [ctypes.c_void_p]
        lib.po_stationary.restype = ctypes.c_void_p
        lib.po_stationary.argtypes = [ctypes.c_void_p]
        lib.po_cell_start.restype = ctypes.c_void_p
        lib.po_cell_start.argtypes = [ctypes.c_void_p]
        lib.po_search.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Params), ctypes.c_void_p,
                                  ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(_Trace)]
        lib.po_search_batch.argtypes = [ctypes.c_void_p, ctypes.POINTER(_Params), ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.po_search_scan.argtypes = lib.po_search.argtypes
        lib.po_search_scan_batch.argtypes = lib.po_search_batch.argtypes
        lib.po_puck_assign.argtypes = [ctypes.c_uint32, ctypes.c_uint64] + [ctypes.c_void_p] * 4 + [
            ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32] + [
            ctypes.c_void_p] * 4
        lib.po_nearest_center.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                                          ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                          ctypes.c_void_p]
        lib.po_nearest_cell_assign.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                               ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                               ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None else None


class OracleIndex:
    """The C restatement loaded on one Puck index directory (Puck-Flat, or with the
    second-level PQ)."""

    def __init__(self, index_dir=None, arrays=None):
        lib = _load()
        err = ctypes.c_int(0)
        if index_dir is not None:
            self._h = lib.po_load(index_dir.encode(), ctypes.byref(err))
        else:
            keys = [("coarse", np.float32), ("fine", np.float32), ("cell_assign", np.uint32),
                    ("filter_codebook", np.float32), ("filter_offsets", np.float32),
                    ("filter_codes", np.uint8)]
            pq = arrays.get("pq_codes") is not None
            keys += [("pq_codebook", np.float32), ("pq_offsets", np.float32),
                     ("pq_codes", np.uint8)] if pq else [("base", np.float32)]
            a = {k: np.ascontiguousarray(arrays[k], t) for k, t in keys}
            n = a["cell_assign"].shape[0]
            d = a["coarse"].shape[1]
            self._h = lib.po_load_arrays_pq(
                d, n, a["coarse"].shape[0], a["fine"].shape[0], a["filter_codes"].shape[1],
                int(bool(arrays.get("whether_norm", False))), a["coarse"].ctypes.data,
                a["fine"].ctypes.data, a["base"].ctypes.data if not pq else None,
                a["cell_assign"].ctypes.data, a["filter_codebook"].ctypes.data,
                a["filter_offsets"].ctypes.data, a["filter_codes"].ctypes.data,
                a["pq_codes"].shape[1] if pq else 0,
                a["pq_codebook"].ctypes.data if pq else None,
                a["pq_offsets"].ctypes.data if pq else None,
                a["pq_codes"].ctypes.data if pq else None, ctypes.byref(err))
        if not self._h:
            raise RuntimeError(f"oracle could not load the index (error {err.value})")
        if index_dir is None and int(arrays.get("ip2cos", 0) or 0):
            if lib.po_set_ip2cos(self._h, int(arrays["ip2cos"])) != 0:
                raise RuntimeError("oracle: ip2cos must be 0 or 1")
        vals = [ctypes.c_uint32() for _ in range(6)]
        wn = ctypes.c_int()
        lib.po_info(self._h, *[ctypes.byref(v) for v in vals], ctypes.byref(wn))
        self.d, self.n, self.C, self.F, self.nsq, self.lsq = [v.value for v in vals]
        self.whether_norm = bool(wn.value)
        self.ip2cos = bool(int(arrays.get("ip2cos", 0) or 0)) if index_dir is None else None

    def close(self):
        if self._h:
            _load().po_free(self._h)
            self._h = None

    __del__ = close

    def realtime_open(self):
        """Switch to RealtimeInsertPuckIndex semantics (realtime_insert_puck_index.cpp)."""
        if _load().po_realtime_open(self._h) != 0:
            raise RuntimeError("oracle: realtime open failed")
        self._inserted = 0

    def insert(self, feature):
        """Insert one point (d floats); returns its local id (n + insert id)."""
        x = np.ascontiguousarray(feature, np.float32)
        lid = _load().po_insert(self._h, x.ctypes.data)
        if lid < 0:
            raise RuntimeError("oracle: insert failed")
        self._inserted += 1
        return lid

    def inserted_records(self, pq_nsq=0):
        """(cells, filter offsets, filter codes, pq offsets, pq codes) of the inserts."""
        m = self._inserted
        cell = np.zeros(m, np.uint32)
        off = np.zeros(m, np.float32)
        codes = np.zeros((m, self.nsq), np.uint8)
        poff = np.zeros(m, np.float32) if pq_nsq else None
        pcodes = np.zeros((m, pq_nsq), np.uint8) if pq_nsq else None
        _load().po_inserted_records(self._h, cell.ctypes.data, off.ctypes.data, codes.ctypes.data,
                                    _ptr(poff), _ptr(pcodes))
        return cell, off, codes, poff, pcodes

    def memory_to_local(self):
        p = _load().po_memory_to_local(self._h)
        return np.ctypeslib.as_array((ctypes.c_uint32 * self.n).from_address(p)).copy()

    def stationary(self):
        p = _load().po_stationary(self._h)
        return np.ctypeslib.as_array((ctypes.c_float * (self.C * self.F)).from_address(p)).copy()

    def cell_start(self):
        p = _load().po_cell_start(self._h)
        return np.ctypeslib.as_array(
            (ctypes.c_uint32 * (self.C * self.F + 1)).from_address(p)).copy()

    def params(self, search_coarse_count, filter_topk, topk_max=100, radius_rate=1.0):
        return _Params(search_coarse_count, filter_topk, topk_max, radius_rate)

    def search_one(self, q, topk, search_coarse_count, filter_topk, topk_max=None,
                   radius_rate=1.0, trace=False, scan=False):
        """Returns (rc, dist[topk], ids[topk], result_num, trace dict or None)."""
        lib = _load()
        P = min(search_coarse_count, self.C)
        p = _Params(search_coarse_count, filter_topk, topk_max or max(topk, 100), radius_rate)
        q = np.ascontiguousarray(q, np.float32)
        dist = np.zeros(topk, np.float32)
        ids = np.full(topk, 0xFFFFFFFF, np.uint32)
        rn = ctypes.c_uint32(0)
        tr = None
        arrs = None
        if trace:
            arrs = dict(coarse_tag=np.zeros(P, np.uint32), coarse_dist=np.zeros(P, np.float32),
                        filter_tag=np.zeros(filter_topk, np.uint32),
                        filter_dist=np.zeros(filter_topk, np.float32),
                        lut=np.zeros(self.nsq * 256, np.float32))
            tr = _Trace(_ptr(arrs["coarse_tag"]), _ptr(arrs["coarse_dist"]),
                        _ptr(arrs["filter_tag"]), _ptr(arrs["filter_dist"]), 0, _ptr(arrs["lut"]),
                        0, 0, 0, 0)
        fn = lib.po_search_scan if scan else lib.po_search
        rc = fn(self._h, ctypes.byref(p), q.ctypes.data, topk, dist.ctypes.data,
                           ids.ctypes.data, ctypes.byref(rn),
                           ctypes.byref(tr) if tr is not None else None)
        if trace:
            arrs["filter_cnt"] = tr.filter_cnt
            arrs["scanned_points"] = tr.scanned_points
            arrs["scanned_cells"] = tr.scanned_cells
            arrs["visited_cells"] = tr.visited_cells
            arrs["low_stat_cells"] = tr.low_stat_cells
        return rc, dist, ids, rn.value, arrs

    def search_batch(self, q, topk, search_coarse_count, filter_topk, topk_max=None,
                     radius_rate=1.0, nthreads=None, scan=False):
        lib = _load()
        q = np.ascontiguousarray(q, np.float32)
        n = q.shape[0]
        p = _Params(search_coarse_count, filter_topk, topk_max or max(topk, 100), radius_rate)
        dist = np.zeros((n, topk), np.float32)
        ids = np.full((n, topk), 0xFFFFFFFF, np.uint32)
        status = np.zeros(n, np.int32)
        fn = lib.po_search_scan_batch if scan else lib.po_search_batch
        fn(self._h, ctypes.byref(p), n, q.ctypes.data, topk, dist.ctypes.data,
                            ids.ctypes.data, status.ctypes.data, nthreads or os.cpu_count())
        return dist, ids, status


def nearest_center(centroids, x):
    lib = _load()
    centroids = np.ascontiguousarray(centroids, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    n = x.shape[0]
    assign = np.zeros(n, np.int32)
    dis = np.zeros(n, np.float32)
    lib.po_nearest_center(x.shape[1], centroids.ctypes.data, centroids.shape[0], x.ctypes.data, n,
                          assign.ctypes.data, dis.ctypes.data)
    return assign, dis


def nearest_cell_assign(coarse, fine, x):
    lib = _load()
    coarse = np.ascontiguousarray(coarse, np.float32)
    fine = np.ascontiguousarray(fine, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    n = x.shape[0]
    cell = np.zeros(n, np.uint32)
    dist = np.zeros(n, np.float32)
    lib.po_nearest_cell_assign(x.shape[1], coarse.ctypes.data, coarse.shape[0], fine.ctypes.data,
                               fine.shape[0], x.ctypes.data, n, cell.ctypes.data,
                               dist.ctypes.data)
    return cell, dist


def puck_assign(base, cell_assign, coarse, fine, filter_codebook, pq_codebook=None):
    """puck_assign (puck/puck/puck_index.cpp:602-709) for points whose cells are known:
    (filter_offsets [n], filter_codes [n, fnsq]) and, with a second-level PQ codebook,
    (pq_offsets, pq_codes) as well (else None, None)."""
    lib = _load()
    base = np.ascontiguousarray(base, np.float32)
    n, d = base.shape
    ca = np.ascontiguousarray(cell_assign, np.uint32)
    coarse = np.ascontiguousarray(coarse, np.float32)
    fine = np.ascontiguousarray(fine, np.float32)
    fcb = np.ascontiguousarray(filter_codebook, np.float32)
    fnsq = fcb.shape[0]
    pcb = None if pq_codebook is None else np.ascontiguousarray(pq_codebook, np.float32)
    pnsq = 0 if pcb is None else pcb.shape[0]
    f_off = np.zeros(n, np.float32)
    f_codes = np.zeros((n, fnsq), np.uint8)
    p_off = np.zeros(n, np.float32) if pnsq else None
    p_codes = np.zeros((n, pnsq), np.uint8) if pnsq else None
    lib.po_puck_assign(d, n, base.ctypes.data, ca.ctypes.data, coarse.ctypes.data,
                       fine.ctypes.data, fine.shape[0], fcb.ctypes.data, fnsq, _ptr(pcb), pnsq,
                       f_off.ctypes.data, f_codes.ctypes.data, _ptr(p_off), _ptr(p_codes))
    return f_off, f_codes, p_off, p_codes

