"""Drop-in mirror of the reference's Python module ``py_puck_api``.

The reference exposes (pyapi_wrapper/py_api_wrapper.h:30-42, SWIG
pyapi_wrapper/py_puck_api.i:126-137):

    update_gflag(key, value)
    PySearcher().init()
    PySearcher().search(n, query, topk, distance, labels)

with search parameters read from gflags (puck/gflags/puck_gflags.cpp:26-81) and
the index read from ``FLAGS_index_path``. This module keeps the same names,
argument meanings and flag names; ``search`` runs on the GPU through the C ABI
(pgpu_search_batch). ``query``, ``distance`` and ``labels`` may be numpy arrays
or raw host addresses (the reference's callers pass ``swig_ptr`` addresses).
"""
import numpy as np

from . import native

_FLAG_DEFAULTS = {
    "index_path": "puck_index",
    "search_coarse_count": 200,
    "topk": 100,
    "filter_topk": None,           # default topk * 11 (puck/index_conf.cpp:178-180)
    "radius_rate": 1.0,
    "context_initial_pool_size": 0,  # thread pool of the CPU reference; unused on the GPU
    "gpu_device": 0,
    "gpu_max_batch": 8192,
}
_flags = dict(_FLAG_DEFAULTS)
_set = set()


def update_gflag(gflag_key, gflag_val):
    """google::SetCommandLineOption (pyapi_wrapper/py_api_wrapper.cpp:33-35).

    Like gflags, unknown keys are ignored (the reference returns the empty
    string for them)."""
    key = gflag_key.decode() if isinstance(gflag_key, bytes) else str(gflag_key)
    val = gflag_val.decode() if isinstance(gflag_val, bytes) else str(gflag_val)
    if key not in _flags:
        return ""
    default = _FLAG_DEFAULTS[key]
    if key == "index_path":
        _flags[key] = val
    elif key == "radius_rate":
        _flags[key] = float(val)
    elif isinstance(default, int) or default is None:
        _flags[key] = int(val)
    else:
        _flags[key] = val
    _set.add(key)
    return f"{key} set to {val}\n"


def reset_gflags():
    _flags.clear()
    _flags.update(_FLAG_DEFAULTS)
    _set.clear()


def current_params():
    topk = int(_flags["topk"])
    ft = _flags["filter_topk"]
    filter_topk = topk * 11 if ft is None else int(ft)
    return dict(search_coarse_count=int(_flags["search_coarse_count"]), topk=topk,
                filter_topk=filter_topk, radius_rate=float(_flags["radius_rate"]),
                device=int(_flags["gpu_device"]), max_batch=int(_flags["gpu_max_batch"]))


class PySearcher:
    """PySearcher over a GPU-resident Puck-Flat index."""

    def __init__(self):
        self._index = None
        self._dim = 0

    def show(self):
        print("1")

    def init(self):
        """Loads FLAGS_index_path (PySearcher::init, py_api_wrapper.cpp:78-108).
        Returns 0, or -1 when the index cannot be loaded."""
        if self._index is not None:
            self._index.close()
            self._index = None
        try:
            self._index = native.GpuIndex(_flags["index_path"], **current_params())
        except native.PuckGpuError:
            return -1
        self._dim = self._index.d
        return 0

    def build(self, n):
        raise NotImplementedError("index training/building is outside the GPU search path")

    def search(self, n, query_fea, topk, distance, labels):
        """PySearcher::search (py_api_wrapper.cpp:154-170): n queries, results
        written into distance[n*topk] and labels[n*topk]. Returns 0."""
        if self._index is None:
            raise RuntimeError("PySearcher.init() has not succeeded")
        if isinstance(query_fea, np.ndarray):
            query_fea = np.ascontiguousarray(query_fea, dtype=np.float32)
        try:
            self._index.search_into(int(n), query_fea, int(topk), distance, labels)
        except native.PuckGpuError as e:
            # The reference ignores per-query failures here (py_api_wrapper.cpp:166):
            # a rejected request leaves distance/labels untouched and returns 0.
            if e.code != native.PGPU_E_INVALID:
                raise
        return 0

    @property
    def index(self):
        return self._index
