"""Host-side checks of the C ABI library (no GPU compute).

The shared library must build for sm_103a, load, and export every entry point
include/puck_gb300.h declares. Calls that fail before touching a GPU (null
arguments, bad parameters, no device) must return their documented codes.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from puck_gb300 import build, index_io, native, py_puck_api

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    src = open(os.path.join(REPO, "include", "puck_gb300.h")).read()
    return sorted(set(re.findall(r"\b(pgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return native.load()


def test_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(native.EXPORTED_SYMBOLS)


def test_params_default_matches_reference_flags(lib):
    p = native.default_params()
    # puck/gflags/puck_gflags.cpp:70-78 and index_conf.cpp:178-180
    assert p.search_coarse_count == 200
    assert p.topk == 100
    assert p.filter_topk == 1100
    assert p.radius_rate == 1.0
    assert p.mode == native.PGPU_MODE_EXACT
    assert p.precision == native.PGPU_PRECISION_FP32 and p.filter_margin == 0


def test_null_arguments_rejected(lib):
    h = ctypes.c_void_p()
    assert lib.pgpu_open(None, None, ctypes.byref(h)) == native.PGPU_E_INVALID
    assert lib.pgpu_search_batch(None, 1, None, 10, None, None, None) == native.PGPU_E_INVALID
    assert lib.pgpu_close(None) == 0
    assert b"null" in lib.pgpu_last_error()


def test_bad_search_params_rejected_before_device(lib, tmp_path):
    h = ctypes.c_void_p()
    p = native.default_params(radius_rate=0.5)
    assert lib.pgpu_open(str(tmp_path).encode(), ctypes.byref(p), ctypes.byref(h)) in (
        native.PGPU_E_IO, native.PGPU_E_INVALID)
    p = native.default_params(filter_topk=50, topk=100)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_INVALID
    p = native.default_params(filter_topk=100000)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_LIMIT
    # the precision form runs in scan mode only, within the scan's candidate buffer
    p = native.default_params(precision=native.PGPU_PRECISION_BF16)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_INVALID
    p = native.default_params(precision=7, mode=native.PGPU_MODE_SCAN, filter_topk=500)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_INVALID
    p = native.default_params(precision=native.PGPU_PRECISION_BF16, mode=native.PGPU_MODE_SCAN,
                              filter_topk=1900, filter_margin=200)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_LIMIT
    p = native.default_params(mode=native.PGPU_MODE_SCAN, filter_topk=2049)
    assert lib.pgpu_open(b"/nonexistent", ctypes.byref(p), ctypes.byref(h)) == native.PGPU_E_LIMIT


def test_missing_index_files(lib, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("covered on the GPU")
    h = ctypes.c_void_p()
    rc = lib.pgpu_open(str(tmp_path).encode(), None, ctypes.byref(h))
    assert rc == native.PGPU_E_IO


def test_index_io_roundtrip(tmp_path, golden):
    name, z, index_dir = golden
    ix = index_io.read_index(index_dir)
    out = str(tmp_path / "copy")
    index_io.write_index(out, base=ix["base"], coarse=ix["coarse"], fine=ix["fine"],
                         cell_assign=ix["cell_assign"], filter_codebook=ix["filter_codebook"],
                         filter_offsets=ix["filter_offsets"], filter_codes=ix["filter_codes"],
                         whether_norm=ix["conf"]["whether_norm"],
                         pq_codebook=ix.get("pq_codebook"), pq_offsets=ix.get("pq_offsets"),
                         pq_codes=ix.get("pq_codes"), ip2cos=ix["ip2cos"])
    for fn in os.listdir(index_dir):
        assert open(os.path.join(index_dir, fn), "rb").read() == \
            open(os.path.join(out, fn), "rb").read(), fn


def test_gflag_mirror_defaults():
    py_puck_api.reset_gflags()
    p = py_puck_api.current_params()
    assert p["filter_topk"] == 1100 and p["search_coarse_count"] == 200
    py_puck_api.update_gflag("topk", "10")
    assert py_puck_api.current_params()["filter_topk"] == 110
    py_puck_api.update_gflag("filter_topk", "500")
    assert py_puck_api.current_params()["filter_topk"] == 500
    assert py_puck_api.update_gflag("no_such_flag", "1") == ""
    py_puck_api.reset_gflags()


def test_ip2cos_conf_checked_before_device(lib, tmp_path):
    """ip2cos = 2 is refused from index.dat alone (the reference's search reads past a
    feature_dim - 1 query there); ip2cos = 1 passes the config check and fails only on
    the missing vector files."""
    for ip2cos, want in ((2, native.PGPU_E_UNSUPPORTED), (1, native.PGPU_E_IO)):
        d = tmp_path / f"ip{ip2cos}"
        d.mkdir()
        index_io.write_index_conf(str(d / "index.dat"), feature_dim=8, total_point_count=4,
                                  coarse_cluster_count=2, fine_cluster_count=2, filter_nsq=2,
                                  whether_norm=False, ip2cos=ip2cos)
        h = ctypes.c_void_p()
        p = native.default_params()
        assert lib.pgpu_open(str(d).encode(), ctypes.byref(p), ctypes.byref(h)) == want
