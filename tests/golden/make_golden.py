"""Generate the golden fixtures under tests/golden/ from the reference itself.

For each small case below this script
  1. writes a seeded synthetic base set and query set (same mixture families as
     the benchmark workloads, at test sizes),
  2. runs the reference's own ``PuckIndex::train()`` and ``build()``
     (puck/puck/puck_index.cpp:764-874, hierarchical_cluster_index.cpp:987-1017)
     to produce a Puck index in the reference's file formats: Puck-Flat
     (whether_pq=false) or, for the pq_* cases, with the second-level PQ,
  3. runs the reference's batch entry point ``PySearcher::search``
     (pyapi_wrapper/py_api_wrapper.cpp:154-170) over the queries, and probes
     the per-query intermediates with the reference's own stage functions
     (coarse list, filter heap, LUT); for ip2cos cases the final results come
     from the reference's ``Index::search`` (puck_index.cpp:559-600) on the
     probe's contexts (see run_case),
  4. stores index files + queries + outputs in ``<case>.npz``.

The reference is the copy compiled from its sources by oracle/ref/Makefile
(parity build: -O2, AVX2 without FMA, no FP contraction, deterministic BLAS).
Its training is seeded from time(0) (puck/hierarchical_cluster/kmeans.h:47-48),
so the index files themselves are committed rather than regenerated.

Usage: python tests/golden/make_golden.py [case ...]
"""
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from puck_gb300 import index_io  # noqa: E402

REF_LIB = os.path.join(REPO, "oracle", "_ref", "libpuckref.so")

# name: (n, d, C, F, whether_norm, mixture, P, T, topk, nq, extra flags)
CASES = {
    # L2 on integer-valued data (ties in exact distances are common), d=32,
    # filter_nsq = 8 (lsq = 4). Includes exact duplicate base rows.
    "l2_int_d32": dict(n=6000, d=32, C=16, F=16, norm=False, mix="int", P=8, T=64, topk=10,
                       nq=64, dup=200),
    # Cosine on L2-normalised data, d=24, filter_nsq = 6; P = C probes all.
    "cos_d24": dict(n=8000, d=24, C=24, F=24, norm=True, mix="gauss", P=12, T=100, topk=20,
                    nq=64, dup=0),
    # d=30 -> the reference picks lsq=5, filter_nsq=6 (index_conf.cpp:123-131):
    # exercises the generic LUT path and the scalar tail of the rerank.
    "l2_d30_lsq5": dict(n=4000, d=30, C=12, F=12, norm=False, mix="gauss", P=5, T=48, topk=10,
                        nq=48, dup=0),
    # Filter heap larger than the scanned set -> the not-full reorder path,
    # and topk > candidates for some queries.
    "l2_small_heap": dict(n=1500, d=16, C=8, F=8, norm=False, mix="int", P=2, T=400, topk=100,
                          nq=32, dup=50),
    # whether_pq=true (the reference's default): the rerank ranks the filter survivors
    # by the second-level PQ (nsq = feature_dim, lsq = 1) instead of the original
    # vectors (puck_index.cpp:402-427).
    "pq_l2_int_d32": dict(n=6000, d=32, C=16, F=16, norm=False, mix="int", P=8, T=64, topk=10,
                          nq=64, dup=200, pq=True),
    "pq_cos_d24": dict(n=8000, d=24, C=24, F=24, norm=True, mix="gauss", P=12, T=100, topk=20,
                       nq=64, dup=0, pq=True),
    # ip2cos=1: inner-product data recast as L2. The base file holds d+1 dims,
    # [x, sqrt(M^2 - |x|^2)] with M the largest |x|; the reference raises feature_dim to
    # d+1 (index_conf.cpp:34-36) and widens each d-dim query with a 0 (hierarchical_
    # cluster_index.cpp:1516-1520). filter_nsq = 6 (its ip2cos rule, index_conf.cpp:132-141).
    "ip2cos_d23": dict(n=6000, d=23, C=16, F=16, norm=False, mix="raw", P=8, T=64, topk=10,
                       nq=64, dup=0, ip2cos=True),
    # RealtimeInsertPuckIndex (realtime_insert_puck_index.cpp): 4000 base points, then 240
    # inserts (near the data, far from it into cells empty in the base, and repeats into
    # one cell), then searches through the reference's Index::search. 16 x 16 cells, so
    # about half the cells are empty in the base.
    "insert_pq_d16": dict(n=4000, d=16, C=16, F=16, norm=False, mix="int", P=4, T=64, topk=10,
                          nq=48, dup=0, pq=True, insert=240),
    "insert_flat_d16": dict(n=4000, d=16, C=16, F=16, norm=False, mix="int", P=4, T=64, topk=10,
                            nq=48, dup=0, insert=240),
    # the same on L2-normalised data (whether_norm): inserts are normalised by single_build
    "insert_cos_d16": dict(n=4000, d=16, C=16, F=16, norm=True, mix="gauss", P=4, T=64, topk=10,
                           nq=48, dup=0, pq=True, insert=240),
}


def make_data(case, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    n, d = case["n"], case["d"]
    ncomp = 64
    if case["mix"] == "int":
        centers = rng.uniform(0, 128, size=(ncomp, d))
        def draw(m):
            comp = rng.integers(0, ncomp, size=m)
            x = centers[comp] + rng.normal(0, 12, size=(m, d))
            return np.rint(np.clip(x, 0, 255)).astype(np.float32)
    else:
        centers = rng.normal(0, 1, size=(ncomp, d))
        def draw(m):
            comp = rng.integers(0, ncomp, size=m)
            x = (centers[comp] + rng.normal(0, 0.3, size=(m, d))).astype(np.float32)
            if case["mix"] != "raw":
                x /= np.linalg.norm(x, axis=1, keepdims=True)
            return x.astype(np.float32)
    base = draw(n)
    if case["dup"]:
        src = rng.integers(0, n, size=case["dup"])
        dst = rng.integers(0, n, size=case["dup"])
        base[dst] = base[src]
    queries = draw(case["nq"])
    if case.get("ip2cos"):
        sq = (base.astype(np.float64) ** 2).sum(1)
        extra = np.sqrt(np.maximum(sq.max() - sq, 0.0)).astype(np.float32)
        base = np.concatenate([base, extra[:, None]], axis=1)
    return base, queries


def insert_points(case, base, queries, seed=11):
    """Points to insert: near the data, far from it, and repeats of a few (integer
    data stays integer; other data is left unnormalised, the index normalises it)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    m, d = case["insert"], case["d"]
    integer = case["mix"] == "int"
    scale = 4.0 if integer else 0.2
    near = base[rng.integers(0, base.shape[0], m // 2)] + rng.normal(0, scale, (m // 2, d))
    far = rng.uniform(0, 255, (m // 4, d)) if integer else rng.normal(0, 3, (m // 4, d))
    rep = np.repeat(near[:(m - m // 2 - m // 4) // 2], 2, axis=0)
    pts = np.concatenate([near, far, rep])[:m]
    if integer:
        pts = np.rint(np.clip(pts, 0, 255))
    return pts.astype(np.float32)


def run_insert_case(name):
    """Base index by train()/build(); its files are kept as they are before any insert.
    Then RealtimeInsertPuckIndex::init() over them (plus the label file), insert() of
    every point in order, and Index::search of every query, one at a time."""
    case = CASES[name]
    base, queries = make_data(case)
    ins = insert_points(case, base, queries)
    # a third of the queries are inserted points, so their own records are found
    queries = np.concatenate([ins[::max(1, ins.shape[0] // (case["nq"] // 3))][:case["nq"] // 3],
                              queries[:case["nq"] - case["nq"] // 3]]).astype(np.float32)
    lib = ctypes.CDLL(REF_LIB)
    lib.ref_set_flag.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    lib.ref_open_realtime.restype = ctypes.c_void_p
    lib.ref_realtime_insert.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                        ctypes.c_char_p]
    lib.ref_realtime_search.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_uint32] + [
        ctypes.c_void_p] * 3
    lib.ref_close_realtime.argtypes = [ctypes.c_void_p]

    def flag(k, v):
        assert lib.ref_set_flag(k.encode(), str(v).encode()) == 0, k

    n, d, m = case["n"], case["d"], case["insert"]
    with tempfile.TemporaryDirectory() as tmp:
        idx = os.path.join(tmp, "index")
        os.makedirs(idx)
        index_io.write_fvecs(os.path.join(idx, "all_data.feat.bin"), base)
        flag("index_path", idx)
        flag("feature_dim", d)
        flag("coarse_cluster_count", case["C"])
        flag("fine_cluster_count", case["F"])
        flag("whether_norm", "true" if case["norm"] else "false")
        flag("whether_pq", "true" if case.get("pq") else "false")
        flag("kmeans_iterations_count", 2)
        flag("train_points_count", n)
        flag("pq_train_points_count", n)
        flag("threads_count", 4)
        flag("train_fea_file_name", os.path.join(tmp, "train_clusters.dat"))
        flag("train_pq_file_name", os.path.join(tmp, "train_pq.dat"))
        assert lib.ref_train_build() == 0, "reference train/build failed"
        flag("search_coarse_count", case["P"])
        flag("filter_topk", case["T"])
        flag("topk", case["topk"])
        flag("context_initial_pool_size", 2)
        files = {}
        for fn in sorted(os.listdir(idx)):
            with open(os.path.join(idx, fn), "rb") as f:
                files["file:" + fn] = np.frombuffer(f.read(), np.uint8)
        lengths = {fn: os.path.getsize(os.path.join(idx, fn)) for fn in os.listdir(idx)}
        with open(os.path.join(idx, "all_data.url"), "w") as f:
            for i in range(n):
                f.write(f"p{i}\n")
        h = lib.ref_open_realtime()
        assert h, "reference realtime init failed"
        for i in range(m):
            x = np.ascontiguousarray(ins[i])
            assert lib.ref_realtime_insert(h, x.ctypes.data, d, f"i{i}".encode()) == 0, i
        nq, k = queries.shape[0], case["topk"]
        dist = np.zeros((nq, k), np.float32)
        labels = np.full((nq, k), 0xFFFFFFFF, np.uint32)
        rn = ctypes.c_uint32(0)
        for i in range(nq):
            q = np.ascontiguousarray(queries[i])
            assert lib.ref_realtime_search(h, q.ctypes.data, k, dist[i].ctypes.data,
                                           labels[i].ctypes.data, ctypes.byref(rn)) == 0, i
        lib.ref_close_realtime(h)

        def tail(fn):
            with open(os.path.join(idx, fn), "rb") as f:
                return np.frombuffer(f.read()[lengths[fn]:], np.uint8)
        appended = {"appended:" + fn: tail(fn) for fn in lengths
                    if fn in ("cell_assign.dat", "filter_data.dat", "pq_data.dat")}
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, queries=queries, inserted=ins, dist=dist, labels=labels,
                            params=np.array([case["P"], case["T"], case["topk"]], np.int64),
                            **files, **appended)
        print(f"{name}: wrote {out} ({os.path.getsize(out)} bytes)")


def run_case(name):
    case = CASES[name]
    if case.get("insert"):
        return run_insert_case(name)
    base, queries = make_data(case)
    lib = ctypes.CDLL(REF_LIB)
    lib.ref_set_flag.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    lib.ref_open_searcher.restype = ctypes.c_void_p
    lib.ref_open_probe.restype = ctypes.c_void_p
    lib.ref_search.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                               ctypes.c_void_p, ctypes.c_void_p]
    lib.ref_probe.argtypes = [ctypes.c_void_p] + [ctypes.c_void_p] * 7
    lib.ref_memory_to_local.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.ref_search_one.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_uint32] + [ctypes.c_void_p] * 3

    def flag(k, v):
        assert lib.ref_set_flag(k.encode(), str(v).encode()) == 0, k

    with tempfile.TemporaryDirectory() as tmp:
        idx = os.path.join(tmp, "index")
        os.makedirs(idx)
        index_io.write_fvecs(os.path.join(idx, "all_data.feat.bin"), base)
        flag("index_path", idx)
        flag("feature_dim", case["d"])
        flag("coarse_cluster_count", case["C"])
        flag("fine_cluster_count", case["F"])
        flag("whether_norm", "true" if case["norm"] else "false")
        flag("whether_pq", "true" if case.get("pq") else "false")
        flag("ip2cos", 1 if case.get("ip2cos") else 0)
        flag("kmeans_iterations_count", 2)
        flag("train_points_count", case["n"])
        flag("pq_train_points_count", case["n"])
        flag("threads_count", 4)
        flag("train_fea_file_name", os.path.join(tmp, "train_clusters.dat"))
        flag("train_pq_file_name", os.path.join(tmp, "train_pq.dat"))
        assert lib.ref_train_build() == 0, "reference train/build failed"

        flag("search_coarse_count", case["P"])
        flag("filter_topk", case["T"])
        flag("topk", case["topk"])
        flag("context_initial_pool_size", 4)

        searcher = lib.ref_open_searcher()
        assert searcher, "reference init failed"
        nq, k = queries.shape[0], case["topk"]
        dist = np.zeros((nq, k), np.float32)
        labels = np.full((nq, k), 0xFFFFFFFF, np.uint32)
        q = np.ascontiguousarray(queries)
        lib.ref_search(searcher, nq, q.ctypes.data, k, dist.ctypes.data, labels.ctypes.data)

        probe = lib.ref_open_probe()
        assert probe
        P, T = case["P"], case["T"]
        nsq = index_io.read_index_conf(os.path.join(idx, "index.dat"))["filter_nsq"]
        ctag = np.zeros((nq, P), np.uint32)
        cdist = np.zeros((nq, P), np.float32)
        ftag = np.zeros((nq, T), np.uint32)
        fdist = np.zeros((nq, T), np.float32)
        fcnt = np.zeros(nq, np.uint32)
        nlut = min(nq, 8)
        lut = np.zeros((nlut, nsq * 256), np.float32)
        for i in range(nq):
            lp = lut[i].ctypes.data if i < nlut else None
            rc = lib.ref_probe(probe, q[i].ctypes.data, ctag[i].ctypes.data, cdist[i].ctypes.data,
                               ftag[i].ctypes.data, fdist[i].ctypes.data,
                               fcnt[i:i + 1].ctypes.data, lp)
            assert rc == 0, rc
        m2l = np.zeros(case["n"], np.uint32)
        lib.ref_memory_to_local(probe, m2l.ctypes.data)
        if case.get("ip2cos"):
            # PySearcher's contexts can carry a stale last query float on an ip2cos index
            # (normalization's memset counts bytes); the final results come from the
            # reference's Index::search on the probe's contexts instead, whose filter
            # tables above were computed with that float at 0.
            rn = ctypes.c_uint32(0)
            for i in range(nq):
                assert lib.ref_search_one(probe, q[i].ctypes.data, k, dist[i].ctypes.data,
                                          labels[i].ctypes.data, ctypes.byref(rn)) == 0

        files = {}
        for fn in sorted(os.listdir(idx)):
            with open(os.path.join(idx, fn), "rb") as f:
                files["file:" + fn] = np.frombuffer(f.read(), np.uint8)
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(
            out, queries=queries, dist=dist, labels=labels, coarse_tag=ctag, coarse_dist=cdist,
            filter_tag=ftag, filter_dist=fdist, filter_cnt=fcnt, lut=lut, memory_to_local=m2l,
            params=np.array([case["P"], case["T"], case["topk"]], np.int64), **files)
        print(f"{name}: wrote {out} ({os.path.getsize(out)} bytes)")


def main():
    names = sys.argv[1:] or list(CASES)
    if not os.path.exists(REF_LIB):
        subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j8"])
    for name in names:
        # One process per case: the reference keeps its flags in globals.
        if len(names) > 1:
            subprocess.check_call([sys.executable, os.path.abspath(__file__), name])
        else:
            run_case(name)


if __name__ == "__main__":
    main()
