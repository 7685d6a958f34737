"""Parity of the CUDA search path (through the C ABI) with the reference.

* golden cases: indexes built by the reference's own train()/build() and the
  outputs of its PySearcher::search -> distances and labels bit-identical,
  including tie order and the unfilled slots;
* indexes produced by the GPU builder at larger sizes -> bit-identical to the
  oracle (the C restatement pinned to the reference by test_oracle_golden.py);
* size-independent properties at the largest size (sortedness, exact
  distances of the returned ids, batch == one-at-a-time).
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
from puck_gb300 import index_io, native, py_puck_api

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    native.load(build_if_missing=True)


def test_golden_bit_exact(golden):
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = native.GpuIndex(index_dir, search_coarse_count=P, filter_topk=T, topk=k, max_batch=64)
    dist, ids, status = ix.search(z["queries"], k, return_status=True)
    assert (status == 0).all()
    assert np.array_equal(_bits(dist), _bits(z["dist"])), name
    assert np.array_equal(ids, z["labels"]), name
    ix.close()


def test_golden_py_api_mirror(golden):
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    py_puck_api.reset_gflags()
    py_puck_api.update_gflag("index_path", index_dir)
    py_puck_api.update_gflag("search_coarse_count", str(P))
    py_puck_api.update_gflag("filter_topk", str(T))
    py_puck_api.update_gflag("topk", str(k))
    s = py_puck_api.PySearcher()
    assert s.init() == 0
    q = z["queries"]
    n = q.shape[0]
    dist = np.zeros(n * k, np.float32)
    labels = np.zeros(n * k, np.uint32)
    assert s.search(n, q, k, dist, labels) == 0
    assert np.array_equal(_bits(dist), _bits(z["dist"].reshape(-1)))
    assert np.array_equal(labels, z["labels"].reshape(-1))
    # Index::search for one query
    d1, i1, rn = s.index.search_one(q[3], k)
    m = int((z["labels"][3] != native.NO_LABEL).sum())
    assert rn == m
    assert np.array_equal(_bits(d1[:rn]), _bits(z["dist"][3, :rn]))
    # topk above FLAGS_topk: the reference returns -1 per query and leaves outputs
    dist2 = np.full(n * (k + 1), 7.0, np.float32)
    labels2 = np.full(n * (k + 1), 5, np.uint32)
    assert s.search(n, q, k + 1, dist2, labels2) == 0
    assert (dist2 == 7.0).all() and (labels2 == 5).all()
    py_puck_api.reset_gflags()


def test_golden_scan_mode_matches_oracle(golden):
    """Scan mode: every record of the probed clusters; bit-identical to the oracle's
    restatement of the mode (same per-record distances as the reference)."""
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    T = min(T, 2048)
    ix = native.GpuIndex(index_dir, search_coarse_count=P, filter_topk=T, topk=k, max_batch=64,
                         mode=native.PGPU_MODE_SCAN)
    dist, ids, status = ix.search(z["queries"], k, return_status=True)
    orc = oracle.OracleIndex(index_dir)
    od, oi, ost = orc.search_batch(z["queries"], k, P, T, topk_max=k, scan=True)
    assert (status == 0).all() and (ost == 0).all()
    assert np.array_equal(_bits(dist), _bits(od)), name
    assert np.array_equal(ids, oi), name


def test_small_batches_and_chunking(golden):
    """max_batch smaller than n: several device passes give the same bits."""
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = native.GpuIndex(index_dir, search_coarse_count=P, filter_topk=T, topk=k, max_batch=7)
    dist, ids = ix.search(z["queries"], k)
    assert np.array_equal(_bits(dist), _bits(z["dist"]))
    assert np.array_equal(ids, z["labels"])


def _built_index(tmpdir, n, d, C, F, nsq, kind, seed, norm, pq=False):
    import torch
    from puck_gb300 import builder
    base = builder.gmm(n, d, 256, kind, seed)
    arrays = builder.build_index(base, C, F, nsq, norm, train_sample=min(n, 65536), iters=6,
                                 pq_sample=min(n, 32768), seed=seed, whether_pq=pq)
    index_io.write_index(tmpdir, base=arrays["base"], coarse=arrays["coarse"],
                         fine=arrays["fine"], cell_assign=arrays["cell_assign"],
                         filter_codebook=arrays["filter_codebook"],
                         filter_offsets=arrays["filter_offsets"],
                         filter_codes=arrays["filter_codes"], whether_norm=norm,
                         pq_codebook=arrays.get("pq_codebook"),
                         pq_offsets=arrays.get("pq_offsets"), pq_codes=arrays.get("pq_codes"))
    q = builder.gmm(256, d, 256, kind, seed, row_seed=seed + 77).cpu().numpy()
    del base
    torch.cuda.empty_cache()
    return q


@pytest.mark.parametrize("mode", [native.PGPU_MODE_EXACT, native.PGPU_MODE_SCAN])
@pytest.mark.parametrize("n,d,C,F,nsq,kind,norm,P,T,k,pq", [
    (60000, 64, 64, 64, 16, "int", False, 16, 200, 10, False),
    (80000, 96, 96, 80, 24, "unit", True, 24, 500, 100, False),
    (40000, 128, 50, 40, 32, "int", False, 50, 300, 20, False),
    (50000, 96, 64, 64, 24, "unit", True, 8, 300, 10, True),   # second-level PQ rerank
    (60000, 64, 32, 32, 16, "int", False, 12, 1280, 10, False),
    (60000, 64, 32, 32, 16, "int", False, 12, 2048, 10, False),  # the scan's largest filter_topk
])
def test_gpu_equals_oracle_builder_index(n, d, C, F, nsq, kind, norm, P, T, k, pq, mode):
    with tempfile.TemporaryDirectory() as tmp:
        q = _built_index(tmp, n, d, C, F, nsq, kind, 11, norm, pq=pq)
        ix = native.GpuIndex(tmp, search_coarse_count=P, filter_topk=T, topk=k, max_batch=100,
                             mode=mode)
        dist, ids = ix.search(q, k)
        orc = oracle.OracleIndex(tmp)
        od, oi, st = orc.search_batch(q, k, P, T, topk_max=k, nthreads=os.cpu_count(),
                                      scan=(mode == native.PGPU_MODE_SCAN))
        assert (st == 0).all()
        assert np.array_equal(_bits(dist), _bits(od))
        assert np.array_equal(ids, oi)
        stats = ix.last_stats()
        assert stats["records_scanned"] > 0 and stats["kernels"] > 0


def test_properties_large():
    """A 1M-point index: exact mode bit-identical to the oracle's restatement of the
    reference's search and scan mode to its restatement of the mode; size-independent
    checks: ascending distances, the returned distance equals the exact squared L2
    of the returned id, batch search equals one-query searches, and the zero-norm
    rejection."""
    import torch
    with tempfile.TemporaryDirectory() as tmp:
        q = _built_index(tmp, 1_000_000, 96, 512, 512, 24, "unit", 5, True)
        base = index_io.read_fvecs(os.path.join(tmp, "all_data.feat.bin"), 96)
        ix = native.GpuIndex(tmp, search_coarse_count=64, filter_topk=500, topk=100, max_batch=4096)
        dist, ids, status = ix.search(q, 100, return_status=True)
        assert (status == 0).all()
        assert (ids != native.NO_LABEL).all()
        assert np.all(np.diff(dist, axis=1) >= 0)
        qn = q / np.linalg.norm(q, axis=1, keepdims=True)
        exact = ((base[ids.astype(np.int64)] - qn[:, None, :]) ** 2).sum(-1)
        np.testing.assert_allclose(dist, exact, rtol=1e-4, atol=1e-5)
        for i in (0, 17, 255):
            d1, i1, rn = ix.search_one(q[i], 100)
            assert rn == 100
            assert np.array_equal(_bits(d1), _bits(dist[i]))
            assert np.array_equal(i1, ids[i])
        # the same queries through the oracle's restatement of the reference's search:
        # exact mode bit for bit at this size, and scan mode against its restatement
        orc = oracle.OracleIndex(tmp)
        od, oi, ost = orc.search_batch(q, 100, 64, 500, topk_max=100, nthreads=os.cpu_count())
        assert (ost == 0).all()
        assert np.array_equal(_bits(dist), _bits(od))
        assert np.array_equal(ids, oi)
        ix.set_search_params(mode=native.PGPU_MODE_SCAN, search_coarse_count=8)
        sd, si = ix.search(q, 10)
        od, oi, _ = orc.search_batch(q, 10, 8, 500, topk_max=100, nthreads=os.cpu_count(),
                                     scan=True)
        assert np.array_equal(_bits(sd), _bits(od))
        assert np.array_equal(si, oi)
        orc.close()
        ix.set_search_params(mode=native.PGPU_MODE_EXACT, search_coarse_count=64)
        bad = q[:4].copy()
        bad[1] = 0.0
        d2, i2, st2 = ix.search(bad, 10, return_status=True)
        assert st2.tolist() == [0, native.PGPU_E_ZERO_NORM, 0, 0]
        assert (i2[1] == native.NO_LABEL).all()
        assert np.array_equal(i2[0], ids[0, :10])
        del base
        torch.cuda.empty_cache()


def test_nearest_center_matches_oracle():
    import torch
    rng = np.random.default_rng(0)
    cents = rng.normal(size=(300, 24)).astype(np.float32)
    x = rng.normal(size=(5000, 24)).astype(np.float32)
    x[:10] = cents[:10]  # exact hits
    oa, od = oracle.nearest_center(cents, x)
    ct = torch.from_numpy(cents).cuda()
    xt = torch.from_numpy(x).cuda()
    a = torch.empty(5000, dtype=torch.int32, device="cuda")
    dd = torch.empty(5000, dtype=torch.float32, device="cuda")
    native.nearest_center(ct, xt, a, dd, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert np.array_equal(a.cpu().numpy(), oa)
    assert np.array_equal(_bits(dd.cpu().numpy()), _bits(od))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [native.PGPU_MODE_EXACT, native.PGPU_MODE_SCAN])
def test_ip2cos_index_equals_oracle(mode):
    """ip2cos = 1 (inner product recast as L2): the index holds [x, sqrt(M^2 - |x|^2)]
    rows of d + 1 values; callers pass d-value queries, which get a 0 appended and no
    normalisation (hierarchical_cluster_index.cpp:1516-1520). Host batch, single-query,
    device-buffer and serving entry points all read d floats per query."""
    import torch
    from puck_gb300 import builder
    D = 47
    x = builder.gmm(40000, D, 256, "int", 21).float() / 64.0
    sq = (x.double() ** 2).sum(1)
    extra = torch.sqrt(torch.clamp(sq.max() - sq, min=0.0)).float()
    base = torch.cat([x, extra[:, None]], dim=1).contiguous()
    arrays = builder.build_index(base, 48, 40, 12, False, train_sample=40000, iters=6,
                                 pq_sample=32768, seed=21)
    arrays["ip2cos"] = 1
    q = (builder.gmm(200, D, 256, "int", 21, row_seed=99).float() / 64.0).cpu().numpy()
    del x, base
    torch.cuda.empty_cache()
    P, T, k = 12, 300, 10
    ix = native.GpuIndex(arrays=arrays, search_coarse_count=P, filter_topk=T, topk=k,
                         max_batch=64, mode=mode)
    assert ix.info.feature_dim == D + 1 and ix.info.query_dim == D and ix.info.ip2cos == 1
    dist, ids, status = ix.search(q, k, return_status=True)
    orc = oracle.OracleIndex(arrays=arrays)
    od, oi, st = orc.search_batch(q, k, P, T, topk_max=k, nthreads=os.cpu_count(),
                                  scan=(mode == native.PGPU_MODE_SCAN))
    assert (status == 0).all() and (st == 0).all()
    assert np.array_equal(_bits(dist), _bits(od))
    assert np.array_equal(ids, oi)
    d1, i1, rn = ix.search_one(q[5], k)
    assert rn == k and np.array_equal(_bits(d1), _bits(dist[5])) and np.array_equal(i1, ids[5])
    qd = torch.from_numpy(q).cuda()
    dd = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    di = torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda")
    ix.search_device(q.shape[0], qd, k, dd, di)
    torch.cuda.synchronize()
    assert np.array_equal(_bits(dd.cpu().numpy()), _bits(dist))
    assert np.array_equal(di.cpu().numpy().view(np.uint32), ids)
    srv = native.Server(ix, max_batch=64, scratch_budget_bytes=64 << 20, max_slots=2)
    try:
        t = srv.submit(q[:37], k)
        sd, si, sst, _ = srv.wait(t, timeout_ms=60000)
    finally:
        srv.close()
    assert (sst == 0).all()
    assert np.array_equal(_bits(sd), _bits(dist[:37])) and np.array_equal(si, ids[:37])
