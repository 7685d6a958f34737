"""GPU tests of the serving loop (pgpu_server_*): continuous batching on CUDA graphs.

Requests of uneven size and top-k are submitted from several threads while
others are on the GPU. Each request's results must be bit-identical to a
synchronous pgpu_search_batch of the same queries (alone), in both search modes.
"""
import os
import random
import tempfile
import threading

import numpy as np
import pytest

from puck_gb300 import builder, index_io, native

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def built_index():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    native.load(build_if_missing=True)
    tmp = tempfile.mkdtemp(prefix="puck_server_")
    base = builder.gmm(120_000, 64, 256, "unit", 21)
    arrays = builder.build_index(base, 96, 96, 16, True, train_sample=65536, iters=6,
                                 pq_sample=32768, seed=21)
    index_io.write_index(tmp, base=arrays["base"], coarse=arrays["coarse"], fine=arrays["fine"],
                         cell_assign=arrays["cell_assign"],
                         filter_codebook=arrays["filter_codebook"],
                         filter_offsets=arrays["filter_offsets"],
                         filter_codes=arrays["filter_codes"], whether_norm=True)
    q = builder.gmm(3000, 64, 256, "unit", 21, row_seed=99).cpu().numpy()
    del base
    torch.cuda.empty_cache()
    return tmp, q


@pytest.mark.parametrize("mode", [native.PGPU_MODE_SCAN, native.PGPU_MODE_EXACT])
def test_server_results_equal_synchronous(built_index, mode):
    path, q = built_index
    ix = native.GpuIndex(path, search_coarse_count=6, filter_topk=300, topk=50, max_batch=4096,
                         mode=mode)
    ref = {k: ix.search(q, k) for k in (10, 50)}
    srv = native.Server(ix, max_batch=256, scratch_budget_bytes=256 << 20, max_slots=3)
    rng = random.Random(5)
    reqs = []
    pos = 0
    while pos < q.shape[0]:
        n = min(rng.randint(1, 96), q.shape[0] - pos)
        reqs.append((pos, n, rng.choice((10, 50))))
        pos += n
    results = {}
    lock = threading.Lock()

    def client(part):
        for (start, n, k) in part:
            t = srv.submit(q[start:start + n], k)
            with lock:
                results[(start, n, k)] = t

    threads = [threading.Thread(target=client, args=(reqs[i::3],)) for i in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    lat = []
    for (start, n, k), ticket in results.items():
        dist, ids, status, us = srv.wait(ticket, timeout_ms=60000)
        assert (status == 0).all()
        assert np.array_equal(_bits(dist), _bits(ref[k][0][start:start + n]))
        assert np.array_equal(ids, ref[k][1][start:start + n])
        lat.append(us)
    st = srv.stats()
    assert st["requests_done"] == len(reqs) and st["queries_done"] == q.shape[0]
    assert st["slots"] >= 2
    assert st["batches"] < len(reqs)          # several requests shared one batch
    assert st["graphs_captured"] >= 1 and st["graph_launches"] == st["batches"]
    assert min(lat) > 0
    srv.close()
    ix.close()


def test_server_rejects_bad_requests(built_index):
    path, q = built_index
    ix = native.GpuIndex(path, search_coarse_count=4, filter_topk=200, topk=20, max_batch=512,
                         mode=native.PGPU_MODE_SCAN)
    srv = native.Server(ix, max_batch=64, scratch_budget_bytes=64 << 20, max_slots=2)
    with pytest.raises(native.PuckGpuError) as e:
        srv.submit(q[:65], 10)
    assert e.value.code == native.PGPU_E_LIMIT
    with pytest.raises(native.PuckGpuError) as e:
        srv.submit(q[:4], 21)
    assert e.value.code == native.PGPU_E_INVALID
    t = srv.submit(q[:3], 20)
    dist, ids, status, us = srv.wait(t, timeout_ms=60000)
    d2, i2 = ix.search(q[:3], 20)
    assert np.array_equal(ids, i2)
    with pytest.raises(native.PuckGpuError) as e:
        native.Server(ix, max_batch=1024, scratch_budget_bytes=1024, max_slots=2)
    assert e.value.code == native.PGPU_E_LIMIT
    srv.close()
    ix.close()
