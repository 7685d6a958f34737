"""GPU tests of the realtime-insert overlay (pgpu_realtime_open / pgpu_insert,
RealtimeInsertPuckIndex, puck/puck/realtime_insert_puck_index.cpp).

* after the reference's own base index and its 240 inserts (golden fixtures made by
  the reference itself), exact-mode searches are bit-identical to the reference's
  Index::search over base and inserted points, ids included;
* scan mode (and the precision form) over inserted points: bit-identical to the
  oracle's restatement of the mode, and a query equal to an inserted point finds it
  at distance 0;
* inserting in several batches gives the same index as one batch;
* a non-finite feature is not inserted, and the capacity is enforced.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
from puck_gb300 import index_io, native

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NAMES = ["insert_pq_d16", "insert_flat_d16", "insert_cos_d16"]


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _open(name, **params):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    tmp = tempfile.mkdtemp(prefix="puck_ins_")
    index_io.materialize_npz_index(z, tmp)
    P, T, k = [int(v) for v in z["params"]]
    ix = native.GpuIndex(tmp, search_coarse_count=P, filter_topk=T, topk=max(k, 10),
                         max_batch=128, **params)
    return z, tmp, ix, (P, T, k)


def _oracle_after_inserts(tmp, inserted):
    orc = oracle.OracleIndex(tmp)
    orc.realtime_open()
    for x in inserted:
        orc.insert(x)
    return orc


@pytest.mark.parametrize("name", NAMES)
def test_exact_mode_matches_reference_after_inserts(name):
    native.load(build_if_missing=True)
    z, tmp, ix, (P, T, k) = _open(name)
    ix.realtime_open(1000)
    ids = ix.insert(z["inserted"])
    conf = index_io.read_index_conf(os.path.join(tmp, "index.dat"))
    n = conf["total_point_count"]
    assert ids.tolist() == list(range(n, n + len(ids)))
    dist, labels, status = ix.search(z["queries"], k, return_status=True)
    assert (status == 0).all()
    assert np.array_equal(_bits(dist), _bits(z["dist"])), name
    assert np.array_equal(labels, z["labels"]), name
    # single-query entry point too
    for i in (0, len(z["queries"]) - 1):
        d1, i1, rn = ix.search_one(z["queries"][i], k)
        assert np.array_equal(_bits(d1), _bits(z["dist"][i]))
        assert np.array_equal(i1, z["labels"][i])
    ix.close()


@pytest.mark.parametrize("name", NAMES)
def test_scan_mode_over_inserts_matches_oracle(name):
    """Scan mode over base and inserted records, FP32: the oracle's restatement of
    the mode on the same realtime index, bit for bit; a query equal to an inserted
    point (not normalised away) finds it first at distance 0."""
    z, tmp, ix, (P, T, k) = _open(name, mode=native.PGPU_MODE_SCAN)
    ix.realtime_open(1000)
    ids = ix.insert(z["inserted"])
    dist, labels, status = ix.search(z["queries"], k, return_status=True)
    assert (status == 0).all()
    orc = _oracle_after_inserts(tmp, z["inserted"])
    od, oi, st = orc.search_batch(z["queries"], k, P, T, topk_max=max(k, 10), scan=True)
    assert (st == 0).all()
    assert np.array_equal(_bits(dist), _bits(od)), name
    assert np.array_equal(labels, oi), name
    if "pq" not in name:
        # the inserted points themselves as queries: found among the results, at
        # distance 0 on an index that stores them as given
        q = z["inserted"][:16]
        d2, l2 = ix.search(q, k)
        found = [ids[i] in l2[i].astype(np.int64).tolist() for i in range(len(q))]
        assert np.mean(found) >= 0.9
        if "flat" in name:
            assert np.mean(d2[:, 0] == 0.0) >= 0.9
    orc.close()
    ix.close()


def test_precision_form_over_inserts():
    """The precision form (BF16 screen, FP16 table) over the realtime index: its ids
    agree with the FP32 scan's on nearly every query, and an id both return has the
    same exact FP32 distance."""
    z, tmp, ix, (P, T, k) = _open("insert_flat_d16", mode=native.PGPU_MODE_SCAN,
                                  precision=native.PGPU_PRECISION_BF16, filter_margin=16)
    ix.realtime_open(1000)
    ix.insert(z["inserted"])
    dist, labels = ix.search(z["queries"], k)
    orc = _oracle_after_inserts(tmp, z["inserted"])
    od, oi, _ = orc.search_batch(z["queries"], k, P, T, topk_max=max(k, 10), scan=True)
    agree = np.mean([len(set(a.tolist()) & set(b.tolist())) / k for a, b in zip(labels, oi)])
    assert agree >= 0.95, agree
    for i in range(len(labels)):
        mine = dict(zip(labels[i].tolist(), dist[i].tolist()))
        ref = dict(zip(oi[i].tolist(), od[i].tolist()))
        for t in set(mine) & set(ref):
            assert mine[t] == pytest.approx(ref[t], rel=1e-6, abs=1e-6), (i, t)
    orc.close()
    ix.close()


def test_batches_equal_one_batch():
    z, tmp, ix, (P, T, k) = _open("insert_flat_d16")
    ix.realtime_open(1000)
    ix.insert(z["inserted"])
    d1, l1 = ix.search(z["queries"], k)
    ix.close()
    z, tmp, ix, _ = _open("insert_flat_d16")
    ix.realtime_open(1000)
    x = z["inserted"]
    ids = np.concatenate([ix.insert(x[:7]), ix.insert(x[7:100]), ix.insert(x[100:])])
    d2, l2 = ix.search(z["queries"], k)
    n = index_io.read_index_conf(os.path.join(tmp, "index.dat"))["total_point_count"]
    assert ids.tolist() == list(range(n, n + len(x)))
    assert np.array_equal(_bits(d1), _bits(d2))
    assert np.array_equal(l1, l2)
    ix.close()


def test_rejects_bad_features_and_enforces_capacity():
    z, tmp, ix, (P, T, k) = _open("insert_cos_d16")
    ix.realtime_open(4)
    x = z["inserted"][:3].copy()
    x[1] = np.nan
    ids = ix.insert(x)
    assert ids[1] == -1 and ids[0] >= 0 and ids[2] == ids[0] + 1
    zero = np.zeros((1, x.shape[1]), np.float32)  # zero norm on a normalising index
    assert ix.insert(zero)[0] == -1
    ix.insert(z["inserted"][3:5])  # fills the capacity of 4
    with pytest.raises(native.PuckGpuError):
        ix.insert(z["inserted"][5:6])
    with pytest.raises(native.PuckGpuError):
        ix.realtime_open(10)  # already open
    ix.close()
