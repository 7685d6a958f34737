"""Pins the oracle (the C restatement) to the reference's own outputs.

The golden fixtures hold index files built by the reference's train()/build()
and the outputs of its PySearcher::search plus per-query intermediates. The
oracle must reproduce every one bit for bit: memory order, probed coarse list,
LUT, filter-heap layout (the reference leaves a full heap unsorted and the
rerank walks it in that order), final distances and ids.
"""
import numpy as np
import pytest

import oracle
from puck_gb300 import index_io


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_oracle_matches_reference(golden):
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = oracle.OracleIndex(index_dir)
    assert np.array_equal(ix.memory_to_local(), z["memory_to_local"])
    nq = z["queries"].shape[0]
    for i in range(nq):
        rc, dist, ids, rn, tr = ix.search_one(z["queries"][i], k, P, T, topk_max=k, trace=True)
        assert rc == 0
        assert np.array_equal(tr["coarse_tag"], z["coarse_tag"][i])
        assert np.array_equal(_bits(tr["coarse_dist"]), _bits(z["coarse_dist"][i]))
        cnt = tr["filter_cnt"]
        assert cnt == z["filter_cnt"][i]
        assert np.array_equal(tr["filter_tag"][:cnt], z["filter_tag"][i, :cnt])
        assert np.array_equal(_bits(tr["filter_dist"][:cnt]), _bits(z["filter_dist"][i, :cnt]))
        if i < z["lut"].shape[0]:
            assert np.array_equal(_bits(tr["lut"]), _bits(z["lut"][i]))
        assert np.array_equal(_bits(dist[:rn]), _bits(z["dist"][i, :rn]))
        assert np.array_equal(ids[:rn], z["labels"][i, :rn])


def test_oracle_batch_equals_single(golden):
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = oracle.OracleIndex(index_dir)
    dist, ids, status = ix.search_batch(z["queries"], k, P, T, topk_max=k, nthreads=4)
    assert (status == 0).all()
    for i in range(z["queries"].shape[0]):
        _, d1, i1, rn, _ = ix.search_one(z["queries"][i], k, P, T, topk_max=k)
        assert np.array_equal(_bits(dist[i, :rn]), _bits(d1[:rn]))
        assert np.array_equal(ids[i, :rn], i1[:rn])


def test_oracle_rejects_bad_requests(golden):
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = oracle.OracleIndex(index_dir)
    # topk above the configured maximum is an error (puck_index.cpp:560-563)
    rc, *_ = ix.search_one(z["queries"][0], k + 1, P, T, topk_max=k)
    assert rc == -1
    if ix.whether_norm:
        rc, *_ = ix.search_one(np.zeros(ix.d, np.float32), k, P, T, topk_max=k)
        assert rc == -2


def test_nearest_center_known_answer():
    # kmeans.cpp:221-258: argmin of |x|^2 + |c|^2 - 2 x.c, first index wins ties.
    cents = np.array([[0, 0], [2, 0], [0, 2], [2, 0]], np.float32)
    x = np.array([[0.1, 0.1], [1.9, 0.2], [1.0, 0.0], [0.0, 3.0]], np.float32)
    assign, dis = oracle.nearest_center(cents, x)
    assert assign.tolist() == [0, 1, 0, 2]  # [1,0] ties between 0 and 1 -> 0
    np.testing.assert_allclose(dis, [0.02, 0.05, 1.0, 1.0], rtol=1e-5, atol=1e-6)


def test_nearest_cell_assign_is_exact_argmin():
    rng = np.random.default_rng(3)
    coarse = rng.normal(size=(6, 8)).astype(np.float32)
    fine = (0.3 * rng.normal(size=(5, 8))).astype(np.float32)
    # the reference sorts fine rows by descending norm at train time
    fine = fine[np.argsort(-np.linalg.norm(fine, axis=1), kind="stable")]
    x = rng.normal(size=(200, 8)).astype(np.float32)
    cell, dist = oracle.nearest_cell_assign(coarse, fine, x)
    cent = (coarse[:, None, :] + fine[None, :, :]).reshape(-1, 8).astype(np.float64)
    full = ((x[:, None, :].astype(np.float64) - cent[None]) ** 2).sum(-1) / 2
    best = full.min(1)
    # the pruned walk must land on an exact minimiser (up to float rounding)
    assert np.all(full[np.arange(len(x)), cell] <= best + 1e-4)


def test_nearest_cell_assign_matches_reference(golden):
    """The oracle's nearest_cell_assign gives the reference's own cell_assign.dat
    (hierarchical_cluster_index.cpp:1042-1138) on every golden index."""
    name, z, index_dir = golden
    a = index_io.read_index(index_dir)
    base = np.ascontiguousarray(a["base"], np.float32)
    cell, _ = oracle.nearest_cell_assign(a["coarse"], a["fine"], base)
    assert np.array_equal(cell, np.asarray(a["cell_assign"]).astype(np.uint32)), name


def test_scan_mode_distances_agree_with_walk(golden):
    """Both modes compute a record's filter distance with the reference's formula.
    Where scan mode sums the table in its rotated order (nsq a multiple of 4 up to
    32), every record in the walk's filter heap that the scan also keeps has the
    same distance to within the rounding of the reassociated sum (bounded from the
    query's table in FP64); otherwise the same bits. The scan keeps at least as good
    a filter_topk, to the same slack."""
    name, z, index_dir = golden
    P, T, k = [int(v) for v in z["params"]]
    ix = oracle.OracleIndex(index_dir)
    a = index_io.read_index(index_dir)
    nsq = int(np.asarray(a["filter_codebook"]).shape[0])
    rotated = nsq % 4 == 0 and nsq <= 32
    for i in range(0, z["queries"].shape[0], 4):
        _, _, _, _, tw = ix.search_one(z["queries"][i], k, P, T, topk_max=k, trace=True)
        _, _, _, _, ts = ix.search_one(z["queries"][i], k, P, T, topk_max=k, trace=True,
                                       scan=True)
        walk = dict(zip(tw["filter_tag"][:tw["filter_cnt"]].tolist(),
                        tw["filter_dist"][:tw["filter_cnt"]].tolist()))
        scan = dict(zip(ts["filter_tag"][:ts["filter_cnt"]].tolist(),
                        ts["filter_dist"][:ts["filter_cnt"]].tolist()))
        # a record's table sum is at most nsq times the largest entry; bound the
        # reassociation by (nsq + 2) roundings of that and of the largest |t|
        lut = tw["lut"].astype(np.float64)
        slack = (nsq + 2) * 2.0 ** -23 * (2 * np.abs(lut).max() * nsq + max(
            np.abs(tw["filter_dist"][:tw["filter_cnt"]]).max(initial=0.0), 1e-30))
        for tag in set(walk) & set(scan):
            if rotated:
                assert abs(walk[tag] - scan[tag]) <= slack, (name, tag)
            else:
                assert _bits(np.float32(walk[tag])) == _bits(np.float32(scan[tag])), (name, tag)
        assert ts["filter_cnt"] >= tw["filter_cnt"]
        ws = np.sort(tw["filter_dist"][:tw["filter_cnt"]]).astype(np.float64)
        ss = ts["filter_dist"][:ts["filter_cnt"]].astype(np.float64)
        assert np.all(ss[:len(ws)] <= ws + (slack if rotated else 0.0))


def test_oracle_puck_assign_matches_reference(golden):
    """The build's encoder (puck_assign): re-encoding each golden index's vectors from
    its cell assignment and codebooks gives the reference's filter_data.dat (and
    pq_data.dat) records byte for byte."""
    from puck_gb300 import index_io
    name, z, index_dir = golden
    a = index_io.read_index(index_dir)
    f_off, f_codes, p_off, p_codes = oracle.puck_assign(
        a["base"], a["cell_assign"], a["coarse"], a["fine"], a["filter_codebook"],
        a.get("pq_codebook"))
    assert np.array_equal(_bits(f_off), _bits(a["filter_offsets"])), name
    assert np.array_equal(f_codes, a["filter_codes"]), name
    if a.get("pq_codebook") is not None:
        assert np.array_equal(_bits(p_off), _bits(a["pq_offsets"])), name
        assert np.array_equal(p_codes, a["pq_codes"]), name


def test_oracle_ip2cos_arrays_equal_files():
    """The ip2cos golden index loaded from its files and from arrays (with ip2cos set)
    searches alike: d - 1 value queries widened by a 0."""
    import os
    import tempfile
    from puck_gb300 import index_io
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ip2cos_d23.npz"))
    P, T, k = [int(v) for v in z["params"]]
    with tempfile.TemporaryDirectory() as tmp:
        index_io.materialize_npz_index(z, tmp)
        a = index_io.read_index(tmp)
        assert a["ip2cos"] == 1 and a["coarse"].shape[1] == z["queries"].shape[1] + 1
        by_file = oracle.OracleIndex(tmp)
        by_arrays = oracle.OracleIndex(arrays=a)
        d1, i1, s1 = by_file.search_batch(z["queries"], k, P, T, topk_max=100)
        d2, i2, s2 = by_arrays.search_batch(z["queries"], k, P, T, topk_max=100)
    assert (s1 == 0).all() and (s2 == 0).all()
    assert np.array_equal(_bits(d1), _bits(d2)) and np.array_equal(i1, i2)
    assert np.array_equal(_bits(d1), _bits(z["dist"])) and np.array_equal(i1, z["labels"])


@pytest.mark.parametrize("name", ["insert_pq_d16", "insert_flat_d16", "insert_cos_d16"])
def test_oracle_realtime_insert_matches_reference(name):
    """RealtimeInsertPuckIndex (realtime_insert_puck_index.cpp): after the reference's own
    base index, 240 inserts. The oracle's inserted records equal what the reference
    appended to its index files (cell_assign.dat, filter_data.dat, pq_data.dat), and its
    searches over base and inserted points equal the reference's Index::search, bit for
    bit."""
    import os
    import tempfile
    from puck_gb300 import index_io
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    P, T, k = [int(v) for v in z["params"]]
    with tempfile.TemporaryDirectory() as tmp:
        index_io.materialize_npz_index(z, tmp)
        conf = index_io.read_index_conf(os.path.join(tmp, "index.dat"))
        orc = oracle.OracleIndex(tmp)
    orc.realtime_open()
    n = conf["total_point_count"]
    ids = [orc.insert(x) for x in z["inserted"]]
    assert ids == list(range(n, n + len(ids)))
    pq_nsq = conf["nsq"] if conf["whether_pq"] else 0
    cell, off, codes, poff, pcodes = orc.inserted_records(pq_nsq)
    ac = z["appended:cell_assign.dat"].view(np.uint32)
    rec = z["appended:filter_data.dat"].reshape(len(ac), -1)
    assert np.array_equal(cell, ac)
    assert np.array_equal(_bits(off), rec[:, :4].copy().view(np.uint32).ravel())
    assert np.array_equal(codes, rec[:, 4:4 + codes.shape[1]])
    if pq_nsq:
        prec = z["appended:pq_data.dat"].reshape(len(ac), -1)
        assert np.array_equal(_bits(poff), prec[:, :4].copy().view(np.uint32).ravel())
        assert np.array_equal(pcodes, prec[:, 4:4 + pq_nsq])
    for i, q in enumerate(z["queries"]):
        rc, d, ids_, rn, _ = orc.search_one(q, k, P, T, topk_max=k)
        assert rc == 0
        assert np.array_equal(_bits(d), _bits(z["dist"][i])), (name, i)
        assert np.array_equal(ids_, z["labels"][i]), (name, i)


def test_oracle_realtime_scan_mode_finds_inserted_points():
    """The library's scan mode on a realtime index: every inserted point of a probed cell
    is a candidate, so a query equal to an inserted point (the first third of the
    golden queries) finds its own id at distance 0, as the exact walk does."""
    import os
    import tempfile
    from puck_gb300 import index_io
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "insert_flat_d16.npz"))
    P, T, k = [int(v) for v in z["params"]]
    with tempfile.TemporaryDirectory() as tmp:
        index_io.materialize_npz_index(z, tmp)
        n = index_io.read_index_conf(os.path.join(tmp, "index.dat"))["total_point_count"]
        orc = oracle.OracleIndex(tmp)
    orc.realtime_open()
    ins = z["inserted"]
    for x in ins:
        orc.insert(x)
    nq = len(z["queries"]) // 3
    for scan in (False, True):
        d, ids, st = orc.search_batch(z["queries"][:nq], k, P, T, topk_max=k, scan=scan)
        assert (st == 0).all()
        for i in range(nq):
            own = [n + j for j in range(len(ins)) if np.array_equal(ins[j], z["queries"][i])]
            assert own and any(o in ids[i] for o in own), (scan, i)
            assert d[i][0] == 0.0
