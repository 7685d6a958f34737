"""CPU tests of the benchmark's host logic (no GPU).

* recall@10 is tie-aware as ann-benchmarks computes it
  (ann-benchmarks/benchmark/plotting/metrics.py:15-40): ground-truth ids whose FP64
  distance is within 1e-6 of the 10th count as hits;
* the CPU port's operating point is the smallest search_coarse_count of the sweep whose
  recall reaches 0.95, else the most accurate one;
* the default workload keeps the shapes of the 100M learned-probe configuration, and
  the file cache of a workload is keyed by its parameters.
"""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _gt(nq=4, cand=16):
    ids = np.tile(np.arange(cand), (nq, 1))
    dist = np.tile(np.arange(cand, dtype=np.float64), (nq, 1))
    return ids, dist


def test_recall_exact_and_partial():
    gt_ids, gt_dist = _gt()
    run = gt_ids[:, :10].copy()
    assert bench.recall_at(gt_ids, gt_dist, run) == 1.0
    run[:, 5:] = 100 + np.arange(5)  # half of the ids are not neighbours
    assert bench.recall_at(gt_ids, gt_dist, run) == 0.5


def test_recall_counts_ties_at_the_tenth_distance():
    gt_ids, gt_dist = _gt(nq=1)
    gt_dist[0, 10] = gt_dist[0, 9] + 5e-7  # the 11th neighbour ties the 10th within 1e-6
    gt_dist[0, 11] = gt_dist[0, 9] + 5e-6  # the 12th does not
    run = gt_ids[:, :10].copy()
    run[0, 9] = 10  # the tied one instead of the 10th: still a hit
    assert bench.recall_at(gt_ids, gt_dist, run) == 1.0
    run[0, 9] = 11  # the untied one: a miss
    assert bench.recall_at(gt_ids, gt_dist, run) == 0.9
    rows = bench.recall_rows(gt_ids, gt_dist, run)
    assert rows.shape == (1,) and rows[0] == 0.9


class _FakePort:
    """search_batch returning the true top-10 on a fraction of queries that grows with P."""

    def __init__(self, gt_ids, good_by_p):
        self.gt_ids = gt_ids
        self.good_by_p = good_by_p

    def search_batch(self, q, k, P, T, topk_max=100, nthreads=1):
        n = q.shape[0]
        ids = self.gt_ids[:n, :k].copy()
        bad = int(round(n * (1.0 - self.good_by_p[P])))
        ids[:bad] = 10_000 + np.arange(k)  # all misses
        return np.zeros((n, k), np.float32), ids, np.zeros(n, np.int32)


def test_cpu_operating_point_smallest_reaching_target():
    nq = 100
    gt_ids, gt_dist = _gt(nq=nq)
    q = np.zeros((nq, 4), np.float32)
    w = dict(bench.WORKLOADS["cosine_1m"], cpu_sweep=(1, 2, 4, 8))
    port = _FakePort(gt_ids, {1: 0.80, 2: 0.94, 4: 0.96, 8: 0.99})
    P, reached, sweep = bench.cpu_operating_point(port, q, gt_ids, gt_dist, w, sample=nq, threads=1)
    assert (P, reached) == (4, True)
    assert [e["search_coarse_count"] for e in sweep] == [1, 2, 4]  # stops at the first hit


def test_cpu_operating_point_most_accurate_when_none_reaches():
    nq = 100
    gt_ids, gt_dist = _gt(nq=nq)
    q = np.zeros((nq, 4), np.float32)
    w = dict(bench.WORKLOADS["cosine_1m"], cpu_sweep=(1, 2, 4))
    port = _FakePort(gt_ids, {1: 0.80, 2: 0.90, 4: 0.85})
    P, reached, sweep = bench.cpu_operating_point(port, q, gt_ids, gt_dist, w, sample=nq, threads=1)
    assert (P, reached) == (2, False)
    assert len(sweep) == 3


def test_default_workload_is_the_100m_configuration():
    w = bench.WORKLOADS["learned_100m"]
    assert (w["n"], w["d"], w["ncomp"], w["kind"]) == (100_000_000, 96, 16384, "unit")
    assert (w["C"], w["F"], w["nsq"], w["k"], w["nq"]) == (4000, 4000, 24, 10, 10000)
    assert w["norm"] and w["probe_fallback"] == 200
    # filter_topk: the reference's default, 11 x its topk flag of 100
    assert w["T"] == 1100
    cfg = bench.workload_config("learned_100m", w)
    assert cfg["workload"] == "learned_100m" and cfg["filter_topk"] == 1100
    assert cfg["recall_target"] == bench.TARGET_RECALL == 0.95


def test_cache_dir_is_keyed_by_parameters(monkeypatch, tmp_path):
    monkeypatch.setenv("PUCK_BENCH_CACHE", str(tmp_path))
    w = bench.WORKLOADS["cosine_1m"]
    a = bench.cache_dir("cosine_1m", w)
    assert a == bench.cache_dir("cosine_1m", dict(w))
    assert a != bench.cache_dir("cosine_1m", dict(w, T=w["T"] + 1))
    assert os.path.dirname(a) == str(tmp_path)
