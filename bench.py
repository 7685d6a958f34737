#!/usr/bin/env python
"""Benchmark: Puck's batched search on one GB300, QPS at recall@10 >= 0.95.

Workload (default "learned_100m"): 100M base vectors, d=96, float32, drawn from
a 16384-component Gaussian mixture (centres N(0,1), per-dim sigma 0.3) and
L2-normalised; 10k held-out normalised queries from the same mixture; coarse =
fine = 4000 clusters; filter PQ 24 subspaces x 256 (uint8 codes); filter_topk
1100 (the reference's default, 11 x its topk flag of 100); top-10. The learned
probe (MLP 96 -> 512 -> 512 -> 4000, GELU) is trained on the GPU on fresh
queries of the same mixture, labelled with the coarse clusters of their
brute-force top-10, with a confidence fallback to search_coarse_count = 200.
Data are seeded synthetic (no dataset download); the index is built on the GPU
in the reference's formats.

One "step" = one batch search of all 10k queries at an operating point: the
smallest-work setting of a form whose recall@10 against an FP64 brute-force
oracle reaches 0.95.
  value  : queries/s of the learned probe + BF16 form, queries and outputs
           resident in HBM (device API)
  e2e    : the same through pgpu_search_batch with pinned host buffers
           (host->device query copy and device->host result copy inside)
  plain  : the plain FP32 GPU path at its own operating point, timed the same way
The index (codes 2.8 GB, vectors 38 GB) is far larger than L2, so timed steps
run back to back without an L2 flush.

The CPU leg (rank 0) runs the oracle port of the reference's search on the host
cores: it finds the port's own operating point (smallest search_coarse_count
with recall >= 0.95 on a sample, or its most accurate one), times it, and
checks the GPU path against it on a sample of the same queries (exact mode bit
for bit; scan-mode and headline top-10 id agreement with the reference's search).

--impl reference: the CPU implementation of the path (the same oracle port, all
host threads) at its own operating point, on a bounded sample of the queries
each step. Its index and ground truth are prepared by a separate process
(bench.py --prepare-only, the GPU builder) into a file cache; the timed process
only loads the files into the oracle.
"""
import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "QPS at recall@10=0.95, learned+BF16 vs plain GPU path, 1 GB300; p50/p99 ms"
TARGET_RECALL = 0.95

# Workloads. exact_sweep / scan_sweep: search_coarse_count values of the plain
# path's exact and scan modes (the precision form reuses scan_sweep); cpu_sweep:
# values tried for the CPU port's operating point.
WORKLOADS = {
    # the learned-probe configuration: 100M x 96 cosine, 4000 x 4000 clusters, probe MLP
    "learned_100m": dict(n=100_000_000, d=96, ncomp=16384, kind="unit", C=4000, F=4000, nsq=24,
                         T=1100, k=10, exact_sweep=(1, 8, 64), scan_sweep=(1, 2), nq=10000,
                         norm=True, train_sample=1_000_000, iters=10, pq_sample=262_144,
                         probe_train=200_000, probe_mass=(0.5, 0.9), probe_max=8,
                         probe_fallback=200, probe_epochs=8, top100=True,
                         cpu_sweep=(1, 2, 4, 8, 16, 32, 64)),
    # the plain GPU path, cosine: 10M x 96, 2000 x 2000 clusters
    "cosine_10m": dict(n=10_000_000, d=96, ncomp=4096, kind="unit", C=2000, F=2000, nsq=24,
                       T=500, k=10, exact_sweep=(50, 100, 200), scan_sweep=(1, 2, 4), nq=10000,
                       norm=True, train_sample=500_000, iters=12, pq_sample=262_144,
                       probe_train=200_000, probe_mass=(0.5, 0.9), probe_max=8,
                       probe_fallback=200, probe_epochs=8, top100=True,
                       cpu_sweep=(1, 2, 4, 8, 16, 50, 100, 200)),
    # the precision form's configuration: 10M x 128 from the integer mixture below, 2000 x 2000
    # clusters (filter PQ 32 x 256 keeps 4 dims per subspace)
    "precision_10m_d128": dict(n=10_000_000, d=128, ncomp=1024, kind="int", C=2000, F=2000,
                               nsq=32, T=500, k=10, exact_sweep=(50,), scan_sweep=(1, 2, 4, 8),
                               nq=10000, norm=False, train_sample=500_000, iters=12,
                               pq_sample=262_144, probe_train=200_000, probe_mass=(0.5, 0.9),
                               probe_max=8, probe_fallback=200, probe_epochs=8, top100=False,
                               cpu_sweep=(1, 2, 4, 8, 16, 50)),
    # plain Puck, L2: 1M x 128 integer mixture, 1000 x 1000 clusters (the reference CPU build's case)
    "l2int_1m": dict(n=1_000_000, d=128, ncomp=1024, kind="int", C=1000, F=1000, nsq=32, T=200,
                     k=10, exact_sweep=(200,), scan_sweep=(1, 2, 4, 8, 200), nq=10000,
                     norm=False, train_sample=262_144, iters=12, pq_sample=131_072,
                     probe_train=100_000, probe_mass=(0.5, 0.9), probe_max=8,
                     probe_fallback=200, probe_epochs=8, top100=False,
                     cpu_sweep=(1, 2, 4, 8, 16, 32, 200)),
    # profiling case for ncu with the per-query work of learned_100m (about 25k records
    # per coarse cluster, 4000 fine clusters, filter_topk 1100): 10M points, ~6 GB on
    # the device
    "scan25k_10m": dict(n=10_000_000, d=96, ncomp=1638, kind="unit", C=400, F=4000, nsq=24,
                        T=1100, k=10, exact_sweep=(1,), scan_sweep=(1,), nq=10000, norm=True,
                        train_sample=400_000, iters=8, pq_sample=131_072,
                        probe_train=50_000, probe_mass=(0.9,), probe_max=8, probe_fallback=200,
                        probe_epochs=4, top100=False, cpu_sweep=(1,)),
    # smaller profiling case with the same per-query scan (25k records per coarse cluster,
    # 4000 fine clusters, filter_topk 1100): 5M points, interleaved records (150 MB) larger
    # than L2, ~3 GB on the device
    "scan25k_5m": dict(n=5_000_000, d=96, ncomp=819, kind="unit", C=200, F=4000, nsq=24,
                       T=1100, k=10, exact_sweep=(1,), scan_sweep=(1,), nq=10000, norm=True,
                       train_sample=400_000, iters=8, pq_sample=131_072,
                       probe_train=50_000, probe_mass=(0.9,), probe_max=8, probe_fallback=200,
                       probe_epochs=4, top100=False, cpu_sweep=(1,)),
    # profiling case for ncu: codes + offsets (150 MB) larger than L2, ~5 GB on the device
    "cosine_5m": dict(n=5_000_000, d=96, ncomp=4096, kind="unit", C=1414, F=1414, nsq=24,
                      T=500, k=10, exact_sweep=(50,), scan_sweep=(1,), nq=10000, norm=True,
                      train_sample=300_000, iters=10, pq_sample=131_072,
                      probe_train=100_000, probe_mass=(0.9,), probe_max=8, probe_fallback=200,
                      probe_epochs=8, top100=False, cpu_sweep=(1, 2, 4)),
    # reduced workload for quick checks only (never the reported line)
    "cosine_1m": dict(n=1_000_000, d=96, ncomp=4096, kind="unit", C=500, F=500, nsq=24,
                      T=500, k=10, exact_sweep=(25, 50), scan_sweep=(1, 2), nq=10000,
                      norm=True, train_sample=200_000, iters=10, pq_sample=131_072,
                      probe_train=100_000, probe_mass=(0.5, 0.9), probe_max=8,
                      probe_fallback=200, probe_epochs=8, top100=True,
                      cpu_sweep=(1, 2, 4, 8, 25)),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ helpers

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value, ws, device=None):
    """The largest of one float over all ranks (the slowest rank's time); ws == 1: itself."""
    if ws <= 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_qps(total_ms, ws, nq, steps):
    """Whole-job queries/s: every rank searched nq queries per step (weak scaling),
    over the slowest rank's time."""
    return ws * nq * steps / (total_ms / 1e3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def brute_force_gt(base, queries, cand=64, chunk=1 << 20):
    """Exact nearest neighbours by squared L2: FP32 candidate pass, FP64 rescoring.

    Returns ids [nq, cand] and FP64 distances [nq, cand] sorted ascending."""
    import torch
    nq = queries.shape[0]
    qn = (queries * queries).sum(1, keepdim=True)
    best_d = torch.full((nq, cand), float("inf"), device=base.device)
    best_i = torch.zeros((nq, cand), dtype=torch.int64, device=base.device)
    for s in range(0, base.shape[0], chunk):
        xb = base[s:s + chunk]
        d = qn - 2.0 * queries @ xb.T + (xb * xb).sum(1)[None, :]
        vals, idx = torch.topk(d, min(cand, d.shape[1]), dim=1, largest=False)
        allv = torch.cat([best_d, vals], 1)
        alli = torch.cat([best_i, idx + s], 1)
        o = torch.topk(allv, cand, dim=1, largest=False)
        best_d, best_i = o.values, alli.gather(1, o.indices)
    rows = base[best_i.reshape(-1)].reshape(nq, cand, -1).double()
    exact = ((rows - queries.double()[:, None, :]) ** 2).sum(-1)
    order = torch.argsort(exact, dim=1, stable=True)
    return best_i.gather(1, order).cpu().numpy(), exact.gather(1, order).cpu().numpy()


def recall_rows(gt_ids, gt_dist, run_ids, count=10, tie_eps=1e-6):
    """Per-query tie-aware recall@count as ann-benchmarks computes it
    (ann-benchmarks/benchmark/plotting/metrics.py:15-40): ground-truth ids within
    1e-6 of the count-th distance all count as hits."""
    out = np.zeros(run_ids.shape[0])
    for i in range(run_ids.shape[0]):
        anchor = gt_dist[i, count - 1]
        end = count
        while end < gt_dist.shape[1] and abs(gt_dist[i, end] - anchor) < tie_eps:
            end += 1
        out[i] = len(set(gt_ids[i, :end].tolist()) & set(run_ids[i, :count].tolist())) / count
    return out


def recall_at(gt_ids, gt_dist, run_ids, count=10):
    return float(recall_rows(gt_ids, gt_dist, run_ids, count).mean())


# ------------------------------------------------------------------ data + index

def workload_queries(w, device):
    from puck_gb300 import builder
    return builder.gmm(w["nq"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=2, device=device)


def make_workload(w, device):
    """Seeded data and the index built on the GPU (host arrays in the reference's
    file layout), the queries, and the ground truth of the queries."""
    import torch
    from puck_gb300 import builder
    t0 = time.time()
    base = builder.gmm(w["n"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=1, device=device)
    queries = workload_queries(w, device)
    log(f"[bench] data {w['n']}x{w['d']} + {w['nq']} queries in {time.time() - t0:.1f}s")
    t0 = time.time()
    arrays = builder.build_index(base, w["C"], w["F"], w["nsq"], w["norm"],
                                 train_sample=w["train_sample"], iters=w["iters"],
                                 pq_sample=w["pq_sample"], seed=0,
                                 whether_pq=bool(w.get("whether_pq", False)))
    torch.cuda.synchronize()
    log(f"[bench] index built in {time.time() - t0:.1f}s")
    t0 = time.time()
    qn = queries / queries.norm(dim=1, keepdim=True) if w["norm"] else queries
    gt_ids, gt_dist = brute_force_gt(base, qn)
    log(f"[bench] ground truth in {time.time() - t0:.1f}s")
    return base, queries, arrays, gt_ids, gt_dist


CACHE_KEYS = ("coarse", "fine", "base", "cell_assign", "filter_codebook", "filter_offsets",
              "filter_codes", "pq_codebook", "pq_offsets", "pq_codes", "queries", "gt_ids",
              "gt_dist")


def cache_dir(workload, w):
    """File cache of one workload's index, queries and ground truth (keyed by the
    workload's parameters and the builder's source)."""
    h = hashlib.sha256(json.dumps(w, sort_keys=True).encode())
    for f in ("puck_gb300/builder.py",):
        with open(os.path.join(REPO, f), "rb") as fh:
            h.update(fh.read())
    root = os.environ.get("PUCK_BENCH_CACHE") or os.path.join(tempfile.gettempdir(),
                                                              "puck_bench_cache")
    return os.path.join(root, f"{workload}-{h.hexdigest()[:16]}")


def write_cache(path, arrays, queries, gt_ids, gt_dist):
    tmp = path + ".partial"
    shutil.rmtree(tmp, ignore_errors=True)
    os.makedirs(tmp)
    full = dict(arrays, queries=queries, gt_ids=gt_ids, gt_dist=gt_dist)
    for k in CACHE_KEYS:
        if full.get(k) is not None:
            np.save(os.path.join(tmp, k + ".npy"), np.ascontiguousarray(full[k]))
    with open(os.path.join(tmp, "meta.json"), "w") as f:
        json.dump({"whether_norm": bool(arrays.get("whether_norm", False))}, f)
    shutil.rmtree(path, ignore_errors=True)
    os.replace(tmp, path)


def read_cache(path):
    if not os.path.exists(os.path.join(path, "meta.json")):
        return None
    out = {}
    for k in CACHE_KEYS:
        f = os.path.join(path, k + ".npy")
        if os.path.exists(f):
            out[k] = np.load(f, mmap_mode="r")
    with open(os.path.join(path, "meta.json")) as f:
        out.update(json.load(f))
    return out


def workload_config(name, w):
    """The workload definition (identical in both arms' lines)."""
    return {"workload": name, "n": w["n"], "d": w["d"], "mixture": f"{w['ncomp']} comps, "
            + ("centres N(0,1), sigma 0.3, L2-normalised" if w["kind"] == "unit"
               else "centres U[0,128), sigma 12, clipped to [0,255], rounded"),
            "queries": w["nq"], "coarse": w["C"], "fine": w["F"], "filter_nsq": w["nsq"],
            "filter_topk": w["T"], "top_k": w["k"], "recall_target": TARGET_RECALL,
            "whether_pq": bool(w.get("whether_pq", False))}


# ------------------------------------------------------------------ CPU leg

def cpu_operating_point(orc, q_np, gt_ids, gt_dist, w, sample=500, threads=None):
    """The oracle port's own operating point: the smallest search_coarse_count of
    w['cpu_sweep'] whose recall@k on the first `sample` queries reaches the target,
    else the most accurate one. Returns (P, reached, sweep)."""
    threads = threads or os.cpu_count() or 1
    m = min(sample, q_np.shape[0])
    sweep = []
    for P in w["cpu_sweep"]:
        if P > w["C"]:
            continue
        t0 = time.perf_counter()
        _, ids, _ = orc.search_batch(q_np[:m], w["k"], P, w["T"], topk_max=100, nthreads=threads)
        el = time.perf_counter() - t0
        rec = recall_at(gt_ids[:m], gt_dist[:m], ids, w["k"])
        sweep.append(dict(search_coarse_count=P, recall_at_10=round(rec, 5),
                          qps=round(m / el, 1), queries=m))
        log(f"[bench] CPU port P={P}: recall@10={rec:.4f} {m / el:.0f} QPS ({threads} threads)")
        if rec >= TARGET_RECALL:
            return P, True, sweep
    best = max(sweep, key=lambda e: e["recall_at_10"])
    return best["search_coarse_count"], False, sweep


def cpu_time(orc, q_np, w, P, budget_s=20.0, max_q=None, threads=None):
    """Queries/s of the oracle port at P on all host threads, over a bounded sample."""
    threads = threads or os.cpu_count() or 1
    cal = min(64, q_np.shape[0])
    t0 = time.perf_counter()
    orc.search_batch(q_np[:cal], w["k"], P, w["T"], topk_max=100, nthreads=threads)
    per_q = (time.perf_counter() - t0) / cal
    nsamp = int(min(max_q or q_np.shape[0], q_np.shape[0], max(cal, budget_s / max(per_q, 1e-6))))
    t0 = time.perf_counter()
    orc.search_batch(q_np[:nsamp], w["k"], P, w["T"], topk_max=100, nthreads=threads)
    el = time.perf_counter() - t0
    return nsamp / el, nsamp, threads


# ------------------------------------------------------------------ GPU arm

def run_serving(native, ix, q_np, loads_qps, seconds=2.0, max_batch=1024, seed=3):
    """Serving form: Poisson request arrivals at several offered loads (queries/s),
    request sizes uniform in 1..256, top-k uniform in {10, 100}; continuous batching
    on CUDA graphs (pgpu_server). Latency is measured by the server from submit to
    results delivered."""
    import threading
    rng = np.random.default_rng(seed)
    srv = native.Server(ix, max_batch=max_batch, scratch_budget_bytes=2 << 30, max_slots=4)
    nq = q_np.shape[0]

    def one_rate(load, secs, record):
        lam = load / 128.5  # mean request size of U{1..256}
        n_req = max(1, int(lam * secs))
        gaps = rng.exponential(1.0 / lam, n_req)
        sizes = rng.integers(1, 257, n_req)
        ks = rng.choice([10, 100], n_req)
        starts = rng.integers(0, nq - 256, n_req)
        tickets = []
        done = []
        lock = threading.Lock()
        finished = threading.Event()

        def waiter():
            i = 0
            while True:
                with lock:
                    if i >= len(tickets):
                        if finished.is_set() and i >= n_req:
                            return
                        t = None
                    else:
                        t = tickets[i]
                if t is None:
                    time.sleep(0.0002)
                    continue
                _, _, _, us = srv.wait(t, timeout_ms=60000)
                done.append(us)
                i += 1

        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        nxt = t0
        for i in range(n_req):
            nxt += gaps[i]
            while time.perf_counter() < nxt:
                pass
            t = srv.submit(q_np[starts[i]:starts[i] + sizes[i]], int(ks[i]))
            with lock:
                tickets.append(t)
        finished.set()
        th.join()
        wall = time.perf_counter() - t0
        if not record:
            return None
        lat = np.array(done) / 1e3
        return dict(offered_qps=round(load), achieved_qps=round(float(sizes.sum()) / wall, 1),
                    requests=n_req, p50_ms=round(float(np.percentile(lat, 50)), 3),
                    p99_ms=round(float(np.percentile(lat, 99)), 3))

    one_rate(loads_qps[0], 0.5, False)  # warm-up: captures the slots' graphs
    rates = [one_rate(load, seconds, True) for load in loads_qps]
    st = srv.stats()
    srv.close()
    return dict(max_batch=max_batch, slots=st["slots"], graphs_captured=st["graphs_captured"],
                mean_batch_queries=round(st["queries_done"] / max(1, st["batches"]), 1),
                request_sizes="uniform 1..256", topk="uniform {10, 100}", arrivals="Poisson",
                rates=rates)


def precision_errors(native, ix, arrays, q_dev, w, plain_ids, bf16_ids, m=512):
    """Per-stage distance error of the precision form against FP64 on the first m
    queries: the BF16 tensor-core contractions (coarse and fine, the same kernel the
    search launches), the FP16-table filter distances of the candidates the scan
    hands to the rerank (pgpu_filter_candidates), the BF16 rerank screen (its
    arithmetic restated on the GPU from BF16-rounded rows), and the returned FP32
    distances; plus the recall of the form's top-k against the plain FP32 path's."""
    import torch
    dev = q_dev.device
    q = q_dev[:m].double()
    if w["norm"]:
        q = q / q.norm(dim=1, keepdim=True)
    qf = q.float().contiguous()
    out = {}
    for name in ("coarse", "fine"):
        cen = torch.from_numpy(np.ascontiguousarray(arrays[name])).to(dev)
        got = torch.empty((m, cen.shape[0]), dtype=torch.float32, device=dev)
        native.contract_bf16("neg", qf, cen, got)  # -q.c on the tensor cores
        torch.cuda.synchronize()
        exact = -(q @ cen.double().T)
        scale = q.norm(dim=1, keepdim=True) * cen.double().norm(dim=1)[None, :]
        rel = ((got.double() - exact).abs() / scale.clamp(min=1e-30))
        out[f"{name}_contraction"] = dict(max_rel=float(rel.max()), mean_rel=float(rel.mean()),
                                          normalised_by="|q||c|")
    # filter distances of the scan's candidates (FP16 table, FP32 accumulation)
    labels, fdist, cnt = ix.filter_candidates(q_dev[:m].cpu().numpy())
    coarse = arrays["coarse"].astype(np.float64)
    fine = arrays["fine"].astype(np.float64)
    cb = arrays["filter_codebook"].astype(np.float64)  # nsq, 256, lsq
    cell = np.asarray(arrays["cell_assign"])
    codes = np.asarray(arrays["filter_codes"])
    offs = np.asarray(arrays["filter_offsets"])
    qh = q.cpu().numpy()
    abs_err, rel_err = [], []
    nsq, lsq = cb.shape[0], cb.shape[2]
    for i in range(m):
        c = int(cnt[i])
        if c == 0:
            continue
        lab = labels[i, :c].astype(np.int64)
        cl = cell[lab].astype(np.int64)
        cc, ff = cl // w["F"], cl % w["F"]
        cf = coarse[cc] + fine[ff]
        two_cd = ((qh[i] - cf) ** 2).sum(1) - (qh[i] ** 2).sum()
        sub = qh[i].reshape(nsq, lsq)
        cw = cb[np.arange(nsq)[None, :], codes[lab].astype(np.int64)]  # c, nsq, lsq
        look = ((sub[None] - cw) ** 2).sum((1, 2))
        t64 = two_cd + offs[lab].astype(np.float64) + look
        e = np.abs(fdist[i, :c].astype(np.float64) - t64)
        abs_err.append(e)
        rel_err.append(e / np.maximum(np.abs(t64), 1e-12))
    ae, re = np.concatenate(abs_err), np.concatenate(rel_err)
    out["filter_distance_fp16_table"] = dict(max_abs=float(ae.max()), mean_abs=float(ae.mean()),
                                             max_rel=float(re.max()), mean_rel=float(re.mean()),
                                             candidates=int(ae.size))
    # the rerank screen's arithmetic: BF16 rows, FP32 query, FP32 sums
    base = arrays["base"]
    lab = bf16_ids[:m].astype(np.int64)
    ok = lab != 0xFFFFFFFF
    rows = torch.from_numpy(np.asarray(base[np.where(ok, lab, 0).reshape(-1)])).to(dev)
    rows = rows.reshape(m, -1, w["d"])
    scr = ((rows.bfloat16().float() - qf[:, None, :]) ** 2).sum(-1).double()
    ex = ((rows.double() - q[:, None, :]) ** 2).sum(-1)
    okt = torch.from_numpy(ok).to(dev)
    e = (scr - ex).abs()[okt]
    out["rerank_screen_bf16"] = dict(max_abs=float(e.max()), mean_abs=float(e.mean()),
                                     max_rel=float((e / ex[okt].clamp(min=1e-12)).max()),
                                     how="restated from BF16-rounded rows of the returned ids")
    # returned distances: exact FP32 order against FP64
    dist, ids = ix.search(q_dev[:m].cpu().numpy(), w["k"])
    lab = ids.astype(np.int64)
    ok = lab != 0xFFFFFFFF
    rows = torch.from_numpy(np.asarray(base[np.where(ok, lab, 0).reshape(-1)])).to(dev)
    ex = ((rows.reshape(m, -1, w["d"]).double() - q[:, None, :]) ** 2).sum(-1).cpu().numpy()
    e = np.abs(dist.astype(np.float64) - ex)[ok]
    out["returned_fp32"] = dict(max_abs=float(e.max()),
                                max_rel=float((e / np.maximum(ex[ok], 1e-12)).max()))
    agree = np.mean([len(set(a.tolist()) & set(b.tolist())) / w["k"]
                     for a, b in zip(plain_ids, bf16_ids)])
    out["recall_vs_plain_fp32"] = round(float(agree), 5)
    return out


def run_profile(args, w):
    """One form at one setting, a few passes, nothing else: the command that ncu
    captures (bench.py --profile FORM:X --workload W)."""
    import torch
    from puck_gb300 import native
    native.load(build_if_missing=True)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    form, x = args.profile.split(":")
    base, queries, arrays, _, _ = make_workload(w, dev)
    del base
    torch.cuda.empty_cache()
    mode = native.PGPU_MODE_EXACT if form == "exact" else native.PGPU_MODE_SCAN
    prec = native.PGPU_PRECISION_BF16 if form == "bf16" else native.PGPU_PRECISION_FP32
    ix = native.GpuIndex(arrays=arrays, search_coarse_count=int(x), filter_topk=w["T"], topk=100,
                         max_batch=w["nq"], device=0, mode=mode, precision=prec,
                         filter_margin=max(1, w["T"] // 10) if form == "bf16" else 0)
    q = queries.contiguous()
    d = torch.empty((w["nq"], w["k"]), dtype=torch.float32, device=dev)
    i = torch.empty((w["nq"], w["k"]), dtype=torch.int32, device=dev)
    for _ in range(args.steps):
        ix.search_device(w["nq"], q, w["k"], d, i)
    torch.cuda.synchronize()
    # one more pass with the library's per-stage events
    ix.set_profiling(True)
    ix.search_device(w["nq"], q, w["k"], d, i)
    stages = ix.stage_times()
    ix.set_profiling(False)
    ix.search(queries.cpu().numpy(), w["k"])
    log(f"[bench] stage ms: {json.dumps({k: round(v, 4) for k, v in stages.items()})}")
    log(f"[bench] counters: {json.dumps(ix.walk_counters())}")
    ix.close()
    log(f"[bench] profile {form}:{x} on {args.workload}: {args.steps} passes")


def run_gpu(args, w, rank, ws):
    import torch
    from puck_gb300 import native, builder, probe as probe_mod
    native.load(build_if_missing=True)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    nq, k = w["nq"], w["k"]
    cpath = cache_dir(args.workload, w)
    cached = read_cache(cpath) if not args.no_cache else None
    if cached is not None:
        t0 = time.time()
        arrays = {kk: np.asarray(v) if isinstance(v, np.ndarray) else v for kk, v in cached.items()}
        base = builder.gmm(w["n"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=1, device=dev)
        queries = torch.from_numpy(np.ascontiguousarray(arrays["queries"])).to(dev)
        gt_ids, gt_dist = arrays["gt_ids"], arrays["gt_dist"]
        log(f"[bench] index, queries and ground truth from {cpath} in {time.time() - t0:.1f}s")
    else:
        base, queries, arrays, gt_ids, gt_dist = make_workload(w, dev)
    # ---- learned probe: fresh training queries of the same mixture, labelled with the
    # coarse clusters of their brute-force top-10, trained on the GPU
    t0 = time.time()
    qtr = builder.gmm(w["probe_train"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=3,
                      device=dev)
    if w["norm"]:
        qtr = qtr / qtr.norm(dim=1, keepdim=True)
    cell = torch.from_numpy(np.asarray(arrays["cell_assign"]).astype(np.int64)).to(dev)
    ltr, _, _ = probe_mod.knn_cluster_labels(base, qtr, cell, w["F"])
    torch.cuda.synchronize()
    label_s = time.time() - t0
    t0 = time.time()
    probe, probe_losses = probe_mod.train_probe(qtr, ltr, w["C"], hidden=512,
                                                epochs=w["probe_epochs"], batch=2048, lr=2e-3,
                                                seed=0, log=None)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    log(f"[bench] probe: {w['probe_train']} training queries labelled in {label_s:.1f}s, "
        f"trained in {train_s:.1f}s, loss {probe_losses[0]:.3f} -> {probe_losses[-1]:.3f}")
    del qtr, ltr, cell, base
    torch.cuda.empty_cache()
    t0 = time.time()
    ix = native.GpuIndex(arrays=arrays, search_coarse_count=w["exact_sweep"][0], filter_topk=w["T"],
                         topk=100, max_batch=nq, device=dev.index)
    ix_bytes = ix.info.device_bytes
    log(f"[bench] index resident ({ix_bytes / 1e9:.2f} GB) in {time.time() - t0:.1f}s")
    q_dev = queries.contiguous()
    kmax = 100 if w.get("top100") else k
    d_dev = torch.empty((nq, kmax), dtype=torch.float32, device=dev)
    i_dev = torch.empty((nq, kmax), dtype=torch.int32, device=dev)
    s_dev = torch.empty(nq, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    topk_now = [k]

    def step():
        ix.search_device(nq, q_dev, topk_now[0], d_dev, i_dev, s_dev, stream=stream)

    bf16_margin = max(1, w["T"] // 10)
    fallback_P = w["probe_fallback"]
    mode_name = {native.PGPU_MODE_EXACT: "exact", native.PGPU_MODE_SCAN: "scan"}

    def set_form(form, mode, x):
        ix.set_probe(None)
        prec = native.PGPU_PRECISION_FP32 if form == "plain" else native.PGPU_PRECISION_BF16
        P = fallback_P if form == "learned+bf16" else x
        ix.set_search_params(search_coarse_count=P, mode=mode, precision=prec,
                             filter_margin=0 if form == "plain" else bf16_margin)
        if form == "learned+bf16":
            ix.set_probe(probe, mass=x, max_probe=w["probe_max"])

    def ids_now(kk):
        # a search of top-kk writes nq x kk contiguous values
        return i_dev.view(-1)[:nq * kk].view(nq, kk).cpu().numpy().view(np.uint32)

    def measure(form, mode, x, kk):
        topk_now[0] = kk
        set_form(form, mode, x)
        step()
        torch.cuda.synchronize()
        ids = ids_now(kk).copy()
        rec = recall_at(gt_ids, gt_dist, ids, k)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(3):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / 3
        entry = dict(form=form, mode=mode_name[mode], top_k=kk, recall_at_10=round(rec, 5),
                     qps=round(nq / (ms / 1e3), 1), ms=round(ms, 3))
        if form == "learned+bf16":
            ix.search(queries.cpu().numpy(), kk)  # host path: per-call probe counters
            wc = ix.walk_counters()
            entry.update(probe_mass=x, search_coarse_count=fallback_P, probe_max=w["probe_max"],
                         mean_clusters=round((wc["probe_clusters"] +
                                              fallback_P * wc["probe_fallbacks"]) / nq, 3),
                         fallback_queries=int(wc["probe_fallbacks"]))
        else:
            entry.update(search_coarse_count=x, mean_clusters=float(x))
        log(f"[bench] {form} {mode_name[mode]} {x} top-{kk}: recall@10={rec:.4f} "
            f"{nq / (ms / 1e3):.0f} QPS")
        return entry, ids

    configs = [("plain", native.PGPU_MODE_EXACT, P) for P in w["exact_sweep"]] + \
              [("plain", native.PGPU_MODE_SCAN, P) for P in w["scan_sweep"]] + \
              [("bf16", native.PGPU_MODE_SCAN, P) for P in w["scan_sweep"]] + \
              [("learned+bf16", native.PGPU_MODE_SCAN, m) for m in w["probe_mass"]]
    sweep, ids_of = [], {}
    for form, mode, x in configs:
        e, ids = measure(form, mode, x, k)
        sweep.append(e)
        ids_of[(form, mode_name[mode], x)] = ids

    def best_of(form, mode=None, kk=None):
        cand = [c for c in sweep if c["form"] == form and (mode is None or c["mode"] == mode)
                and (kk is None or c["top_k"] == kk)]
        ok = [c for c in cand if c["recall_at_10"] >= TARGET_RECALL]
        if ok:
            return max(ok, key=lambda c: c["qps"]), True
        return max(cand, key=lambda c: c["recall_at_10"]), False

    plain_best, plain_reached = best_of("plain", kk=k)
    bf16_best, bf16_reached = best_of("bf16", kk=k)
    best, reached = best_of("learned+bf16", kk=k)
    exact_best, exact_reached = best_of("plain", mode="exact", kk=k)
    # top-100 at the same operating points (recall@10 of the first 10)
    if w.get("top100"):
        for entry in (plain_best, best):
            mode = native.PGPU_MODE_EXACT if entry["mode"] == "exact" else native.PGPU_MODE_SCAN
            e, _ = measure(entry["form"], mode, entry.get("probe_mass", entry["search_coarse_count"]),
                           100)
            sweep.append(e)
    topk_now[0] = k

    def timed(entry):
        mode = native.PGPU_MODE_EXACT if entry["mode"] == "exact" else native.PGPU_MODE_SCAN
        set_form(entry["form"], mode, entry.get("probe_mass", entry["search_coarse_count"]))
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(dev.index) as clk:
            # the timed region is an NVTX range ("timed") for launch-list captures
            torch.cuda.nvtx.range_push("timed")
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for i in range(args.steps):
                evs[i][0].record(stream)
                step()
                evs[i][1].record(stream)
            end.record(stream)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
        total = start.elapsed_time(end)
        per_step = np.array([a.elapsed_time(b) for a, b in evs])
        total = max_over_ranks(total, ws, dev)
        if ws > 1:
            torch.distributed.barrier()
        return total, per_step, clk.summary()

    # ---- timed regions (device-resident inputs): the plain path, then the headline form
    plain_ms, plain_steps, _ = timed(plain_best)
    plain_value = job_qps(plain_ms, ws, nq, args.steps)
    total_ms, step_ms, clocks = timed(best)
    value = job_qps(total_ms, ws, nq, args.steps)
    step()
    torch.cuda.synchronize()
    launches_per_step = int(ix.last_stats()["kernels"])

    # ---- per-stage device time (CUDA events inside the library, same stream), for
    # the headline form and the plain path's operating point
    def stage_profile(entry):
        mode = native.PGPU_MODE_EXACT if entry["mode"] == "exact" else native.PGPU_MODE_SCAN
        set_form(entry["form"], mode, entry.get("probe_mass", entry["search_coarse_count"]))
        ix.set_profiling(True)
        stage = {s: 0.0 for s in native.STAGES}
        for _ in range(3):
            step()
            st = ix.stage_times()
            for kk in stage:
                stage[kk] += st[kk] / 3
        torch.cuda.synchronize()
        ix.set_profiling(False)
        ix.search(queries.cpu().numpy(), k)  # host API: the filter counters of one pass
        return ({kk: round(v, 4) for kk, v in stage.items()}, ix.last_stats(),
                ix.walk_counters())

    plain_stage, plain_stats, plain_counters = stage_profile(plain_best)
    stage, stats, walk_counters = stage_profile(best)

    def roofline(entry, stage_ms, st, counters):
        R = 4 + w["nsq"]
        recs = st["records_scanned"]
        if entry["mode"] == "exact":
            cells = st["cells_scanned"]
            # records the walk evaluates, stationary + cell bounds of the visited cells,
            # the query's fine order
            byts = recs * R + cells * 12 + nq * w["F"] * 8
            kern = "k_walk_scan"
        else:
            clusters = entry["mean_clusters"] * nq
            # every record of the probed clusters (offset + codes + fine id), the probed
            # clusters' stationary rows, the query's fine terms and the query; the split
            # scan's kernel also writes each record's distance (4 B, not counted here:
            # an intermediate of this design, reported as t_write_bytes)
            byts = recs * (R + 2) + clusters * w["F"] * 4 + nq * w["F"] * 4 + nq * w["d"] * 4
            kern = "k_scan_score"
        # stage 5: the walk, or the scan's record kernel alone
        ms = stage_ms["walk_scan"]
        peak, peak_kind = measured_peaks()
        ach = byts / (ms / 1e3) / 1e9
        traffic = None
        tf = os.path.join(REPO, "profiles", "traffic.json")
        if os.path.exists(tf):
            with open(tf) as f:
                for e in json.load(f).get("entries", []):
                    if (e.get("workload") == args.workload and e.get("kernel") == kern
                            and e.get("form", "plain") == entry["form"]
                            and e.get("filter_topk") == w["T"]):
                        # DRAM bytes per record of a capture, scaled to this launch
                        traffic = int(e["dram_bytes_per_record"] * recs)
        return {"bound": "hbm", "kernel": kern, "achieved": round(ach, 2), "peak": peak,
                "unit": "GB/s", "frac": round(ach / peak, 5), "traffic": traffic,
                "peak_source": peak_kind, "algorithmic_bytes_per_launch": int(byts),
                "kernel_ms": round(ms, 4), "records": int(recs),
                "t_write_bytes": int(recs * 4) if entry["mode"] == "scan" else 0}

    roof = roofline(best, stage, stats, walk_counters)
    plain_roof = roofline(plain_best, plain_stage, plain_stats, plain_counters)

    # ---- e2e through the C ABI with pinned host buffers (headline form)
    set_form(best["form"], native.PGPU_MODE_SCAN if best["mode"] == "scan" else native.PGPU_MODE_EXACT,
             best.get("probe_mass", best["search_coarse_count"]))
    q_host = torch.empty((nq, w["d"]), dtype=torch.float32, pin_memory=True)
    q_host.copy_(queries.cpu())
    d_host = torch.empty((nq, k), dtype=torch.float32, pin_memory=True)
    i_host = torch.empty((nq, k), dtype=torch.int32, pin_memory=True)
    s_host = torch.empty(nq, dtype=torch.int32, pin_memory=True)
    for _ in range(max(1, args.warmup)):
        ix.search_into(nq, q_host, k, d_host, i_host, s_host)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ix.search_into(nq, q_host, k, d_host, i_host, s_host)
    e2e_s = time.perf_counter() - t0
    e2e_value = ws * nq * args.steps / e2e_s
    step()
    torch.cuda.synchronize()
    e2e_ids = i_host.numpy().view(np.uint32)
    assert np.array_equal(e2e_ids, ids_now(k)), "e2e != device results"

    # ---- the precision form: per-stage error against FP64
    prec = None
    if not args.no_precision:
        set_form("bf16", native.PGPU_MODE_SCAN, bf16_best["search_coarse_count"])
        key_plain = ("plain", "scan", bf16_best["search_coarse_count"])
        key_bf16 = ("bf16", "scan", bf16_best["search_coarse_count"])
        if key_plain in ids_of:
            m = 512
            prec = precision_errors(native, ix, arrays, q_dev, w, ids_of[key_plain][:m],
                                    ids_of[key_bf16][:m], m=m)
            prec["search_coarse_count"] = bf16_best["search_coarse_count"]
            log(f"[bench] precision errors: {json.dumps(prec)}")

    serving = None
    if not args.no_serve:
        serving = {}
        for name, entry in (("plain", plain_best), (best["form"], best)):
            set_form(entry["form"],
                     native.PGPU_MODE_EXACT if entry["mode"] == "exact" else native.PGPU_MODE_SCAN,
                     entry.get("probe_mass", entry["search_coarse_count"]))
            # offered loads up to past the loop's saturation (achieved below offered)
            serving[name] = dict(run_serving(native, ix, queries.cpu().numpy(),
                                             loads_qps=(250_000, 500_000, 1_000_000, 2_000_000,
                                                        4_000_000)),
                                 recall_at_10=entry["recall_at_10"])
            log(f"[bench] serving {name}: {serving[name]}")

    # ---- CPU leg: the oracle port's own operating point, its timing, and parity of
    # the GPU path against it at scale
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        q_np = queries.cpu().numpy()
        t0 = time.time()
        orc = oracle.OracleIndex(arrays=arrays)
        log(f"[bench] CPU port index load {time.time() - t0:.1f}s")
        P_cpu, cpu_reached, cpu_sweep = cpu_operating_point(orc, q_np, gt_ids, gt_dist, w)
        qps_cpu, nsamp, threads = cpu_time(orc, q_np, w, P_cpu)
        cpu = dict(value=round(qps_cpu, 1), unit="queries/s", cores=threads, kind="port",
                   search_coarse_count=P_cpu, target_recall_reached=cpu_reached,
                   sample=f"first {nsamp} of the {nq} queries at search_coarse_count={P_cpu} "
                          f"(the port's smallest with recall@10 >= {TARGET_RECALL} on 500 "
                          f"queries, else its most accurate), filter_topk={w['T']}, "
                          f"top-{k}; {threads} threads, oracle C port of PuckIndex::search",
                   sweep=cpu_sweep, search_mode="exact walk (the reference's algorithm)")
        # parity on a sample: the GPU's exact mode against the port, bit for bit; the
        # plain scan path and the headline form against the reference's search
        m = min(args.parity_queries, nq)
        parity = {"queries": m}
        for P in sorted({1, P_cpu}):
            od, oi, ost = orc.search_batch(q_np[:m], k, P, w["T"], topk_max=100,
                                           nthreads=threads)
            set_form("plain", native.PGPU_MODE_EXACT, P)
            gd, gi = ix.search(q_np[:m], k)
            parity[f"exact_P{P}_vs_port"] = dict(
                ids_equal=round(float(np.mean(gi == oi)), 6),
                dist_bits_equal=round(float(np.mean(gd.view(np.uint32) == od.view(np.uint32))), 6),
                all_bit_identical=bool(np.array_equal(gi, oi) and
                                       np.array_equal(gd.view(np.uint32), od.view(np.uint32))))
            ref_rec = recall_rows(gt_ids[:m], gt_dist[:m], oi, k)
            for form, x, label in (("plain", P, "scan"), ("learned+bf16", best.get("probe_mass"),
                                                         "headline")):
                if form == "plain":
                    set_form("plain", native.PGPU_MODE_SCAN, P)
                elif P != 1 or x is None:
                    continue
                else:
                    set_form(form, native.PGPU_MODE_SCAN, x)
                _, si = ix.search(q_np[:m], k)
                agree = np.mean([len(set(a.tolist()) & set(b.tolist())) / k for a, b in zip(si, oi)])
                srec = recall_rows(gt_ids[:m], gt_dist[:m], si, k)
                parity[f"{label}_P{P}_vs_reference_search" if form == "plain" else
                       f"{label}_vs_reference_search_P1"] = dict(
                    top10_id_agreement=round(float(agree), 5),
                    queries_recall_below_reference=int((srec < ref_rec - 1e-12).sum()),
                    queries_recall_above_reference=int((srec > ref_rec + 1e-12).sum()),
                    recall=round(float(srec.mean()), 5),
                    reference_recall=round(float(ref_rec.mean()), 5))
        log(f"[bench] parity: {json.dumps(parity)}")
        orc.close()
    ix.close()
    if cached is not None and not args.keep_cache:
        shutil.rmtree(cpath, ignore_errors=True)

    out = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "queries/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32" if best["form"] == "plain" else "bf16",
        "data": "synthetic (seeded Gaussian mixture, built on the GPU in Puck's index format)",
        "config": dict(workload_config(args.workload, w),
                       l2=f"index ({ix_bytes / 1e9:.2f} GB resident) larger than L2 (129 MB); "
                          f"no flush", parallelism=f"replicas x{ws}"),
        "form": best["form"],
        "path": ("learned probe (adaptive clusters, confidence fallback to search_coarse_count="
                 f"{fallback_P}) on the precision form" if best["form"] == "learned+bf16" else
                 best["form"]),
        "operating_point": best,
        "recall_at_10": best["recall_at_10"],
        "target_recall_reached": reached,
        "p50_ms": round(float(np.percentile(step_ms, 50)), 4),
        "p99_ms": round(float(np.percentile(step_ms, 99)), 4),
        "plain": dict(plain_best, timed_qps=round(plain_value, 1),
                      ms_per_step=round(plain_ms / args.steps, 4),
                      p50_ms=round(float(np.percentile(plain_steps, 50)), 4),
                      p99_ms=round(float(np.percentile(plain_steps, 99)), 4),
                      target_recall_reached=plain_reached, stage_ms=plain_stage,
                      roofline=plain_roof),
        "speedup_vs_plain": round(value / plain_value, 4),
        "bf16_best": dict(bf16_best, target_recall_reached=bf16_reached),
        "exact_mode_best": dict(exact_best, target_recall_reached=exact_reached),
        "probe": dict(hidden=512, layers="d->512->512->C, GELU", train_queries=w["probe_train"],
                      labels="coarse clusters of each query's brute-force top-10",
                      label_seconds=round(label_s, 1), train_seconds=round(train_s, 1),
                      epochs=w["probe_epochs"], batch=2048,
                      loss_first_epoch=round(probe_losses[0], 4),
                      loss_last_epoch=round(probe_losses[-1], 4),
                      fallback_search_coarse_count=fallback_P, max_probe=w["probe_max"]),
        "sweep": sweep,
        "stage_ms": stage,
        "filter_counters": walk_counters,
        "precision_errors": prec,
        "parity": parity,
        "e2e": {"value": round(e2e_value, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * w["d"] * 4,
                "d2h_bytes_per_step": nq * k * 8 + nq * 4},
        "roofline": roof,
        "gpu_launches": launches_per_step * args.steps,
        "serving": serving,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ reference arm

def prepare_only(args, w):
    """Builds the workload's index, queries and ground truth on the GPU and writes
    them to the file cache (a separate process of the reference arm)."""
    import torch
    from puck_gb300 import native
    native.load(build_if_missing=True)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    path = cache_dir(args.workload, w)
    if read_cache(path) is not None:
        return
    base, queries, arrays, gt_ids, gt_dist = make_workload(w, dev)
    del base
    t0 = time.time()
    write_cache(path, arrays, queries.cpu().numpy(), gt_ids, gt_dist)
    log(f"[bench] cache written to {path} in {time.time() - t0:.1f}s")


def run_reference(args, w, rank, ws):
    """The CPU implementation of the path (oracle port), all host threads, at its own
    operating point."""
    if rank != 0:
        return
    path = cache_dir(args.workload, w)
    if read_cache(path) is None:
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--prepare-only",
                            "--workload", args.workload] +
                           (["--filter-topk", str(args.filter_topk)] if args.filter_topk else []),
                           stdout=sys.stderr)
        if r.returncode != 0:
            print(json.dumps({"impl": "reference",
                              "unavailable": "index preparation process failed"}))
            return
    import oracle
    c = read_cache(path)
    t0 = time.time()
    arrays = {kk: np.asarray(v) if isinstance(v, np.ndarray) else v for kk, v in c.items()}
    orc = oracle.OracleIndex(arrays=arrays)
    log(f"[bench] reference: index from {path} loaded into the port in {time.time() - t0:.1f}s")
    q_np = np.ascontiguousarray(arrays["queries"], np.float32)
    threads = os.cpu_count() or 1
    P, reached, sweep = cpu_operating_point(orc, q_np, arrays["gt_ids"], arrays["gt_dist"], w,
                                            threads=threads)
    # one step: a sample of queries sized from a calibration run (~1 s of work)
    cal = min(64, q_np.shape[0])
    t0 = time.perf_counter()
    orc.search_batch(q_np[:cal], w["k"], P, w["T"], topk_max=100, nthreads=threads)
    per_q = (time.perf_counter() - t0) / cal
    per_step = int(max(threads, min(q_np.shape[0] // 2, 1.0 / max(per_q, 1e-6))))
    for i in range(args.warmup):
        orc.search_batch(q_np[:per_step], w["k"], P, w["T"], topk_max=100, nthreads=threads)
    times = []
    for i in range(args.steps):
        s = (i * per_step) % max(1, q_np.shape[0] - per_step)
        t0 = time.perf_counter()
        orc.search_batch(q_np[s:s + per_step], w["k"], P, w["T"], topk_max=100, nthreads=threads)
        times.append(time.perf_counter() - t0)
    orc.close()
    value = per_step * len(times) / sum(times)
    sample = (f"{per_step} queries per step of the {q_np.shape[0]}, search_coarse_count={P} "
              f"(the port's smallest with recall@10 >= {TARGET_RECALL} on 500 queries, else its "
              f"most accurate), filter_topk={w['T']}, top-{w['k']}; oracle C port of "
              f"PuckIndex::search (the reference's own build is x86-only)")
    out = {
        "metric": METRIC, "impl": "reference", "value": round(value, 2), "unit": "queries/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(times) / len(times), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded Gaussian mixture, built on the GPU in Puck's index format "
                "by a separate preparation process)",
        "config": workload_config(args.workload, w),
        "operating_point": dict(search_coarse_count=P, target_recall_reached=reached,
                                sweep=sweep),
        "cpu_baseline": {"value": round(value, 2), "unit": "queries/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 2), "unit": "queries/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="learned_100m", choices=sorted(WORKLOADS))
    ap.add_argument("--pq", action="store_true",
                    help="build the index with the second-level PQ (whether_pq, the "
                         "reference's default): the rerank ranks by PQ, not the vectors")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-cache", action="store_true", help="ignore a prepared file cache")
    ap.add_argument("--keep-cache", action="store_true", help="keep the file cache after use")
    ap.add_argument("--prepare-only", action="store_true",
                    help="build the workload's index and ground truth into the file cache")
    ap.add_argument("--parity-queries", type=int, default=1000)
    ap.add_argument("--profile", default="",
                    help="FORM:X (exact:P, scan:P or bf16:P): only build the workload and run "
                         "--steps passes of that form (the command an ncu capture runs)")
    ap.add_argument("--filter-topk", type=int, default=0,
                    help="override the workload's filter_topk")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup) if args.impl == "gpu" else args.warmup
    ws, rank, local = dist_env()
    w = dict(WORKLOADS[args.workload])
    if args.filter_topk:
        w["T"] = args.filter_topk
    if args.pq:
        w["whether_pq"] = True
    if args.prepare_only:
        prepare_only(args, w)
        return
    if args.profile:
        run_profile(args, w)
        return
    if ws > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    try:
        if args.impl == "reference":
            run_reference(args, w, rank, ws)
        else:
            run_gpu(args, w, rank, ws)
    finally:
        if ws > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
