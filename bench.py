#!/usr/bin/env python
"""Benchmark: Puck-Flat batched search on GB300, QPS at recall@10 = 0.95.

Workload (default "cosine_10m"): 10M base vectors, d=96, float32, drawn from a
4096-component Gaussian mixture (centres N(0,1), per-dim sigma 0.3) and
L2-normalised; 10k normalised queries from the same mixture; coarse = fine =
2000 clusters; filter PQ 24 subspaces x 256 (uint8 codes); filter_topk 500;
top-10. search_coarse_count is swept over {50, 100, 200}; the operating point is
the smallest value whose recall@10 against an FP64 brute-force oracle reaches
0.95. Data are seeded synthetic (no dataset download); the index is built on
the GPU in the reference's formats.

One "step" = one batch search of all 10k queries at the operating point.
  value  : queries/s with queries and outputs resident in HBM (device API)
  e2e    : queries/s through pgpu_search_batch with pinned host buffers
           (host->device query copy and device->host result copy inside)
The index (codes 280 MB, vectors 3.8 GB) is larger than L2, so timed steps run
back to back without an L2 flush.

--impl reference: the CPU implementation of the same path timed on the host
cores (the oracle port of the reference's search, all threads), on a bounded
sample of the same queries each step.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "QPS at recall@10=0.95, learned+BF16 vs plain GPU path, 1 GB300; p50/p99 ms"

WORKLOADS = {
    "cosine_10m": dict(n=10_000_000, d=96, ncomp=4096, kind="unit", C=2000, F=2000, nsq=24,
                       T=500, k=10, sweep=(50, 100, 200), scan_sweep=(1, 2, 3, 4, 8, 16),
                       nq=10000, norm=True, train_sample=500_000, iters=12, pq_sample=262_144,
                       probe_train=200_000, probe_mass=(0.5, 0.8, 0.9, 0.95, 0.99), probe_max=8,
                       probe_fallback=4, probe_epochs=8),
    # profiling case for ncu: codes + offsets (150 MB) larger than L2, ~5 GB on the device
    "cosine_5m": dict(n=5_000_000, d=96, ncomp=4096, kind="unit", C=1414, F=1414, nsq=24,
                      T=500, k=10, sweep=(50,), scan_sweep=(4,), nq=10000, norm=True,
                      train_sample=300_000, iters=10, pq_sample=131_072,
                      probe_train=100_000, probe_mass=(0.9,), probe_max=8, probe_fallback=4, probe_epochs=8),
    # the learned-probe configuration: 100M x 96 normalised, 16384 components, C = F = 4000
    # (run on request: building the index takes minutes)
    "learned_100m": dict(n=100_000_000, d=96, ncomp=16384, kind="unit", C=4000, F=4000, nsq=24,
                         T=500, k=10, sweep=(50,), scan_sweep=(1, 2, 4, 8), nq=10000, norm=True,
                         train_sample=1_000_000, iters=10, pq_sample=262_144,
                         probe_train=200_000, probe_mass=(0.5, 0.8, 0.9, 0.95), probe_max=8,
                         probe_fallback=4, probe_epochs=8),
    # reduced workload for quick checks only (never the reported line)
    "cosine_1m": dict(n=1_000_000, d=96, ncomp=4096, kind="unit", C=500, F=500, nsq=24,
                      T=500, k=10, sweep=(25, 50, 100), scan_sweep=(1, 2, 4, 8), nq=10000,
                      norm=True, train_sample=200_000, iters=10, pq_sample=131_072,
                      probe_train=100_000, probe_mass=(0.5, 0.9, 0.99), probe_max=8,
                      probe_fallback=4, probe_epochs=8),
}
TARGET_RECALL = 0.95


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


def brute_force_gt(base, queries, k, cand=64, chunk=1 << 20):
    """Exact top-k by squared L2: FP32 candidate pass, FP64 rescoring.

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


def recall_at(gt_ids, gt_dist, run_ids, count=10, tie_eps=1e-6):
    """Tie-aware recall@count as ann-benchmarks computes it
    (ann-benchmarks/benchmark/plotting/metrics.py:15-40): ground-truth ids within
    1e-6 of the count-th distance all count as hits."""
    hits = 0
    for i in range(run_ids.shape[0]):
        anchor = gt_dist[i, count - 1]
        end = count
        while end < gt_dist.shape[1] and abs(gt_dist[i, end] - anchor) < tie_eps:
            end += 1
        hits += len(set(gt_ids[i, :end].tolist()) & set(run_ids[i, :count].tolist()))
    return hits / (count * run_ids.shape[0])


def make_workload(w, device):
    import torch
    from puck_gb300 import builder
    t0 = time.time()
    base = builder.gmm(w["n"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=1, device=device)
    queries = builder.gmm(w["nq"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=2,
                          device=device)
    log(f"[bench] data {w['n']}x{w['d']} + {w['nq']} queries in {time.time() - t0:.1f}s")
    t0 = time.time()
    arrays = builder.build_index(base, w["C"], w["F"], w["nsq"], w["norm"],
                                 train_sample=w["train_sample"], iters=w["iters"],
                                 pq_sample=w["pq_sample"], seed=0,
                                 whether_pq=bool(w.get("whether_pq", False)))
    torch.cuda.synchronize()
    log(f"[bench] index built in {time.time() - t0:.1f}s")
    return base, queries, arrays


def cpu_port_baseline(arrays, queries_np, P, T, k, budget_s=20.0, max_q=4000):
    """Oracle port of the reference's search on all host threads, bounded sample."""
    import oracle
    t0 = time.time()
    orc = oracle.OracleIndex(arrays=arrays)
    log(f"[bench] CPU port index load {time.time() - t0:.1f}s")
    threads = os.cpu_count() or 1
    # calibrate on a small sample, then size the measured sample to the budget
    cal = min(64, queries_np.shape[0])
    t0 = time.perf_counter()
    orc.search_batch(queries_np[:cal], k, P, T, topk_max=100, nthreads=threads)
    per_q = (time.perf_counter() - t0) / cal
    nsamp = int(min(max_q, queries_np.shape[0], max(cal, budget_s / max(per_q, 1e-6))))
    t0 = time.perf_counter()
    dist, ids, status = orc.search_batch(queries_np[:nsamp], k, P, T, topk_max=100,
                                         nthreads=threads)
    el = time.perf_counter() - t0
    return orc, dict(value=nsamp / el, unit="queries/s", cores=threads, kind="port",
                     sample=f"first {nsamp} of the {queries_np.shape[0]} queries, "
                            f"search_coarse_count={P}, filter_topk={T}, top-{k}; "
                            f"{threads} threads, oracle C port of PuckIndex::search"), ids


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


# ------------------------------------------------------------------ arms# ------------------------------------------------------------------ arms

def run_gpu(args, w, rank, ws):
    import torch
    from puck_gb300 import native
    native.load(build_if_missing=True)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    base, queries, arrays = make_workload(w, dev)
    nq, k = w["nq"], w["k"]
    qnorm = queries / queries.norm(dim=1, keepdim=True)
    gt_ids, gt_dist = brute_force_gt(base, qnorm, k)
    # ---- learned probe: fresh training queries of the same mixture, labelled with the
    # coarse clusters of their brute-force top-10, trained on the GPU
    from puck_gb300 import builder, probe as probe_mod
    t0 = time.time()
    qtr = builder.gmm(w["probe_train"], w["d"], w["ncomp"], w["kind"], seed=0, row_seed=3,
                      device=dev)
    qtr = qtr / qtr.norm(dim=1, keepdim=True)
    cell = torch.from_numpy(arrays["cell_assign"].astype(np.int64)).to(dev)
    ltr, _, _ = probe_mod.knn_cluster_labels(base, qtr, cell, w["F"])
    torch.cuda.synchronize()
    label_s = time.time() - t0
    t0 = time.time()
    probe, probe_losses = probe_mod.train_probe(qtr, ltr, w["C"], hidden=512,
                                                epochs=w["probe_epochs"], batch=2048, lr=2e-3,
                                                seed=0, log=log)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    log(f"[bench] probe: {w['probe_train']} training queries labelled in {label_s:.1f}s, "
        f"trained in {train_s:.1f}s, loss {probe_losses[0]:.3f} -> {probe_losses[-1]:.3f}")
    del qtr, ltr, cell, base
    torch.cuda.empty_cache()
    t0 = time.time()
    ix = native.GpuIndex(arrays=arrays, search_coarse_count=w["sweep"][0], filter_topk=w["T"],
                         topk=100, max_batch=nq, device=dev.index)
    ix_bytes = ix.info.device_bytes
    log(f"[bench] index resident ({ix_bytes / 1e9:.2f} GB) in {time.time() - t0:.1f}s")
    q_dev = queries.contiguous()
    d_dev = torch.empty((nq, k), dtype=torch.float32, device=dev)
    i_dev = torch.empty((nq, k), dtype=torch.int32, device=dev)
    s_dev = torch.empty(nq, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def step():
        ix.search_device(nq, q_dev, k, d_dev, i_dev, s_dev, stream=stream)

    sweep = []
    bf16_margin = max(1, w["T"] // 10)
    fallback_P = w["probe_fallback"]
    # (form, mode, P or probe mass): the plain FP32 path in both modes, the precision
    # form, and the learned probe on top of the precision form
    configs = [("plain", native.PGPU_MODE_EXACT, P) for P in w["sweep"]] + \
              [("plain", native.PGPU_MODE_SCAN, P) for P in w["scan_sweep"]] + \
              [("bf16", native.PGPU_MODE_SCAN, P) for P in w["scan_sweep"]] + \
              [("learned+bf16", native.PGPU_MODE_SCAN, m) for m in w["probe_mass"]]
    mode_name = {native.PGPU_MODE_EXACT: "exact", native.PGPU_MODE_SCAN: "scan"}

    def set_form(form, mode, x):
        ix.set_probe(None)
        prec = native.PGPU_PRECISION_FP32 if form == "plain" else native.PGPU_PRECISION_BF16
        P = fallback_P if form == "learned+bf16" else x
        ix.set_search_params(search_coarse_count=P, mode=mode, precision=prec,
                             filter_margin=0 if form == "plain" else bf16_margin)
        if form == "learned+bf16":
            ix.set_probe(probe, mass=x, max_probe=w["probe_max"])

    for form, mode, x in configs:
        set_form(form, mode, x)
        step()
        torch.cuda.synchronize()
        ids = i_dev.cpu().numpy().view(np.uint32)
        rec = recall_at(gt_ids, gt_dist, ids, k)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(3):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / 3
        entry = dict(form=form, mode=mode_name[mode], recall_at_10=round(rec, 5),
                     qps=round(nq / (ms / 1e3), 1), ms=round(ms, 3))
        if form == "learned+bf16":
            ix.search(queries.cpu().numpy(), k)  # host path: per-call probe counters
            wc = ix.walk_counters()
            entry.update(probe_mass=x, search_coarse_count=fallback_P,
                         probe_max=w["probe_max"],
                         mean_clusters=round((wc["probe_clusters"] +
                                              fallback_P * wc["probe_fallbacks"]) / nq, 3),
                         fallback_queries=int(wc["probe_fallbacks"]))
        else:
            entry.update(search_coarse_count=x)
        sweep.append(entry)
        log(f"[bench] {form} {mode_name[mode]} {x}: recall@10={rec:.4f} "
            f"{nq / (ms / 1e3):.0f} QPS")

    def best_of(form):
        cand = [c for c in sweep if c["form"] == form]
        ok = [c for c in cand if c["recall_at_10"] >= TARGET_RECALL]
        if ok:
            return max(ok, key=lambda c: c["qps"]), True
        return max(cand, key=lambda c: c["recall_at_10"]), False

    plain_best, plain_reached = best_of("plain")
    bf16_best, _ = best_of("bf16")
    best, reached = best_of("learned+bf16")
    exact_ok = [c for c in sweep if c["form"] == "plain" and c["mode"] == "exact"
                and c["recall_at_10"] >= TARGET_RECALL]
    exact_best = max(exact_ok, key=lambda c: c["qps"]) if exact_ok else None

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
    op_mode = native.PGPU_MODE_EXACT if best["mode"] == "exact" else native.PGPU_MODE_SCAN
    op = best["search_coarse_count"]
    op_recall = best["recall_at_10"]
    step()
    torch.cuda.synchronize()
    launches_per_step = int(ix.last_stats()["kernels"])

    # ---- per-stage device time (CUDA events inside the library, same stream)
    ix.set_profiling(True)
    prof_steps = 3
    stage = {s: 0.0 for s in native.STAGES}
    recs = cells = 0
    for _ in range(prof_steps):
        step()
        st = ix.stage_times()
        for kk in stage:
            stage[kk] += st[kk] / prof_steps
    torch.cuda.synchronize()
    ix.set_profiling(False)
    # records / cells the walk evaluated (host API reports the counters)
    q_np = queries.cpu().numpy()
    ix.search(q_np, k)
    stats = ix.last_stats()
    walk_counters = ix.walk_counters()
    recs, cells = stats["records_scanned"], stats["cells_scanned"]
    R = 4 + w["nsq"]
    if op_mode == native.PGPU_MODE_EXACT:
        # records the walk evaluates (offset + codes), stationary + cell bounds of the
        # cells it visits, the query's fine order
        walk_bytes = recs * R + cells * 12 + nq * w["F"] * 8
        kernel = "k_walk_scan"
    else:
        # every record of the probed clusters (offset + codes + fine id), the probed
        # clusters' stationary rows, the query's fine terms
        walk_bytes = recs * (R + 2) + nq * op * w["F"] * 4 + nq * w["F"] * 4
        kernel = "k_scan_select"
    walk_ms = stage["walk_scan"]
    peak, peak_kind = measured_peaks()
    achieved = walk_bytes / (walk_ms / 1e3) / 1e9
    # DRAM bytes per launch of the dominant kernel, from an ncu capture of the same
    # workload and operating point (profiles/traffic.json), when one exists
    traffic = None
    tf = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            for e in json.load(f).get("entries", []):
                if (e.get("workload") == args.workload and e.get("search_coarse_count") == op
                        and e.get("mode") == best["mode"]
                        and e.get("form", "plain") == best["form"]):
                    traffic = e.get("dram_bytes_per_launch")

    # ---- e2e through the C ABI with pinned host buffers
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
    e2e_ids = i_host.numpy().view(np.uint32)
    assert np.array_equal(e2e_ids, i_dev.cpu().numpy().view(np.uint32)), "e2e != device results"

    serving = None
    if not args.no_serve:
        serving = {}
        for name, entry in (("plain", plain_best), (best["form"], best)):
            set_form(entry["form"],
                     native.PGPU_MODE_EXACT if entry["mode"] == "exact" else native.PGPU_MODE_SCAN,
                     entry.get("probe_mass", entry["search_coarse_count"]))
            serving[name] = dict(run_serving(native, ix, q_np,
                                             loads_qps=(250_000, 500_000, 1_000_000)),
                                 recall_at_10=entry["recall_at_10"])
            log(f"[bench] serving {name}: {serving[name]}")
        set_form(best["form"], op_mode, best.get("probe_mass", op))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_P = exact_best["search_coarse_count"] if exact_best else w["sweep"][0]
        orc, cpu, cpu_ids = cpu_port_baseline(arrays, q_np, cpu_P, w["T"], k)
        cpu["search_mode"] = "exact walk (the reference's algorithm)"
        if op_mode == native.PGPU_MODE_EXACT and cpu_P == op:
            m = cpu_ids.shape[0]
            cpu["matches_gpu_ids"] = bool(np.array_equal(cpu_ids, e2e_ids[:m]))
        orc.close()

    ix.close()
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
        "config": {
            "workload": f"{args.workload}{' + second-level PQ (whether_pq)' if w.get('whether_pq') else ''}: "
                        f"{w['n']} x d{w['d']} L2-normalised GMM "
                        f"({w['ncomp']} comps), {nq} queries, coarse={w['C']} fine={w['F']}, "
                        f"filter PQ {w['nsq']}x256, filter_topk={w['T']}, top-{k}",
            "path": ("learned probe (adaptive clusters, confidence fallback) on the "
                     "precision form" if best["form"] == "learned+bf16" else
                     "precision form: BF16 tensor-core fine terms, FP16 ADC table, "
                     f"filter margin {bf16_margin}, BF16 rerank screen + FP32 window"
                     if best["form"] == "bf16" else
                     "plain GPU path, exact mode (reference-identical results)"
                     if op_mode == native.PGPU_MODE_EXACT else
                     "plain GPU path, scan mode (all records of the probed clusters, "
                     "reference per-record distances, exact rerank)"),
            "form": best["form"],
            "mode": best["mode"],
            "bf16_best": bf16_best,
            "probe": dict(hidden=512, layers="d->512->512->C, GELU", train_queries=w["probe_train"],
                          labels="coarse clusters of each query's brute-force top-10",
                          label_seconds=round(label_s, 1), train_seconds=round(train_s, 1),
                          epochs=w["probe_epochs"], batch=2048, loss_first_epoch=round(probe_losses[0], 4),
                          loss_last_epoch=round(probe_losses[-1], 4),
                          fallback_search_coarse_count=fallback_P, max_probe=w["probe_max"]),
            "plain": dict(plain_best, timed_qps=round(plain_value, 1),
                          ms_per_step=round(plain_ms / args.steps, 4),
                          p50_ms=round(float(np.percentile(plain_steps, 50)), 4),
                          p99_ms=round(float(np.percentile(plain_steps, 99)), 4),
                          target_recall_reached=plain_reached),
            "speedup_vs_plain": round(value / plain_value, 4),
            "search_coarse_count": op,
            "exact_mode_best": exact_best,
            "recall_at_10": op_recall,
            "target_recall_reached": reached,
            "sweep": sweep,
            "p50_ms": round(float(np.percentile(step_ms, 50)), 4),
            "p99_ms": round(float(np.percentile(step_ms, 99)), 4),
            "batch": nq,
            "l2": f"index ({ix_bytes / 1e9:.2f} GB resident) larger than L2 (129 MB); no flush",
            "stage_ms": {kk: round(v, 4) for kk, v in stage.items()},
            "walk_records_scanned": recs,
            "walk_cells_scanned": cells,
            "filter_counters": walk_counters,
            "parallelism": f"replicas x{ws}",
        },
        "e2e": {"value": round(e2e_value, 1), "unit": "queries/s",
                "h2d_bytes_per_step": nq * w["d"] * 4,
                "d2h_bytes_per_step": nq * k * 8 + nq * 4},
        "roofline": {"bound": "hbm", "kernel": kernel,
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": traffic,
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": int(walk_bytes)},
        "gpu_launches": launches_per_step * args.steps,
        "serving": serving,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args, w, rank, ws):
    """The CPU implementation of the path (oracle port), all host threads."""
    if rank != 0:
        return
    import torch
    from puck_gb300 import builder  # noqa: F401  (index preparation only, untimed)
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else None
    if dev is None:
        print(json.dumps({"impl": "reference", "unavailable": "no GPU to prepare the index"}))
        return
    import oracle
    base, queries, arrays = make_workload(w, dev)
    del base
    q_np = queries.cpu().numpy()
    P = args.reference_coarse_count or w["sweep"][1]
    orc = oracle.OracleIndex(arrays=arrays)
    threads = os.cpu_count() or 1
    per_step = args.reference_sample
    for i in range(args.warmup):
        orc.search_batch(q_np[:min(64, per_step)], w["k"], P, w["T"], topk_max=100,
                         nthreads=threads)
    times = []
    for i in range(args.steps):
        s = (i * per_step) % max(1, q_np.shape[0] - per_step)
        t0 = time.perf_counter()
        orc.search_batch(q_np[s:s + per_step], w["k"], P, w["T"], topk_max=100, nthreads=threads)
        times.append(time.perf_counter() - t0)
    value = per_step * len(times) / sum(times)
    sample = (f"{per_step} queries per step of the {q_np.shape[0]}, search_coarse_count={P}, "
              f"filter_topk={w['T']}, top-{w['k']}; oracle C port of PuckIndex::search "
              f"(the reference's own build is x86-only)")
    out = {
        "metric": METRIC, "impl": "reference", "value": round(value, 2), "unit": "queries/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(times) / len(times), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded Gaussian mixture)",
        "config": {"workload": args.workload, "search_coarse_count": P, "filter_topk": w["T"],
                   "top_k": w["k"]},
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
    ap.add_argument("--workload", default="cosine_10m", choices=sorted(WORKLOADS))
    ap.add_argument("--pq", action="store_true",
                    help="build the index with the second-level PQ (whether_pq, the "
                         "reference's default): the rerank ranks by PQ, not the vectors")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--reference-sample", type=int, default=500)
    ap.add_argument("--reference-coarse-count", type=int, default=0)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup) if args.impl == "gpu" else args.warmup
    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    w = dict(WORKLOADS[args.workload])
    if args.pq:
        w["whether_pq"] = True
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
