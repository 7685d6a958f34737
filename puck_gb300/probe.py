"""Learned probe predictor: label generation and training on the GPU.

Labels: for each training query, the coarse clusters holding its exact top-k
neighbours, found by brute force over the indexed vectors (pgpu_knn: BF16
tensor-core screen of every pair, FP32 rescoring). Training: Adam on the
softmax cross-entropy against the distribution of those clusters
(pgpu_probe_train_step: forward and backward GEMMs on the tensor cores).
PyTorch only allocates device memory, shuffles and slices.
"""
import math
import time

import numpy as np

from . import native


def knn_cluster_labels(base, queries, cell_assign, fine_count, k=10):
    """Coarse cluster ids [nq, k] (int32, CUDA) of each query's exact top-k.

    base [n, d] and queries [nq, d] are float32 CUDA tensors (queries already
    normalised when the index normalises); cell_assign is the index's
    coarse * fine_count + fine per point (CUDA int64 or int32 tensor)."""
    import torch
    nq = queries.shape[0]
    ids = torch.empty((nq, k), dtype=torch.int32, device=queries.device)
    dist = torch.empty((nq, k), dtype=torch.float32, device=queries.device)
    torch.cuda.synchronize()
    native.knn(base, queries, k, ids, dist)
    cells = cell_assign[ids.long()]
    return (cells // fine_count).to(torch.int32), ids, dist


def train_probe(queries, labels, clusters, hidden=512, epochs=3, batch=4096, lr=2e-3, seed=0,
                log=None):
    """Trains a Probe on normalised queries [n, d] and cluster labels [n, L]
    (CUDA tensors). Returns (probe, per-epoch mean losses)."""
    import torch
    n, d = queries.shape
    probe = native.Probe(d, hidden, clusters, seed=seed, device=queries.device.index or 0)
    gen = torch.Generator(device=queries.device).manual_seed(seed)
    steps = epochs * max(1, n // batch)
    step = 0
    losses = []
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device=queries.device)
        tot, cnt = 0.0, 0
        for b0 in range(0, n - batch + 1 if n >= batch else 1, batch):
            idx = perm[b0:b0 + batch]
            xb = queries[idx].contiguous()
            yb = labels[idx].contiguous()
            torch.cuda.current_stream().synchronize()
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(1, steps)))
            tot += probe.train_step(xb, yb, rate)
            cnt += 1
            step += 1
        losses.append(tot / max(1, cnt))
        if log:
            log(f"[probe] epoch {ep}: loss {losses[-1]:.4f} ({time.time() - t0:.1f}s)")
    return probe, losses


def cluster_recall(probe, queries, labels, max_probe):
    """Fraction of label entries covered by the probe's max_probe best clusters,
    and the same for a given scores tensor; used to compare with the centroid rule."""
    import torch
    nq = queries.shape[0]
    scores = torch.empty((nq, probe.clusters), dtype=torch.float32, device=queries.device)
    torch.cuda.synchronize()
    probe.forward(queries, scores)
    top = torch.topk(scores, max_probe, dim=1).indices
    hit = (labels.long()[:, :, None] == top[:, None, :]).any(-1)
    return float(hit.float().mean())
