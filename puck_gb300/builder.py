"""GPU index builder producing Puck-Flat indexes in the reference's formats.

Follows the structure of PuckIndex::train / build (puck/puck/puck_index.cpp:602-874,
puck/hierarchical_cluster/hierarchical_cluster_index.cpp:882-1138):

  1. coarse k-means on a sample; fine k-means on the coarse residuals;
     fine centroids re-ordered by descending norm (hierarchical_cluster_index.cpp:958-980)
  2. every point assigned to its nearest cell c*F + f by the reference's own walk
     (pgpu_nearest_cell_assign: the same cells as its build for these centroids); above
     EXACT_ASSIGN_MAX_POINTS points, by the nearest cell within the 8 nearest coarse
     clusters (assign_cells)
  3. filter PQ (filter_nsq subspaces x 256 codewords) trained by k-means on the cell
     residuals x - c - f; every point encoded, with its offset 2 <decoded residual,
     c + f> (quantization.cpp:244-258), by the library's puck_assign kernel
     (pgpu_puck_assign): the records the reference writes for these cells and codebooks

The k-means assignment step is the library's own kernel (pgpu_nearest_center,
kmeans.cpp:221-258). Training is seeded, unlike the reference's time(0) seeds;
the index it writes is an ordinary Puck index the reference loads unchanged.
Torch is used for device memory, the k-means update and the probe assignment of
large builds.
"""
import numpy as np
import torch

from . import native


def _nearest(cents, x):
    assign = torch.empty(x.shape[0], dtype=torch.int32, device=x.device)
    dist = torch.empty(x.shape[0], dtype=torch.float32, device=x.device)
    native.nearest_center(cents.contiguous(), x.contiguous(), assign, dist,
                          stream=torch.cuda.current_stream())
    return assign.long(), dist


def kmeans(x, k, iters=12, seed=0, chunk=1 << 20):
    """Lloyd's k-means on a device tensor; the assignment step runs on pgpu_nearest_center."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    n, d = x.shape
    idx = torch.randperm(n, generator=g)[:k].to(x.device)
    cents = x[idx].clone()
    for _ in range(iters):
        sums = torch.zeros_like(cents)
        counts = torch.zeros(k, dtype=torch.float32, device=x.device)
        for s in range(0, n, chunk):
            xs = x[s:s + chunk]
            a, _ = _nearest(cents, xs)
            sums.index_add_(0, a, xs)
            counts.index_add_(0, a, torch.ones_like(a, dtype=torch.float32))
        empty = counts == 0
        cents = torch.where(empty[:, None], cents, sums / counts.clamp(min=1)[:, None])
        if empty.any():  # re-seed empty clusters from random points
            ne = int(empty.sum())
            pick = torch.randint(0, n, (ne,), generator=g).to(x.device)
            cents[empty] = x[pick]
    return cents


def _pq_train(res, nsq, iters=10, seed=0):
    n, d = res.shape
    lsq = d // nsq
    sub = res.view(n, nsq, lsq)
    books = []
    for m in range(nsq):
        books.append(kmeans(sub[:, m, :].contiguous(), 256, iters=iters, seed=seed + 101 * m))
    return torch.stack(books)  # [nsq, 256, lsq]


def _pq_encode(res, books):
    n = res.shape[0]
    nsq, _, lsq = books.shape
    sub = res.view(n, nsq, lsq)
    codes = torch.empty(n, nsq, dtype=torch.uint8, device=res.device)
    for m in range(nsq):
        a, _ = _nearest(books[m], sub[:, m, :].contiguous())
        codes[:, m] = a.to(torch.uint8)
    return codes


# Largest point count the builder assigns with the reference's exact walk. Above it
# the walk's cost (every near coarse cluster walked per point, exact FP32 dots of
# every point with every centroid) runs to hours at 100M points, and the builder
# takes the probe assignment below.
EXACT_ASSIGN_MAX_POINTS = 4_000_000


def assign_cells(x, coarse, fine, exact=None, probe=8, chunk=32768):
    """Nearest cell c * F + f of every row of x (int64).

    exact (default: n <= EXACT_ASSIGN_MAX_POINTS): the reference's own walk
    (pgpu_nearest_cell_assign, hierarchical_cluster_index.cpp:1042-1138), the cells
    its build writes for these centroids. Otherwise the smallest 0.5|x - c - f|^2
    over the `probe` coarse clusters nearest to x (all fine ids of each): the cell
    the walk finds whenever it lies in those clusters, at a fraction of the cost."""
    n = x.shape[0]
    if exact is None:
        exact = n <= EXACT_ASSIGN_MAX_POINTS
    if exact:
        cell = torch.empty(n, dtype=torch.int32, device=x.device)
        dist = torch.empty(n, dtype=torch.float32, device=x.device)
        native.nearest_cell_assign(coarse.contiguous(), fine.contiguous(), x.contiguous(), cell,
                                   dist, stream=torch.cuda.current_stream())
        return cell.long()
    C, F = coarse.shape[0], fine.shape[0]
    cn = (coarse * coarse).sum(1) / 2
    fn = (fine * fine).sum(1) / 2
    stat = fn[None, :] + coarse @ fine.T  # [C, F] stationary terms
    out = torch.empty(n, dtype=torch.int64, device=x.device)
    probe = min(probe, C)
    for s in range(0, n, chunk):
        xs = x[s:s + chunk]
        xn = (xs * xs).sum(1, keepdim=True) / 2
        cterm = cn[None, :] - xs @ coarse.T + xn  # 0.5|x - c|^2
        top = torch.topk(cterm, probe, dim=1, largest=False)
        fterm = xs @ fine.T  # x.f
        score = top.values[:, :, None] - fterm[:, None, :] + stat[top.indices]  # [b, probe, F]
        best = score.view(xs.shape[0], -1).argmin(1)
        out[s:s + chunk] = top.indices.gather(1, (best // F)[:, None])[:, 0] * F + best % F
    return out


def build_index(base, C, F, filter_nsq, whether_norm, train_sample=262144, iters=12,
                pq_sample=131072, seed=0, whether_pq=False, pq_nsq=None, exact_assign=None):
    """Trains and builds a Puck index from a device tensor `base` [n, d].

    Returns host numpy arrays in input order (the contents of the index files):
    coarse, fine, base, cell_assign, filter_codebook, filter_offsets, filter_codes,
    and with whether_pq the second-level PQ (pq_nsq subspaces, d by default):
    pq_codebook, pq_offsets, pq_codes. As in puck_assign (puck_index.cpp:602-709)
    the PQ encodes the residual left by the filter quantization, and each
    quantization's offset is 2 * decoded . (coarse + fine + the earlier decodings).
    """
    dev = base.device
    n, d = base.shape
    assert d % filter_nsq == 0, "feature_dim must be a multiple of filter_nsq"
    g = torch.Generator(device="cpu").manual_seed(seed)
    sample = base[torch.randperm(n, generator=g)[:min(train_sample, n)].to(dev)].contiguous()
    coarse = kmeans(sample, C, iters=iters, seed=seed + 1)
    ca, _ = _nearest(coarse, sample)
    fine = kmeans((sample - coarse[ca]).contiguous(), F, iters=iters, seed=seed + 2)
    order = torch.argsort(-(fine * fine).sum(1), stable=True)
    fine = fine[order].contiguous()

    cell = assign_cells(base, coarse, fine, exact=exact_assign)
    pq_idx = torch.randperm(n, generator=g)[:min(pq_sample, n)].to(dev)
    pcell = cell[pq_idx]
    res = base[pq_idx] - coarse[pcell // F] - fine[pcell % F]
    books = _pq_train(res.contiguous(), filter_nsq, iters=10, seed=seed + 3)
    pn = (d if pq_nsq is None else pq_nsq) if whether_pq else 0
    if whether_pq:
        assert d % pn == 0, "feature_dim must be a multiple of pq_nsq"
        sc = _pq_encode(res.contiguous(), books)
        sdec = books[torch.arange(filter_nsq, device=dev)[None, :], sc.long()].reshape(-1, d)
        pq_books = _pq_train((res - sdec).contiguous(), pn, iters=10, seed=seed + 4)

    # the encode itself: puck_assign's float order on the GPU (pgpu_puck_assign), so
    # the records are the ones the reference writes for these cells and codebooks
    lsq = d // filter_nsq
    offsets, codes, pq_offsets, pq_codes = native.puck_assign(
        base.contiguous(), cell.to(torch.int32), coarse.contiguous(), fine.contiguous(),
        books.reshape(filter_nsq, 256, lsq).contiguous(),
        pq_books.reshape(pn, 256, d // pn).contiguous() if whether_pq else None)
    out = dict(coarse=coarse.cpu().numpy(), fine=fine.cpu().numpy(),
               base=base.cpu().numpy(), cell_assign=cell.to(torch.int64).cpu().numpy().astype(np.uint32),
               filter_codebook=books.reshape(filter_nsq, 256, lsq).cpu().numpy(),
               filter_offsets=offsets.cpu().numpy(), filter_codes=codes.cpu().numpy(),
               whether_norm=bool(whether_norm))
    if whether_pq:
        out.update(pq_codebook=pq_books.reshape(pn, 256, d // pn).cpu().numpy(),
                   pq_offsets=pq_offsets.cpu().numpy(), pq_codes=pq_codes.cpu().numpy())
    return out


def gmm(n, d, ncomp, kind, seed, row_seed=None, device="cuda", chunk=1 << 21):
    """Seeded Gaussian-mixture data of the benchmark families, generated on the GPU.

    kind="int":  centres U[0,128), per-dim sigma 12, clipped to [0,255], rounded
    kind="unit": centres N(0,1), per-dim sigma 0.3, rows L2-normalised
    Component centres come from `seed`; rows from `row_seed` (default seed + 1),
    one generator per chunk, so base and query sets share one mixture.
    """
    row_seed = seed + 1 if row_seed is None else row_seed
    gc = torch.Generator(device=device).manual_seed(seed)
    if kind == "int":
        centers = torch.rand(ncomp, d, generator=gc, device=device) * 128
        sigma = 12.0
    else:
        centers = torch.randn(ncomp, d, generator=gc, device=device)
        sigma = 0.3
    out = torch.empty(n, d, dtype=torch.float32, device=device)
    for i, s in enumerate(range(0, n, chunk)):
        m = min(chunk, n - s)
        gr = torch.Generator(device=device).manual_seed(row_seed * 1000003 + i)
        comp = torch.randint(0, ncomp, (m,), generator=gr, device=device)
        x = centers[comp] + sigma * torch.randn(m, d, generator=gr, device=device)
        if kind == "int":
            x = x.clamp_(0, 255).round_()
        else:
            x = x / x.norm(dim=1, keepdim=True)
        out[s:s + m] = x
    return out
