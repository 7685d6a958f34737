"""GPU tests of the precision form (pgpu_params.precision = BF16, scan mode).

* the BF16 rerank screen returns the FP32 rerank of the same filter candidates:
  each returned distance is the exact FP32 squared L2 of its id (rtol 1e-6 vs
  FP64) and no candidate outside the result is closer than the topk-th;
* the filter distances (BF16 tensor-core fine terms + FP16 table, FP32
  accumulation) stay within their stated error bound of the FP64 ADC value:
  |t - t64| <= 4 * 2^-7 * |q| |f| + 2^-10 * sum_m LUT64_m + 1e-5 * (1 + |t64|);
* recall against the FP32 path on the same index stays >= 0.97 at top-10.
"""
import tempfile

import numpy as np
import pytest

from puck_gb300 import builder, index_io, native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def idx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    native.load(build_if_missing=True)
    tmp = tempfile.mkdtemp(prefix="puck_prec_")
    base = builder.gmm(150_000, 96, 512, "unit", 31)
    arrays = builder.build_index(base, 128, 128, 24, True, train_sample=65536, iters=6,
                                 pq_sample=32768, seed=31)
    host = {k: (v.cpu().numpy() if hasattr(v, "cpu") else np.asarray(v)) for k, v in arrays.items()}
    index_io.write_index(tmp, base=host["base"], coarse=host["coarse"], fine=host["fine"],
                         cell_assign=host["cell_assign"], filter_codebook=host["filter_codebook"],
                         filter_offsets=host["filter_offsets"], filter_codes=host["filter_codes"],
                         whether_norm=True)
    q = builder.gmm(400, 96, 512, "unit", 31, row_seed=5).cpu().numpy()
    del base
    torch.cuda.empty_cache()
    return tmp, host, q


def _qn(q):
    q64 = q.astype(np.float64)
    return q64 / np.linalg.norm(q64, axis=1, keepdims=True)


def test_bf16_rerank_is_exact_over_its_candidates(idx):
    path, host, q = idx
    base = host["base"].astype(np.float64)
    ix = native.GpuIndex(path, search_coarse_count=4, filter_topk=300, filter_margin=60, topk=20,
                         max_batch=512, mode=native.PGPU_MODE_SCAN,
                         precision=native.PGPU_PRECISION_BF16)
    labels, fdist, cnt = ix.filter_candidates(q)
    dist, ids = ix.search(q, 20)
    qn = _qn(q)
    assert (cnt > 20).all()
    for i in range(q.shape[0]):
        cand = labels[i, :cnt[i]].astype(np.int64)
        exact = ((base[cand] - qn[i]) ** 2).sum(1)
        kth = np.sort(exact)[19]
        got = ids[i].astype(np.int64)
        assert len(set(got.tolist())) == 20 and set(got.tolist()) <= set(cand.tolist())
        ge = ((base[got] - qn[i]) ** 2).sum(1)
        np.testing.assert_allclose(dist[i], ge, rtol=2e-6, atol=1e-7)
        assert np.all(np.diff(dist[i]) >= 0)
        # nothing left out is closer than the returned topk-th (FP32 rounding slack)
        assert ge.max() <= kth * (1 + 4e-6) + 1e-7
    ix.close()


def test_filter_distance_error_bound(idx):
    path, host, q = idx
    ix = native.GpuIndex(path, search_coarse_count=2, filter_topk=200, filter_margin=0, topk=10,
                         max_batch=512, mode=native.PGPU_MODE_SCAN,
                         precision=native.PGPU_PRECISION_BF16)
    labels, fdist, cnt = ix.filter_candidates(q[:64])
    qn = _qn(q[:64])
    coarse = host["coarse"].astype(np.float64)
    fine = host["fine"].astype(np.float64)
    cb = host["filter_codebook"].astype(np.float64).reshape(24, 256, 4)
    F = fine.shape[0]
    worst = 0.0
    for i in range(64):
        lab = labels[i, :cnt[i]].astype(np.int64)
        cell = host["cell_assign"][lab].astype(np.int64)
        c, f = cell // F, cell % F
        cd = 0.5 * (coarse[c] ** 2).sum(1) - coarse[c] @ qn[i]
        stat = 0.5 * (fine[f] ** 2).sum(1) + (fine[f] * coarse[c]).sum(1)
        fd = -(fine[f] @ qn[i])
        codes = host["filter_codes"][lab].astype(np.int64)
        sub = qn[i].reshape(24, 4)
        lut = ((sub[:, None, :] - cb) ** 2).sum(-1)            # [24, 256]
        parts = lut[np.arange(24)[None, :], codes]             # [m, 24]
        t64 = 2.0 * (cd + stat + fd) + host["filter_offsets"][lab] + parts.sum(1)
        fnorm = np.linalg.norm(fine[f], axis=1)
        bound = 4 * 2.0 ** -7 * fnorm + 2.0 ** -10 * parts.sum(1) + 1e-5 * (1 + np.abs(t64))
        err = np.abs(fdist[i, :cnt[i]].astype(np.float64) - t64)
        assert (err <= bound).all(), float((err / bound).max())
        worst = max(worst, float(err.max()))
    assert worst > 0.0  # the precision form is not bit-identical to FP64
    ix.close()


def _filter_bound_check(path, host, q, nsq, lsq):
    """The filter distances of the precision form stay within the stated bound."""
    ix = native.GpuIndex(path, search_coarse_count=2, filter_topk=200, filter_margin=0, topk=10,
                         max_batch=512, mode=native.PGPU_MODE_SCAN,
                         precision=native.PGPU_PRECISION_BF16)
    labels, fdist, cnt = ix.filter_candidates(q)
    qn = _qn(q)
    coarse = host["coarse"].astype(np.float64)
    fine = host["fine"].astype(np.float64)
    cb = host["filter_codebook"].astype(np.float64).reshape(nsq, 256, lsq)
    F = fine.shape[0]
    for i in range(q.shape[0]):
        lab = labels[i, :cnt[i]].astype(np.int64)
        cell = host["cell_assign"][lab].astype(np.int64)
        c, f = cell // F, cell % F
        cd = 0.5 * (coarse[c] ** 2).sum(1) - coarse[c] @ qn[i]
        stat = 0.5 * (fine[f] ** 2).sum(1) + (fine[f] * coarse[c]).sum(1)
        fd = -(fine[f] @ qn[i])
        codes = host["filter_codes"][lab].astype(np.int64)
        sub = qn[i].reshape(nsq, lsq)
        lut = ((sub[:, None, :] - cb) ** 2).sum(-1)
        parts = lut[np.arange(nsq)[None, :], codes]
        t64 = 2.0 * (cd + stat + fd) + host["filter_offsets"][lab] + parts.sum(1)
        fnorm = np.linalg.norm(fine[f], axis=1)
        bound = 4 * 2.0 ** -7 * fnorm + 2.0 ** -10 * parts.sum(1) + 1e-5 * (1 + np.abs(t64))
        err = np.abs(fdist[i, :cnt[i]].astype(np.float64) - t64)
        assert (err <= bound).all(), float((err / bound).max())
    ix.close()


@pytest.mark.parametrize("d,nsq", [
    (128, 32),  # rotated one-bank-per-subspace table over all 32 banks
    (60, 15),   # nsq not a multiple of 4: the FP16 table in the reference's layout
])
def test_filter_distance_error_bound_layouts(d, nsq):
    import torch
    native.load(build_if_missing=True)
    with tempfile.TemporaryDirectory() as tmp:
        base = builder.gmm(60_000, d, 256, "unit", 17)
        arrays = builder.build_index(base, 48, 48, nsq, True, train_sample=40000, iters=5,
                                     pq_sample=20000, seed=17)
        host = {k: (v.cpu().numpy() if hasattr(v, "cpu") else np.asarray(v))
                for k, v in arrays.items()}
        index_io.write_index(tmp, base=host["base"], coarse=host["coarse"], fine=host["fine"],
                             cell_assign=host["cell_assign"],
                             filter_codebook=host["filter_codebook"],
                             filter_offsets=host["filter_offsets"],
                             filter_codes=host["filter_codes"], whether_norm=True)
        q = builder.gmm(48, d, 256, "unit", 17, row_seed=9).cpu().numpy()
        del base
        torch.cuda.empty_cache()
        _filter_bound_check(tmp, host, q, nsq, d // nsq)


def test_bf16_recall_against_fp32_path(idx):
    path, host, q = idx
    fp = native.GpuIndex(path, search_coarse_count=4, filter_topk=300, topk=10, max_batch=512,
                         mode=native.PGPU_MODE_SCAN)
    d32, i32 = fp.search(q, 10)
    fp.set_search_params(precision=native.PGPU_PRECISION_BF16, filter_margin=60)
    d16, i16 = fp.search(q, 10)
    overlap = np.mean([len(set(a.tolist()) & set(b.tolist())) / 10.0 for a, b in zip(i32, i16)])
    assert overlap >= 0.97, overlap
    # the same ids carry the same FP32 distances in both forms
    for i in range(q.shape[0]):
        common = set(i32[i].tolist()) & set(i16[i].tolist())
        for lab in common:
            a = d32[i][list(i32[i]).index(lab)]
            b = d16[i][list(i16[i]).index(lab)]
            assert a == b
    fp.close()


def test_bf16_needs_scan_mode(idx):
    path, host, q = idx
    with pytest.raises(native.PuckGpuError) as e:
        native.GpuIndex(path, search_coarse_count=4, filter_topk=300, topk=10,
                        mode=native.PGPU_MODE_EXACT, precision=native.PGPU_PRECISION_BF16)
    assert e.value.code == native.PGPU_E_INVALID
