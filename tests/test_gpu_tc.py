"""GPU tests of the BF16 tensor-core contraction (tcgen05) and of the exact
selections built on it.

* pgpu_contract_bf16 against an FP64 product of the BF16-rounded operands, in
  every epilogue and for row-major and transposed operands, with the FP32
  accumulation bound |err| <= k * 2^-23 * sum_t |a_t b_t| written in the test;
* pgpu_contract_bf16_rows (BF16 rows in memory: the persistent TMA kernel when the
  rows are 16-byte aligned) against the same bound, over ragged rows and K, many
  tiles per CTA and every epilogue;
* nearest_center (tensor-core screen + exact FP32 window) bit-identical to the
  oracle, including exact ties between duplicated centroids;
* the coarse top-P window: with duplicated coarse centroids (ties at the cut)
  the search falls back to the exact heap and still equals the oracle.
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
from puck_gb300 import builder, index_io, native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    native.load(build_if_missing=True)


def _bf16(x):
    import torch
    return x.to(torch.bfloat16).to(torch.float64)


def _operand(rows, k, transposed, gen):
    import torch
    if transposed:
        return torch.randn(k, rows, device="cuda", generator=gen).t()
    return torch.randn(rows, k, device="cuda", generator=gen)


def _check_acc(out_acc, a, b):
    ref = _bf16(a) @ _bf16(b).t()
    bound = (_bf16(a).abs() @ _bf16(b).abs().t()) * (a.shape[1] * 2.0 ** -23) + 1e-30
    err = (out_acc.double() - ref).abs()
    assert bool((err <= bound).all()), float((err / bound).max())


@pytest.mark.parametrize("na,nb,k,ta,tb", [
    (1, 1, 16, False, False),
    (300, 200, 96, False, False),
    (128, 128, 64, False, False),
    (257, 513, 100, False, False),
    (64, 4000, 512, False, False),
    (1000, 96, 1003, False, False),
    (130, 70, 200, True, False),
    (96, 512, 777, True, True),
    (513, 33, 129, False, True),
])
def test_contract_store(na, nb, k, ta, tb):
    import torch
    g = torch.Generator(device="cuda").manual_seed(na * 131 + nb * 7 + k)
    a = _operand(na, k, ta, g)
    b = _operand(nb, k, tb, g)
    out = torch.full((na, nb), float("nan"), device="cuda")
    native.contract_bf16("store", a, b, out)
    _check_acc(out, a, b)


def test_contract_epilogues():
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    na, nb, k = 200, 300, 96
    a = torch.randn(na, k, device="cuda", generator=g)
    b = torch.randn(nb, k, device="cuda", generator=g)
    bias = torch.randn(nb, device="cuda", generator=g)
    acc = torch.empty(na, nb, device="cuda")
    native.contract_bf16("store", a, b, acc)
    _check_acc(acc, a, b)
    # score: bias - acc (one rounding)
    out = torch.empty_like(acc)
    native.contract_bf16("score", a, b, out, bias=bias)
    assert torch.equal(out, bias[None, :] - acc)
    native.contract_bf16("neg", a, b, out)
    assert torch.equal(out, -acc)
    native.contract_bf16("bias", a, b, out, bias=bias)
    assert torch.equal(out, acc + bias[None, :])
    # alpha/beta accumulate into the existing output
    prev = torch.randn(na, nb, device="cuda", generator=g)
    out.copy_(prev)
    native.contract_bf16("store", a, b, out, alpha=0.5, beta=2.0)
    torch.testing.assert_close(out, 0.5 * acc + 2.0 * prev, rtol=1e-6, atol=1e-6)
    # bias + GELU, keeping the pre-activation
    pre = torch.empty_like(acc)
    native.contract_bf16("bias_gelu", a, b, out, bias=bias, out2=pre)
    assert torch.equal(pre, acc + bias[None, :])
    torch.testing.assert_close(out, torch.nn.functional.gelu(pre), rtol=1e-5, atol=1e-6)
    # GELU backward: acc * GELU'(aux)
    aux = torch.randn(na, nb, device="cuda", generator=g)
    native.contract_bf16("gelu_bwd", a, b, out, aux=aux)
    x = aux.double().requires_grad_(True)
    torch.nn.functional.gelu(x).sum().backward()
    torch.testing.assert_close(out.double(), acc.double() * x.grad, rtol=1e-5, atol=1e-6)


def _bf16_rows(rows, k, pad, gen):
    """A random BF16 operand [rows, k] whose rows are `pad` elements apart."""
    import torch
    full = torch.randn(rows, pad, device="cuda", generator=gen).to(torch.bfloat16)
    return full[:, :k]


@pytest.mark.parametrize("na,nb,k,pad", [
    (1, 1, 16, 16),
    (300, 200, 96, 96),        # one 128-column tile
    (129, 257, 100, 104),      # ragged rows and K (zero fill past the ends), 256-column tiles
    (1000, 4000, 512, 512),    # the probe's output layer shape: many tiles per CTA
    (4100, 512, 96, 96),       # more row tiles than SMs
    (5, 300, 40, 40),          # K below one 64-wide chunk
    (257, 130, 8, 8),
    (130, 70, 100, 100),       # rows not 16-byte aligned: the cp.async kernel
])
def test_contract_rows_store(na, nb, k, pad):
    import torch
    g = torch.Generator(device="cuda").manual_seed(na * 17 + nb + k)
    a = _bf16_rows(na, k, pad, g)
    b = _bf16_rows(nb, k, pad, g)
    out = torch.full((na, nb), float("nan"), device="cuda")
    native.contract_bf16_rows("store", a, b, out)
    _check_acc(out, a.float(), b.float())


def test_contract_rows_epilogues():
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    na, nb, k = 700, 600, 96
    a = _bf16_rows(na, k, k, g)
    b = _bf16_rows(nb, k, k, g)
    bias = torch.randn(nb, device="cuda", generator=g)
    acc = torch.empty(na, nb, device="cuda")
    native.contract_bf16_rows("store", a, b, acc)
    _check_acc(acc, a.float(), b.float())
    out = torch.empty_like(acc)
    native.contract_bf16_rows("score", a, b, out, bias=bias)
    assert torch.equal(out, bias[None, :] - acc)
    native.contract_bf16_rows("neg", a, b, out)
    assert torch.equal(out, -acc)
    native.contract_bf16_rows("bias", a, b, out, bias=bias)
    assert torch.equal(out, acc + bias[None, :])
    pre = torch.empty_like(acc)
    native.contract_bf16_rows("bias_gelu", a, b, out, bias=bias, out2=pre)
    assert torch.equal(pre, acc + bias[None, :])
    torch.testing.assert_close(out, torch.nn.functional.gelu(pre), rtol=1e-5, atol=1e-6)
    # the same accumulators as the FP32-operand entry point on the same BF16 values
    ref = torch.empty_like(acc)
    native.contract_bf16("store", a.float(), b.float(), ref)
    _check_acc(ref, a.float(), b.float())


def test_contract_rejects_bad_arguments():
    import torch
    a = torch.randn(4, 8, device="cuda")
    out = torch.empty(4, 4, device="cuda")
    with pytest.raises(native.PuckGpuError) as e:
        native.contract_bf16("score", a, a[:4], out)  # score needs a bias
    assert e.value.code == native.PGPU_E_INVALID


@pytest.mark.parametrize("n,k,d,kind", [(4000, 2000, 96, "normal"), (3000, 500, 128, "int"),
                                        (2500, 64, 20, "normal")])
def test_nearest_center_tc_equals_oracle(n, k, d, kind):
    import torch
    rng = np.random.default_rng(n + k)
    if kind == "int":
        cents = rng.integers(0, 8, size=(k, d)).astype(np.float32)
        x = rng.integers(0, 8, size=(n, d)).astype(np.float32)
    else:
        cents = rng.normal(size=(k, d)).astype(np.float32)
        x = rng.normal(size=(n, d)).astype(np.float32)
    cents[5] = cents[3]       # duplicated centroid: exact ties, the lower id wins
    x[:20] = cents[3]
    x[20:40] = cents[rng.integers(0, k, 20)]
    oa, od = oracle.nearest_center(cents, x)
    ct = torch.from_numpy(cents).cuda()
    xt = torch.from_numpy(x).cuda()
    a = torch.empty(n, dtype=torch.int32, device="cuda")
    dd = torch.empty(n, dtype=torch.float32, device="cuda")
    native.nearest_center(ct, xt, a, dd, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    assert np.array_equal(a.cpu().numpy(), oa)
    assert np.array_equal(dd.cpu().numpy().view(np.uint32), od.view(np.uint32))
    assert (a.cpu().numpy()[:20] == 3).all()


@pytest.mark.parametrize("mode", [native.PGPU_MODE_EXACT, native.PGPU_MODE_SCAN])
def test_coarse_window_ties_fall_back_exactly(mode):
    import torch
    with tempfile.TemporaryDirectory() as tmp:
        base = builder.gmm(40000, 32, 64, "unit", 8)
        arrays = builder.build_index(base, 48, 32, 8, True, train_sample=40000, iters=4,
                                     pq_sample=20000, seed=8)
        coarse = np.array(arrays["coarse"], np.float32)
        # duplicated coarse centroids -> equal coarse distances at or inside the cut
        for a_, b_ in ((1, 0), (7, 6), (20, 19), (33, 32)):
            coarse[a_] = coarse[b_]
        index_io.write_index(tmp, base=arrays["base"], coarse=coarse, fine=arrays["fine"],
                             cell_assign=arrays["cell_assign"],
                             filter_codebook=arrays["filter_codebook"],
                             filter_offsets=arrays["filter_offsets"],
                             filter_codes=arrays["filter_codes"], whether_norm=True)
        q = builder.gmm(300, 32, 64, "unit", 8, row_seed=1234).cpu().numpy()
        del base
        torch.cuda.empty_cache()
        P, T, k = 8, 200, 10
        ix = native.GpuIndex(tmp, search_coarse_count=P, filter_topk=T, topk=k, max_batch=128,
                             mode=mode)
        dist, ids = ix.search(q, k)
        assert ix.walk_counters()["coarse_window_fallbacks"] > 0
        orc = oracle.OracleIndex(tmp)
        od, oi, st = orc.search_batch(q, k, P, T, topk_max=k, nthreads=os.cpu_count(),
                                      scan=(mode == native.PGPU_MODE_SCAN))
        assert (st == 0).all()
        assert np.array_equal(dist.view(np.uint32), od.view(np.uint32))
        assert np.array_equal(ids, oi)
        ix.close()
