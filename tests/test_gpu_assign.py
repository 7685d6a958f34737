"""The build's encoder on the GPU (pgpu_puck_assign, PuckIndex::puck_assign,
puck/puck/puck_index.cpp:602-709): filter-PQ (and second-level PQ) offsets and codes
bit-identical to the reference's own index files, and to the oracle at larger sizes."""
import numpy as np
import pytest

import oracle
from puck_gb300 import index_io, native

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _cuda(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a if dtype is None else a.astype(dtype)))
    return t.cuda()


def _gpu_assign(a):
    import torch
    pcb = a.get("pq_codebook")
    f_off, f_codes, p_off, p_codes = native.puck_assign(
        _cuda(a["base"], np.float32), _cuda(a["cell_assign"].view(np.int32)),
        _cuda(a["coarse"], np.float32), _cuda(a["fine"], np.float32),
        _cuda(a["filter_codebook"], np.float32),
        None if pcb is None else _cuda(pcb, np.float32))
    torch.cuda.synchronize()
    out = [f_off.cpu().numpy(), f_codes.cpu().numpy()]
    out += [None, None] if p_off is None else [p_off.cpu().numpy(), p_codes.cpu().numpy()]
    return out


def test_gpu_puck_assign_matches_reference(golden):
    name, z, index_dir = golden
    a = index_io.read_index(index_dir)
    f_off, f_codes, p_off, p_codes = _gpu_assign(a)
    assert np.array_equal(_bits(f_off), _bits(a["filter_offsets"])), name
    assert np.array_equal(f_codes, a["filter_codes"]), name
    if a.get("pq_codebook") is not None:
        assert np.array_equal(_bits(p_off), _bits(a["pq_offsets"])), name
        assert np.array_equal(p_codes, a["pq_codes"]), name


def test_gpu_puck_assign_equals_oracle_large():
    """50k points of the benchmark's mixture, d = 96, filter 24 x 256 and the
    second-level PQ (96 one-dimensional subspaces): GPU == oracle, bit for bit."""
    import torch
    from puck_gb300 import builder
    base = builder.gmm(50000, 96, 512, "unit", 7)
    a = builder.build_index(base, 64, 64, 24, True, train_sample=50000, iters=4,
                            pq_sample=32768, seed=7, whether_pq=True)
    a["base"] = base.cpu().numpy()
    del base
    torch.cuda.empty_cache()
    g = _gpu_assign(a)
    o = oracle.puck_assign(a["base"], a["cell_assign"], a["coarse"], a["fine"],
                           a["filter_codebook"], a["pq_codebook"])
    assert np.array_equal(_bits(g[0]), _bits(o[0]))
    assert np.array_equal(g[1], o[1])
    assert np.array_equal(_bits(g[2]), _bits(o[2]))
    assert np.array_equal(g[3], o[3])


def test_gpu_puck_assign_rejects_bad_cells():
    import torch
    d, n = 8, 40
    base = torch.rand(n, d, device="cuda")
    coarse = torch.rand(2, d, device="cuda")
    fine = torch.rand(3, d, device="cuda")
    cb = torch.rand(2, 256, 4, device="cuda")
    cells = torch.zeros(n, dtype=torch.int32, device="cuda")
    cells[17] = 6  # C * F = 6: out of range
    with pytest.raises(native.PuckGpuError) as e:
        native.puck_assign(base, cells, coarse, fine, cb)
    assert e.value.code == native.PGPU_E_INVALID


def _gpu_cells(coarse, fine, x):
    import torch
    xs = _cuda(x, np.float32)
    cell = torch.empty(x.shape[0], dtype=torch.int32, device="cuda")
    dist = torch.empty(x.shape[0], dtype=torch.float32, device="cuda")
    native.nearest_cell_assign(_cuda(coarse, np.float32), _cuda(fine, np.float32), xs, cell, dist)
    torch.cuda.synchronize()
    return cell.cpu().numpy().view(np.uint32), dist.cpu().numpy()


def test_gpu_nearest_cell_assign_matches_reference(golden):
    """pgpu_nearest_cell_assign gives the reference's own cell_assign.dat
    (hierarchical_cluster_index.cpp:1042-1138) and the oracle's distances bit for bit."""
    name, z, index_dir = golden
    a = index_io.read_index(index_dir)
    base = np.ascontiguousarray(a["base"], np.float32)
    cell, dist = _gpu_cells(a["coarse"], a["fine"], base)
    assert np.array_equal(cell, np.asarray(a["cell_assign"]).astype(np.uint32)), name
    ocell, odist = oracle.nearest_cell_assign(a["coarse"], a["fine"], base)
    assert np.array_equal(cell, ocell)
    assert np.array_equal(_bits(dist), _bits(odist))


def test_gpu_nearest_cell_assign_equals_oracle_many_chunks():
    """Several point chunks (1024 + 1024 centroids), ties and points with many
    equally near coarse clusters (the walk's slow path): bit-identical to the oracle."""
    rng = np.random.default_rng(5)
    d, C, F = 16, 1024, 1024
    coarse = rng.normal(size=(C, d)).astype(np.float32)
    coarse[:200] = coarse[:200] / np.linalg.norm(coarse[:200], axis=1, keepdims=True)  # a shell
    coarse[300:310] = coarse[200]                                                      # duplicates
    fine = (0.3 * rng.normal(size=(F, d))).astype(np.float32)
    fine = fine[np.argsort(-np.linalg.norm(fine, axis=1), kind="stable")]
    x = rng.normal(size=(140_000, d)).astype(np.float32)
    x[:64] = 0.0                      # equidistant from the 200 shell centroids
    x[64:128] = coarse[200] + fine[7]  # exact ties between duplicated cells
    cell, dist = _gpu_cells(coarse, fine, x)
    ocell, odist = oracle.nearest_cell_assign(coarse, fine, x)
    assert np.array_equal(cell, ocell)
    assert np.array_equal(_bits(dist), _bits(odist))
