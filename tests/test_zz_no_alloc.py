"""GPU test of pgpu_nearest_center_noalloc, the assignment entry point for
callers that must not allocate device memory.

It is called through the C ABI twice in a row (the second call reuses the
library's fixed scratch array, which still holds the first call's norms) and
each result is compared with pgpu_nearest_center's on the same inputs: the
assignments and distances must be identical, as every other parity check in
this suite requires. This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from puck_gb300 import native

pytestmark = pytest.mark.gpu


def _assign_both(torch, cents_np, x_np):
    cents = torch.from_numpy(cents_np).cuda()
    x = torch.from_numpy(x_np).cuda()
    n = x.shape[0]
    a_ref = torch.empty(n, dtype=torch.int32, device="cuda")
    d_ref = torch.empty(n, dtype=torch.float32, device="cuda")
    a_new = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    d_new = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    native.nearest_center(cents, x, a_ref, d_ref, stream=stream)
    native.nearest_center_noalloc(cents, x, a_new, d_new, stream=stream)
    torch.cuda.synchronize()
    return (a_ref.cpu().numpy(), d_ref.cpu().numpy(), a_new.cpu().numpy(), d_new.cpu().numpy())


def test_noalloc_assign_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    native.load(build_if_missing=True)
    rng = np.random.default_rng(7)
    # first call: more points and centroids; second call: fewer, so stale norms of
    # the first call remain in the shared array beyond the second call's range
    for n, k, dim in ((50_000, 1000, 96), (3_000, 37, 24)):
        cents = rng.normal(size=(k, dim)).astype(np.float32)
        x = rng.normal(size=(n, dim)).astype(np.float32)
        x[:5] = cents[:5]
        a_ref, d_ref, a_new, d_new = _assign_both(torch, cents, x)
        assert np.array_equal(a_new, a_ref)
        assert np.array_equal(d_new.view(np.uint32), d_ref.view(np.uint32))


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    lib = native.load(build_if_missing=True)
    # the size check happens before any device work; the pointers are never read
    dummy = ctypes.c_void_p(16)
    rc = lib.pgpu_nearest_center_noalloc(8, dummy, 4, dummy, native.NOALLOC_MAX_POINTS + 1,
                                         dummy, dummy, None)
    assert rc == native.PGPU_E_LIMIT
    assert b"at most" in lib.pgpu_last_error()
    rc = lib.pgpu_nearest_center_noalloc(8, dummy, native.NOALLOC_MAX_CENTROIDS + 1, dummy, 10,
                                         dummy, dummy, None)
    assert rc == native.PGPU_E_LIMIT
