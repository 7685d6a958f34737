"""CPU model of the split scan's selection (k_scan_score in scan_select.cu).

The kernel counts every record's distance t in 4096 bins,
    bin(t) = clamp(trunc((t - lo) * scale), 0, 4095)      (FP32, each step rounded),
with lo and scale from a sample of the records, cuts at the first bin b where the
running count reaches T, keeps the records of bins <= b and selects the exact T
smallest (t, id) among them. The argument: bin is non-decreasing in t, so a record
of a bin above b has T records strictly below it and is not in the result. This
test restates the binning in float32 NumPy and checks, over distributions that stress
it (ties, negative values, all values equal, a sample range that misses part of the
data), that the kept set always contains the exact top T and that bin is monotone.
"""
import zlib

import numpy as np
import pytest

BINS = 4096


def bins_of(t, lo, scale):
    t = np.asarray(t, np.float32)
    with np.errstate(over="ignore", invalid="ignore"):
        x = (t - np.float32(lo)).astype(np.float32) * np.float32(scale)
        x = x.astype(np.float32)
    # __float2int_rz: truncation, NaN -> 0, saturating
    x = np.where(np.isnan(x), np.float32(0.0), x)
    x = np.clip(x, -2.0 ** 31, 2.0 ** 31 - 1)
    b = np.trunc(x).astype(np.int64)
    return np.clip(b, 0, BINS - 1)


def range_of(sample):
    mn, mx = np.float32(np.min(sample)), np.float32(np.max(sample))
    if mx > mn:
        with np.errstate(over="ignore"):  # an infinite width gives scale 0, as on the GPU
            return mn, np.float32(np.float32(BINS - 1) / np.float32(mx - mn))
    return (mn if abs(mn) < 3e38 else np.float32(0.0)), np.float32(0.0)


def cut_bin(counts, T):
    n = int(counts.sum())
    if n <= T:
        return BINS - 1
    return int(np.searchsorted(np.cumsum(counts), T))  # first bin with running count >= T


def split_select(t, ids, T, sample_idx):
    lo, scale = range_of(t[sample_idx])
    b = bins_of(t, lo, scale)
    bstar = cut_bin(np.bincount(b, minlength=BINS), T)
    keep = b <= bstar
    kt, kid = t[keep], ids[keep]
    order = np.lexsort((kid, kt))[:T]
    return set(kid[order].tolist()), int(keep.sum())


def exact_top(t, ids, T):
    order = np.lexsort((ids, t))[:T]
    return set(ids[order].tolist())


CASES = {
    "normal": lambda r, n: r.normal(0.0, 1.0, n),
    "shifted_positive": lambda r, n: r.normal(50.0, 3.0, n),
    "duplicates": lambda r, n: r.integers(0, 40, n).astype(np.float64) * 0.25,
    "negative_and_positive": lambda r, n: np.concatenate([r.normal(-2.0, 0.1, n // 2),
                                                          r.normal(2.0, 0.1, n - n // 2)]),
    "all_equal": lambda r, n: np.full(n, 1.5),
    "heavy_tail": lambda r, n: r.standard_cauchy(n),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("T", [1, 100, 1100])
def test_kept_set_contains_exact_top(case, T):
    r = np.random.default_rng(zlib.crc32(f"{case}/{T}".encode()))
    n = 28_500
    t = CASES[case](r, n).astype(np.float32)
    ids = r.permutation(n).astype(np.int64) + 7
    for sample in (np.linspace(0, n - 1, 256).astype(np.int64),   # spread over the records
                   np.arange(256),                                 # the first records only
                   np.argsort(t)[-256:]):                          # only the largest values
        got, kept = split_select(t, ids, T, sample)
        assert got == exact_top(t, ids, T)
        assert kept >= min(T, n)


def test_bin_is_monotone_in_t():
    r = np.random.default_rng(5)
    t = np.sort(np.concatenate([r.normal(0, 1, 10_000), [-3e38, 3e38, -0.0, 0.0]]).astype(np.float32))
    for lo, scale in [range_of(t[:100]), range_of(t), (np.float32(0.5), np.float32(1e30)),
                      (np.float32(0.0), np.float32(0.0))]:
        b = bins_of(t, lo, scale)
        assert np.all(np.diff(b) >= 0)
