"""The bucket function the crowded-cell ranking relies on (k_rank_cells,
k_rank_big_cells in pibiti_gb300/csrc/sph_segsort.cuh): in FP32,
bucket(id) = min(trunc(float(id - lo) * (B / (float(hi - lo) + 1))), B - 1)
must not decrease with the id, so that every id of a lower bucket is
smaller and rank = start of the bucket + the ids of its own bucket below it.
Checked on the CPU with NumPy's IEEE FP32 (round to nearest, as the GPU's
conversions and multiply), over dense id ranges and the widths where the
float conversion of id - lo starts to round."""
import numpy as np
import pytest


def buckets(ids, lo, hi, nb):
    ids = np.asarray(ids, np.uint32)
    scale = np.float32(nb) / (np.float32(np.uint32(hi - lo)) + np.float32(1.0))
    x = (ids - np.uint32(lo)).astype(np.float32) * scale
    return np.minimum(x.astype(np.uint32), np.uint32(nb - 1))


@pytest.mark.parametrize("nb", [1024, 4096])
@pytest.mark.parametrize("lo,span", [(0, 33), (5, 1000), (123456, 1 << 20), (0, (1 << 24) + 7),
                                     (1 << 30, (1 << 26) + 12345), (0, 0xFFFFFFFF)])
def test_bucket_is_non_decreasing(nb, lo, span):
    hi = lo + span
    rng = np.random.default_rng(span % 1000)
    ids = np.unique(np.concatenate([
        np.arange(lo, lo + min(span, 200_000) + 1, dtype=np.uint64),
        rng.integers(lo, hi, 200_000, endpoint=True, dtype=np.uint64),
        np.arange(max(lo, hi - 1000), hi + 1, dtype=np.uint64)])).astype(np.uint32)
    b = buckets(ids, lo, hi, nb)
    assert np.all(np.diff(b.astype(np.int64)) >= 0)
    assert b[0] == 0 and b.max() <= nb - 1


def test_rank_from_buckets_matches_sort():
    """The ranking procedure itself on random id sets, against argsort."""
    rng = np.random.default_rng(3)
    for n in (33, 100, 1024, 5000):
        ids = rng.choice(1 << 20, n, replace=False).astype(np.uint32)
        lo, hi = int(ids.min()), int(ids.max())
        b = buckets(ids, lo, hi, 1024).astype(np.int64)
        start = np.concatenate([[0], np.cumsum(np.bincount(b, minlength=1024))[:-1]])
        rank = np.array([start[bi] + np.sum((b == bi) & (ids < x)) for x, bi in zip(ids, b)])
        np.testing.assert_array_equal(rank, np.argsort(np.argsort(ids)))
