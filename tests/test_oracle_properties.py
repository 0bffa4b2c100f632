"""Independent checks of the oracle against numpy (not a parity oracle itself).

The BBD-tree filtering step of KMeans::fit (src/algorithm/neighbour/
bbd_tree.rs:62-193) is exact: its labels equal a brute-force FP64 argmin.
The GPU path relies on that equivalence, so it is checked here on seeded
blobs, together with kNN set equality against a numpy argsort.
"""
import numpy as np
import pytest

import oracle
from tests.datagen import blobs


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_bbd_labels_equal_bruteforce(dtype):
    x, _ = blobs(3000, 8, 6, seed=1, dtype=dtype)
    rng = np.random.default_rng(5)
    cents = x[rng.choice(len(x), 6, replace=False)].astype(np.float64)
    _, sums, counts, memb = oracle.bbd_clustering(x, cents)
    d2 = ((x.astype(np.float64)[:, None, :] - cents[None]) ** 2).sum(-1)
    assert np.array_equal(memb, d2.argmin(1))
    assert np.array_equal(counts, np.bincount(memb, minlength=6))
    ref = np.zeros_like(sums)
    np.add.at(ref, memb, x.astype(np.float64))
    assert np.allclose(sums, ref, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fit_tree_matches_bruteforce_loop(dtype):
    x, _ = blobs(4000, 16, 8, seed=2, dtype=dtype)
    fit = oracle.kmeans_fit(x, 8, 100, seed=42)
    # replay the same Lloyd loop brute force from the same k-means++ start
    first, u = oracle.kmeanspp_draws(len(x), 8, seed=42)
    y0, _ = oracle.kmeanspp(x, 8, first, u)
    c0 = np.zeros((8, 16))
    np.add.at(c0, y0, x.astype(np.float64))
    c0 /= np.bincount(y0, minlength=8)[:, None]
    bf = oracle.lloyd_bruteforce(x, c0, 100)
    assert np.array_equal(fit.labels, bf.labels)
    assert np.allclose(fit.centroids, bf.centroids, rtol=1e-12, atol=1e-12)
    assert abs(fit.distortion - bf.distortion) <= 1e-9 * abs(bf.distortion)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_knn_find_set_matches_argsort(dtype):
    rng = np.random.default_rng(3)
    train = rng.normal(size=(700, 5)).astype(dtype)
    q = rng.normal(size=(40, 5)).astype(dtype)
    idx, dist = oracle.knn_find(train, q, 7)
    d = np.sqrt(((q.astype(np.float64)[:, None] - train.astype(np.float64)[None]) ** 2).sum(-1))
    want = np.argsort(d, axis=1, kind="stable")[:, :7]
    for r in range(len(q)):
        assert set(idx[r]) == set(want[r])
        # the root of the heap array is the farthest kept neighbour
        assert dist[r, 0] == dist[r].max()


def test_kmeanspp_chosen_distinct():
    x, _ = blobs(2000, 4, 10, seed=9)
    first, u = oracle.kmeanspp_draws(len(x), 10, seed=11)
    y, chosen = oracle.kmeanspp(x, 10, first, u)
    assert len(set(chosen.tolist())) == 10
    assert set(y.tolist()) == set(range(10))
