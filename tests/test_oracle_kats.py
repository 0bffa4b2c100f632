"""Pin the CPU oracle to the reference's own known-answer tests.

Each test restates one smartcore test (the fixture names its file:line) and
runs it against the oracle.  These pins are what make the oracle a trustworthy
reference for the GPU parity tests.
"""
import math

import numpy as np
import pytest

import oracle


def test_bbdtree_iris(kats):
    kat = kats["bbdtree_iris"]
    x = np.array(kat["x"], np.float64)
    dist, sums, counts, memb = oracle.bbd_clustering(x, np.array(kat["centroids"]))
    got = {"dist": dist, "sums[0][0]": sums[0][0], "sums[1][3]": sums[1][3]}
    for name, want, tol in kat["expect_close"]:
        assert abs(got[name] - want) < tol, (name, got[name], want)
    i, want = kat["expect_membership"]
    assert memb[i] == want
    assert counts.sum() == x.shape[0]


@pytest.mark.parametrize("layout", ["C", "F"])
def test_kmeans_fit_predict(kats, layout):
    kat = kats["kmeans_fit_predict"]
    x = np.array(kat["x"], np.float64, order=layout)
    p = kat["params"]
    fit = oracle.kmeans_fit(x, p["k"], p["max_iter"], seed=0)  # seed None -> 0
    y = oracle.kmeans_predict(x, fit.centroids)
    assert np.array_equal(y, fit.labels)
    assert fit.sizes.sum() == x.shape[0]


def test_kmeans_invalid_k(kats):
    kat = kats["kmeans_invalid_k"]
    x = np.array(kat["x"], np.float64)
    for k in kat["k_err"]:
        with pytest.raises(ValueError) as e:
            oracle.kmeans_fit(x, k, 100, first=0, uniforms=np.zeros(1))
        if k == 1:
            assert str(e.value) == kat["message_k1"]


@pytest.mark.parametrize("case", range(4))
def test_heap_select(kats, case):
    c = kats["heap_select"]["cases"][case]
    heap, n = oracle.heap_add_sequence(c["adds"], c["k"])
    assert n == c["n"]
    assert list(heap) == c["heap"], c["name"]


def test_knn_find(kats):
    kat = kats["knn_find"]
    s = kat["scalar"]
    train = np.array(s["data"], np.float64)[:, None]
    idx, _ = oracle.knn_find(train, np.array([[s["query"]]], np.float64), s["k"])
    assert sorted(idx[0]) == s["expect_sorted_idx"]
    r = kat["scalar_radius"]
    counts, ridx, _ = oracle.knn_find_radius(train, np.array([[r["query"]]], np.float64), r["radius"])
    assert sorted(int(train[i, 0]) for i in ridx) == r["expect_sorted_values"]
    e = kat["euclid"]
    idx, _ = oracle.knn_find(np.array(e["data"]), np.array([e["query"]]), e["k"])
    assert sorted(idx[0]) == e["expect_sorted_idx"]
    with pytest.raises(ValueError):
        oracle.knn_find(np.array(e["data"]), np.array([e["query"]]), 0)
    with pytest.raises(ValueError):
        oracle.knn_find(np.array(e["data"]), np.array([e["query"]]), len(e["data"]) + 1)
    with pytest.raises(ValueError):
        oracle.knn_find_radius(train, np.array([[1.0]]), 0.0)


def test_euclidian_distance(kats):
    kat = kats["euclidian_distance"]
    l2 = math.sqrt(oracle.sqdist(np.array(kat["a"]), np.array(kat["b"])))
    assert abs(l2 - kat["expect"]) < kat["tol"]


def _classes(y):
    classes = sorted(set(y))  # y.unique(): sorted, deduplicated (arrays.rs:223-231)
    return classes, np.array([classes.index(v) for v in y], np.int64)


def test_knn_classifier_weighted(kats):
    kat = kats["knn_classifier_weighted"]
    classes, yi = _classes(kat["y"])
    idx, dist = oracle.knn_find(np.array(kat["x"]), np.array(kat["query"]), kat["k"])
    out = oracle.knn_vote(idx, dist, yi, len(classes), weight=1)
    assert [classes[c] for c in out] == kat["expect"]


def test_knn_classifier_default(kats):
    kat = kats["knn_classifier_default"]
    classes, yi = _classes(kat["y"])
    x = np.array(kat["x"])
    idx, dist = oracle.knn_find(x, x, kat["k"])
    out = oracle.knn_vote(idx, dist, yi, len(classes), weight=0)
    assert [classes[c] for c in out] == kat["y"]


@pytest.mark.parametrize("key", ["knn_regressor_weighted", "knn_regressor_uniform"])
def test_knn_regressor(kats, key):
    kat = kats[key]
    x = np.array(kat["x"])
    idx, dist = oracle.knn_find(x, x, kat["k"])
    out = oracle.knn_regress(idx, dist, np.array(kat["y"]), weight=1 if kat["weight"] == "distance" else 0)
    assert np.all(np.abs(out - np.array(kat["expect"])) < kat["tol"])


def test_rng_draws_shape_and_range():
    for rng in (oracle.RNG_SMALL, oracle.RNG_STD):
        first, u = oracle.kmeanspp_draws(1000, 16, seed=42, rng=rng)
        assert 0 <= first < 1000 and u.shape == (15,)
        assert np.all((u >= 0) & (u < 1))
        f2, u2 = oracle.kmeanspp_draws(1000, 16, seed=42, rng=rng)
        assert f2 == first and np.array_equal(u, u2)
    a = oracle.rng_u64(8, seed=7, rng=oracle.RNG_SMALL)
    b = oracle.rng_u64(8, seed=7, rng=oracle.RNG_STD)
    assert not np.array_equal(a, b)


def test_rng_std_straddle():
    # next_u64 across the 64-word block buffer reads the same words as u32 pairs
    many = oracle.rng_u64(40, seed=3, rng=oracle.RNG_STD)
    assert len(set(many.tolist())) == 40


def test_dbscan_fit_predict(kats):
    c = kats["dbscan_fit_predict"]
    x = np.array(c["x"])
    y, k = oracle.dbscan_fit(x, c["eps"], c["min_samples"])
    assert oracle.dbscan_predict(x, y, k, x, c["eps"]).tolist() == c["expect"]
    for bad, msg in (((c["eps"], 0), c["errors"][0]), ((0.0, 2), c["errors"][1])):
        with pytest.raises(ValueError, match=msg.strip()):
            oracle.dbscan_fit(x, *bad)


def test_fastpair(kats):
    c = kats["fastpair"]
    nb, dist, closest = oracle.fastpair(np.array(c["x"]))
    for i, (node, neighbour, d) in c["distances"].items():
        i = int(i)
        assert nb[i] == neighbour
        assert dist[i] == (np.finfo(np.float64).max if d == float("inf") else d)
    for case in c["closest"].values():
        assert list(oracle.fastpair(np.array(case["x"]))[2]) == case["expect"]
    with pytest.raises(ValueError, match=c["error"]):
        oracle.fastpair(np.zeros((2, 2)))
