"""GPU parity of LinearKNNSearch::find and the kNN estimators (through the C
ABI) against the CPU oracle: neighbour indices and distances bit-identical,
in the reference's heap-array order."""
import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.error import Failed
from smartcore_gb300.neighbors import (KNNAlgorithmName, KNNClassifier, KNNClassifierParameters,
                                       KNNRegressor, KNNRegressorParameters, KNNWeightFunction,
                                       LinearKNNSearch)
from tests.datagen import knn_blobs_f32

pytestmark = pytest.mark.gpu

FORMS = [pytest.param(_lib.FORM_FP64, id="fp64"), pytest.param(_lib.FORM_SPLIT_BF16, id="split")]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("k", [1, 5, 16])
def test_find_heap_order(form, dtype, k):
    rng = np.random.default_rng(k)
    train = rng.normal(size=(3000, 13)).astype(dtype)
    q = rng.normal(size=(300, 13)).astype(dtype)
    s = LinearKNNSearch(train, form=form)
    idx, dist = s.find_batch(q, k)
    ridx, rdist = oracle.knn_find(train, q, k)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)


@pytest.mark.parametrize("form", FORMS)
def test_find_d128_k10(form):
    # the shape of the large kNN workload (d = 128, k = 10) at a reduced size
    rng = np.random.default_rng(128)
    centres = rng.uniform(-50, 50, size=(64, 128))
    train = (centres[rng.integers(0, 64, 20000)] + rng.normal(scale=2.0, size=(20000, 128))).astype(np.float32)
    q = (centres[rng.integers(0, 64, 400)] + rng.normal(scale=2.0, size=(400, 128))).astype(np.float32)
    s = LinearKNNSearch(train, form=form)
    idx, dist = s.find_batch(q, 10)
    ridx, rdist = oracle.knn_find(train, q, 10)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d", [16, 32, 64, 200])
def test_find_wide_exponent_span(form, d):
    # features scaled from 1e-3 to 1e3: the squared terms of one distance span
    # up to ~40 bits, so every path of the exact sequential f64 sum is taken
    # (the warp's exact integer total, its 64-bit form, and the sequential
    # form where a running sum rounds), at one, two and eight features a lane
    rng = np.random.default_rng(d)
    scale = np.logspace(-3, 3, d)
    train = (rng.normal(size=(6000, d)) * scale).astype(np.float32)
    q = (rng.normal(size=(300, d)) * scale).astype(np.float32)
    q[:40] = train[rng.integers(0, 6000, 40)] * np.float32(1.0 + 1e-6)  # near-duplicates
    s = LinearKNNSearch(train, form=form)
    idx, dist = s.find_batch(q, 7)
    ridx, rdist = oracle.knn_find(train, q, 7)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_find_radius_matches_oracle(form, dtype):
    rng = np.random.default_rng(17)
    train = rng.normal(size=(5000, 12)).astype(dtype)
    q = rng.normal(size=(200, 12)).astype(dtype)
    s = LinearKNNSearch(train, form=form)
    for radius in (0.5, 1.5, 3.0):
        counts, idx, dist = s.find_radius_batch(q, radius)
        rc, ridx, rdist = oracle.knn_find_radius(train, q, radius)
        assert np.array_equal(counts, rc)
        assert np.array_equal(idx, ridx)
        assert np.array_equal(dist, rdist)
    # a radius that hits exact distances of integer grid data (d <= radius is inclusive)
    g = rng.integers(-2, 3, size=(3000, 3)).astype(dtype)
    s2 = LinearKNNSearch(g, form=form)
    for radius in (1.0, 2.0, np.sqrt(2.0)):
        counts, idx, dist = s2.find_radius_batch(g[:50], radius)
        rc, ridx, rdist = oracle.knn_find_radius(g, g[:50], radius)
        assert np.array_equal(counts, rc) and np.array_equal(idx, ridx) and np.array_equal(dist, rdist)
    assert s.find_radius(q[0], 1.5) == [(int(i), float(d)) for i, d in
                                        zip(*oracle.knn_find_radius(train, q[:1], 1.5)[1:])]
    # every row inside the radius: more rows than the first output size, so a
    # second call with the exact size serves
    counts, idx, dist = s.find_radius_batch(q, 100.0)
    rc, ridx, rdist = oracle.knn_find_radius(train, q, 100.0)
    assert np.array_equal(counts, rc) and counts.sum() == len(q) * len(train)
    assert np.array_equal(idx, ridx) and np.array_equal(dist, rdist)
    with pytest.raises(Failed, match="radius should be > 0"):
        s.find_radius(q[0], 0.0)


@pytest.mark.parametrize("form", FORMS)
def test_find_ties_and_duplicates(form):
    # integer grid data: many exact distance ties, replay order matters
    rng = np.random.default_rng(0)
    train = rng.integers(-2, 3, size=(2000, 3)).astype(np.float32)
    q = rng.integers(-2, 3, size=(200, 3)).astype(np.float32)
    s = LinearKNNSearch(train, form=form)
    for k in (1, 4, 7):
        idx, dist = s.find_batch(q, k)
        ridx, rdist = oracle.knn_find(train, q, k)
        assert np.array_equal(idx, ridx)
        assert np.array_equal(dist, rdist)


def test_find_k_equals_n_and_errors():
    train = np.random.default_rng(1).normal(size=(9, 4))
    s = LinearKNNSearch(train)
    idx, dist = s.find_batch(train, 9)
    ridx, rdist = oracle.knn_find(train, train, 9)
    assert np.array_equal(idx, ridx) and np.array_equal(dist, rdist)
    for bad in (0, 10):
        with pytest.raises(Exception) as e:
            s.find_batch(train, bad)
        assert "k should be >= 1 and <= length(data)" in str(e.value)


def test_reference_kats(kats):
    kat = kats["knn_find"]
    e = kat["euclid"]
    s = LinearKNNSearch(np.array(e["data"]))
    got = s.find(np.array(e["query"]), e["k"])
    assert sorted(i for i, _ in got) == e["expect_sorted_idx"]
    sc = kat["scalar"]
    s1 = LinearKNNSearch(np.array(sc["data"], np.float64)[:, None])
    assert sorted(i for i, _ in s1.find(np.array([float(sc["query"])]), sc["k"])) == sc["expect_sorted_idx"]
    r = kat["scalar_radius"]  # linear_search.rs:166-174: the values within radius 3 of 5
    for form in (_lib.FORM_FP64, _lib.FORM_SPLIT_BF16):
        s2 = LinearKNNSearch(np.array(sc["data"], np.float64)[:, None], form=form)
        got = s2.find_radius(np.array([float(r["query"])]), r["radius"])
        assert sorted(int(sc["data"][i]) for i, _ in got) == r["expect_sorted_values"]

    w = kats["knn_classifier_weighted"]
    m = KNNClassifier.fit(np.array(w["x"]), np.array(w["y"], np.int64),
                          KNNClassifierParameters().with_k(w["k"])
                          .with_algorithm(KNNAlgorithmName.LinearSearch)
                          .with_weight(KNNWeightFunction.Distance))
    assert list(m.predict(np.array(w["query"]))) == w["expect"]

    dflt = kats["knn_classifier_default"]
    x = np.array(dflt["x"])
    m = KNNClassifier.fit(x, np.array(dflt["y"], np.int64))
    assert list(m.predict(x)) == dflt["y"]

    for key in ("knn_regressor_weighted", "knn_regressor_uniform"):
        r = kats[key]
        p = KNNRegressorParameters().with_k(r["k"]).with_algorithm(KNNAlgorithmName.LinearSearch)
        if r["weight"] == "distance":
            p = p.with_weight(KNNWeightFunction.Distance)
        m = KNNRegressor.fit(np.array(r["x"]), np.array(r["y"]), p)
        out = m.predict(np.array(r["x"]))
        assert np.all(np.abs(out - np.array(r["expect"])) < r["tol"])


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("weight", [0, 1])
def test_classifier_matches_oracle(form, weight):
    xt, yt, xq, _ = knn_blobs_f32(n_train=20_000, n_query=2_000, seed=3)
    m = KNNClassifier.fit(xt, yt, KNNClassifierParameters(k=5, algorithm=KNNAlgorithmName.LinearSearch,
                                                         weight=KNNWeightFunction(weight), form=form))
    got = m.predict(xq)
    idx, dist = oracle.knn_find(xt, xq, 5)
    want = oracle.knn_vote(idx, dist, yt, 10, weight=weight)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("weight", [0, 1])
def test_regressor_matches_oracle(weight):
    rng = np.random.default_rng(8)
    xt = rng.normal(size=(5000, 6))
    y = rng.normal(size=5000)
    xq = rng.normal(size=(500, 6))
    m = KNNRegressor.fit(xt, y, KNNRegressorParameters(k=4, algorithm=KNNAlgorithmName.LinearSearch,
                                                       weight=KNNWeightFunction(weight)))
    got = m.predict(xq)
    idx, dist = oracle.knn_find(xt, xq, 4)
    assert np.array_equal(got, oracle.knn_regress(idx, dist, y, weight=weight))


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("k", [65, 100, 700])
def test_find_large_k(form, dtype, k):
    """LinearKNNSearch::find accepts any 1 <= k <= n (linear_search.rs:53-58):
    k beyond the split kernel's 64-entry heaps runs the FP64 kernel (shared-
    memory heaps up to its limit, then heaps in global memory)."""
    rng = np.random.default_rng(k)
    train = rng.normal(size=(2500, 9)).astype(dtype)
    q = rng.normal(size=(150, 9)).astype(dtype)
    s = LinearKNNSearch(train, form=form)
    idx, dist = s.find_batch(q, k)
    ridx, rdist = oracle.knn_find(train, q, k)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("d", [200, 1000])
def test_find_wide_rows(form, d):
    """Rows wider than the split kernel's 256-feature tiles (and, at d = 1000,
    wider than the FP64 kernel's shared-memory staging) are served."""
    rng = np.random.default_rng(d)
    train = rng.normal(size=(1500, d)).astype(np.float32)
    q = rng.normal(size=(64, d)).astype(np.float32)
    s = LinearKNNSearch(train, form=form)
    idx, dist = s.find_batch(q, 100)
    ridx, rdist = oracle.knn_find(train, q, 100)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)
    counts, ridxs, _ = s.find_radius_batch(q, float(np.median(rdist)))
    rc, rr, _ = oracle.knn_find_radius(train, q, float(np.median(rdist)))
    assert np.array_equal(counts, rc) and np.array_equal(ridxs, rr)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("weight", [0, 1])
def test_classifier_regressor_large_k(form, weight):
    """Vote and regression over 100 neighbours (the aggregation's work arrays
    in global memory)."""
    xt, yt, xq, _ = knn_blobs_f32(n_train=4000, n_query=300, d=8, classes=6, seed=3)
    m = KNNClassifier.fit(xt, yt, KNNClassifierParameters(k=100, algorithm=KNNAlgorithmName.LinearSearch,
                                                         weight=KNNWeightFunction(weight), form=form))
    idx, dist = oracle.knn_find(xt, xq, 100)
    assert np.array_equal(m.predict(xq), oracle.knn_vote(idx, dist, yt, 6, weight=weight))
    yr = yt.astype(np.float64) * 0.5
    r = KNNRegressor.fit(xt, yr, KNNRegressorParameters(k=100, algorithm=KNNAlgorithmName.LinearSearch,
                                                        weight=KNNWeightFunction(weight), form=form))
    assert np.array_equal(r.predict(xq), oracle.knn_regress(idx, dist, yr, weight=weight))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("cap", [8, 64])
def test_find_candidate_overflow(dtype, cap):
    """Split find lists each query's candidate rows (a certified superset of
    the rows the reference inserts) before the exact replay; a query with more
    candidates than its slots is served by the streaming kernel afterwards.  A
    small cap sends most (8) or some (64) queries down that path, with the same
    heaps."""
    L = _lib.load()
    rng = np.random.default_rng(cap)
    train = rng.normal(size=(4000, 24)).astype(dtype)
    q = rng.normal(size=(300, 24)).astype(dtype)
    s = LinearKNNSearch(train, form=_lib.FORM_SPLIT_BF16)
    ridx, rdist = oracle.knn_find(train, q, 10)
    try:
        _lib.check(L.sc_debug_knn_candidate_cap(cap))
        idx, dist = s.find_batch(q, 10)
    finally:
        L.sc_debug_knn_candidate_cap(0)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)
    idx, dist = s.find_batch(q, 10)
    assert np.array_equal(idx, ridx) and np.array_equal(dist, rdist)


@pytest.mark.parametrize("d", [8, 32, 100])
@pytest.mark.parametrize("cap", [0, 64])
def test_find_query_chunks(d, cap):
    """Split find runs its filter and replay over chunks of whole query tiles
    (by default as many queries as keep the candidate lists within 2 GB).
    Chunks of one tile, a ragged last chunk, and queries past the candidate
    slots in several chunks give the same heaps."""
    L = _lib.load()
    rng = np.random.default_rng(d + cap)
    train = rng.normal(size=(5000, d)).astype(np.float32)
    q = rng.normal(size=(1000, d)).astype(np.float32)
    s = LinearKNNSearch(train, form=_lib.FORM_SPLIT_BF16)
    ridx, rdist = oracle.knn_find(train, q, 10)
    try:
        _lib.check(L.sc_debug_knn_chunk_queries(1))
        _lib.check(L.sc_debug_knn_candidate_cap(cap))
        idx, dist = s.find_batch(q, 10)
    finally:
        L.sc_debug_knn_chunk_queries(0)
        L.sc_debug_knn_candidate_cap(0)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(dist, rdist)


def test_find_sorted_training_rows():
    """Training rows sorted by decreasing distance to the queries make every
    row a heap insertion: the candidate lists overflow and the streaming
    kernel serves those queries."""
    rng = np.random.default_rng(11)
    q = rng.normal(size=(40, 8)).astype(np.float32)
    t = rng.normal(size=(3000, 8)).astype(np.float32)
    order = np.argsort(-((t - q[0]) ** 2).sum(axis=1))
    train = np.ascontiguousarray(t[order])
    s = LinearKNNSearch(train, form=_lib.FORM_SPLIT_BF16)
    idx, dist = s.find_batch(q, 5)
    ridx, rdist = oracle.knn_find(train, q, 5)
    assert np.array_equal(idx, ridx) and np.array_equal(dist, rdist)
