"""GPU parity of the batched KMeans::fit (sc_kmeans_fit_batched) against the
CPU oracle and against single-problem fits.

Bar, per problem: labels, sizes and iteration count equal to the oracle's
KMeans::fit (src/cluster/kmeans.rs:254-323), centroids within 1e-12
relative, distortion within 1e-12 relative plus the identity's cancellation
term 1e-14 sum ||x||^2 (the batched distortion is sum ||x||^2 - 2 c.S +
n ||c||^2 from exact sums).
"""
import multiprocessing as mp
import os
import tempfile

import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.cluster import KMeans, KMeansParameters, batch_tune, batch_variant
from tests.datagen import batched_problems, blobs
from tests.oracle_jobs import fit_batched_problem

pytestmark = pytest.mark.gpu

CENT_RTOL = 1e-12


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=-1, keepdims=True), 1e-300)
    with np.errstate(invalid="ignore"):
        e = np.abs(a - b) / scale
    both_nan = np.isnan(a) & np.isnan(b)
    return float(np.where(both_nan, 0.0, e).max())


def check_against_oracle(x, km, labels, sizes, cent, iters, dist, iters_slack=0):
    assert np.array_equal(km._y, labels)
    assert np.array_equal(km.size, sizes)
    assert abs(km.iters - iters) <= iters_slack
    assert rel_err(km.centroids, cent) <= CENT_RTOL
    xx = float((np.asarray(x, np.float64) ** 2).sum())
    assert abs(km._distortion - dist) <= 1e-12 * abs(dist) + 1e-14 * xx


def test_512_problems_match_oracle():
    """The batched k-means workload (512 problems, n log-uniform in [1e3,
    1e5], d in {8, 16, 32, 64}, k in [4, 64], max_iter 30) in one call, every
    problem against the oracle (a spawn pool of CPU workers)."""
    count, max_iter = 512, 30
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(16, os.cpu_count() or 1)) as pool:
        jobs = pool.imap_unordered(fit_batched_problem, [(i, count, max_iter) for i in range(count)], chunksize=4)
        probs = batched_problems(count=count)
        stats = []
        fits = KMeans.fit_many([(x, KMeansParameters(k=k, max_iter=max_iter, seed=s)) for x, k, s in probs],
                               stats=stats)
        for i, labels, sizes, cent, iters, dist in jobs:
            check_against_oracle(probs[i][0], fits[i], labels, sizes, cent, iters, dist)
    assert sum(r for r, _ in stats) < 0.01 * sum(len(p[0]) for p in probs) * max_iter


def test_batched_equals_single_fits():
    """Each problem's result equals KMeans.fit of that problem alone (FP64
    form): labels, sizes, iterations; centroids to the rounding of the sums."""
    probs = batched_problems(count=24, seed0=900)
    fits = KMeans.fit_many([(x, KMeansParameters(k=k, max_iter=40, seed=s)) for x, k, s in probs])
    for (x, k, s), km in zip(probs, fits):
        one = KMeans.fit(x, KMeansParameters(k=k, max_iter=40, seed=s, form=_lib.FORM_FP64))
        assert np.array_equal(km._y, one._y)
        assert np.array_equal(km.size, one.size)
        assert km.iters == one.iters
        assert rel_err(km.centroids, one.centroids) <= 1e-14


def edge_problems(dtype):
    rng = np.random.default_rng(5)
    out = []
    for n, d, k, it, seed in [(500, 1, 2, 50, 1), (777, 3, 5, 30, 2), (1500, 5, 17, 30, 3), (2049, 13, 33, 20, 4),
                              (900, 50, 100, 15, 5), (4100, 64, 128, 10, 6), (300, 7, 64, 25, 7),
                              (3000, 16, 2, 1, 8), (5000, 8, 9, 100, 9)]:
        x, _ = blobs(n, d, max(2, k // 2), seed=seed, dtype=dtype)
        out.append((x, KMeansParameters(k=k, max_iter=it, seed=seed)))
    # duplicated points: k-means++ picks equal rows, empty clusters keep NaN
    # centroids.  The reference's initial means of 50 equal f64 rows carry the
    # rounding of its running f64 sum (a distortion of ~1e-28 in its first
    # step) where the exact sums give the rows themselves, so its break can
    # come one iteration later; labels, sizes and centroids agree.
    base = rng.normal(size=(6, 4)).astype(dtype)
    out.append((np.ascontiguousarray(np.repeat(base, 50, axis=0)), KMeansParameters(k=9, max_iter=20, seed=11)))
    # k = n
    xs, _ = blobs(12, 6, 3, seed=12, dtype=dtype)
    out.append((xs, KMeansParameters(k=12, max_iter=10, seed=12)))
    # column-major
    xf, _ = blobs(1200, 10, 6, seed=13, dtype=dtype)
    out.append((np.asfortranarray(xf), KMeansParameters(k=6, max_iter=30, seed=13)))
    # beyond the batched kernels' limits: served one by one
    xw, _ = blobs(800, 100, 5, seed=14, dtype=dtype)
    out.append((xw, KMeansParameters(k=5, max_iter=20, seed=14)))
    xk, _ = blobs(1000, 4, 80, seed=15, dtype=dtype)
    out.append((xk, KMeansParameters(k=200, max_iter=10, seed=15)))
    return out


@pytest.fixture
def force_variant():
    L = _lib.load()
    yield lambda v: _lib.check(L.sc_debug_batch_variant(v))
    L.sc_debug_batch_variant(-1)


@pytest.mark.parametrize("variant", [-1, 2], ids=["tuned", "cu2"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_edge_problems_match_oracle(dtype, variant, force_variant):
    probs = edge_problems(dtype)
    force_variant(variant)
    fits = KMeans.fit_many(probs)
    for i, ((x, p), km) in enumerate(zip(probs, fits)):
        r = oracle.kmeans_fit(x, p.k, p.max_iter, seed=p.seed)
        duplicated = i == 9
        check_against_oracle(x, km, r.labels, r.sizes, r.centroids, r.iters, r.distortion,
                             iters_slack=1 if duplicated else 0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_assignment_variants_agree(dtype, force_variant):
    """The assignment variants (2, 4 or 8 centroids per inner pass) score every
    (row, centroid) pair in the same order, so whole fits agree bit for bit:
    labels, sizes, iterations, centroids, distortion and re-scored rows, for
    every width class and k up to 128."""
    probs = batched_problems(count=80, seed0=300, n_range=(300, 20_000))
    probs += batched_problems(count=16, seed0=400, n_range=(300, 20_000), ds=(3, 13, 50, 64), k_range=(65, 128))
    par = [(x.astype(dtype), KMeansParameters(k=k, max_iter=12, seed=s)) for x, k, s in probs]
    out = {}
    for v in (2, 4, 8):
        force_variant(v)
        stats = []
        out[v] = (KMeans.fit_many(par, stats=stats), stats)
    for v in (4, 8):
        for a, b in zip(out[2][0], out[v][0]):
            assert np.array_equal(a._y, b._y) and np.array_equal(a.size, b.size) and a.iters == b.iters
            assert np.array_equal(a.centroids, b.centroids, equal_nan=True)
            assert a._distortion == b._distortion
        assert out[2][1] == out[v][1]


def test_pinned_host_rows():
    """Rows in pinned host memory are read by the device in place (one gather
    kernel for all of them); the fits equal those from pageable copies of the
    same rows, in both element types, with misaligned and column-major
    inputs in the same call taking the copy path."""
    torch = pytest.importorskip("torch")
    probs = batched_problems(count=24, seed0=500, n_range=(500, 20_000))
    for dt in (np.float32, np.float64):
        xs = [np.ascontiguousarray(x.astype(dt)) for x, _, _ in probs]
        pinned = [torch.from_numpy(x).pin_memory().numpy() for x in xs]
        # a pinned buffer offset by one element (not 16-byte aligned) and a column-major one
        big = torch.from_numpy(np.concatenate([np.zeros(1, dt), xs[1].ravel()])).pin_memory().numpy()
        pinned[1] = big[1:].reshape(xs[1].shape)
        pinned[2] = np.asfortranarray(xs[2])
        par_p = [(x, KMeansParameters(k=k, max_iter=15, seed=s)) for x, (_, k, s) in zip(pinned, probs)]
        par_h = [(x, KMeansParameters(k=k, max_iter=15, seed=s)) for x, (_, k, s) in zip(xs, probs)]
        for a, b in zip(KMeans.fit_many(par_p), KMeans.fit_many(par_h)):
            assert np.array_equal(a._y, b._y) and np.array_equal(a.size, b.size) and a.iters == b.iters
            assert np.array_equal(a.centroids, b.centroids, equal_nan=True)


@pytest.mark.parametrize("bad", [np.nan, np.inf], ids=["nan", "inf"])
def test_non_finite_rows_rejected(bad):
    """A problem with a non-finite value fails the whole call with the
    problem's index (the check runs on the device scan of max |x|); the next
    call works."""
    probs = batched_problems(count=6, seed0=80, n_range=(500, 5_000))
    par = [(x.copy(), KMeansParameters(k=k, max_iter=10, seed=s)) for x, k, s in probs]
    par[3][0][7, 1] = bad
    from smartcore_gb300.error import Failed
    with pytest.raises(Failed) as e:
        KMeans.fit_many(par)
    assert "problem 3: x contains NaN or infinity" in str(e.value)
    par[3][0][7, 1] = 0.0
    fits = KMeans.fit_many(par)
    r = oracle.kmeans_fit(par[3][0], par[3][1].k, 10, seed=par[3][1].seed)
    assert np.array_equal(fits[3]._y, r.labels)


def test_validation_writes_nothing():
    x, _ = blobs(100, 4, 3, seed=1, dtype=np.float32)
    from smartcore_gb300.error import Failed
    with pytest.raises(Failed) as e:
        KMeans.fit_many([(x, KMeansParameters(k=3)), (x, KMeansParameters(k=1))])
    assert "invalid number of clusters: 1" in str(e.value)


def test_tuner_table_round_trip():
    """The tuner measures every (d class, k class), writes its table, and a
    load of that file gives the same choices; the batched fit then uses them."""
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "tune.txt")
        batch_tune(path, force=True)
        chosen = {(d, k): batch_variant(d, k) for d in (8, 16, 32, 64) for k in (8, 16, 32, 64, 128)}
        for cu, rows in chosen.values():
            assert cu in (2, 4, 8) and rows in (1024, 2048, 4096)
        with open(path) as f:
            lines = f.read().splitlines()
        assert lines[0].startswith("smartcore_gb300") and len(lines) == 22
        batch_tune(path)  # loads the file
        assert {(d, k): batch_variant(d, k) for d, k in chosen} == chosen
    probs = batched_problems(count=6, seed0=50)
    fits = KMeans.fit_many([(x, KMeansParameters(k=k, max_iter=30, seed=s)) for x, k, s in probs])
    for (x, k, s), km in zip(probs, fits):
        r = oracle.kmeans_fit(x, k, 30, seed=s)
        check_against_oracle(x, km, r.labels, r.sizes, r.centroids, r.iters, r.distortion)
