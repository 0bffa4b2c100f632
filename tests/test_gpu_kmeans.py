"""GPU parity of the KMeans path against the CPU oracle (through the C ABI).

Bar: labels bit-identical, centroids within 1e-12 relative, distortion within
1e-12 relative, iteration count equal (both stop when the distortion stops
strictly decreasing, kmeans.rs:305-309).
"""
import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.cluster import KMeans, KMeansHandle, KMeansParameters, kmeanspp_draws
from smartcore_gb300.linalg import DenseMatrix
from tests.datagen import batched_problems, blobs, kmeans_small_f64

pytestmark = pytest.mark.gpu

FORMS = [pytest.param(_lib.FORM_FP64, id="fp64"), pytest.param(_lib.FORM_SPLIT_BF16, id="split")]
CENT_RTOL = 1e-12


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=-1, keepdims=True), 1e-300)
    return float((np.abs(a - b) / scale).max())


def assert_fit_parity(x, k, max_iter, seed, form):
    gpu = KMeans.fit(x, KMeansParameters(k=k, max_iter=max_iter, seed=seed, form=form))
    ref = oracle.kmeans_fit(x, k, max_iter, seed=0 if seed is None else seed)
    assert np.array_equal(gpu._y, ref.labels)
    assert np.array_equal(gpu.size, ref.sizes)
    assert rel_err(gpu.centroids, ref.centroids) <= CENT_RTOL
    # FP64 form: the distortion is the sum of the per-point FP64 distances.
    # Split form: sum ||x||^2 - 2 c.S + n ||c||^2 from exact sums, whose
    # cancellation error is a few ulps of sum ||x||^2.
    xx = float((np.asarray(x, np.float64) ** 2).sum())
    tol = 1e-12 * abs(ref.distortion) + (1e-14 * xx if form == _lib.FORM_SPLIT_BF16 else 0.0)
    assert abs(gpu._distortion - ref.distortion) <= tol
    assert gpu.iters == ref.iters
    return gpu, ref


@pytest.mark.parametrize("form", FORMS)
def test_small_f64_blobs(form):
    """Plain KMeans f64: 10,000 x 16, k=8, max_iter=100, seed 42."""
    x, _ = kmeans_small_f64()
    assert_fit_parity(x, 8, 100, 42, form)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("order", ["C", "F"])
def test_f32_layouts(form, order):
    x, _ = blobs(5000, 24, 12, seed=4, dtype=np.float32)
    assert_fit_parity(np.asarray(x, order=order), 12, 60, 7, form)


@pytest.mark.parametrize("form", FORMS)
def test_iris_fit_predict(kats, form):
    """kmeans.rs:473-505 on the GPU: predict(x) == fit labels, default params."""
    x = DenseMatrix.from_2d_array(kats["kmeans_fit_predict"]["x"])
    gpu, ref = assert_fit_parity(x.array(), 2, 100, None, form)
    p = KMeans.fit(x, KMeansParameters(form=form)).predict(x)
    assert np.array_equal(p, gpu._y)


def test_bbdtree_iris_step(kats):
    """One clustering step from the bbdtree_iris centroids (bbd_tree.rs:323-364)."""
    kat = kats["bbdtree_iris"]
    x = np.array(kat["x"])
    h = KMeansHandle(x)
    h.set_centroids(np.array(kat["centroids"]))
    assert h.iterate(1) == 1
    cent, sizes, labels, dist, _ = h.get()
    r_dist, r_sums, r_counts, r_memb = oracle.bbd_clustering(x, np.array(kat["centroids"]))
    assert np.array_equal(labels, r_memb)
    assert np.array_equal(sizes, r_counts)
    assert abs(dist - r_dist) <= 1e-12 * r_dist
    for name, want, tol in kat["expect_close"]:
        if name == "dist":
            assert abs(dist - want) < tol
    assert rel_err(cent, r_sums / r_counts[:, None]) <= CENT_RTOL
    h.close()


# (n, d, blobs, k): d % 4 == 0 f32 rows take the 16-byte staged copies, other
# f32 rows up to d = 128 the 4-byte ones, f64 rows and d > 128 the plain
# kernel; well separated blobs let most rows skip the distance (far test).
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n,d,c,k", [(20_000, 8, 16, 16), (30_000, 7, 40, 48), (20_000, 64, 64, 64),
                                     (9_000, 100, 30, 40), (5_000, 200, 8, 12), (3_001, 1, 5, 9)])
def test_kmeanspp_labels(form, dtype, n, d, c, k):
    # the split form's update also bounds rows through their BF16 high halves;
    # a split-form handle of d > 128 runs the FP64 form
    x, _ = blobs(n, d, c, seed=12, dtype=dtype)
    first, u = kmeanspp_draws(len(x), k, 5)
    h = KMeansHandle(x, form=form)
    h.seed(k, first, u)
    _, sizes, labels, _, _ = h.get()
    y, _ = oracle.kmeanspp(x, k, first, u)
    assert np.array_equal(labels, y)
    assert np.array_equal(sizes, np.bincount(y, minlength=k))
    h.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_kmeanspp_uncertified_draw_replays(dtype):
    """A cutoff a hair below the total lands inside the rounding band of the
    parallel prefix: the draw is resolved by the exact sequential replay."""
    rng = np.random.default_rng(4)
    x = rng.normal(0.0, 1e-6, size=(2000, 4))
    x[0] = 1e3
    x = x.astype(dtype)
    u = np.array([1.0 - 2.0 ** -53, 0.3, 0.999, 0.5, 0.01])
    h = KMeansHandle(x)
    h.seed(6, 1, u)
    _, _, labels, _, _ = h.get()
    assert h.stats()[1] >= 1
    y, _ = oracle.kmeanspp(x, 6, 1, u)
    assert np.array_equal(labels, y)
    h.close()


@pytest.mark.parametrize("form", FORMS)
def test_predict_matches_oracle(form):
    x, _ = blobs(7000, 20, 9, seed=21, dtype=np.float32)
    c = np.random.default_rng(3).normal(size=(9, 20)) * 5
    km = KMeans(9, None, None, 0.0, c, 0, form)
    assert np.array_equal(km.predict(x), oracle.kmeans_predict(x, c))


def test_predict_ties_lowest_index():
    # integer grid: many exact ties between duplicated centroids
    x = np.random.default_rng(0).integers(-3, 4, size=(3000, 4)).astype(np.float64)
    c = np.array([[0, 0, 0, 0], [1, 1, 0, 0], [0, 0, 0, 0], [1, 1, 0, 0], [2, 2, 2, 2.0]])
    km = KMeans(5, None, None, 0.0, c, 0, _lib.FORM_FP64)
    got = km.predict(x)
    assert np.array_equal(got, oracle.kmeans_predict(x, c))
    assert not np.any(got == 2) and not np.any(got == 3)


@pytest.mark.parametrize("form", FORMS)
def test_plain_kmeans_10k_x16_k8(form):
    # the plain-KMeans workload: 8 blobs, 10,000 x 16 f64, k = 8, max_iter = 100, seed 42
    x, _ = kmeans_small_f64(42)
    assert_fit_parity(x, 8, 100, 42, form)


@pytest.mark.parametrize("form", FORMS)
def test_independent_small_problems(form):
    # the first 8 of the 512-problem workload: n log-uniform in [1e3, 1e5],
    # d in {8, 16, 32, 64}, k in [4, 64], max_iter = 30, f32
    for x, k, seed in batched_problems(count=8):
        assert_fit_parity(x, k, 30, seed, form)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n,d,k", [(20000, 64, 300), (12000, 128, 1000), (8000, 128, 2048), (6000, 16, 500)])
def test_predict_many_centroids(form, n, d, k):
    # more centroids than stay resident in shared memory: streamed in blocks of 128
    x, _ = blobs(n, d, 64, seed=n + k, dtype=np.float32, box=(-50.0, 50.0), std=2.0)
    c = np.ascontiguousarray(x[np.random.default_rng(k).choice(n, k, replace=False)], np.float64)
    km = KMeans(k, None, None, 0.0, c, 0, form)
    assert np.array_equal(km.predict(x), oracle.kmeans_predict(x, c))


@pytest.mark.parametrize("form", FORMS)
def test_fit_many_centroids_d128(form):
    x, _ = blobs(10000, 128, 40, seed=11, dtype=np.float32, box=(-50.0, 50.0), std=2.0)
    assert_fit_parity(x, 300, 4, 5, form)


@pytest.mark.parametrize("form", FORMS)
def test_predict_many_tied_candidates(form):
    # 40 centroids drawn from the 16 vectors +-e_t (duplicates included), all
    # of norm 1: points at the origin tie with every centroid exactly, points
    # near it are near ties with many.  Exercises the split form's fallback
    # for rows with more candidates than one list holds.
    rng = np.random.default_rng(11)
    basis = np.concatenate([np.eye(8), -np.eye(8)])
    c = basis[rng.integers(0, 16, size=40)]
    x = np.concatenate([np.zeros((300, 8)), rng.normal(scale=1e-7, size=(700, 8)), rng.normal(size=(1000, 8))])
    for dt in (np.float64, np.float32):
        xd = x.astype(dt)
        km = KMeans(40, None, None, 0.0, c, 0, form)
        got = km.predict(xd)
        assert np.array_equal(got, oracle.kmeans_predict(xd, c))
        assert np.all(got[:300] == 0)


@pytest.mark.parametrize("form", FORMS)
def test_edge_shapes(form):
    x, _ = blobs(64, 3, 4, seed=2)
    assert_fit_parity(x, 64, 10, 1, form)  # k == n
    x1 = np.random.default_rng(1).normal(size=(257, 1))
    assert_fit_parity(x1, 3, 20, 9, form)  # d == 1, n not a multiple of any tile
    xd = np.repeat(np.random.default_rng(2).normal(size=(10, 5)), 30, axis=0)
    assert_fit_parity(xd, 4, 20, 3, form)  # duplicated points


def test_throughput_mode_runs_all_iterations():
    x, _ = blobs(4000, 8, 4, seed=5, dtype=np.float32)
    h = KMeansHandle(x)
    first, u = kmeanspp_draws(len(x), 4, 0)
    h.seed(4, first, u)
    assert h.iterate(17, stop_on_converge=False) == 17
    h.close()


@pytest.mark.parametrize("form", FORMS)
def test_values_below_the_sum_grid(form):
    """f32 points whose features span ~60 binades: the tiny ones fall outside
    the packed fixed-point form of the centroid sums and take the exact
    conversion from f32 (subnormals included)."""
    x, _ = blobs(6000, 8, 5, seed=31, dtype=np.float32)
    x[:, 3] *= np.float32(1e-18)
    x[::7, 5] = np.float32(3e-39)  # subnormal
    x = np.ascontiguousarray(x)
    assert_fit_parity(x, 5, 20, 6, form)


@pytest.mark.parametrize("form", FORMS)
def test_serde_round_trip(kats, form):
    """kmeans.rs:512-546: a fitted model survives serialisation unchanged
    (PartialEq), in the reference's serde layout."""
    import json
    x = np.array(kats["kmeans_fit_predict"]["x"], np.float32)
    km = KMeans.fit(x, KMeansParameters(k=2, max_iter=100, seed=3, form=form))
    text = km.to_json()
    assert list(json.loads(text).keys()) == list(KMeans._SERDE_FIELDS)
    back = KMeans.from_json(text, form=form)
    assert back == km
    assert np.array_equal(back.predict(x), km.predict(x))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_split_form_wide_rows_fit(dtype):
    """KMeans::fit on d = 200 asked for in the split form: rows wider than its
    128-feature tiles run the FP64 form, with the oracle's results."""
    x, _ = blobs(4000, 200, 10, seed=21, dtype=dtype)
    assert_fit_parity(x, 10, 30, 3, _lib.FORM_SPLIT_BF16)
    km = KMeans.fit(x, KMeansParameters(k=10, max_iter=30, seed=3, form=_lib.FORM_SPLIT_BF16))
    assert np.array_equal(km.predict(x), km._y)


@pytest.mark.parametrize("form", FORMS)
def test_incremental_sums_equal_full_pass(form):
    """Steps whose sums move only the relabelled rows (few rows change label)
    give the same bits as steps that sum every row: one handle iterates on
    its own, the other is re-set to the same centroids before each step
    (which forces the full pass)."""
    x, _ = blobs(60_000, 24, 20, seed=8, dtype=np.float32)
    c0 = np.ascontiguousarray(x[np.random.default_rng(3).choice(len(x), 20, replace=False)], np.float64)
    a = KMeansHandle(x, form=form)
    b = KMeansHandle(x, form=form)
    a.set_centroids(c0)
    inc = 0
    cent = c0
    for step in range(12):
        b.set_centroids(cent)
        a.iterate(1, stop_on_converge=False)
        inc += a.incremental_steps()
        b.iterate(1, stop_on_converge=False)
        ca, sa, la, da, _ = a.get()
        cb, sb, lb, db, _ = b.get()
        assert np.array_equal(la, lb) and np.array_equal(sa, sb)
        assert np.array_equal(ca, cb)
        assert da == db
        assert b.incremental_steps() == 0
        cent = ca
    assert inc >= 6  # the later steps move few rows
    a.close()
    b.close()


def replay_cases():
    rng = np.random.default_rng(11)
    # rows spanning 32 decades: the sequential f64 sum absorbs the small terms
    wide = rng.normal(size=(40_000, 3)) * (10.0 ** rng.uniform(-8, 8, size=(40_000, 1)))
    # integer rows far apart: squared distances are integers whose running sum
    # passes 2^53, where additions round and ties go to even
    grid = rng.integers(-2 ** 12, 2 ** 12, size=(60_000, 4)).astype(np.float64) * 2.0 ** 10
    u = np.array([1.0 - 2.0 ** -53, 1.0 - 2.0 ** -52, 0.5, 1.0 - 2.0 ** -50, 0.25, 1.0 - 2.0 ** -53, 0.75])
    return [(wide, u), (grid, u)]


@pytest.mark.parametrize("case", [0, 1], ids=["wide_span", "integer_grid"])
def test_kmeanspp_exact_replay_adversarial(case):
    """Draws whose cutoff is inside the rounding band take the CTA-wide exact
    reproduction of the sequential sum and prefix (binade by binade, ties to
    even): the chosen seeds equal the oracle's sequential loop."""
    x, u = replay_cases()[case]
    k = len(u) + 1
    h = KMeansHandle(x)
    h.seed(k, 3, u)
    _, _, labels, _, _ = h.get()
    assert h.stats()[1] >= 2
    y, chosen = oracle.kmeanspp(x, k, 3, u)
    assert np.array_equal(labels, y)
    h.close()


def test_batched_exact_replay_adversarial():
    """The batched selection takes the same exact reproduction: problems with
    hand-set draws whose cutoffs fall inside the rounding band."""
    import ctypes as C
    L = _lib.load()
    cases = replay_cases()
    arr = (_lib.KMeansProblem * len(cases))()
    keep, outs = [], []
    for i, (x, u) in enumerate(cases):
        x = np.ascontiguousarray(x)
        k = len(u) + 1
        n, d = x.shape
        labels = np.zeros(n, np.int64)
        cent = np.zeros((k, d))
        iters = np.zeros(1, np.int64)
        keep += [x, u, labels, cent, iters]
        outs.append((x, u, labels, cent, iters))
        q = arr[i]
        q.x, q.layout, q.n, q.d, q.ld = x.ctypes.data, _lib.ROW_MAJOR, n, d, d
        q.k, q.max_iter, q.first_index, q.uniforms = k, 5, 3, u.ctypes.data
        q.labels_out, q.centroids_out, q.iters_out = labels.ctypes.data, cent.ctypes.data, iters.ctypes.data
    _lib.check(L.sc_kmeans_fit_batched(C.cast(arr, C.c_void_p), len(cases), _lib.F64, _lib.FORM_FP64))
    assert sum(arr[i].pp_replays for i in range(len(cases))) >= 2
    for x, u, labels, cent, iters in outs:
        ref = oracle.kmeans_fit(x, len(u) + 1, 5, first=3, uniforms=u)
        assert np.array_equal(labels, ref.labels)
        assert int(iters[0]) == ref.iters
