"""CPU-side checks of the C ABI: the library builds, loads and exports every
symbol the header declares; argument validation answers with the
reference's messages without touching a GPU; the host-side rand 0.8
restatement agrees with the oracle's independent one."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib, build
from smartcore_gb300.cluster import KMeans, KMeansParameters, kmeanspp_draws
from smartcore_gb300.error import Failed, FailedError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def header_symbols():
    with open(os.path.join(ROOT, "include", "smartcore_gb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sc_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(L):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.SIGNATURES), set(syms) ^ set(_lib.SIGNATURES)


def test_version_and_device(L):
    assert L.sc_abi_version() == 100
    assert L.sc_device_ok() in (0, 1)


def test_kmeans_fit_validation_messages(L):
    x = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    out = np.zeros(16)
    for k, msg in ((0, "invalid number of clusters: 0"), (1, "invalid number of clusters: 1")):
        rc = L.sc_kmeans_fit(_lib.ptr(x), _lib.F64, _lib.ROW_MAJOR, 2, 3, 3, k, 100, 0, _lib.ptr(out), 0,
                             _lib.ptr(out), _lib.ptr(out), _lib.ptr(out), _lib.ptr(out), _lib.ptr(out))
        assert rc == _lib.SC_ERR_INVALID
        assert _lib.last_error() == msg
    rc = L.sc_kmeans_fit(_lib.ptr(x), _lib.F64, _lib.ROW_MAJOR, 2, 3, 3, 2, 0, 0, _lib.ptr(out), 0,
                         _lib.ptr(out), _lib.ptr(out), _lib.ptr(out), _lib.ptr(out), _lib.ptr(out))
    assert rc == _lib.SC_ERR_INVALID
    assert _lib.last_error() == "invalid maximum number of iterations: 0"


def test_python_mirror_messages():
    x = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]])
    with pytest.raises(Failed) as e:
        KMeans.fit(x, KMeansParameters().with_k(1))
    assert str(e.value) == "Fit failed: invalid number of clusters: 1"  # kmeans.rs:434-442
    assert e.value.error() == FailedError.FitFailed


def test_bad_arguments_rejected(L):
    h = C.c_void_p()
    x = np.zeros((4, 3))
    assert L.sc_kmeans_create(_lib.ptr(x), 7, 0, 0, 4, 3, 3, 0, C.byref(h)) == _lib.SC_ERR_INVALID
    assert L.sc_kmeans_create(_lib.ptr(x), 1, 0, 0, 4, 3, 2, 0, C.byref(h)) == _lib.SC_ERR_INVALID
    assert "leading dimension" in _lib.last_error()
    assert L.sc_knn_create(None, 1, 0, 0, 4, 3, 3, C.byref(h)) == _lib.SC_ERR_INVALID


@pytest.mark.parametrize("rng", [_lib.RNG_SMALL, _lib.RNG_STD])
@pytest.mark.parametrize("n,k,seed", [(10, 3, 0), (10_000, 8, 42), (1_000_000, 256, 3), (7, 2, 2**63 + 5)])
def test_draws_match_oracle(rng, n, k, seed):
    first, u = kmeanspp_draws(n, k, seed, rng)
    of, ou = oracle.kmeanspp_draws(n, k, seed, rng)
    assert first == of
    assert np.array_equal(u, ou)


def test_draws_reject_empty(L):
    a = np.zeros(2, np.int64)
    assert L.sc_kmeanspp_draws(0, 0, 0, 2, _lib.ptr(a), _lib.ptr(a)) == _lib.SC_ERR_INVALID


def test_null_handles_rejected_before_any_device_call(L):
    """The entry points added after find check their handle and arguments on
    the host first; these calls touch no GPU."""
    out = np.zeros(4, np.int64)
    dist = np.zeros(4)
    k = np.zeros(1, np.int64)
    assert L.sc_dbscan_fit(None, 0.5, 5, 1, _lib.ptr(out), _lib.ptr(k)) == _lib.SC_ERR_INVALID
    assert L.sc_dbscan_predict(None, None, 0, 0, 0, 0, 0.5, 1, None, 0, None) == _lib.SC_ERR_INVALID
    assert L.sc_fastpair(None, _lib.ptr(out), _lib.ptr(dist), None, None) == _lib.SC_ERR_INVALID
    assert L.sc_knn_find_radius(None, None, 0, 0, 0, 0, 1.0, 1, None, 0, None, None, None) == _lib.SC_ERR_INVALID
    assert "null handle" in _lib.last_error()


def test_batched_validation_before_any_device_call(L):
    """sc_kmeans_fit_batched validates every problem first, with KMeans::fit's
    messages prefixed by the problem's index; an empty batch is a no-op."""
    x = np.zeros((5, 2))
    u = np.zeros(4)
    arr = (_lib.KMeansProblem * 2)()
    for i, k in enumerate((3, 1)):
        q = arr[i]
        q.x, q.layout, q.n, q.d, q.ld = x.ctypes.data, _lib.ROW_MAJOR, 5, 2, 2
        q.k, q.max_iter, q.first_index, q.uniforms = k, 10, 0, u.ctypes.data
    rc = L.sc_kmeans_fit_batched(C.cast(arr, C.c_void_p), 2, _lib.F64, _lib.FORM_FP64)
    assert rc == _lib.SC_ERR_INVALID
    assert _lib.last_error() == "problem 1: invalid number of clusters: 1"
    arr[1].k, arr[1].max_iter = 2, 0
    assert L.sc_kmeans_fit_batched(C.cast(arr, C.c_void_p), 2, _lib.F64, _lib.FORM_FP64) == _lib.SC_ERR_INVALID
    assert _lib.last_error() == "problem 1: invalid maximum number of iterations: 0"
    assert L.sc_kmeans_fit_batched(None, 0, _lib.F32, _lib.FORM_FP64) == _lib.SC_OK


def test_batch_tune_rejects_foreign_files(L, tmp_path):
    p = tmp_path / "t.txt"
    p.write_text("not a table\n")
    assert L.sc_batch_tune_load(str(p).encode()) == _lib.SC_ERR_INVALID
    assert L.sc_batch_tune_load(str(tmp_path / "missing.txt").encode()) == _lib.SC_ERR_INVALID
    assert L.sc_batch_tune_get(200, 5, None, None) == _lib.SC_ERR_INVALID


def test_batch_variant_override(L):
    """sc_debug_batch_variant accepts the assignment variants (2, 4, 8) and -1
    (the tuning table's choice), rejects anything else, and is what
    sc_batch_tune_get reports while it is set."""
    assert L.sc_debug_batch_variant(3) == _lib.SC_ERR_INVALID
    assert "unknown batched assignment variant 3" in _lib.last_error()
    cu, rows = np.zeros(1, np.int32), np.zeros(1, np.int32)
    try:
        for v in (2, 4, 8):
            _lib.check(L.sc_debug_batch_variant(v))
            _lib.check(L.sc_batch_tune_get(32, 16, _lib.ptr(cu), _lib.ptr(rows)))
            assert int(cu[0]) == v and int(rows[0]) in (1024, 2048, 4096)
    finally:
        _lib.check(L.sc_debug_batch_variant(-1))


def test_problem_record_matches_the_c_struct():
    """KMeans.fit_many fills the problem table as NumPy columns: the record's
    fields sit where sc_kmeans_problem's do."""
    from smartcore_gb300.cluster import PROBLEM_DTYPE
    assert PROBLEM_DTYPE.itemsize == C.sizeof(_lib.KMeansProblem)
    for name in PROBLEM_DTYPE.names:
        assert PROBLEM_DTYPE.fields[name][1] == getattr(_lib.KMeansProblem, name).offset


def test_fastpair_neighbour_map():
    """FastPair.distances reads like the reference's HashMap of
    PairwiseDistance, each entry built from the neighbour arrays on access."""
    from smartcore_gb300.neighbors import PairwiseDistance, _NeighbourMap
    m = _NeighbourMap(np.array([2, 2, 2]), np.array([0.25, 1.5, 3.4e38]))
    assert len(m) == 3 and list(m) == [0, 1, 2]
    assert m[1] == PairwiseDistance(1, 2, 1.5)
    assert dict(m)[2] == PairwiseDistance(2, 2, 3.4e38)
    with pytest.raises(KeyError):
        m[3]


def test_find_radius_batch_sizing():
    """find_radius_batch sizes its first output from the previous call's rows
    per query; when the library reports more rows than that (SC_ERR_INVALID
    with the total set), it calls once more with the exact size.  A fake
    library with fixed per-query counts stands in for the device."""
    from smartcore_gb300.neighbors import LinearKNNSearch

    class Fake:
        def __init__(self, per_query):
            self.per_query, self.calls = per_query, []

        def sc_knn_find_radius(self, h, q, lay, mem, m, ld, radius, form, counts, cap, idx, dist, total):
            self.calls.append(cap)
            c = np.ctypeslib.as_array(C.cast(counts, C.POINTER(C.c_int64)), (m,))
            c[:] = self.per_query
            t = self.per_query * m
            np.ctypeslib.as_array(C.cast(total, C.POINTER(C.c_int64)), (1,))[0] = t
            if cap < t:
                return _lib.SC_ERR_INVALID
            out = np.ctypeslib.as_array(C.cast(idx, C.POINTER(C.c_int64)), (t,))
            out[:] = np.tile(np.arange(self.per_query), m)
            np.ctypeslib.as_array(C.cast(dist, C.POINTER(C.c_double)), (t,))[:] = 0.5
            return _lib.SC_OK

    s = object.__new__(LinearKNNSearch)
    s.dtype, s.n, s.d, s.h, s.form, s._per_query = np.dtype(np.float32), 10, 3, None, 1, 64.0
    q = np.zeros((40, 3), np.float32)
    s._L = Fake(200)  # 8,000 rows > the first size (1.25 * 64 * 40 = 3,200): two calls
    counts, idx, dist = s.find_radius_batch(q, 1.0)
    assert s._L.calls == [3200, 8000]
    assert counts.tolist() == [200] * 40 and len(idx) == 8000 and idx[:3].tolist() == [0, 1, 2]
    assert s._per_query == 200.0
    s._L = Fake(150)  # now sized from 200 rows per query: one call
    counts, idx, dist = s.find_radius_batch(q, 1.0)
    assert s._L.calls == [10000] and len(idx) == 6000 and np.all(dist == 0.5)
    s._L = Fake(0)  # no rows
    counts, idx, dist = s.find_radius_batch(q, 1.0)
    assert len(idx) == 0 and counts.sum() == 0


def test_fit_many_problem_table(monkeypatch):
    """KMeans.fit_many fills one sc_kmeans_problem per fit (shape, layout,
    k-means++ draws, and each output pointer at the problem's slice of the
    shared output arrays).  A fake library checks the table and writes each
    problem's index into its outputs."""
    from smartcore_gb300 import cluster

    rng = np.random.default_rng(3)
    shapes = [(50, 4, 3), (7, 2, 5), (120, 9, 2)]
    xs = [rng.normal(size=(n, d)).astype(np.float32) for n, d, _ in shapes]
    xs[1] = np.asfortranarray(xs[1])
    seen = {}

    real = _lib.load()

    class Fake:
        def __getattr__(self, name):
            return getattr(real, name)

        def sc_kmeans_fit_batched(self, ptr, m, dt, form):
            arr = (_lib.KMeansProblem * m).from_address(ptr)
            for i in range(m):
                q = arr[i]
                n, d, k = shapes[i]
                assert (q.n, q.d, q.k, q.max_iter) == (n, d, k, 9)
                assert (q.layout, q.ld) == ((_lib.COL_MAJOR, n) if i == 1 else (_lib.ROW_MAJOR, d))
                first, u = kmeanspp_draws(n, k, 100 + i)
                got = np.ctypeslib.as_array((C.c_double * (k - 1)).from_address(q.uniforms))
                assert q.first_index == first and np.array_equal(got, u)
                for f, cnt, ct in (("labels_out", n, C.c_int64), ("sizes_out", k, C.c_int64),
                                   ("centroids_out", k * d, C.c_double), ("distortion_out", 1, C.c_double),
                                   ("iters_out", 1, C.c_int64)):
                    np.ctypeslib.as_array((ct * cnt).from_address(getattr(q, f)))[:] = i
                q.rescored, q.pp_replays = 10 + i, 20 + i
            seen["m"] = m
            return _lib.SC_OK

    monkeypatch.setattr(cluster._lib, "load", lambda: Fake())
    stats = []
    fits = cluster.KMeans.fit_many([(x, KMeansParameters(k=k, max_iter=9, seed=100 + i))
                                    for i, (x, (_, _, k)) in enumerate(zip(xs, shapes))], stats=stats)
    assert seen["m"] == 3 and stats == [(10, 20), (11, 21), (12, 22)]
    for i, (km, (n, d, k)) in enumerate(zip(fits, shapes)):
        assert km._y.shape == (n,) and np.all(km._y == i)
        assert km.centroids.shape == (k, d) and np.all(km.centroids == i)
        assert km.size.shape == (k,) and np.all(km.size == i)
        assert km.iters == i and km._distortion == float(i)
