"""Failure paths, made to happen on purpose without faulting the GPU.

- Device allocation failures are injected on the host (the library's
  allocator refuses after N allocations): every entry point returns
  SC_ERR_OOM, releases what it had allocated, and the next call works.
- A bounded wait of the split-form assignment kernel is made to run out (its
  bound set to 1 ns): the kernel stops, drains its own copies and
  tensor-core work, frees its tensor memory and reports SC_ERR_TIMEOUT; the
  GPU context stays usable and a fresh fit gives the oracle's results.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.cluster import KMeans, KMeansHandle, KMeansParameters, kmeanspp_draws
from smartcore_gb300.error import Failed
from smartcore_gb300.neighbors import LinearKNNSearch
from tests.datagen import batched_problems, blobs

pytestmark = pytest.mark.gpu


@pytest.fixture
def L():
    lib = _lib.load()
    yield lib
    lib.sc_debug_fail_alloc_after(-1)


def assert_oom(fn):
    with pytest.raises(Failed) as e:
        fn()
    assert "[status 3]" in str(e.value) and "injected" in str(e.value), str(e.value)


@pytest.mark.parametrize("form", [_lib.FORM_FP64, _lib.FORM_SPLIT_BF16], ids=["fp64", "split"])
def test_allocation_failures_release_everything(L, form):
    x, _ = blobs(20_000, 24, 10, seed=2, dtype=np.float32)
    p = KMeansParameters(k=10, max_iter=20, seed=1, form=form)
    ref = KMeans.fit(x, p)  # grows the pools once
    base = L.sc_debug_live_allocations()
    failures = 0
    for after in range(0, 40, 3):
        L.sc_debug_fail_alloc_after(after)
        try:
            km = KMeans.fit(x, p)
            assert np.array_equal(km._y, ref._y)
        except Failed as e:
            assert "[status 3]" in str(e) and "injected" in str(e), str(e)
            failures += 1
        L.sc_debug_fail_alloc_after(-1)
        assert L.sc_debug_live_allocations() == base
    assert failures > 0
    km = KMeans.fit(x, p)
    assert np.array_equal(km._y, ref._y) and np.array_equal(km.centroids, ref.centroids)


def test_allocation_failures_knn_and_batched(L):
    xt = np.random.default_rng(3).normal(size=(5000, 16)).astype(np.float32)
    q = xt[:100]
    base = L.sc_debug_live_allocations()
    L.sc_debug_fail_alloc_after(0)
    assert_oom(lambda: LinearKNNSearch(xt))
    L.sc_debug_fail_alloc_after(-1)
    assert L.sc_debug_live_allocations() == base
    s = LinearKNNSearch(xt, form=_lib.FORM_SPLIT_BF16)
    L.sc_debug_fail_alloc_after(1)
    assert_oom(lambda: s.find_batch(q, 5))
    L.sc_debug_fail_alloc_after(-1)
    idx, dist = s.find_batch(q, 5)
    ridx, rdist = oracle.knn_find(xt, q, 5)
    assert np.array_equal(idx, ridx) and np.array_equal(dist, rdist)
    s.close()
    probs = batched_problems(count=4, seed0=70)
    par = [(x, KMeansParameters(k=k, max_iter=10, seed=sd)) for x, k, sd in probs]
    base = L.sc_debug_live_allocations()
    L.sc_debug_fail_alloc_after(0)
    assert_oom(lambda: KMeans.fit_many(par))
    L.sc_debug_fail_alloc_after(-1)
    assert L.sc_debug_live_allocations() == base
    fits = KMeans.fit_many(par)
    for (x, k, sd), km in zip(probs, fits):
        assert np.array_equal(km._y, oracle.kmeans_fit(x, k, 10, seed=sd).labels)


def test_split_assignment_wait_runs_out(L):
    x, _ = blobs(50_000, 32, 16, seed=4, dtype=np.float32)
    first, u = kmeanspp_draws(len(x), 16, 7)
    h = KMeansHandle(x, form=_lib.FORM_SPLIT_BF16)
    h.seed(16, first, u)
    _lib.check(L.sc_kmeans_set_wait_limit(h.h, 1))
    it = np.zeros(1, np.int64)
    rc = L.sc_kmeans_iterate(h.h, 3, 1, _lib.ptr(it))
    assert rc == _lib.SC_ERR_TIMEOUT, (rc, _lib.last_error())
    assert "device-side check failed" in _lib.last_error()
    h.close()
    # the context is still usable: a fresh handle fits with the oracle's results
    km = KMeans.fit(x, KMeansParameters(k=16, max_iter=30, seed=7, form=_lib.FORM_SPLIT_BF16))
    ref = oracle.kmeans_fit(x, 16, 30, seed=7)
    assert np.array_equal(km._y, ref.labels) and km.iters == ref.iters
    # and the default bound restores normal steps on a handle
    h = KMeansHandle(x, form=_lib.FORM_SPLIT_BF16)
    h.seed(16, first, u)
    _lib.check(L.sc_kmeans_set_wait_limit(h.h, 1))
    _lib.check(L.sc_kmeans_set_wait_limit(h.h, 0))
    assert h.iterate(2, stop_on_converge=False) == 2
    h.close()
