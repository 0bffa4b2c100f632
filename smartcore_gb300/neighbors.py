"""Brute-force kNN on the GPU with smartcore's API.

Mirrors LinearKNNSearch (src/algorithm/neighbour/linear_search.rs),
KNNClassifier (src/neighbors/knn_classifier.rs) and KNNRegressor
(src/neighbors/knn_regressor.rs).  find() returns, per query, the
reference's heap array in its own order; the classifier vote and the
regressor mean run on the device in that order.
"""
from __future__ import annotations

import ctypes as C
import enum
from collections.abc import Mapping
from dataclasses import dataclass

import numpy as np

from . import _lib
from .error import Failed, FailedError
from .linalg import as_matrix, layout_of


class KNNAlgorithmName(enum.Enum):
    """src/algorithm/neighbour/mod.rs:53-59.  Both names are served by the
    GPU brute-force search: it returns the exact k nearest neighbours, which
    is also what the cover tree returns (only the order of exact ties inside
    the returned set can differ from a cover-tree search)."""
    LinearSearch = 0
    CoverTree = 1


class KNNWeightFunction(enum.IntEnum):
    """src/neighbors/mod.rs:53-59."""
    Uniform = 0
    Distance = 1


class LinearKNNSearch:
    """Training rows resident on the device (sc_knn handle)."""

    def __init__(self, data, form=_lib.FORM_FP64):
        L = _lib.load()
        a = as_matrix(data)
        self.dtype = a.dtype
        self.n, self.d = a.shape
        lay, ld = layout_of(a)
        dt = _lib.F32 if a.dtype == np.float32 else _lib.F64
        h = C.c_void_p()
        _lib.check(L.sc_knn_create(_lib.ptr(a), dt, lay, _lib.MEM_HOST, self.n, self.d, ld, C.byref(h)))
        self._L, self.h, self.form = L, h, form
        self._per_query = 64.0  # find_radius: rows per query of the previous call, for the output's first size

    def _q(self, queries):
        a = as_matrix(queries, dtype=self.dtype)
        if a.shape[1] != self.d:
            raise Failed(FailedError.FindFailed, "Input vector sizes are different.")
        return a

    def find_batch(self, queries, k):
        """find() for every row of queries: (idx, dist), each m x k, heap order."""
        a = self._q(queries)
        m = a.shape[0]
        lay, ld = layout_of(a)
        idx = np.zeros((m, max(k, 1)), np.int64)
        dist = np.zeros((m, max(k, 1)), np.float64)
        _lib.check(self._L.sc_knn_find(self.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, k, self.form,
                                       _lib.MEM_HOST, _lib.ptr(idx), _lib.ptr(dist)), FailedError.FindFailed)
        return idx, dist

    def find(self, from_, k):
        """LinearKNNSearch::find: list of (index, distance) in heap order,
        entries with index None dropped (linear_search.rs:79-83)."""
        idx, dist = self.find_batch(np.asarray(from_)[None, :], k)
        return [(int(i), float(dd)) for i, dd in zip(idx[0], dist[0]) if i >= 0]

    def find_radius_batch(self, queries, radius):
        """find_radius() for every row of queries: (counts, idx, dist), the
        rows of query 0 first, each query's rows in index order.  The output
        is sized from the previous call's rows per query, so one call (a
        counting and a filling pass) usually serves; when the rows do not
        fit, a second call with the exact size does."""
        a = self._q(queries)
        m = a.shape[0]
        lay, ld = layout_of(a)
        counts = np.zeros(max(m, 1), np.int64)
        total = np.zeros(1, np.int64)
        cap = max(1024, int(1.25 * self._per_query * m))
        idx = np.empty(cap, np.int64)
        dist = np.empty(cap, np.float64)
        rc = self._L.sc_knn_find_radius(self.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, float(radius), self.form,
                                        _lib.ptr(counts), cap, _lib.ptr(idx), _lib.ptr(dist), _lib.ptr(total))
        t = int(total[0])
        if rc != _lib.SC_OK and not (rc == _lib.SC_ERR_INVALID and t > cap):
            _lib.check(rc, FailedError.FindFailed)
        if t > cap:  # more rows than the first size: the exact size
            idx = np.empty(t, np.int64)
            dist = np.empty(t, np.float64)
            _lib.check(self._L.sc_knn_find_radius(self.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, float(radius),
                                                  self.form, _lib.ptr(counts), t, _lib.ptr(idx), _lib.ptr(dist),
                                                  _lib.ptr(total)), FailedError.FindFailed)
        if m:
            self._per_query = max(1.0, t / m)
        return counts[:m], idx[:t], dist[:t]

    def find_radius(self, from_, radius):
        """LinearKNNSearch::find_radius (linear_search.rs:89-108): list of
        (index, distance) of the rows with distance <= radius, in index order."""
        _, idx, dist = self.find_radius_batch(np.asarray(from_)[None, :], radius)
        return [(int(i), float(dd)) for i, dd in zip(idx, dist)]

    def classify(self, queries, k, weight, y_class, n_classes):
        a = self._q(queries)
        m = a.shape[0]
        lay, ld = layout_of(a)
        out = np.zeros(m, np.int64)
        yc = np.ascontiguousarray(y_class, np.int64)
        _lib.check(self._L.sc_knn_classify(self.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, k, self.form,
                                           int(weight), _lib.ptr(yc), n_classes, _lib.ptr(out)),
                   FailedError.PredictFailed)
        return out

    def regress(self, queries, k, weight, y):
        a = self._q(queries)
        m = a.shape[0]
        lay, ld = layout_of(a)
        out = np.zeros(m, np.float64)
        yy = np.ascontiguousarray(y, np.float64)
        _lib.check(self._L.sc_knn_regress(self.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, k, self.form,
                                          int(weight), _lib.ptr(yy), _lib.ptr(out)),
                   FailedError.PredictFailed)
        return out

    def rescored(self):
        v = np.zeros(1, np.int64)
        _lib.check(self._L.sc_knn_stats(self.h, _lib.ptr(v)))
        return int(v[0])

    def stream(self):
        return self._L.sc_knn_stream(self.h)

    def close(self):
        if self.h:
            self._L.sc_knn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class KNNClassifierParameters:
    """knn_classifier.rs:48-69, :144-154 (defaults: k=3, CoverTree, Uniform,
    Euclidean).  `form` selects FP64 or split-BF16 distances."""
    k: int = 3
    algorithm: KNNAlgorithmName = KNNAlgorithmName.CoverTree
    weight: KNNWeightFunction = KNNWeightFunction.Uniform
    form: int = _lib.FORM_FP64

    def with_k(self, k):
        self.k = k
        return self

    def with_algorithm(self, a):
        self.algorithm = a
        return self

    def with_weight(self, w):
        self.weight = w
        return self

    def with_form(self, f):
        self.form = f
        return self


@dataclass
class KNNRegressorParameters(KNNClassifierParameters):
    """knn_regressor.rs defaults: k=3, CoverTree, Uniform, Euclidean."""


class KNNClassifier:
    @staticmethod
    def fit(x, y, parameters: KNNClassifierParameters = None) -> "KNNClassifier":
        p = parameters or KNNClassifierParameters()
        a = as_matrix(x)
        y = np.asarray(y)
        classes = np.unique(y)  # y.unique(): sorted, deduplicated (arrays.rs:223-231)
        yi = np.searchsorted(classes, y).astype(np.int64)
        if a.shape[0] != y.shape[0]:  # knn_classifier.rs:237-241
            raise Failed.fit(f"Size of x should equal size of y; |x|=[{a.shape[0]}], |y|=[{y.shape[0]}]")
        if p.k <= 1:  # :243-248
            raise Failed.fit(f"k should be > 1, k=[{p.k}]")
        m = KNNClassifier()
        m.classes, m.y, m.k, m.weight = classes, yi, p.k, p.weight
        m.knn = LinearKNNSearch(a, form=p.form)
        return m

    def predict(self, x) -> np.ndarray:
        cls = self.knn.classify(x, self.k, self.weight, self.y, len(self.classes))
        return self.classes[cls]


class KNNRegressor:
    @staticmethod
    def fit(x, y, parameters: KNNRegressorParameters = None) -> "KNNRegressor":
        p = parameters or KNNRegressorParameters()
        a = as_matrix(x)
        y = np.asarray(y, np.float64)
        if a.shape[0] != y.shape[0]:  # knn_regressor.rs:224-228
            raise Failed.fit(f"Size of x should equal size of y; |x|=[{a.shape[0]}], |y|=[{y.shape[0]}]")
        if p.k < 1:  # :230-235
            raise Failed.fit(f"k should be > 0, k=[{p.k}]")
        m = KNNRegressor()
        m.y, m.k, m.weight = y, p.k, p.weight
        m.knn = LinearKNNSearch(a, form=p.form)
        return m

    def predict(self, x) -> np.ndarray:
        return self.knn.regress(x, self.k, self.weight, self.y)


@dataclass(frozen=True)
class PairwiseDistance:
    """PairwiseDistance (src/metrics/distance/mod.rs:84-110)."""
    node: int
    neighbour: Optional[int]
    distance: Optional[float]


class _NeighbourMap(Mapping):
    """Row -> PairwiseDistance over the device's neighbour arrays, each entry
    built when it is read (a map of n entries up front costs more than the
    scan itself)."""

    def __init__(self, nb, dist):
        self._nb, self._dist = nb, dist

    def __getitem__(self, i):
        if not 0 <= i < len(self._nb):
            raise KeyError(i)
        return PairwiseDistance(i, int(self._nb[i]), float(self._dist[i]))

    def __len__(self):
        return len(self._nb)

    def __iter__(self):
        return iter(range(len(self._nb)))


class FastPair:
    """FastPair::new / closest_pair (src/algorithm/neighbour/fastpair.rs:59-182).

    `distances[i]` is the reference's entry for row i: the nearest later row
    by squared distance (the running best kept in the element type), and for
    the last row itself with the element type's maximum; `neighbours` is the
    list 0 .. n - 1.  The scan runs on the device."""

    def __init__(self, x):
        a = as_matrix(x)
        n = a.shape[0]
        if n < 3:
            raise Failed(FailedError.FindFailed, "min number of rows should be 3")
        s = LinearKNNSearch(a)
        nb = np.zeros(n, np.int64)
        dist = np.zeros(n, np.float64)
        pair = np.zeros(2, np.int64)
        pd = np.zeros(1, np.float64)
        try:
            _lib.check(s._L.sc_fastpair(s.h, _lib.ptr(nb), _lib.ptr(dist), _lib.ptr(pair), _lib.ptr(pd)),
                       FailedError.FindFailed)
        finally:
            s.close()
        self.distances = _NeighbourMap(nb, dist)
        self.neighbours = list(range(n))
        self._closest = PairwiseDistance(int(pair[0]), int(pair[1]), float(pd[0]))

    @staticmethod
    def new(x) -> "FastPair":
        return FastPair(x)

    def closest_pair(self) -> PairwiseDistance:
        return self._closest
