"""KMeans on the GPU, with smartcore's API (src/cluster/kmeans.rs).

    from smartcore_gb300.cluster import KMeans, KMeansParameters
    km = KMeans.fit(x, KMeansParameters().with_k(2))
    y = km.predict(x)

fit = k-means++ seeding (host draws from the rand 0.8 generator the crate
would use, device D^2 passes) + the Lloyd loop on the device; predict = the
nearest-centroid assignment.  Labels equal the reference's; centroids agree
to ~1e-15 relative (exact fixed-point sums rounded once).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib
from .error import Failed, FailedError
from .linalg import as_matrix, layout_of


@dataclass
class KMeansParameters:
    """KMeansParameters (kmeans.rs:109-146): k, max_iter, seed.

    `form` selects the distance arithmetic (FP64 or split-BF16, identical
    results) and `rng` which rand 0.8 generator stands in for get_rng_impl
    (SmallRng without std_rand, StdRng with it); neither exists in the
    reference, both default to the reference's behaviour."""
    k: int = 2
    max_iter: int = 100
    seed: Optional[int] = None
    form: int = _lib.FORM_FP64
    rng: int = _lib.RNG_SMALL

    def with_k(self, k):
        self.k = k
        return self

    def with_max_iter(self, max_iter):
        self.max_iter = max_iter
        return self

    def with_seed(self, seed):
        self.seed = seed
        return self

    def with_form(self, form):
        self.form = form
        return self


def kmeanspp_draws(n, k, seed=None, rng=_lib.RNG_SMALL):
    """The draws kmeans_plus_plus takes from get_rng_impl(seed): seed None is
    seed 0 without std_rand (src/rand_custom.rs:26-27)."""
    L = _lib.load()
    first = np.zeros(1, np.int64)
    u = np.zeros(max(k - 1, 1), np.float64)
    _lib.check(L.sc_kmeanspp_draws(rng, 0 if seed is None else seed, n, k, _lib.ptr(first), _lib.ptr(u)))
    return int(first[0]), u[: max(k - 1, 0)]


# sc_kmeans_problem of include/smartcore_gb300.h as a NumPy record (the same
# layout as _lib.KMeansProblem), so that a batch's fields fill as columns
PROBLEM_DTYPE = np.dtype([("x", np.uint64), ("layout", np.int32), ("status", np.int32), ("n", np.int64),
                          ("d", np.int64), ("ld", np.int64), ("k", np.int64), ("max_iter", np.int64),
                          ("first_index", np.int64), ("uniforms", np.uint64), ("centroids_out", np.uint64),
                          ("sizes_out", np.uint64), ("labels_out", np.uint64), ("distortion_out", np.uint64),
                          ("iters_out", np.uint64), ("rescored", np.int64), ("pp_replays", np.int64)])
assert PROBLEM_DTYPE.itemsize == C.sizeof(_lib.KMeansProblem)
assert all(PROBLEM_DTYPE.fields[n][1] == getattr(_lib.KMeansProblem, n).offset for n in PROBLEM_DTYPE.names)


class KMeans:
    """Fitted model: k, size, _y, _distortion, centroids (kmeans.rs:73-83)."""

    def __init__(self, k, y, size, distortion, centroids, iters, form):
        self.k = k
        self._y = y
        self.size = size
        self._distortion = distortion
        self.centroids = centroids
        self.iters = iters
        self.form = form

    @staticmethod
    def fit(x, parameters: KMeansParameters = None) -> "KMeans":
        p = parameters or KMeansParameters()
        a = as_matrix(x)
        n, d = a.shape
        if p.k < 2:
            raise Failed(FailedError.FitFailed, f"invalid number of clusters: {p.k}")
        if p.max_iter == 0:
            raise Failed(FailedError.FitFailed, f"invalid maximum number of iterations: {p.max_iter}")
        first, u = kmeanspp_draws(n, p.k, p.seed, p.rng)
        L = _lib.load()
        lay, ld = layout_of(a)
        dt = _lib.F32 if a.dtype == np.float32 else _lib.F64
        cent = np.zeros((p.k, d), np.float64)
        sizes = np.zeros(p.k, np.int64)
        labels = np.zeros(n, np.int64)
        dist = np.zeros(1, np.float64)
        iters = np.zeros(1, np.int64)
        uu = np.ascontiguousarray(u, np.float64) if len(u) else np.zeros(1)
        _lib.check(L.sc_kmeans_fit(_lib.ptr(a), dt, lay, n, d, ld, p.k, p.max_iter, first, _lib.ptr(uu),
                                   p.form, _lib.ptr(cent), _lib.ptr(sizes), _lib.ptr(labels),
                                   _lib.ptr(dist), _lib.ptr(iters)))
        return KMeans(p.k, labels, sizes, float(dist[0]), cent, int(iters[0]), p.form)

    @staticmethod
    def fit_many(problems, form=_lib.FORM_SPLIT_BF16, stats=None) -> List["KMeans"]:
        """KMeans::fit for many independent problems in one call
        (sc_kmeans_fit_batched): `problems` is a list of (x, KMeansParameters),
        every x of the same element type.  Each result equals KMeans.fit of
        its problem alone.  `form` serves the problems beyond the batched
        kernels' limits (d > 64 or k > 128).  With a list `stats`, one
        (rescored rows, k-means++ replays) pair per problem is appended."""
        if not problems:
            return []
        L = _lib.load()
        mats = [as_matrix(x) for x, _ in problems]
        dts = {a.dtype for a in mats}
        if len(dts) != 1:
            raise ValueError("every problem of one call must have the same element type")
        dt = _lib.F32 if mats[0].dtype == np.float32 else _lib.F64
        pars = [p or KMeansParameters() for _, p in problems]
        for p in pars:
            if p.k < 2:
                raise Failed(FailedError.FitFailed, f"invalid number of clusters: {p.k}")
            if p.max_iter == 0:
                raise Failed(FailedError.FitFailed, f"invalid maximum number of iterations: {p.max_iter}")
        m = len(problems)
        ns = np.array([a.shape[0] for a in mats], np.int64)
        ds = np.array([a.shape[1] for a in mats], np.int64)
        ks = np.array([p.k for p in pars], np.int64)
        # every output in one array per kind; each problem gets its slice
        n_off = np.concatenate(([0], np.cumsum(ns)))
        c_off = np.concatenate(([0], np.cumsum(ks * ds)))
        k_off = np.concatenate(([0], np.cumsum(ks)))
        u_off = np.concatenate(([0], np.cumsum(np.maximum(ks - 1, 1))))
        labels = np.empty(int(n_off[-1]), np.int64)
        cent = np.empty(int(c_off[-1]), np.float64)
        sizes = np.empty(int(k_off[-1]), np.int64)
        dist = np.empty(m, np.float64)
        iters = np.empty(m, np.int64)
        first = np.empty(m, np.int64)
        uu = np.empty(int(u_off[-1]), np.float64)
        fb, ub = first.ctypes.data, uu.ctypes.data
        for i, (p, a) in enumerate(zip(pars, mats)):  # k-means++ draws of each problem (kmeanspp_draws)
            _lib.check(L.sc_kmeanspp_draws(p.rng, 0 if p.seed is None else p.seed, int(ns[i]), p.k, fb + 8 * i,
                                           ub + 8 * int(u_off[i])))
        arr = np.zeros(m, PROBLEM_DTYPE)
        lay = [layout_of(a) for a in mats]
        arr["x"] = [a.ctypes.data for a in mats]
        arr["layout"] = [l for l, _ in lay]
        arr["ld"] = [ld for _, ld in lay]
        arr["n"], arr["d"], arr["k"] = ns, ds, ks
        arr["max_iter"] = [p.max_iter for p in pars]
        arr["first_index"] = first
        arr["uniforms"] = ub + 8 * u_off[:-1]
        arr["centroids_out"] = cent.ctypes.data + 8 * c_off[:-1]
        arr["sizes_out"] = sizes.ctypes.data + 8 * k_off[:-1]
        arr["labels_out"] = labels.ctypes.data + 8 * n_off[:-1]
        arr["distortion_out"] = dist.ctypes.data + 8 * np.arange(m)
        arr["iters_out"] = iters.ctypes.data + 8 * np.arange(m)
        _lib.check(L.sc_kmeans_fit_batched(arr.ctypes.data, m, dt, form))
        if stats is not None:
            stats.extend(zip(arr["rescored"].tolist(), arr["pp_replays"].tolist()))
        return [KMeans(p.k, labels[n_off[i]:n_off[i + 1]], sizes[k_off[i]:k_off[i + 1]], float(dist[i]),
                       cent[c_off[i]:c_off[i + 1]].reshape(p.k, -1), int(iters[i]), form)
                for i, p in enumerate(pars)]

    def predict(self, x) -> np.ndarray:
        a = as_matrix(x)
        n, d = a.shape
        L = _lib.load()
        lay, ld = layout_of(a)
        dt = _lib.F32 if a.dtype == np.float32 else _lib.F64
        labels = np.zeros(n, np.int64)
        c = np.ascontiguousarray(self.centroids, np.float64)
        _lib.check(L.sc_kmeans_predict(_lib.ptr(a), dt, lay, n, d, ld, _lib.ptr(c), self.k, self.form,
                                       _lib.ptr(labels)), FailedError.PredictFailed)
        return labels

    # serde form of the reference's struct (kmeans.rs:71-83, `derive(Serialize,
    # Deserialize)`): its fields in declaration order, the four PhantomData
    # fields as unit (null).
    _SERDE_FIELDS = ("k", "_y", "size", "_distortion", "centroids",
                     "_phantom_tx", "_phantom_ty", "_phantom_x", "_phantom_y")

    def to_serde(self) -> dict:
        return {"k": int(self.k), "_y": [int(v) for v in self._y], "size": [int(v) for v in self.size],
                "_distortion": float(self._distortion),
                "centroids": [[float(v) for v in row] for row in np.asarray(self.centroids)],
                "_phantom_tx": None, "_phantom_ty": None, "_phantom_x": None, "_phantom_y": None}

    def to_json(self) -> str:
        """The model as serde_json writes the reference's KMeans (compact, fields in order)."""
        import json
        return json.dumps(self.to_serde(), separators=(",", ":"), allow_nan=False)

    @staticmethod
    def from_json(text: str, form=_lib.FORM_SPLIT_BF16) -> "KMeans":
        """A model written by serde_json from the reference's KMeans (or by to_json)."""
        import json
        d = json.loads(text)
        missing = [f for f in KMeans._SERDE_FIELDS if f not in d]
        if missing:
            raise ValueError(f"missing field `{missing[0]}`")
        cent = np.asarray(d["centroids"], np.float64).reshape(len(d["centroids"]), -1)
        return KMeans(int(d["k"]), np.asarray(d["_y"], np.int64), np.asarray(d["size"], np.int64),
                      float(d["_distortion"]), cent, 0, form)

    def __eq__(self, other):
        """PartialEq of kmeans.rs:85-107: k, size and centroids within f64::EPSILON."""
        if self.k != other.k or not np.array_equal(self.size, other.size):
            return False
        if self.centroids.shape != other.centroids.shape:
            return False
        return bool(np.all(np.abs(self.centroids - other.centroids) <= np.finfo(np.float64).eps))


def batch_tune(path=None, force=False):
    """Tuning table of the batched assignment kernel on the current device:
    loaded from `path` when it holds one made on this kind of device, else
    measured (about a second) and written there.  The default path is in the
    package's build folder.  Returns the path."""
    import os
    from . import build as _build
    L = _lib.load()
    path = path or os.path.join(_build.BUILD, "batch_tune.txt")
    if not force and os.path.exists(path) and L.sc_batch_tune_load(path.encode()) == _lib.SC_OK:
        return path
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    _lib.check(L.sc_batch_tune(path.encode()))
    return path


def batch_variant(d, k):
    """(centroids per inner pass, rows per work item) the batched call uses for (d, k)."""
    L = _lib.load()
    a = np.zeros(2, np.int32)
    _lib.check(L.sc_batch_tune_get(d, k, _lib.ptr(a[:1]), _lib.ptr(a[1:])))
    return int(a[0]), int(a[1])


class KMeansHandle:
    """Device-resident dataset for repeated Lloyd runs (sc_kmeans_* handle API)."""

    def __init__(self, x, form=_lib.FORM_FP64, device_ptr=None, dtype=None, shape=None):
        L = _lib.load()
        self._L = L
        h = C.c_void_p()
        if device_ptr is not None:
            n, d = shape
            dt = _lib.F32 if dtype == np.float32 else _lib.F64
            _lib.check(L.sc_kmeans_create(C.c_void_p(device_ptr), dt, _lib.ROW_MAJOR, _lib.MEM_DEVICE, n, d, d,
                                          form, C.byref(h)))
        else:
            a = as_matrix(x)
            n, d = a.shape
            lay, ld = layout_of(a)
            dt = _lib.F32 if a.dtype == np.float32 else _lib.F64
            _lib.check(L.sc_kmeans_create(_lib.ptr(a), dt, lay, _lib.MEM_HOST, n, d, ld, form, C.byref(h)))
        self.h, self.n, self.d, self.k = h, n, d, 0

    def seed(self, k, first, uniforms):
        u = np.ascontiguousarray(uniforms, np.float64) if len(uniforms) else np.zeros(1)
        _lib.check(self._L.sc_kmeans_seed(self.h, k, first, _lib.ptr(u)))
        self.k = k

    def set_centroids(self, c):
        c = np.ascontiguousarray(c, np.float64)
        _lib.check(self._L.sc_kmeans_set_centroids(self.h, c.shape[0], _lib.ptr(c)))
        self.k = c.shape[0]

    def iterate(self, max_iter, stop_on_converge=True, wait=True):
        it = np.zeros(1, np.int64)
        _lib.check(self._L.sc_kmeans_iterate(self.h, max_iter, 1 if stop_on_converge else 0,
                                             _lib.ptr(it) if wait else None))
        return int(it[0])

    def get(self):
        cent = np.zeros((self.k, self.d), np.float64)
        sizes = np.zeros(self.k, np.int64)
        labels = np.zeros(self.n, np.int64)
        dist = np.zeros(1, np.float64)
        iters = np.zeros(1, np.int64)
        _lib.check(self._L.sc_kmeans_get(self.h, _lib.ptr(cent), _lib.ptr(sizes), _lib.ptr(labels),
                                         _lib.ptr(dist), _lib.ptr(iters)))
        return cent, sizes, labels, float(dist[0]), int(iters[0])

    def stats(self):
        a = np.zeros(2, np.int64)
        _lib.check(self._L.sc_kmeans_stats(self.h, _lib.ptr(a[:1]), _lib.ptr(a[1:])))
        return int(a[0]), int(a[1])

    def incremental_steps(self):
        """Steps of the last iterate() whose sums moved only the relabelled rows."""
        a = np.zeros(1, np.int64)
        _lib.check(self._L.sc_kmeans_sum_stats(self.h, _lib.ptr(a)))
        return int(a[0])

    def stream(self):
        return self._L.sc_kmeans_stream(self.h)

    def sync(self):
        _lib.check(self._L.sc_kmeans_sync(self.h))

    def close(self):
        if self.h:
            self._L.sc_kmeans_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class DBSCANParameters:
    """DBSCANParameters (src/cluster/dbscan.rs:79-96, defaults :239-249).

    `algorithm` keeps the reference's default (CoverTree); the device always
    searches linearly, whose neighbourhoods come in index order.  The cluster
    of a point that borders two clusters can depend on that order."""
    min_samples: int = 5
    eps: float = 0.5
    algorithm: "object" = None
    form: int = _lib.FORM_SPLIT_BF16

    def with_min_samples(self, v):
        self.min_samples = v
        return self

    def with_eps(self, v):
        self.eps = v
        return self

    def with_algorithm(self, v):
        self.algorithm = v
        return self


class DBSCAN:
    """DBSCAN::fit / predict (src/cluster/dbscan.rs:274-398) on the device."""

    def __init__(self, search, cluster_labels, num_classes, eps, form):
        self._search = search
        self.cluster_labels = cluster_labels
        self.num_classes = num_classes
        self.eps = eps
        self.form = form

    @staticmethod
    def fit(x, parameters: DBSCANParameters = None) -> "DBSCAN":
        from .neighbors import LinearKNNSearch
        p = parameters or DBSCANParameters()
        if p.min_samples < 1:
            raise Failed(FailedError.FitFailed, "Invalid minPts")
        if not p.eps > 0:
            raise Failed(FailedError.FitFailed, "Invalid radius: ")
        search = LinearKNNSearch(x, form=p.form)
        labels = np.zeros(search.n, np.int64)
        k = np.zeros(1, np.int64)
        _lib.check(search._L.sc_dbscan_fit(search.h, float(p.eps), int(p.min_samples), p.form,
                                           _lib.ptr(labels), _lib.ptr(k)))
        return DBSCAN(search, labels, int(k[0]), float(p.eps), p.form)

    def predict(self, x) -> np.ndarray:
        s = self._search
        a = s._q(x)
        m = a.shape[0]
        lay, ld = layout_of(a)
        out = np.zeros(m, np.int64)
        _lib.check(s._L.sc_dbscan_predict(s.h, _lib.ptr(a), lay, _lib.MEM_HOST, m, ld, self.eps, self.form,
                                          _lib.ptr(self.cluster_labels), self.num_classes, _lib.ptr(out)),
                   FailedError.PredictFailed)
        return out
