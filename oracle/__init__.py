"""CPU oracle for smartcore's distance-argmin path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package: it checks the product and is never part of it.
The C sources (``rng.c``, ``kmeans.c``, ``knn.c``) restate the reference
algorithm function by function, each citing the smartcore file:line it
follows; this module only loads them through ctypes and converts arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

F32, F64 = 0, 1
ROW_MAJOR, COL_MAJOR = 0, 1
RNG_SMALL, RNG_STD = 0, 1

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    for f in ("rng.c", "kmeans.c", "knn.c", "oracle.h"):
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            P, I64, D, I = C.c_void_p, C.c_int64, C.c_double, C.c_int
            L.orc_kmeanspp_draws.argtypes = [I, C.c_uint64, I64, I64, P, P]
            L.orc_rng_u64.argtypes = [I, C.c_uint64, I64, P]
            L.orc_xoshiro256pp.argtypes = [P, I64, P]
            L.orc_splitmix64.argtypes = [C.c_uint64, I64, P]
            L.orc_chacha_block.argtypes = [P, P, I, P]
            L.orc_chacha_quarter_round.argtypes = [P]
            L.orc_pcg32.argtypes = [C.c_uint64, C.c_uint64, I, I64, P]
            L.orc_sqdist.argtypes = [I, P, P, I64]
            L.orc_sqdist.restype = D
            L.orc_kmeans_fit.argtypes = [I, I, P, I64, I64, I64, I64, I64, I64, P, P, P, P, P, P, P]
            L.orc_kmeans_fit.restype = I
            L.orc_kmeanspp.argtypes = [I, I, P, I64, I64, I64, I64, I64, P, P, P]
            L.orc_kmeans_predict.argtypes = [I, I, P, I64, I64, I64, P, I64, P]
            L.orc_bbd_clustering.argtypes = [I, I, P, I64, I64, I64, P, I64, P, P, P]
            L.orc_bbd_clustering.restype = D
            L.orc_lloyd_bruteforce.argtypes = [I, I, P, I64, I64, I64, I64, I64, P, P, P, P, P]
            L.orc_bbd_lloyd_timed.argtypes = [I, I, P, I64, I64, I64, I64, I64, P, P, P]
            L.orc_bbd_lloyd_timed.restype = D
            L.orc_heap_add_sequence.argtypes = [P, I64, I64, P]
            L.orc_heap_add_sequence.restype = I64
            L.orc_knn_find.argtypes = [I, P, I64, I64, P, I64, I64, P, P]
            L.orc_knn_find.restype = I
            L.orc_knn_find_radius.argtypes = [I, P, I64, I64, P, I64, D, P, P, P, I64]
            L.orc_knn_find_radius.restype = I64
            L.orc_dbscan_fit.argtypes = [I, P, I64, I64, D, I64, P]
            L.orc_dbscan_fit.restype = I64
            L.orc_dbscan_predict.argtypes = [I, P, I64, I64, P, I64, P, I64, D, P]
            L.orc_fastpair.argtypes = [I, P, I64, I64, P, P]
            L.orc_fastpair.restype = I
            L.orc_knn_vote.argtypes = [P, P, I64, I64, P, I64, I, P]
            L.orc_knn_regress.argtypes = [P, P, I64, I64, P, I, P]
            L.orc_last_error.restype = C.c_char_p
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _mat(x):
    """(dtype code, layout, array, ld) for a 2-D float32/float64 array."""
    x = np.asarray(x)
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float64)
    dt = F32 if x.dtype == np.float32 else F64
    if x.flags.c_contiguous:
        return dt, ROW_MAJOR, x, x.shape[1]
    if x.flags.f_contiguous:
        return dt, COL_MAJOR, x, x.shape[0]
    x = np.ascontiguousarray(x)
    return dt, ROW_MAJOR, x, x.shape[1]


def kmeanspp_draws(n, k, seed=0, rng=RNG_SMALL):
    first = np.zeros(1, np.int64)
    u = np.zeros(max(k - 1, 1), np.float64)
    lib().orc_kmeanspp_draws(rng, C.c_uint64(seed), n, k, _ptr(first), _ptr(u))
    return int(first[0]), u[: max(k - 1, 0)]


def rng_u64(count, seed=0, rng=RNG_SMALL):
    out = np.zeros(count, np.uint64)
    lib().orc_rng_u64(rng, C.c_uint64(seed), count, _ptr(out))
    return out


def xoshiro256pp(state, count):
    """count outputs of xoshiro256++ from the 4-word state."""
    st = np.ascontiguousarray(state, np.uint64)
    out = np.zeros(count, np.uint64)
    lib().orc_xoshiro256pp(_ptr(st), count, _ptr(out))
    return out


def splitmix64(seed, count):
    out = np.zeros(count, np.uint64)
    lib().orc_splitmix64(C.c_uint64(seed), count, _ptr(out))
    return out


def chacha_block(key, words12_15, rounds):
    """The ChaCha block function: 16 output words of the given key (8 words),
    words 12..15 (counter / nonce) and round count."""
    k = np.ascontiguousarray(key, np.uint32)
    w = np.ascontiguousarray(words12_15, np.uint32)
    out = np.zeros(16, np.uint32)
    lib().orc_chacha_block(_ptr(k), _ptr(w), rounds, _ptr(out))
    return out


def chacha_quarter_round(a, b, c, d):
    v = np.array([a, b, c, d], np.uint32)
    lib().orc_chacha_quarter_round(_ptr(v))
    return [int(t) for t in v]


def pcg32(state, inc, count, after_step=False):
    out = np.zeros(count, np.uint32)
    lib().orc_pcg32(C.c_uint64(state), C.c_uint64(inc), 1 if after_step else 0, count, _ptr(out))
    return out


def sqdist(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    dt = F32 if a.dtype == np.float32 else F64
    return lib().orc_sqdist(dt, _ptr(a), _ptr(b), a.shape[0])


class FitResult:
    def __init__(self, centroids, sizes, labels, distortion, iters, trace):
        self.centroids, self.sizes, self.labels = centroids, sizes, labels
        self.distortion, self.iters, self.trace = distortion, iters, trace


def kmeans_fit(x, k, max_iter, first=None, uniforms=None, seed=0, rng=RNG_SMALL):
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    if first is None:
        first, uniforms = kmeanspp_draws(n, k, seed, rng) if k >= 2 else (0, np.zeros(0))
    u = np.ascontiguousarray(uniforms, np.float64)
    cent = np.zeros((max(k, 1), d), np.float64)
    sizes = np.zeros(max(k, 1), np.int64)
    labels = np.zeros(n, np.int64)
    dist = np.zeros(1, np.float64)
    iters = np.zeros(1, np.int64)
    trace = np.zeros(max(max_iter, 1), np.float64)
    rc = lib().orc_kmeans_fit(dt, lay, _ptr(x), n, d, ld, k, max_iter, first, _ptr(u),
                              _ptr(cent), _ptr(sizes), _ptr(labels), _ptr(dist), _ptr(iters),
                              _ptr(trace))
    if rc != 0:
        raise ValueError(lib().orc_last_error().decode())
    it = int(iters[0])
    return FitResult(cent, sizes, labels, float(dist[0]), it, trace[:it])


def kmeanspp(x, k, first, uniforms):
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    labels = np.zeros(n, np.int64)
    chosen = np.zeros(k, np.int64)
    u = np.ascontiguousarray(uniforms, np.float64)
    lib().orc_kmeanspp(dt, lay, _ptr(x), n, d, ld, k, first, _ptr(u), _ptr(labels), _ptr(chosen))
    return labels, chosen


def kmeans_predict(x, centroids):
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    c = np.ascontiguousarray(centroids, np.float64)
    labels = np.zeros(n, np.int64)
    lib().orc_kmeans_predict(dt, lay, _ptr(x), n, d, ld, _ptr(c), c.shape[0], _ptr(labels))
    return labels


def bbd_clustering(x, centroids):
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    c = np.ascontiguousarray(centroids, np.float64)
    k = c.shape[0]
    sums = np.zeros((k, d), np.float64)
    counts = np.zeros(k, np.int64)
    memb = np.zeros(n, np.int64)
    r = lib().orc_bbd_clustering(dt, lay, _ptr(x), n, d, ld, _ptr(c), k, _ptr(sums),
                                 _ptr(counts), _ptr(memb))
    return r, sums, counts, memb


def lloyd_bruteforce(x, centroids, max_iter):
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    c = np.array(centroids, np.float64, copy=True, order="C")
    k = c.shape[0]
    sizes = np.zeros(k, np.int64)
    labels = np.zeros(n, np.int64)
    dist = np.zeros(1, np.float64)
    iters = np.zeros(1, np.int64)
    lib().orc_lloyd_bruteforce(dt, lay, _ptr(x), n, d, ld, k, max_iter, _ptr(c), _ptr(sizes),
                               _ptr(labels), _ptr(dist), _ptr(iters))
    return FitResult(c, sizes, labels, float(dist[0]), int(iters[0]), None)


def heap_add_sequence(values, k):
    v = np.ascontiguousarray(values, np.float64)
    out = np.zeros(max(k, 1), np.float64)
    n = lib().orc_heap_add_sequence(_ptr(v), v.shape[0], k, _ptr(out))
    return out[: min(k, v.shape[0])], int(n)


def knn_find(train, queries, k):
    train = np.ascontiguousarray(train)
    if train.dtype not in (np.float32, np.float64):
        train = train.astype(np.float64)
    queries = np.ascontiguousarray(queries, dtype=train.dtype)
    dt = F32 if train.dtype == np.float32 else F64
    n, d = train.shape
    m = queries.shape[0]
    idx = np.zeros((m, max(k, 1)), np.int64)
    dist = np.zeros((m, max(k, 1)), np.float64)
    rc = lib().orc_knn_find(dt, _ptr(train), n, d, _ptr(queries), m, k, _ptr(idx), _ptr(dist))
    if rc != 0:
        raise ValueError("Find failed: k should be >= 1 and <= length(data)")
    return idx, dist


def knn_find_radius(train, queries, radius, cap=None):
    train = np.ascontiguousarray(train)
    if train.dtype not in (np.float32, np.float64):
        train = train.astype(np.float64)
    queries = np.ascontiguousarray(queries, dtype=train.dtype)
    dt = F32 if train.dtype == np.float32 else F64
    n, d = train.shape
    m = queries.shape[0]
    cap = cap or n * m
    counts = np.zeros(m, np.int64)
    idx = np.zeros(cap, np.int64)
    dist = np.zeros(cap, np.float64)
    tot = lib().orc_knn_find_radius(dt, _ptr(train), n, d, _ptr(queries), m, float(radius),
                                    _ptr(counts), _ptr(idx), _ptr(dist), cap)
    if tot == -1:
        raise ValueError("Find failed: radius should be > 0")
    return counts, idx[:tot], dist[:tot]


def dbscan_fit(x, eps, min_samples):
    """DBSCAN::fit with the linear search: (cluster labels with -1 for noise, number of clusters)."""
    x = np.ascontiguousarray(x)
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float64)
    dt = F32 if x.dtype == np.float32 else F64
    n, d = x.shape
    y = np.zeros(n, np.int64)
    k = lib().orc_dbscan_fit(dt, _ptr(x), n, d, float(eps), int(min_samples), _ptr(y))
    if k == -1:
        raise ValueError("Fit failed: Invalid minPts")
    if k == -2:
        raise ValueError("Fit failed: Invalid radius: ")
    return y, int(k)


def dbscan_predict(x, y, k, queries, eps):
    x = np.ascontiguousarray(x)
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float64)
    queries = np.ascontiguousarray(queries, dtype=x.dtype)
    dt = F32 if x.dtype == np.float32 else F64
    n, d = x.shape
    out = np.zeros(queries.shape[0], np.int64)
    lib().orc_dbscan_predict(dt, _ptr(x), n, d, _ptr(np.ascontiguousarray(y, np.int64)), int(k),
                             _ptr(queries), queries.shape[0], float(eps), _ptr(out))
    return out


def fastpair(x):
    """FastPair::new + closest_pair: (neighbour per row, distance per row, (a, b, d))."""
    x = np.ascontiguousarray(x)
    if x.dtype not in (np.float32, np.float64):
        x = x.astype(np.float64)
    dt = F32 if x.dtype == np.float32 else F64
    n, d = x.shape
    nb = np.zeros(max(n, 1), np.int64)
    dist = np.zeros(max(n, 1), np.float64)
    if lib().orc_fastpair(dt, _ptr(x), n, d, _ptr(nb), _ptr(dist)) != 0:
        raise ValueError("Find failed: min number of rows should be 3")
    a = 0
    for p in range(n):  # closest_pair (fastpair.rs:165-182)
        if dist[p] < dist[a]:
            a = p
    return nb[:n], dist[:n], (a, int(nb[a]), float(dist[a]))


def knn_vote(idx, dist, y_index, n_classes, weight=0):
    idx = np.ascontiguousarray(idx, np.int64)
    dist = np.ascontiguousarray(dist, np.float64)
    y = np.ascontiguousarray(y_index, np.int64)
    m, k = idx.shape
    out = np.zeros(m, np.int64)
    lib().orc_knn_vote(_ptr(idx), _ptr(dist), m, k, _ptr(y), n_classes, weight, _ptr(out))
    return out


def knn_regress(idx, dist, y, weight=0):
    idx = np.ascontiguousarray(idx, np.int64)
    dist = np.ascontiguousarray(dist, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    m, k = idx.shape
    out = np.zeros(m, np.float64)
    lib().orc_knn_regress(_ptr(idx), _ptr(dist), m, k, _ptr(y), weight, _ptr(out))
    return out


def bbd_lloyd_timed(x, centroids, iters):
    """(tree build seconds, per-iteration seconds, final centroids, labels)."""
    dt, lay, x, ld = _mat(x)
    n, d = x.shape
    c = np.array(centroids, np.float64, copy=True, order="C")
    labels = np.zeros(n, np.int64)
    secs = np.zeros(max(iters, 1), np.float64)
    build = lib().orc_bbd_lloyd_timed(dt, lay, _ptr(x), n, d, ld, c.shape[0], iters, _ptr(c),
                                      _ptr(labels), _ptr(secs))
    return build, secs[:iters], c, labels
