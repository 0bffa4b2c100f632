"""sc_kmeans_step_noalloc: one FP64 Lloyd iteration whose scratch is a static
device array of the library (no allocation during the call).

Its results must equal the handle API's (sc_kmeans_set_centroids + one
sc_kmeans_iterate with the break rule off + sc_kmeans_get) bit for bit, on
two calls in a row over the same buffers.  The file is named to be collected
last, so it also runs after every other GPU test in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from smartcore_gb300 import _lib, build
from smartcore_gb300.cluster import KMeansHandle
from tests.datagen import blobs


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.load()


def step(L, x_dev, dtype, n, d, cent_dev, k, labels_dev, sizes_dev):
    dist = np.zeros(1, np.float64)
    rc = L.sc_kmeans_step_noalloc(C.c_void_p(x_dev), dtype, n, d, C.c_void_p(cent_dev), k,
                                  C.c_void_p(labels_dev), C.c_void_p(sizes_dev), _lib.ptr(dist), None)
    _lib.check(rc)
    return float(dist[0])


@pytest.mark.parametrize("n,d,k", [(5000, 24, 17), (70000, 64, 256), (300, 3, 2)])
@pytest.mark.parametrize("np_dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.gpu
def test_step_matches_handle_two_calls(L, n, d, k, np_dtype):
    torch = pytest.importorskip("torch")
    x, _ = blobs(n, d, max(k // 2, 2), seed=n + d + k)
    x = np.ascontiguousarray(x, np_dtype)
    rng = np.random.default_rng(k)
    c0 = np.ascontiguousarray(x[rng.choice(n, k, replace=False)], np.float64)

    ref = KMeansHandle(x, form=_lib.FORM_FP64)
    ref.set_centroids(c0)

    dev = torch.device("cuda:0")
    x_dev = torch.from_numpy(x).to(dev)
    cent_dev = torch.from_numpy(c0.copy()).to(dev)
    labels_dev = torch.full((n,), -7, dtype=torch.int32, device=dev)
    sizes_dev = torch.full((k,), -7, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    dt = _lib.F32 if np_dtype == np.float32 else _lib.F64

    for _ in range(2):
        ref.iterate(1, stop_on_converge=False)
        r_cent, r_sizes, r_labels, r_dist, _ = ref.get()
        dist = step(L, x_dev.data_ptr(), dt, n, d, cent_dev.data_ptr(), k, labels_dev.data_ptr(),
                    sizes_dev.data_ptr())
        assert np.array_equal(labels_dev.cpu().numpy().astype(np.int64), r_labels)
        assert np.array_equal(sizes_dev.cpu().numpy(), r_sizes)
        assert np.array_equal(cent_dev.cpu().numpy(), r_cent)
        assert dist == r_dist
    ref.close()


@pytest.mark.gpu
def test_step_matches_handle_values_below_the_sum_grid(L):
    """f32 points with a column scaled by 1e-18 and subnormal entries: their
    fixed-point roundings depend on the scale of the sums, which must be the
    one the handle API picks for the same data."""
    torch = pytest.importorskip("torch")
    n, d, k = 6000, 8, 5
    x, _ = blobs(n, d, k, seed=31, dtype=np.float32)
    x[:, 3] *= np.float32(1e-18)
    x[::7, 5] = np.float32(3e-39)
    x = np.ascontiguousarray(x)
    c0 = np.ascontiguousarray(x[np.random.default_rng(5).choice(n, k, replace=False)], np.float64)
    ref = KMeansHandle(x, form=_lib.FORM_FP64)
    ref.set_centroids(c0)
    x_dev = torch.from_numpy(x).cuda()
    cent_dev = torch.from_numpy(c0.copy()).cuda()
    labels_dev = torch.zeros(n, dtype=torch.int32, device="cuda")
    sizes_dev = torch.zeros(k, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        ref.iterate(1, stop_on_converge=False)
        r_cent, r_sizes, r_labels, r_dist, _ = ref.get()
        dist = step(L, x_dev.data_ptr(), _lib.F32, n, d, cent_dev.data_ptr(), k, labels_dev.data_ptr(),
                    sizes_dev.data_ptr())
        assert np.array_equal(labels_dev.cpu().numpy().astype(np.int64), r_labels)
        assert np.array_equal(sizes_dev.cpu().numpy(), r_sizes)
        assert np.array_equal(cent_dev.cpu().numpy(), r_cent)
        assert dist == r_dist
    ref.close()


@pytest.mark.gpu
def test_step_null_sizes_and_distortion(L):
    torch = pytest.importorskip("torch")
    n, d, k = 2000, 8, 5
    x, _ = blobs(n, d, k, seed=3)
    x = np.ascontiguousarray(x, np.float64)
    c0 = np.ascontiguousarray(x[:k], np.float64)
    ref = KMeansHandle(x, form=_lib.FORM_FP64)
    ref.set_centroids(c0)
    ref.iterate(1, stop_on_converge=False)
    r_cent, _, r_labels, _, _ = ref.get()
    ref.close()
    x_dev = torch.from_numpy(x).cuda()
    cent_dev = torch.from_numpy(c0.copy()).cuda()
    labels_dev = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.sc_kmeans_step_noalloc(C.c_void_p(x_dev.data_ptr()), _lib.F64, n, d, C.c_void_p(cent_dev.data_ptr()),
                                  k, C.c_void_p(labels_dev.data_ptr()), None, None, None)
    _lib.check(rc)
    assert np.array_equal(labels_dev.cpu().numpy().astype(np.int64), r_labels)
    assert np.array_equal(cent_dev.cpu().numpy(), r_cent)


@pytest.mark.parametrize("n,d,k,what", [
    (1000, 2, 4097, "k <= 4096"),
    (1000, 300, 256, "k*d <= 65536"),
    (8388609, 2, 4, "n <= 8388608"),
])
def test_step_rejects_oversize_without_touching_the_gpu(L, n, d, k, what):
    # The size limits are checked before the pointers and before any CUDA
    # call, so null pointers are safe here.
    rc = L.sc_kmeans_step_noalloc(None, _lib.F32, n, d, None, k, None, None, None, None)
    assert rc == _lib.SC_ERR_INVALID
    msg = _lib.last_error()
    assert "exceeds the no-allocation scratch" in msg and what in msg, msg


def test_step_rejects_null_pointers(L):
    rc = L.sc_kmeans_step_noalloc(None, _lib.F64, 10, 2, None, 2, None, None, None, None)
    assert rc == _lib.SC_ERR_INVALID
    assert _lib.last_error() == "null device pointer"
