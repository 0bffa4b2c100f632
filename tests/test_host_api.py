"""Host-side logic of the Python mirror that needs no GPU: the serde layout of
a fitted KMeans (src/cluster/kmeans.rs:71-83) and the validation that runs
before any device call."""
import json

import numpy as np
import pytest

from smartcore_gb300.cluster import DBSCAN, DBSCANParameters, KMeans, KMeansParameters
from smartcore_gb300.error import Failed


def model():
    cent = np.array([[1.0, 2.5, -3.0], [0.1, 1e-7, 7.25e21]])
    return KMeans(2, np.array([0, 1, 1, 0, 1]), np.array([2, 3]), 12.5, cent, 4, 0)


def test_kmeans_serde_layout_and_round_trip():
    m = model()
    d = json.loads(m.to_json())
    assert list(d) == ["k", "_y", "size", "_distortion", "centroids",
                       "_phantom_tx", "_phantom_ty", "_phantom_x", "_phantom_y"]
    assert d["_y"] == [0, 1, 1, 0, 1] and d["size"] == [2, 3] and d["_phantom_x"] is None
    back = KMeans.from_json(m.to_json())
    assert back == m
    assert np.array_equal(back.centroids, m.centroids)  # shortest round-trip decimal form


def test_kmeans_from_json_missing_field():
    d = json.loads(model().to_json())
    del d["size"]
    with pytest.raises(ValueError, match="missing field `size`"):
        KMeans.from_json(json.dumps(d))


def test_kmeans_partial_eq_epsilon():
    a, b = model(), model()
    b.centroids = b.centroids + np.finfo(np.float64).eps / 2
    assert a == b
    b.centroids = b.centroids + 1e-9
    assert not a == b


def test_validation_before_device():
    x = np.zeros((10, 2))
    with pytest.raises(Failed, match="invalid number of clusters: 1"):
        KMeans.fit(x, KMeansParameters(k=1))
    with pytest.raises(Failed, match="Invalid minPts"):
        DBSCAN.fit(x, DBSCANParameters().with_min_samples(0))
    with pytest.raises(Failed, match="Invalid radius"):
        DBSCAN.fit(x, DBSCANParameters().with_eps(-1.0))


def test_dbscan_defaults():
    p = DBSCANParameters()  # dbscan.rs:239-249
    assert (p.min_samples, p.eps) == (5, 0.5)
