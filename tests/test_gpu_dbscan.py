"""GPU parity of DBSCAN (src/cluster/dbscan.rs:274-398) against the CPU
oracle: the device computes every neighbourhood with the linear search, the
host runs the reference's expansion loop.  Bar: cluster labels and predicted
labels bit-identical to the oracle's (which follows the reference's own
find_radius calls), and the reference's own known answer."""
import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.cluster import DBSCAN, DBSCANParameters
from smartcore_gb300.error import Failed
from tests.datagen import blobs

pytestmark = pytest.mark.gpu

FORMS = [pytest.param(_lib.FORM_FP64, id="fp64"), pytest.param(_lib.FORM_SPLIT_BF16, id="split")]


@pytest.mark.parametrize("form", FORMS)
def test_reference_kat(kats, form):
    c = kats["dbscan_fit_predict"]
    x = np.array(c["x"])
    m = DBSCAN.fit(x, DBSCANParameters(form=form).with_eps(c["eps"]).with_min_samples(c["min_samples"]))
    assert m.predict(x).tolist() == c["expect"]


@pytest.mark.parametrize("form", FORMS)
def test_reference_errors(kats, form):
    c = kats["dbscan_fit_predict"]
    x = np.array(c["x"])
    with pytest.raises(Failed, match="Invalid minPts"):
        DBSCAN.fit(x, DBSCANParameters(form=form).with_min_samples(0))
    with pytest.raises(Failed, match="Invalid radius"):
        DBSCAN.fit(x, DBSCANParameters(form=form).with_eps(0.0))


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n,d,c,eps,min_samples", [(3000, 2, 6, 0.35, 5), (4000, 8, 10, 2.0, 8),
                                                   (2500, 33, 5, 6.5, 4), (1200, 1, 3, 0.05, 3)])
def test_fit_predict_match_oracle(form, dtype, n, d, c, eps, min_samples):
    # overlapping blobs: border points, noise and chains of core points
    x, _ = blobs(n, d, c, seed=n + d, dtype=dtype)
    m = DBSCAN.fit(x, DBSCANParameters(form=form).with_eps(eps).with_min_samples(min_samples))
    y, k = oracle.dbscan_fit(x, eps, min_samples)
    assert m.num_classes == k
    assert np.array_equal(m.cluster_labels, y)
    q, _ = blobs(500, d, c, seed=7, dtype=dtype)
    assert np.array_equal(m.predict(q), oracle.dbscan_predict(x, y, k, q, eps))


@pytest.mark.parametrize("form", FORMS)
def test_duplicates_and_ties(form):
    # integer grid with duplicates: many distances exactly equal to eps
    rng = np.random.default_rng(5)
    x = rng.integers(0, 12, size=(2000, 3)).astype(np.float64)
    for eps, ms in ((1.0, 4), (np.sqrt(2.0), 6), (2.0, 30)):
        m = DBSCAN.fit(x, DBSCANParameters(form=form).with_eps(eps).with_min_samples(ms))
        y, k = oracle.dbscan_fit(x, eps, ms)
        assert m.num_classes == k and np.array_equal(m.cluster_labels, y)
