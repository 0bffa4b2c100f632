"""The headline k-means workload (1,000,000 x 64 f32 points in 256 anisotropic
Gaussian clusters with Dirichlet(2) sizes, k = 256) against the CPU oracle.

- At n = 100,000 (the same generator, seed 42) the whole KMeans::fit
  (src/cluster/kmeans.rs:254-323), k-means++ included, in both forms: labels,
  sizes and iteration count equal, centroids within 1e-12 relative.
- At the full 1,000,000 points: the device k-means++ partition against the
  oracle's (kmeans.rs:354-413) from the same draws, then one Lloyd step from
  the resulting centroids against the oracle's BBD-tree clustering
  (src/algorithm/neighbour/bbd_tree.rs:62-193).
"""
import numpy as np
import pytest

import oracle
from smartcore_gb300 import _lib
from smartcore_gb300.cluster import KMeans, KMeansHandle, KMeansParameters, kmeanspp_draws
from tests.datagen import anisotropic_dirichlet_f32

pytestmark = pytest.mark.gpu

FORMS = [pytest.param(_lib.FORM_FP64, id="fp64"), pytest.param(_lib.FORM_SPLIT_BF16, id="split")]


def rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=-1, keepdims=True), 1e-300)
    return float((np.abs(a - b) / scale).max())


@pytest.fixture(scope="module")
def reduced():
    x, _ = anisotropic_dirichlet_f32(n=100_000, d=64, k=256, seed=42)
    return x, oracle.kmeans_fit(x, 256, 50, seed=42)


@pytest.mark.parametrize("form", FORMS)
def test_reduced_fit_matches_oracle(reduced, form):
    x, ref = reduced
    km = KMeans.fit(x, KMeansParameters(k=256, max_iter=50, seed=42, form=form))
    assert np.array_equal(km._y, ref.labels)
    assert np.array_equal(km.size, ref.sizes)
    assert km.iters == ref.iters
    assert rel_err(km.centroids, ref.centroids) <= 1e-12
    xx = float((x.astype(np.float64) ** 2).sum())
    tol = 1e-12 * ref.distortion + (1e-14 * xx if form == _lib.FORM_SPLIT_BF16 else 0.0)
    assert abs(km._distortion - ref.distortion) <= tol


@pytest.mark.slow
def test_full_size_seeding_and_one_step():
    x, _ = anisotropic_dirichlet_f32()
    first, u = kmeanspp_draws(len(x), 256, 42)
    ref_labels, _ = oracle.kmeanspp(x, 256, first, u)
    h = KMeansHandle(x, form=_lib.FORM_SPLIT_BF16)
    h.seed(256, first, u)
    cent0, sizes0, labels0, _, _ = h.get()
    assert np.array_equal(labels0, ref_labels)
    assert np.array_equal(sizes0, np.bincount(ref_labels, minlength=256))
    h.iterate(1, stop_on_converge=False)
    cent1, sizes1, labels1, dist1, _ = h.get()
    r_dist, r_sums, r_counts, r_memb = oracle.bbd_clustering(x, cent0)
    assert np.array_equal(labels1, r_memb)
    assert np.array_equal(sizes1, r_counts)
    assert rel_err(cent1, r_sums / r_counts[:, None]) <= 1e-12
    assert abs(dist1 - r_dist) <= 1e-12 * r_dist + 1e-14 * float((x.astype(np.float64) ** 2).sum())
    h.close()
