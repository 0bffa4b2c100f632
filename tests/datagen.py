"""Seeded inputs for the tests (re-exported from the package generator)."""
from smartcore_gb300.synthetic import (anisotropic_dirichlet_f32, batched_problems, blobs,  # noqa: F401
                                       kmeans_small_f64, knn_blobs_f32)
