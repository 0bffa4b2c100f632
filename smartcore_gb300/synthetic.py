"""Seeded synthetic inputs for the k-means and kNN workloads.

smartcore's own generator (src/dataset/generator.rs:10-48, make_blobs) draws
from thread_rng and cannot be seeded, so every workload here is generated with
numpy's default_rng from a fixed seed.  Shapes and value distributions follow
the workloads the benchmark and the parity tests use.
"""
from __future__ import annotations

import numpy as np


def blobs(n, d, k, seed=0, dtype=np.float64, box=(-10.0, 10.0), std=1.0, shuffle=True):
    """k isotropic Gaussian blobs, centres uniform in box^d, equal sizes
    (the first n % k blobs get one extra point), rows shuffled."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(box[0], box[1], size=(k, d))
    sizes = np.full(k, n // k)
    sizes[: n % k] += 1
    lab = np.repeat(np.arange(k), sizes)
    x = centers[lab] + rng.normal(0.0, std, size=(n, d))
    if shuffle:
        p = rng.permutation(n)
        x, lab = x[p], lab[p]
    return np.ascontiguousarray(x.astype(dtype)), lab.astype(np.int64)


def kmeans_small_f64(seed=42):
    """Plain KMeans, f64: 10,000 points, d=16, 8 blobs (centres U[-10,10],
    std 1.0), equal sizes, shuffled."""
    return blobs(10_000, 16, 8, seed=seed, dtype=np.float64)


def knn_blobs_f32(n_train=200_000, n_query=50_000, d=32, classes=10, seed=7):
    """kNN classifier workload: 10 classes, each an isotropic blob with centre
    U[-5,5]^32 and std 1.5; queries from the same mixture."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-5.0, 5.0, size=(classes, d))
    yt = rng.integers(0, classes, size=n_train)
    xt = centers[yt] + rng.normal(0.0, 1.5, size=(n_train, d))
    yq = rng.integers(0, classes, size=n_query)
    xq = centers[yq] + rng.normal(0.0, 1.5, size=(n_query, d))
    return (xt.astype(np.float32), yt.astype(np.int64), xq.astype(np.float32),
            yq.astype(np.int64))


def anisotropic_dirichlet_f32(n=1_000_000, d=64, k=256, seed=3, chunk=1 << 17):
    """k anisotropic Gaussian clusters: centres U[-20,20]^d, covariance A^T A
    with A_ij ~ N(0, 0.3^2), sizes drawn from Dirichlet(alpha=2) * n.
    Generated in chunks to keep host memory small; returned as float32."""
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-20.0, 20.0, size=(k, d))
    A = rng.normal(0.0, 0.3, size=(k, d, d))
    w = rng.dirichlet(np.full(k, 2.0))
    sizes = np.floor(w * n).astype(np.int64)
    sizes[: n - sizes.sum()] += 1
    x = np.empty((n, d), np.float32)
    lab = np.repeat(np.arange(k), sizes)
    s = 0
    for c in range(k):
        # rows c + z A (row-vector convention: covariance A^T A)
        z = rng.normal(size=(sizes[c], d))
        x[s:s + sizes[c]] = (centers[c] + z @ A[c]).astype(np.float32)
        s += sizes[c]
    p = rng.permutation(n)
    return np.ascontiguousarray(x[p]), lab[p]


def batched_problem(p, seed0=0, n_range=(1_000, 100_000), ds=(8, 16, 32, 64), k_range=(4, 64)):
    """Problem p of the batched k-means workload: n log-uniform in n_range, d
    from ds, k uniform in k_range, blobs with centres U[-10,10]^d and std
    U[0.5, 2.0], generated from seed seed0 + p.  Returns (x, k, seed)."""
    rng = np.random.default_rng(seed0 + p)
    n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
    d = int(rng.choice(ds))
    k = int(rng.integers(k_range[0], k_range[1] + 1))
    std = float(rng.uniform(0.5, 2.0))
    x, _ = blobs(n, d, k, seed=seed0 + p + 100_000, dtype=np.float32, std=std)
    return x, k, seed0 + p


def batched_problems(count=512, seed0=0, n_range=(1_000, 100_000), ds=(8, 16, 32, 64),
                     k_range=(4, 64)):
    """Independent k-means problems 0 .. count-1 of batched_problem."""
    return [batched_problem(p, seed0, n_range, ds, k_range) for p in range(count)]
