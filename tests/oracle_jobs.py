"""Oracle jobs for a spawn process pool: each worker regenerates its own
seeded problem and fits it with the CPU restatement of KMeans::fit, so only
the small results travel back to the test process."""
import numpy as np


def fit_batched_problem(args):
    """(index, count, max_iter) -> the oracle's fit of problem `index` of
    batched_problems(count)."""
    import oracle
    from smartcore_gb300.synthetic import batched_problem
    index, count, max_iter = args
    x, k, seed = batched_problem(index)
    r = oracle.kmeans_fit(x, k, max_iter, seed=seed)
    return index, r.labels.astype(np.int32), r.sizes, r.centroids, r.iters, r.distortion
