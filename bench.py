"""Benchmark of the distance-argmin path: Lloyd iterations per second of
KMeans on 1,000,000 x 64 float32 points, k = 256 (anisotropic Gaussian
clusters, Dirichlet(2) sizes), split-BF16 form.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one full Lloyd iteration over the whole dataset (assignment,
FP64 re-score of near ties, centroid sums, new centroids, distortion and
break test), inputs resident in HBM.  Under torchrun each rank runs an
independent replica of the workload on its own GPU (the path has no
cross-GPU exchange); value = iterations of all ranks / max-over-ranks time.

--impl reference times the reference algorithm on the host CPU: the C
restatement of smartcore's KMeans Lloyd step (BBD-tree filtering, single
thread, as the reference) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, D, K_CLUSTERS, MAX_ITER = 1_000_000, 64, 256, 50
SEED_DATA, SEED_KMEANS = 3, 42
CPU_SAMPLE = 32_768  # points of the workload timed on the host CPU
METRIC = "k-means Lloyd iter/s (1Mx64, k=256)"
UNIT = "iter/s"
WORKLOAD = "kmeans_f32_1Mx64_k256_anisotropic_dirichlet"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms, device):
    """Largest per-rank time (ms) over all ranks of the process group; the
    local value when the job runs without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(steps, world_size, max_ms):
    """Whole-job throughput: every rank runs `steps` steps of its own replica,
    and the slowest rank's time is the job's time."""
    return world_size * steps / (max_ms / 1e3)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples (every 20 ms) of SM clocks and throttle reasons;
    summary() keeps the samples taken inside the timed region."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.p, self.rows, self.t0, self.t1 = index, None, [], None, None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "20"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(1.0)  # let the sampler start before the timed region
        except OSError:
            self.p = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.p is None:
            return
        time.sleep(0.1)
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        import datetime
        for line in out.strip().splitlines():
            f = [t.strip() for t in line.split(",")]
            if len(f) != 7:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                continue
            self.rows.append((ts, f[1:]))

    def summary(self):
        inside = [r for ts, r in self.rows if self.t0 is not None and self.t0 - 0.02 <= ts <= self.t1 + 0.02]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no sample inside the timed region"],
                    "samples": 0}
        num = lambda v: float(v) if v.replace(".", "", 1).isdigit() else None
        sm = [num(r[0]) for r in inside if num(r[0]) is not None]
        mx = [num(r[1]) for r in inside if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i in range(4) if r[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def cpu_baseline(x, seed_centroids, iters=3):
    """The reference Lloyd step (BBD tree, 1 thread) on a CPU_SAMPLE-point
    sample; returns the full-size rate by linear scaling in n."""
    import oracle
    sub = np.ascontiguousarray(x[:CPU_SAMPLE])
    build, secs, _, _ = oracle.bbd_lloyd_timed(sub, seed_centroids, iters)
    per_iter = float(np.median(secs))
    return {
        "value": (1.0 / per_iter) * (CPU_SAMPLE / N),
        "unit": UNIT,
        "cores": 1,
        "kind": "port",
        "sample": (f"C restatement of KMeans Lloyd step (BBD-tree filtering, src/algorithm/neighbour/"
                   f"bbd_tree.rs) on the first {CPU_SAMPLE} of {N} points, k={K_CLUSTERS}; median of "
                   f"{iters} iterations = {per_iter:.3f} s; rate scaled by {CPU_SAMPLE}/{N}; tree build "
                   f"{build:.3f} s excluded; single thread (the reference is single-threaded); "
                   f"host has {os.cpu_count()} cores"),
    }


KNN_N, KNN_M, KNN_D, KNN_K = 200_000, 50_000, 32, 5
KNN_CPU_QUERIES = 200


def bench_knn(torch, local, reps=5, n_query=None, with_fp64=True):
    """Brute-force kNN classifier workload: 200,000 x 32 f32 training rows in
    10 Gaussian classes, 50,000 queries from the same mixture, k=5, uniform
    weights.  Device-resident queries/s of find() for both forms, agreement of
    the two forms' heap arrays and votes, and the reference's CPU search on a
    sample of the queries."""
    import oracle
    from smartcore_gb300 import _lib
    from smartcore_gb300.neighbors import LinearKNNSearch
    from smartcore_gb300.synthetic import knn_blobs_f32
    L = _lib.load()
    m = n_query or KNN_M
    xt, yt, xq, _ = knn_blobs_f32(KNN_N, m, KNN_D)
    q_dev = torch.from_numpy(xq).to(f"cuda:{local}")
    out = {}
    res = {}
    forms = (("split_bf16", _lib.FORM_SPLIT_BF16), ("fp64", _lib.FORM_FP64)) if with_fp64 else \
        (("split_bf16", _lib.FORM_SPLIT_BF16),)
    for name, form in forms:
        s = LinearKNNSearch(xt, form=form)
        idx = torch.empty((m, KNN_K), dtype=torch.int64, device=f"cuda:{local}")
        dist = torch.empty((m, KNN_K), dtype=torch.float64, device=f"cuda:{local}")
        stream = torch.cuda.ExternalStream(s.stream())

        def find():
            _lib.check(L.sc_knn_find(s.h, C.c_void_p(q_dev.data_ptr()), _lib.ROW_MAJOR, _lib.MEM_DEVICE, m,
                                     KNN_D, KNN_K, form, _lib.MEM_DEVICE, C.c_void_p(idx.data_ptr()),
                                     C.c_void_p(dist.data_ptr())))
        find()  # warm-up (also builds the split training operand)
        n_rep = reps if form == _lib.FORM_SPLIT_BF16 else 1
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(n_rep):
            find()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / n_rep
        out[name] = {"queries_per_s": m / (ms / 1e3), "ms_per_find": ms,
                     "exact_distance_evals": s.rescored() if form == _lib.FORM_SPLIT_BF16 else m * KNN_N}
        res[name] = (idx.cpu().numpy(), dist.cpu().numpy())
        s.close()
    if not with_fp64:
        return out
    out["heaps_equal"] = bool(np.array_equal(res["split_bf16"][0], res["fp64"][0]) and
                              np.array_equal(res["split_bf16"][1], res["fp64"][1]))
    votes = [oracle.knn_vote(res[f][0], res[f][1], yt, 10) for f in ("split_bf16", "fp64")]
    out["labels_equal"] = bool(np.array_equal(votes[0], votes[1]))
    t0 = time.perf_counter()
    ridx, rdist = oracle.knn_find(xt, xq[:KNN_CPU_QUERIES], KNN_K)
    cpu_s = time.perf_counter() - t0
    out["oracle_sample_equal"] = bool(np.array_equal(ridx, res["split_bf16"][0][:KNN_CPU_QUERIES]) and
                                      np.array_equal(rdist, res["split_bf16"][1][:KNN_CPU_QUERIES]))
    out["split_speedup_vs_fp64"] = out["split_bf16"]["queries_per_s"] / out["fp64"]["queries_per_s"]
    out["cpu_baseline"] = {"value": KNN_CPU_QUERIES / cpu_s, "unit": "queries/s", "cores": 1, "kind": "port",
                           "sample": f"C restatement of LinearKNNSearch::find + heap replay on the first "
                                     f"{KNN_CPU_QUERIES} of {KNN_M} queries against all {KNN_N} rows, single thread"}
    out["config"] = {"n_train": KNN_N, "n_query": KNN_M, "d": KNN_D, "k": KNN_K, "classes": 10, "dtype": "f32"}
    out["find_radius"] = bench_radius(torch, local, xt, xq)
    out["dbscan"] = bench_dbscan(torch, xt)
    out["fastpair"] = bench_fastpair(torch, xt)
    return out


KNN_RADIUS = 8.0
RADIUS_CPU_QUERIES = 200


def bench_radius(torch, local, xt, xq):
    """LinearKNNSearch::find_radius on the kNN workload (radius 8.0, ~56 rows per query): queries/s
    of both forms through the C ABI with host queries and results (counting
    and filling passes), agreement of the two forms on every query, and the
    reference's CPU scan on a sample of the queries."""
    import oracle
    from smartcore_gb300 import _lib
    from smartcore_gb300.neighbors import LinearKNNSearch
    res, out = {}, {}
    for name, form in (("split_bf16", _lib.FORM_SPLIT_BF16), ("fp64", _lib.FORM_FP64)):
        s = LinearKNNSearch(xt, form=form)
        s.find_radius_batch(xq[:1024], KNN_RADIUS)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res[name] = s.find_radius_batch(xq, KNN_RADIUS)
        dt = time.perf_counter() - t0
        out[name] = {"queries_per_s": len(xq) / dt, "ms": 1e3 * dt, "neighbours": int(res[name][0].sum())}
        s.close()
    out["forms_equal"] = bool(all(np.array_equal(a, b) for a, b in zip(res["split_bf16"], res["fp64"])))
    t0 = time.perf_counter()
    rc, ridx, rdist = oracle.knn_find_radius(xt, xq[:RADIUS_CPU_QUERIES], KNN_RADIUS)
    cpu_s = time.perf_counter() - t0
    c, idx, dist = res["split_bf16"]
    nsamp = int(rc.sum())
    out["oracle_sample_equal"] = bool(np.array_equal(c[:RADIUS_CPU_QUERIES], rc) and
                                      np.array_equal(idx[:nsamp], ridx) and np.array_equal(dist[:nsamp], rdist))
    out["cpu_baseline"] = {"value": RADIUS_CPU_QUERIES / cpu_s, "unit": "queries/s", "cores": 1, "kind": "port",
                           "sample": f"C restatement of LinearKNNSearch::find_radius on the first "
                                     f"{RADIUS_CPU_QUERIES} queries against all {KNN_N} rows, single thread"}
    out["config"] = {"radius": KNN_RADIUS, "n_train": KNN_N, "n_query": len(xq), "d": KNN_D,
                     "e2e": "host queries in, host rows out, both passes"}
    return out


FASTPAIR_N = 20_000


def bench_fastpair(torch, xt):
    """FastPair::new + closest_pair on the first 20,000 kNN training rows:
    rows/s on the device (every row's nearest later row, exact reference
    distances) and the reference's CPU algorithm on the same rows, whose
    entries must agree."""
    import oracle
    from smartcore_gb300.neighbors import FastPair
    x = np.ascontiguousarray(xt[:FASTPAIR_N])
    FastPair(x[:1024])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fp = FastPair(x)
    dt = time.perf_counter() - t0
    t0 = time.perf_counter()
    nb, dist, closest = oracle.fastpair(x)
    cpu_s = time.perf_counter() - t0
    c = fp.closest_pair()
    equal = bool([fp.distances[i].neighbour for i in range(len(x))] == nb.tolist() and
                 np.array_equal(np.array([fp.distances[i].distance for i in range(len(x))]), dist) and
                 (c.node, c.neighbour, c.distance) == closest)
    return {"rows_per_s": len(x) / dt, "ms": 1e3 * dt, "closest_pair": [c.node, c.neighbour, c.distance],
            "oracle_equal": equal,
            "cpu_baseline": {"value": len(x) / cpu_s, "unit": "rows/s", "cores": 1, "kind": "port",
                             "sample": f"C restatement of FastPair::init on the same {len(x)} rows "
                                       f"({cpu_s:.1f} s), single thread"},
            "config": {"n": len(x), "d": KNN_D, "e2e": "host rows in, host map out"}}


MANY_PROBLEMS = 512
MANY_MAX_ITER = 30
MANY_CPU_SAMPLE = 4


def bench_many_problems(torch):
    """512 independent k-means problems (n log-uniform in [1e3, 1e5], d in
    {8, 16, 32, 64}, k in [4, 64], max_iter 30) through one call of the
    batched KMeans::fit (sc_kmeans_fit_batched) with host input and output:
    problem-iterations per second of the whole batch, best of three calls
    after a warm-up call.  The tuning table of the batched kernel is loaded
    (or measured) before the timed calls.  On the first four problems the
    same fits run through the reference's CPU algorithm (BBD tree), whose
    labels must agree."""
    import oracle
    from smartcore_gb300 import _lib
    from smartcore_gb300.cluster import KMeans, KMeansParameters, batch_tune
    from smartcore_gb300.synthetic import batched_problems
    L = _lib.load()
    probs = batched_problems(count=MANY_PROBLEMS)
    # the host rows live in pinned memory, as an application feeding a GPU keeps them
    pinned = [torch.from_numpy(x).pin_memory().numpy() for x, _, _ in probs]
    par = [(xp, KMeansParameters(k=k, max_iter=MANY_MAX_ITER, seed=seed)) for xp, (_, k, seed) in zip(pinned, probs)]
    t0 = time.perf_counter()
    batch_tune()
    tune_s = time.perf_counter() - t0
    KMeans.fit_many(par)  # warm-up
    torch.cuda.synchronize()
    best, fits, launches, stats = None, None, 0, []
    for _ in range(3):
        st = []
        l0 = L.sc_kernel_launches()
        t0 = time.perf_counter()
        f = KMeans.fit_many(par, stats=st)
        dt = time.perf_counter() - t0
        if best is None or dt < best:
            best, fits, launches, stats = dt, f, L.sc_kernel_launches() - l0, st
    iters = sum(km.iters for km in fits)
    sample_iters, cpu_s, labels_equal = 0, 0.0, True
    for (x, k, seed), km in zip(probs[:MANY_CPU_SAMPLE], fits):
        t1 = time.perf_counter()
        ref = oracle.kmeans_fit(x, k, MANY_MAX_ITER, seed=seed)
        cpu_s += time.perf_counter() - t1
        sample_iters += ref.iters
        labels_equal &= bool(np.array_equal(km._y, ref.labels)) and km.iters == ref.iters
    points = int(sum(len(p[0]) for p in probs))
    return {"problem_iters_per_s": iters / best, "problems": len(probs), "iterations": iters, "ms": 1e3 * best,
            "points": points, "gpu_launches": int(launches), "sample_labels_equal": labels_equal,
            "rescored_rows": int(sum(a for a, _ in stats)), "pp_replays": int(sum(b for _, b in stats)),
            "tuning_s": tune_s,
            "cpu_baseline": {"value": sample_iters / cpu_s, "unit": "problem-iterations/s", "cores": 1,
                             "kind": "port",
                             "sample": f"C restatement of KMeans::fit (k-means++ and BBD-tree Lloyd) on the "
                                       f"first {MANY_CPU_SAMPLE} problems, single thread"},
            "config": {"n": "log-uniform [1e3, 1e5]", "d": [8, 16, 32, 64], "k": "[4, 64]",
                       "max_iter": MANY_MAX_ITER, "h2d_bytes": int(sum(p[0].nbytes for p in probs)),
                       "e2e": "one sc_kmeans_fit_batched call, host data (pinned) in and results out"}}


def measure_pipe_peaks(torch, local):
    """FP64 and FP32 (no TF32) GEMM rates of this GPU through cuBLAS (torch
    matmul, 8192^3 for FP32, 4096^3 for FP64, best of 5 after a warm-up):
    the denominators of the FP64 form's roofline, which the driver's peak
    file does not record."""
    dev = torch.device(f"cuda:{local}")
    old_tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    out = {}
    try:
        for name, dt, n in (("fp64_tflops", torch.float64, 4096), ("fp32_tflops", torch.float32, 8192)):
            a = torch.randn((n, n), device=dev, dtype=dt)
            b = torch.randn((n, n), device=dev, dtype=dt)
            torch.matmul(a, b)
            torch.cuda.synchronize()
            best = 1e30
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b)
                e1.record()
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            out[name] = 2.0 * n ** 3 / (best / 1e3) / 1e12
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old_tf32
    out["how"] = "cuBLAS via torch.matmul, FP64 4096^3 and FP32 8192^3 (TF32 off), best of 5, CUDA events"
    return out


def bench_fp64_kernels(torch, local):
    """The FP64 form's kernels alone (for profiler runs): one Lloyd step of
    the 1M x 64, k = 256 workload and a kNN find of 2,000 queries of the
    200,000 x 32 training rows."""
    from smartcore_gb300 import _lib
    from smartcore_gb300.cluster import KMeansHandle, kmeanspp_draws
    from smartcore_gb300.neighbors import LinearKNNSearch
    from smartcore_gb300.synthetic import anisotropic_dirichlet_f32, knn_blobs_f32
    x, _ = anisotropic_dirichlet_f32(N, D, K_CLUSTERS, seed=SEED_DATA)
    h = KMeansHandle(x, form=_lib.FORM_FP64)
    first, u = kmeanspp_draws(N, K_CLUSTERS, SEED_KMEANS)
    h.seed(K_CLUSTERS, first, u)
    t0 = time.perf_counter()
    h.iterate(1, stop_on_converge=False)
    lloyd_ms = 1e3 * (time.perf_counter() - t0)
    h.close()
    xt, _, xq, _ = knn_blobs_f32(KNN_N, 2000, KNN_D)
    s = LinearKNNSearch(xt, form=_lib.FORM_FP64)
    t0 = time.perf_counter()
    s.find_batch(xq, KNN_K)
    knn_ms = 1e3 * (time.perf_counter() - t0)
    s.close()
    return {"fp64_lloyd_step_ms": lloyd_ms, "fp64_knn_2000_queries_ms": knn_ms}


LARGE_N, LARGE_D, LARGE_K, LARGE_MAX_ITER = 16_000_000, 128, 4096, 20
LARGE_Q, LARGE_KNN_K = 1_000_000, 10
LARGE_PREDICT_SAMPLE, LARGE_KNN_ORACLE_SAMPLE = 10_000, 8


def large_data(torch, dev, n_query):
    """16,000,000 x 128 f32 points in 4,096 isotropic Gaussian blobs (centres
    U[-50,50]^128, std 2.0, equal sizes, rows shuffled) and n_query queries
    from the same mixture, generated on the device from seeded generators."""
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    centers = torch.rand((LARGE_K, LARGE_D), generator=g, device=dev, dtype=torch.float32) * 100.0 - 50.0
    lab = torch.arange(LARGE_N, device=dev) % LARGE_K
    lab = lab[torch.randperm(LARGE_N, generator=g, device=dev)]
    x = torch.empty((LARGE_N, LARGE_D), device=dev, dtype=torch.float32)
    for r0 in range(0, LARGE_N, 1 << 20):
        r1 = min(LARGE_N, r0 + (1 << 20))
        x[r0:r1] = centers[lab[r0:r1]] + 2.0 * torch.randn((r1 - r0, LARGE_D), generator=g, device=dev)
    qlab = torch.randint(0, LARGE_K, (n_query,), generator=g, device=dev)
    q = centers[qlab] + 2.0 * torch.randn((n_query, LARGE_D), generator=g, device=dev)
    return x, q.contiguous()


def bench_large(torch, local, n_query=LARGE_Q):
    """The large workload: KMeans::fit on 16M x 128 f32 points, k = 4,096,
    max_iter 20 (k-means++ and the Lloyd loop on device-resident data, split-
    BF16 form: the streamed-centroid assignment kernel), then brute-force kNN
    (k = 10) of n_query queries from the same mixture against the 16M rows.
    Checks: the split form's predict with the final centroids against the
    oracle on 10,000 sample rows; the kNN heaps against the oracle on 8
    queries (the FP64 form runs one thread per query over all 16M rows, so a
    sample of queries keeps one SM busy for minutes)."""
    import oracle
    from smartcore_gb300 import _lib
    from smartcore_gb300.cluster import KMeans, KMeansHandle, kmeanspp_draws
    L = _lib.load()
    dev = torch.device(f"cuda:{local}")
    t0 = time.perf_counter()
    x, q = large_data(torch, dev, n_query)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    out = {"config": {"n": LARGE_N, "d": LARGE_D, "k": LARGE_K, "max_iter": LARGE_MAX_ITER, "dtype": "f32",
                      "data": f"4096 blobs, centres U[-50,50]^128, std 2 (generated on the device, {gen_s:.1f} s)",
                      "knn_queries": n_query, "knn_k": LARGE_KNN_K}}
    pk, pk_kind = peaks()
    # ---- KMeans::fit, device-resident ----
    h = KMeansHandle(None, form=_lib.FORM_SPLIT_BF16, device_ptr=x.data_ptr(), dtype=np.float32,
                     shape=(LARGE_N, LARGE_D))
    first, u = kmeanspp_draws(LARGE_N, LARGE_K, SEED_KMEANS)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h.seed(LARGE_K, first, u)
    seed_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(h.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    L.sc_kmeans_profile(h.h, 1)
    e0.record(stream)
    iters = h.iterate(LARGE_MAX_ITER, stop_on_converge=True)
    e1.record(stream)
    e1.synchronize()
    lloyd_ms = e0.elapsed_time(e1)
    kms = np.zeros(1)
    kl = np.zeros(1, np.int64)
    L.sc_kmeans_profile_read(h.h, _lib.ptr(kms), _lib.ptr(kl))
    rescored, replays = h.stats()
    cent, sizes, _, dist, _ = h.get()
    h.close()
    assign_ms = float(kms[0]) / max(int(kl[0]), 1)
    flop = 2.0 * LARGE_N * LARGE_K * LARGE_D
    rs = np.random.default_rng(0).choice(LARGE_N, LARGE_PREDICT_SAMPLE, replace=False)
    xs = x[torch.from_numpy(rs).to(dev)].cpu().numpy()
    km = KMeans(LARGE_K, None, sizes, dist, cent, iters, _lib.FORM_SPLIT_BF16)
    t0 = time.perf_counter()
    ref = oracle.kmeans_predict(xs, cent)
    cpu_pred_s = time.perf_counter() - t0
    achieved = flop / (assign_ms / 1e3) / 1e12
    out["kmeans"] = {
        "lloyd_iters_per_s": iters / (lloyd_ms / 1e3), "iterations": iters, "lloyd_ms": lloyd_ms,
        "seeding_s": seed_s, "assign_kernel_ms": assign_ms, "rescored_points_per_iter": rescored / max(iters, 1),
        "pp_replays": replays, "distortion": dist,
        "roofline": {"bound": "tensor", "kernel": "split_wide_kernel", "achieved": achieved,
                     "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"],
                     "peak_kind": f"{pk_kind} bf16 burst", "algorithmic_flop_per_launch": flop},
        "predict_sample_oracle_equal": bool(np.array_equal(km.predict(xs), ref)),
        "cpu_baseline": {"value": (LARGE_PREDICT_SAMPLE / LARGE_N) / cpu_pred_s,
                         "unit": "assignment passes/s", "cores": 1, "kind": "port",
                         "sample": f"C restatement of KMeans::predict (the brute-force assignment a BBD-tree step "
                                   f"reduces to at d = 128) on {LARGE_PREDICT_SAMPLE} rows ({cpu_pred_s:.1f} s), "
                                   f"scaled by {LARGE_PREDICT_SAMPLE}/{LARGE_N}, single thread"},
    }
    # ---- kNN: the queries against the 16M rows ----
    hk = C.c_void_p()
    _lib.check(L.sc_knn_create(C.c_void_p(x.data_ptr()), _lib.F32, _lib.ROW_MAJOR, _lib.MEM_DEVICE, LARGE_N,
                               LARGE_D, LARGE_D, C.byref(hk)))
    kstream = torch.cuda.ExternalStream(L.sc_knn_stream(hk))
    idx = torch.empty((n_query, LARGE_KNN_K), dtype=torch.int64, device=dev)
    dst = torch.empty((n_query, LARGE_KNN_K), dtype=torch.float64, device=dev)

    def find(form, m):
        _lib.check(L.sc_knn_find(hk, C.c_void_p(q.data_ptr()), _lib.ROW_MAJOR, _lib.MEM_DEVICE, m, LARGE_D,
                                 LARGE_KNN_K, form, _lib.MEM_DEVICE, C.c_void_p(idx.data_ptr()),
                                 C.c_void_p(dst.data_ptr())))
    find(_lib.FORM_SPLIT_BF16, min(1024, n_query))  # warm-up: builds the training operand
    torch.cuda.synchronize()
    e0.record(kstream)
    find(_lib.FORM_SPLIT_BF16, n_query)
    e1.record(kstream)
    e1.synchronize()
    knn_ms = e0.elapsed_time(e1)
    ev = np.zeros(1, np.int64)
    L.sc_knn_stats(hk, _lib.ptr(ev))
    no = min(LARGE_KNN_ORACLE_SAMPLE, n_query)
    si, sd = idx[:no].cpu().numpy(), dst[:no].cpu().numpy()
    L.sc_knn_destroy(hk)
    xt = x.cpu().numpy()
    t0 = time.perf_counter()
    ridx, rdist = oracle.knn_find(xt, q[:no].cpu().numpy(), LARGE_KNN_K)
    cpu_s = time.perf_counter() - t0
    kflop = 2.0 * n_query * LARGE_N * LARGE_D
    kach = kflop / (knn_ms / 1e3) / 1e12
    out["knn"] = {
        "queries_per_s": n_query / (knn_ms / 1e3), "ms": knn_ms, "exact_distance_evals": int(ev[0]),
        "roofline": {"bound": "tensor", "kernel": "knn_filter_kernel", "achieved": kach,
                     "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": kach / pk["bf16_tflops"],
                     "peak_kind": f"{pk_kind} bf16 burst",
                     "timed": "the whole find: candidate filter, exact replay and any queries past the "
                              "candidate capacity"},
        "oracle_sample_equal": bool(np.array_equal(ridx, si) and np.array_equal(rdist, sd)),
        "cpu_baseline": {"value": no / cpu_s, "unit": "queries/s", "cores": 1, "kind": "port",
                         "sample": f"C restatement of LinearKNNSearch::find on {no} queries "
                                   f"against all {LARGE_N} rows ({cpu_s:.1f} s), single thread"},
    }
    del x, q, idx, dst, xt
    torch.cuda.empty_cache()
    return out


DBSCAN_EPS = 8.0
DBSCAN_MIN_SAMPLES = 10
DBSCAN_SAMPLE = 20_000


def bench_dbscan(torch, xt):
    """DBSCAN::fit on the kNN training rows (eps 8.0, min_samples 10): points/s
    of the split form with host input (every neighbourhood on the device, the
    reference's expansion loop on the host), and on the first 20,000 rows both
    forms and the reference's CPU algorithm (its own find_radius calls),
    whose labels must agree; the CPU rate is scaled by 20,000 / n because each
    neighbourhood query scans all n rows."""
    import oracle
    from smartcore_gb300 import _lib
    from smartcore_gb300.cluster import DBSCAN, DBSCANParameters
    par = lambda form: DBSCANParameters(form=form).with_eps(DBSCAN_EPS).with_min_samples(DBSCAN_MIN_SAMPLES)
    DBSCAN.fit(xt[:4096], par(_lib.FORM_SPLIT_BF16))  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = DBSCAN.fit(xt, par(_lib.FORM_SPLIT_BF16))
    dt = time.perf_counter() - t0
    out = {"split_bf16": {"points_per_s": len(xt) / dt, "ms": 1e3 * dt, "clusters": m.num_classes,
                          "noise": int((m.cluster_labels < 0).sum())}}
    sub = np.ascontiguousarray(xt[:DBSCAN_SAMPLE])
    ms = DBSCAN.fit(sub, par(_lib.FORM_SPLIT_BF16))
    mf = DBSCAN.fit(sub, par(_lib.FORM_FP64))
    t0 = time.perf_counter()
    y, k = oracle.dbscan_fit(sub, DBSCAN_EPS, DBSCAN_MIN_SAMPLES)
    cpu_s = time.perf_counter() - t0
    out["sample_forms_equal"] = bool(np.array_equal(ms.cluster_labels, mf.cluster_labels))
    out["sample_oracle_equal"] = bool(np.array_equal(ms.cluster_labels, y) and ms.num_classes == k)
    out["cpu_baseline"] = {"value": DBSCAN_SAMPLE / cpu_s * (DBSCAN_SAMPLE / len(xt)), "unit": "points/s",
                           "cores": 1, "kind": "port",
                           "sample": f"C restatement of DBSCAN::fit with LinearKNNSearch on the first "
                                     f"{DBSCAN_SAMPLE} rows ({cpu_s:.1f} s), rate scaled by "
                                     f"{DBSCAN_SAMPLE}/{len(xt)}, single thread"}
    out["config"] = {"eps": DBSCAN_EPS, "min_samples": DBSCAN_MIN_SAMPLES, "n": len(xt), "d": KNN_D,
                     "e2e": "host rows in, host labels out"}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from smartcore_gb300.synthetic import anisotropic_dirichlet_f32
    x, _ = anisotropic_dirichlet_f32(N, D, K_CLUSTERS, seed=SEED_DATA)
    import oracle

    def start(m):
        sub = np.ascontiguousarray(x[:m])
        first, u = oracle.kmeanspp_draws(m, K_CLUSTERS, SEED_KMEANS)
        y0, _ = oracle.kmeanspp(sub, K_CLUSTERS, first, u)
        c0 = np.zeros((K_CLUSTERS, D))
        np.add.at(c0, y0, sub.astype(np.float64))
        c0 /= np.maximum(np.bincount(y0, minlength=K_CLUSTERS), 1)[:, None]
        return sub, c0

    # size the per-step sample so that warmup + steps stay within ~2 minutes
    sub, c0 = start(4096)
    _, secs, _, _ = oracle.bbd_lloyd_timed(sub, c0, 3)
    per_point = float(np.median(secs)) / 4096
    budget = 120.0 / (args.warmup + args.steps)
    m = int(min(CPU_SAMPLE, max(2048, budget / per_point)) // 1024 * 1024)
    sub, c0 = start(m)
    build, secs, _, _ = oracle.bbd_lloyd_timed(sub, c0, args.warmup + args.steps)
    timed = secs[args.warmup:]
    total = float(timed.sum())
    value = (args.steps / total) * (m / N)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps * (N / m),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "n": N, "d": D, "k": K_CLUSTERS,
                                        "form": "reference CPU (BBD tree)", "sample_points": m},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": (f"each step = one BBD-tree Lloyd iteration on the first {m} of "
                                    f"{N} points (k={K_CLUSTERS}, d={D}); rate scaled by {m}/{N}; "
                                    f"tree build {build:.3f} s excluded; single thread, host has "
                                    f"{os.cpu_count()} cores")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from smartcore_gb300 import _lib
    from smartcore_gb300.cluster import KMeans, KMeansHandle, KMeansParameters, kmeanspp_draws
    from smartcore_gb300.synthetic import anisotropic_dirichlet_f32
    L = _lib.load()
    if not L.sc_device_ok():
        raise RuntimeError("no usable sm_103 device")

    x, _ = anisotropic_dirichlet_f32(N, D, K_CLUSTERS, seed=SEED_DATA)
    x_pinned = torch.from_numpy(x).pin_memory()
    x_dev = x_pinned.to(f"cuda:{local}", non_blocking=False)
    first, u = kmeanspp_draws(N, K_CLUSTERS, SEED_KMEANS)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident throughput, split-BF16 form ----
    h = KMeansHandle(None, form=_lib.FORM_SPLIT_BF16, device_ptr=x_dev.data_ptr(), dtype=np.float32,
                     shape=(N, D))
    h.seed(K_CLUSTERS, first, u)
    c_start, _, _, _, _ = h.get()
    stream = torch.cuda.ExternalStream(h.stream())
    for _ in range(args.warmup):
        h.iterate(1, stop_on_converge=False, wait=False)
    h.sync()
    L.sc_kmeans_profile(h.h, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = L.sc_kernel_launches()
    barrier()
    with ClockSampler(local) as clk:
        clk.mark_start()
        e0.record(stream)
        h.iterate(args.steps, stop_on_converge=False, wait=False)
        e1.record(stream)
        e1.synchronize()
        clk.mark_end()
    launches = L.sc_kernel_launches() - launches0
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), f"cuda:{local}")
    kms = np.zeros(1)
    kl = np.zeros(1, np.int64)
    L.sc_kmeans_profile_read(h.h, _lib.ptr(kms), _lib.ptr(kl))
    L.sc_kmeans_profile(h.h, 0)
    rescored, _ = h.stats()
    incremental = h.incremental_steps()
    kernel_ms = float(kms[0]) / max(int(kl[0]), 1)
    value = job_rate(args.steps, ws, ms)

    if rank != 0 or args.lloyd_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "steps": args.steps,
                              "ms_per_step": ms / args.steps, "kernel_ms": kernel_ms,
                              "gpu_launches": int(launches), "mode": "lloyd-only"}), flush=True)
        h.close()
        return

    # ---- same start, FP64 form: rate and agreement of labels / distortion ----
    hf = KMeansHandle(None, form=_lib.FORM_FP64, device_ptr=x_dev.data_ptr(), dtype=np.float32,
                      shape=(N, D))
    hs = KMeansHandle(None, form=_lib.FORM_SPLIT_BF16, device_ptr=x_dev.data_ptr(), dtype=np.float32,
                      shape=(N, D))
    agree = []
    fp64_ms = []
    for hh in (hf, hs):
        hh.set_centroids(c_start)
    for it in range(2):
        t0 = time.perf_counter()
        hf.iterate(1, stop_on_converge=False)
        fp64_ms.append((time.perf_counter() - t0) * 1e3)
        hs.iterate(1, stop_on_converge=False)
        cf, sf, lf, df, _ = hf.get()
        cs, ss, ls, dsp, _ = hs.get()
        agree.append({"labels_equal": bool(np.array_equal(lf, ls)),
                      "inertia_rel_err": abs(dsp - df) / abs(df),
                      "centroid_max_rel_err": float(np.max(np.abs(cs - cf)) / np.max(np.abs(cf)))})
    hf.close()
    hs.close()

    # ---- end to end through the public API: host buffers in and out ----
    e2e_steps = max(1, min(3, args.steps))
    e2e_iters, e2e_time = 0, 0.0
    xh = x_pinned.numpy()
    e2e_warm = 2  # the first fits grow the device memory pool and the pinned staging buffer
    for s in range(e2e_steps + e2e_warm):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        km = KMeans.fit(xh, KMeansParameters(k=K_CLUSTERS, max_iter=MAX_ITER, seed=SEED_KMEANS,
                                             form=_lib.FORM_SPLIT_BF16))
        dt = time.perf_counter() - t0
        if s >= e2e_warm:
            e2e_iters += km.iters
            e2e_time += dt
    h2d = N * D * 4 + 8 * K_CLUSTERS
    d2h = K_CLUSTERS * D * 8 + K_CLUSTERS * 8 + N * 8 + 16

    pk, pk_kind = peaks()
    flop = 2.0 * N * K_CLUSTERS * D
    achieved = flop / (kernel_ms / 1e3) / 1e12
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "split_assign_kmeans_1Mx64_k256.txt")
    if os.path.exists(tfile):
        for line in open(tfile):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = float(line.split(":", 1)[1])

    knn = bench_knn(torch, local) if not args.no_knn else None
    many = bench_many_problems(torch) if not args.no_knn else None
    large = bench_large(torch, local) if not (args.no_knn or args.no_large) else None
    pipes = measure_pipe_peaks(torch, local)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3-split/fp32-acc/f64-rescore",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": N, "d": D, "k": K_CLUSTERS, "form": "split_bf16",
                   "parallelism": f"replicas x{ws}", "l2": "inputs larger than L2 (256 MB bf16 + 256 MB f32 "
                   "read per step)"},
        "roofline": {"bound": "tensor", "kernel": "split_assign_kernel", "achieved": achieved,
                     "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"],
                     "peak_kind": f"{pk_kind} bf16 burst", "traffic": traffic,
                     "algorithmic_flop_per_launch": flop, "issued_flop_per_launch": 3 * flop,
                     "kernel_ms": kernel_ms, "algorithmic_bytes_per_launch": N * D * 2 * 2},
        "cpu_baseline": cpu_baseline(x, c_start),
        "e2e": {"value": e2e_iters / e2e_time, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "note": f"KMeans.fit with host input: upload, k-means++, up to {MAX_ITER} Lloyd iterations, "
                        f"results to host; {e2e_iters} iterations in {e2e_time:.3f} s over {e2e_steps} fits"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "fp64_form": {"value": 1e3 / float(np.median(fp64_ms)), "unit": UNIT,
                      "split_speedup": value / ws / (1e3 / float(np.median(fp64_ms))),
                      "roofline": {"bound": "fp64", "kernel": "assign_fp64_kernel",
                                   "achieved": 1.5 * flop / (float(np.median(fp64_ms)) / 1e3) / 1e12,
                                   "peak": pipes["fp64_tflops"], "unit": "TFLOP/s",
                                   "frac": 1.5 * flop / (float(np.median(fp64_ms)) / 1e3) / 1e12 / pipes["fp64_tflops"],
                                   "note": "3 n k d FP64 operations (subtract, multiply, add: the reference's "
                                           "unfused order) per step over the whole step's time, against cuBLAS "
                                           "DGEMM's FMA rate"}},
        "pipe_peaks": pipes,
        "parity_vs_fp64_form": agree,
        "rescored_points": int(rescored),
        "incremental_sum_steps": int(incremental),
        "knn": knn,
        "many_problems": many,
        "large": large,
    }
    print(json.dumps(line), flush=True)
    h.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-knn", action="store_true", help="skip the kNN block of the JSON line")
    ap.add_argument("--lloyd-only", action="store_true",
                    help="time the device-resident Lloyd loop only (for profiler runs)")
    ap.add_argument("--knn-only", type=int, default=0, metavar="QUERIES",
                    help="time only the split-BF16 kNN find with this many queries (for profiler runs)")
    ap.add_argument("--neighbours-only", action="store_true",
                    help="time only the find_radius, DBSCAN and FastPair blocks (for profiler runs)")
    ap.add_argument("--no-large", action="store_true", help="skip the 16M x 128 block")
    ap.add_argument("--large-only", type=int, default=0, metavar="QUERIES",
                    help="run only the 16M x 128 block, with this many kNN queries")
    ap.add_argument("--many-only", action="store_true", help="run only the 512-problem block")
    ap.add_argument("--fp64-kernels", action="store_true",
                    help="run the FP64 form's assignment and kNN kernels once each (for profiler runs)")
    ap.add_argument("--peaks-only", action="store_true", help="measure the FP64 and FP32 GEMM rates only")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.knn_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(bench_knn(torch, 0, reps=2, n_query=args.knn_only, with_fp64=False)), flush=True)
        return
    if args.neighbours_only:
        import torch
        from smartcore_gb300.synthetic import knn_blobs_f32
        torch.cuda.set_device(0)
        xt, _, xq, _ = knn_blobs_f32(KNN_N, KNN_M, KNN_D)
        print(json.dumps({"find_radius": bench_radius(torch, 0, xt, xq), "dbscan": bench_dbscan(torch, xt),
                          "fastpair": bench_fastpair(torch, xt)}), flush=True)
        return
    if args.large_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(bench_large(torch, 0, n_query=args.large_only)), flush=True)
        return
    if args.fp64_kernels:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(bench_fp64_kernels(torch, 0)), flush=True)
        return
    if args.peaks_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(measure_pipe_peaks(torch, 0)), flush=True)
        return
    if args.many_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(bench_many_problems(torch)), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
