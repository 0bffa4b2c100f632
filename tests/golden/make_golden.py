"""Extract the known-answer tests of smartcore's hot path into a JSON fixture.

Reads the reference's own Rust test bodies (inputs and asserted answers) as
text and writes ``reference_kats.json`` beside this script.  Run it where the
smartcore sources are available:

    python tests/golden/make_golden.py <path to the smartcore source tree>

The GPU tests only read the JSON it wrote.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def fn_body(src, name):
    """Source text of `fn name() { ... }` (brace matched)."""
    m = re.search(r"fn\s+%s\s*\(\s*\)\s*\{" % re.escape(name), src)
    if not m:
        raise KeyError(name)
    i, depth = m.end(), 1
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    return src[m.end():i - 1]


def num(s):
    s = s.strip()
    if s.endswith("INFINITY"):
        return float("-inf") if s.startswith("-") else float("inf")
    s = re.sub(r"(f64|f32)$", "", s).replace("_", "")
    return float(s)


def rows(text):
    """All `&[a, b, ...]` or `vec![a, b]` row literals, in order."""
    out = []
    for m in re.finditer(r"(?:&|vec!)\[([^\[\]]*)\]", text):
        items = [t for t in m.group(1).split(",") if t.strip()]
        out.append([num(t) for t in items])
    return out


def main(root):
    kats = {"source": "smartcore 0.4.0 test bodies (paths relative to the crate root)"}

    src = read(root, "src/algorithm/neighbour/bbd_tree.rs")
    body = fn_body(src, "bbdtree_iris")
    data_txt = body[body.index("from_2d_array"):body.index(".unwrap()")]
    iris = rows(data_txt)
    cent_txt = re.search(r"let centroids = vec!\[(.*?)\];", body, re.S).group(1)
    cents = rows(cent_txt)
    memb = rows(re.search(r"let mut membership = (vec!\[.*?\]);", body, re.S).group(1))[0]
    counts = rows(re.search(r"let mut counts = (vec!\[.*?\]);", body, re.S).group(1))[0]
    asserts = re.findall(r"assert!\(\(\s*([a-z\[\]0-9]+)\s*-\s*([0-9.]+)\)\.abs\(\)\s*<\s*([0-9e.-]+)\)", body)
    memb_assert = re.search(r"assert_eq!\(membership\[(\d+)\],\s*(\d+)\)", body)
    kats["bbdtree_iris"] = {
        "cite": "src/algorithm/neighbour/bbd_tree.rs:323-364",
        "x": iris,
        "centroids": cents,
        "counts_in": counts,
        "membership_in": memb,
        "expect_close": [[a, float(b), float(t)] for a, b, t in asserts],
        "expect_membership": [int(memb_assert.group(1)), int(memb_assert.group(2))],
    }

    src = read(root, "src/cluster/kmeans.rs")
    body = fn_body(src, "fit_predict")
    kats["kmeans_fit_predict"] = {
        "cite": "src/cluster/kmeans.rs:472-505",
        "x": rows(body[body.index("from_2d_array"):body.index(".unwrap()")]),
        "params": {"k": 2, "max_iter": 100, "seed": None},
    }
    body = fn_body(src, "invalid_k")
    msg = re.search(r'"(Fit failed: invalid number of clusters: \d+)"', body).group(1)
    kats["kmeans_invalid_k"] = {
        "cite": "src/cluster/kmeans.rs:425-443",
        "x": rows(body[body.index("from_2d_array"):body.index(".unwrap()")]),
        "k_err": [0, 1],
        "message_k1": msg,
    }
    dflt = re.search(r"KMeansParameters\s*\{\s*k:\s*(\d+),\s*max_iter:\s*(\d+)", src)
    kats["kmeans_defaults"] = {"cite": "src/cluster/kmeans.rs:138-146",
                               "k": int(dflt.group(1)), "max_iter": int(dflt.group(2))}

    src = read(root, "src/algorithm/sort/heap_select.rs")
    heaps = []
    for name in ("test_add", "test_add1", "test_add2", "test_add_ordered"):
        body = fn_body(src, name)
        k = int(re.search(r"with_capacity\((\d+)\)", body).group(1))
        adds = [num(a) for a in re.findall(r"heap\.add\(([^)]*)\)", body)]
        n_expect = re.search(r"assert_eq!\((\d+),\s*heap\.n\)", body)
        got = re.search(r"assert_eq!\(vec!\[(.*?)\],\s*heap\.get\(\)\)", body).group(1)
        heaps.append({"name": name, "k": k, "adds": adds,
                      "n": int(n_expect.group(1)) if n_expect else len(adds),
                      "heap": [num(t) for t in got.split(",")]})
    kats["heap_select"] = {"cite": "src/algorithm/sort/heap_select.rs:103-178", "cases": heaps}

    src = read(root, "src/algorithm/neighbour/linear_search.rs")
    body = fn_body(src, "knn_find")
    data1 = rows(re.search(r"let data1 = (vec!\[.*?\]);", body, re.S).group(1))[0]
    f1 = re.search(r"\.find\(&(\d+),\s*(\d+)\)", body)
    e1 = rows(re.search(r"assert_eq!\((vec!\(.*?\)|vec!\[.*?\]),\s*found_idxs1\)", body).group(1).replace("vec!(", "vec![").replace(")", "]"))[0]
    fr = re.search(r"\.find_radius\(&(\d+),\s*([0-9.]+)\)", body)
    er = re.findall(r"assert_eq!\(vec!\((.*?)\),\s*found_idxs1\)", body)
    data2_txt = re.search(r"let data2 = vec!\[(.*?)\];", body, re.S).group(1)
    data2 = rows(data2_txt)
    f2 = re.search(r"\.find\(&vec!\[(.*?)\],\s*(\d+)\)", body)
    e2 = re.search(r"assert_eq!\(vec!\((.*?)\),\s*found_idxs2\)", body).group(1)
    kats["knn_find"] = {
        "cite": "src/algorithm/neighbour/linear_search.rs:150-195",
        "scalar": {"data": data1, "query": int(f1.group(1)), "k": int(f1.group(2)),
                   "expect_sorted_idx": [int(v) for v in e1]},
        "scalar_radius": {"query": int(fr.group(1)), "radius": float(fr.group(2)),
                          "expect_sorted_values": [int(v) for v in er[-1].split(",")]},
        "euclid": {"data": data2, "query": [num(t) for t in f2.group(1).split(",")],
                   "k": int(f2.group(2)), "expect_sorted_idx": [int(v) for v in e2.split(",")]},
    }

    src = read(root, "src/metrics/distance/euclidian.rs")
    body = fn_body(src, "squared_distance")
    a = rows(re.search(r"let a = (vec!\[.*?\]);", body).group(1))[0]
    b = rows(re.search(r"let b = (vec!\[.*?\]);", body).group(1))[0]
    exp = re.search(r"\(l2 - ([0-9.]+)\)\.abs\(\) < ([0-9e.-]+)", body)
    kats["euclidian_distance"] = {"cite": "src/metrics/distance/euclidian.rs:83-91", "a": a, "b": b,
                                  "expect": float(exp.group(1)), "tol": float(exp.group(2))}

    src = read(root, "src/neighbors/knn_classifier.rs")
    body = fn_body(src, "knn_fit_predict_weighted")
    xs = rows(body[body.index("from_2d_array"):body.index(".unwrap()")])
    y = rows(re.search(r"let y = (vec!\[.*?\]);", body).group(1))[0]
    k = int(re.search(r"with_k\((\d+)\)", body).group(1))
    q = rows(re.search(r"predict\(&DenseMatrix::from_2d_array\((.*?)\)", body, re.S).group(1))
    exp = rows(re.search(r"assert_eq!\((vec!\[.*?\]),\s*y_hat\)", body).group(1))[0]
    kats["knn_classifier_weighted"] = {"cite": "src/neighbors/knn_classifier.rs:327-344",
                                       "x": xs, "y": y, "k": k, "weight": "distance",
                                       "query": q, "expect": exp}
    body = fn_body(src, "knn_fit_predict")
    xs = rows(body[body.index("from_2d_array"):body.index(".unwrap()")])
    y = rows(re.search(r"let y = (vec!\[.*?\]);", body).group(1))[0]
    kats["knn_classifier_default"] = {"cite": "src/neighbors/knn_classifier.rs:311-321",
                                      "x": xs, "y": y, "k": 3, "weight": "uniform",
                                      "note": "reference default backend is CoverTree; the "
                                              "answer is backend independent (exact kNN)"}

    src = read(root, "src/neighbors/knn_regressor.rs")
    for name, key in (("knn_fit_predict_weighted", "knn_regressor_weighted"),
                      ("knn_fit_predict_uniform", "knn_regressor_uniform")):
        body = fn_body(src, name)
        xs = rows(body[body.index("from_2d_array"):body.index(".unwrap()")])
        y = rows(re.search(r"let y: Vec<f64> = (vec!\[.*?\]);", body).group(1))[0]
        yexp = rows(re.search(r"let y_exp = (\[.*?\]);", body).group(1).replace("[", "vec![", 1))[0]
        km = re.search(r"with_k\((\d+)\)", body)
        tol = re.search(r"\.abs\(\) < ([0-9e.-]+|std::f64::EPSILON)\)", body).group(1)
        kats[key] = {"cite": "src/neighbors/knn_regressor.rs:296-345", "x": xs, "y": y,
                     "k": int(km.group(1)) if km else 3,
                     "weight": "distance" if "Distance)" in body else "uniform",
                     "expect": yexp,
                     "tol": 2.220446049250313e-16 if "EPSILON" in tol else float(tol)}

    src = read(root, "src/cluster/dbscan.rs")
    body = fn_body(src, "fit_predict_dbscan")
    kats["dbscan_fit_predict"] = {
        "cite": "src/cluster/dbscan.rs:427-461",
        "x": rows(body[body.index("from_2d_array"):body.index(".unwrap()")]),
        "eps": float(re.search(r"with_eps\(([0-9.]+)\)", body).group(1)),
        "min_samples": int(re.search(r"with_min_samples\((\d+)\)", body).group(1)),
        "expect": [int(v) for v in re.search(r"let expected_labels = vec!\[(.*?)\];", body).group(1).split(",")],
        "errors": re.findall(r'Failed::fit\("(Invalid [^"]*)"\)', src),
    }

    src = read(root, "src/algorithm/neighbour/fastpair.rs")
    body = fn_body(src, "fastpair_new")
    entries = re.findall(r"\(\s*(\d+),\s*PairwiseDistance\s*\{\s*node:\s*(\d+),\s*neighbour:\s*Some\((\d+)\),"
                         r"\s*distance:\s*Some\(([^)]*)\),", body)
    closest = {}
    for name in ("fastpair_closest_pair", "one_dimensional_dataset_minimal", "one_dimensional_dataset_2"):
        b = fn_body(src, name)
        m = re.search(r"node:\s*(\d+),\s*neighbour:\s*Some\((\d+)\),\s*distance:\s*Some\(([^)]*)\)", b)
        closest[name] = {"x": rows(b[b.index("from_2d_array"):b.index(".unwrap()")]),
                         "expect": [int(m.group(1)), int(m.group(2)), num(m.group(3))]}
    kats["fastpair"] = {
        "cite": "src/algorithm/neighbour/fastpair.rs:270-510",
        "x": rows(body[body.index("from_2d_array"):body.index(".unwrap()")]),
        "distances": {int(k): [int(nd), int(nb), float("inf") if "MAX" in dv else num(dv)]
                      for k, nd, nb, dv in entries},
        "closest": closest,
        "error": re.search(r'"(min number of rows should be \d+)"', src).group(1),
    }

    out = os.path.join(HERE, "reference_kats.json")
    with open(out, "w") as f:
        json.dump(kats, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the smartcore source tree>")
    main(sys.argv[1])
