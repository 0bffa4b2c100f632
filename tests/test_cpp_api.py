"""Builds and runs tests/cpp/test_api.cpp: the reference's known-answer tests
written against the C++ host API, data generated from the golden fixture."""
import json
import os
import subprocess

import pytest

from smartcore_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _vec2(rows):
    return "{" + ", ".join("{" + ", ".join(repr(float(v)) for v in r) + "}" for r in rows) + "}"


def _vec(vals, ty="double"):
    return "{" + ", ".join(repr(ty == "double" and float(v) or int(v)) for v in vals) + "}"


def write_kats(path):
    with open(os.path.join(ROOT, "tests", "golden", "reference_kats.json")) as f:
        k = json.load(f)
    e = k["knn_find"]["euclid"]
    lines = [
        "#pragma once",
        "#include <string>",
        "#include <vector>",
        "namespace kats {",
        f"static const std::vector<std::vector<double>> invalid_k_x = {_vec2(k['kmeans_invalid_k']['x'])};",
        f"static const std::string invalid_k_message = {json.dumps(k['kmeans_invalid_k']['message_k1'])};",
        f"static const std::vector<std::vector<double>> iris_x = {_vec2(k['kmeans_fit_predict']['x'])};",
        f"static const std::vector<std::vector<double>> knn_euclid_data = {_vec2(e['data'])};",
        f"static const std::vector<double> knn_euclid_query = {_vec(e['query'])};",
        f"static const std::vector<double> knn_scalar_data = {_vec(k['knn_find']['scalar']['data'])};",
        f"static const double knn_radius_query = {float(k['knn_find']['scalar_radius']['query'])!r};",
        f"static const double knn_radius = {float(k['knn_find']['scalar_radius']['radius'])!r};",
        f"static const std::vector<int> knn_radius_expect = {_vec(k['knn_find']['scalar_radius']['expect_sorted_values'], 'int')};",
        f"static const std::vector<std::vector<double>> clf_x = {_vec2(k['knn_classifier_default']['x'])};",
        f"static const std::vector<int> clf_y = {_vec(k['knn_classifier_default']['y'], 'int')};",
        f"static const std::vector<std::vector<double>> clfw_x = {_vec2(k['knn_classifier_weighted']['x'])};",
        f"static const std::vector<int> clfw_y = {_vec(k['knn_classifier_weighted']['y'], 'int')};",
        f"static const std::vector<std::vector<double>> clfw_query = {_vec2(k['knn_classifier_weighted']['query'])};",
        f"static const std::vector<std::vector<double>> reg_x = {_vec2(k['knn_regressor_weighted']['x'])};",
        f"static const std::vector<double> reg_y = {_vec(k['knn_regressor_weighted']['y'])};",
        f"static const std::vector<double> reg_w_expect = {_vec(k['knn_regressor_weighted']['expect'])};",
        f"static const std::vector<double> reg_u_expect = {_vec(k['knn_regressor_uniform']['expect'])};",
        f"static const std::vector<std::vector<double>> dbscan_x = {_vec2(k['dbscan_fit_predict']['x'])};",
        f"static const double dbscan_eps = {float(k['dbscan_fit_predict']['eps'])!r};",
        f"static const int dbscan_min_samples = {int(k['dbscan_fit_predict']['min_samples'])};",
        f"static const std::vector<long> dbscan_expect = {_vec(k['dbscan_fit_predict']['expect'], 'long')};",
        "}",
    ]
    with open(os.path.join(path, "kats.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")


@pytest.fixture(scope="module")
def test_binary(tmp_path_factory):
    lib = build.build()
    d = tmp_path_factory.mktemp("cpp")
    write_kats(str(d))
    exe = os.path.join(str(d), "test_api")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", str(d),
                    os.path.join(ROOT, "tests", "cpp", "test_api.cpp"), "-o", exe, lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_cpp_api_validation(test_binary):
    r = subprocess.run([test_binary, "--cpu-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout


@pytest.mark.gpu
def test_cpp_api_reference_kats(test_binary):
    r = subprocess.run([test_binary], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
