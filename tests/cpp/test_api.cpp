// The reference's known-answer tests for the distance-argmin path, written
// against the C++ host API (include/smartcore_gb300.hpp).  The data comes
// from tests/golden/reference_kats.json through the generated kats.inc.
// Run with --cpu-only to execute only the checks that fail before any device
// call (argument validation).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "smartcore_gb300.hpp"
#include "kats.inc"

using namespace smartcore;

static int failures = 0;
#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                     \
    }                                                                 \
  } while (0)

// src/cluster/kmeans.rs:426-443
static void invalid_k() {
  auto x = DenseMatrix<double>::from_2d_array(kats::invalid_k_x);
  bool threw = false;
  try {
    KMeans<double, int>::fit(x, KMeansParameters().with_k(0));
  } catch (const Failed &) {
    threw = true;
  }
  CHECK(threw);
  std::string msg;
  try {
    KMeans<double, int>::fit(x, KMeansParameters().with_k(1));
  } catch (const Failed &e) {
    msg = e.to_string();
  }
  CHECK(msg == kats::invalid_k_message);
  // knn_classifier.rs:243-248 and :237-241
  try {
    KNNClassifier<double, int>::fit(x, {1, 2}, KNNClassifierParameters().with_k(1));
    CHECK(false);
  } catch (const Failed &e) {
    CHECK(e.to_string() == "Fit failed: k should be > 1, k=[1]");
  }
  try {
    KNNClassifier<double, int>::fit(x, {1, 2, 3});
    CHECK(false);
  } catch (const Failed &e) {
    CHECK(e.to_string() == "Fit failed: Size of x should equal size of y; |x|=[2], |y|=[3]");
  }
}

// src/cluster/kmeans.rs:473-505
static void fit_predict(Form form) {
  auto x = DenseMatrix<double>::from_2d_array(kats::iris_x);
  auto kmeans = KMeans<double, size_t>::fit(x, KMeansParameters().with_form(form));
  auto y = kmeans.predict(x);
  CHECK(y.size() == 20);
  for (size_t i = 0; i < y.size(); ++i) CHECK(y[i] == kmeans.labels()[i]);
}

// src/algorithm/neighbour/linear_search.rs:150-195 (Euclidean part)
static void knn_find(Form form) {
  auto data = DenseMatrix<double>::from_2d_array(kats::knn_euclid_data);
  LinearKNNSearch<double> s(data, form);
  auto found = s.find(kats::knn_euclid_query, 3);
  std::vector<size_t> idx;
  for (auto &p : found) idx.push_back(p.first);
  std::sort(idx.begin(), idx.end());
  CHECK(idx == std::vector<size_t>({1, 2, 3}));
  bool threw = false;
  try {
    s.find(kats::knn_euclid_query, 0);
  } catch (const Failed &e) {
    threw = e.to_string() == "Find failed: k should be >= 1 and <= length(data)";
  }
  CHECK(threw);
  // find_radius (linear_search.rs:166-174): the values within radius 3 of 5
  std::vector<std::vector<double>> rows;
  for (double v : kats::knn_scalar_data) rows.push_back({v});
  LinearKNNSearch<double> s1(DenseMatrix<double>::from_2d_array(rows), form);
  std::vector<int> vals;
  for (auto &p : s1.find_radius({kats::knn_radius_query}, kats::knn_radius))
    vals.push_back((int)kats::knn_scalar_data[p.first]);
  std::sort(vals.begin(), vals.end());
  CHECK(vals == kats::knn_radius_expect);
}

// src/neighbors/knn_classifier.rs:311-344
static void knn_classifier(Form form) {
  auto x = DenseMatrix<double>::from_2d_array(kats::clf_x);
  std::vector<int> y(kats::clf_y.begin(), kats::clf_y.end());
  auto knn = KNNClassifier<double, int>::fit(x, y, KNNClassifierParameters().with_form(form));
  CHECK(knn.predict(x) == y);
  auto x1 = DenseMatrix<double>::from_2d_array(kats::clfw_x);
  std::vector<int> y1(kats::clfw_y.begin(), kats::clfw_y.end());
  auto knn1 = KNNClassifier<double, int>::fit(x1, y1,
                                              KNNClassifierParameters()
                                                  .with_k(5)
                                                  .with_algorithm(KNNAlgorithmName::LinearSearch)
                                                  .with_weight(KNNWeightFunction::Distance)
                                                  .with_form(form));
  CHECK(knn1.predict(DenseMatrix<double>::from_2d_array(kats::clfw_query)) == std::vector<int>({3}));
}

// src/neighbors/knn_regressor.rs:296-345
static void knn_regressor(Form form) {
  auto x = DenseMatrix<double>::from_2d_array(kats::reg_x);
  auto w = KNNRegressor<double>::fit(x, kats::reg_y,
                                     KNNRegressorParameters()
                                         .with_k(3)
                                         .with_algorithm(KNNAlgorithmName::LinearSearch)
                                         .with_weight(KNNWeightFunction::Distance)
                                         .with_form(form));
  auto yw = w.predict(x);
  for (size_t i = 0; i < yw.size(); ++i) CHECK(std::abs(yw[i] - kats::reg_w_expect[i]) < 2.220446049250313e-16);
  auto u = KNNRegressor<double>::fit(x, kats::reg_y, KNNRegressorParameters().with_form(form));
  auto yu = u.predict(x);
  for (size_t i = 0; i < yu.size(); ++i) CHECK(std::abs(yu[i] - kats::reg_u_expect[i]) < 1e-7);
}

static void dbscan(Form form) {
  // dbscan.rs:427-461 (fit_predict_dbscan)
  const auto x = DenseMatrix<double>::from_2d_array(kats::dbscan_x);
  DBSCANParameters p;
  p.form = form;
  const auto m = DBSCAN<double>::fit(x, p.with_eps(kats::dbscan_eps).with_min_samples(kats::dbscan_min_samples));
  const auto y = m.predict(x);
  CHECK(y.size() == kats::dbscan_expect.size());
  for (size_t i = 0; i < y.size(); ++i) CHECK(y[i] == kats::dbscan_expect[i]);
}

int main(int argc, char **argv) {
  const bool cpu_only = argc > 1 && std::strcmp(argv[1], "--cpu-only") == 0;
  invalid_k();
  if (!cpu_only) {
    for (Form f : {Form::FP64, Form::SplitBF16}) {
      fit_predict(f);
      knn_find(f);
      knn_classifier(f);
      knn_regressor(f);
      dbscan(f);
    }
  }
  std::printf("%s: %d failure(s)\n", cpu_only ? "cpu-only" : "all", failures);
  return failures ? 1 : 0;
}
