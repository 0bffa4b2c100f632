// C++ host API over the C ABI (include/smartcore_gb300.h), mirroring the
// smartcore 0.4.0 estimators on the distance-argmin path: same type names,
// parameter structs with the same fields, defaults and builder methods, the
// same validation order and error messages, and Result-style errors
// (Failed with FailedError kinds, displayed "{err}: {msg}").
//
//   smartcore::KMeans<double, int64_t>::fit(x, smartcore::KMeansParameters().with_k(2))
//   smartcore::KNNClassifier<double, int>::fit(x, y, params)
//
// Header-only; link with libsmartcore_gb300.so.  Every compute call needs a
// GB300 (sm_103) device: there is no CPU fallback.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <type_traits>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "smartcore_gb300.h"

namespace smartcore {

// src/error/mod.rs:16-37
enum class FailedError {
  FitFailed = 1,
  PredictFailed,
  TransformFailed,
  FindFailed,
  DecompositionFailed,
  SolutionFailed,
  ParametersError,
  InvalidStateError,
};

inline const char *to_string(FailedError e) {  // src/error/mod.rs:108-122
  switch (e) {
    case FailedError::FitFailed: return "Fit failed";
    case FailedError::PredictFailed: return "Predict failed";
    case FailedError::TransformFailed: return "Transform failed";
    case FailedError::FindFailed: return "Find failed";
    case FailedError::DecompositionFailed: return "Decomposition failed";
    case FailedError::SolutionFailed: return "Can't find solution";
    case FailedError::ParametersError: return "Error in input, check parameters";
    case FailedError::InvalidStateError: return "Invalid state, this should never happen";
  }
  return "";
}

// src/error/mod.rs:11-14, Display at :124-128
class Failed : public std::runtime_error {
 public:
  Failed(FailedError err, std::string msg)
      : std::runtime_error(std::string(::smartcore::to_string(err)) + ": " + msg), err_(err), msg_(std::move(msg)) {}
  static Failed fit(const std::string &m) { return Failed(FailedError::FitFailed, m); }
  static Failed predict(const std::string &m) { return Failed(FailedError::PredictFailed, m); }
  static Failed because(FailedError e, const std::string &m) { return Failed(e, m); }
  FailedError error() const { return err_; }
  const std::string &msg() const { return msg_; }
  std::string to_string() const { return what(); }
  bool operator==(const Failed &o) const { return err_ == o.err_ && msg_ == o.msg_; }

 private:
  FailedError err_;
  std::string msg_;
};

namespace detail {
inline void check(sc_status s, FailedError kind) {
  if (s == SC_OK) return;
  const std::string m = sc_last_error();
  if (s == SC_ERR_INVALID) throw Failed(kind, m);
  throw Failed(FailedError::InvalidStateError, "[status " + std::to_string(s) + "] " + m);
}
template <class T>
constexpr int32_t dtype() {
  static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                "the GPU path serves f32 and f64 matrices");
  return std::is_same<T, float>::value ? SC_F32 : SC_F64;
}
}  // namespace detail

// DenseMatrix (src/linalg/basic/matrix.rs:24-32, :187-238): column-major by
// default; element (i, j) as in DenseMatrix::get (:367-381).
template <class T>
class DenseMatrix {
 public:
  DenseMatrix(size_t nrows, size_t ncols, std::vector<T> values, bool column_major)
      : nrows_(nrows), ncols_(ncols), values_(std::move(values)), column_major_(column_major) {
    if (nrows * ncols != values_.size())
      throw Failed(FailedError::ParametersError,
                   "The specified shape: (cols: " + std::to_string(ncols) + ", rows: " + std::to_string(nrows) +
                       ") does not align with data len: " + std::to_string(values_.size()));
  }
  static DenseMatrix from_2d_vec(const std::vector<std::vector<T>> &rows) {
    if (rows.empty() || rows[0].empty())
      throw Failed(FailedError::ParametersError, "The 2d vec provided is empty; cannot instantiate the matrix");
    const size_t r = rows.size(), c = rows[0].size();
    std::vector<T> v;
    v.reserve(r * c);
    for (size_t j = 0; j < c; ++j)
      for (size_t i = 0; i < r; ++i) v.push_back(rows[i][j]);
    return DenseMatrix(r, c, std::move(v), true);
  }
  static DenseMatrix from_2d_array(const std::vector<std::vector<T>> &rows) { return from_2d_vec(rows); }
  std::pair<size_t, size_t> shape() const { return {nrows_, ncols_}; }
  const T &get(size_t i, size_t j) const {
    return column_major_ ? values_[j * nrows_ + i] : values_[i * ncols_ + j];
  }
  const T *data() const { return values_.data(); }
  bool column_major() const { return column_major_; }
  int32_t layout() const { return column_major_ ? SC_COL_MAJOR : SC_ROW_MAJOR; }
  int64_t ld() const { return (int64_t)(column_major_ ? nrows_ : ncols_); }

 private:
  size_t nrows_, ncols_;
  std::vector<T> values_;
  bool column_major_;
};

enum class Form { FP64 = SC_FORM_FP64, SplitBF16 = SC_FORM_SPLIT_BF16 };

// KMeansParameters (src/cluster/kmeans.rs:109-146).  form and rng are
// extensions: the arithmetic form (identical results) and which rand 0.8
// generator get_rng_impl would use (SmallRng unless std_rand).
struct KMeansParameters {
  size_t k = 2;
  size_t max_iter = 100;
  std::optional<uint64_t> seed;
  Form form = Form::FP64;
  int32_t rng = SC_RNG_SMALL;
  KMeansParameters with_k(size_t v) const { auto p = *this; p.k = v; return p; }
  KMeansParameters with_max_iter(size_t v) const { auto p = *this; p.max_iter = v; return p; }
  KMeansParameters with_seed(uint64_t v) const { auto p = *this; p.seed = v; return p; }
  KMeansParameters with_form(Form f) const { auto p = *this; p.form = f; return p; }
};

// KMeans (src/cluster/kmeans.rs:73-83, fit :254-323, predict :327-352).
template <class TX, class TY>
class KMeans {
 public:
  static KMeans fit(const DenseMatrix<TX> &x, const KMeansParameters &p = KMeansParameters()) {
    if (p.k < 2) throw Failed::fit("invalid number of clusters: " + std::to_string(p.k));
    if (p.max_iter == 0) throw Failed::fit("invalid maximum number of iterations: " + std::to_string(p.max_iter));
    const auto [n, d] = x.shape();
    int64_t first = 0;
    std::vector<double> u(p.k - 1 > 0 ? p.k - 1 : 1);
    detail::check(sc_kmeanspp_draws(p.rng, p.seed.value_or(0), (int64_t)n, (int64_t)p.k, &first, u.data()),
                  FailedError::FitFailed);
    KMeans m;
    m.k_ = p.k;
    m.d_ = d;
    m.form_ = p.form;
    m.centroids_.assign(p.k * d, 0.0);
    m.size_.assign(p.k, 0);
    std::vector<int64_t> labels(n);
    int64_t iters = 0;
    detail::check(sc_kmeans_fit(x.data(), detail::dtype<TX>(), x.layout(), (int64_t)n, (int64_t)d, x.ld(),
                                (int64_t)p.k, (int64_t)p.max_iter, first, u.data(), (int32_t)p.form,
                                m.centroids_.data(), m.size_.data(), labels.data(), &m.distortion_, &iters),
                  FailedError::FitFailed);
    m.y_.assign(labels.begin(), labels.end());
    m.iters_ = (size_t)iters;
    return m;
  }

  std::vector<TY> predict(const DenseMatrix<TX> &x) const {
    const auto [n, d] = x.shape();
    std::vector<int64_t> labels(n);
    detail::check(sc_kmeans_predict(x.data(), detail::dtype<TX>(), x.layout(), (int64_t)n, (int64_t)d, x.ld(),
                                    centroids_.data(), (int64_t)k_, (int32_t)form_, labels.data()),
                  FailedError::PredictFailed);
    return std::vector<TY>(labels.begin(), labels.end());
  }

  // kmeans.rs:85-107: k, size, centroids within f64::EPSILON
  bool operator==(const KMeans &o) const {
    if (k_ != o.k_ || size_ != o.size_ || centroids_.size() != o.centroids_.size()) return false;
    for (size_t i = 0; i < centroids_.size(); ++i)
      if (std::abs(centroids_[i] - o.centroids_[i]) > 2.220446049250313e-16) return false;
    return true;
  }

  size_t k() const { return k_; }
  const std::vector<int64_t> &size() const { return size_; }
  const std::vector<size_t> &labels() const { return y_; }  // the fitted `_y`
  double distortion() const { return distortion_; }
  size_t iterations() const { return iters_; }
  std::vector<double> centroid(size_t i) const {
    return std::vector<double>(centroids_.begin() + i * d_, centroids_.begin() + (i + 1) * d_);
  }

 private:
  size_t k_ = 0, d_ = 0, iters_ = 0;
  Form form_ = Form::FP64;
  std::vector<size_t> y_;
  std::vector<int64_t> size_;
  double distortion_ = 0.0;
  std::vector<double> centroids_;
};

// src/algorithm/neighbour/mod.rs:53-59.  Both names run the GPU brute-force
// search, which returns the exact k nearest neighbours.
enum class KNNAlgorithmName { LinearSearch, CoverTree };
// src/neighbors/mod.rs:53-59
enum class KNNWeightFunction { Uniform = SC_KNN_UNIFORM, Distance = SC_KNN_DISTANCE };

// LinearKNNSearch (src/algorithm/neighbour/linear_search.rs:36-84) over the
// rows of a matrix, resident on the device.
template <class T>
class LinearKNNSearch {
 public:
  explicit LinearKNNSearch(const DenseMatrix<T> &data, Form form = Form::FP64) : form_(form) {
    const auto [n, d] = data.shape();
    n_ = n;
    d_ = d;
    detail::check(sc_knn_create(data.data(), detail::dtype<T>(), data.layout(), SC_MEM_HOST, (int64_t)n,
                                (int64_t)d, data.ld(), &h_),
                  FailedError::FitFailed);
  }
  LinearKNNSearch(const LinearKNNSearch &) = delete;
  LinearKNNSearch &operator=(const LinearKNNSearch &) = delete;
  ~LinearKNNSearch() { sc_knn_destroy(h_); }

  // find() for one query: (index, distance) pairs in the heap-array order,
  // entries whose index is None dropped (linear_search.rs:79-83).
  std::vector<std::pair<size_t, double>> find(const std::vector<T> &from, size_t k) const {
    if (from.size() != d_) throw std::invalid_argument("Input vector sizes are different.");
    std::vector<int64_t> idx(k ? k : 1);
    std::vector<double> dist(k ? k : 1);
    detail::check(sc_knn_find(h_, from.data(), SC_ROW_MAJOR, SC_MEM_HOST, 1, (int64_t)d_, (int64_t)k,
                              (int32_t)form_, SC_MEM_HOST, idx.data(), dist.data()),
                  FailedError::FindFailed);
    std::vector<std::pair<size_t, double>> out;
    for (size_t s = 0; s < k; ++s)
      if (idx[s] >= 0) out.emplace_back((size_t)idx[s], dist[s]);
    return out;
  }

  // find_radius() for one query (linear_search.rs:89-108): (index, distance)
  // of every row with distance <= radius, in index order.
  // The output is sized from the previous call's row count, so one library
  // call (a counting and a filling pass) usually serves; when the rows do not
  // fit, a second call with the exact size does.
  std::vector<std::pair<size_t, double>> find_radius(const std::vector<T> &from, double radius) const {
    if (from.size() != d_) throw std::invalid_argument("Input vector sizes are different.");
    int64_t count = 0, total = 0;
    const int64_t cap = (int64_t)radius_rows_;
    std::vector<int64_t> idx((size_t)cap);
    std::vector<double> dist((size_t)cap);
    const sc_status st = sc_knn_find_radius(h_, from.data(), SC_ROW_MAJOR, SC_MEM_HOST, 1, (int64_t)d_, radius,
                                            (int32_t)form_, &count, cap, idx.data(), dist.data(), &total);
    if (st != SC_OK && !(st == SC_ERR_INVALID && total > cap)) detail::check(st, FailedError::FindFailed);
    if (total > cap) {
      idx.resize((size_t)total);
      dist.resize((size_t)total);
      detail::check(sc_knn_find_radius(h_, from.data(), SC_ROW_MAJOR, SC_MEM_HOST, 1, (int64_t)d_, radius,
                                       (int32_t)form_, &count, total, idx.data(), dist.data(), &total),
                    FailedError::FindFailed);
    }
    radius_rows_ = std::max<size_t>(64, (size_t)(total + total / 4 + 1));
    std::vector<std::pair<size_t, double>> out;
    for (int64_t s = 0; s < total; ++s) out.emplace_back((size_t)idx[s], dist[s]);
    return out;
  }

  sc_knn *handle() const { return h_; }
  Form form() const { return form_; }
  size_t len() const { return n_; }

 private:
  sc_knn *h_ = nullptr;
  Form form_;
  size_t n_ = 0, d_ = 0;
  mutable size_t radius_rows_ = 256;  // find_radius: the output's first size
};

// KNNClassifierParameters (src/neighbors/knn_classifier.rs:48-69, :144-154).
struct KNNClassifierParameters {
  KNNAlgorithmName algorithm = KNNAlgorithmName::CoverTree;
  KNNWeightFunction weight = KNNWeightFunction::Uniform;
  size_t k = 3;
  Form form = Form::FP64;
  KNNClassifierParameters with_k(size_t v) const { auto p = *this; p.k = v; return p; }
  KNNClassifierParameters with_algorithm(KNNAlgorithmName a) const { auto p = *this; p.algorithm = a; return p; }
  KNNClassifierParameters with_weight(KNNWeightFunction w) const { auto p = *this; p.weight = w; return p; }
  KNNClassifierParameters with_form(Form f) const { auto p = *this; p.form = f; return p; }
};
using KNNRegressorParameters = KNNClassifierParameters;

// KNNClassifier (src/neighbors/knn_classifier.rs:74-89, fit :216-260,
// predict :265-299); the vote runs on the device in the heap order.
template <class TX, class TY>
class KNNClassifier {
 public:
  static KNNClassifier fit(const DenseMatrix<TX> &x, const std::vector<TY> &y,
                           const KNNClassifierParameters &p = KNNClassifierParameters()) {
    KNNClassifier m;
    m.classes_ = y;  // y.unique(): sorted, deduplicated (src/linalg/basic/arrays.rs:223-231)
    std::sort(m.classes_.begin(), m.classes_.end());
    m.classes_.erase(std::unique(m.classes_.begin(), m.classes_.end()), m.classes_.end());
    m.y_.resize(y.size());
    for (size_t i = 0; i < y.size(); ++i)
      m.y_[i] = std::lower_bound(m.classes_.begin(), m.classes_.end(), y[i]) - m.classes_.begin();
    const size_t x_n = x.shape().first;
    if (x_n != y.size())
      throw Failed::fit("Size of x should equal size of y; |x|=[" + std::to_string(x_n) + "], |y|=[" +
                        std::to_string(y.size()) + "]");
    if (p.k <= 1) throw Failed::fit("k should be > 1, k=[" + std::to_string(p.k) + "]");
    m.k_ = p.k;
    m.weight_ = p.weight;
    m.knn_.reset(new LinearKNNSearch<TX>(x, p.form));
    return m;
  }

  std::vector<TY> predict(const DenseMatrix<TX> &x) const {
    const auto [m, d] = x.shape();
    std::vector<int64_t> cls(m);
    detail::check(sc_knn_classify(knn_->handle(), x.data(), x.layout(), SC_MEM_HOST, (int64_t)m, x.ld(),
                                  (int64_t)k_, (int32_t)knn_->form(), (int32_t)weight_, y_.data(),
                                  (int64_t)classes_.size(), cls.data()),
                  FailedError::PredictFailed);
    std::vector<TY> out(m);
    for (size_t i = 0; i < m; ++i) out[i] = classes_[(size_t)cls[i]];
    return out;
  }

 private:
  std::vector<TY> classes_;
  std::vector<int64_t> y_;
  size_t k_ = 3;
  KNNWeightFunction weight_ = KNNWeightFunction::Uniform;
  std::shared_ptr<LinearKNNSearch<TX>> knn_;
};

// KNNRegressor (src/neighbors/knn_regressor.rs fit :212-249, predict :254-282).
template <class TX>
class KNNRegressor {
 public:
  static KNNRegressor fit(const DenseMatrix<TX> &x, const std::vector<double> &y,
                          const KNNRegressorParameters &p = KNNRegressorParameters()) {
    const size_t x_n = x.shape().first;
    if (x_n != y.size())
      throw Failed::fit("Size of x should equal size of y; |x|=[" + std::to_string(x_n) + "], |y|=[" +
                        std::to_string(y.size()) + "]");
    if (p.k < 1) throw Failed::fit("k should be > 0, k=[" + std::to_string(p.k) + "]");
    KNNRegressor m;
    m.y_ = y;
    m.k_ = p.k;
    m.weight_ = p.weight;
    m.knn_.reset(new LinearKNNSearch<TX>(x, p.form));
    return m;
  }

  std::vector<double> predict(const DenseMatrix<TX> &x) const {
    const auto [m, d] = x.shape();
    std::vector<double> out(m);
    detail::check(sc_knn_regress(knn_->handle(), x.data(), x.layout(), SC_MEM_HOST, (int64_t)m, x.ld(),
                                 (int64_t)k_, (int32_t)knn_->form(), (int32_t)weight_, y_.data(), out.data()),
                  FailedError::PredictFailed);
    return out;
  }

 private:
  std::vector<double> y_;
  size_t k_ = 3;
  KNNWeightFunction weight_ = KNNWeightFunction::Uniform;
  std::shared_ptr<LinearKNNSearch<TX>> knn_;
};

// DBSCANParameters (src/cluster/dbscan.rs:79-96, defaults :239-249); the
// device always searches linearly (neighbourhoods in index order).
struct DBSCANParameters {
  size_t min_samples = 5;
  double eps = 0.5;
  Form form = Form::SplitBF16;
  DBSCANParameters &with_min_samples(size_t v) { min_samples = v; return *this; }
  DBSCANParameters &with_eps(double v) { eps = v; return *this; }
};

// DBSCAN::fit / predict (src/cluster/dbscan.rs:274-398).
template <typename T>
class DBSCAN {
 public:
  static DBSCAN fit(const DenseMatrix<T> &x, const DBSCANParameters &p = DBSCANParameters()) {
    if (p.min_samples < 1) throw Failed::fit("Invalid minPts");
    if (!(p.eps > 0)) throw Failed::fit("Invalid radius: ");
    DBSCAN m(x, p);
    const size_t n = m.search_->len();
    m.labels_.assign(n ? n : 1, 0);
    int64_t k = 0;
    detail::check(sc_dbscan_fit(m.search_->handle(), p.eps, (int64_t)p.min_samples, (int32_t)p.form,
                                m.labels_.data(), &k),
                  FailedError::FitFailed);
    m.labels_.resize(n);
    m.k_ = k;
    return m;
  }

  // cluster + 1 per row, 0 for noise
  std::vector<int64_t> predict(const DenseMatrix<T> &x) const {
    const auto [m, d] = x.shape();
    std::vector<int64_t> out(m ? m : 1);
    detail::check(sc_dbscan_predict(search_->handle(), x.data(), x.layout(), SC_MEM_HOST, (int64_t)m, x.ld(),
                                    eps_, (int32_t)form_, labels_.data(), k_, out.data()),
                  FailedError::PredictFailed);
    out.resize(m);
    return out;
  }

  const std::vector<int64_t> &cluster_labels() const { return labels_; }
  size_t num_classes() const { return (size_t)k_; }

 private:
  DBSCAN(const DenseMatrix<T> &x, const DBSCANParameters &p)
      : search_(std::make_shared<LinearKNNSearch<T>>(x, p.form)), eps_(p.eps), form_(p.form) {}
  std::shared_ptr<LinearKNNSearch<T>> search_;
  std::vector<int64_t> labels_;
  int64_t k_ = 0;
  double eps_;
  Form form_;
};

}  // namespace smartcore
