// frovedis_gb300.hpp — C++ host API with the reference's names and
// signatures for the sparse logistic-regression path, running on one GB300
// through the C ABI of fvg.h.  A caller of frovedis's local matrices and
// logistic-regression trainers can switch by including this header and
// linking libfvg.so:
//
//   crs_matrix_local<T,I,O>            matrix/crs_matrix.hpp:240-331
//     operator*(crs_matrix_local, std::vector<T>)     crs_matrix.hpp:1518-1525
//     crs_matrix_local::transpose()                   crs_matrix.hpp:404-412
//     operator*(crs_matrix_local, rowmajor_matrix_local) crs_matrix.hpp:2053-2064
//   ell_matrix_local<T,I>              ell_matrix.hpp:11-95, operator* 229, trans_mv 357
//   jds_matrix_local<T,I,O,P>          jds_matrix.hpp:15-146, operator* 419-426
//   jds_crs_hybrid_local<T,I,O,P>      jds_crs_hybrid.hpp:8-153, operator* 213-221
//   logistic_regression_model<T>       ml/glm/linear_model.hpp:306-446
//   logistic_regression_with_lbfgs::train   ml/glm/logistic_regression_with_lbfgs.hpp:8-437
//   logistic_regression_with_sgd::train     ml/glm/logistic_regression_with_sgd.hpp:8-441
//   multinomial_logistic_regression::train  ml/glm/multinomial_logistic_regression.hpp:8-378
//   multinomial_logistic_regression_model<T> ml/glm/multinomial_logistic_regression_model.hpp:10-258
//   MatType, RegType                   ml/utility/mattype.hpp:6-11, ml/glm/regularizer.hpp:8-12
//
// The matrices keep the reference's public fields (val, idx, off, perm,
// local_num_row, local_num_col) filled in the reference's array order; the
// products and the training run on the device.  Errors surface as the
// reference's exception types: std::runtime_error for operator* size
// mismatches, frovedis_gb300::error (a std::runtime_error) otherwise, with
// the reference's messages.  Index types must hold values below 2^31.
#ifndef FROVEDIS_GB300_HPP
#define FROVEDIS_GB300_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fvg.h"

namespace frovedis_gb300 {

struct error : std::runtime_error {
  fvg_status code;
  error(fvg_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// One context per process (device 0 unless FVG_DEVICE selects another).
inline fvg_ctx* context() {
  static std::unique_ptr<fvg_ctx, void (*)(fvg_ctx*)> ctx(nullptr, fvg_ctx_destroy);
  if (!ctx) {
    int dev = 0;
    if (const char* e = std::getenv("FVG_DEVICE")) dev = std::atoi(e);
    fvg_ctx* c = nullptr;
    fvg_status st = fvg_ctx_create(dev, &c);
    if (st != FVG_OK) throw error(st, "no usable CUDA device for the GB300 sparse path");
    ctx.reset(c);
  }
  return ctx.get();
}

inline void check(fvg_status st) {
  if (st != FVG_OK) throw error(st, fvg_ctx_last_error(context()));
}

template <class T> struct dtype_of;
template <> struct dtype_of<double> { static constexpr fvg_dtype value = FVG_F64; };
template <> struct dtype_of<float> { static constexpr fvg_dtype value = FVG_F32; };

template <class V> std::vector<int32_t> to_i32(const std::vector<V>& v) {
  std::vector<int32_t> r(v.size());
  for (size_t i = 0; i < v.size(); i++) {
    if (v[i] > (V)2147483647) throw error(FVG_ERR_INVALID_ARG, "index does not fit in 32 bits");
    r[i] = (int32_t)v[i];
  }
  return r;
}

// RAII device copy of a host CRS matrix.
struct device_matrix {
  fvg_matrix* h = nullptr;
  template <class M> explicit device_matrix(const M& m) {
    auto off = to_i32(m.off);
    auto idx = to_i32(m.idx);
    if (off.empty()) off.push_back(0);
    check(fvg_matrix_create_crs(context(), (int64_t)m.local_num_row, (int64_t)m.local_num_col, off.data(),
                                idx.data(), m.val.data(), dtype_of<typename M::value_type>::value, 0, &h));
  }
  device_matrix(const device_matrix&) = delete;
  device_matrix& operator=(const device_matrix&) = delete;
  ~device_matrix() { fvg_matrix_destroy(h); }
};

}  // namespace frovedis_gb300

namespace frovedis {

enum MatType { CRS = 0, JDS, ELL, HYBRID };
enum RegType { ZERO = 0, L1, L2 };
enum { NONE = 0xDEAD };  // cleared threshold (ml/utility/mattype.hpp:13)

template <class T> struct rowmajor_matrix_local {
  rowmajor_matrix_local() : local_num_row(0), local_num_col(0) {}
  rowmajor_matrix_local(size_t r, size_t c) : val(r * c), local_num_row(r), local_num_col(c) {}
  std::vector<T> val;
  size_t local_num_row, local_num_col;
};

template <class T, class I = size_t, class O = size_t>
struct crs_matrix_local {
  crs_matrix_local() : local_num_row(0), local_num_col(0) { off.push_back(0); }
  crs_matrix_local(size_t nrows, size_t ncols) : local_num_row(nrows), local_num_col(ncols) { off.push_back(0); }
  std::vector<T> val;
  std::vector<I> idx;
  std::vector<O> off;  // local_num_row + 1 entries, off[0] = 0
  size_t local_num_row;
  size_t local_num_col;
  typedef T value_type;
  typedef I index_type;
  typedef O offset_type;
  // transpose_compressed_matrix semantics (stable by row), built on the device
  crs_matrix_local<T, I, O> transpose() const {
    frovedis_gb300::device_matrix d(*this);
    std::vector<int32_t> toff(local_num_col + 1), tidx(val.size());
    std::vector<double> tval(val.size());
    frovedis_gb300::check(fvg_matrix_get_transpose(frovedis_gb300::context(), d.h, toff.data(), tidx.data(),
                                                   tval.data()));
    crs_matrix_local<T, I, O> t(local_num_col, local_num_row);
    t.off.assign(toff.begin(), toff.end());
    t.idx.assign(tidx.begin(), tidx.end());
    t.val.assign(tval.begin(), tval.end());
    return t;
  }
  void clear() {
    val.clear(); idx.clear(); off.assign(1, 0);
    local_num_row = local_num_col = 0;
  }
};

namespace detail {
template <class T, class M>
std::vector<T> product(const M& crs, const std::vector<T>& v, fvg_format fmt, bool trans) {
  const size_t nin = trans ? crs.local_num_row : crs.local_num_col;
  const size_t nout = trans ? crs.local_num_col : crs.local_num_row;
  if (v.size() != nin) throw std::runtime_error("operator*: size of vector does not match");
  std::vector<T> ret(nout);
  if (crs.local_num_row == 0 || crs.local_num_col == 0) return ret;
  frovedis_gb300::device_matrix d(crs);
  const fvg_dtype dt = frovedis_gb300::dtype_of<T>::value;
  frovedis_gb300::check((trans ? fvg_trans_mv : fvg_spmv)(frovedis_gb300::context(), d.h, fmt, dt, dt, v.data(),
                                                          ret.data(), 0));
  return ret;
}
}  // namespace detail

template <class T, class I, class O>
std::vector<T> operator*(const crs_matrix_local<T, I, O>& mat, const std::vector<T>& v) {
  return detail::product<T>(mat, v, FVG_CRS, false);
}

template <class T, class I, class O>
rowmajor_matrix_local<T> operator*(const crs_matrix_local<T, I, O>& mat, const rowmajor_matrix_local<T>& v) {
  if (mat.local_num_col != v.local_num_row) throw std::runtime_error("invalid size for matrix multiplication");
  rowmajor_matrix_local<T> ret(mat.local_num_row, v.local_num_col);
  if (mat.local_num_row == 0 || v.local_num_col == 0) return ret;
  frovedis_gb300::device_matrix d(mat);
  const fvg_dtype dt = frovedis_gb300::dtype_of<T>::value;
  frovedis_gb300::check(fvg_spmm(frovedis_gb300::context(), d.h, FVG_CRS, dt, dt, v.val.data(),
                                 (int64_t)v.local_num_col, ret.val.data(), 0));
  return ret;
}

// ELL (column-major, padded to the longest row), built from CRS on the device.
template <class T, class I = size_t>
struct ell_matrix_local {
  ell_matrix_local() : local_num_row(0), local_num_col(0) {}
  template <class O> explicit ell_matrix_local(const crs_matrix_local<T, I, O>& crs) : src(new crs_matrix_local<T, I, size_t>()) {
    local_num_row = crs.local_num_row;
    local_num_col = crs.local_num_col;
    src->val = crs.val;
    src->idx = crs.idx;
    src->off.assign(crs.off.begin(), crs.off.end());
    src->local_num_row = crs.local_num_row;
    src->local_num_col = crs.local_num_col;
    if (local_num_row == 0) { local_num_col = 0; return; }
    frovedis_gb300::device_matrix d(*src);
    int64_t w = 0;
    frovedis_gb300::check(fvg_matrix_get_ell(frovedis_gb300::context(), d.h, &w, nullptr, nullptr));
    std::vector<int32_t> ei((size_t)w * local_num_row);
    std::vector<double> ev((size_t)w * local_num_row);
    frovedis_gb300::check(fvg_matrix_get_ell(frovedis_gb300::context(), d.h, &w, ei.data(), ev.data()));
    idx.assign(ei.begin(), ei.end());
    val.assign(ev.begin(), ev.end());
  }
  std::vector<T> val;
  std::vector<I> idx;
  size_t local_num_row, local_num_col;
  std::shared_ptr<crs_matrix_local<T, I, size_t>> src;  // the CRS it was built from (device products)
};

template <class T, class I>
std::vector<T> operator*(const ell_matrix_local<T, I>& mat, const std::vector<T>& v) {
  if (!mat.src) return std::vector<T>(mat.local_num_row);
  return detail::product<T>(*mat.src, v, FVG_ELL, false);
}
template <class T, class I>
std::vector<T> trans_mv(const ell_matrix_local<T, I>& mat, const std::vector<T>& v) {
  if (!mat.src) return std::vector<T>(mat.local_num_col);
  return detail::product<T>(*mat.src, v, FVG_ELL, true);
}

// JDS: rows sorted by length (descending, ties by descending row id).
template <class T, class I = size_t, class O = size_t, class P = size_t>
struct jds_matrix_local {
  jds_matrix_local() : local_num_col(0), local_num_row(0) { off.push_back(0); }
  explicit jds_matrix_local(const crs_matrix_local<T, I, O>& m) : src(new crs_matrix_local<T, I, size_t>()) {
    local_num_col = m.local_num_col;
    local_num_row = m.local_num_row;
    src->val = m.val; src->idx = m.idx; src->off.assign(m.off.begin(), m.off.end());
    src->local_num_row = m.local_num_row; src->local_num_col = m.local_num_col;
    if (m.val.empty()) { off.assign(1, 0); return; }
    frovedis_gb300::device_matrix d(*src);
    int64_t nd = 0;
    frovedis_gb300::check(fvg_matrix_get_jds(frovedis_gb300::context(), d.h, &nd, nullptr, nullptr, nullptr, nullptr));
    std::vector<int32_t> pm(local_num_row), ji(m.val.size());
    std::vector<int64_t> jo(nd + 1);
    std::vector<double> jv(m.val.size());
    frovedis_gb300::check(fvg_matrix_get_jds(frovedis_gb300::context(), d.h, &nd, pm.data(), jo.data(), ji.data(),
                                             jv.data()));
    perm.assign(pm.begin(), pm.end()); off.assign(jo.begin(), jo.end());
    idx.assign(ji.begin(), ji.end()); val.assign(jv.begin(), jv.end());
  }
  std::vector<T> val;
  std::vector<I> idx;
  std::vector<O> off;
  std::vector<P> perm;
  size_t local_num_col, local_num_row;
  std::shared_ptr<crs_matrix_local<T, I, size_t>> src;
};

template <class T, class I, class O, class P>
std::vector<T> operator*(const jds_matrix_local<T, I, O, P>& mat, const std::vector<T>& v) {
  if (mat.local_num_col != v.size()) throw std::runtime_error("operator*: size of vector does not match");
  if (!mat.src) return std::vector<T>(mat.local_num_row);
  return detail::product<T>(*mat.src, v, FVG_JDS, false);
}

// JDS for the first crs_start_off entries of every row + CRS tail of the
// longest rows (threshold 256 rows), as the reference builds it.
template <class T, class I = size_t, class O = size_t, class P = size_t>
struct jds_crs_hybrid_local {
  jds_crs_hybrid_local() : local_num_col(0), local_num_row(0) {}
  explicit jds_crs_hybrid_local(const crs_matrix_local<T, I, O>& m) : src(new crs_matrix_local<T, I, size_t>()) {
    local_num_col = m.local_num_col;
    local_num_row = m.local_num_row;
    src->val = m.val; src->idx = m.idx; src->off.assign(m.off.begin(), m.off.end());
    src->local_num_row = m.local_num_row; src->local_num_col = m.local_num_col;
    frovedis_gb300::device_matrix d(*src);
    int64_t info[5];
    auto ctx = frovedis_gb300::context();
    frovedis_gb300::check(fvg_matrix_get_hybrid(ctx, d.h, info, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                                nullptr));
    std::vector<int32_t> pm(info[4] ? info[4] : 1), ji(info[3] + 1), ci(info[2] + 1);
    std::vector<int64_t> jo(info[0] + 1), co(info[1] + 1);
    std::vector<double> jv(info[3] + 1), cv(info[2] + 1);
    frovedis_gb300::check(fvg_matrix_get_hybrid(ctx, d.h, info, pm.data(), jo.data(), ji.data(), jv.data(),
                                                co.data(), ci.data(), cv.data()));
    jds.local_num_col = crs.local_num_col = local_num_col;
    jds.local_num_row = local_num_row;
    jds.perm.assign(pm.begin(), pm.begin() + info[4]);
    jds.off.assign(jo.begin(), jo.end());
    jds.idx.assign(ji.begin(), ji.begin() + info[3]);
    jds.val.assign(jv.begin(), jv.begin() + info[3]);
    crs.local_num_row = (size_t)info[1];
    crs.off.assign(co.begin(), co.end());
    crs.idx.assign(ci.begin(), ci.begin() + info[2]);
    crs.val.assign(cv.begin(), cv.begin() + info[2]);
  }
  jds_matrix_local<T, I, O, P> jds;
  crs_matrix_local<T, I, O> crs;
  size_t local_num_col, local_num_row;
  std::shared_ptr<crs_matrix_local<T, I, size_t>> src;
};

template <class T, class I, class O, class P>
std::vector<T> operator*(const jds_crs_hybrid_local<T, I, O, P>& mat, const std::vector<T>& v) {
  if (mat.local_num_col != v.size()) throw std::runtime_error("operator*: size of vector does not match");
  if (!mat.src) return std::vector<T>(mat.local_num_row);
  return detail::product<T>(*mat.src, v, FVG_HYBRID, false);
}

// logistic_regression_model<T> (ml/glm/linear_model.hpp:306-446)
template <class T>
struct logistic_regression_model {
  logistic_regression_model() : intercept(0.0), threshold(0.5) {}
  logistic_regression_model(size_t numFtr, T intercpt = 0.0, T thr = 0.5)
      : weight(numFtr, 1), intercept(intercpt), threshold(thr) {
    if (!(thr >= 0)) throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "checkAssumption failed: thr >= 0");
  }
  template <class I, class O>
  std::vector<T> predict_probability(const crs_matrix_local<T, I, O>& mat, bool use_score = false) const {
    std::vector<T> v = mat * weight;
    if (intercept != 0)
      for (auto& x : v) x += intercept;
    if (!use_score)
      for (auto& x : v) {
        T e = -1.0 * x;
        x = (e > 709) ? 0 : 1.0 / (1.0 + std::exp(e));
      }
    return v;
  }
  template <class I, class O>
  std::vector<T> predict(const crs_matrix_local<T, I, O>& mat, bool use_score = false) const {
    auto p = predict_probability(mat, use_score);
    if (threshold == (T)NONE) return p;  // cleared threshold: raw probabilities
    std::vector<T> r(p.size());
    for (size_t i = 0; i < p.size(); i++) r[i] = use_score ? (p[i] > 0 ? 1 : -1) : (p[i] >= threshold ? 1 : -1);
    return r;
  }
  template <class I, class O>
  rowmajor_matrix_local<T> compute_probability_matrix(const crs_matrix_local<T, I, O>& mat) const {
    auto p = predict_probability(mat);
    rowmajor_matrix_local<T> ret(p.size(), 2);
    for (size_t i = 0; i < p.size(); i++) {
      const bool yes = p[i] >= threshold;
      ret.val[2 * i + 0] = yes ? 1.0 - p[i] : p[i];
      ret.val[2 * i + 1] = yes ? p[i] : 1.0 - p[i];
    }
    return ret;
  }
  void set_threshold(T thr) {
    if (thr < 0) throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Negative Threshold Value\n");
    threshold = thr;
  }
  T get_threshold() const { return threshold; }
  size_t get_num_features() const { return weight.size(); }
  size_t get_num_classes() const { return 2; }
  std::vector<T> weight;
  T intercept;
  T threshold;
};

namespace detail {
template <class T, class I, class O>
logistic_regression_model<T> train(bool sgd, crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                   logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                   size_t& n_iter, size_t numIteration, double alpha, size_t hist_size,
                                   double miniBatchFraction, double regParam, RegType regTyp, bool isIntercept,
                                   double convergenceTol, MatType mType) {
  if (data.local_num_col != initModel.get_num_features())
    throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Incompatible Test Vector with Provided Initial Model\n");
  if (data.local_num_row != label.size())
    throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Number of label and data are different\n");
  if (sample_weight.empty()) sample_weight.assign(data.local_num_row, 1);
  frovedis_gb300::device_matrix d(data);
  fvg_glm_params p;
  fvg_glm_params_default(&p);
  p.num_iteration = (int64_t)numIteration;
  p.alpha = alpha;
  p.hist_size = (int64_t)hist_size;
  p.reg_param = regParam;
  p.reg_type = regTyp;
  p.intercept = isIntercept;
  p.convergence_tol = convergenceTol;
  p.mat_type = mType;
  p.mini_batch_fraction = miniBatchFraction;
  p.storage = frovedis_gb300::dtype_of<T>::value;
  std::vector<double> lab(label.begin(), label.end()), sw(sample_weight.begin(), sample_weight.end());
  std::vector<double> w(initModel.weight.begin(), initModel.weight.end());
  double b = initModel.intercept, loss = 0;
  int64_t it = 0;
  frovedis_gb300::check((sgd ? fvg_logreg_sgd : fvg_logreg_lbfgs)(frovedis_gb300::context(), d.h, lab.data(),
                                                                  sw.data(), &p, w.data(), &b, &it, &loss));
  n_iter = (size_t)it;
  logistic_regression_model<T> ret = initModel;
  ret.weight.assign(w.begin(), w.end());
  ret.intercept = (T)b;
  return ret;
}
}  // namespace detail

// logistic_regression_with_lbfgs (ml/glm/logistic_regression_with_lbfgs.hpp)
struct logistic_regression_with_lbfgs {
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.local_num_col, isIntercept ? 1.0 : 0.0);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                            double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.local_num_col, isIntercept ? 1.0 : 0.0);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType);
  }
  // main API (logistic_regression_with_lbfgs.hpp:395-437)
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            size_t hist_size = 10, double regParam = 0.01, RegType regTyp = ZERO,
                                            bool isIntercept = false, double convergenceTol = 0.001,
                                            MatType mType = CRS, bool inputMovable = false) {
    auto m = detail::train(false, data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, 1.0,
                           regParam, regTyp, isIntercept, convergenceTol, mType);
    if (inputMovable) data.clear();
    return m;
  }
};

// logistic_regression_with_sgd (ml/glm/logistic_regression_with_sgd.hpp)
struct logistic_regression_with_sgd {
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.local_num_col, isIntercept ? 1.0 : 0.0);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType);
  }
  // main API (logistic_regression_with_sgd.hpp:392-441)
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS,
                                            bool inputMovable = false) {
    auto m = detail::train(true, data, label, initModel, sample_weight, n_iter, numIteration, alpha, 10,
                           miniBatchFraction, regParam, regTyp, isIntercept, convergenceTol, mType);
    if (inputMovable) data.clear();
    return m;
  }
};

// multinomial_logistic_regression_model<T>
// (ml/glm/multinomial_logistic_regression_model.hpp:10-258)
template <class T>
struct multinomial_logistic_regression_model {
  multinomial_logistic_regression_model() : nfeatures(0), nclasses(0), isIntercept(false), threshold(0.5) {}
  multinomial_logistic_regression_model(size_t feature, size_t classes, bool isIcpt = false, double thr = 0.5)
      : weight(feature, classes), intercept(classes, 0), nfeatures(feature), nclasses(classes),
        isIntercept(isIcpt), threshold(thr) {}
  // softmax(X W + intercept), num_row x nclasses (lines 82-89)
  template <class I, class O>
  rowmajor_matrix_local<T> compute_probability_matrix(const crs_matrix_local<T, I, O>& mat) const {
    rowmajor_matrix_local<T> ret(mat.local_num_row, nclasses);
    if (mat.local_num_row == 0 || nclasses == 0) return ret;
    crs_matrix_local<double, I, O> m64;
    m64.local_num_row = mat.local_num_row;
    m64.local_num_col = mat.local_num_col;
    m64.val.assign(mat.val.begin(), mat.val.end());
    m64.idx = mat.idx;
    m64.off = mat.off;
    frovedis_gb300::device_matrix d(m64);
    std::vector<double> w(weight.val.begin(), weight.val.end()), b(intercept.begin(), intercept.end());
    std::vector<double> prob(mat.local_num_row * nclasses);
    frovedis_gb300::check(fvg_multinomial_probability(frovedis_gb300::context(), d.h, w.data(), b.data(),
                                                      (int64_t)nclasses, isIntercept, prob.data()));
    ret.val.assign(prob.begin(), prob.end());
    return ret;
  }
  // arg max class per row, ties to the lower class; a cleared threshold
  // returns the winning probability instead (lines 91-112)
  template <class I, class O>
  std::vector<T> predict(const crs_matrix_local<T, I, O>& mat) const {
    auto p = compute_probability_matrix(mat);
    const size_t m = mat.local_num_row;
    std::vector<T> lbl(m, 0), proba(m, 0);
    for (size_t i = 0; i < m; i++) proba[i] = p.val[i * nclasses];
    for (size_t j = 1; j < nclasses; j++)
      for (size_t i = 0; i < m; i++)
        if (p.val[i * nclasses + j] > proba[i]) {
          lbl[i] = (T)j;
          proba[i] = p.val[i * nclasses + j];
        }
    return threshold == (T)NONE ? proba : lbl;
  }
  template <class I, class O>
  std::vector<T> predict_probability(const crs_matrix_local<T, I, O>& mat, bool = false) {
    const T thr = threshold;
    threshold = NONE;
    auto r = predict(mat);
    threshold = thr;
    return r;
  }
  size_t get_num_features() const { return nfeatures; }
  size_t get_num_classes() const { return nclasses; }
  T get_threshold() const { return threshold; }
  void set_threshold(T thr) { threshold = thr; }
  rowmajor_matrix_local<T> weight;  // nfeatures x nclasses
  std::vector<T> intercept;
  size_t nfeatures, nclasses;
  bool isIntercept;
  T threshold;
};

// multinomial_logistic_regression (ml/glm/multinomial_logistic_regression.hpp)
struct multinomial_logistic_regression {
  template <class T, class I, class O>
  static multinomial_logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                                         size_t numIteration = 1000, double alpha = 0.01,
                                                         double regParam = 0.01, RegType regTyp = ZERO,
                                                         bool isIntercept = false, double convergenceTol = 0.001,
                                                         MatType mType = CRS) {
    // compute_nclasses: the number of distinct labels (line 238-240)
    std::vector<T> u(label);
    std::sort(u.begin(), u.end());
    const size_t nclasses = (size_t)(std::unique(u.begin(), u.end()) - u.begin());
    multinomial_logistic_regression_model<T> initModel(data.local_num_col, nclasses, isIntercept);
    std::vector<T> sample_weight;
    size_t n_iter = 0;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, regParam, regTyp, isIntercept,
                 convergenceTol, mType);
  }
  // main API (lines 342-378)
  template <class T, class I, class O>
  static multinomial_logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                                         multinomial_logistic_regression_model<T>& initModel,
                                                         std::vector<T>& sample_weight, size_t& n_iter,
                                                         size_t numIteration = 1000, double alpha = 0.01,
                                                         double regParam = 0.01, RegType regTyp = ZERO,
                                                         bool isIntercept = false, double convergenceTol = 0.001,
                                                         MatType mType = CRS, bool inputMovable = false) {
    if (data.local_num_col != initModel.get_num_features())
      throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Incompatible Test Vector with Provided Initial Model\n");
    if (data.local_num_row != label.size())
      throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Number of label and data are different\n");
    if (sample_weight.empty()) sample_weight.assign(data.local_num_row, 1);
    frovedis_gb300::device_matrix d(data);
    fvg_glm_params p;
    fvg_glm_params_default(&p);
    p.num_iteration = (int64_t)numIteration;
    p.alpha = alpha;
    p.reg_param = regParam;
    p.reg_type = regTyp;
    p.intercept = isIntercept;
    p.convergence_tol = convergenceTol;
    p.mat_type = mType;
    p.storage = frovedis_gb300::dtype_of<T>::value;
    const size_t K = initModel.get_num_classes();
    std::vector<double> lab(label.begin(), label.end()), sw(sample_weight.begin(), sample_weight.end());
    std::vector<double> w(initModel.weight.val.begin(), initModel.weight.val.end());
    std::vector<double> b(initModel.intercept.begin(), initModel.intercept.end());
    int64_t it = 0;
    frovedis_gb300::check(fvg_multinomial_train(frovedis_gb300::context(), d.h, lab.data(), sw.data(), &p,
                                                (int64_t)K, w.data(), b.data(), &it));
    n_iter = (size_t)it;
    multinomial_logistic_regression_model<T> ret = initModel;
    ret.weight.val.assign(w.begin(), w.end());
    ret.intercept.assign(b.begin(), b.end());
    ret.isIntercept = isIntercept;
    if (inputMovable) data.clear();
    return ret;
  }
};

}  // namespace frovedis

#endif  // FROVEDIS_GB300_HPP
