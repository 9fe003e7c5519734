// Exercises the C++ API of include/frovedis_gb300.hpp the way a frovedis
// program calls the reference: build crs_matrix_local, multiply, convert to
// ELL/JDS/hybrid, train with logistic_regression_with_{lbfgs,sgd}::train and
// the other GLM trainers, and predict.  Reads a CRS matrix, a vector and labels from the text file
// argv[1]; writes one "name v0 v1 ..." line per result to argv[2], which
// tests/test_cpp_api.py compares with the oracle.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "frovedis_gb300.hpp"

using namespace frovedis;

template <class V> static void put(FILE* f, const char* name, const V& v) {
  std::fprintf(f, "%s", name);
  for (auto x : v) std::fprintf(f, " %.17g", (double)x);
  std::fprintf(f, "\n");
}
static void put1(FILE* f, const char* name, double v) { std::fprintf(f, "%s %.17g\n", name, v); }

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: api_check input.txt output.txt\n");
    return 2;
  }
  std::ifstream in(argv[1]);
  size_t m, n, nnz;
  in >> m >> n >> nnz;
  crs_matrix_local<double> A(m, n);
  A.off.resize(m + 1);
  A.idx.resize(nnz);
  A.val.resize(nnz);
  for (auto& v : A.off) in >> v;
  for (auto& v : A.idx) in >> v;
  for (auto& v : A.val) in >> v;
  std::vector<double> x(n), label(m);
  for (auto& v : x) in >> v;
  for (auto& v : label) in >> v;
  if (!in) {
    std::fprintf(stderr, "bad input\n");
    return 2;
  }
  FILE* f = std::fopen(argv[2], "w");

  // products (crs_matrix.hpp:1518, ell_matrix.hpp:229/357, jds_matrix.hpp:419, jds_crs_hybrid.hpp:213)
  put(f, "crs_mv", A * x);
  auto t = A.transpose();
  put(f, "t_off", t.off);
  put(f, "t_idx", t.idx);
  put(f, "t_val", t.val);
  put(f, "t_shape", std::vector<size_t>{t.local_num_row, t.local_num_col});
  ell_matrix_local<double> E(A);
  put(f, "ell_mv", E * x);
  put(f, "ell_trans", trans_mv(E, label));
  put(f, "ell_width", std::vector<size_t>{E.val.size() / (m ? m : 1)});
  jds_matrix_local<double> J(A);
  put(f, "jds_mv", J * x);
  put(f, "jds_perm", J.perm);
  put(f, "jds_off", J.off);
  jds_crs_hybrid_local<double> H(A);
  put(f, "hyb_mv", H * x);
  put(f, "hyb_crs_rows", std::vector<size_t>{H.crs.local_num_row});
  rowmajor_matrix_local<double> X(n, 3);
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < 3; j++) X.val[i * 3 + j] = x[i] * (double)(j + 1) + (double)j;
  put(f, "spmm", (A * X).val);

  // FP32 instantiation
  crs_matrix_local<float, int, size_t> Af(m, n);
  Af.off.assign(A.off.begin(), A.off.end());
  Af.idx.assign(A.idx.begin(), A.idx.end());
  Af.val.assign(A.val.begin(), A.val.end());
  std::vector<float> xf(x.begin(), x.end());
  put(f, "crs_mv_f32", Af * xf);

  // the reference's error on a size mismatch (std::runtime_error)
  int threw = 0;
  try {
    std::vector<double> bad(n + 1);
    auto r = A * bad;
    (void)r;
  } catch (std::runtime_error&) {
    threw = 1;
  }
  put1(f, "mismatch_throws", threw);

  // training (logistic_regression_with_lbfgs.hpp:395, logistic_regression_with_sgd.hpp:392)
  {
    logistic_regression_model<double> init(n, 1.0);
    std::vector<double> sw;
    size_t n_iter = 0;
    auto model = logistic_regression_with_lbfgs::train(A, label, init, sw, n_iter, 20, 0.01, 10, 1e-3, L2, true,
                                                       0.001, CRS);
    put(f, "lbfgs_w", model.weight);
    put1(f, "lbfgs_b", model.intercept);
    put1(f, "lbfgs_n_iter", (double)n_iter);
    put(f, "lbfgs_prob", model.predict_probability(A));
    put(f, "lbfgs_pred", model.predict(A));
  }
  {
    std::vector<double> lab = label;
    auto model = logistic_regression_with_lbfgs::train(A, lab, 20, 0.01, 10, 1e-3, ZERO, true, 0.001, HYBRID);
    put(f, "lbfgs_hyb_w", model.weight);
    put1(f, "lbfgs_hyb_b", model.intercept);
    // JDS is rejected for L-BFGS (lbfgs_parallelizer.hpp:596-597)
    int jds_threw = 0;
    try {
      logistic_regression_with_lbfgs::train(A, lab, 20, 0.01, 10, 1e-3, ZERO, true, 0.001, JDS);
    } catch (frovedis_gb300::error& e) {
      jds_threw = std::string(e.what()).find("Unsupported input matrix type") != std::string::npos;
    }
    put1(f, "lbfgs_jds_throws", jds_threw);
  }
  {
    logistic_regression_model<double> init(n, 1.0);
    std::vector<double> sw;
    size_t n_iter = 0;
    auto model = logistic_regression_with_sgd::train(A, label, init, sw, n_iter, 15, 0.05, 0.3, 1e-2, L2, true,
                                                     0.001, CRS);
    put(f, "sgd_w", model.weight);
    put1(f, "sgd_b", model.intercept);
    put1(f, "sgd_n_iter", (double)n_iter);
  }
  {
    // multinomial: five classes assigned round-robin to the rows
    std::vector<double> cls(m);
    for (size_t i = 0; i < m; i++) cls[i] = (double)(i % 5);
    multinomial_logistic_regression_model<double> init(n, 5, false);
    std::vector<double> sw;
    size_t n_iter = 0;
    auto model = multinomial_logistic_regression::train(A, cls, init, sw, n_iter, 12, 0.05, 1e-3, L2, false, 0.0,
                                                        CRS);
    put(f, "mlr_w", model.weight.val);
    put1(f, "mlr_n_iter", (double)n_iter);
    put(f, "mlr_prob", model.compute_probability_matrix(A).val);
    put(f, "mlr_pred", model.predict(A));
    put(f, "mlr_maxprob", model.predict_probability(A));
  }
  {
    // loaders: the matrix written by the reference's text and binary writers
    // and read back on the device
    const std::string base = std::string(argv[2]) + ".dir";
    save(A, base + ".txt");
    auto At = make_crs_matrix_local_load<double>(base + ".txt");
    put(f, "load_text_off", At.off);
    put(f, "load_text_idx", At.idx);
    put(f, "load_text_val", At.val);
    savebinary(A, base + ".bin");
    auto Ab = make_crs_matrix_local_loadbinary<double>(base + ".bin");
    put(f, "load_bin_val", Ab.val);
    put(f, "load_bin_shape", std::vector<size_t>{Ab.local_num_row, Ab.local_num_col});
    {
      std::ofstream svm((base + ".svm").c_str());
      for (size_t r = 0; r < m; r++) {
        svm << label[r];
        for (size_t e = A.off[r]; e < A.off[r + 1]; e++) svm << " " << A.idx[e] + 1 << ":" << A.val[e];
        svm << "\n";
      }
    }
    std::vector<double> lab;
    auto As = make_crs_matrix_local_loadlibsvm<double>(base + ".svm", lab);
    put(f, "load_svm_idx", As.idx);
    put(f, "load_svm_label", lab);
    put(f, "load_svm_shape", std::vector<size_t>{As.local_num_row, As.local_num_col});
  }
  {
    // the estimator: L-BFGS binary model, then a multinomial one (five
    // classes), each saved and loaded in the text and binary formats
    const std::string base = std::string(argv[2]) + ".est";
    logistic_regression<double> est(30, 0.01, "lbfgs", 1e-3, "L2", true);
    std::vector<double> lab = label;
    est.fit(A, lab);
    put(f, "est_w", est.get_weight());
    put(f, "est_b", est.get_intercept());
    put1(f, "est_n_iter", (double)est.n_iter_);
    put1(f, "est_score", est.score(A, label));
    est.save(base + ".txt");
    est.savebinary(base + ".bin");
    logistic_regression<double> e2, e3;
    e2.load(base + ".txt");
    e3.loadbinary(base + ".bin");
    put(f, "est_text_w", e2.get_weight());
    put(f, "est_bin_w", e3.get_weight());
    put1(f, "est_pred_same", e2.predict(A) == est.predict(A) && e3.predict(A) == est.predict(A));
    std::vector<double> cls(m);
    for (size_t i = 0; i < m; i++) cls[i] = (double)(i % 5);
    logistic_regression<double> em(10, 0.05, "sgd");
    em.fit(A, cls);
    put1(f, "estm_is_mult", em.is_mult);
    put(f, "estm_w", em.get_weight());
    put1(f, "estm_n_iter", (double)em.n_iter_);
    em.savebinary(base + ".mbin");
    em.save(base + ".mtxt");
    logistic_regression<double> e4, e5;
    e4.loadbinary(base + ".mbin");
    e5.load(base + ".mtxt");
    put(f, "estm_bin_w", e4.get_weight());
    put1(f, "estm_pred_same", e4.predict(A) == em.predict(A));
    put1(f, "estm_text_classes", (double)e5.get_num_classes());
    int lbfgs_mult_threw = 0;
    try {
      logistic_regression<double> bad(5, 0.01, "lbfgs");
      bad.fit(A, cls);
    } catch (frovedis_gb300::error&) {
      lbfgs_mult_threw = 1;
    }
    put1(f, "estm_lbfgs_throws", lbfgs_mult_threw);
  }
  {
    // the regression and SVM trainers (linear_regression_with_*, lasso_with_*,
    // ridge_regression_with_*, svm_with_*, svm_regression_with_sgd)
    auto z = A * x;
    std::vector<double> y(m);
    for (size_t i = 0; i < m; i++) y[i] = 0.25 * z[i] + 0.5 * label[i];
    put(f, "reg_y", y);
    std::vector<double> sw;
    size_t it = 0;
    auto lr = linear_regression_with_sgd::train(A, y, sw, it, 20, 1e-4, 0.3, true, 0.0);
    put(f, "lin_sgd_w", lr.weight);
    put1(f, "lin_sgd_b", lr.intercept);
    put1(f, "lin_sgd_n_iter", (double)it);
    put(f, "lin_pred", lr.predict(A));
    auto ll = linear_regression_with_lbfgs::train(A, y, sw, it, 25, 0.01, 10, true);
    put(f, "lin_lbfgs_w", ll.weight);
    put1(f, "lin_lbfgs_b", ll.intercept);
    put1(f, "lin_lbfgs_n_iter", (double)it);
    put(f, "lasso_sgd_w", lasso_with_sgd::train(A, y, 20, 1e-4, 1.0, 1e-3, false, 0.0).weight);
    put(f, "ridge_lbfgs_w", ridge_regression_with_lbfgs::train(A, y, 25, 0.01, 10, 1e-2, true).weight);
    auto sv = svm_with_sgd::train(A, label, 30, 0.05, 1.0, 1e-2, L2, true, 0.0);
    put(f, "svm_sgd_w", sv.weight);
    put1(f, "svm_sgd_b", sv.intercept);
    put(f, "svm_pred", sv.predict(A));
    put(f, "svm_score", sv.predict_probability(A));
    auto sl = svm_with_lbfgs::train(A, label, sw, it, 25, 0.01, 10, 1e-2, L1, true);
    put(f, "svm_lbfgs_w", sl.weight);
    put1(f, "svm_lbfgs_n_iter", (double)it);
    put(f, "svr_eps_w", svm_regression_with_sgd::train(A, y, 20, 0.01, 1.0, 0.0, ZERO, true, 0.0, 0.1, EPS).weight);
    put(f, "svr_sqeps_w",
        svm_regression_with_sgd::train(A, y, 20, 1e-4, 1.0, 1e-3, L2, false, 0.0, 0.05, SQEPS).weight);
    int svm_jds_threw = 0;
    try {
      svm_with_lbfgs::train(A, label, 5, 0.01, 10, 0.01, ZERO, false, 0.001, JDS);
    } catch (frovedis_gb300::error& e) {
      svm_jds_threw = std::string(e.what()).find("Unsupported input matrix type") != std::string::npos;
    }
    put1(f, "svm_jds_throws", svm_jds_threw);
    // member persistence (linear_model.hpp:284-295, 569-583)
    const std::string base = std::string(argv[2]);
    lr.save(base + ".lin.txt");
    sv.savebinary(base + ".svm.bin");
    linear_regression_model<double> lr2;
    svm_model<double> sv2;
    lr2.load(base + ".lin.txt");
    sv2.loadbinary(base + ".svm.bin");
    put(f, "lin_loaded_w", lr2.weight);
    put1(f, "lin_loaded_b", lr2.intercept);
    put1(f, "svm_loaded_same", sv2.weight == sv.weight && sv2.intercept == sv.intercept &&
                                   sv2.threshold == sv.threshold);
  }
  {
    // shrink::logistic_regression_with_sgd and the estimator's shrink-sgd solver
    std::vector<double> sw;
    size_t it = 0;
    auto sm = shrink::logistic_regression_with_sgd::train(A, label, sw, it, 15, 0.05, 0.3, 1e-2, L2, true, 0.0);
    put(f, "shrink_w", sm.weight);
    put1(f, "shrink_b", sm.intercept);
    put1(f, "shrink_n_iter", (double)it);
    logistic_regression<double> es(12, 0.05, "shrink-sgd", 1e-3, "L1", true);
    std::vector<double> lab = label;
    es.fit(A, lab);
    put(f, "est_shrink_w", es.get_weight());
    put1(f, "est_shrink_n_iter", (double)es.n_iter_);
  }
  std::fclose(f);
  return 0;
}
