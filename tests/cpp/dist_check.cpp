// A reference-style program on the distributed containers (the shape of
// samples/glm/lr.cc: crs_matrix + dvector handed to
// logistic_regression_with_lbfgs::train), built against
// include/frovedis_gb300.hpp.  The C-ABI binding shown in INTEGRATION.md is
// pasted in verbatim by tests/test_cpp_api.py (it is an explicit
// specialisation of train() for crs_matrix<double,int,int>), so this
// program also checks that the binding compiles and gives the library's own
// result.  Reads a CRS matrix and labels from argv[1]; writes result lines
// to argv[2].
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "frovedis_gb300.hpp"

// what the binding needs from the reference's core/exceptions.hpp
enum { USER_ERROR = 1, INTERNAL_ERROR = 2 };
#define REPORT_ERROR(kind, msg) throw std::runtime_error(std::string(msg))

// @@BINDING@@

using namespace frovedis;

template <class V> static void put(FILE* f, const char* name, const V& v) {
  std::fprintf(f, "%s", name);
  for (auto x : v) std::fprintf(f, " %.17g", (double)x);
  std::fprintf(f, "\n");
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: dist_check input.txt output.txt\n");
    return 2;
  }
  std::ifstream in(argv[1]);
  size_t m, n, nnz;
  in >> m >> n >> nnz;
  crs_matrix_local<double, int, int> L(m, n);
  L.off.resize(m + 1);
  L.idx.resize(nnz);
  L.val.resize(nnz);
  for (auto& v : L.off) in >> v;
  for (auto& v : L.idx) in >> v;
  for (auto& v : L.val) in >> v;
  std::vector<double> lab(m);
  for (auto& v : lab) in >> v;
  FILE* out = std::fopen(argv[2], "w");

  // the binding: crs_matrix<double,int,int> takes the specialisation
  auto A = make_crs_matrix_scatter(L);
  auto label = make_dvector_scatter(lab);
  logistic_regression_model<double> init(A.num_col, 0.0);
  init.weight.assign(A.num_col, 0.0);
  std::vector<double> sw;
  size_t it = 0;
  auto mb = logistic_regression_with_lbfgs::train(A, label, init, sw, it, 15, 0.01, 10, 1e-3, L2, false, 0.001, CRS,
                                                  false);
  put(out, "binding_w", mb.weight);
  put(out, "binding_iter", std::vector<double>{(double)it});

  // the library's own distributed overloads on size_t offsets
  crs_matrix_local<double> L2m(m, n);
  L2m.off.assign(L.off.begin(), L.off.end());
  L2m.idx.assign(L.idx.begin(), L.idx.end());
  L2m.val = L.val;
  crs_matrix<double> B(L2m);
  logistic_regression_model<double> init2(B.num_col, 0.0);
  init2.weight.assign(B.num_col, 0.0);
  std::vector<double> sw2;
  size_t it2 = 0;
  auto ml = logistic_regression_with_lbfgs::train(B, label, init2, sw2, it2, 15, 0.01, 10, 1e-3, L2);
  put(out, "own_w", ml.weight);
  put(out, "own_iter", std::vector<double>{(double)it2});
  // defaults overload and the && overload (inputMovable: the matrix is cleared)
  auto md = logistic_regression_with_lbfgs::train(B, label, 15, 0.01, 10, 1e-3, L2, true);
  put(out, "defaults_w", md.weight);
  put(out, "defaults_b", std::vector<double>{md.intercept});
  crs_matrix<double> C(L2m);
  auto mr = logistic_regression_with_lbfgs::train(std::move(C), label, 15, 0.01, 10, 1e-3, L2, true);
  put(out, "moved_w", mr.weight);
  put(out, "moved_cleared", std::vector<double>{(double)(C.num_row == 0 && C.data.val.empty())});
  // SGD through the distributed overloads
  auto ms = logistic_regression_with_sgd::train(B, label, 10, 0.05, 1.0, 1e-2, L2, true);
  put(out, "sgd_w", ms.weight);
  put(out, "sgd_b", std::vector<double>{ms.intercept});
  std::fclose(out);
  return 0;
}
