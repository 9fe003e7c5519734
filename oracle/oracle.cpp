// CPU ORACLE — test infrastructure only.
//
// A plain C++ restatement of the reference's sparse logistic-regression
// path (frovedis: src/frovedis/matrix/{crs_matrix,ell_matrix,jds_matrix,
// jds_crs_hybrid}.hpp and src/frovedis/ml/glm/*.hpp).  Every function cites
// the reference lines it follows.  It exists so that the tests, the smoke
// check and the CPU-baseline leg of the benchmark have something to compare
// the CUDA path against.  Nothing in the product links or calls it.
//
// Arithmetic follows the reference loop order exactly (same summation order,
// no fused multiply-add: build with -ffp-contract=off) so that its results
// equal what the reference computes on one rank.  Multi-rank runs of the
// reference are emulated by splitting rows into P contiguous blocks, running
// each block as a rank and summing per-rank vectors in rank order (the
// reference reduces with MPI_Reduce / MPI_Allreduce).
//
// Parity pins: tests/golden holds the reference's own fixtures and expected
// outputs (tutorial SpMV and transpose, test2.1-1 SGD, test2.1-2 L-BFGS),
// checked by tests/test_oracle_golden.py.

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace orc {

using i64 = int64_t;
using i32 = int32_t;

// ---------------------------------------------------------------- formats
// crs_matrix_local<T,I,O>  (matrix/crs_matrix.hpp:240-331)
template <class T> struct CRS {
  i64 nrow = 0, ncol = 0;
  std::vector<T> val;
  std::vector<i32> idx;
  std::vector<i64> off{0};
};
// ell_matrix_local<T,I>  (matrix/ell_matrix.hpp:11-61): column-major, padded
template <class T> struct ELL {
  i64 nrow = 0, ncol = 0;
  std::vector<T> val;
  std::vector<i32> idx;
};
// jds_matrix_local<T,I,O,P>  (matrix/jds_matrix.hpp:15-79)
template <class T> struct JDS {
  i64 nrow = 0, ncol = 0;
  std::vector<T> val;
  std::vector<i32> idx;
  std::vector<i64> off{0};
  std::vector<i32> perm;
};
// jds_crs_hybrid_local<T,I,O,P>  (matrix/jds_crs_hybrid.hpp:8-36)
template <class T> struct HYB {
  i64 nrow = 0, ncol = 0;
  JDS<T> jds;
  CRS<T> crs;
};

// crs_matrix_spmv_impl  (matrix/crs_matrix.hpp:1505-1516)
template <class T> void crs_spmv(const CRS<T>& a, const T* x, T* y) {
  for (i64 r = 0; r < a.nrow; r++) {
    T acc = y[r];
    for (i64 c = a.off[r]; c < a.off[r + 1]; c++) acc = acc + a.val[c] * x[a.idx[c]];
    y[r] = acc;
  }
}
template <class T> std::vector<T> mv(const CRS<T>& a, const std::vector<T>& x) {
  // operator*(crs_matrix_local, vector)  (crs_matrix.hpp:1518-1525)
  if ((i64)x.size() != a.ncol) throw std::runtime_error("operator*: size of vector does not match");
  std::vector<T> y(a.nrow, T(0));
  crs_spmv(a, x.data(), y.data());
  return y;
}

// transpose_compressed_matrix + crs_matrix_local::transpose
// (crs_matrix.hpp:356-412): counting sort by column, stable in row order.
template <class T> CRS<T> transpose(const CRS<T>& a) {
  CRS<T> t;
  t.nrow = a.ncol;
  t.ncol = a.nrow;
  i64 nnz = (i64)a.val.size();
  t.val.resize(nnz);
  t.idx.resize(nnz);
  t.off.assign(a.ncol + 1, 0);
  std::vector<i64> num(a.ncol, 0), cur(a.ncol, 0);
  for (i64 r = 0; r < a.nrow; r++)
    for (i64 p = a.off[r]; p < a.off[r + 1]; p++) num[a.idx[p]]++;
  for (i64 c = 0; c < a.ncol; c++) t.off[c + 1] = t.off[c] + num[c];  // prefix_sum
  for (i64 r = 0; r < a.nrow; r++)
    for (i64 p = a.off[r]; p < a.off[r + 1]; p++) {
      i32 c = a.idx[p];
      i64 dst = t.off[c] + cur[c];
      t.val[dst] = a.val[p];
      t.idx[dst] = (i32)r;
      cur[c]++;
    }
  return t;
}

// ell_matrix_local(crs)  (ell_matrix.hpp:63-95)
template <class T> ELL<T> to_ell(const CRS<T>& a) {
  ELL<T> e;
  if (a.nrow == 0) return e;
  e.nrow = a.nrow;
  e.ncol = a.ncol;
  i64 width = 0;
  for (i64 r = 0; r < a.nrow; r++) width = std::max<i64>(width, a.off[r + 1] - a.off[r]);
  e.val.assign(e.nrow * width, T(0));
  e.idx.assign(e.nrow * width, 0);
  for (i64 r = 0; r < a.nrow; r++)
    for (i64 c = 0; c < a.off[r + 1] - a.off[r]; c++) {
      e.val[e.nrow * c + r] = a.val[a.off[r] + c];
      e.idx[e.nrow * c + r] = a.idx[a.off[r] + c];
    }
  return e;
}

// operator*(ell_matrix_local, vector)  (ell_matrix.hpp:229-355).  Rows in
// blocks of ELL_VLEN=256; ELL columns consumed 16/8/4/2/1 at a time, each
// group summed left to right and then added to the row's running value.
template <class T> std::vector<T> mv(const ELL<T>& e, const std::vector<T>& x) {
  std::vector<T> y(e.nrow, T(0));
  if (e.nrow == 0) return y;
  const i64 VLEN = 256;
  i64 width = (i64)e.val.size() / e.nrow, stride = e.nrow;
  auto P = [&](i64 pos) { return e.val[pos] * x[e.idx[pos]]; };
  auto rows = [&](i64 base, i64 cnt) {
    i64 j = 0;
    for (int g : {16, 8, 4, 2}) {
      for (; j + g - 1 < width; j += g)
        for (i64 k = 0; k < cnt; k++) {
          i64 rp = base + k;
          T s = P(stride * j + rp);
          for (int u = 1; u < g; u++) s = s + P(stride * (j + u) + rp);
          y[rp] = y[rp] + s;
        }
    }
    for (; j < width; j++)
      for (i64 k = 0; k < cnt; k++) y[base + k] = y[base + k] + P(stride * j + base + k);
  };
  i64 nblk = e.nrow / VLEN;
  for (i64 i = 0; i < nblk; i++) rows(VLEN * i, VLEN);
  // remainder rows: one ELL column at a time (ell_matrix.hpp:342-352)
  i64 rest = e.nrow - nblk * VLEN;
  for (i64 j = 0; j < width; j++)
    for (i64 k = 0; k < rest; k++) {
      i64 rp = VLEN * nblk + k;
      y[rp] = y[rp] + P(stride * j + rp);
    }
  return y;
}

// trans_mv(ell_matrix_local, vector)  (ell_matrix.hpp:357-380): scatter.
template <class T> std::vector<T> trans_mv(const ELL<T>& e, const std::vector<T>& v) {
  std::vector<T> y(e.ncol, T(0));
  if (e.nrow == 0) return y;
  i64 width = (i64)e.val.size() / e.nrow;
  for (i64 r = 0; r < e.nrow; r++)
    for (i64 pc = 0; pc < width; pc++) {
      i64 p = pc * e.nrow + r;
      y[e.idx[p]] = y[e.idx[p]] + e.val[p] * v[r];
    }
  return y;
}

// Row order used by JDS and the hybrid: (len,row) pairs sorted with
// std::greater, i.e. longest first and, among equal lengths, the larger row
// id first (jds_matrix.hpp:110-119; jds_crs_hybrid.hpp:89-98).
template <class T> std::vector<std::pair<i64, i64>> jds_order(const CRS<T>& a) {
  std::vector<std::pair<i64, i64>> p(a.nrow);
  for (i64 i = 0; i < a.nrow; i++) p[i] = {a.off[i + 1] - a.off[i], i};
  std::sort(p.begin(), p.end(), std::greater<std::pair<i64, i64>>());
  return p;
}

// jds_matrix_local(crs)  (jds_matrix.hpp:81-146, x86 branch)
template <class T> JDS<T> to_jds(const CRS<T>& a) {
  JDS<T> j;
  j.ncol = a.ncol;
  j.nrow = a.nrow;
  j.off.clear();
  if (a.val.empty()) {
    j.off.push_back(0);
    return j;
  }
  j.val.resize(a.val.size());
  j.idx.resize(a.idx.size());
  j.perm.resize(a.nrow);
  auto pt = jds_order(a);
  for (i64 i = 0; i < a.nrow; i++) j.perm[i] = (i32)pt[i].second;
  j.off.push_back(0);
  i64 col = 0, st = 0;
  for (i64 rmax = a.nrow; rmax != 0; rmax--) {
    i64 niter = pt[rmax - 1].first - col;
    for (i64 i = 0; i < niter; i++, col++) {
      for (i64 r = 0; r < rmax; r++, st++) {
        j.val[st] = a.val[a.off[j.perm[r]] + col];
        j.idx[st] = a.idx[a.off[j.perm[r]] + col];
      }
      j.off.push_back(st);
    }
  }
  return j;
}

// jds_spmv_helper{16,8,4,2,1}  (jds_matrix.hpp:244-374).  A group of K
// diagonals starting at c first covers the rows present in all K diagonals
// (from col_offset), then splits the rest into groups of K/2, K/4, ..., 1.
template <class T>
void jds_group(const JDS<T>& j, const T* x, T* tmp, int K, i64 c, i64 co) {
  i64 len = (j.off[c + K] - j.off[c + K - 1]) - co;
  for (i64 i = 0; i < len; i++) {
    if (K == 1) {
      i64 p = j.off[c] + co + i;
      tmp[co + i] = tmp[co + i] + j.val[p] * x[j.idx[p]];
    } else {
      i64 p0 = j.off[c] + co + i;
      T s = j.val[p0] * x[j.idx[p0]];
      for (int k = 1; k < K; k++) {
        i64 p = j.off[c + k] + co + i;
        s = s + j.val[p] * x[j.idx[p]];
      }
      tmp[co + i] = tmp[co + i] + s;
    }
  }
  i64 sub = c;
  for (int h = K / 2; h >= 1; h /= 2) {
    jds_group(j, x, tmp, h, sub, co + len);
    sub += h;
  }
}

// jds_matrix_spmv_impl  (jds_matrix.hpp:376-417)
template <class T> void jds_spmv(const JDS<T>& j, const T* x, T* y) {
  std::vector<T> tmp(j.nrow, T(0));
  i64 D = (i64)j.off.size() - 1;
  i64 ng = D / 16, c = 0;
  for (i64 g = 0; g < ng; g++) jds_group(j, x, tmp.data(), 16, g * 16, 0);
  c = ng * 16;
  if (c + 7 < D) { jds_group(j, x, tmp.data(), 8, c, 0); c += 8; }
  if (c + 3 < D) { jds_group(j, x, tmp.data(), 4, c, 0); c += 4; }
  if (c + 1 < D) { jds_group(j, x, tmp.data(), 2, c, 0); c += 2; }
  if (c < D) jds_group(j, x, tmp.data(), 1, c, 0);
  // The reference reads perm[] even when it is empty (all-zero matrix);
  // here an empty perm means an all-zero result.
  if ((i64)j.perm.size() == j.nrow)
    for (i64 i = 0; i < j.nrow; i++) y[j.perm[i]] = tmp[i];
  else
    for (i64 i = 0; i < j.nrow; i++) y[i] = T(0);
}
template <class T> std::vector<T> mv(const JDS<T>& j, const std::vector<T>& x) {
  if ((i64)x.size() != j.ncol) throw std::runtime_error("operator*: size of vector does not match");
  std::vector<T> y(j.nrow, T(0));
  jds_spmv(j, x.data(), y.data());
  return y;
}

// jds_crs_hybrid_local(crs, threshold)  (jds_crs_hybrid.hpp:38-153, x86)
template <class T> HYB<T> to_hyb(const CRS<T>& m, i64 thr = 256) {
  HYB<T> h;
  h.ncol = m.ncol;
  h.nrow = m.nrow;
  h.jds.ncol = m.ncol;
  h.jds.nrow = m.nrow;
  if (m.val.empty()) {
    h.crs = m;
    return h;
  } else if (m.nrow <= thr) {
    h.crs = m;
    h.jds.perm.resize(m.nrow);
    for (i64 i = 0; i < m.nrow; i++) h.jds.perm[i] = (i32)i;
    return h;
  } else if (thr == 0) {
    h.jds = to_jds(m);
    h.crs.ncol = m.ncol;
    h.crs.nrow = 0;
    return h;
  }
  auto pt = jds_order(m);
  h.jds.perm.resize(m.nrow);
  for (i64 i = 0; i < m.nrow; i++) h.jds.perm[i] = (i32)pt[i].second;
  i64 start = pt[thr].first;
  i64 crs_rows = thr;
  for (; crs_rows != 0; crs_rows--)
    if (pt[crs_rows - 1].first != start) break;
  i64 crs_size = 0;
  for (i64 i = 0; i < crs_rows; i++) crs_size += pt[i].first - start;
  h.jds.val.resize(m.val.size() - crs_size);
  h.jds.idx.resize(m.idx.size() - crs_size);
  h.crs.val.resize(crs_size);
  h.crs.idx.resize(crs_size);
  h.crs.ncol = m.ncol;
  h.crs.nrow = crs_rows;
  const i32* perm = h.jds.perm.data();
  i64 col = 0, st = 0;
  for (i64 rmax = m.nrow; rmax != crs_rows; rmax--) {
    i64 niter = pt[rmax - 1].first - col;
    for (i64 i = 0; i < niter; i++, col++) {
      for (i64 r = 0; r < rmax; r++, st++) {
        h.jds.val[st] = m.val[m.off[perm[r]] + col];
        h.jds.idx[st] = m.idx[m.off[perm[r]] + col];
      }
      h.jds.off.push_back(st);
    }
  }
  st = 0;
  for (i64 r = 0; r < crs_rows; r++) {
    for (i64 c = m.off[perm[r]] + start; c < m.off[perm[r] + 1]; c++, st++) {
      h.crs.val[st] = m.val[c];
      h.crs.idx[st] = m.idx[c];
    }
    h.crs.off.push_back(st);
  }
  return h;
}

// jds_crs_hybrid_spmv_impl  (jds_crs_hybrid.hpp:198-211)
template <class T> std::vector<T> mv(const HYB<T>& h, const std::vector<T>& x) {
  if ((i64)x.size() != h.ncol) throw std::runtime_error("operator*: size of vector does not match");
  std::vector<T> y(h.nrow, T(0));
  if ((i64)h.jds.perm.size() != h.nrow) return y;  // all-zero matrix (reference: UB)
  jds_spmv(h.jds, x.data(), y.data());
  std::vector<T> part(h.crs.nrow, T(0));
  crs_spmv(h.crs, x.data(), part.data());
  for (i64 i = 0; i < h.crs.nrow; i++) y[h.jds.perm[i]] = y[h.jds.perm[i]] + part[i];
  return y;
}

// crs_matrix_spmm_impl, x86 branch  (crs_matrix.hpp:2036-2050)
template <class T> void crs_spmm(const CRS<T>& a, const T* X, i64 k, T* Y) {
  for (i64 r = 0; r < a.nrow; r++)
    for (i64 c = a.off[r]; c < a.off[r + 1]; c++)
      for (i64 mc = 0; mc < k; mc++)
        Y[r * k + mc] = Y[r * k + mc] + a.val[c] * X[(i64)a.idx[c] * k + mc];
}

// ---------------------------------------------------------- vector helpers
// SIGN / ABS  (core/vector_operations.hpp:18-19)
template <class T> inline int SIGN(T x) { return (int)(x >= 0) - (int)(x < 0); }
template <class T> inline T ABS(T x) { return x * SIGN(x); }

// vector_dot  (vector_operations.hpp:1123-1138)
template <class T> T dot(const std::vector<T>& a, const std::vector<T>& b) {
  T r = 0;
  for (size_t i = 0; i < a.size(); i++) r += a[i] * b[i];
  return r;
}
// vector_norm via vector_squared_sum_impl  (vector_operations.hpp:227-264)
template <class T> T norm(const std::vector<T>& v) {
  if (v.empty()) return 0;
  T mx = ABS(v[0]);
  for (auto x : v) {
    T a = ABS(x);
    if (a > mx) mx = a;
  }
  if (mx == 0) return 0;
  T inv = T(1.0) / mx, s = 0;
  for (auto x : v) {
    T t = x * inv;
    s += t * t;
  }
  return std::sqrt(s) * mx;
}
// vector_sum  (vector_operations.hpp:183-189)
template <class T> T vsum(const std::vector<T>& v) {
  T s = 0;
  for (auto x : v) s += x;
  return s;
}

// ------------------------------------------------------------- logistic
// logistic_gradient<T>::compute_dloss  (ml/glm/gradient.hpp:15-53)
template <class T>
std::vector<T> logistic_dloss(const std::vector<T>& label, const std::vector<T>& wtx, double& sumloss) {
  size_t n = wtx.size();
  double loss = 0.0;
  for (size_t i = 0; i < n; i++) {
    T z = label[i] * wtx[i];
    if (z > 18.0) loss = std::exp((double)-z);
    else if (z < -18.0) loss = -z;
    else loss = std::log(1.0 + std::exp((double)-z));
    sumloss += loss;
  }
  std::vector<T> d(n, T(0));
  for (size_t i = 0; i < n; i++) {
    double neg = label[i] * -1.0;
    T z = label[i] * wtx[i];
    if (z > 18.0) d[i] = (T)(std::exp((double)-z) * neg);
    else if (z < -18.0) d[i] = (T)neg;
    else d[i] = (T)(neg * (1.0 / (1.0 + std::exp((double)z))));
    if (d[i] > 1e12) d[i] = (T)1e12;
    else if (d[i] < -1e12) d[i] = (T)-1e12;
  }
  return d;
}

// ------------------------------------------------------- other GLM losses
// Loss kinds of the GLM family (ml/glm/gradient.hpp): 0 logistic_gradient,
// 1 linear_gradient (55-87), 2 hinge_gradient (89-121), 3 epsilon_insensitive
// (123-159), 4 squared_epsilon_insensitive (161-202).  MAX_LOSS / MIN_LOSS
// clip ±1e12, HINGE_THRESHOLD 1 (gradient.hpp:8-10).
enum LossKind { L_LOGISTIC = 0, L_LINEAR = 1, L_HINGE = 2, L_EPS = 3, L_SQEPS = 4 };
struct Loss {
  int kind = L_LOGISTIC;
  double eps = 0.0;
};

template <class T> inline T clip_loss(T d) {
  if (d > 1e12) return (T)1e12;
  if (d < -1e12) return (T)-1e12;
  return d;
}

// compute_dloss of the chosen kind.  sumloss is the caller's running loss:
// the linear kind halves the whole running value (gradient.hpp:70-73), so a
// minibatch sequence accumulating into one variable halves earlier batches
// again; kept as the reference does it.
template <class T>
std::vector<T> glm_dloss(const Loss& L, const std::vector<T>& label, const std::vector<T>& wtx, double& sumloss) {
  if (L.kind == L_LOGISTIC) return logistic_dloss(label, wtx, sumloss);
  size_t n = wtx.size();
  std::vector<T> d(n, T(0));
  const double eps = L.eps;
  if (L.kind == L_LINEAR) {
    for (size_t i = 0; i < n; i++) {
      T e = wtx[i] - label[i];
      sumloss += (e * e);
    }
    sumloss *= 0.5;
    for (size_t i = 0; i < n; i++) d[i] = clip_loss<T>(wtx[i] - label[i]);
  } else if (L.kind == L_HINGE) {
    for (size_t i = 0; i < n; i++) {
      T z = wtx[i] * label[i];
      sumloss += (z <= 1.0) ? (double)(1.0 - z) : 0.0;
    }
    for (size_t i = 0; i < n; i++) d[i] = (wtx[i] * label[i] <= 1.0) ? -label[i] : T(0);
  } else if (L.kind == L_EPS) {
    for (size_t i = 0; i < n; i++) {
      double e = std::fabs(label[i] - wtx[i]) - eps;
      sumloss += (e > 0) ? e : 0.0;
    }
    for (size_t i = 0; i < n; i++) {
      if ((label[i] - wtx[i]) > eps) d[i] = -1;
      else if ((wtx[i] - label[i]) > eps) d[i] = 1;
      else d[i] = 0;
    }
  } else {
    for (size_t i = 0; i < n; i++) {
      double e = std::fabs(label[i] - wtx[i]) - eps;
      sumloss += (e > 0) ? e * e : 0.0;
    }
    for (size_t i = 0; i < n; i++) {
      T z = label[i] - wtx[i];
      if (z > eps) d[i] = (T)(-2 * (z - eps));
      else if (z < -eps) d[i] = (T)(2 * (-z - eps));
      else d[i] = 0;
      d[i] = clip_loss<T>(d[i]);
    }
  }
  return d;
}

// ---------------------------------------------- per-rank matrices (glm)
enum Fmt { CRS_F = 0, JDS_F = 1, ELL_F = 2, HYB_F = 3 };

// One rank's data: the forward matrix in the chosen format and, for the
// "with trans" paths, the transposed copy in the same format
// (ml/utility/matrix_conversion.hpp:22-111; lbfgs_parallelizer.hpp:562-597).
template <class T> struct RankData {
  int fmt = CRS_F;
  CRS<T> crs, tcrs;
  JDS<T> jds, tjds;
  ELL<T> ell;
  HYB<T> hyb, thyb;
  i64 nrow = 0, ncol = 0;
  void build(const CRS<T>& a, int f) {
    fmt = f;
    nrow = a.nrow;
    ncol = a.ncol;
    if (f == CRS_F) { crs = a; tcrs = transpose(a); }
    else if (f == HYB_F) { hyb = to_hyb(a); thyb = to_hyb(transpose(a)); }
    else if (f == JDS_F) { jds = to_jds(a); tjds = to_jds(transpose(a)); }
    else if (f == ELL_F) { ell = to_ell(a); }
  }
  std::vector<T> fwd(const std::vector<T>& x) const {
    if (fmt == CRS_F) return mv(crs, x);
    if (fmt == HYB_F) return mv(hyb, x);
    if (fmt == JDS_F) return mv(jds, x);
    return mv(ell, x);
  }
  std::vector<T> bwd(const std::vector<T>& r) const {
    if (fmt == CRS_F) return mv(tcrs, r);   // trans * dloss (gradient_descent.hpp:211)
    if (fmt == HYB_F) return mv(thyb, r);
    if (fmt == JDS_F) return mv(tjds, r);
    return trans_mv(ell, r);                 // gradient_descent.hpp:183
  }
};

// Row block [r0, r1) of a CRS matrix as its own local matrix
// (the per-rank piece, or a minibatch: ml/glm/common.hpp:232-257).
template <class T> CRS<T> rows_of(const CRS<T>& a, i64 r0, i64 r1) {
  CRS<T> b;
  b.nrow = r1 - r0;
  b.ncol = a.ncol;
  i64 s = a.off[r0], e = a.off[r1];
  b.val.assign(a.val.begin() + s, a.val.begin() + e);
  b.idx.assign(a.idx.begin() + s, a.idx.begin() + e);
  b.off.resize(b.nrow + 1);
  b.off[0] = 0;
  for (i64 i = 0; i < b.nrow; i++) b.off[i + 1] = b.off[i] + (a.off[r0 + i + 1] - a.off[r0 + i]);
  return b;
}

// gradient_descent::compute_gradient (with trans)  (gradient_descent.hpp:196-225;
// the no-trans variant 166-194 differs only in the backward product).
template <class T>
std::vector<T> compute_gradient(const RankData<T>& d, const std::vector<T>& w, T b,
                                const std::vector<T>& label, const std::vector<T>& sw,
                                bool icpt, T& bias, double& loss, const Loss& L = Loss()) {
  if (d.nrow == 0) return std::vector<T>(w.size(), T(0));
  auto wtx = d.fwd(w);                        // compute_wtx  (227-240)
  if (icpt) for (auto& v : wtx) v += b;
  auto dl = glm_dloss(L, label, wtx, loss);
  for (size_t i = 0; i < dl.size(); i++) dl[i] = dl[i] * sw[i];
  if (icpt) bias = vsum(dl);
  return d.bwd(dl);
}

// Runs fn(rank) for every rank, in parallel when nthreads > 1.
inline void for_ranks(int P, int nthreads, const std::function<void(int)>& fn) {
  if (nthreads <= 1 || P <= 1) {
    for (int r = 0; r < P; r++) fn(r);
    return;
  }
  std::vector<std::thread> th;
  int nt = std::min(nthreads, P);
  for (int t = 0; t < nt; t++)
    th.emplace_back([&, t]() { for (int r = t; r < P; r += nt) fn(r); });
  for (auto& x : th) x.join();
}

template <class T> struct Problem {
  std::vector<RankData<T>> ranks;
  std::vector<std::vector<T>> label, sw;
  i64 ncol = 0;
  int nthreads = 1;
  Loss loss;
};

template <class T>
Problem<T> make_problem(const CRS<T>& a, const T* label, const T* sw, const i64* splits, int P,
                        int fmt, int nthreads) {
  Problem<T> pr;
  pr.ncol = a.ncol;
  pr.nthreads = nthreads;
  pr.ranks.resize(P);
  pr.label.resize(P);
  pr.sw.resize(P);
  for_ranks(P, nthreads, [&](int r) {
    i64 r0 = splits[r], r1 = splits[r + 1];
    pr.ranks[r].build(rows_of(a, r0, r1), fmt);
    pr.label[r].assign(label + r0, label + r1);
    pr.sw[r].assign(sw + r0, sw + r1);
  });
  return pr;
}

// One distributed evaluation: every rank computes its [grad, bias] part
// (lbfgs_dtrain_with_trans, lbfgs_parallelizer.hpp:36-58), parts are summed
// in rank order (vector_sum → MPI_Reduce, core/DVID.hpp:859-873) and losses
// likewise (dloss.reduce(add)).
template <class T>
std::vector<T> evaluate(const Problem<T>& pr, const std::vector<T>& w, T b, bool icpt, double& loss) {
  int P = (int)pr.ranks.size();
  std::vector<std::vector<T>> parts(P);
  std::vector<double> losses(P, 0.0);
  for_ranks(P, pr.nthreads, [&](int r) {
    T bias = 0;
    double l = 0.0;
    auto g = compute_gradient(pr.ranks[r], w, b, pr.label[r], pr.sw[r], icpt, bias, l, pr.loss);
    g.push_back(bias);
    parts[r] = std::move(g);
    losses[r] = l;
  });
  std::vector<T> g = parts[0];
  for (int r = 1; r < P; r++)
    for (size_t i = 0; i < g.size(); i++) g[i] += parts[r][i];
  loss = losses[0];
  for (int r = 1; r < P; r++) loss += losses[r];
  return g;
}

// Regularisers as post-step weight transforms  (ml/glm/regularizer.hpp:14-61).
// no_eta selects the branch compiled without USE_ETA (regularizer.hpp:50-54),
// w -= λ·w; the stored expectation of test/ml/test2.1-1 was produced that way.
template <class T> void regularize(std::vector<T>& w, int rtype, T lambda, double eta, bool no_eta = false) {
  if (rtype == 1) {          // l1_regularizer
    for (auto& x : w) x -= lambda * SIGN(x);
  } else if (rtype == 2 && no_eta) {
    for (auto& x : w) x -= lambda * x;
  } else if (rtype == 2) {   // l2_regularizer with USE_ETA: scal(w, max(0, 1-λη))
    double n = 1.0 - (lambda * eta);
    T s = (T)std::max(0.0, n);
    for (auto& x : w) x = s * x;
  }
}

// lbfgs<T> + cir_array_list  (ml/glm/lbfgs.hpp:8-143, matrix/cir_array_list.hpp)
template <class T> struct LBFGS {
  i64 len;
  std::vector<T> old_model, old_grad;
  std::vector<T> rho;
  std::vector<std::vector<T>> S, Y;  // ring slots
  i64 rear = -1, front = -1, active = 0;
  explicit LBFGS(i64 h) : len(h), rho(h), S(h), Y(h) {}
  i64 slot(i64 i) const { return (rear + i) % len; }  // operator[] (119-133)
  void push(T r, std::vector<T>&& s, std::vector<T>&& y) {  // push_back_impl (77-89)
    if (active == 0) rear = front = 0;
    else if (active == len) { rear = (rear + 1) % len; front = (front + 1) % len; }
    else front = (front + 1) % len;
    active = active < len ? active + 1 : len;
    rho[front] = r;
    S[front] = std::move(s);
    Y[front] = std::move(y);
  }
  // compute_hkgk  (lbfgs.hpp:79-112)
  std::vector<T> hkgk(const std::vector<T>& g) const {
    size_t n = g.size();
    std::vector<T> z(n);
    if (active == 0) {
      T H0 = 0.1;
      T gn = norm(g);
      if (gn > 1) gn = T(1.0) / gn;
      for (size_t i = 0; i < n; i++) z[i] = -gn * H0 * g[i];
    } else {
      std::vector<T> q = g, al(active);
      for (i64 i = active - 1; i >= 0; --i) {
        al[i] = rho[slot(i)] * dot(S[slot(i)], q);
        const auto& y = Y[slot(i)];
        for (size_t j = 0; j < n; j++) q[j] = q[j] - (y[j] * al[i]);
      }
      i64 last = active - 1;
      T yy = dot(Y[slot(last)], Y[slot(last)]);
      if (yy == 0) yy = 1.0;
      double ys = 1.0 / rho[slot(last)];
      T H0 = (T)(ys / yy);
      for (size_t j = 0; j < n; j++) z[j] = q[j] * H0;
      for (i64 i = 0; i < active; ++i) {
        T beta = rho[slot(i)] * dot(Y[slot(i)], z);
        const auto& s = S[slot(i)];
        T f = al[i] - beta;
        for (size_t j = 0; j < n; j++) z[j] = z[j] + (s[j] * f);
      }
    }
    for (auto& v : z) v = v * T(-1.0);
    return z;
  }
  // update_history  (lbfgs.hpp:114-143)
  void update(const std::vector<T>& cur_model, std::vector<T>& cur_grad) {
    size_t n = cur_model.size();
    std::vector<T> md(n), gd(n);
    for (size_t i = 0; i < n; i++) md[i] = cur_model[i] - old_model[i];
    for (size_t i = 0; i < n; i++) gd[i] = cur_grad[i] - old_grad[i];
    for (size_t i = 0; i < n; i++) if (ABS(gd[i]) < 1e-10) gd[i] = 0;  // IGNORABLE_DIFF
    T dv = dot(md, gd);
    if (dv == 0) dv = 1;
    push(T(1.0) / dv, std::move(md), std::move(gd));
    old_model = cur_model;
    old_grad = cur_grad;
  }
};

// lbfgs_parallelizer::do_train  (ml/glm/lbfgs_parallelizer.hpp:267-364 with
// trans; 366-462 without).  Constants 153-156.  eval(w, b, loss) returns the
// gradient [g, bias] (the GLM evaluation, or the softmax one below).
template <class T, class Eval>
void lbfgs_driver(Eval&& eval, int fmt, std::vector<T>& w, T& b, i64 num_iter, i64 hist, T lambda, int rtype,
                  double tol, i64& n_iter, double& final_loss,
                  double* trace /* per iteration: loss, trials, rms, factor */, bool no_eta = false) {
  const double MAX_STEP = 1e20, SEARCH_TOL = 1e-4;
  const i64 MAX_SEARCH = 10;
  LBFGS<T> opt(hist);
  double loss = 0.0;
  auto grad = eval(w, b, loss);
  opt.old_model = w;
  opt.old_model.push_back(b);
  opt.old_grad = grad;
  i64 i = 1;
  for (; i <= num_iter; i++) {
    auto step = opt.hkgk(grad);
    if (dot(grad, step) > 0) for (auto& v : step) v = v * T(-1.0);
    T factor = 1.0;
    T stepsize = norm(step);
    if (factor * stepsize > MAX_STEP) factor = (T)(MAX_STEP / stepsize);
    T bstep = step.back();
    step.pop_back();
    std::vector<T> nw(w.size()), ng;
    T nb = 0;
    double nloss = 0;
    i64 j = 1;
    for (; j <= MAX_SEARCH; ++j) {
      for (size_t k = 0; k < w.size(); k++) nw[k] = w[k] + (factor * step[k]);
      nb = b + (factor * bstep);
      // CRS/HYBRID pass the step factor as eta (321); the no-trans ELL
      // path calls regularize(w) with the default eta = 1 (419).
      regularize(nw, rtype, lambda, fmt == ELL_F ? 1.0 : (double)factor, no_eta);
      ng = eval(nw, nb, nloss);
      if (nloss - loss < SEARCH_TOL) break;
      factor /= T(10.0);
    }
    loss = nloss;
    grad = ng;
    w = nw;
    b = nb;
    T rms = norm(grad) / (T)std::sqrt((double)grad.size());
    if (trace) {
      trace[4 * (i - 1) + 0] = loss;
      trace[4 * (i - 1) + 1] = (double)j;  // MAX_SEARCH + 1 = search exhausted
      trace[4 * (i - 1) + 2] = rms;
      trace[4 * (i - 1) + 3] = factor;
    }
    auto cm = w;
    cm.push_back(b);
    opt.update(cm, grad);
    if (rms <= tol) break;
  }
  n_iter = (i == num_iter + 1) ? num_iter : i;
  final_loss = loss;
}

template <class T>
void lbfgs_train(const Problem<T>& pr, int fmt, std::vector<T>& w, T& b, i64 num_iter, i64 hist,
                 T lambda, int rtype, bool icpt, double tol, i64& n_iter, double& final_loss,
                 double* trace /* per iteration: loss, trials, rms, factor */, bool no_eta = false) {
  lbfgs_driver<T>([&](const std::vector<T>& ww, T bb, double& l) { return evaluate(pr, ww, bb, icpt, l); }, fmt, w, b,
                  num_iter, hist, lambda, rtype, tol, n_iter, final_loss, trace, no_eta);
}

// ------------------------------------------------------------------ SGD
// LR_VLEN = 1024 minibatch granularity  (ml/glm/common.hpp:18, 283-321)
inline i64 minibatch_size(i64 ns, double frac) {
  i64 tmp = (i64)std::ceil(ns * frac);
  i64 t2 = (tmp == 0 ? 0 : (tmp - 1) / 1024 + 1) * 1024;
  return t2 < ns ? t2 : ns;
}

// sgd_parallelizer::parallelize + do_train_with_trans / do_train_notrans
// (ml/glm/sgd_parallelizer.hpp:132-378, 441-550) with gradient_descent::
// optimize and update_model (gradient_descent.hpp:128-164, 242-259).
template <class T>
void sgd_train(const CRS<T>& a, const T* label, const T* sw, const i64* splits, int P, int fmt,
               std::vector<T>& w, T& b, i64 num_iter, double alpha, double frac, T lambda, int rtype,
               bool icpt, double tol, i64& n_iter, double& final_loss, int nthreads, bool no_eta = false,
               const Loss& L = Loss(), bool shrink = false) {
  struct RankSGD {
    std::vector<RankData<T>> batches;
    std::vector<std::vector<T>> label, sw;
  };
  std::vector<RankSGD> rk(P);
  for_ranks(P, nthreads, [&](int r) {
    i64 r0 = splits[r], r1 = splits[r + 1], ns = r1 - r0;
    i64 mbs = minibatch_size(ns, frac);
    i64 nb = (ns == 0) ? 0 : (ns - 1) / mbs + 1;
    for (i64 k = 0; k < nb; k++) {
      i64 s = r0 + k * mbs, e = std::min(r0 + (k + 1) * mbs, r1);
      RankData<T> d;
      d.build(rows_of(a, s, e), fmt);
      rk[r].batches.push_back(std::move(d));
      rk[r].label.emplace_back(label + s, label + e);
      rk[r].sw.emplace_back(sw + s, sw + e);
    }
  });
  i64 n = (i64)w.size();
  // shrink::sgd_parallelizer: shrink_column per rank (matrix/shrink_matrix.hpp);
  // used = columns of any rank, n_used0 = rank 0's own column count
  std::vector<char> used(n, 0), used0(n, 0);
  if (shrink)
    for (int r = 0; r < P; r++)
      for (i64 q = a.off[splits[r]]; q < a.off[splits[r + 1]]; q++) {
        used[a.idx[q]] = 1;
        if (r == 0) used0[a.idx[q]] = 1;
      }
  i64 n_used0 = 0;
  for (char u : used0) n_used0 += u;
  double sumloss = 0.0;
  i64 i;
  for (i = 1; i <= num_iter; i++) {
    std::vector<std::vector<T>> delta(P);
    std::vector<double> lloss(P, 0.0);
    for_ranks(P, nthreads, [&](int r) {
      std::vector<T> lw = w;  // MODEL lModel = gModel
      T lb = b, bias = 0;
      double loss = 0.0;
      T ra = (T)(alpha / std::sqrt((double)i));  // update_model (247)
      for (size_t k = 0; k < rk[r].batches.size(); k++) {
        auto g = compute_gradient(rk[r].batches[k], lw, lb, rk[r].label[k], rk[r].sw[k], icpt, bias, loss, L);
        for (i64 q = 0; q < n; q++) lw[q] -= ra * g[q];
        if (icpt) lb -= ra * bias;
      }
      std::vector<T> d(n + 1);
      for (i64 q = 0; q < n; q++) d[q] = lw[q] - w[q];  // calc_diff_inplace
      d[n] = lb - b;
      delta[r] = std::move(d);
      lloss[r] = loss;
    });
    std::vector<T> tot = delta[0];
    for (int r = 1; r < P; r++)
      for (i64 q = 0; q <= n; q++) tot[q] += delta[r][q];
    sumloss = lloss[0];
    for (int r = 1; r < P; r++) sumloss += lloss[r];
    if (shrink) {
      // update_model_local (shrink_sgd_parallelizer.hpp:99-151): global -=
      // Σ(global - local) on the used columns, regularize(w) with eta = 1,
      // RMSE of the summed change + rank 0's own intercept change over rank
      // 0's column count + 1
      T sq = 0;
      for (i64 q = 0; q < n; q++) {
        if (!used[q]) continue;
        w[q] += tot[q];
        sq += tot[q] * tot[q];
      }
      if (icpt) b += tot[n];
      std::vector<T> uw;
      for (i64 q = 0; q < n; q++)
        if (used[q]) uw.push_back(w[q]);
      regularize(uw, rtype, lambda, 1.0, no_eta);
      for (i64 q = 0, k = 0; q < n; q++)
        if (used[q]) w[q] = uw[k++];
      if (icpt) sq += delta[0][n] * delta[0][n];
      double rmse = std::sqrt(sq / (T)(n_used0 + 1));
      if (rmse < tol) break;
      continue;
    }
    std::vector<T> prev = w;
    T prevb = b;
    for (i64 q = 0; q < n; q++) w[q] += tot[q];
    b += tot[n];
    regularize(w, rtype, lambda, alpha / std::sqrt((double)i), no_eta);
    // _RMSE_CONV_RATE_CHECK_: per-rank slices of Σ(prev-w)², summed in rank order
    i64 each = (n == 0) ? 0 : (n - 1) / P + 1;
    T red = 0;
    for (int r = 0; r < P; r++) {
      T s = 0;
      i64 st = each * r, en = std::min(each * (r + 1), n);
      for (i64 q = st; q < en; q++) {
        T df = prev[q] - w[q];
        s += df * df;
      }
      red += s;
    }
    red += (prevb - b) * (prevb - b);
    T rmse = (T)std::sqrt((double)(red / (T)(n + 1)));
    if (rmse < tol) break;
  }
  n_iter = (i == num_iter + 1) ? num_iter : i;
  if (shrink && fmt == ELL_F) n_iter = i;  // do_train_notrans reports i (shrink_sgd_parallelizer.hpp:315)
  if (shrink)
    for (i64 q = 0; q < n; q++)
      if (!used[q]) w[q] = 0;  // shrink_vector_merge: unheld columns are 0
  final_loss = sumloss;
}

// ------------------------------------------------------------ multinomial
// softmax_gradient_descent (ml/glm/softmax_gradient_descent.hpp): compute_wtx
// (159-177: data * weight, then + icpt per column), compute_exp_matrix
// (179-213, the max-stabilised branch: row max starting from column 0, then
// exp(x - max)), compute_softmax_probability (192-215: sum_of_cols, i.e. the
// row sums in column order, rowmajor_matrix.hpp:600-625, then diag(1/sum) *
// mat, rowmajor_matrix.hpp:452-480).
template <class T>
void softmax_probability(const CRS<T>& a, const std::vector<T>& W, const T* icpt, bool use_icpt, i64 K,
                         std::vector<T>& P) {
  const i64 m = a.nrow;
  P.assign((size_t)(m * K), T(0));
  crs_spmm(a, W.data(), K, P.data());
  if (use_icpt)
    for (i64 j = 0; j < K; j++)
      for (i64 i = 0; i < m; i++) P[i * K + j] = P[i * K + j] + icpt[j];
  for (i64 i = 0; i < m; i++) {
    T* row = &P[i * K];
    T mx = row[0];
    for (i64 j = 1; j < K; j++)
      if (row[j] > mx) mx = row[j];
    for (i64 j = 0; j < K; j++) row[j] = std::exp(row[j] - mx);
    T sum = 0;
    for (i64 j = 0; j < K; j++) sum = sum + row[j];
    const T inv = 1 / sum;
    for (i64 j = 0; j < K; j++) row[j] = inv * row[j];
  }
}

// softmax_parallelizer::do_train with the transposed copy
// (softmax_parallelizer.hpp:210-242): per iteration the gradient
// trans * ((softmax - onehot(label)) * sw) (compute_error_inplace 217-235),
// then update_global_model (147-200): w -= alpha/sqrt(i) * g, intercept -=
// alpha/sqrt(i) * sum_of_rows(g) (the column sums of the gradient matrix,
// rowmajor_matrix.hpp:555-565), regularize(w) with eta = 1, and the
// _CONV_RATE_CHECK_ test (common.hpp:21): RMS of the change of weights and
// intercepts over (nfeatures [+1]) * nclasses entries <= tol stops.
template <class T>
void softmax_train(const CRS<T>& a, const T* label, const T* sw, i64 K, i64 num_iter, double alpha, T lambda,
                   int rtype, bool icpt, double tol, std::vector<T>& W, std::vector<T>& b, i64& n_iter) {
  const i64 m = a.nrow, n = a.ncol;
  const CRS<T> t = transpose(a);
  std::vector<T> P, G;
  i64 i;
  for (i = 1; i <= num_iter; i++) {
    softmax_probability(a, W, b.data(), icpt, K, P);
    for (i64 j = 0; j < K; j++)
      for (i64 r = 0; r < m; r++) {
        P[r * K + j] -= (label[r] == (T)j) ? T(1) : T(0);
        P[r * K + j] *= sw[r];
      }
    G.assign((size_t)(n * K), T(0));
    crs_spmm(t, P.data(), K, G.data());
    const std::vector<T> Wp = W, bp = b;
    const T ra = alpha / std::sqrt((double)i);
    for (i64 e = 0; e < n * K; e++) W[e] = W[e] - ra * G[e];
    if (icpt) {
      std::vector<T> bias(K, T(0));
      for (i64 r = 0; r < n; r++)
        for (i64 j = 0; j < K; j++) bias[j] = bias[j] + G[r * K + j];
      for (i64 j = 0; j < K; j++) b[j] = b[j] - ra * bias[j];
    }
    regularize(W, rtype, lambda, 1.0);
    T sum = 0;
    for (i64 e = 0; e < n * K; e++) {
      const T d = W[e] - Wp[e];
      sum = sum + d * d;
    }
    i64 nft = n;
    if (icpt) {
      for (i64 j = 0; j < K; j++) {
        const T d = b[j] - bp[j];
        sum = sum + d * d;
      }
      nft++;
    }
    const T rmse = std::sqrt(sum / (T)(nft * K));
    if (rmse <= tol) break;
  }
  n_iter = (i == num_iter + 1) ? num_iter : i;
}

// Multinomial logistic regression by L-BFGS.  The reference trains the
// softmax model by gradient descent only (softmax_parallelizer.hpp); this
// composes its gradient — softmax_gradient_descent::compute_gradient with the
// transposed copy (softmax_gradient_descent.hpp:119-136): G = X^T ((softmax(X
// W) - onehot(label)) * sw), the softmax as compute_exp_matrix /
// compute_softmax_probability (159-215) — with the L-BFGS driver above.  The
// line search needs a loss, which the reference's softmax path does not
// compute: the cross-entropy sum_i -log p[i, label_i] = log(sum_j exp(z_ij -
// max_i)) - (z_i,label - max_i), unweighted as logistic_gradient's loss is
// while its dloss is weighted (gradient_descent.hpp:209); G is its gradient
// for unit weights.  The model vector is W row-major (n x K), no intercept.
template <class T>
void softmax_lbfgs_train(const CRS<T>& a, const T* label, const T* sw, i64 K, i64 num_iter, i64 hist, T lambda,
                         int rtype, double tol, std::vector<T>& W, i64& n_iter, double& final_loss, double* trace) {
  const i64 m = a.nrow, n = a.ncol;
  const CRS<T> t = transpose(a);
  auto eval = [&](const std::vector<T>& w, T, double& loss) {
    std::vector<T> Z((size_t)(m * K), T(0));
    crs_spmm(a, w.data(), K, Z.data());
    double sumloss = 0.0;
    for (i64 i = 0; i < m; i++) {
      T* row = &Z[(size_t)(i * K)];
      T mx = row[0];
      for (i64 j = 1; j < K; j++)
        if (row[j] > mx) mx = row[j];
      const i64 y = (i64)label[i];
      const T zy = row[y] - mx;
      T sum = 0;
      for (i64 j = 0; j < K; j++) {
        row[j] = std::exp(row[j] - mx);
        sum = sum + row[j];
      }
      const T inv = 1 / sum;
      for (i64 j = 0; j < K; j++) {
        T pr = inv * row[j];
        pr -= (y == j) ? T(1) : T(0);
        row[j] = pr * sw[i];
      }
      sumloss += (double)(std::log(sum) - zy);
    }
    loss = sumloss;
    std::vector<T> G((size_t)(n * K), T(0));
    crs_spmm(t, Z.data(), K, G.data());
    G.push_back(T(0));  // no intercept
    return G;
  };
  T b = 0;
  lbfgs_driver<T>(eval, CRS_F, W, b, num_iter, hist, lambda, rtype, tol, n_iter, final_loss, trace);
}

template <class T>
CRS<T> make_crs(i64 m, i64 n, const i32* off, const i32* idx, const T* val) {
  CRS<T> a;
  a.nrow = m;
  a.ncol = n;
  a.off.assign(off, off + m + 1);
  i64 nnz = a.off[m];
  a.idx.assign(idx, idx + nnz);
  a.val.assign(val, val + nnz);
  return a;
}

inline std::vector<i64> default_splits(i64 m, const i64* splits, int P) {
  std::vector<i64> s(P + 1);
  if (splits) for (int i = 0; i <= P; i++) s[i] = splits[i];
  else { s[0] = 0; s[1] = m; }
  return s;
}

}  // namespace orc

// =================================================================== C ABI
using namespace orc;

extern "C" {

void orc_crs_spmv_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* x, double* y) {
  auto a = make_crs<double>(m, n, off, idx, val);
  std::fill(y, y + m, 0.0);
  crs_spmv(a, x, y);
}
void orc_crs_spmv_f32(i64 m, i64 n, const i32* off, const i32* idx, const float* val, const float* x, float* y) {
  auto a = make_crs<float>(m, n, off, idx, val);
  std::fill(y, y + m, 0.0f);
  crs_spmv(a, x, y);
}

void orc_crs_transpose_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i32* toff, i32* tidx,
                           double* tval) {
  auto t = transpose(make_crs<double>(m, n, off, idx, val));
  for (i64 i = 0; i <= n; i++) toff[i] = (i32)t.off[i];
  std::copy(t.idx.begin(), t.idx.end(), tidx);
  std::copy(t.val.begin(), t.val.end(), tval);
}

void orc_crs_spmm_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* X, i64 k,
                      double* Y) {
  auto a = make_crs<double>(m, n, off, idx, val);
  std::fill(Y, Y + m * k, 0.0);
  crs_spmm(a, X, k, Y);
}

i64 orc_ell_width(i64 m, const i32* off) {
  i64 w = 0;
  for (i64 r = 0; r < m; r++) w = std::max<i64>(w, (i64)off[r + 1] - off[r]);
  return w;
}
void orc_ell_build_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i32* eidx, double* eval) {
  auto e = to_ell(make_crs<double>(m, n, off, idx, val));
  std::copy(e.idx.begin(), e.idx.end(), eidx);
  std::copy(e.val.begin(), e.val.end(), eval);
}
void orc_ell_spmv_f64(i64 m, i64 n, i64 width, const i32* eidx, const double* eval, const double* x, double* y) {
  ELL<double> e;
  e.nrow = m;
  e.ncol = n;
  e.idx.assign(eidx, eidx + m * width);
  e.val.assign(eval, eval + m * width);
  auto r = mv(e, std::vector<double>(x, x + n));
  std::copy(r.begin(), r.end(), y);
}
void orc_ell_trans_mv_f64(i64 m, i64 n, i64 width, const i32* eidx, const double* eval, const double* v, double* y) {
  ELL<double> e;
  e.nrow = m;
  e.ncol = n;
  e.idx.assign(eidx, eidx + m * width);
  e.val.assign(eval, eval + m * width);
  auto r = trans_mv(e, std::vector<double>(v, v + m));
  std::copy(r.begin(), r.end(), y);
}

// JDS: out_ndiag receives the number of diagonals; joff has ndiag+1 entries.
void orc_jds_build_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i32* perm, i64* joff,
                       i32* jidx, double* jval, i64* out_ndiag) {
  auto j = to_jds(make_crs<double>(m, n, off, idx, val));
  std::copy(j.perm.begin(), j.perm.end(), perm);
  std::copy(j.off.begin(), j.off.end(), joff);
  std::copy(j.idx.begin(), j.idx.end(), jidx);
  std::copy(j.val.begin(), j.val.end(), jval);
  *out_ndiag = (i64)j.off.size() - 1;
}
void orc_jds_spmv_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* x, double* y) {
  auto j = to_jds(make_crs<double>(m, n, off, idx, val));
  auto r = mv(j, std::vector<double>(x, x + n));
  std::copy(r.begin(), r.end(), y);
}

// Hybrid: info = [jds_ndiag, crs_num_row, crs_nnz, jds_nnz, perm_len]
void orc_hyb_info(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i64 thr, i64* info) {
  auto h = to_hyb(make_crs<double>(m, n, off, idx, val), thr);
  info[0] = (i64)h.jds.off.size() - 1;
  info[1] = h.crs.nrow;
  info[2] = (i64)h.crs.val.size();
  info[3] = (i64)h.jds.val.size();
  info[4] = (i64)h.jds.perm.size();
}
void orc_hyb_build_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i64 thr, i32* perm,
                       i64* joff, i32* jidx, double* jval, i64* coff, i32* cidx, double* cval) {
  auto h = to_hyb(make_crs<double>(m, n, off, idx, val), thr);
  std::copy(h.jds.perm.begin(), h.jds.perm.end(), perm);
  std::copy(h.jds.off.begin(), h.jds.off.end(), joff);
  std::copy(h.jds.idx.begin(), h.jds.idx.end(), jidx);
  std::copy(h.jds.val.begin(), h.jds.val.end(), jval);
  std::copy(h.crs.off.begin(), h.crs.off.end(), coff);
  std::copy(h.crs.idx.begin(), h.crs.idx.end(), cidx);
  std::copy(h.crs.val.begin(), h.crs.val.end(), cval);
}
void orc_hyb_spmv_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, i64 thr, const double* x,
                      double* y) {
  auto h = to_hyb(make_crs<double>(m, n, off, idx, val), thr);
  auto r = mv(h, std::vector<double>(x, x + n));
  std::copy(r.begin(), r.end(), y);
}

// Forward / backward product in any format as the glm path uses them.
void orc_fmt_mv_f64(int fmt, int trans, i64 m, i64 n, const i32* off, const i32* idx, const double* val,
                    const double* x, double* y) {
  RankData<double> d;
  d.build(make_crs<double>(m, n, off, idx, val), fmt);
  auto r = trans ? d.bwd(std::vector<double>(x, x + m)) : d.fwd(std::vector<double>(x, x + n));
  std::copy(r.begin(), r.end(), y);
}

void orc_glm_dloss_f64(int lkind, double eps, i64 m, const double* label, const double* wtx, double* dloss,
                       double* sumloss) {
  double s = 0;
  auto d = glm_dloss(Loss{lkind, eps}, std::vector<double>(label, label + m), std::vector<double>(wtx, wtx + m), s);
  std::copy(d.begin(), d.end(), dloss);
  *sumloss = s;
}

// One loss/gradient evaluation; grad has n+1 entries (bias last).
// loss: 0 logistic, 1 linear (squared), 2 hinge, 3 epsilon-insensitive,
// 4 squared epsilon-insensitive; eps used by 3 and 4.
void orc_glm_eval_f64(int fmt, i64 m, i64 n, const i32* off, const i32* idx, const double* val,
                      const double* label, const double* sw, const double* w, double b, int icpt,
                      const i64* splits, int P, int nthreads, double* grad, double* loss, int lkind, double eps) {
  auto a = make_crs<double>(m, n, off, idx, val);
  auto sp = default_splits(m, splits, P);
  auto pr = make_problem(a, label, sw, sp.data(), P, fmt, nthreads);
  pr.loss = Loss{lkind, eps};
  auto g = evaluate(pr, std::vector<double>(w, w + n), b, icpt != 0, *loss);
  std::copy(g.begin(), g.end(), grad);
}

int orc_glm_lbfgs_f64(int fmt, i64 m, i64 n, const i32* off, const i32* idx, const double* val,
                      const double* label, const double* sw, const i64* splits, int P, int nthreads,
                      i64 num_iter, i64 hist, double lambda, int rtype, int icpt, double tol, double* w,
                      double* b, i64* n_iter, double* final_loss, double* trace, int flags, int lkind, double eps) {
  if (fmt == JDS_F || fmt < 0 || fmt > 3) return 4;  // lbfgs_parallelizer.hpp:596-597
  if (hist < 1 || num_iter < 1 || lambda < 0 || tol < 0) return 1;
  if (lkind < 0 || lkind > 4) return 1;
  auto a = make_crs<double>(m, n, off, idx, val);
  auto sp = default_splits(m, splits, P);
  auto pr = make_problem(a, label, sw, sp.data(), P, fmt, nthreads);
  pr.loss = Loss{lkind, eps};
  std::vector<double> wv(w, w + n);
  double bb = *b;
  lbfgs_train(pr, fmt, wv, bb, num_iter, hist, lambda, rtype, icpt != 0, tol, *n_iter, *final_loss, trace,
              (flags & 1) != 0);
  std::copy(wv.begin(), wv.end(), w);
  *b = bb;
  return 0;
}

// The same trainer on a problem built once: the per-rank matrices and their
// transposed copies (lbfgs_parallelizer.hpp:562-597) are made by
// orc_problem_create and reused by every orc_problem_lbfgs call, so a timing
// of orc_problem_lbfgs covers the training loop alone.
struct OrcProblem {
  int fmt = CRS_F;
  i64 n = 0;
  Problem<double> pr;
};

void* orc_problem_create(int fmt, i64 m, i64 n, const i32* off, const i32* idx, const double* val,
                         const double* label, const double* sw, const i64* splits, int P, int nthreads, int lkind,
                         double eps) {
  if (fmt == JDS_F || fmt < 0 || fmt > 3 || lkind < 0 || lkind > 4) return nullptr;
  auto* h = new OrcProblem();
  h->fmt = fmt;
  h->n = n;
  auto a = make_crs<double>(m, n, off, idx, val);
  auto sp = default_splits(m, splits, P);
  h->pr = make_problem(a, label, sw, sp.data(), P, fmt, nthreads);
  h->pr.loss = Loss{lkind, eps};
  return h;
}

int orc_problem_lbfgs(void* hp, i64 num_iter, i64 hist, double lambda, int rtype, int icpt, double tol, double* w,
                      double* b, i64* n_iter, double* final_loss, double* trace, int flags) {
  auto* h = static_cast<OrcProblem*>(hp);
  if (!h || hist < 1 || num_iter < 1 || lambda < 0 || tol < 0) return 1;
  std::vector<double> wv(w, w + h->n);
  double bb = *b;
  lbfgs_train(h->pr, h->fmt, wv, bb, num_iter, hist, lambda, rtype, icpt != 0, tol, *n_iter, *final_loss, trace,
              (flags & 1) != 0);
  std::copy(wv.begin(), wv.end(), w);
  *b = bb;
  return 0;
}

void orc_problem_destroy(void* hp) { delete static_cast<OrcProblem*>(hp); }

// shrink::logistic_regression_with_sgd::train (flags bit 1 of orc_glm_sgd_f64)
int orc_glm_sgd_f64(int fmt, i64 m, i64 n, const i32* off, const i32* idx, const double* val,
                    const double* label, const double* sw, const i64* splits, int P, int nthreads,
                    i64 num_iter, double alpha, double frac, double lambda, int rtype, int icpt, double tol,
                    double* w, double* b, i64* n_iter, double* final_loss, int flags, int lkind, double eps) {
  if (fmt < 0 || fmt > 3) return 4;
  if (num_iter < 1 || alpha <= 0 || frac <= 0 || frac > 1 || lambda < 0 || tol < 0) return 1;
  if (lkind < 0 || lkind > 4) return 1;
  auto a = make_crs<double>(m, n, off, idx, val);
  auto sp = default_splits(m, splits, P);
  std::vector<double> wv(w, w + n);
  double bb = *b;
  sgd_train(a, label, sw, sp.data(), P, fmt, wv, bb, num_iter, alpha, frac, lambda, rtype, icpt != 0, tol, *n_iter,
            *final_loss, nthreads, (flags & 1) != 0, Loss{lkind, eps}, (flags & 2) != 0);
  std::copy(wv.begin(), wv.end(), w);
  *b = bb;
  return 0;
}

// logistic_regression_model<T>::predict_probability  (ml/glm/linear_model.hpp:376-392)
void orc_predict_probability_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* w,
                                 double b, double* out) {
  auto a = make_crs<double>(m, n, off, idx, val);
  auto v = mv(a, std::vector<double>(w, w + n));
  if (b != 0) for (auto& x : v) x += b;
  for (i64 i = 0; i < m; i++) {
    double e = -1.0 * v[i];
    out[i] = (e > 709) ? 0.0 : 1.0 / (1.0 + std::exp(e));
  }
}

// multinomial_logistic_regression::train main API
// (ml/glm/multinomial_logistic_regression.hpp:342-378) with CRS data:
// W[n*K] row-major and b[K] hold the initial model and receive the result.
int orc_softmax_lbfgs_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* label,
                          const double* sw, i64 K, i64 num_iter, i64 hist, double lambda, int rtype, double tol,
                          double* W, i64* n_iter, double* final_loss, double* trace) {
  if (K < 1 || num_iter < 1 || hist < 1 || lambda < 0 || tol < 0) return 1;
  auto a = make_crs<double>(m, n, off, idx, val);
  std::vector<double> w(W, W + n * K), swv(sw ? sw : nullptr, sw ? sw + m : nullptr);
  if (!sw) swv.assign((size_t)m, 1.0);
  softmax_lbfgs_train(a, label, swv.data(), K, num_iter, hist, lambda, rtype, tol, w, *n_iter, *final_loss, trace);
  std::copy(w.begin(), w.end(), W);
  return 0;
}

int orc_softmax_train_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* label,
                          const double* sw, i64 K, i64 num_iter, double alpha, double lambda, int rtype, int icpt,
                          double tol, double* W, double* b, i64* n_iter) {
  if (num_iter < 1 || alpha <= 0 || lambda < 0 || tol < 0 || K < 1) return 1;
  auto a = make_crs<double>(m, n, off, idx, val);
  std::vector<double> w(W, W + n * K), bb(b, b + K), ones;
  if (!sw) {
    ones.assign((size_t)m, 1.0);
    sw = ones.data();
  }
  softmax_train(a, label, sw, K, num_iter, alpha, lambda, rtype, icpt != 0, tol, w, bb, *n_iter);
  std::copy(w.begin(), w.end(), W);
  std::copy(bb.begin(), bb.end(), b);
  return 0;
}

// multinomial_logistic_regression_model<T>::compute_probability_matrix
// (multinomial_logistic_regression_model.hpp:82-89): prob[m*K].
void orc_softmax_probability_f64(i64 m, i64 n, const i32* off, const i32* idx, const double* val, const double* W,
                                 const double* b, i64 K, int icpt, double* prob) {
  auto a = make_crs<double>(m, n, off, idx, val);
  std::vector<double> w(W, W + n * K), P;
  softmax_probability(a, w, b, icpt != 0, K, P);
  std::copy(P.begin(), P.end(), prob);
}

}  // extern "C"
