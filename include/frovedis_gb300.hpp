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
//   make_crs_matrix_local_load / _loadlibsvm / _loadbinary, save, savebinary
//                                      crs_matrix.hpp:440-450, 565-634, 757-775, 874-899
//   logistic_regression<T> estimator   ml/glm/logistic_regression.hpp:13-460
//   model save / load (text, binary)   ml/glm/linear_model.hpp:39-150,
//                                      multinomial_logistic_regression_model.hpp:136-201
//   MatType, RegType, IndexOrigin      ml/utility/mattype.hpp:6-11, ml/glm/regularizer.hpp:8-12,
//                                      matrix/crs_matrix.hpp:30-34
//
// The matrices keep the reference's public fields (val, idx, off, perm,
// local_num_row, local_num_col) filled in the reference's array order; the
// products and the training run on the device.  Errors surface as the
// reference's exception types: std::runtime_error for operator* size
// mismatches, frovedis_gb300::error (a std::runtime_error) otherwise, with
// the reference's messages.  Index types must hold values below 2^31.
#ifndef FROVEDIS_GB300_HPP
#define FROVEDIS_GB300_HPP

#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
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

// IndexOrigin (matrix/crs_matrix.hpp:30-34)
enum IndexOrigin { AUTO = 0, ZERO_ORIG, ONE_ORIG };

namespace detail {
// get_type_name<T>() (core/utility.hpp:76-99) for the index / offset types
template <class X> inline const char* type_name() {
  static_assert(std::is_integral<X>::value && (sizeof(X) == 4 || sizeof(X) == 8), "32/64-bit integer index");
  return std::is_signed<X>::value ? (sizeof(X) == 4 ? "int32_t" : "int64_t")
                                  : (sizeof(X) == 4 ? "uint32_t" : "uint64_t");
}
// a device matrix read back into the reference's struct
template <class T, class I, class O> crs_matrix_local<T, I, O> to_local(fvg_matrix* h) {
  int64_t m = 0, n = 0, nnz = 0;
  frovedis_gb300::check(fvg_matrix_info(h, &m, &n, &nnz));
  std::vector<int32_t> off(m + 1), idx(nnz ? nnz : 1);
  std::vector<double> val(nnz ? nnz : 1);
  frovedis_gb300::check(fvg_matrix_get_crs(frovedis_gb300::context(), h, off.data(), idx.data(), val.data()));
  crs_matrix_local<T, I, O> r((size_t)m, (size_t)n);
  r.off.assign(off.begin(), off.end());
  r.idx.assign(idx.begin(), idx.begin() + nnz);
  r.val.assign(val.begin(), val.begin() + nnz);
  return r;
}
struct handle {
  fvg_matrix* h = nullptr;
  ~handle() { fvg_matrix_destroy(h); }
};
}  // namespace detail

// make_crs_matrix_local_load(file[, num_col]) (crs_matrix.hpp:757-775):
// "col:value" lines, parsed on the device
template <class T, class I = size_t, class O = size_t>
crs_matrix_local<T, I, O> make_crs_matrix_local_load(const std::string& file, long long num_col = -1) {
  detail::handle d;
  frovedis_gb300::check(fvg_matrix_load_text(frovedis_gb300::context(), file.c_str(),
                                             frovedis_gb300::dtype_of<T>::value, num_col, &d.h));
  return detail::to_local<T, I, O>(d.h);
}

// make_crs_matrix_local_loadlibsvm (crs_matrix.hpp:874-899)
template <class T, class I = size_t, class O = size_t>
crs_matrix_local<T, I, O> make_crs_matrix_local_loadlibsvm(const std::string& file, std::vector<T>& label,
                                                           IndexOrigin idxorg = AUTO) {
  detail::handle d;
  frovedis_gb300::check(fvg_matrix_load_libsvm(frovedis_gb300::context(), file.c_str(),
                                               frovedis_gb300::dtype_of<T>::value, (int)idxorg, &d.h));
  auto r = detail::to_local<T, I, O>(d.h);
  std::vector<double> lab(r.local_num_row);
  if (!lab.empty()) frovedis_gb300::check(fvg_matrix_get_labels(d.h, lab.data()));
  label.assign(lab.begin(), lab.end());
  return r;
}

// make_crs_matrix_local_loadbinary (crs_matrix.hpp:565-603)
template <class T, class I = size_t, class O = size_t>
crs_matrix_local<T, I, O> make_crs_matrix_local_loadbinary(const std::string& input) {
  detail::handle d;
  frovedis_gb300::check(fvg_matrix_load_binary(frovedis_gb300::context(), input.c_str(),
                                               frovedis_gb300::dtype_of<T>::value, detail::type_name<I>(),
                                               detail::type_name<O>(), &d.h));
  return detail::to_local<T, I, O>(d.h);
}

// ------------------------------------------------ distributed containers
// The reference's distributed types hold one block per MPI rank:
// crs_matrix<T,I,O> (matrix/crs_matrix.hpp) a node_local<crs_matrix_local>
// plus the global num_row / num_col, dvector<T> (core/dvector.hpp) a
// distributed vector.  One process drives one GPU here, so each holds a single
// block; gather() returns it as the reference's gather() returns the
// concatenated blocks.  The trainers take them as the reference's do
// (logistic_regression_with_lbfgs.hpp:11-128, logistic_regression_with_sgd.hpp:
// 11-128), so reference programs such as samples/glm/lr.cc compile unchanged.
template <class T> struct dvector {
  dvector() = default;
  explicit dvector(const std::vector<T>& v) : val(v) {}
  explicit dvector(std::vector<T>&& v) : val(std::move(v)) {}
  std::vector<T> gather() const { return val; }
  size_t size() const { return val.size(); }
  void clear() { std::vector<T>().swap(val); }
  std::vector<T> val;  // the one block
};
template <class T> dvector<T> make_dvector_scatter(const std::vector<T>& v) { return dvector<T>(v); }

template <class T, class I = size_t, class O = size_t> struct crs_matrix {
  crs_matrix() = default;
  explicit crs_matrix(const crs_matrix_local<T, I, O>& m)
      : data(m), num_row(m.local_num_row), num_col(m.local_num_col) {}
  explicit crs_matrix(crs_matrix_local<T, I, O>&& m)
      : data(std::move(m)), num_row(data.local_num_row), num_col(data.local_num_col) {}
  crs_matrix_local<T, I, O> gather() const { return data; }
  crs_matrix<T, I, O> transpose() const { return crs_matrix<T, I, O>(data.transpose()); }
  size_t get_local_num_row() const { return data.local_num_row; }
  void clear() {
    data.clear();
    num_row = num_col = 0;
  }
  crs_matrix_local<T, I, O> data;  // the one block (the reference: a node_local of them)
  size_t num_row = 0, num_col = 0;
};
template <class T, class I, class O>
crs_matrix<T, I, O> make_crs_matrix_scatter(const crs_matrix_local<T, I, O>& m) {
  return crs_matrix<T, I, O>(m);
}
// make_crs_matrix_load / _loadbinary / _loadlibsvm (crs_matrix.hpp:720-899,
// 1549-1627): the local loaders into one block
template <class T, class I = size_t, class O = size_t>
crs_matrix<T, I, O> make_crs_matrix_load(const std::string& file, long long num_col = -1) {
  return crs_matrix<T, I, O>(make_crs_matrix_local_load<T, I, O>(file, num_col));
}
template <class T, class I = size_t, class O = size_t>
crs_matrix<T, I, O> make_crs_matrix_loadbinary(const std::string& input) {
  return crs_matrix<T, I, O>(make_crs_matrix_local_loadbinary<T, I, O>(input));
}
template <class T, class I = size_t, class O = size_t>
crs_matrix<T, I, O> make_crs_matrix_loadlibsvm(const std::string& file, dvector<T>& label, IndexOrigin idxorg = AUTO) {
  std::vector<T> lab;
  auto r = crs_matrix<T, I, O>(make_crs_matrix_local_loadlibsvm<T, I, O>(file, lab, idxorg));
  label = dvector<T>(std::move(lab));
  return r;
}

// crs_matrix_local::save (operator<<, crs_matrix.hpp:440-450): "col:value"
// lines
template <class T, class I, class O>
void save(const crs_matrix_local<T, I, O>& mat, const std::string& file) {
  std::ofstream str(file.c_str());
  for (size_t row = 0; row < mat.local_num_row; row++) {
    for (O col = mat.off[row]; col < mat.off[row + 1]; col++) {
      str << mat.idx[col] << ":" << mat.val[col];
      if (col != mat.off[row + 1] - 1) str << " ";
    }
    str << "\n";
  }
  if (!str) throw std::runtime_error("cannot write " + file);
}

// crs_matrix_local::savebinary (crs_matrix.hpp:604-634): nums, type and the
// native-order val / idx / off arrays
template <class T, class I, class O>
void savebinary(const crs_matrix_local<T, I, O>& mat, const std::string& dir) {
  struct stat sb;
  if (stat(dir.c_str(), &sb) != 0) {
    if (mkdir(dir.c_str(), S_IRWXU | S_IRWXG | S_IRWXO) != 0) throw std::runtime_error("mkdir failed");
  } else if (!S_ISDIR(sb.st_mode)) {
    throw std::runtime_error(dir + " is not a directory");
  }
  std::ofstream nums((dir + "/nums").c_str());
  nums << mat.local_num_row << "\n" << mat.local_num_col << std::endl;
  std::ofstream type((dir + "/type").c_str());
  type << (sizeof(T) == 4 ? "float" : "double") << "\n" << detail::type_name<I>() << "\n"
       << detail::type_name<O>() << std::endl;
  auto dump = [&](const std::string& f, const void* p, size_t bytes) {
    std::ofstream o((dir + "/" + f).c_str(), std::ios::binary);
    o.write(static_cast<const char*>(p), (std::streamsize)bytes);
    if (!o) throw std::runtime_error("cannot write " + dir + "/" + f);
  };
  dump("val", mat.val.data(), sizeof(T) * mat.val.size());
  dump("idx", mat.idx.data(), sizeof(I) * mat.idx.size());
  dump("off", mat.off.data(), sizeof(O) * mat.off.size());
}

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
  void save(const std::string& path) const;
  void savebinary(const std::string& path) const;
  void load(const std::string& path);
  void loadbinary(const std::string& path);
  std::vector<T> weight;
  T intercept;
  T threshold;
};

namespace detail {
// One train() of any binary GLM: the model type carries weight / intercept;
// loss selects the gradient (fvg_loss), eps its epsilon.
template <class T, class I, class O, class MODEL>
MODEL train(bool sgd, crs_matrix_local<T, I, O>& data, std::vector<T>& label, MODEL& initModel,
            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration, double alpha, size_t hist_size,
            double miniBatchFraction, double regParam, RegType regTyp, bool isIntercept, double convergenceTol,
            MatType mType, fvg_loss loss = FVG_LOSS_LOGISTIC, double eps = 0.0, bool shrink = false) {
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
  p.loss = loss;
  p.epsilon = eps;
  std::vector<double> lab(label.begin(), label.end()), sw(sample_weight.begin(), sample_weight.end());
  std::vector<double> w(initModel.weight.begin(), initModel.weight.end());
  double b = initModel.intercept, fl = 0;
  int64_t it = 0;
  auto fn = sgd ? fvg_glm_sgd : fvg_glm_lbfgs;
  if (shrink) fn = fvg_logreg_shrink_sgd;
  frovedis_gb300::check(fn(frovedis_gb300::context(), d.h, lab.data(), sw.data(), &p, w.data(), &b, &it, &fl));
  n_iter = (size_t)it;
  MODEL ret = initModel;
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
  // the distributed overloads (logistic_regression_with_lbfgs.hpp:11-128);
  // the && ones set inputMovable, so the matrix is cleared after training
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            size_t hist_size = 10, double regParam = 0.01, RegType regTyp = ZERO,
                                            bool isIntercept = false, double convergenceTol = 0.001,
                                            MatType mType = CRS, bool inputMovable = false) {
    auto lab = label.gather();
    auto m = train(data.data, lab, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                   isIntercept, convergenceTol, mType, false);
    if (inputMovable) data.clear();
    return m;
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col, isIntercept ? 1.0 : 0.0);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType, false);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                            double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col, isIntercept ? 1.0 : 0.0);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType, false);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col, isIntercept ? 1.0 : 0.0);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType, true);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                            double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col, isIntercept ? 1.0 : 0.0);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType, true);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            size_t hist_size = 10, double regParam = 0.01, RegType regTyp = ZERO,
                                            bool isIntercept = false, double convergenceTol = 0.001,
                                            MatType mType = CRS) {
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType, true);
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
    logistic_regression_model<T> initModel(data.local_num_col);  // intercept 0 (line 300)
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
  // the distributed overloads (logistic_regression_with_sgd.hpp:11-128);
  // the && ones set inputMovable
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS,
                                            bool inputMovable = false) {
    auto lab = label.gather();
    auto m = train(data.data, lab, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction,
                   regParam, regTyp, isIntercept, convergenceTol, mType, false);
    if (inputMovable) data.clear();
    return m;
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType, false);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>& data, dvector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                            double alpha = 0.01, double miniBatchFraction = 1.0,
                                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType, false);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col);
    size_t n_iter = 0;
    std::vector<T> sample_weight;
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType, true);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                            double alpha = 0.01, double miniBatchFraction = 1.0,
                                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType, true);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix<T, I, O>&& data, dvector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType, true);
  }
};

namespace shrink {
// shrink::logistic_regression_with_sgd (ml/glm/shrink_logistic_regression_with_sgd.hpp
// → shrink_sgd_parallelizer.hpp): SGD over per-rank shrunk column sets.
struct logistic_regression_with_sgd {
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, miniBatchFraction, regParam, regTyp, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            std::vector<T>& sample_weight, size_t& n_iter,
                                            size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS) {
    logistic_regression_model<T> initModel(data.local_num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static logistic_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                            logistic_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                            double miniBatchFraction = 1.0, double regParam = 0.01,
                                            RegType regTyp = ZERO, bool isIntercept = false,
                                            double convergenceTol = 0.001, MatType mType = CRS,
                                            bool inputMovable = false) {
    auto m = detail::train(true, data, label, initModel, sample_weight, n_iter, numIteration, alpha, 10,
                           miniBatchFraction, regParam, regTyp, isIntercept, convergenceTol, mType,
                           FVG_LOSS_LOGISTIC, 0.0, true);
    if (inputMovable) data.clear();
    return m;
  }
};
}  // namespace shrink

// linear_regression_model<T> (ml/glm/linear_model.hpp:211-298): weights
// start at 1; predict = mat * weight (+ intercept when non-zero).
template <class T>
struct linear_regression_model {
  linear_regression_model() : intercept(0.0) {}
  linear_regression_model(size_t numFtr, T intercpt = 0.0) : weight(numFtr, 1), intercept(intercpt) {}
  template <class MATRIX>
  std::vector<T> predict(const MATRIX& mat) const {
    std::vector<T> v = mat * weight;
    if (intercept != 0)
      for (auto& x : v) x += intercept;
    return v;
  }
  size_t get_num_features() const { return weight.size(); }
  void save(const std::string& path) const;
  void savebinary(const std::string& path) const;
  void load(const std::string& path);
  void loadbinary(const std::string& path);
  std::vector<T> weight;
  T intercept;
};

#define FVG_YES_RESPONSE 1   // linear_model.hpp:13-14
#define FVG_NO_RESPONSE -1

// svm_model<T> (ml/glm/linear_model.hpp:466-594): predict_probability is the
// raw score mat * weight (+ intercept); predict is +1 where the score is
// above 0, else -1 (the threshold is kept but not used, lines 538-549).
template <class T>
struct svm_model {
  svm_model() : intercept(0.0), threshold(0.0) {}
  svm_model(size_t numFtr, T intercpt = 0.0, T thr = 0.0) : weight(numFtr, 1), intercept(intercpt), threshold(thr) {
    if (!(thr >= 0)) throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "checkAssumption failed: thr >= 0");
  }
  template <class MATRIX>
  std::vector<T> predict_probability(const MATRIX& mat, bool = false) const {
    std::vector<T> v = mat * weight;
    if (intercept != 0)
      for (auto& x : v) x += intercept;
    return v;
  }
  template <class MATRIX>
  std::vector<T> predict(const MATRIX& mat) const {
    auto s = predict_probability(mat);
    std::vector<T> r(s.size());
    for (size_t i = 0; i < s.size(); i++) r[i] = s[i] > 0 ? FVG_YES_RESPONSE : FVG_NO_RESPONSE;
    return r;
  }
  void set_threshold(T thr) {
    if (thr < 0) throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Negative Threshold Value\n");
    threshold = thr;
  }
  T get_threshold() const { return threshold; }
  size_t get_num_features() const { return weight.size(); }
  size_t get_num_classes() const { return 2; }
  void save(const std::string& path) const;
  void savebinary(const std::string& path) const;
  void load(const std::string& path);
  void loadbinary(const std::string& path);
  std::vector<T> weight;
  T intercept;
  T threshold;
};

// The regression and SVM trainers: one template per (model, loss,
// regulariser) over the shared device driver.  SGD trainers start from
// initModel(numFeatures) (intercept 0), L-BFGS trainers from
// initModel(numFeatures, isIntercept) (e.g. linear_regression_with_sgd.hpp:242,
// linear_regression_with_lbfgs.hpp:243).
namespace detail {
template <class MODEL, class T, class I, class O>
MODEL glm_sgd(crs_matrix_local<T, I, O>& data, std::vector<T>& label, MODEL& initModel,
              std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration, double alpha,
              double miniBatchFraction, double regParam, RegType regTyp, bool isIntercept, double convergenceTol,
              MatType mType, bool inputMovable, fvg_loss loss, double eps = 0.0) {
  auto m = train(true, data, label, initModel, sample_weight, n_iter, numIteration, alpha, 10, miniBatchFraction,
                 regParam, regTyp, isIntercept, convergenceTol, mType, loss, eps);
  if (inputMovable) data.clear();
  return m;
}
template <class MODEL, class T, class I, class O>
MODEL glm_lbfgs(crs_matrix_local<T, I, O>& data, std::vector<T>& label, MODEL& initModel,
                std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration, double alpha, size_t hist_size,
                double regParam, RegType regTyp, bool isIntercept, double convergenceTol, MatType mType,
                bool inputMovable, fvg_loss loss) {
  auto m = train(false, data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, 1.0,
                 regParam, regTyp, isIntercept, convergenceTol, mType, loss);
  if (inputMovable) data.clear();
  return m;
}
}  // namespace detail

// linear_regression_with_sgd (ml/glm/linear_regression_with_sgd.hpp:304-330):
// linear_gradient, zero_regularizer.
struct linear_regression_with_sgd {
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, miniBatchFraction, isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                          double alpha = 0.01, double miniBatchFraction = 1.0,
                                          bool isIntercept = false, double convergenceTol = 0.001,
                                          MatType mType = CRS) {
    linear_regression_model<T> initModel(data.local_num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          linear_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                          size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS,
                                          bool inputMovable = false) {
    return detail::glm_sgd(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, 0.0,
                           ZERO, isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_SQUARED);
  }
};

// linear_regression_with_lbfgs (ml/glm/linear_regression_with_lbfgs.hpp:319-352)
struct linear_regression_with_lbfgs {
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                                          bool isIntercept = false, double convergenceTol = 0.001,
                                          MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, hist_size, isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                          double alpha = 0.01, size_t hist_size = 10, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS) {
    linear_regression_model<T> initModel(data.local_num_col, isIntercept);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          linear_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                          size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                          size_t hist_size = 10, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS,
                                          bool inputMovable = false) {
    return detail::glm_lbfgs(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, 0.0, ZERO,
                             isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_SQUARED);
  }
};

// lasso_with_sgd / ridge_regression_with_sgd (ml/glm/lasso_with_sgd.hpp,
// ridge_regression_with_sgd.hpp): linear_gradient with l1_regularizer /
// l2_regularizer(regParam).
template <RegType REG>
struct penalized_regression_with_sgd {
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, double regParam = 0.01,
                                          bool isIntercept = false, double convergenceTol = 0.001,
                                          MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, miniBatchFraction, regParam, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                          double alpha = 0.01, double miniBatchFraction = 1.0,
                                          double regParam = 0.01, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS) {
    linear_regression_model<T> initModel(data.local_num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          linear_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                          size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, double regParam = 0.01,
                                          bool isIntercept = false, double convergenceTol = 0.001,
                                          MatType mType = CRS, bool inputMovable = false) {
    return detail::glm_sgd(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction,
                           regParam, REG, isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_SQUARED);
  }
};
using lasso_with_sgd = penalized_regression_with_sgd<L1>;
using ridge_regression_with_sgd = penalized_regression_with_sgd<L2>;

// lasso_with_lbfgs / ridge_regression_with_lbfgs (lasso_with_lbfgs.hpp,
// ridge_regression_with_lbfgs.hpp)
template <RegType REG>
struct penalized_regression_with_lbfgs {
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                                          double regParam = 0.01, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, hist_size, regParam, isIntercept, convergenceTol,
                 mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                          double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                                          bool isIntercept = false, double convergenceTol = 0.001,
                                          MatType mType = CRS) {
    linear_regression_model<T> initModel(data.local_num_col, isIntercept);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam,
                 isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          linear_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                          size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                          size_t hist_size = 10, double regParam = 0.01, bool isIntercept = false,
                                          double convergenceTol = 0.001, MatType mType = CRS,
                                          bool inputMovable = false) {
    return detail::glm_lbfgs(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size,
                             regParam, REG, isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_SQUARED);
  }
};
using lasso_with_lbfgs = penalized_regression_with_lbfgs<L1>;
using ridge_regression_with_lbfgs = penalized_regression_with_lbfgs<L2>;

// svm_with_sgd (ml/glm/svm_with_sgd.hpp): hinge_gradient, labels +-1.
struct svm_with_sgd {
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, size_t numIteration = 1000,
                            double alpha = 0.01, double miniBatchFraction = 1.0, double regParam = 0.01,
                            RegType regTyp = ZERO, bool isIntercept = false, double convergenceTol = 0.001,
                            MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, miniBatchFraction, regParam, regTyp, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, std::vector<T>& sample_weight,
                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                            double miniBatchFraction = 1.0, double regParam = 0.01, RegType regTyp = ZERO,
                            bool isIntercept = false, double convergenceTol = 0.001, MatType mType = CRS) {
    svm_model<T> initModel(data.local_num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, svm_model<T>& initModel,
                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                            double alpha = 0.01, double miniBatchFraction = 1.0, double regParam = 0.01,
                            RegType regTyp = ZERO, bool isIntercept = false, double convergenceTol = 0.001,
                            MatType mType = CRS, bool inputMovable = false) {
    return detail::glm_sgd(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction,
                           regParam, regTyp, isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_HINGE);
  }
};

// svm_with_lbfgs (ml/glm/svm_with_lbfgs.hpp)
struct svm_with_lbfgs {
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, size_t numIteration = 1000,
                            double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                            RegType regTyp = ZERO, bool isIntercept = false, double convergenceTol = 0.001,
                            MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, hist_size, regParam, regTyp, isIntercept,
                 convergenceTol, mType);
  }
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, std::vector<T>& sample_weight,
                            size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01, size_t hist_size = 10,
                            double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                            double convergenceTol = 0.001, MatType mType = CRS) {
    svm_model<T> initModel(data.local_num_col, isIntercept);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam, regTyp,
                 isIntercept, convergenceTol, mType);
  }
  template <class T, class I, class O>
  static svm_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label, svm_model<T>& initModel,
                            std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                            double alpha = 0.01, size_t hist_size = 10, double regParam = 0.01,
                            RegType regTyp = ZERO, bool isIntercept = false, double convergenceTol = 0.001,
                            MatType mType = CRS, bool inputMovable = false) {
    return detail::glm_lbfgs(data, label, initModel, sample_weight, n_iter, numIteration, alpha, hist_size, regParam,
                             regTyp, isIntercept, convergenceTol, mType, inputMovable, FVG_LOSS_HINGE);
  }
};

// SVRLossType and svm_regression_with_sgd (ml/glm/svm_regression_with_sgd.hpp:
// 8-11, 373-444): epsilon_insensitive (EPS) or squared_epsilon_insensitive
// (SQEPS) with epsilon; a linear_regression_model.
enum SVRLossType { EPS = 0, SQEPS };
struct svm_regression_with_sgd {
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, double regParam = 0.01,
                                          RegType regTyp = ZERO, bool isIntercept = false,
                                          double convergenceTol = 0.001, double epsilon = 0.0,
                                          SVRLossType lossType = EPS, MatType mType = CRS) {
    std::vector<T> sw;
    size_t n_iter = 0;
    return train(data, label, sw, n_iter, numIteration, alpha, miniBatchFraction, regParam, regTyp, isIntercept,
                 convergenceTol, epsilon, lossType, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          std::vector<T>& sample_weight, size_t& n_iter, size_t numIteration = 1000,
                                          double alpha = 0.01, double miniBatchFraction = 1.0,
                                          double regParam = 0.01, RegType regTyp = ZERO, bool isIntercept = false,
                                          double convergenceTol = 0.001, double epsilon = 0.0,
                                          SVRLossType lossType = EPS, MatType mType = CRS) {
    linear_regression_model<T> initModel(data.local_num_col);
    return train(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction, regParam,
                 regTyp, isIntercept, convergenceTol, epsilon, lossType, mType);
  }
  template <class T, class I, class O>
  static linear_regression_model<T> train(crs_matrix_local<T, I, O>& data, std::vector<T>& label,
                                          linear_regression_model<T>& initModel, std::vector<T>& sample_weight,
                                          size_t& n_iter, size_t numIteration = 1000, double alpha = 0.01,
                                          double miniBatchFraction = 1.0, double regParam = 0.01,
                                          RegType regTyp = ZERO, bool isIntercept = false,
                                          double convergenceTol = 0.001, double epsilon = 0.0,
                                          SVRLossType lossType = EPS, MatType mType = CRS,
                                          bool inputMovable = false) {
    if (lossType != EPS && lossType != SQEPS)
      throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Unsupported SVR Loss!\n");
    return detail::glm_sgd(data, label, initModel, sample_weight, n_iter, numIteration, alpha, miniBatchFraction,
                           regParam, regTyp, isIntercept, convergenceTol, mType, inputMovable,
                           lossType == EPS ? FVG_LOSS_EPS_INSENSITIVE : FVG_LOSS_SQ_EPS_INSENSITIVE, epsilon);
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
  void save(const std::string& dir) const;
  void savebinary(const std::string& dir) const;
  void load(const std::string& dir);
  void loadbinary(const std::string& dir);
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

// ------------------------------------------------------------ persistence
namespace detail {
inline void make_directory(const std::string& dir) {
  struct stat sb;
  if (stat(dir.c_str(), &sb) != 0) {
    if (mkdir(dir.c_str(), S_IRWXU | S_IRWXG | S_IRWXO) != 0) throw std::runtime_error("mkdir failed");
  } else if (!S_ISDIR(sb.st_mode)) {
    throw std::runtime_error(dir + " is not a directory");
  }
}
// dvector<T>::savebinary / make_dvector_loadbinary: a raw native array
template <class T> void write_raw(const std::string& f, const std::vector<T>& v) {
  std::ofstream o(f.c_str(), std::ios::binary);
  o.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(sizeof(T) * v.size()));
  if (!o) throw std::runtime_error("cannot write " + f);
}
template <class T> std::vector<T> read_raw(const std::string& f) {
  std::ifstream i(f.c_str(), std::ios::binary | std::ios::ate);
  if (!i) throw std::runtime_error("cannot open " + f);
  const std::streamsize sz = i.tellg();
  if (sz % (std::streamsize)sizeof(T)) throw std::runtime_error("make_dvector_loadbinary: incorrect filesize");
  std::vector<T> v((size_t)sz / sizeof(T));
  i.seekg(0);
  i.read(reinterpret_cast<char*>(v.data()), sz);
  return v;
}
template <class T> const char* value_type_name() { return sizeof(T) == 4 ? "float" : "double"; }
}  // namespace detail

// rowmajor_matrix_local<T>::save / make_rowmajor_matrix_local_load
// (rowmajor_matrix.hpp:227-240, 323-340, 366-370): one row per line
template <class T> void save(const rowmajor_matrix_local<T>& m, const std::string& file) {
  std::ofstream str(file.c_str());
  for (size_t r = 0; r < m.local_num_row; r++) {
    for (size_t c = 0; c + 1 < m.local_num_col; c++) str << m.val[m.local_num_col * r + c] << " ";
    if (m.local_num_col) str << m.val[m.local_num_col * r + m.local_num_col - 1];
    str << "\n";
  }
}
template <class T> rowmajor_matrix_local<T> make_rowmajor_matrix_local_load(const std::string& file) {
  std::ifstream str(file.c_str());
  rowmajor_matrix_local<T> ret;
  std::string line;
  size_t lines = 0, width = 0;
  while (std::getline(str, line)) {
    std::istringstream ls(line);
    size_t k = 0;
    for (T x; ls >> x; k++) ret.val.push_back(x);
    if (lines == 0) width = k;
    lines++;
  }
  ret.local_num_row = lines;
  ret.local_num_col = width;
  return ret;
}
// rowmajor_matrix_local<T>::savebinary / make_rowmajor_matrix_local_loadbinary
// (rowmajor_matrix.hpp:760-810): nums, type, val
template <class T> void savebinary(const rowmajor_matrix_local<T>& m, const std::string& dir) {
  detail::make_directory(dir);
  std::ofstream((dir + "/nums").c_str()) << m.local_num_row << "\n" << m.local_num_col << std::endl;
  std::ofstream((dir + "/type").c_str()) << detail::value_type_name<T>() << std::endl;
  detail::write_raw(dir + "/val", m.val);
}
template <class T> rowmajor_matrix_local<T> make_rowmajor_matrix_local_loadbinary(const std::string& dir) {
  rowmajor_matrix_local<T> ret;
  std::ifstream nums((dir + "/nums").c_str());
  if (!(nums >> ret.local_num_row >> ret.local_num_col)) throw std::runtime_error("cannot read " + dir + "/nums");
  std::ifstream ty((dir + "/type").c_str());
  std::string t;
  if (ty >> t && t != detail::value_type_name<T>())
    throw std::runtime_error(std::string("make_rowmajor_matrix_local_loadbinary: val type mismatch detected! "
                                         "expected type: ") + t + "; given type: " + detail::value_type_name<T>() +
                             "\n");
  ret.val = detail::read_raw<T>(dir + "/val");
  return ret;
}

// glm_save / glm_savebinary / glm_load / glm_loadbinary
// (ml/glm/linear_model.hpp:39-140): the weights, the intercept and, for the
// classifiers, the threshold, one value per line (12 significant digits) or
// as one raw array.  The linear-regression overloads have no threshold.
namespace detail {
template <class T> void glm_save(const std::vector<T>& w, T icpt, const T* thr, const std::string& path) {
  std::ofstream out(path.c_str());
  out << std::setprecision(12);
  for (auto x : w) out << x << "\n";
  out << icpt << std::endl;
  if (thr) out << *thr << std::endl;
}
template <class T> void glm_savebinary(const std::vector<T>& w, T icpt, const T* thr, const std::string& path) {
  std::vector<T> tmp(w);
  tmp.push_back(icpt);
  if (thr) tmp.push_back(*thr);
  write_raw(path, tmp);
}
template <class T> void glm_split(std::vector<T>& w, T& icpt, T* thr, const std::string& path) {
  if (w.size() < (thr ? 2u : 1u)) throw std::runtime_error("model file " + path + " is too short");
  if (thr) {
    *thr = w.back();
    w.pop_back();
  }
  icpt = w.back();
  w.pop_back();
}
template <class T> void glm_load(std::vector<T>& w, T& icpt, T* thr, const std::string& path) {
  std::ifstream in(path.c_str());
  w.clear();
  for (T x; in >> x;) w.push_back(x);
  glm_split(w, icpt, thr, path);
}
template <class T> void glm_loadbinary(std::vector<T>& w, T& icpt, T* thr, const std::string& path) {
  w = read_raw<T>(path);
  glm_split(w, icpt, thr, path);
}
}  // namespace detail

template <class T> void save(const logistic_regression_model<T>& m, const std::string& path) {
  detail::glm_save(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void savebinary(const logistic_regression_model<T>& m, const std::string& path) {
  detail::glm_savebinary(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void load(logistic_regression_model<T>& m, const std::string& path) {
  detail::glm_load(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void loadbinary(logistic_regression_model<T>& m, const std::string& path) {
  detail::glm_loadbinary(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void save(const svm_model<T>& m, const std::string& path) {
  detail::glm_save(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void savebinary(const svm_model<T>& m, const std::string& path) {
  detail::glm_savebinary(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void load(svm_model<T>& m, const std::string& path) {
  detail::glm_load(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void loadbinary(svm_model<T>& m, const std::string& path) {
  detail::glm_loadbinary(m.weight, m.intercept, &m.threshold, path);
}
template <class T> void save(const linear_regression_model<T>& m, const std::string& path) {
  detail::glm_save<T>(m.weight, m.intercept, nullptr, path);
}
template <class T> void savebinary(const linear_regression_model<T>& m, const std::string& path) {
  detail::glm_savebinary<T>(m.weight, m.intercept, nullptr, path);
}
template <class T> void load(linear_regression_model<T>& m, const std::string& path) {
  detail::glm_load<T>(m.weight, m.intercept, nullptr, path);
}
template <class T> void loadbinary(linear_regression_model<T>& m, const std::string& path) {
  detail::glm_loadbinary<T>(m.weight, m.intercept, nullptr, path);
}

// multinomial model save / savebinary / load / loadbinary
// (multinomial_logistic_regression_model.hpp:136-201): weight, intercept,
// metadata (nclasses, nfeatures, isIntercept, threshold)
template <class T> void save(const multinomial_logistic_regression_model<T>& m, const std::string& dir) {
  detail::make_directory(dir);
  save(m.weight, dir + "/weight");
  std::ofstream ic((dir + "/intercept").c_str());
  for (auto& e : m.intercept) ic << e << std::endl;
  std::ofstream md((dir + "/metadata").c_str());
  md << m.nclasses << std::endl << m.nfeatures << std::endl << m.isIntercept << std::endl << m.threshold << std::endl;
}
template <class T> void savebinary(const multinomial_logistic_regression_model<T>& m, const std::string& dir) {
  detail::make_directory(dir);
  savebinary(m.weight, dir + "/weight");
  detail::write_raw(dir + "/intercept", m.intercept);
  std::ofstream md((dir + "/metadata").c_str());
  md << m.nclasses << std::endl << m.nfeatures << std::endl << m.isIntercept << std::endl << m.threshold << std::endl;
}
template <class T> void load(multinomial_logistic_regression_model<T>& m, const std::string& dir) {
  m.weight = make_rowmajor_matrix_local_load<T>(dir + "/weight");
  std::ifstream ic((dir + "/intercept").c_str());
  m.intercept.clear();
  for (T x; ic >> x;) m.intercept.push_back(x);
  std::ifstream md((dir + "/metadata").c_str());
  md >> m.nclasses >> m.nfeatures >> m.isIntercept >> m.threshold;
}
template <class T> void loadbinary(multinomial_logistic_regression_model<T>& m, const std::string& dir) {
  m.weight = make_rowmajor_matrix_local_loadbinary<T>(dir + "/weight");
  m.intercept = detail::read_raw<T>(dir + "/intercept");
  std::ifstream md((dir + "/metadata").c_str());
  md >> m.nclasses >> m.nfeatures >> m.isIntercept >> m.threshold;
}

// Member forms of the persistence calls (model.save(path) ... as the
// reference's models declare them).
#define FVG_GLM_MEMBERS(MODEL)                                                                            \
  template <class T> void MODEL<T>::save(const std::string& p) const { frovedis::save(*this, p); }             \
  template <class T> void MODEL<T>::savebinary(const std::string& p) const { frovedis::savebinary(*this, p); } \
  template <class T> void MODEL<T>::load(const std::string& p) { frovedis::load(*this, p); }                   \
  template <class T> void MODEL<T>::loadbinary(const std::string& p) { frovedis::loadbinary(*this, p); }
FVG_GLM_MEMBERS(logistic_regression_model)
FVG_GLM_MEMBERS(linear_regression_model)
FVG_GLM_MEMBERS(svm_model)
FVG_GLM_MEMBERS(multinomial_logistic_regression_model)
#undef FVG_GLM_MEMBERS

// accuracy_score (ml/metrics.hpp:383-396)
template <class T> float accuracy_score(const std::vector<T>& true_label, const std::vector<T>& pred_label) {
  if (true_label.size() != pred_label.size())
    throw std::runtime_error("accuracy_score: size differs in predicted labels and actual labels!\n");
  size_t count = 0;
  for (size_t i = 0; i < true_label.size(); i++) count += true_label[i] == pred_label[i];
  return true_label.empty() ? 0.0f : (float)count / (float)true_label.size();
}

// logistic_regression<T> estimator (ml/glm/logistic_regression.hpp:13-460),
// on a local CRS matrix: the solver dispatch of _fit (lines 237-298), a
// multinomial model when the labels hold more than two classes.
template <class T>
struct logistic_regression {
  logistic_regression(int max_iter = 1000, double alpha = 0.01, const std::string& solver = "sgd",
                      double reg_param = 0.01, const std::string& reg_type = "ZERO", bool fit_intercept = false,
                      double mini_batch_fraction = 1.0, int hs = 10, double convergence_tol = 0.001,
                      bool is_mult = false, bool warm_start = false, MatType mType = CRS)
      : max_iter(max_iter), hist_size(hs), alpha(alpha), mbf(mini_batch_fraction), tol(convergence_tol),
        reg_param(reg_param), solver(solver), reg_type(reg_type), fit_intercept(fit_intercept), is_mult(is_mult),
        warm_start(warm_start), is_fitted(false), mat_type(mType), n_iter_(0), n_features_(0), n_classes_(0) {}

  static void require(bool c, const std::string& msg) {
    if (!c) throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, msg);
  }
  logistic_regression& set_max_iter(int v) {
    require(v > 0, "expected a positive max_iter; received: " + std::to_string(v) + "\n");
    max_iter = v;
    return *this;
  }
  logistic_regression& set_alpha(double v) {
    require(v > 0, "expected a positive alpha (learning rate); received: " + std::to_string(v) + "\n");
    alpha = v;
    return *this;
  }
  logistic_regression& set_solver(const std::string& s) {
    require(s == "sgd" || s == "shrink-sgd" || s == "lbfgs", "expected sgd, shrink-sgd or lbfgs; received: " + s + "\n");
    solver = s;
    return *this;
  }
  logistic_regression& set_reg_param(double v) {
    require(v > 0, "expected a positive regularization parameter; received: " + std::to_string(v) + "\n");
    reg_param = v;
    return *this;
  }
  logistic_regression& set_reg_type(const std::string& s) {
    require(s == "ZERO" || s == "L1" || s == "L2", "expected ZERO, L1 or L2; received: " + s + "\n");
    reg_type = s;
    return *this;
  }
  logistic_regression& set_intercept(bool v) {
    fit_intercept = v;
    return *this;
  }
  logistic_regression& set_mini_batch_fraction(double v) {
    require(v > 0, "expected a positive mini-batch fraction; received: " + std::to_string(v) + "\n");
    mbf = v;
    return *this;
  }
  logistic_regression& set_hist_size(int v) {
    require(v > 0, "expected a positive history size; received: " + std::to_string(v) + "\n");
    hist_size = v;
    return *this;
  }
  logistic_regression& set_tol(double v) {
    require(v >= 0, "expected a positive or zero convergence tolerance; received: " + std::to_string(v) + "\n");
    tol = v;
    return *this;
  }
  logistic_regression& set_is_mult(bool v) {
    is_mult = v;
    return *this;
  }
  logistic_regression& set_warm_start(bool v) {
    warm_start = v;
    return *this;
  }
  RegType get_regularizer() const {
    if (reg_type == "ZERO") return ZERO;
    if (reg_type == "L1") return L1;
    if (reg_type == "L2") return L2;
    throw frovedis_gb300::error(FVG_ERR_INVALID_ARG,
                                "[logistic_regression] Unknown regularizer '" + reg_type + "' is encountered!\n");
  }

  template <class I, class O>
  logistic_regression& fit(crs_matrix_local<T, I, O>& mat, std::vector<T>& label) {
    std::vector<T> sample_weight;
    return fit(mat, label, sample_weight);
  }
  template <class I, class O>
  logistic_regression& fit(crs_matrix_local<T, I, O>& mat, std::vector<T>& label, std::vector<T>& sample_weight) {
    std::vector<T> u(label);
    std::sort(u.begin(), u.end());
    const size_t nclasses = (size_t)(std::unique(u.begin(), u.end()) - u.begin());
    if (nclasses > 2) is_mult = true;
    const size_t nfeatures = mat.local_num_col;
    if (!(warm_start && is_fitted)) {
      if (is_mult) model_mult = multinomial_logistic_regression_model<T>(nfeatures, nclasses, fit_intercept);
      else model_bin = logistic_regression_model<T>(nfeatures, fit_intercept ? 1.0 : 0.0);
    } else {
      require(nfeatures == n_features_, "Fitted model dimension does not match with number of features in input data\n");
      require(nclasses == n_classes_, "Fitted model dimension does not match with number of labels in input data\n");
    }
    size_t n_iter = 0;
    if (is_mult) {
      require(solver == "sgd", "Multinomil classification is only supported for sgd solver\n");
      model_mult = multinomial_logistic_regression::train(mat, label, model_mult, sample_weight, n_iter, max_iter,
                                                          alpha, reg_param, get_regularizer(), fit_intercept, tol,
                                                          mat_type);
    } else if (solver == "sgd") {
      model_bin = logistic_regression_with_sgd::train(mat, label, model_bin, sample_weight, n_iter, max_iter, alpha,
                                                      mbf, reg_param, get_regularizer(), fit_intercept, tol,
                                                      mat_type);
    } else if (solver == "shrink-sgd") {
      model_bin = shrink::logistic_regression_with_sgd::train(mat, label, model_bin, sample_weight, n_iter, max_iter,
                                                              alpha, mbf, reg_param, get_regularizer(),
                                                              fit_intercept, tol, mat_type);
    } else if (solver == "lbfgs") {
      model_bin = logistic_regression_with_lbfgs::train(mat, label, model_bin, sample_weight, n_iter, max_iter,
                                                        alpha, hist_size, reg_param, get_regularizer(),
                                                        fit_intercept, tol, mat_type);
    } else {
      throw frovedis_gb300::error(FVG_ERR_INVALID_ARG, "Unknown solver is encountered!\n");
    }
    is_fitted = true;
    n_iter_ = n_iter;
    n_features_ = nfeatures;
    n_classes_ = nclasses;
    return *this;
  }
  template <class I, class O> std::vector<T> predict(const crs_matrix_local<T, I, O>& mat) {
    require(is_fitted, "[logistic_regression] predict is called before fit\n");
    return is_mult ? model_mult.predict(mat) : model_bin.predict(mat);
  }
  template <class I, class O>
  std::vector<T> predict_probability(const crs_matrix_local<T, I, O>& mat, bool use_score = false) {
    require(is_fitted, "[logistic_regression] predict_probability is called before fit\n");
    return is_mult ? model_mult.predict_probability(mat, use_score) : model_bin.predict_probability(mat, use_score);
  }
  template <class I, class O> rowmajor_matrix_local<T> compute_probability_matrix(const crs_matrix_local<T, I, O>& mat) {
    require(is_fitted, "[logistic_regression] compute_probability_matrix is called before fit\n");
    return is_mult ? model_mult.compute_probability_matrix(mat) : model_bin.compute_probability_matrix(mat);
  }
  template <class I, class O> float score(const crs_matrix_local<T, I, O>& mat, const std::vector<T>& label) {
    require(is_fitted, "[logistic_regression] score is called before fit\n");
    return accuracy_score(label, predict(mat));
  }
  std::vector<T> get_intercept() const {
    return is_mult ? model_mult.intercept : std::vector<T>({model_bin.intercept});
  }
  std::vector<T> get_weight() const { return is_mult ? model_mult.weight.val : model_bin.weight; }
  size_t get_num_features() const { return is_mult ? model_mult.get_num_features() : model_bin.get_num_features(); }
  size_t get_num_classes() const { return is_mult ? model_mult.get_num_classes() : model_bin.get_num_classes(); }

  // save / savebinary / load / loadbinary (lines 404-458): <dir>/model and
  // <dir>/type ("binomial" or "multinomial")
  void save(const std::string& dir) {
    detail::make_directory(dir);
    is_mult ? frovedis::save(model_mult, dir + "/model") : frovedis::save(model_bin, dir + "/model");
    std::ofstream((dir + "/type").c_str()) << (is_mult ? "multinomial" : "binomial") << std::endl;
  }
  void savebinary(const std::string& dir) {
    detail::make_directory(dir);
    is_mult ? frovedis::savebinary(model_mult, dir + "/model") : frovedis::savebinary(model_bin, dir + "/model");
    std::ofstream((dir + "/type").c_str()) << (is_mult ? "multinomial" : "binomial") << std::endl;
  }
  logistic_regression& load(const std::string& dir) { return load_impl(dir, false); }
  logistic_regression& loadbinary(const std::string& dir) { return load_impl(dir, true); }

  int max_iter, hist_size;
  double alpha, mbf, tol, reg_param;
  std::string solver, reg_type;
  bool fit_intercept, is_mult, warm_start, is_fitted;
  MatType mat_type;
  size_t n_iter_, n_features_, n_classes_;
  logistic_regression_model<T> model_bin;
  multinomial_logistic_regression_model<T> model_mult;

 private:
  logistic_regression& load_impl(const std::string& dir, bool binary) {
    std::string model_type;
    std::ifstream((dir + "/type").c_str()) >> model_type;
    is_mult = model_type == "multinomial";
    if (is_mult) binary ? frovedis::loadbinary(model_mult, dir + "/model") : frovedis::load(model_mult, dir + "/model");
    else binary ? frovedis::loadbinary(model_bin, dir + "/model") : frovedis::load(model_bin, dir + "/model");
    n_classes_ = get_num_classes();
    n_features_ = get_num_features();
    is_fitted = true;
    return *this;
  }
};

}  // namespace frovedis

#endif  // FROVEDIS_GB300_HPP
