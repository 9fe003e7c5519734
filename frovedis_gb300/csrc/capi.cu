// C ABI (include/fvg.h): argument checks, host<->device staging, and
// dispatch to the builders, products and drivers.  No C++ exception leaves
// this file; every entry point returns an fvg_status and records the
// message in the context.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "fvg_internal.cuh"

namespace fvg {
void lbfgs_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h, const fvg_glm_params* p,
                 double* w_h, double* b_h, i64* n_iter, double* loss_out);
void sgd_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h, const fvg_glm_params* p,
               double* w_h, double* b_h, i64* n_iter, double* loss_out, bool shrink);
void logreg_eval(fvg_ctx* c, fvg_matrix* M, int fmt, int storage, const double* label_h, const double* sw_h,
                 const double* w_h, double b, int icpt, double* grad_h, double* loss_h, int loss_kind, double eps);
void lbfgs_batched_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                         const fvg_glm_params* p, i64 k, const double* lam_h, double* w_h, double* b_h,
                         i64* n_iter_h, double* loss_h);
void lbfgs_multi_train(fvg_ctx* c, const std::vector<fvg_matrix*>& mats, const std::vector<const double*>& labels_h,
                       const std::vector<const double*>& sws_h, const fvg_glm_params* p, i64 k, const double* lam_h,
                       double* w_h, double* b_h, i64* n_iter_h, double* loss_h);
void multinomial_lbfgs_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                             const fvg_glm_params* p, i64 K, double* w_h, i64* n_iter, double* loss_out);
void multinomial_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                       const fvg_glm_params* p, i64 K, double* w_h, double* b_h, i64* n_iter);
void multinomial_probability(fvg_ctx* c, fvg_matrix* M, const double* w_h, const double* b_h, i64 K, int icpt_on,
                             double* prob_h);
void load_text_matrix(fvg_ctx* c, const char* path, int dt, i64 num_col, DevCRS& A);
void load_libsvm_matrix(fvg_ctx* c, const char* path, int dt, int origin, DevCRS& A, std::vector<double>& label);
void load_binary_matrix(fvg_ctx* c, const char* dir, int dt, const char* idx_type, const char* off_type,
                        DevCRS& A);
int crs_blocks_per_sm();
void sigmoid_probability(fvg_ctx* c, double* v, i64 m, double b);
}  // namespace fvg

using namespace fvg;

#define API_BEGIN try {
#define API_END(ctxp)                                                   \
  }                                                                     \
  catch (const fvg::Error& e) {                                         \
    if (ctxp) (ctxp)->last_error = e.msg;                               \
    return e.code;                                                      \
  }                                                                     \
  catch (const std::bad_alloc&) {                                       \
    if (ctxp) (ctxp)->last_error = "host allocation failed";            \
    return FVG_ERR_OUT_OF_MEMORY;                                       \
  }                                                                     \
  catch (const std::exception& e) {                                     \
    if (ctxp) (ctxp)->last_error = e.what();                            \
    return FVG_ERR_INTERNAL;                                            \
  }                                                                     \
  return FVG_OK;

static void need(bool cond, fvg_status code, const char* msg) {
  if (!cond) fail(code, msg);
}

// A matrix handle around a loader that fills M->A.
template <class F>
static fvg_status load_matrix(fvg_ctx* c, fvg_dtype dt, fvg_matrix** out, F&& fill) {
  if (!c || !out) return FVG_ERR_INVALID_ARG;
  *out = nullptr;
  fvg_matrix* M = nullptr;
  try {
    need(dt == FVG_F64 || dt == FVG_F32, FVG_ERR_INVALID_ARG, "files hold FP64 or FP32 values");
    M = new fvg_matrix();
    M->ctx = c;
    M->master = dt;
    fill(M);
    c->matrices.push_back(M);
    *out = M;
    return FVG_OK;
  } catch (const fvg::Error& e) {
    delete M;
    c->last_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    delete M;
    c->last_error = "host allocation failed";
    return FVG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    delete M;
    c->last_error = e.what();
    return FVG_ERR_INTERNAL;
  }
}


extern "C" {

FVG_API fvg_status fvg_ctx_create(int device, fvg_ctx** out) {
  if (!out) return FVG_ERR_INVALID_ARG;
  *out = nullptr;
  fvg_ctx* c = nullptr;
  try {
    c = new fvg_ctx();
    int ndev = 0;
    FVG_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) fail(FVG_ERR_INVALID_ARG, "no such CUDA device");
    c->device = device;
    FVG_CUDA(cudaSetDevice(device));
    FVG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    FVG_CUDA(cudaMalloc(&c->dev_err, 256));
    FVG_CUDA(cudaMemset(c->dev_err, 0, 256));
    FVG_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    c->grid_spmv = c->num_sms * std::max(1, crs_blocks_per_sm());
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;  // keep freed blocks cached in this process
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    prof_create(c);
    df64_init(c);
    *out = c;
    return FVG_OK;
  } catch (const fvg::Error& e) {
    fprintf(stderr, "fvg_ctx_create: %s\n", e.msg.c_str());
    if (c) {
      if (c->stream) cudaStreamDestroy(c->stream);
      delete c;
    }
    return e.code;
  } catch (...) {
    delete c;
    return FVG_ERR_INTERNAL;
  }
}

// Frees every device buffer of a matrix (its host handle stays valid).
static void release_device(fvg_matrix* M) {
  M->A = DevCRS();
  M->AT.reset();
  M->ell.reset();
  M->jds.reset();
  M->tjds.reset();
  M->hyb.reset();
  M->thyb.reset();
}

FVG_API void fvg_ctx_destroy(fvg_ctx* c) {
  if (!c) return;
  cudaStreamSynchronize(c->stream);
  for (fvg_matrix* M : c->matrices) {  // orphan the matrices still alive
    release_device(M);
    M->ctx = nullptr;
  }
  c->matrices.clear();
  cudaStreamSynchronize(c->stream);
  if (c->dev_err) cudaFree(c->dev_err);
  prof_destroy(c);
  cudaStreamDestroy(c->stream);
  delete c;
}

FVG_API const char* fvg_ctx_last_error(const fvg_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

FVG_API void* fvg_ctx_stream(fvg_ctx* c) { return c ? (void*)c->stream : nullptr; }

FVG_API fvg_status fvg_ctx_synchronize(fvg_ctx* c) {
  if (!c) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

static const char* kProfNames[P_NKEYS] = {"spmv_crs", "pass1", "pass2", "finalize", "lbfgs_vec",
                                          "transpose", "spmv_ell", "spmv_jds", "spmv_hyb", "spmm",
                                          "pass1_f32", "pass2_f32", "batch_pass1", "batch_pass2",
                                          "panel_build", "head_build", "schedule"};

FVG_API fvg_status fvg_ctx_set_profiling(fvg_ctx* c, int enable) {
  if (!c) return FVG_ERR_INVALID_ARG;
  c->profiling = enable != 0;
  return FVG_OK;
}

FVG_API fvg_status fvg_ctx_get_profile(fvg_ctx* c, const char* name, double* total_ms, int64_t* launches) {
  if (!c || !name || !total_ms || !launches) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  if (!strcmp(name, "batch_evals")) {  // counters, not timings
    *total_ms = (double)c->batch_model_evals;
    *launches = c->batch_evals;
    return FVG_OK;
  }
  int key = -1;
  for (int k = 0; k < P_NKEYS; k++)
    if (!strcmp(name, kProfNames[k])) key = k;
  need(key >= 0, FVG_ERR_INVALID_ARG, "unknown profile name");
  prof_collect(c, key, total_ms, launches);
  API_END(c)
}

FVG_API fvg_status fvg_ctx_reset_profile(fvg_ctx* c) {
  if (!c) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  prof_reset(c);
  API_END(c)
}

FVG_API int64_t fvg_ctx_kernel_launches(fvg_ctx* c) { return c ? c->launches : -1; }

FVG_API fvg_status fvg_ctx_set_wait_limit(fvg_ctx* c, int64_t polls) {
  if (!c) return FVG_ERR_INVALID_ARG;
  c->wait_limit = polls < 0 ? -1 : std::min<int64_t>(polls, 0xffffffffll);
  return FVG_OK;
}

FVG_API void fvg_debug_inject_alloc_failure(int64_t after) { inject_alloc_failure(after < 0 ? -1 : after); }

// ------------------------------------------------------------------ matrix
FVG_API fvg_status fvg_matrix_create_crs(fvg_ctx* c, int64_t num_row, int64_t num_col, const int32_t* off,
                                         const int32_t* idx, const void* val, fvg_dtype val_dtype, int on_device,
                                         fvg_matrix** out) {
  if (!c || !out) return FVG_ERR_INVALID_ARG;
  *out = nullptr;
  fvg_matrix* M = nullptr;
  API_BEGIN
  need(val_dtype >= FVG_F64 && val_dtype <= FVG_BF16, FVG_ERR_INVALID_ARG, "unknown value dtype");
  need(num_row >= 0 && num_col >= 0 && num_row < (1ll << 31) && num_col < (1ll << 31), FVG_ERR_INVALID_ARG,
       "matrix dimensions must be in [0, 2^31)");
  M = new fvg_matrix();
  M->ctx = c;
  M->master = val_dtype;
  crs_upload(c, M->A, num_row, num_col, off, idx, val, val_dtype, on_device != 0);
  c->matrices.push_back(M);
  *out = M;
  M = nullptr;
  }
  catch (const fvg::Error& e) {
    delete M;
    c->last_error = e.msg;
    return e.code;
  }
  catch (...) {
    delete M;
    c->last_error = "internal error";
    return FVG_ERR_INTERNAL;
  }
  return FVG_OK;
}

FVG_API void fvg_matrix_destroy(fvg_matrix* M) {
  if (!M) return;
  fvg_ctx* c = M->ctx;
  if (!c) {  // its context is gone; device memory was released with it
    delete M;
    return;
  }
  auto& v = c->matrices;
  v.erase(std::remove(v.begin(), v.end(), M), v.end());
  delete M;  // buffers are freed stream-ordered
  cudaStreamSynchronize(c->stream);
}

static void own(fvg_ctx* c, fvg_matrix* M) {
  if (M->ctx != c) fail(FVG_ERR_INVALID_ARG, "the matrix belongs to another (or a destroyed) context");
}

FVG_API fvg_status fvg_matrix_info(const fvg_matrix* M, int64_t* m, int64_t* n, int64_t* nnz) {
  if (!M) return FVG_ERR_INVALID_ARG;
  if (m) *m = M->A.m;
  if (n) *n = M->A.n;
  if (nnz) *nnz = M->A.nnz;
  return FVG_OK;
}

static void ensure_transpose(fvg_ctx* c, fvg_matrix* M) {
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
}

static void prepare(fvg_ctx* c, fvg_matrix* M, int fmt, bool trans) {
  if (fmt == FVG_CRS) {
    crs_sched(c, M->A, kWarpTile);  // the CRS kernel's work schedule
    if (trans) {
      ensure_transpose(c, M);
      crs_sched(c, *M->AT, kWarpTile);
    }
  } else if (fmt == FVG_ELL) {
    if (!M->ell) {
      M->ell.reset(new DevELL());
      ell_build(c, M->A, *M->ell, M->master);
    }
    if (trans) ensure_transpose(c, M);
  } else if (fmt == FVG_JDS) {
    if (!M->jds) {
      M->jds.reset(new DevJDS());
      jds_build(c, M->A, *M->jds, M->master);
    }
    if (trans && !M->tjds) {
      ensure_transpose(c, M);
      M->tjds.reset(new DevJDS());
      jds_build(c, *M->AT, *M->tjds, M->master);
    }
  } else if (fmt == FVG_HYBRID) {
    if (!M->hyb) {
      M->hyb.reset(new DevHYB());
      hyb_build(c, M->A, *M->hyb, M->master, 256);
    }
    if (trans && !M->thyb) {
      ensure_transpose(c, M);
      M->thyb.reset(new DevHYB());
      hyb_build(c, *M->AT, *M->thyb, M->master, 256);
    }
  } else {
    fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  }
}

FVG_API fvg_status fvg_matrix_prepare(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, int with_transpose) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  prepare(c, M, fmt, with_transpose != 0);
  if (with_transpose && M->A.lo.p && M->AT) crs_ensure_split(c, *M->AT, M->master);
  // a matrix that already holds FP32 / BF16 values gets its row-panel
  // backward layout and its forward head now rather than at the first product
  if (with_transpose && (fmt == FVG_CRS || fmt == FVG_ELL) && (M->A.val[FVG_F32].p || M->A.val[FVG_BF16].p)) {
    DevPanels* pt = panels_for(c, M);
    DevPanels* hd = fmt == FVG_CRS ? head_for(c, M) : nullptr;
    for (int dt : {FVG_F32, FVG_BF16})
      if (M->A.val[dt].p) {
        if (pt) panel_ensure_plane(c, *pt, dt);
        if (hd) head_ensure_plane(c, *hd, dt);
      }
  }
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

FVG_API fvg_status fvg_matrix_set_panels(fvg_ctx* c, fvg_matrix* M, int64_t rows, double min_per_panel) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(rows < 0 || rows == 0 || rows % 4 == 0, FVG_ERR_INVALID_ARG, "panel rows must be a multiple of 4");
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  M->pan.reset();
  M->pan_tried = false;
  M->panel_rows = rows < 0 ? -1 : rows;
  M->panel_min = min_per_panel;
  API_END(c)
}

FVG_API fvg_status fvg_matrix_autotune(fvg_ctx* c, fvg_matrix* M, fvg_dtype storage, const double* label,
                                       int32_t reps, fvg_tune_choice* best, fvg_tune_choice* tried,
                                       int64_t max_tried, int64_t* n_tried) {
  if (!c || !M || !best) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  std::vector<fvg_tune_choice> all;
  autotune(c, M, storage, label, reps, all, *best);
  if (n_tried) *n_tried = (int64_t)all.size();
  for (size_t i = 0; tried && i < all.size() && (int64_t)i < max_tried; i++) tried[i] = all[i];
  API_END(c)
}

FVG_API fvg_status fvg_matrix_set_head(fvg_ctx* c, fvg_matrix* M, int64_t columns) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  M->head.reset();
  M->head_tried = false;
  M->head_cols = columns < 0 ? -1 : columns;
  API_END(c)
}

FVG_API fvg_status fvg_matrix_head_info(fvg_ctx* c, fvg_matrix* M, int64_t* info) {
  if (!c || !M || !info) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  DevPanels* hd = head_for(c, M);
  info[0] = hd ? hd->rows : 0;
  info[1] = hd ? hd->E : 0;
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

FVG_API fvg_status fvg_matrix_panel_info(fvg_ctx* c, fvg_matrix* M, int64_t* info) {
  if (!c || !M || !info) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  DevPanels* pt = panels_for(c, M);
  info[0] = pt ? pt->rows : 0;
  info[1] = pt ? pt->npanels : 0;
  info[2] = pt ? pt->nhot : 0;
  info[3] = pt ? pt->E : 0;
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

static void ensure_plane_all(fvg_ctx* c, fvg_matrix* M, int dt) {
  if (dt == FVG_SPLIT) {  // the CRS layouts only (the products run on them)
    crs_ensure_split(c, M->A, M->master);
    if (M->AT) crs_ensure_split(c, *M->AT, M->master);
    return;
  }
  crs_ensure_plane(c, M->A, dt, M->master);
  if (M->AT) crs_ensure_plane(c, *M->AT, dt, M->master);
  if (M->ell) ensure_plane_generic(c, M->ell->val, M->ell->m * M->ell->width, dt, M->master);
  for (DevJDS* j : {M->jds.get(), M->tjds.get()})
    if (j) ensure_plane_generic(c, j->val, j->nnz, dt, M->master);
  for (DevHYB* h : {M->hyb.get(), M->thyb.get()})
    if (h) {
      ensure_plane_generic(c, h->jds.val, h->jds.nnz, dt, M->master);
      crs_ensure_plane(c, h->crs, dt, M->master);
    }
}

FVG_API fvg_status fvg_matrix_add_storage(fvg_ctx* c, fvg_matrix* M, fvg_dtype storage) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(storage >= FVG_F64 && storage <= FVG_SPLIT, FVG_ERR_INVALID_ARG, "unknown storage dtype");
  ensure_plane_all(c, M, storage);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

static int64_t crs_bytes(const DevCRS& a) {
  int64_t b = (int64_t)a.off.bytes + (int64_t)a.idx.bytes;
  for (auto& v : a.val) b += (int64_t)v.bytes;
  b += (int64_t)a.lo.bytes;
  for (auto& s : a.sched)
    if (s) b += (int64_t)(s->items.bytes + s->long_rows.bytes + s->long_piece0.bytes);
  return b;
}
static int64_t jds_bytes(const DevJDS& j) {
  int64_t b = (int64_t)(j.perm.bytes + j.off.bytes + j.idx.bytes);
  for (auto& v : j.val) b += (int64_t)v.bytes;
  return b;
}

FVG_API int64_t fvg_matrix_device_bytes(const fvg_matrix* M) {
  if (!M) return 0;
  int64_t b = crs_bytes(M->A);
  if (M->AT) b += crs_bytes(*M->AT);
  if (M->ell) {
    b += (int64_t)M->ell->idx.bytes;
    for (auto& v : M->ell->val) b += (int64_t)v.bytes;
  }
  if (M->jds) b += jds_bytes(*M->jds);
  if (M->tjds) b += jds_bytes(*M->tjds);
  for (const DevHYB* h : {M->hyb.get(), M->thyb.get()})
    if (h) b += jds_bytes(h->jds) + crs_bytes(h->crs);
  for (const DevPanels* p : {M->pan.get(), M->head.get()}) {
    if (!p) continue;
    b += crs_bytes(p->cold);
    for (const DBuf* d : {&p->hot_cols, &p->poff, &p->prow, &p->items, &p->pitem0, &p->long_rows, &p->plong0,
                          &p->long_piece0, &p->ypan, &p->partials})
      b += (int64_t)d->bytes;
    for (auto& v : p->val) b += (int64_t)v.bytes;
  }
  return b;
}

// value plane as FP64 on the host
static void download_values(fvg_ctx* c, const DBuf* planes, int master, int64_t n, double* out) {
  if (!out || n <= 0) return;
  if (master == FVG_F64) {
    FVG_CUDA(cudaMemcpyAsync(out, planes[FVG_F64].p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  } else {
    DBuf tmp;
    tmp.alloc(sizeof(double) * n, c->stream);
    convert_values(c, planes[master].p, master, tmp.p, FVG_F64, n);
    FVG_CUDA(cudaMemcpyAsync(out, tmp.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
  }
}

FVG_API fvg_status fvg_matrix_get_transpose(fvg_ctx* c, fvg_matrix* M, int32_t* toff, int32_t* tidx,
                                            double* tval) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  ensure_transpose(c, M);
  const DevCRS& t = *M->AT;
  if (toff) FVG_CUDA(cudaMemcpyAsync(toff, t.off.p, sizeof(int32_t) * (t.m + 1), cudaMemcpyDeviceToHost, c->stream));
  if (tidx && t.nnz)
    FVG_CUDA(cudaMemcpyAsync(tidx, t.idx.p, sizeof(int32_t) * t.nnz, cudaMemcpyDeviceToHost, c->stream));
  download_values(c, t.val, M->master, t.nnz, tval);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

FVG_API fvg_status fvg_matrix_get_crs(fvg_ctx* c, fvg_matrix* M, int32_t* off, int32_t* idx, double* val) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  const DevCRS& a = M->A;
  if (off) FVG_CUDA(cudaMemcpyAsync(off, a.off.p, sizeof(int32_t) * (a.m + 1), cudaMemcpyDeviceToHost, c->stream));
  if (idx && a.nnz)
    FVG_CUDA(cudaMemcpyAsync(idx, a.idx.p, sizeof(int32_t) * a.nnz, cudaMemcpyDeviceToHost, c->stream));
  download_values(c, a.val, M->master, a.nnz, val);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

FVG_API fvg_status fvg_matrix_load_text(fvg_ctx* c, const char* path, fvg_dtype val_dtype, int64_t num_col,
                                        fvg_matrix** out) {
  if (!path) return FVG_ERR_INVALID_ARG;
  return load_matrix(c, val_dtype, out, [&](fvg_matrix* M) { load_text_matrix(c, path, val_dtype, num_col, M->A); });
}

FVG_API fvg_status fvg_matrix_load_libsvm(fvg_ctx* c, const char* path, fvg_dtype val_dtype, int index_origin,
                                          fvg_matrix** out) {
  if (!path || index_origin < 0 || index_origin > 2) return FVG_ERR_INVALID_ARG;
  return load_matrix(c, val_dtype, out, [&](fvg_matrix* M) {
    load_libsvm_matrix(c, path, val_dtype, index_origin, M->A, M->labels);
    M->has_labels = true;
  });
}

FVG_API fvg_status fvg_matrix_get_labels(const fvg_matrix* M, double* labels) {
  if (!M || !labels || !M->has_labels) return FVG_ERR_INVALID_ARG;
  std::copy(M->labels.begin(), M->labels.end(), labels);
  return FVG_OK;
}

FVG_API fvg_status fvg_matrix_load_binary(fvg_ctx* c, const char* dir, fvg_dtype val_dtype, const char* idx_type,
                                          const char* off_type, fvg_matrix** out) {
  if (!dir) return FVG_ERR_INVALID_ARG;
  const char* it = idx_type ? idx_type : "uint64_t";
  const char* ot = off_type ? off_type : "uint64_t";
  return load_matrix(c, val_dtype, out, [&](fvg_matrix* M) { load_binary_matrix(c, dir, val_dtype, it, ot, M->A); });
}

FVG_API fvg_status fvg_matrix_get_ell(fvg_ctx* c, fvg_matrix* M, int64_t* width, int32_t* eidx, double* eval) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  prepare(c, M, FVG_ELL, false);
  const DevELL& e = *M->ell;
  if (width) *width = e.width;
  int64_t cells = e.m * e.width;
  if (eidx && cells)
    FVG_CUDA(cudaMemcpyAsync(eidx, e.idx.p, sizeof(int32_t) * cells, cudaMemcpyDeviceToHost, c->stream));
  download_values(c, e.val, M->master, cells, eval);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

static void get_jds(fvg_ctx* c, const DevJDS& j, int master, int32_t* perm, int64_t* joff, int32_t* jidx,
                    double* jval) {
  if (perm && !j.empty_perm && j.m)
    FVG_CUDA(cudaMemcpyAsync(perm, j.perm.p, sizeof(int32_t) * j.m, cudaMemcpyDeviceToHost, c->stream));
  if (joff) FVG_CUDA(cudaMemcpyAsync(joff, j.off.p, sizeof(int64_t) * (j.ndiag + 1), cudaMemcpyDeviceToHost, c->stream));
  if (jidx && j.nnz) FVG_CUDA(cudaMemcpyAsync(jidx, j.idx.p, sizeof(int32_t) * j.nnz, cudaMemcpyDeviceToHost, c->stream));
  download_values(c, j.val, master, j.nnz, jval);
}

FVG_API fvg_status fvg_matrix_get_jds(fvg_ctx* c, fvg_matrix* M, int64_t* ndiag, int32_t* perm, int64_t* joff,
                                      int32_t* jidx, double* jval) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  prepare(c, M, FVG_JDS, false);
  if (ndiag) *ndiag = M->jds->ndiag;
  get_jds(c, *M->jds, M->master, perm, joff, jidx, jval);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

FVG_API fvg_status fvg_matrix_get_hybrid(fvg_ctx* c, fvg_matrix* M, int64_t* info, int32_t* perm, int64_t* joff,
                                         int32_t* jidx, double* jval, int64_t* coff, int32_t* cidx,
                                         double* cval) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  prepare(c, M, FVG_HYBRID, false);
  const DevHYB& h = *M->hyb;
  if (info) {
    info[0] = h.jds.ndiag;
    info[1] = h.crs.m;
    info[2] = h.crs.nnz;
    info[3] = h.jds.nnz;
    info[4] = h.jds.empty_perm ? 0 : h.m;
  }
  get_jds(c, h.jds, M->master, perm, joff, jidx, jval);
  if (coff) {
    std::vector<int32_t> o(h.crs.m + 1);
    FVG_CUDA(cudaMemcpyAsync(o.data(), h.crs.off.p, sizeof(int32_t) * (h.crs.m + 1), cudaMemcpyDeviceToHost,
                             c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
    for (int64_t i = 0; i <= h.crs.m; i++) coff[i] = o[i];
  }
  if (cidx && h.crs.nnz)
    FVG_CUDA(cudaMemcpyAsync(cidx, h.crs.idx.p, sizeof(int32_t) * h.crs.nnz, cudaMemcpyDeviceToHost, c->stream));
  download_values(c, h.crs.val, M->master, h.crs.nnz, cval);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

// --------------------------------------------------------------- products
// Stages x (len nx) / y (len ny) on the device in the kernel's vector type.
struct VecStage {
  DBuf xb, yb, xconv, yconv;
  const void* dx = nullptr;
  void* dy = nullptr;
  int kdt = FVG_F64;  // kernel vector dtype
};

static void stage_in(fvg_ctx* c, VecStage& v, const void* x, int64_t nx, int vec_dt, int storage, bool on_dev) {
  v.kdt = (storage == FVG_F64) ? FVG_F64 : FVG_F32;
  const void* src = x;
  if (!on_dev) {
    v.xb.alloc((size_t)dtype_size(vec_dt) * std::max<int64_t>(nx, 1), c->stream);
    if (nx) FVG_CUDA(cudaMemcpyAsync(v.xb.p, x, (size_t)dtype_size(vec_dt) * nx, cudaMemcpyHostToDevice, c->stream));
    src = v.xb.p;
  }
  if (vec_dt != v.kdt) {
    v.xconv.alloc((size_t)dtype_size(v.kdt) * std::max<int64_t>(nx, 1), c->stream);
    convert_values(c, src, vec_dt, v.xconv.p, v.kdt, nx);
    src = v.xconv.p;
  }
  v.dx = src;
}

static void stage_out_alloc(fvg_ctx* c, VecStage& v, void* y, int64_t ny, int vec_dt, bool on_dev, int out_dt) {
  // kernels write out_dt; y wants vec_dt
  if (on_dev && vec_dt == out_dt) {
    v.dy = y;
    return;
  }
  v.yb.alloc((size_t)dtype_size(out_dt) * std::max<int64_t>(ny, 1), c->stream);
  v.dy = v.yb.p;
}

static void stage_out_finish(fvg_ctx* c, VecStage& v, void* y, int64_t ny, int vec_dt, bool on_dev, int out_dt) {
  if (v.dy == y) return;
  const void* src = v.dy;
  if (vec_dt != out_dt) {
    v.yconv.alloc((size_t)dtype_size(vec_dt) * std::max<int64_t>(ny, 1), c->stream);
    convert_values(c, src, out_dt, v.yconv.p, vec_dt, ny);
    src = v.yconv.p;
  }
  if (ny)
    FVG_CUDA(cudaMemcpyAsync(y, src, (size_t)dtype_size(vec_dt) * ny,
                             on_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
}

static void check_vec_args(int storage, int vec_dt) {
  need(storage >= FVG_F64 && storage <= FVG_SPLIT, FVG_ERR_INVALID_ARG, "unknown storage dtype");
  need(vec_dt == FVG_F64 || vec_dt == FVG_F32, FVG_ERR_INVALID_ARG, "vectors must be FP64 or FP32");
  need(!(storage == FVG_F64 && vec_dt != FVG_F64), FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
  need(!(storage == FVG_SPLIT && vec_dt != FVG_F64), FVG_ERR_INVALID_ARG, "split storage needs FP64 vectors");
}

// split storage: y = A x or A^T x over the CRS layouts in df64 arithmetic
static void run_product_split(fvg_ctx* c, fvg_matrix* M, int fmt, const void* x, void* y, bool trans, bool on_dev) {
  need(fmt == FVG_CRS, FVG_ERR_UNSUPPORTED, "split storage runs on the CRS format");
  prepare(c, M, fmt, trans);
  ensure_plane_all(c, M, FVG_SPLIT);
  const int64_t nx = trans ? M->A.m : M->A.n, ny = trans ? M->A.n : M->A.m;
  DBuf xb, x2, yb;
  const double* dx = (const double*)x;
  if (!on_dev) {
    xb.alloc(sizeof(double) * std::max<int64_t>(nx, 1), c->stream);
    if (nx) FVG_CUDA(cudaMemcpyAsync(xb.p, x, sizeof(double) * nx, cudaMemcpyHostToDevice, c->stream));
    dx = xb.as<double>();
  }
  x2.alloc(sizeof(float2) * std::max<int64_t>(nx, 1), c->stream);
  split_vector(c, dx, x2.p, nx);
  double* dy = (double*)y;
  if (!on_dev) {
    yb.alloc(sizeof(double) * std::max<int64_t>(ny, 1), c->stream);
    dy = yb.as<double>();
  }
  DevPanels* pt = trans ? panels_for(c, M) : nullptr;
  if (pt) {
    ProfScope ps(c, P_SPMV_CRS);
    panel_trans_mv_split(c, *pt, x2.p, dy, nullptr);
  } else {
    crs_pass_split(c, trans ? *M->AT : M->A, x2.p, false, dy, nullptr, P_SPMV_CRS);
  }
  if (!on_dev && ny)
    FVG_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * ny, cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  check_device_error(c);
}

static void run_product(fvg_ctx* c, fvg_matrix* M, int fmt, int storage, int vec_dt, const void* x, void* y,
                        bool trans, bool on_dev) {
  check_vec_args(storage, vec_dt);
  need(fmt >= 0 && fmt <= 3, FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  if (storage == FVG_SPLIT) {
    run_product_split(c, M, fmt, x, y, trans, on_dev);
    return;
  }
  prepare(c, M, fmt, trans);
  ensure_plane_all(c, M, storage);
  const int64_t nx = trans ? M->A.m : M->A.n, ny = trans ? M->A.n : M->A.m;
  VecStage v;
  stage_in(c, v, x, nx, vec_dt, storage, on_dev);
  // FP32-vector kernels can write FP64 directly
  const int out_dt = (v.kdt == FVG_F64) ? FVG_F64 : vec_dt;
  stage_out_alloc(c, v, y, ny, vec_dt, on_dev, out_dt);
  if (!trans) {
    if (fmt == FVG_CRS) crs_pass(c, M->A, storage, v.kdt, v.dx, out_dt, v.dy, EPI_STORE, nullptr, nullptr, P_SPMV_CRS);
    else if (fmt == FVG_ELL) ell_spmv(c, *M->ell, storage, v.kdt, v.dx, out_dt, v.dy);
    else if (fmt == FVG_JDS) jds_spmv(c, *M->jds, storage, v.kdt, v.dx, out_dt, v.dy, false);
    else hyb_spmv(c, *M->hyb, storage, v.kdt, v.dx, out_dt, v.dy);
  } else {
    DevPanels* pt = (storage != FVG_F64 && (fmt == FVG_CRS || fmt == FVG_ELL)) ? panels_for(c, M) : nullptr;
    if (pt)
      panel_trans_mv(c, *pt, storage, (const float*)v.dx, out_dt, v.dy, nullptr, P_SPMV_CRS);
    else if (fmt == FVG_CRS || fmt == FVG_ELL)
      crs_pass(c, *M->AT, storage, v.kdt, v.dx, out_dt, v.dy, EPI_STORE, nullptr, nullptr, P_SPMV_CRS);
    else if (fmt == FVG_JDS) jds_spmv(c, *M->tjds, storage, v.kdt, v.dx, out_dt, v.dy, false);
    else hyb_spmv(c, *M->thyb, storage, v.kdt, v.dx, out_dt, v.dy);
  }
  stage_out_finish(c, v, y, ny, vec_dt, on_dev, out_dt);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  check_device_error(c);
}

FVG_API fvg_status fvg_spmv(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, fvg_dtype storage, fvg_dtype vec_dtype,
                            const void* x, void* y, int on_device) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need((x && y) || M->A.m == 0 || M->A.n == 0, FVG_ERR_INVALID_ARG, "null vector");
  run_product(c, M, fmt, storage, vec_dtype, x, y, false, on_device != 0);
  API_END(c)
}

FVG_API fvg_status fvg_trans_mv(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, fvg_dtype storage, fvg_dtype vec_dtype,
                                const void* x, void* y, int on_device) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need((x && y) || M->A.m == 0 || M->A.n == 0, FVG_ERR_INVALID_ARG, "null vector");
  run_product(c, M, fmt, storage, vec_dtype, x, y, true, on_device != 0);
  API_END(c)
}

FVG_API fvg_status fvg_spmm(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, fvg_dtype storage, fvg_dtype vec_dtype,
                            const void* X, int64_t k, void* Y, int on_device) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  check_vec_args(storage, vec_dtype);
  need(storage != FVG_SPLIT, FVG_ERR_UNSUPPORTED, "split storage is not offered by the SpMM");
  need(k >= 0, FVG_ERR_INVALID_ARG, "negative number of columns");
  need(fmt >= 0 && fmt <= 3, FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  ensure_plane_all(c, M, storage);
  const int64_t nx = M->A.n * k, ny = M->A.m * k;
  VecStage v;
  stage_in(c, v, X, nx, vec_dtype, storage, on_device != 0);
  stage_out_alloc(c, v, Y, ny, vec_dtype, on_device != 0, v.kdt);
  crs_spmm(c, M->A, storage, v.kdt, v.dx, k, v.dy);
  stage_out_finish(c, v, Y, ny, vec_dtype, on_device != 0, v.kdt);
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  API_END(c)
}

// --------------------------------------------------------------- training
FVG_API void fvg_glm_params_default(fvg_glm_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->num_iteration = 1000;
  p->alpha = 0.01;
  p->hist_size = 10;
  p->reg_param = 0.01;
  p->reg_type = FVG_REG_ZERO;
  p->intercept = 0;
  p->convergence_tol = 0.001;
  p->mat_type = FVG_CRS;
  p->mini_batch_fraction = 1.0;
  p->num_partitions = 1;
  p->storage = FVG_F64;
  p->refine = 1;
  p->refine_stall = 0.97;
  p->l2_no_eta = 0;
  p->use_graph = 1;
  p->trace = nullptr;
  p->row_splits = nullptr;
  p->loss = FVG_LOSS_LOGISTIC;
  p->epsilon = 0.0;
}

// The fvg_logreg_* entry points train logistic regression whatever
// params->loss holds.
static fvg_glm_params logistic_of(const fvg_glm_params* p) {
  fvg_glm_params q = *p;
  q.loss = FVG_LOSS_LOGISTIC;
  return q;
}

FVG_API fvg_status fvg_logreg_lbfgs(fvg_ctx* c, fvg_matrix* M, const double* label, const double* sample_weight,
                                    const fvg_glm_params* p, double* weight, double* intercept, int64_t* n_iter,
                                    double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(p != nullptr, FVG_ERR_INVALID_ARG, "null params");
  const fvg_glm_params q = logistic_of(p);
  lbfgs_train(c, M, label, sample_weight, &q, weight, intercept, n_iter, final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_glm_lbfgs(fvg_ctx* c, fvg_matrix* M, const double* label, const double* sample_weight,
                                 const fvg_glm_params* p, double* weight, double* intercept, int64_t* n_iter,
                                 double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  lbfgs_train(c, M, label, sample_weight, p, weight, intercept, n_iter, final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_logreg_lbfgs_batched(fvg_ctx* c, fvg_matrix* M, const double* label,
                                            const double* sample_weight, const fvg_glm_params* p, int64_t k,
                                            const double* reg_params, double* weight, double* intercept,
                                            int64_t* n_iter, double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss || !reg_params) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(p != nullptr, FVG_ERR_INVALID_ARG, "null params");
  const fvg_glm_params q = logistic_of(p);
  lbfgs_batched_train(c, M, label, sample_weight, &q, k, reg_params, weight, intercept, n_iter, final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_glm_lbfgs_batched(fvg_ctx* c, fvg_matrix* M, const double* label,
                                         const double* sample_weight, const fvg_glm_params* p, int64_t k,
                                         const double* reg_params, double* weight, double* intercept,
                                         int64_t* n_iter, double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss || !reg_params) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  lbfgs_batched_train(c, M, label, sample_weight, p, k, reg_params, weight, intercept, n_iter, final_loss);
  check_device_error(c);
  API_END(c)
}

static void multi_call(fvg_ctx* c, int64_t nd, fvg_matrix* const* mats, const double* const* labels,
                       const double* const* sws, const fvg_glm_params* p, int64_t k, const double* reg_params,
                       double* weight, double* intercept, int64_t* n_iter, double* final_loss) {
  need(nd >= 1 && nd <= 65535, FVG_ERR_INVALID_ARG, "number of datasets must be in [1, 65535]");
  need(mats != nullptr && labels != nullptr, FVG_ERR_INVALID_ARG, "null dataset arrays");
  std::vector<fvg_matrix*> ms((size_t)nd);
  std::vector<const double*> ls((size_t)nd), ws((size_t)nd, nullptr);
  for (int64_t d = 0; d < nd; d++) {
    need(mats[d] != nullptr, FVG_ERR_INVALID_ARG, "null matrix");
    own(c, mats[d]);
    ms[(size_t)d] = mats[d];
    ls[(size_t)d] = labels[d];
    if (sws) ws[(size_t)d] = sws[d];
  }
  lbfgs_multi_train(c, ms, ls, ws, p, k, reg_params, weight, intercept, n_iter, final_loss);
}

FVG_API fvg_status fvg_logreg_lbfgs_multi(fvg_ctx* c, int64_t num_datasets, fvg_matrix* const* mats,
                                          const double* const* labels, const double* const* sample_weights,
                                          const fvg_glm_params* p, int64_t k, const double* reg_params,
                                          double* weight, double* intercept, int64_t* n_iter, double* final_loss) {
  if (!c || !weight || !intercept || !n_iter || !final_loss || !reg_params) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  need(p != nullptr, FVG_ERR_INVALID_ARG, "null params");
  const fvg_glm_params q = logistic_of(p);
  multi_call(c, num_datasets, mats, labels, sample_weights, &q, k, reg_params, weight, intercept, n_iter,
             final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_glm_lbfgs_multi(fvg_ctx* c, int64_t num_datasets, fvg_matrix* const* mats,
                                       const double* const* labels, const double* const* sample_weights,
                                       const fvg_glm_params* p, int64_t k, const double* reg_params, double* weight,
                                       double* intercept, int64_t* n_iter, double* final_loss) {
  if (!c || !weight || !intercept || !n_iter || !final_loss || !reg_params) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  multi_call(c, num_datasets, mats, labels, sample_weights, p, k, reg_params, weight, intercept, n_iter,
             final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_multinomial_train(fvg_ctx* c, fvg_matrix* M, const double* label,
                                         const double* sample_weight, const fvg_glm_params* p, int64_t nclasses,
                                         double* weight, double* intercept, int64_t* n_iter) {
  if (!c || !M || !weight || !intercept || !n_iter) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  multinomial_train(c, M, label, sample_weight, p, nclasses, weight, intercept, n_iter);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_multinomial_lbfgs(fvg_ctx* c, fvg_matrix* M, const double* label,
                                         const double* sample_weight, const fvg_glm_params* p, int64_t nclasses,
                                         double* weight, int64_t* n_iter, double* final_loss) {
  if (!c || !M || !weight || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  multinomial_lbfgs_train(c, M, label, sample_weight, p, nclasses, weight, n_iter, final_loss);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_multinomial_probability(fvg_ctx* c, fvg_matrix* M, const double* weight,
                                               const double* intercept, int64_t nclasses, int intercept_on,
                                               double* prob) {
  if (!c || !M || !weight || !intercept || !prob) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  multinomial_probability(c, M, weight, intercept, nclasses, intercept_on, prob);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_logreg_sgd(fvg_ctx* c, fvg_matrix* M, const double* label, const double* sample_weight,
                                  const fvg_glm_params* p, double* weight, double* intercept, int64_t* n_iter,
                                  double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(p != nullptr, FVG_ERR_INVALID_ARG, "null params");
  const fvg_glm_params q = logistic_of(p);
  sgd_train(c, M, label, sample_weight, &q, weight, intercept, n_iter, final_loss, false);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_logreg_shrink_sgd(fvg_ctx* c, fvg_matrix* M, const double* label,
                                         const double* sample_weight, const fvg_glm_params* p, double* weight,
                                         double* intercept, int64_t* n_iter, double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(p != nullptr, FVG_ERR_INVALID_ARG, "null params");
  const fvg_glm_params q = logistic_of(p);
  sgd_train(c, M, label, sample_weight, &q, weight, intercept, n_iter, final_loss, true);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_glm_sgd(fvg_ctx* c, fvg_matrix* M, const double* label, const double* sample_weight,
                               const fvg_glm_params* p, double* weight, double* intercept, int64_t* n_iter,
                               double* final_loss) {
  if (!c || !M || !weight || !intercept || !n_iter || !final_loss) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  sgd_train(c, M, label, sample_weight, p, weight, intercept, n_iter, final_loss, false);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_logreg_eval(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, fvg_dtype storage,
                                   const double* label, const double* sample_weight, const double* weight,
                                   double intercept, int intercept_on, double* grad, double* loss) {
  if (!c || !M || !grad || !loss || !weight) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(storage >= FVG_F64 && storage <= FVG_SPLIT, FVG_ERR_INVALID_ARG, "unknown storage dtype");
  logreg_eval(c, M, fmt, storage, label, sample_weight, weight, intercept, intercept_on, grad, loss,
              FVG_LOSS_LOGISTIC, 0.0);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_glm_eval(fvg_ctx* c, fvg_matrix* M, fvg_format fmt, fvg_dtype storage, int32_t loss,
                                double epsilon, const double* label, const double* sample_weight,
                                const double* weight, double intercept, int intercept_on, double* grad,
                                double* loss_out) {
  if (!c || !M || !grad || !loss_out || !weight) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(storage >= FVG_F64 && storage <= FVG_SPLIT, FVG_ERR_INVALID_ARG, "unknown storage dtype");
  logreg_eval(c, M, fmt, storage, label, sample_weight, weight, intercept, intercept_on, grad, loss_out, loss,
              epsilon);
  check_device_error(c);
  API_END(c)
}

FVG_API fvg_status fvg_logreg_predict_probability(fvg_ctx* c, fvg_matrix* M, const double* weight,
                                                  double intercept, double* prob) {
  if (!c || !M || !weight || !prob) return FVG_ERR_INVALID_ARG;
  API_BEGIN
  own(c, M);
  need(M->master == FVG_F64, FVG_ERR_INVALID_ARG, "predict_probability needs FP64 values");
  DBuf w, y;
  w.alloc(sizeof(double) * std::max<int64_t>(M->A.n, 1), c->stream);
  y.alloc(sizeof(double) * std::max<int64_t>(M->A.m, 1), c->stream);
  if (M->A.n)
    FVG_CUDA(cudaMemcpyAsync(w.p, weight, sizeof(double) * M->A.n, cudaMemcpyHostToDevice, c->stream));
  crs_pass(c, M->A, FVG_F64, FVG_F64, w.p, FVG_F64, y.p, EPI_STORE, nullptr, nullptr, P_SPMV_CRS);
  sigmoid_probability(c, y.as<double>(), M->A.m, intercept);
  if (M->A.m) FVG_CUDA(cudaMemcpyAsync(prob, y.p, sizeof(double) * M->A.m, cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  check_device_error(c);
  API_END(c)
}

}  // extern "C"
