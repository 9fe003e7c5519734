// CPU ORACLE — test infrastructure only (see oracle.cpp).  C entry points
// used by the Python tests through ctypes.  Index arrays are int32, row
// offsets int32 on input (the layout the CUDA path uses), int64 where the
// reference's JDS offsets can exceed the input's.  Trainer flags: bit 0 =
// L2 without USE_ETA (w -= lambda*w, regularizer.hpp:50-54); bit 1 (SGD) =
// the shrink driver (shrink_sgd_parallelizer.hpp).
#ifndef FVG_ORACLE_H
#define FVG_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
void orc_crs_spmv_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                      const double* x, double* y);
void orc_crs_spmv_f32(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const float* val,
                      const float* x, float* y);
void orc_crs_transpose_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                           int32_t* toff, int32_t* tidx, double* tval);
void orc_crs_spmm_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                      const double* X, int64_t k, double* Y);
int64_t orc_ell_width(int64_t m, const int32_t* off);
void orc_ell_build_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                       int32_t* eidx, double* eval);
void orc_ell_spmv_f64(int64_t m, int64_t n, int64_t width, const int32_t* eidx, const double* eval,
                      const double* x, double* y);
void orc_ell_trans_mv_f64(int64_t m, int64_t n, int64_t width, const int32_t* eidx, const double* eval,
                          const double* v, double* y);
void orc_jds_build_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                       int32_t* perm, int64_t* joff, int32_t* jidx, double* jval, int64_t* out_ndiag);
void orc_jds_spmv_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                      const double* x, double* y);
void orc_hyb_info(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val, int64_t thr,
                  int64_t* info);
void orc_hyb_build_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                       int64_t thr, int32_t* perm, int64_t* joff, int32_t* jidx, double* jval, int64_t* coff,
                       int32_t* cidx, double* cval);
void orc_hyb_spmv_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                      int64_t thr, const double* x, double* y);
void orc_fmt_mv_f64(int fmt, int trans, int64_t m, int64_t n, const int32_t* off, const int32_t* idx,
                    const double* val, const double* x, double* y);
// GLM loss kinds (lkind): 0 logistic, 1 linear, 2 hinge, 3 epsilon-
// insensitive, 4 squared epsilon-insensitive (eps used by 3 and 4).
void orc_glm_dloss_f64(int lkind, double eps, int64_t m, const double* label, const double* wtx, double* dloss,
                       double* sumloss);
void orc_glm_eval_f64(int fmt, int64_t m, int64_t n, const int32_t* off, const int32_t* idx,
                      const double* val, const double* label, const double* sw, const double* w, double b,
                      int icpt, const int64_t* splits, int P, int nthreads, double* grad, double* loss, int lkind,
                      double eps);
int orc_glm_lbfgs_f64(int fmt, int64_t m, int64_t n, const int32_t* off, const int32_t* idx,
                      const double* val, const double* label, const double* sw, const int64_t* splits, int P,
                      int nthreads, int64_t num_iter, int64_t hist, double lambda, int rtype, int icpt,
                      double tol, double* w, double* b, int64_t* n_iter, double* final_loss, double* trace,
                      int flags, int lkind, double eps);
// A problem built once (per-rank matrices and transposed copies) for
// repeated L-BFGS runs; orc_problem_create returns NULL on bad arguments.
void* orc_problem_create(int fmt, int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                         const double* label, const double* sw, const int64_t* splits, int P, int nthreads,
                         int lkind, double eps);
int orc_problem_lbfgs(void* h, int64_t num_iter, int64_t hist, double lambda, int rtype, int icpt, double tol,
                      double* w, double* b, int64_t* n_iter, double* final_loss, double* trace, int flags);
void orc_problem_destroy(void* h);
int orc_glm_sgd_f64(int fmt, int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                    const double* label, const double* sw, const int64_t* splits, int P, int nthreads,
                    int64_t num_iter, double alpha, double frac, double lambda, int rtype, int icpt, double tol,
                    double* w, double* b, int64_t* n_iter, double* final_loss, int flags, int lkind, double eps);
void orc_predict_probability_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx,
                                 const double* val, const double* w, double b, double* out);
// multinomial logistic regression by L-BFGS (the softmax gradient with the
// L-BFGS driver, cross-entropy loss, no intercept); W row-major n x K in/out
int orc_softmax_lbfgs_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                          const double* label, const double* sw, int64_t K, int64_t num_iter, int64_t hist,
                          double lambda, int rtype, double tol, double* W, int64_t* n_iter, double* final_loss,
                          double* trace);
int orc_softmax_train_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                          const double* label, const double* sw, int64_t K, int64_t num_iter, double alpha,
                          double lambda, int rtype, int icpt, double tol, double* W, double* b, int64_t* n_iter);
void orc_softmax_probability_f64(int64_t m, int64_t n, const int32_t* off, const int32_t* idx, const double* val,
                                 const double* W, const double* b, int64_t K, int icpt, double* prob);
#ifdef __cplusplus
}
#endif
#endif
