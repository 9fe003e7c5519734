/*
 * fvg.h — C ABI of the GB300 sparse logistic-regression path.
 *
 * One process drives one GPU.  A context owns a CUDA stream; matrices are
 * uploaded once (CRS, int32 row offsets and column ids, FP64/FP32/BF16
 * values), and the derived device layouts the reference builds on the host
 * (transposed CRS, ELL, JDS, JDS/CRS hybrid) are built on the device.
 * Every call returns an fvg_status; no C++ exception crosses this boundary.
 * fvg_ctx_last_error() gives the message of the last failing call, which for
 * argument errors repeats the reference's own message.
 *
 * Threading: a context is used by one host thread at a time; calls on one
 * context run in order on its stream.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the frovedis source tree).
 */
#ifndef FVG_H
#define FVG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FVG_API __attribute__((visibility("default")))
#else
#define FVG_API
#endif

typedef struct fvg_ctx fvg_ctx;
typedef struct fvg_matrix fvg_matrix;

typedef enum {
  FVG_OK = 0,
  FVG_ERR_INVALID_ARG = 1,   /* reference: REPORT_ERROR(USER_ERROR, ...) / checkAssumption */
  FVG_ERR_SIZE_MISMATCH = 2, /* reference: std::runtime_error from operator* */
  FVG_ERR_UNSUPPORTED = 3,   /* reference: "Unsupported input matrix type!!" */
  FVG_ERR_CUDA = 4,
  FVG_ERR_OUT_OF_MEMORY = 5,
  FVG_ERR_INTERNAL = 6
} fvg_status;

/* value / vector element types.  FVG_SPLIT is a storage choice only: each
 * FP64 value kept as its FP32 rounding plus the BF16 rounding of the
 * remainder (relative error below 2^-32), multiplied in double-FP32
 * arithmetic (about 48 significant bits) with FP64 vectors at the interface;
 * results agree with FP64 storage to about 1e-10 relative. */
typedef enum { FVG_F64 = 0, FVG_F32 = 1, FVG_BF16 = 2, FVG_SPLIT = 3 } fvg_dtype;

/* same numbering as frovedis::MatType (ml/utility/mattype.hpp:6-11) */
typedef enum { FVG_CRS = 0, FVG_JDS = 1, FVG_ELL = 2, FVG_HYBRID = 3 } fvg_format;

/* same numbering as frovedis::RegType (ml/glm/regularizer.hpp:8-12) */
typedef enum { FVG_REG_ZERO = 0, FVG_REG_L1 = 1, FVG_REG_L2 = 2 } fvg_regtype;
/* Loss of the GLM family (ml/glm/gradient.hpp): logistic_gradient (logistic
 * regression), linear_gradient (linear / ridge / lasso regression),
 * hinge_gradient (linear SVM), epsilon_insensitive and
 * squared_epsilon_insensitive (SVM regression, SVRLossType EPS / SQEPS,
 * svm_regression_with_sgd.hpp:8-11). */
typedef enum {
  FVG_LOSS_LOGISTIC = 0,
  FVG_LOSS_SQUARED = 1,
  FVG_LOSS_HINGE = 2,
  FVG_LOSS_EPS_INSENSITIVE = 3,
  FVG_LOSS_SQ_EPS_INSENSITIVE = 4
} fvg_loss;

/* ------------------------------------------------------------- context */
FVG_API fvg_status fvg_ctx_create(int device, fvg_ctx** out);
FVG_API void fvg_ctx_destroy(fvg_ctx* ctx);
FVG_API const char* fvg_ctx_last_error(const fvg_ctx* ctx);
/* The context's cudaStream_t, for callers that order their own work with it. */
FVG_API void* fvg_ctx_stream(fvg_ctx* ctx);
FVG_API fvg_status fvg_ctx_synchronize(fvg_ctx* ctx);
/* Kernel timing with CUDA events on the context stream (off by default).
 * Names: "spmv_crs", "pass1", "pass2", "finalize", "lbfgs_vec", "transpose",
 * "spmv_ell", "spmv_jds", "spmv_hyb", "spmm", "pass1_f32", "pass2_f32"
 * ("pass1"/"pass2" are the training passes over FP64 or BF16 values, the
 * "_f32" keys those over FP32 values, e.g. after the refinement switch).
 * "batch_evals" is a counter kept whether timing is on or not: *launches =
 * evaluations run by the batched trainers since the context was created,
 * *total_ms = the (dataset, model) evaluations inside them (a count). */
FVG_API fvg_status fvg_ctx_set_profiling(fvg_ctx* ctx, int enable);
FVG_API fvg_status fvg_ctx_get_profile(fvg_ctx* ctx, const char* name, double* total_ms, int64_t* launches);
FVG_API fvg_status fvg_ctx_reset_profile(fvg_ctx* ctx);
/* Number of CUDA kernels this context launched since creation. */
FVG_API int64_t fvg_ctx_kernel_launches(fvg_ctx* ctx);
/* Poll budget of the bounded device-side waits of this context's kernels
 * (the L-BFGS direction's grid barriers, the row-panel and forward-head
 * kernels' bulk-copy waits).  A wait that runs out is abandoned: the kernel
 * records it in the context's error word and finishes (a copy in flight is
 * still drained), and the call returns FVG_ERR_INTERNAL; the context stays
 * usable.  polls < 0 restores the defaults (2^24 barrier polls, 2^16 copy
 * polls of up to 20 us each — about a second, far beyond any healthy wait);
 * 0 makes every wait that is not already complete give up at once.  No reference counterpart (the
 * reference's ranks report failures through MPI, core/mpi_rpc.cc:471-491);
 * a small budget lets a test exercise the give-up path. */
FVG_API fvg_status fvg_ctx_set_wait_limit(fvg_ctx* ctx, int64_t polls);
/* Testing aid: the `after`-th next device allocation made by the library
 * (any context; 0 = the next one) fails as if the device were out of memory,
 * so the call returns FVG_ERR_OUT_OF_MEMORY after releasing what it had
 * allocated.  after < 0 switches it off.  No reference counterpart (the
 * reference surfaces allocation failures as std::bad_alloc,
 * core/exceptions.hpp:22-43). */
FVG_API void fvg_debug_inject_alloc_failure(int64_t after);

/* -------------------------------------------------------------- matrix */
/* Upload a CRS matrix (crs_matrix_local<T,I,O>, matrix/crs_matrix.hpp:240-331):
 * off[num_row+1] with off[0]=0, idx[nnz], val[nnz] of val_dtype.  Pointers
 * are host memory unless on_device != 0 (then they are copied device to
 * device).  nnz = off[num_row] must be < 2^31.  Column ids must lie in
 * [0, num_col) (checked). */
FVG_API fvg_status fvg_matrix_create_crs(fvg_ctx* ctx, int64_t num_row, int64_t num_col, const int32_t* off,
                                         const int32_t* idx, const void* val, fvg_dtype val_dtype, int on_device,
                                         fvg_matrix** out);
FVG_API void fvg_matrix_destroy(fvg_matrix* mat);
FVG_API fvg_status fvg_matrix_info(const fvg_matrix* mat, int64_t* num_row, int64_t* num_col, int64_t* nnz);
/* Build the device layout `fmt` (and its transposed counterpart when
 * with_transpose != 0), replacing the host conversions of
 * ml/utility/matrix_conversion.hpp:12-111.  Idempotent. */
FVG_API fvg_status fvg_matrix_prepare(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, int with_transpose);
/* Add a value plane of another precision (FP32 or BF16, rounded to nearest
 * even from the uploaded values) used when a call asks for that storage. */
FVG_API fvg_status fvg_matrix_add_storage(fvg_ctx* ctx, fvg_matrix* mat, fvg_dtype storage);
/* Layout of the backward product A^T r on FP32 / BF16 values.  No reference
 * counterpart (the reference multiplies its transposed copy,
 * gradient_descent.hpp:211; this is a GPU data-layout choice with the same
 * sums).  A's rows are cut into panels; columns with at least min_per_panel
 * entries per panel on average are summed panel by panel from a shared-memory
 * copy of r's slice, the rest through the transposed CRS.
 * rows < 0: chosen from the matrix (the default; off for small matrices or
 * when few entries fall in such columns); 0: off; > 0: panels of that many
 * rows (a multiple of 4, at most what four CTAs per SM can hold in shared
 * memory).  min_per_panel <= 0 takes the default (2).  Drops a layout built
 * earlier; the next FP32 / BF16 backward product builds the new one. */
FVG_API fvg_status fvg_matrix_set_panels(fvg_ctx* ctx, fvg_matrix* mat, int64_t rows, double min_per_panel);
/* The layout in use (built if needed): info[0] rows per panel (0: none),
 * info[1] panels, info[2] columns kept in the panels, info[3] their entries. */
FVG_API fvg_status fvg_matrix_panel_info(fvg_ctx* ctx, fvg_matrix* mat, int64_t* info);
/* Forward head of A for the FP32 / BF16 forward product A w.  No reference
 * counterpart (the reference multiplies the CRS matrix row by row,
 * crs_matrix.hpp:1505-1516; this is a GPU data-layout choice with the same
 * sums): the entries of A's most frequent columns are multiplied from a
 * shared-memory copy of w at those columns, the rest of each row through the
 * CRS kernel, whose epilogue adds both parts.  columns < 0: chosen from the
 * matrix (the default; off for small matrices or when those columns hold
 * less than half of the entries); 0: off; > 0: that many columns (at most
 * what a CTA can hold in shared memory).  Drops a head built earlier. */
FVG_API fvg_status fvg_matrix_set_head(fvg_ctx* ctx, fvg_matrix* mat, int64_t columns);
/* The head in use (built if needed): info[0] columns (0: none), info[1] their entries. */
FVG_API fvg_status fvg_matrix_head_info(fvg_ctx* ctx, fvg_matrix* mat, int64_t* info);
/* Autotuner of the training layout.  The reference picks the format by
 * MatType alone (CRS on x86, HYBRID on VE,
 * ml/glm/logistic_regression_with_lbfgs.hpp:280-285); every layout here gives
 * the same sums up to summation order, so the choice is one of speed.  Each
 * candidate — format (CRS; for FP32 / BF16 values also ELL when its padding
 * stays within 4x the nonzeros, and HYBRID), the forward head on or off, the
 * row panels off or on with a hot threshold of 1, 2 or 4 entries per panel —
 * is timed over `reps` loss/gradient evaluations with `label` (NULL: all
 * ones), and the fastest layout is left set on the matrix (as
 * fvg_matrix_set_head / fvg_matrix_set_panels would); train with
 * mat_type = best->format.  tried[0..max_tried) receives the candidates that
 * applied, *n_tried their number (both may be NULL). */
typedef struct {
  int32_t format;   /* fvg_format */
  int32_t head;     /* forward head: 0 off, 1 on (columns chosen from the matrix) */
  double panel_min; /* row panels: 0 off, > 0 the hot threshold (entries per panel) */
  double eval_ms;   /* time of one loss/gradient evaluation */
} fvg_tune_choice;
FVG_API fvg_status fvg_matrix_autotune(fvg_ctx* ctx, fvg_matrix* mat, fvg_dtype storage, const double* label,
                                       int32_t reps, fvg_tune_choice* best, fvg_tune_choice* tried,
                                       int64_t max_tried, int64_t* n_tried);
/* Device bytes held by the matrix and everything derived from it. */
FVG_API int64_t fvg_matrix_device_bytes(const fvg_matrix* mat);

/* The uploaded matrix itself: off[num_row+1], idx[nnz], val[nnz] (FP64). */
FVG_API fvg_status fvg_matrix_get_crs(fvg_ctx* ctx, fvg_matrix* mat, int32_t* off, int32_t* idx, double* val);

/* ------------------------------------------------------------- loaders
 * The reference's on-disk CRS formats, parsed on the device (values
 * bit-identical to strtod / strtof; lines must be well formed: "col:value"
 * tokens separated by white space).  val_dtype: FVG_F64 (T = double) or
 * FVG_F32 (T = float). */
/* make_crs_matrix_local_load(file[, num_col]) (matrix/crs_matrix.hpp:757-775):
 * one row per line, 0-based column ids; num_col < 0: largest id + 1. */
FVG_API fvg_status fvg_matrix_load_text(fvg_ctx* ctx, const char* path, fvg_dtype val_dtype, int64_t num_col,
                                        fvg_matrix** out);
/* make_crs_matrix_local_loadlibsvm(file, label, idxorg) (crs_matrix.hpp:874-899):
 * "label col:value ..." per line; index_origin as frovedis::IndexOrigin
 * (0 AUTO, 1 ZERO_ORIG, 2 ONE_ORIG); num_col = largest id in the file + 1.
 * The labels are kept with the matrix: fvg_matrix_get_labels. */
FVG_API fvg_status fvg_matrix_load_libsvm(fvg_ctx* ctx, const char* path, fvg_dtype val_dtype, int index_origin,
                                          fvg_matrix** out);
FVG_API fvg_status fvg_matrix_get_labels(const fvg_matrix* mat, double* labels);
/* make_crs_matrix_local_loadbinary(dir) (crs_matrix.hpp:565-603): nums, an
 * optional type file checked against (val_dtype, idx_type, off_type) — type
 * names as the reference writes them ("int32_t", "uint32_t", "int64_t",
 * "uint64_t"; NULL = "uint64_t", i.e. size_t) — and the val/idx/off arrays
 * in native byte order. */
FVG_API fvg_status fvg_matrix_load_binary(fvg_ctx* ctx, const char* dir, fvg_dtype val_dtype, const char* idx_type,
                                          const char* off_type, fvg_matrix** out);

/* Copies of the derived layouts to host memory, in the reference's array
 * order, for checking the device builders against the reference's:
 *  transpose  — crs_matrix_local::transpose (crs_matrix.hpp:356-412):
 *               toff[num_col+1], tidx[nnz], tval[nnz] (FP64).
 *  ELL        — ell_matrix_local(crs) (ell_matrix.hpp:63-95): width, then
 *               eidx/eval column-major [width*num_row].
 *  JDS        — jds_matrix_local(crs) (jds_matrix.hpp:81-146): perm[num_row],
 *               joff[ndiag+1], jidx/jval[nnz].
 *  hybrid     — jds_crs_hybrid_local(crs, 256) (jds_crs_hybrid.hpp:38-153):
 *               info = {jds ndiag, crs rows, crs nnz, jds nnz, perm length},
 *               then the JDS part and the CRS tail.
 * Pass NULL array pointers to query sizes only. */
FVG_API fvg_status fvg_matrix_get_transpose(fvg_ctx* ctx, fvg_matrix* mat, int32_t* toff, int32_t* tidx,
                                            double* tval);
FVG_API fvg_status fvg_matrix_get_ell(fvg_ctx* ctx, fvg_matrix* mat, int64_t* width, int32_t* eidx, double* eval);
FVG_API fvg_status fvg_matrix_get_jds(fvg_ctx* ctx, fvg_matrix* mat, int64_t* ndiag, int32_t* perm, int64_t* joff,
                                      int32_t* jidx, double* jval);
FVG_API fvg_status fvg_matrix_get_hybrid(fvg_ctx* ctx, fvg_matrix* mat, int64_t* info, int32_t* perm,
                                         int64_t* joff, int32_t* jidx, double* jval, int64_t* coff, int32_t* cidx,
                                         double* cval);

/* ------------------------------------------------------------ products */
/* y = A x: operator*(crs_matrix_local, vector) (crs_matrix.hpp:1518-1525),
 * operator*(ell_matrix_local, vector) (ell_matrix.hpp:229), operator*(
 * jds_matrix_local, vector) (jds_matrix.hpp:419-426), operator*(
 * jds_crs_hybrid_local, vector) (jds_crs_hybrid.hpp:213-221).
 * x has num_col and y num_row elements of vec_dtype (FVG_F64 or FVG_F32);
 * storage picks the value plane (FP64 values need FVG_F64 vectors).
 * Accumulation is FP64 for FP64 vectors and FP32 otherwise.
 * on_device != 0: x and y are device pointers (ordered on the ctx stream). */
FVG_API fvg_status fvg_spmv(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, fvg_dtype storage, fvg_dtype vec_dtype,
                            const void* x, void* y, int on_device);
/* y = A^T x, x has num_row and y num_col elements: trans_mv(ell_matrix_local,
 * vector) (ell_matrix.hpp:357-380) and `trans * v` on the transposed copy
 * (gradient_descent.hpp:211).  Always computed as a gather over a device
 * transposed copy in `fmt` (deterministic; no atomics). */
FVG_API fvg_status fvg_trans_mv(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, fvg_dtype storage,
                                fvg_dtype vec_dtype, const void* x, void* y, int on_device);
/* Y = A X, X row-major num_col x k, Y row-major num_row x k:
 * operator*(crs_matrix_local, rowmajor_matrix_local) (crs_matrix.hpp:2053-2064),
 * jds (jds_matrix.hpp:799-807), hybrid (jds_crs_hybrid.hpp:244-252). */
FVG_API fvg_status fvg_spmm(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, fvg_dtype storage, fvg_dtype vec_dtype,
                            const void* X, int64_t k, void* Y, int on_device);

/* y = A x over the CRS layout, x and y device pointers (FP64 vectors for
 * FVG_F64 storage, FP32 vectors for FVG_F32 / FVG_BF16), queued on the
 * context stream without waiting for it.  No counterpart in the reference.
 * It allocates nothing, for callers that cannot allocate device memory: a
 * plug-in inside a host framework that owns all device allocations, or a
 * latency-critical loop that must not pay cudaMalloc's implicit
 * synchronisation.  Its scratch is a fixed 8 MiB device array inside the
 * library (held by every GPU that loads it, until exit), enough for long rows
 * totalling ~512 million nonzeros; larger matrices get FVG_ERR_INVALID_ARG.
 * The matrix must be prepared first (fvg_matrix_prepare with FVG_CRS, and
 * fvg_matrix_add_storage for FP32/BF16).  The first call on a device looks up
 * the array's device address (one-time set-up; make it before any stream
 * capture).  The call runs with the context's device current and restores
 * the caller's device before it returns.  Calls share the array: calls that
 * overlap on the GPU race.  Calls on one context are ordered by its stream;
 * calls from different contexts on the same device (each context has its own
 * stream, e.g. one per host thread) must be serialised by the caller —
 * synchronise the first context, or make the second context's stream wait on
 * an event recorded after the first call. */
FVG_API fvg_status fvg_spmv_no_alloc(fvg_ctx* ctx, fvg_matrix* mat, fvg_dtype storage, fvg_dtype vec_dtype,
                                     const void* x, void* y);

/* ------------------------------------------------------------ training */
typedef struct {
  int64_t num_iteration;      /* numIteration (default 1000) */
  double alpha;               /* alpha (default 0.01) */
  int64_t hist_size;          /* L-BFGS history (default 10) */
  double reg_param;           /* regParam (default 0.01) */
  int32_t reg_type;           /* fvg_regtype (default ZERO) */
  int32_t intercept;          /* isIntercept (default 0) */
  double convergence_tol;     /* convergenceTol (default 0.001) */
  int32_t mat_type;           /* fvg_format (default CRS) */
  double mini_batch_fraction; /* SGD miniBatchFraction (default 1.0) */
  int32_t num_partitions;     /* SGD/L-BFGS: emulate this many MPI ranks
                                 (row blocks; default 1) */
  int32_t storage;            /* value precision: FVG_F64 (default), FVG_F32, FVG_BF16 */
  int32_t refine;             /* BF16/F32 storage: switch to FP32 values once the
                                 gradient norm stalls (default 1) */
  double refine_stall;        /* stall test: rms > refine_stall * best rms of the
                                 last 3 iterations (default 0.97) */
  int32_t l2_no_eta;          /* L2 as w -= lambda*w (the reference built without
                                 USE_ETA, regularizer.hpp:50-54) (default 0) */
  int32_t use_graph;          /* capture per-trial work as CUDA graphs (default 1) */
  double* trace;              /* optional host array, 4 doubles per iteration:
                                 loss, line-search trials, rms, step factor */
  const int64_t* row_splits;  /* optional num_partitions+1 row splits */
  int32_t loss;               /* fvg_loss of fvg_glm_* trainers (default
                                 LOGISTIC; the fvg_logreg_* entry points
                                 always use LOGISTIC) */
  double epsilon;             /* epsilon of the eps-insensitive losses (default 0) */
} fvg_glm_params;

FVG_API void fvg_glm_params_default(fvg_glm_params* p);

/* logistic_regression_with_lbfgs::train main API
 * (ml/glm/logistic_regression_with_lbfgs.hpp:395-437 →
 *  lbfgs_parallelizer.hpp:267-364, 366-462, 515-600).
 * label[num_row] (±1), sample_weight[num_row] or NULL (= all ones),
 * weight[num_col] and intercept hold the initial model on entry and the
 * trained model on return.  Host pointers. */
FVG_API fvg_status fvg_logreg_lbfgs(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                    const double* sample_weight, const fvg_glm_params* params, double* weight,
                                    double* intercept, int64_t* n_iter, double* final_loss);
/* k logistic_regression_with_lbfgs::train runs on one matrix, trained
 * together (a regularisation path, or a hyper-parameter sweep): model j uses
 * regParam = reg_params[j] and every other setting of params (CRS format,
 * one partition).  One forward product A W (W num_col x k) with the logistic
 * epilogue per (row, model) and one backward product A^T R serve all models
 * per evaluation.  Each model takes its own line-search decisions and stops
 * on its own convergence test, so its result is that of a separate
 * fvg_logreg_lbfgs run up to summation order (with FVG_BF16 storage all
 * models move to FP32 values together, once any model's gradient stalls).
 * weight[k*num_col] (model j at j*num_col) and intercept[k] hold the initial
 * models on entry and the trained ones on return; n_iter[k], final_loss[k].
 * 1 <= k <= 256.  The reference runs the models one train() call at a time
 * (logistic_regression_with_lbfgs.hpp:395-437). */
FVG_API fvg_status fvg_logreg_lbfgs_batched(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                            const double* sample_weight, const fvg_glm_params* params, int64_t k,
                                            const double* reg_params, double* weight, double* intercept,
                                            int64_t* n_iter, double* final_loss);
/* The batched trainer over several datasets at once: the k models of every
 * dataset (num_datasets x k in all, model (d, j) on mats[d] with regParam =
 * reg_params[j]) train together, the datasets' matrices stacked
 * block-diagonally so that one forward and one backward product per
 * evaluation serve all of them.  Each model takes its own line-search
 * decisions and stops on its own, so its result is that of a separate
 * fvg_logreg_lbfgs run on its dataset up to summation order.  The whole
 * training is one CUDA-graph launch (the line-search and stop decisions are
 * taken on the device).  labels[d] / sample_weights[d] (the array or any
 * entry may be NULL = all ones) have mats[d]'s num_row entries;
 * weight: dataset d's models follow those of datasets 0..d-1, model j at
 * offset j*num_col(d) inside them; intercept, n_iter, final_loss:
 * [num_datasets][k].  The stacked matrices must stay below 2^31 rows,
 * columns (sum of num_col + 1) and nonzeros; 1 <= k <= 256.  No counterpart
 * in the reference, which trains one model per train() call
 * (logistic_regression_with_lbfgs.hpp:395-437). */
FVG_API fvg_status fvg_logreg_lbfgs_multi(fvg_ctx* ctx, int64_t num_datasets, fvg_matrix* const* mats,
                                          const double* const* labels, const double* const* sample_weights,
                                          const fvg_glm_params* params, int64_t k, const double* reg_params,
                                          double* weight, double* intercept, int64_t* n_iter, double* final_loss);
/* multinomial_logistic_regression::train main API
 * (ml/glm/multinomial_logistic_regression.hpp:342-378 → softmax_parallelizer::
 * parallelize / do_train, softmax_parallelizer.hpp:210-242, 277-345):
 * gradient descent with step alpha/sqrt(i) on the softmax error, the
 * reference's intercept update (column sums of the gradient matrix) and its
 * RMS-of-change stop test.  label[num_row] holds class ids 0..nclasses-1;
 * weight[num_col*nclasses] (row-major, feature-major like the reference's
 * rowmajor_matrix_local weight) and intercept[nclasses] hold the initial model
 * on entry and the trained one on return.  params: num_iteration, alpha,
 * reg_param, reg_type, intercept, convergence_tol, mat_type (CRS or HYBRID,
 * both computed on the CRS layout), storage. */
FVG_API fvg_status fvg_multinomial_train(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                         const double* sample_weight, const fvg_glm_params* params, int64_t nclasses,
                                         double* weight, double* intercept, int64_t* n_iter);
/* Multinomial logistic regression by L-BFGS: no reference counterpart (the
 * reference trains it by gradient descent only).  The gradient is the
 * reference's softmax gradient with the transposed copy
 * (ml/glm/softmax_gradient_descent.hpp:119-136), the L-BFGS loop that of the
 * binary trainers (lbfgs.hpp:79-143, lbfgs_parallelizer.hpp:267-364), and
 * the line search's loss the cross-entropy sum_i -log p[i, label_i]
 * (unweighted, as logistic_gradient's loss).  No intercept; 2 <= nclasses
 * <= 128.  label[num_row] holds class ids; weight[num_col*nclasses]
 * (row-major) the initial model on entry, the trained one on return.
 * params: num_iteration, hist_size, reg_param, reg_type, convergence_tol,
 * mat_type (CRS or HYBRID, computed on the CRS layout), storage (FP64, FP32
 * or BF16 values), trace. */
FVG_API fvg_status fvg_multinomial_lbfgs(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                         const double* sample_weight, const fvg_glm_params* params, int64_t nclasses,
                                         double* weight, int64_t* n_iter, double* final_loss);
/* multinomial_logistic_regression_model<T>::compute_probability_matrix
 * (multinomial_logistic_regression_model.hpp:82-89): prob[num_row*nclasses],
 * FP64. */
FVG_API fvg_status fvg_multinomial_probability(fvg_ctx* ctx, fvg_matrix* mat, const double* weight,
                                               const double* intercept, int64_t nclasses, int intercept_on,
                                               double* prob);
/* logistic_regression_with_sgd::train main API
 * (ml/glm/logistic_regression_with_sgd.hpp:392-441 →
 *  sgd_parallelizer.hpp:132-378, 441-550). */
FVG_API fvg_status fvg_logreg_sgd(fvg_ctx* ctx, fvg_matrix* mat, const double* label, const double* sample_weight,
                                  const fvg_glm_params* params, double* weight, double* intercept, int64_t* n_iter,
                                  double* final_loss);
/* shrink::logistic_regression_with_sgd::train main API
 * (ml/glm/shrink_logistic_regression_with_sgd.hpp → shrink_sgd_parallelizer.hpp:
 * 82-151, 153-253, 378-494): SGD as fvg_logreg_sgd, except that every rank
 * keeps only the columns its rows use (shrink_column) — those alone are
 * regularised, with eta = 1, and columns no rank uses come back as 0; the
 * RMS stop test takes the summed change before regularisation plus rank 0's
 * intercept change over rank 0's column count + 1; with FVG_ELL the
 * reported iteration count is numIteration + 1 when the test never passed
 * (the driver's no-trans loop). */
FVG_API fvg_status fvg_logreg_shrink_sgd(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                         const double* sample_weight, const fvg_glm_params* params, double* weight,
                                         double* intercept, int64_t* n_iter, double* final_loss);
/* One loss/gradient evaluation (gradient_descent::compute_gradient,
 * gradient_descent.hpp:196-225): grad[num_col+1] (bias last), *loss. */
FVG_API fvg_status fvg_logreg_eval(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, fvg_dtype storage,
                                   const double* label, const double* sample_weight, const double* weight,
                                   double intercept, int intercept_on, double* grad, double* loss);
/* The GLM family on the same device path, the loss taken from params->loss
 * (params->epsilon for the eps-insensitive kinds); otherwise as
 * fvg_logreg_lbfgs / fvg_logreg_sgd / fvg_logreg_lbfgs_batched:
 *   FVG_LOSS_SQUARED: linear_regression_with_{sgd,lbfgs} (reg_type ZERO),
 *     ridge_regression_with_{sgd,lbfgs} (L2), lasso_with_{sgd,lbfgs} (L1)
 *     (ml/glm/linear_regression_with_sgd.hpp:304-330, ..._with_lbfgs.hpp,
 *     ridge_regression_with_*.hpp, lasso_with_*.hpp);
 *   FVG_LOSS_HINGE: svm_with_{sgd,lbfgs} (svm_with_sgd.hpp, svm_with_lbfgs.hpp),
 *     label +-1;
 *   FVG_LOSS_EPS_INSENSITIVE / FVG_LOSS_SQ_EPS_INSENSITIVE:
 *     svm_regression_with_sgd (svm_regression_with_sgd.hpp:373-444).
 * The reference's SGD trainers start from intercept 0, its L-BFGS trainers
 * from intercept = isIntercept (…_with_sgd.hpp initModel(numFeatures) vs
 * …_with_lbfgs.hpp initModel(numFeatures, intercept)); the caller passes the
 * initial model. */
FVG_API fvg_status fvg_glm_lbfgs(fvg_ctx* ctx, fvg_matrix* mat, const double* label, const double* sample_weight,
                                 const fvg_glm_params* params, double* weight, double* intercept, int64_t* n_iter,
                                 double* final_loss);
FVG_API fvg_status fvg_glm_sgd(fvg_ctx* ctx, fvg_matrix* mat, const double* label, const double* sample_weight,
                               const fvg_glm_params* params, double* weight, double* intercept, int64_t* n_iter,
                               double* final_loss);
FVG_API fvg_status fvg_glm_lbfgs_batched(fvg_ctx* ctx, fvg_matrix* mat, const double* label,
                                         const double* sample_weight, const fvg_glm_params* params, int64_t k,
                                         const double* reg_params, double* weight, double* intercept,
                                         int64_t* n_iter, double* final_loss);
FVG_API fvg_status fvg_glm_lbfgs_multi(fvg_ctx* ctx, int64_t num_datasets, fvg_matrix* const* mats,
                                       const double* const* labels, const double* const* sample_weights,
                                       const fvg_glm_params* params, int64_t k, const double* reg_params,
                                       double* weight, double* intercept, int64_t* n_iter, double* final_loss);
/* One loss/gradient evaluation for any fvg_loss (compute_gradient with the
 * kind's compute_dloss, gradient.hpp). */
FVG_API fvg_status fvg_glm_eval(fvg_ctx* ctx, fvg_matrix* mat, fvg_format fmt, fvg_dtype storage, int32_t loss,
                                double epsilon, const double* label, const double* sample_weight,
                                const double* weight, double intercept, int intercept_on, double* grad,
                                double* loss_out);
/* logistic_regression_model<T>::predict_probability (ml/glm/linear_model.hpp:376-392). */
FVG_API fvg_status fvg_logreg_predict_probability(fvg_ctx* ctx, fvg_matrix* mat, const double* weight,
                                                  double intercept, double* prob);

#ifdef __cplusplus
}
#endif
#endif /* FVG_H */
