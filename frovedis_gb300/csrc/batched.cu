// Batched L-BFGS: k GLM models on each of nd datasets, trained together.
// Model (d, j) trains on dataset d with regularisation value lam[j] and its
// own initial model, every other setting shared.  Each model follows
// lbfgs_parallelizer::do_train (ml/glm/lbfgs_parallelizer.hpp:267-364) with
// lbfgs<T>::compute_hkgk / update_history (ml/glm/lbfgs.hpp:79-143) exactly
// as the single-model driver does.  The reference trains one model per
// train() call (logistic_regression_with_lbfgs.hpp:395-437); here all
// models share the matrix passes.
//
// Datasets are stacked block-diagonally: the rows of all datasets form one
// CRS whose column ids are shifted to each dataset's own block of model
// rows, so one forward product A W (W: the stacked model vectors, models as
// columns) with the per-(row, model) loss epilogue and one backward product
// A^T R per evaluation serve every model of every dataset, reading each
// matrix once.  Per-dataset loss and bias sums come from the forward pass's
// stacked-dataset partials (crs_spmm_logreg_seg).
//
// Vectors are row-major with the models as columns: dataset d owns rows
// [doff[d], doff[d+1]) = its num_col weight rows and one bias row, ld = k
// rounded up to 8 columns (whole 32-byte lane groups for the products).  The per-model
// reductions of the two-loop recursion run as column reductions: a CTA of 256
// threads covers 256/kp rows x kp columns (kp = k rounded up to a power of
// two), blockIdx.y is the dataset, and partial sums per (dataset, CTA,
// column) are combined in CTA order by the dataset's last CTA
// (deterministic).
//
// The loop runs on the device.  Line search: every model still searching
// takes its next trial; a model that accepted keeps its trial weights, so
// re-evaluating it in later trials of the same iteration reproduces the same
// loss and gradient.  A converged model stops (its weights are frozen) while
// the others continue.  The history ring (cir_array_list) advances
// identically for all active models, so its indices are host constants of
// the iteration.  Control words on the device (models searching, models
// active, the precision switch) gate every launch: a launch whose word is 0
// returns at once, so the whole training is one fixed launch sequence,
// captured once as a CUDA graph and launched once.  With BF16 values the
// switch to FP32 values (the refinement phase) is decided on the device too,
// once any model's gradient norm stalls.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fvg_internal.cuh"

namespace fvg {

constexpr int kBT = 256;
constexpr int kBMaxHist = 32;
constexpr int kBMaxModels = 256;

struct ColState {
  double rho[kBMaxHist], yy[kBMaxHist], al[kBMaxHist], beta[kBMaxHist];
  double factor[12];
  double dot_gs, smax, stepsize, flip, bstep;
  double loss;                  // accepted loss
  double gmax, gnorm, rms;      // of the accepted gradient
  double gmax_t, gnorm_t, rms_t;  // of the last evaluated gradient
  double lambda;
  double rh[4];                 // gradient rms after the last four iterations
  int nrh;
  int active, searching, trials, n_iter;
};

// control words
enum BCtl {
  C_SEARCH = 0,  // models still searching in this iteration
  C_ACTIVE,      // models not yet converged
  C_SWITCHED,    // BF16 -> FP32 values done
  C_REEVAL,      // re-evaluate the accepted models in FP32 (just switched)
  C_EVAL_LO,     // trial evaluation in the starting storage
  C_EVAL_HI,     // trial evaluation in FP32 after the switch
  C_TRIAL,       // C_SEARCH > 0
  C_ONE,         // always 1
  C_NEVAL,       // evaluations run
  C_NMODEL,      // (dataset, model) evaluations run
  C_NCTL = 16
};

__device__ __forceinline__ void set_flags(int* ctl) {
  const int tr = ctl[C_SEARCH] > 0;
  ctl[C_TRIAL] = tr;
  ctl[C_EVAL_LO] = tr && !ctl[C_SWITCHED];
  ctl[C_EVAL_HI] = tr && ctl[C_SWITCHED];
}

struct BArgs {
  int k, ld, kp, rpb, h;
  const i64* doff;   // [nd+1] first vector row of each dataset
  i64 plane;         // elements of one vector (all datasets)
  double* part;      // [nd][grid][k][NV]
  unsigned* ticket;  // [nd]
  ColState* st;      // [nd][ld]
  const int* ctl;
  int gate;          // control word gating the launch (< 0: none)
  const unsigned long long* mask;  // [nd][nwd] models the launch serves (null: all)
  int nwd;
};

__device__ __forceinline__ bool model_on(const BArgs& a, int ds, int j) {
  if (!a.mask) return true;
  return (__ldcg(a.mask + (i64)ds * a.nwd + (j >> 6)) >> (j & 63)) & 1ull;
}
__device__ __forceinline__ bool dataset_on(const BArgs& a, int ds) {
  if (!a.mask) return true;
  unsigned long long any = 0;
  for (int w = 0; w < a.nwd; w++) any |= __ldcg(a.mask + (i64)ds * a.nwd + w);
  return any != 0;
}

// model masks of nd datasets from the state flag picked by `field`
// (0: searching, 1: active), a 64-bit word per 64 models
__device__ __forceinline__ void build_masks(const ColState* st, int nd, int ld, int nwd, int field,
                                            unsigned long long* out) {
  for (int w = threadIdx.x; w < nd * nwd; w += blockDim.x) {
    const int d = w / nwd, j0 = (w % nwd) * 64;
    unsigned long long m = 0;
    for (int b = 0; b < 64 && j0 + b < ld; b++) {
      const ColState& s = st[(i64)d * ld + j0 + b];
      if (field == 0 ? s.searching : s.active) m |= 1ull << b;
    }
    out[w] = m;
  }
}

// Fixed-order reduction of NV values per column; fin(j, totals) runs once
// per column in the dataset's last CTA.
template <int NV, class Fin>
__device__ __forceinline__ void col_reduce(double (&v)[NV], const bool (&is_max)[NV], const BArgs& a, Fin fin) {
  __shared__ double sm[NV][kBT];
  __shared__ bool last;
  const int j = threadIdx.x % a.kp, rr = threadIdx.x / a.kp;
  double* part = a.part + (i64)blockIdx.y * gridDim.x * a.k * NV;
  unsigned* ticket = a.ticket + blockIdx.y;
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int s = a.rpb / 2; s > 0; s >>= 1) {
    if (rr < s)
#pragma unroll
      for (int q = 0; q < NV; q++) {
        const double o = sm[q][threadIdx.x + s * a.kp];
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], o) : sm[q][threadIdx.x] + o;
      }
    __syncthreads();
  }
  if (rr == 0 && j < a.k)
#pragma unroll
    for (int q = 0; q < NV; q++) part[((i64)blockIdx.x * a.k + j) * NV + q] = sm[q][threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) t[q] = 0.0;
  if (j < a.k) {
    // the CTAs' partials in CTA order; eight loads issued before they are
    // combined (same order as one at a time)
    i64 b = rr;
    for (; b + 7 * a.rpb < gridDim.x; b += 8 * a.rpb) {
      double x[8][NV];
#pragma unroll
      for (int u = 0; u < 8; u++)
#pragma unroll
        for (int q = 0; q < NV; q++) x[u][q] = __ldcg(&part[((b + u * a.rpb) * a.k + j) * NV + q]);
#pragma unroll
      for (int u = 0; u < 8; u++)
#pragma unroll
        for (int q = 0; q < NV; q++) t[q] = is_max[q] ? fmax(t[q], x[u][q]) : t[q] + x[u][q];
    }
    for (; b < gridDim.x; b += a.rpb)
#pragma unroll
      for (int q = 0; q < NV; q++) {
        const double x = __ldcg(&part[(b * a.k + j) * NV + q]);
        t[q] = is_max[q] ? fmax(t[q], x) : t[q] + x;
      }
  }
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = t[q];
  __syncthreads();
  for (int s = a.rpb / 2; s > 0; s >>= 1) {
    if (rr < s)
#pragma unroll
      for (int q = 0; q < NV; q++) {
        const double o = sm[q][threadIdx.x + s * a.kp];
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], o) : sm[q][threadIdx.x] + o;
      }
    __syncthreads();
  }
  if (rr == 0 && j < a.k) {
    double tot[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) tot[q] = sm[q][threadIdx.x];
    fin(j, tot);
  }
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;
}

// thread -> (column j, first row r0 of dataset blockIdx.y); rows advance by
// rpb * gridDim.x; element (r, j) of the dataset at e0 + r * ld, model
// (dataset, j) at st[mj] (read only where `on`)
#define BCOL                                                  \
  if (a.gate >= 0 && __ldcg(a.ctl + a.gate) == 0) return;     \
  const int j = threadIdx.x % a.kp;                           \
  const int rr = threadIdx.x / a.kp;                          \
  const bool on = j < a.k;                                    \
  const int ds = blockIdx.y;                                  \
  const i64 rb = __ldg(a.doff + ds);                          \
  const i64 n1 = __ldg(a.doff + ds + 1) - rb;                 \
  const i64 n = n1 - 1;                                       \
  const i64 rstep = (i64)gridDim.x * a.rpb;                   \
  const i64 r0 = (i64)blockIdx.x * a.rpb + rr;                \
  const i64 ld = a.ld;                                        \
  const i64 e0 = rb * ld + j;                                 \
  const int mj = ds * a.ld + j;                               \
  (void)n;                                                    \
  (void)mj
// The rows of a column in groups of U: every load of a group is issued
// before the first use, so a thread keeps U row-loads in flight (the column
// kernels stream large planes and are bound by memory-level parallelism).
// use() runs in increasing row order, as the plain loop does.
template <int U, class Load, class Use>
__device__ __forceinline__ void rows_grouped(i64 r0, i64 rstep, i64 nrows, Load load, Use use) {
  using V = decltype(load(r0));
  for (i64 rb = r0; rb < nrows; rb += (i64)U * rstep) {
    V buf[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const i64 r = rb + u * rstep;
      if (r < nrows) buf[u] = load(r);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const i64 r = rb + u * rstep;
      if (r < nrows) use(r, buf[u]);
    }
  }
}
constexpr int kRowGroup = 4;
struct V2 { double a, b; };
struct V3 { double a, b, c; };
struct V4 { double a, b, c, d; };

__device__ __forceinline__ i64 hslot(int rear, int i, int h) { return (i64)((rear + i) % h); }

// two-loop recursion, first loop (as in the single-model k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_down(int i, int kh, int rear, const double* __restrict__ G,
                                               double* __restrict__ Q, const double* __restrict__ S,
                                               const double* __restrict__ Y, BArgs a) {
  BCOL;
  const bool act = on && a.st[mj].active;
  const bool first = (i == kh - 1);
  const double* Si = S + hslot(rear, i, a.h) * a.plane;
  const double* Yp = Y + hslot(rear, i + 1, a.h) * a.plane;
  const double alp = (act && !first) ? a.st[mj].al[i + 1] : 0.0;
  double v[1] = {0.0};
  if (act && first)
    rows_grouped<kRowGroup>(r0, rstep, n1, [&](i64 r) { const i64 e = e0 + r * ld; return V2{G[e], Si[e]}; },
                            [&](i64 r, const V2& x) {
                              Q[e0 + r * ld] = x.a;
                              v[0] += x.b * x.a;
                            });
  else if (act)
    rows_grouped<kRowGroup>(r0, rstep, n1,
                            [&](i64 r) { const i64 e = e0 + r * ld; return V3{Q[e], Yp[e], Si[e]}; },
                            [&](i64 r, const V3& x) {
                              const double q = __dsub_rn(x.a, __dmul_rn(x.b, alp));
                              Q[e0 + r * ld] = q;
                              v[0] += x.c * q;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[ds * ld + c];
    if (s.active) s.al[i] = s.rho[hslot(rear, i, a.h)] * t[0];
  });
}

// second loop (as in the single-model k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_up(int i, int kh, int rear, const double* __restrict__ Q,
                                             double* __restrict__ Z, const double* __restrict__ S,
                                             const double* __restrict__ Y, BArgs a) {
  BCOL;
  const bool act = on && a.st[mj].active;
  const double* Yi = Y + hslot(rear, i, a.h) * a.plane;
  const double* Sp = S + hslot(rear, i > 0 ? i - 1 : 0, a.h) * a.plane;
  double H0 = 0.0, f = 0.0, al0 = 0.0;
  if (act) {
    const ColState& s = a.st[mj];
    if (i == 0) {
      const i64 sl = hslot(rear, kh - 1, a.h);
      double yy = s.yy[sl];
      if (yy == 0) yy = 1.0;
      const double ys = 1.0 / s.rho[sl];
      H0 = ys / yy;
      al0 = s.al[0];
    } else {
      f = s.al[i - 1] - s.beta[i - 1];
    }
  }
  double v[1] = {0.0};
  if (act && i == 0)
    rows_grouped<kRowGroup>(r0, rstep, n1, [&](i64 r) { const i64 e = e0 + r * ld; return V2{Q[e], Yi[e]}; },
                            [&](i64 r, const V2& x) {
                              const double z = __dmul_rn(__dsub_rn(x.a, __dmul_rn(x.b, al0)), H0);
                              Z[e0 + r * ld] = z;
                              v[0] += x.b * z;
                            });
  else if (act)
    rows_grouped<kRowGroup>(r0, rstep, n1,
                            [&](i64 r) { const i64 e = e0 + r * ld; return V3{Z[e], Sp[e], Yi[e]}; },
                            [&](i64 r, const V3& x) {
                              const double z = __dadd_rn(x.a, __dmul_rn(x.b, f));
                              Z[e0 + r * ld] = z;
                              v[0] += x.c * z;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[ds * ld + c];
    if (s.active) s.beta[i] = s.rho[hslot(rear, i, a.h)] * t[0];
  });
}

// step = -z, or the no-history step (as in k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_step(int kh, int rear, const double* __restrict__ G,
                                               const double* __restrict__ Z, double* __restrict__ STEP,
                                               const double* __restrict__ S, BArgs a) {
  BCOL;
  const bool act = on && a.st[mj].active;
  const double* Sp = S + hslot(rear, kh > 0 ? kh - 1 : 0, a.h) * a.plane;
  double c = 0.0, f = 0.0;
  if (act) {
    const ColState& s = a.st[mj];
    if (kh == 0) {
      double gn = s.gnorm;
      if (gn > 1) gn = 1.0 / gn;
      c = __dmul_rn(-gn, 0.1);
    } else {
      f = s.al[kh - 1] - s.beta[kh - 1];
    }
  }
  double v[2] = {0.0, 0.0};
  if (act)
    rows_grouped<kRowGroup>(r0, rstep, n1,
                            [&](i64 r) {
                              const i64 e = e0 + r * ld;
                              return kh == 0 ? V3{G[e], 0.0, 0.0} : V3{G[e], Z[e], Sp[e]};
                            },
                            [&](i64 r, const V3& x) {
                              const double z = (kh == 0) ? __dmul_rn(c, x.a) : __dadd_rn(x.b, __dmul_rn(x.c, f));
                              const double st = -z;
                              STEP[e0 + r * ld] = st;
                              v[0] += x.a * st;
                              v[1] = fmax(v[1], fabs(st));
                            });
  const bool mx[2] = {false, true};
  col_reduce<2>(v, mx, a, [&](int c2, double* t) {
    ColState& s = a.st[ds * ld + c2];
    if (!s.active) return;
    s.dot_gs = t[0];
    s.smax = t[1];
  });
}

// max-scaled step norm, uphill flip, factors of the 10 trials (as in k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_step_norm(const double* __restrict__ STEP, BArgs a) {
  BCOL;
  const bool act = on && a.st[mj].active;
  const double mxv = act ? a.st[mj].smax : 0.0;
  const double inv = mxv == 0 ? 0.0 : 1.0 / mxv;
  double v[1] = {0.0};
  if (act)
    rows_grouped<kRowGroup>(r0, rstep, n1, [&](i64 r) { return STEP[e0 + r * ld]; },
                            [&](i64, double x) {
                              const double t = x * inv;
                              v[0] += t * t;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[ds * ld + c];
    if (!s.active) return;
    const double m = s.smax;
    const double ss = (m == 0) ? 0.0 : sqrt(t[0]) * m;
    s.stepsize = ss;
    s.flip = (s.dot_gs > 0) ? -1.0 : 1.0;
    double fac = 1.0;
    if (fac * ss > 1e20) fac = 1e20 / ss;
    s.factor[1] = fac;
    for (int q = 2; q <= 10; q++) s.factor[q] = s.factor[q - 1] / 10.0;
    s.bstep = STEP[(rb + n1 - 1) * ld + c] * s.flip;
  });
}

// models still searching: trial model + regulariser (see k_trial)
__global__ void __launch_bounds__(kBT, 4) kb_trial(int t, const double* __restrict__ W, const double* __restrict__ STEP,
                                                double* __restrict__ NW, float* __restrict__ NWF,
                                                const double* __restrict__ B0, double* __restrict__ B1, int rtype,
                                                int eta_one, int no_eta, BArgs a) {
  BCOL;
  if (!on) return;
  const ColState& s = a.st[mj];
  if (!s.searching) return;
  const double f = s.factor[t], fl = s.flip, lambda = s.lambda;
  const double eta = eta_one ? 1.0 : f;
  const double scale = fmax(0.0, 1.0 - (lambda * eta));
  rows_grouped<kRowGroup>(r0, rstep, n, [&](i64 r) { const i64 e = e0 + r * ld; return V2{W[e], STEP[e]}; },
                          [&](i64 r, const V2& x) {
                            const i64 e = e0 + r * ld;
                            double w = __dadd_rn(x.a, __dmul_rn(f, __dmul_rn(x.b, fl)));
                            if (rtype == FVG_REG_L2) {
                              w = no_eta ? __dsub_rn(w, __dmul_rn(lambda, w)) : __dmul_rn(scale, w);
                            } else if (rtype == FVG_REG_L1) {
                              const double sg = (double)((w >= 0) - (w < 0));
                              w = __dsub_rn(w, __dmul_rn(lambda, sg));
                            }
                            NW[e] = w;
                            if (NWF) NWF[e] = (float)w;
                          });
  if (r0 == 0) B1[mj] = __dadd_rn(B0[mj], __dmul_rn(f, s.bstep));
}

// (a.mask: only the models evaluated last; the others keep their norms)
__global__ void __launch_bounds__(kBT, 4) kb_gmax(const double* __restrict__ G, BArgs a) {
  BCOL;
  if (!dataset_on(a, ds)) return;
  const bool use = on && model_on(a, ds, j);
  double v[1] = {0.0};
  if (use)
    rows_grouped<kRowGroup>(r0, rstep, n1, [&](i64 r) { return G[e0 + r * ld]; },
                            [&](i64, double x) { v[0] = fmax(v[0], fabs(x)); });
  const bool mx[1] = {true};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    if (model_on(a, ds, c)) a.st[ds * ld + c].gmax_t = t[0];
  });
}

// gradient norm and rms; `accepted`: the evaluation is of the accepted
// model (the initial one, or the re-evaluation after a precision switch)
__global__ void __launch_bounds__(kBT, 4) kb_gnorm(const double* __restrict__ G, const double* __restrict__ EV,
                                                int accepted, BArgs a) {
  BCOL;
  if (!dataset_on(a, ds)) return;
  const bool use = on && model_on(a, ds, j);
  const double mxv = use ? a.st[mj].gmax_t : 0.0;
  const double inv = mxv == 0 ? 0.0 : 1.0 / mxv;
  double v[1] = {0.0};
  if (use)
    rows_grouped<kRowGroup>(r0, rstep, n1, [&](i64 r) { return G[e0 + r * ld]; },
                            [&](i64, double x) {
                              const double t = x * inv;
                              v[0] += t * t;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    if (!model_on(a, ds, c)) return;
    const i64 mc = ds * ld + c;
    ColState& s = a.st[mc];
    const double m = s.gmax_t;
    const double nrm = (m == 0) ? 0.0 : sqrt(t[0]) * m;
    s.gnorm_t = nrm;
    s.rms_t = nrm / sqrt((double)n1);
    if (accepted && s.active) {
      s.gnorm = nrm;
      s.rms = s.rms_t;
      s.gmax = m;
      s.loss = EV[2 * mc];
    }
  });
}

// 256-thread count of the models, into ctl[w]; then the derived flags
__device__ __forceinline__ void count_into(int n, int* ctl, int w) {
  __shared__ int cnt[kBT];
  cnt[threadIdx.x] = n;
  __syncthreads();
  for (int s = kBT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) cnt[threadIdx.x] += cnt[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ctl[w] = cnt[0];
    set_flags(ctl);
  }
}

// accept decision of trial t (LBFGS_SEARCH_TOL, lbfgs_parallelizer.hpp:
// 155, 329; the 10th trial is taken whatever its loss)
// (the models still searching: their masks in smask)
__global__ void __launch_bounds__(kBT, 4) kb_decide(int t, const double* __restrict__ EV, int nd, int ld, int nwd,
                                                 ColState* st, int* ctl, unsigned long long* smask) {
  if (ctl[C_TRIAL] == 0) return;
  const int nm = nd * ld;
  if (threadIdx.x == 0) {  // the trial's evaluation ran
    ctl[C_NEVAL] += 1;
    ctl[C_NMODEL] += ctl[C_SEARCH];
  }
  int n = 0;
  for (int j = threadIdx.x; j < nm; j += kBT) {
    ColState& s = st[j];
    if (!s.searching) continue;
    if (EV[2 * j] - s.loss < 1e-4 || t == 10) {
      s.searching = 0;
      s.trials = t;
    } else {
      n++;
    }
  }
  count_into(n, ctl, C_SEARCH);
  __syncthreads();
  build_masks(st, nd, ld, nwd, 0, smask);
}

__global__ void __launch_bounds__(kBT, 4) kb_begin_search(int nd, int ld, int nwd, ColState* st, int* ctl,
                                                       unsigned long long* smask) {
  const int nm = nd * ld;
  int n = 0;
  for (int j = threadIdx.x; j < nm; j += kBT) {
    st[j].searching = st[j].active;
    n += st[j].active;
  }
  count_into(n, ctl, C_SEARCH);
  __syncthreads();
  build_masks(st, nd, ld, nwd, 0, smask);
}

// accept + history push (see k_accept); convergence: rms <= tol stops the model
__global__ void __launch_bounds__(kBT, 4) kb_accept(int nf, int it, double tol, double* __restrict__ W,
                                                 double* __restrict__ G, const double* __restrict__ NW,
                                                 const double* __restrict__ NG, double* __restrict__ S,
                                                 double* __restrict__ Y, double* __restrict__ B0,
                                                 const double* __restrict__ B1, const double* __restrict__ EV,
                                                 BArgs a) {
  BCOL;
  const bool act = on && a.st[mj].active;
  double* Sn = S + (i64)nf * a.plane;
  double* Yn = Y + (i64)nf * a.plane;
  const double bn = act ? B1[mj] : 0.0, bo = act ? B0[mj] : 0.0;
  double v[2] = {0.0, 0.0};
  if (act)  // four planes read per row: groups of two rows keep it within 64 registers
    rows_grouped<2>(r0, rstep, n1,
                    [&](i64 r) {
                      const i64 e = e0 + r * ld;
                      return (r < n) ? V4{NW[e], W[e], NG[e], G[e]} : V4{bn, bo, NG[e], G[e]};
                    },
                    [&](i64 r, const V4& x) {
                      const i64 e = e0 + r * ld;
                      const double s = __dsub_rn(x.a, x.b);
                      double y = __dsub_rn(x.c, x.d);
                      if (fabs(y) < 1e-10) y = 0.0;
                      Sn[e] = s;
                      Yn[e] = y;
                      if (r < n) W[e] = x.a;
                      G[e] = x.c;
                      v[0] += s * y;
                      v[1] += y * y;
                    });
  const bool mx[2] = {false, false};
  col_reduce<2>(v, mx, a, [&](int c, double* t) {
    const i64 mc = ds * ld + c;
    ColState& s = a.st[mc];
    if (!s.active) return;
    double dv = t[0];
    if (dv == 0) dv = 1;
    s.rho[nf] = 1.0 / dv;
    s.yy[nf] = t[1];
    s.loss = EV[2 * mc];
    B0[mc] = B1[mc];
    s.gnorm = s.gnorm_t;
    s.rms = s.rms_t;
    if (s.rms_t <= tol) {
      s.active = 0;
      s.n_iter = it;
    }
  });
}

// End of an iteration: models still active into ctl[C_ACTIVE]; with the
// refinement on (BF16 values), the stall test of the single-model driver on
// every active model's gradient rms — above `stall` times the smallest of
// its three previous values switches all models to FP32 values and asks for
// the accepted models' re-evaluation.
__global__ void __launch_bounds__(kBT, 4) kb_status(int nd, int ld, int nwd, ColState* st, int* ctl, int refine,
                                                 double stall, unsigned long long* amask) {
  const int nm = nd * ld;
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  const bool test = refine && ctl[C_SWITCHED] == 0;
  int n = 0;
  for (int j = threadIdx.x; j < nm; j += kBT) {
    ColState& s = st[j];
    if (!s.active) continue;
    n++;
    if (!test) continue;
    s.rh[s.nrh % 4] = s.rms_t;
    s.nrh++;
    if (s.nrh >= 4) {
      double best = INFINITY;
      for (int q = 2; q <= 4; q++) best = fmin(best, s.rh[(s.nrh - q) % 4]);
      if (s.rms_t > stall * best) any = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && any) {
    ctl[C_SWITCHED] = 1;
    ctl[C_REEVAL] = 1;
  }
  count_into(n, ctl, C_ACTIVE);
  __syncthreads();
  build_masks(st, nd, ld, nwd, 1, amask);
}

__global__ void kb_clear_reeval(int* ctl) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && ctl[C_REEVAL]) {
    ctl[C_NEVAL] += 1;
    ctl[C_NMODEL] += ctl[C_ACTIVE];
    ctl[C_REEVAL] = 0;
  }
}

// model-major [k][n] <-> column layout (one dataset's rows, stride ld; the
// bias row is left untouched by the forward copy)
__global__ void kb_to_cols(const double* __restrict__ src, double* __restrict__ dst, i64 n, int k, i64 ld) {
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (i64)gridDim.x * blockDim.x) {
    const i64 i = e / k;
    const int j = (int)(e - i * k);
    dst[i * ld + j] = src[(i64)j * n + i];
  }
}
__global__ void kb_from_cols(const double* __restrict__ src, double* __restrict__ dst, i64 n, int k, i64 ld) {
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (i64)gridDim.x * blockDim.x) {
    const int j = (int)(e / n);
    const i64 i = e - (i64)j * n;
    dst[e] = src[i * ld + j];
  }
}

__global__ void kb_d2f(const double* __restrict__ s, float* __restrict__ d, i64 n, const int* gate) {
  if (gate && __ldcg(gate) == 0) return;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) d[i] = (float)s[i];
}

// stacked CRS pieces: dst[i] = src[i] + add
__global__ void kb_shift_i32(const i32* __restrict__ src, i64 n, i32 add, i32* __restrict__ dst) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    dst[i] = src[i] + add;
}

// ------------------------------------------------------------ host driver
namespace {

unsigned grid_for(fvg_ctx* c, i64 n) {
  return (unsigned)std::max<i64>(1, std::min<i64>((n + 255) / 256, 4 * (i64)c->num_sms));
}

void shift_copy(fvg_ctx* c, const i32* src, i64 n, i64 add, i32* dst) {
  if (n <= 0) return;
  kb_shift_i32<<<grid_for(c, n), 256, 0, c->stream>>>(src, n, (i32)add, dst);
  check_launch("kb_shift_i32");
  count_launch(c);
}

// Block-diagonal stack of the datasets' matrices (A: rows of all datasets,
// column ids shifted by each dataset's first vector row; AT: the vector rows
// of all datasets, each dataset's bias row empty, column ids shifted by its
// first matrix row), with the value planes `planes`.
void stack_datasets(fvg_ctx* c, const std::vector<fvg_matrix*>& mats, const std::vector<i64>& doff,
                    const std::vector<i64>& roff, const std::vector<int>& planes, DevCRS& A, DevCRS& AT) {
  const int nd = (int)mats.size();
  cudaStream_t s = c->stream;
  i64 nnz = 0;
  for (auto* M : mats) nnz += M->A.nnz;
  if (nnz >= (1ll << 31) - 1 || doff[nd] >= (1ll << 31) - 1 || roff[nd] >= (1ll << 31) - 1)
    fail(FVG_ERR_INVALID_ARG, "stacked datasets exceed 2^31 - 1 rows, columns or nonzeros");
  A.m = roff[nd];
  A.n = doff[nd];
  A.nnz = nnz;
  AT.m = doff[nd];
  AT.n = roff[nd];
  AT.nnz = nnz;
  for (DevCRS* X : {&A, &AT}) {
    X->off.alloc(sizeof(i32) * (X->m + 1), s);
    X->idx.alloc(sizeof(i32) * (nnz + kPad), s);
    FVG_CUDA(cudaMemsetAsync(X->idx.as<i32>() + nnz, 0, sizeof(i32) * kPad, s));
    for (int dt : planes) {
      X->val[dt].alloc((size_t)(nnz + kPad) * dtype_size(dt), s);
      FVG_CUDA(cudaMemsetAsync((char*)X->val[dt].p + (size_t)nnz * dtype_size(dt), 0, (size_t)kPad * dtype_size(dt), s));
    }
  }
  i64 base = 0;
  for (int d = 0; d < nd; d++) {
    DevCRS& a = mats[d]->A;
    DevCRS& t = *mats[d]->AT;
    // A: rows roff[d] .. roff[d] + m_d (the last entry is rewritten by the
    // next dataset with the same value)
    shift_copy(c, a.off.as<i32>(), a.m + 1, base, A.off.as<i32>() + roff[d]);
    shift_copy(c, a.idx.as<i32>(), a.nnz, doff[d], A.idx.as<i32>() + base);
    // AT: rows doff[d] .. doff[d] + n_d, then the empty bias row (its end is
    // the next dataset's first offset, or the total)
    shift_copy(c, t.off.as<i32>(), t.m + 1, base, AT.off.as<i32>() + doff[d]);
    shift_copy(c, t.idx.as<i32>(), t.nnz, roff[d], AT.idx.as<i32>() + base);
    for (int dt : planes) {
      const size_t es = (size_t)dtype_size(dt);
      FVG_CUDA(cudaMemcpyAsync((char*)A.val[dt].p + base * es, a.val[dt].p, a.nnz * es, cudaMemcpyDeviceToDevice, s));
      FVG_CUDA(cudaMemcpyAsync((char*)AT.val[dt].p + base * es, t.val[dt].p, t.nnz * es, cudaMemcpyDeviceToDevice, s));
    }
    A.max_row = std::max(A.max_row, a.max_row);
    AT.max_row = std::max(AT.max_row, t.max_row);
    base += a.nnz;
  }
  const i32 tot = (i32)nnz;
  FVG_CUDA(cudaMemcpyAsync(AT.off.as<i32>() + doff[nd], &tot, sizeof(i32), cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaStreamSynchronize(s));  // `tot` goes out of scope
}

struct BatchEval {
  fvg_ctx* c = nullptr;
  DevCRS* A = nullptr;
  DevCRS* AT = nullptr;
  i64 m = 0;
  int k = 0, ld = 0, nd = 1, icpt = 0;
  int loss = 0;  // GLM loss kind shared by the models
  double eps = 0.0;
  const double* label = nullptr;
  const double* sw = nullptr;
  DBuf label_f, sw_f, R, s1, s2, slots, seg_row, seg_rowT, grow;
  int nwd = 1;
  i64 slab = 0;  // rows of R in one slab of the backward product's pieces

  void init(fvg_ctx* c_, DevCRS* A_, DevCRS* AT_, int k_, int ld_, const double* label_, const double* sw_,
            int icpt_, const std::vector<i64>& roff, const std::vector<i64>& doff, const std::vector<int>& planes) {
    c = c_;
    A = A_;
    AT = AT_;
    m = A->m;
    k = k_;
    ld = ld_;
    nd = (int)roff.size() - 1;
    label = label_;
    sw = sw_;
    icpt = icpt_;
    cudaStream_t s = c->stream;
    label_f.alloc(sizeof(float) * std::max<i64>(m, 1), s);
    convert_values(c, label, FVG_F64, label_f.p, FVG_F32, m);
    if (sw) {
      sw_f.alloc(sizeof(float) * std::max<i64>(m, 1), s);
      convert_values(c, sw, FVG_F64, sw_f.p, FVG_F32, m);
    }
    i64 s1b = 0, s2b = 0;
    bool f64 = false;
    for (int st : planes) f64 = f64 || st == FVG_F64;
    // the backward product gathers rows of R (ld columns): its long rows in
    // pieces listed by slabs of R that fit in L2 (48 MiB)
    slab = std::max<i64>(4096, (i64)((48ull << 20) / ((size_t)ld * (f64 ? 8 : 4))));
    for (int st : planes) {
      crs_sched(c, *A, tile_for_storage(st));  // built before any capture
      crs_sched_slabs(c, *AT, tile_for_storage(st), slab);
      s1b = std::max(s1b, spmm_scratch_bytes(c, *A, st));
      s2b = std::max(s2b, spmm_scratch_bytes(c, *AT, st, slab));
    }
    R.alloc((size_t)(f64 ? 8 : 4) * std::max<i64>(m * ld, 1), s);
    s1.alloc((size_t)s1b, s);
    s2.alloc((size_t)s2b, s);
    slots.alloc((size_t)spmm_seg_slot_bytes(c, nd, std::min(ld, 64)), s);
    std::vector<i32> sr((size_t)nd + 1);
    std::vector<i64> gr((size_t)nd);
    for (int d = 0; d <= nd; d++) sr[d] = (i32)roff[d];
    for (int d = 0; d < nd; d++) gr[d] = doff[d + 1] - 1;  // the dataset's bias row
    std::vector<i32> srT((size_t)nd + 1);  // the transposed matrix's rows: the vector rows
    for (int d = 0; d <= nd; d++) srT[d] = (i32)doff[d];
    seg_row.alloc(sizeof(i32) * (nd + 1), s);
    seg_rowT.alloc(sizeof(i32) * (nd + 1), s);
    grow.alloc(sizeof(i64) * nd, s);
    FVG_CUDA(cudaMemcpyAsync(seg_row.p, sr.data(), sizeof(i32) * (nd + 1), cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(seg_rowT.p, srT.data(), sizeof(i32) * (nd + 1), cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(grow.p, gr.data(), sizeof(i64) * nd, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    nwd = (ld + 63) / 64;
  }
  // x: weight vectors (FP64 for FP64 storage, FP32 otherwise) of all
  // datasets; bias[nd][ld]; g: gradient vectors; ev[nd][ld][2] = loss, bias
  // sum.  Nothing runs while *gate == 0; with `mask` ([nd][nwd] model bits)
  // only those models are evaluated, the others' g and ev columns keep what
  // they held.
  void eval(int storage, const void* x, const double* bias, double* g, double* ev, const int* gate,
            const unsigned long long* mask) {
    const size_t xs = storage == FVG_F64 ? 8 : 4;
    for (int c0 = 0; c0 < ld; c0 += 64) {
      const int kb = std::min(64, ld - c0);
      SpmmSeg sg;
      sg.nseg = nd;
      sg.seg_row = seg_row.as<i32>();
      sg.ldb = ld;
      sg.slots = slots.as<double>();
      sg.kout = std::max(0, std::min(kb, k - c0));
      sg.out = ev + 2 * c0;
      sg.ldo = ld;
      sg.gb = g + c0;
      sg.grow = grow.as<i64>();
      sg.ldg = ld;
      sg.gate = gate;
      sg.mask = mask;
      sg.mstride = nwd;
      sg.mword = c0 / 64;
      {
        ProfScope ps(c, P_BATCH_PASS1);
        crs_spmm_logreg_seg(c, *A, storage, (const char*)x + c0 * xs, ld, kb, label, sw, label_f.as<float>(),
                            sw ? sw_f.as<float>() : nullptr, icpt, bias + c0, (char*)R.p + c0 * xs, ld, s1.p, sg,
                            loss, eps);
      }
      {
        ProfScope ps(c, P_BATCH_PASS2);
        SpmmSeg st;
        st.nseg = nd;
        st.seg_row = seg_rowT.as<i32>();
        st.gate = gate;
        st.mask = mask;
        st.mstride = nwd;
        st.mword = c0 / 64;
        crs_spmm_store_seg(c, *AT, storage, (const char*)R.p + c0 * xs, ld, kb, g + c0, ld, s2.p, st, slab);
      }
      crs_spmm_seg_finish(c, sg);
    }
  }
};

// Ends a stream capture that an exception interrupted.
struct CaptureGuard {
  cudaStream_t s;
  bool open = false;
  ~CaptureGuard() {
    if (!open) return;
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
  }
};

}  // namespace

// weight_h: dataset d's k models from woff[d] (model j at woff[d] + j*n_d);
// b_h, n_iter_h, loss_h: [nd][k].
void lbfgs_multi_train(fvg_ctx* c, const std::vector<fvg_matrix*>& mats, const std::vector<const double*>& labels_h,
                       const std::vector<const double*>& sws_h, const fvg_glm_params* p, i64 k, const double* lam_h,
                       double* w_h, double* b_h, i64* n_iter_h, double* loss_h) {
  const int nd = (int)mats.size();
  if (nd < 1) fail(FVG_ERR_INVALID_ARG, "no datasets");
  for (int d = 0; d < nd; d++) {
    if (!mats[d]) fail(FVG_ERR_INVALID_ARG, "null matrix");
    check_common(p, mats[d], labels_h[d]);
  }
  if (k < 1 || k > kBMaxModels) fail(FVG_ERR_INVALID_ARG, "number of models must be in [1, 256]");
  if (!lam_h) fail(FVG_ERR_INVALID_ARG, "null regularisation values");
  for (i64 j = 0; j < k; j++)
    if (!(lam_h[j] >= 0)) fail(FVG_ERR_INVALID_ARG, "checkAssumption failed: regParam >= 0");
  if (p->mat_type != FVG_CRS) fail(FVG_ERR_UNSUPPORTED, "batched training runs on the CRS format");
  if (p->num_partitions > 1 || p->row_splits) fail(FVG_ERR_INVALID_ARG, "batched training takes one partition");
  if (p->hist_size < 1 || p->hist_size > kBMaxHist)
    fail(FVG_ERR_INVALID_ARG, "hist_size must be in [1, " + std::to_string(kBMaxHist) + "]");
  const int storage = p->storage;
  if (storage == FVG_SPLIT)
    fail(FVG_ERR_UNSUPPORTED, "split storage is offered by the L-BFGS trainers, single evaluations and the products");
  const bool sw_any = std::any_of(sws_h.begin(), sws_h.end(), [](const double* x) { return x != nullptr; });
  const int h = (int)p->hist_size;
  const int kk = (int)k;
  const int ld = (kk + 7) & ~7;  // whole 8-column groups of the products' lanes
  cudaStream_t s = c->stream;

  // layout: dataset d's matrix rows from roff[d], its vector rows from doff[d]
  std::vector<i64> roff((size_t)nd + 1, 0), doff((size_t)nd + 1, 0), woff((size_t)nd + 1, 0);
  for (int d = 0; d < nd; d++) {
    fvg_matrix* M = mats[d];
    roff[d + 1] = roff[d] + M->A.m;
    doff[d + 1] = doff[d] + M->A.n + 1;
    woff[d + 1] = woff[d] + M->A.n * k;
  }
  const i64 N1 = doff[nd], mtot = roff[nd];
  const bool mixed = storage != FVG_F64;
  const bool refine = storage == FVG_BF16 && p->refine;
  std::vector<int> planes{storage};
  if (refine) planes.push_back(FVG_F32);
  for (fvg_matrix* M : mats) {
    if (!M->AT) {
      M->AT.reset(new DevCRS());
      crs_build_transpose(c, M->A, *M->AT, M->master);
    }
    for (int st : planes) {
      crs_ensure_plane(c, M->A, st, M->master);
      crs_ensure_plane(c, *M->AT, st, M->master);
    }
  }
  // one dataset: its own matrix and transpose; several: the stacked copies
  DevCRS SA, SAT;
  DevCRS* A = &mats[0]->A;
  DevCRS* AT = mats[0]->AT.get();
  if (nd > 1) {
    stack_datasets(c, mats, doff, roff, planes, SA, SAT);
    A = &SA;
    AT = &SAT;
  }

  DBuf label, sw;
  label.alloc(sizeof(double) * mtot, s);
  if (sw_any) sw.alloc(sizeof(double) * mtot, s);
  for (int d = 0; d < nd; d++) {
    const i64 md = roff[d + 1] - roff[d];
    FVG_CUDA(cudaMemcpyAsync(label.as<double>() + roff[d], labels_h[d], sizeof(double) * md,
                             cudaMemcpyHostToDevice, s));
    if (!sw_any) continue;
    if (sws_h[d]) {
      FVG_CUDA(cudaMemcpyAsync(sw.as<double>() + roff[d], sws_h[d], sizeof(double) * md, cudaMemcpyHostToDevice, s));
    } else {
      std::vector<double> ones((size_t)md, 1.0);
      FVG_CUDA(cudaMemcpyAsync(sw.as<double>() + roff[d], ones.data(), sizeof(double) * md, cudaMemcpyHostToDevice, s));
      FVG_CUDA(cudaStreamSynchronize(s));
    }
  }
  BatchEval ev;
  ev.init(c, A, AT, kk, ld, label.as<double>(), sw_any ? sw.as<double>() : nullptr, p->intercept, roff, doff, planes);
  ev.loss = p->loss;
  ev.eps = p->epsilon;

  const i64 plane = N1 * ld;
  const size_t vec = sizeof(double) * (size_t)plane;
  const int nm = nd * ld;  // model states, the padding columns inactive
  DBuf W, NW, G, NG, Q, Z, STEP, S, Y, WF, B, EV, ST, part, ctl, dof, MSK;
  for (DBuf* b : {&W, &NW, &G, &NG, &Q, &Z, &STEP}) b->alloc(vec, s);
  S.alloc(vec * h, s);
  Y.alloc(vec * h, s);
  WF.alloc(sizeof(float) * (size_t)std::max<i64>(plane, 1), s);
  B.alloc(sizeof(double) * 2 * nm, s);
  EV.alloc(sizeof(double) * 2 * nm, s);
  ST.alloc(sizeof(ColState) * nm, s);
  int kp = 1;
  while (kp < kk) kp <<= 1;
  const int rpb = kBT / kp;
  i64 maxn1 = 0;
  for (int d = 0; d < nd; d++) maxn1 = std::max(maxn1, doff[d + 1] - doff[d]);
  // one wave: the column kernels are built for 4 CTAs of 256 threads per SM,
  // shared by the datasets (blockIdx.y)
  const int vgx = (int)std::max<i64>(
      1, std::min<i64>((maxn1 + rpb - 1) / rpb, std::max<i64>(1, 4 * (i64)c->num_sms / nd)));
  const dim3 vgrid((unsigned)vgx, (unsigned)nd);
  part.alloc(sizeof(double) * 2 * (size_t)vgx * kk * nd, s);
  ctl.alloc(sizeof(int) * C_NCTL + sizeof(unsigned) * (size_t)nd, s);
  dof.alloc(sizeof(i64) * (nd + 1), s);
  const int nwd = (ld + 63) / 64;
  MSK.alloc(sizeof(unsigned long long) * 2 * (size_t)nd * nwd, s);
  FVG_CUDA(cudaMemsetAsync(MSK.p, 0, sizeof(unsigned long long) * 2 * (size_t)nd * nwd, s));
  unsigned long long* smask = MSK.as<unsigned long long>();  // models searching
  unsigned long long* amask = smask + (size_t)nd * nwd;       // models active
  int* ctl_i = ctl.as<int>();
  unsigned* ticket = (unsigned*)(ctl_i + C_NCTL);
  double* B0 = B.as<double>();
  double* B1 = B0 + nm;
  for (DBuf* b : {&W, &NW, &G, &NG, &Q, &Z, &STEP}) FVG_CUDA(cudaMemsetAsync(b->p, 0, vec, s));
  FVG_CUDA(cudaMemsetAsync(S.p, 0, vec * h, s));
  FVG_CUDA(cudaMemsetAsync(Y.p, 0, vec * h, s));
  FVG_CUDA(cudaMemsetAsync(WF.p, 0, sizeof(float) * (size_t)std::max<i64>(plane, 1), s));
  FVG_CUDA(cudaMemsetAsync(EV.p, 0, sizeof(double) * 2 * nm, s));
  {
    // initial models: weight[j*n + i] -> W[i][j] (through NW as staging); per-model state
    std::vector<ColState> cs((size_t)nm);
    std::vector<double> bb((size_t)2 * nm, 0.0);
    std::vector<int> hc(C_NCTL, 0);
    int nact = 0;
    for (int d = 0; d < nd; d++) {
      const i64 nd_ = doff[d + 1] - doff[d] - 1;
      FVG_CUDA(cudaMemcpyAsync(NW.p, w_h + woff[d], sizeof(double) * (size_t)(nd_ * kk), cudaMemcpyHostToDevice, s));
      kb_to_cols<<<grid_for(c, nd_ * kk), 256, 0, s>>>(NW.as<double>(), W.as<double>() + doff[d] * ld, nd_, kk, ld);
      check_launch("kb_to_cols");
      count_launch(c);
      for (int j = 0; j < kk; j++) {
        ColState& x = cs[(size_t)d * ld + j];
        x = ColState{};
        x.lambda = lam_h[j];
        x.active = 1;
        nact++;
        bb[(size_t)d * ld + j] = b_h[(size_t)d * kk + j];
        bb[(size_t)nm + d * ld + j] = b_h[(size_t)d * kk + j];
      }
    }
    hc[C_ACTIVE] = nact;
    hc[C_ONE] = 1;
    hc[C_NEVAL] = 1;  // the initial evaluation
    hc[C_NMODEL] = nact;
    FVG_CUDA(cudaMemcpyAsync(ST.p, cs.data(), sizeof(ColState) * nm, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(B0, bb.data(), sizeof(double) * 2 * nm, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(ctl_i, hc.data(), sizeof(int) * C_NCTL, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned) * nd, s));
    FVG_CUDA(cudaMemcpyAsync(dof.p, doff.data(), sizeof(i64) * (nd + 1), cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaStreamSynchronize(s));  // the host vectors above go out of scope
  }
  FVG_CUDA(cudaMemsetAsync(NW.p, 0, vec, s));  // staging done
  BArgs a{kk, ld, kp, rpb, h, dof.as<i64>(), plane, part.as<double>(), ticket, ST.as<ColState>(), ctl_i, -1,
          nullptr, nwd};
  auto gated = [&](int w, const unsigned long long* mask = nullptr) {
    BArgs g = a;
    g.gate = w;
    g.mask = mask;
    return g;
  };
  const unsigned dg = grid_for(c, plane);

  auto weights_for = [&](int st, const double* w, const int* gate) -> const void* {
    if (st == FVG_F64) return w;
    kb_d2f<<<dg, 256, 0, s>>>(w, WF.as<float>(), plane, gate);
    check_launch("kb_d2f");
    count_launch(c);
    return WF.p;
  };
  auto norms = [&](const double* g, int accepted, int gate, const unsigned long long* mask) {
    ProfScope ps(c, P_LBFGS);
    kb_gmax<<<vgrid, kBT, 0, s>>>(g, gated(gate, mask));
    kb_gnorm<<<vgrid, kBT, 0, s>>>(g, EV.as<double>(), accepted, gated(gate, mask));
    check_launch("kb_gnorm");
    count_launch(c, 2);
  };
  const int* one = ctl_i + C_ONE;

  // the whole training as one launch sequence
  auto run = [&]() {
    ev.eval(storage, weights_for(storage, W.as<double>(), one), B0, G.as<double>(), EV.as<double>(), one, nullptr);
    norms(G.as<double>(), 1, C_ONE, nullptr);
    int rear = 0, front = 0;
    for (i64 it = 1; it <= p->num_iteration; it++) {
      const int kh = (int)std::min<i64>(it - 1, h);
      {
        ProfScope ps(c, P_LBFGS);
        for (int q = kh - 1; q >= 0; q--)
          kb_down<<<vgrid, kBT, 0, s>>>(q, kh, rear, G.as<double>(), Q.as<double>(), S.as<double>(), Y.as<double>(),
                                        gated(C_ACTIVE));
        for (int q = 0; q < kh; q++)
          kb_up<<<vgrid, kBT, 0, s>>>(q, kh, rear, Q.as<double>(), Z.as<double>(), S.as<double>(), Y.as<double>(),
                                      gated(C_ACTIVE));
        kb_step<<<vgrid, kBT, 0, s>>>(kh, rear, G.as<double>(), Z.as<double>(), STEP.as<double>(), S.as<double>(),
                                      gated(C_ACTIVE));
        kb_step_norm<<<vgrid, kBT, 0, s>>>(STEP.as<double>(), gated(C_ACTIVE));
        kb_begin_search<<<1, kBT, 0, s>>>(nd, ld, nwd, a.st, ctl_i, smask);
        check_launch("batched two-loop");
        count_launch(c, 2 * kh + 3);
      }
      for (int t = 1; t <= 10; t++) {
        {
          ProfScope ps(c, P_LBFGS);
          kb_trial<<<vgrid, kBT, 0, s>>>(t, W.as<double>(), STEP.as<double>(), NW.as<double>(),
                                         mixed ? WF.as<float>() : nullptr, B0, B1, p->reg_type, 0, p->l2_no_eta,
                                         gated(C_TRIAL));
          check_launch("kb_trial");
          count_launch(c);
        }
        const void* x = mixed ? WF.p : NW.p;
        // the models still searching only: the others keep their accepted
        // trial's loss and gradient
        ev.eval(storage, x, B1, NG.as<double>(), EV.as<double>(), ctl_i + C_EVAL_LO, smask);
        if (refine) ev.eval(FVG_F32, x, B1, NG.as<double>(), EV.as<double>(), ctl_i + C_EVAL_HI, smask);
        norms(NG.as<double>(), 0, C_TRIAL, smask);
        kb_decide<<<1, kBT, 0, s>>>(t, EV.as<double>(), nd, ld, nwd, a.st, ctl_i, smask);
        check_launch("kb_decide");
        count_launch(c);
      }
      const int nf = (kh == 0) ? 0 : (front + 1) % h;
      {
        ProfScope ps(c, P_LBFGS);
        kb_accept<<<vgrid, kBT, 0, s>>>(nf, (int)it, p->convergence_tol, W.as<double>(), G.as<double>(),
                                        NW.as<double>(), NG.as<double>(), S.as<double>(), Y.as<double>(), B0, B1,
                                        EV.as<double>(), gated(C_ACTIVE));
        kb_status<<<1, kBT, 0, s>>>(nd, ld, nwd, a.st, ctl_i, refine ? 1 : 0, p->refine_stall, amask);
        check_launch("kb_accept");
        count_launch(c, 2);
      }
      if (kh == 0) {
        rear = 0;
        front = 0;
      } else if (kh == h) {
        rear = (rear + 1) % h;
        front = nf;
      } else {
        front = nf;
      }
      if (refine) {  // re-evaluation of the accepted models right after the switch
        const int* re = ctl_i + C_REEVAL;
        ev.eval(FVG_F32, weights_for(FVG_F32, W.as<double>(), re), B0, G.as<double>(), EV.as<double>(), re, amask);
        norms(G.as<double>(), 1, C_REEVAL, amask);
        kb_clear_reeval<<<1, 32, 0, s>>>(ctl_i);
        check_launch("kb_clear_reeval");
        count_launch(c);
      }
    }
  };
  if (c->profiling) {
    run();  // per-phase timing needs the launches issued one by one
  } else {
    CaptureGuard cg{s};
    FVG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cg.open = true;
    run();
    cudaGraph_t graph = nullptr;
    cg.open = false;
    FVG_CUDA(cudaStreamEndCapture(s, &graph));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) fail(FVG_ERR_INTERNAL, std::string("graph instantiation: ") + cudaGetErrorString(ie));
    const cudaError_t le = cudaGraphLaunch(exec, s);
    const cudaError_t se = cudaStreamSynchronize(s);
    cudaGraphExecDestroy(exec);
    if (le != cudaSuccess || se != cudaSuccess)
      fail(FVG_ERR_INTERNAL, std::string("graph launch: ") + cudaGetErrorString(le != cudaSuccess ? le : se));
  }
  // results: W[i][j] -> weight[j*n + i]
  std::vector<ColState> cs((size_t)nm);
  std::vector<double> bb((size_t)nm);
  for (int d = 0; d < nd; d++) {
    const i64 nd_ = doff[d + 1] - doff[d] - 1;
    kb_from_cols<<<grid_for(c, nd_ * kk), 256, 0, s>>>(W.as<double>() + doff[d] * ld, NW.as<double>(), nd_, kk, ld);
    check_launch("kb_from_cols");
    count_launch(c);
    FVG_CUDA(cudaMemcpyAsync(w_h + woff[d], NW.p, sizeof(double) * (size_t)(nd_ * kk), cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
  }
  std::vector<int> hctl(C_NCTL);
  FVG_CUDA(cudaMemcpyAsync(cs.data(), ST.p, sizeof(ColState) * nm, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(bb.data(), B0, sizeof(double) * nm, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(hctl.data(), ctl_i, sizeof(int) * C_NCTL, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  c->batch_evals += hctl[C_NEVAL];
  c->batch_model_evals += hctl[C_NMODEL];
  for (int d = 0; d < nd; d++)
    for (int j = 0; j < kk; j++) {
      const ColState& x = cs[(size_t)d * ld + j];
      const size_t o = (size_t)d * kk + j;
      n_iter_h[o] = x.active ? p->num_iteration : x.n_iter;
      loss_h[o] = x.loss;
      b_h[o] = bb[(size_t)d * ld + j];
    }
}

void lbfgs_batched_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                         const fvg_glm_params* p, i64 k, const double* lam_h, double* w_h, double* b_h,
                         i64* n_iter_h, double* loss_h) {
  if (!M) fail(FVG_ERR_INVALID_ARG, "null matrix");
  lbfgs_multi_train(c, {M}, {label_h}, {sw_h}, p, k, lam_h, w_h, b_h, n_iter_h, loss_h);
}

}  // namespace fvg
