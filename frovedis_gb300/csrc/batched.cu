// Batched L-BFGS: k logistic-regression models trained together on one CRS
// matrix, model j with its own regularisation value and initial model and
// every other setting shared.  Each model follows lbfgs_parallelizer::
// do_train (ml/glm/lbfgs_parallelizer.hpp:267-364) with lbfgs<T>::
// compute_hkgk / update_history (ml/glm/lbfgs.hpp:79-143) exactly as the
// single-model driver does; the batch shares the matrix passes: one forward
// product A W (W num_col x k) with the logistic epilogue per (row, model) and
// one backward product A^T R per evaluation, so A is read once for all k
// models.
//
// Vectors are stored row-major with the models as columns ([n+1][k], FP64),
// so the per-model reductions of the two-loop recursion run as column
// reductions: a CTA of 256 threads covers 256/kp rows x kp columns (kp = k
// rounded up to a power of two), partial sums per (CTA, column) are combined
// in CTA order by the last CTA (deterministic).
//
// Line search: every model still searching takes its next trial; a model
// that accepted keeps its trial weights, so re-evaluating it in later trials
// of the same iteration reproduces the same loss and gradient.  A converged
// model stops (its weights are frozen) while the others continue.  The
// history ring (cir_array_list) advances identically for all active models,
// so its indices are kept on the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fvg_internal.cuh"

namespace fvg {

constexpr int kBT = 256;
constexpr int kBMaxHist = 32;
constexpr int kBMaxModels = 4096;

struct ColState {
  double rho[kBMaxHist], yy[kBMaxHist], al[kBMaxHist], beta[kBMaxHist];
  double factor[12];
  double dot_gs, smax, stepsize, flip, bstep;
  double loss;                  // accepted loss
  double gmax, gnorm, rms;      // of the accepted gradient
  double gmax_t, gnorm_t, rms_t;  // of the last evaluated gradient
  double lambda;
  int active, searching, trials, n_iter;
};

struct BArgs {
  i64 n, n1;
  int k, kp, rpb, h;
  double* part;
  unsigned* ticket;
  ColState* st;
};

// Fixed-order reduction of NV values per column; fin(j, totals) runs once
// per column in the last CTA.
template <int NV, class Fin>
__device__ __forceinline__ void col_reduce(double (&v)[NV], const bool (&is_max)[NV], const BArgs& a, Fin fin) {
  __shared__ double sm[NV][kBT];
  __shared__ bool last;
  const int j = threadIdx.x % a.kp, rr = threadIdx.x / a.kp;
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
    for (int q = 0; q < NV; q++) a.part[((i64)blockIdx.x * a.k + j) * NV + q] = sm[q][threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(a.ticket, 1u) == gridDim.x - 1);
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
        for (int q = 0; q < NV; q++) x[u][q] = __ldcg(&a.part[((b + u * a.rpb) * a.k + j) * NV + q]);
#pragma unroll
      for (int u = 0; u < 8; u++)
#pragma unroll
        for (int q = 0; q < NV; q++) t[q] = is_max[q] ? fmax(t[q], x[u][q]) : t[q] + x[u][q];
    }
    for (; b < gridDim.x; b += a.rpb)
#pragma unroll
      for (int q = 0; q < NV; q++) {
        const double x = __ldcg(&a.part[(b * a.k + j) * NV + q]);
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
  if (threadIdx.x == 0) *a.ticket = 0u;
}

// thread -> (column j, first row r0); rows advance by rpb * gridDim
#define BCOL                                   \
  const int j = threadIdx.x % a.kp;            \
  const int rr = threadIdx.x / a.kp;           \
  const bool on = j < a.k;                     \
  const i64 rstep = (i64)gridDim.x * a.rpb;    \
  const i64 r0 = (i64)blockIdx.x * a.rpb + rr
// The rows of a column in groups of U: every load of a group is issued
// before the first use, so a thread keeps U row-loads in flight (the column
// kernels stream 256 MB planes and are bound by memory-level parallelism).
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
  const bool act = on && a.st[j].active;
  const bool first = (i == kh - 1);
  const i64 plane = a.n1 * a.k;
  const double* Si = S + hslot(rear, i, a.h) * plane;
  const double* Yp = Y + hslot(rear, i + 1, a.h) * plane;
  const double alp = (act && !first) ? a.st[j].al[i + 1] : 0.0;
  double v[1] = {0.0};
  const int k = a.k;
  if (act && first)
    rows_grouped<kRowGroup>(r0, rstep, a.n1, [&](i64 r) { const i64 e = r * k + j; return V2{G[e], Si[e]}; },
                            [&](i64 r, const V2& x) {
                              Q[r * k + j] = x.a;
                              v[0] += x.b * x.a;
                            });
  else if (act)
    rows_grouped<kRowGroup>(r0, rstep, a.n1,
                            [&](i64 r) { const i64 e = r * k + j; return V3{Q[e], Yp[e], Si[e]}; },
                            [&](i64 r, const V3& x) {
                              const double q = __dsub_rn(x.a, __dmul_rn(x.b, alp));
                              Q[r * k + j] = q;
                              v[0] += x.c * q;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[c];
    if (s.active) s.al[i] = s.rho[hslot(rear, i, a.h)] * t[0];
  });
}

// second loop (as in the single-model k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_up(int i, int kh, int rear, const double* __restrict__ Q,
                                             double* __restrict__ Z, const double* __restrict__ S,
                                             const double* __restrict__ Y, BArgs a) {
  BCOL;
  const bool act = on && a.st[j].active;
  const i64 plane = a.n1 * a.k;
  const double* Yi = Y + hslot(rear, i, a.h) * plane;
  const double* Sp = S + hslot(rear, i > 0 ? i - 1 : 0, a.h) * plane;
  double H0 = 0.0, f = 0.0, al0 = 0.0;
  if (act) {
    const ColState& s = a.st[j];
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
  const int k = a.k;
  if (act && i == 0)
    rows_grouped<kRowGroup>(r0, rstep, a.n1, [&](i64 r) { const i64 e = r * k + j; return V2{Q[e], Yi[e]}; },
                            [&](i64 r, const V2& x) {
                              const double z = __dmul_rn(__dsub_rn(x.a, __dmul_rn(x.b, al0)), H0);
                              Z[r * k + j] = z;
                              v[0] += x.b * z;
                            });
  else if (act)
    rows_grouped<kRowGroup>(r0, rstep, a.n1,
                            [&](i64 r) { const i64 e = r * k + j; return V3{Z[e], Sp[e], Yi[e]}; },
                            [&](i64 r, const V3& x) {
                              const double z = __dadd_rn(x.a, __dmul_rn(x.b, f));
                              Z[r * k + j] = z;
                              v[0] += x.c * z;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[c];
    if (s.active) s.beta[i] = s.rho[hslot(rear, i, a.h)] * t[0];
  });
}

// step = -z, or the no-history step (as in k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_step(int kh, int rear, const double* __restrict__ G,
                                               const double* __restrict__ Z, double* __restrict__ STEP,
                                               const double* __restrict__ S, BArgs a) {
  BCOL;
  const bool act = on && a.st[j].active;
  const double* Sp = S + hslot(rear, kh > 0 ? kh - 1 : 0, a.h) * (a.n1 * a.k);
  double c = 0.0, f = 0.0;
  if (act) {
    const ColState& s = a.st[j];
    if (kh == 0) {
      double gn = s.gnorm;
      if (gn > 1) gn = 1.0 / gn;
      c = __dmul_rn(-gn, 0.1);
    } else {
      f = s.al[kh - 1] - s.beta[kh - 1];
    }
  }
  double v[2] = {0.0, 0.0};
  const int k = a.k;
  if (act)
    rows_grouped<kRowGroup>(r0, rstep, a.n1,
                            [&](i64 r) {
                              const i64 e = r * k + j;
                              return kh == 0 ? V3{G[e], 0.0, 0.0} : V3{G[e], Z[e], Sp[e]};
                            },
                            [&](i64 r, const V3& x) {
                              const double z = (kh == 0) ? __dmul_rn(c, x.a) : __dadd_rn(x.b, __dmul_rn(x.c, f));
                              const double st = -z;
                              STEP[r * k + j] = st;
                              v[0] += x.a * st;
                              v[1] = fmax(v[1], fabs(st));
                            });
  const bool mx[2] = {false, true};
  col_reduce<2>(v, mx, a, [&](int c2, double* t) {
    ColState& s = a.st[c2];
    if (!s.active) return;
    s.dot_gs = t[0];
    s.smax = t[1];
  });
}

// max-scaled step norm, uphill flip, factors of the 10 trials (as in k_direction)
__global__ void __launch_bounds__(kBT, 4) kb_step_norm(const double* __restrict__ STEP, BArgs a) {
  BCOL;
  const bool act = on && a.st[j].active;
  const double mxv = act ? a.st[j].smax : 0.0;
  const double inv = mxv == 0 ? 0.0 : 1.0 / mxv;
  double v[1] = {0.0};
  const int k = a.k;
  if (act)
    rows_grouped<kRowGroup>(r0, rstep, a.n1, [&](i64 r) { return STEP[r * k + j]; },
                            [&](i64, double x) {
                              const double t = x * inv;
                              v[0] += t * t;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[c];
    if (!s.active) return;
    const double m = s.smax;
    const double ss = (m == 0) ? 0.0 : sqrt(t[0]) * m;
    s.stepsize = ss;
    s.flip = (s.dot_gs > 0) ? -1.0 : 1.0;
    double fac = 1.0;
    if (fac * ss > 1e20) fac = 1e20 / ss;
    s.factor[1] = fac;
    for (int q = 2; q <= 10; q++) s.factor[q] = s.factor[q - 1] / 10.0;
    s.bstep = STEP[(a.n1 - 1) * a.k + c] * s.flip;
  });
}

// models still searching: trial model + regulariser (see k_trial)
__global__ void __launch_bounds__(kBT, 4) kb_trial(int t, const double* __restrict__ W, const double* __restrict__ STEP,
                                                double* __restrict__ NW, float* __restrict__ NWF,
                                                const double* __restrict__ B0, double* __restrict__ B1, int rtype,
                                                int eta_one, int no_eta, BArgs a) {
  BCOL;
  if (!on) return;
  const ColState& s = a.st[j];
  if (!s.searching) return;
  const double f = s.factor[t], fl = s.flip, lambda = s.lambda;
  const double eta = eta_one ? 1.0 : f;
  const double scale = fmax(0.0, 1.0 - (lambda * eta));
  const int k = a.k;
  rows_grouped<kRowGroup>(r0, rstep, a.n, [&](i64 r) { const i64 e = r * k + j; return V2{W[e], STEP[e]}; },
                          [&](i64 r, const V2& x) {
                            const i64 e = r * k + j;
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
  if (r0 == 0) B1[j] = __dadd_rn(B0[j], __dmul_rn(f, s.bstep));
}

__global__ void __launch_bounds__(kBT, 4) kb_gmax(const double* __restrict__ G, BArgs a) {
  BCOL;
  double v[1] = {0.0};
  const int k = a.k;
  if (on)
    rows_grouped<kRowGroup>(r0, rstep, a.n1, [&](i64 r) { return G[r * k + j]; },
                            [&](i64, double x) { v[0] = fmax(v[0], fabs(x)); });
  const bool mx[1] = {true};
  col_reduce<1>(v, mx, a, [&](int c, double* t) { a.st[c].gmax_t = t[0]; });
}

// gradient norm and rms; `accepted`: the evaluation is of the accepted
// model (the initial one, or the re-evaluation after a precision switch)
__global__ void __launch_bounds__(kBT, 4) kb_gnorm(const double* __restrict__ G, const double* __restrict__ EV,
                                                int accepted, BArgs a) {
  BCOL;
  const double mxv = on ? a.st[j].gmax_t : 0.0;
  const double inv = mxv == 0 ? 0.0 : 1.0 / mxv;
  double v[1] = {0.0};
  const int k = a.k;
  if (on)
    rows_grouped<kRowGroup>(r0, rstep, a.n1, [&](i64 r) { return G[r * k + j]; },
                            [&](i64, double x) {
                              const double t = x * inv;
                              v[0] += t * t;
                            });
  const bool mx[1] = {false};
  col_reduce<1>(v, mx, a, [&](int c, double* t) {
    ColState& s = a.st[c];
    const double m = s.gmax_t;
    const double nrm = (m == 0) ? 0.0 : sqrt(t[0]) * m;
    s.gnorm_t = nrm;
    s.rms_t = nrm / sqrt((double)a.n1);
    if (accepted && s.active) {
      s.gnorm = nrm;
      s.rms = s.rms_t;
      s.gmax = m;
      s.loss = EV[2 * c];
    }
  });
}

// accept decision of trial t (LBFGS_SEARCH_TOL, lbfgs_parallelizer.hpp:
// 155, 329; the 10th trial is taken whatever its loss); ctl[0] = models
// still searching
__global__ void __launch_bounds__(kBT, 4) kb_decide(int t, const double* __restrict__ EV, int k, ColState* st,
                                                 int* ctl) {
  __shared__ int cnt[kBT];
  int n = 0;
  for (int j = threadIdx.x; j < k; j += kBT) {
    ColState& s = st[j];
    if (!s.searching) continue;
    if (EV[2 * j] - s.loss < 1e-4 || t == 10) {
      s.searching = 0;
      s.trials = t;
    } else {
      n++;
    }
  }
  cnt[threadIdx.x] = n;
  __syncthreads();
  for (int s = kBT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) cnt[threadIdx.x] += cnt[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) ctl[0] = cnt[0];
}

__global__ void __launch_bounds__(kBT, 4) kb_begin_search(int k, ColState* st) {
  for (int j = threadIdx.x; j < k; j += kBT) st[j].searching = st[j].active;
}

// accept + history push (see k_accept); convergence: rms <= tol stops the model
__global__ void __launch_bounds__(kBT, 4) kb_accept(int nf, int it, double tol, double* __restrict__ W,
                                                 double* __restrict__ G, const double* __restrict__ NW,
                                                 const double* __restrict__ NG, double* __restrict__ S,
                                                 double* __restrict__ Y, double* __restrict__ B0,
                                                 const double* __restrict__ B1, const double* __restrict__ EV,
                                                 BArgs a) {
  BCOL;
  const bool act = on && a.st[j].active;
  const i64 plane = a.n1 * a.k;
  double* Sn = S + (i64)nf * plane;
  double* Yn = Y + (i64)nf * plane;
  const double bn = act ? B1[j] : 0.0, bo = act ? B0[j] : 0.0;
  double v[2] = {0.0, 0.0};
  const int k = a.k;
  const i64 n = a.n;
  if (act)  // four planes read per row: groups of two rows keep it within 64 registers
    rows_grouped<2>(r0, rstep, a.n1,
                    [&](i64 r) {
                      const i64 e = r * k + j;
                      return (r < n) ? V4{NW[e], W[e], NG[e], G[e]} : V4{bn, bo, NG[e], G[e]};
                    },
                    [&](i64 r, const V4& x) {
                      const i64 e = r * k + j;
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
    ColState& s = a.st[c];
    if (!s.active) return;
    double dv = t[0];
    if (dv == 0) dv = 1;
    s.rho[nf] = 1.0 / dv;
    s.yy[nf] = t[1];
    s.loss = EV[2 * c];
    B0[c] = B1[c];
    s.gnorm = s.gnorm_t;
    s.rms = s.rms_t;
    if (s.rms_t <= tol) {
      s.active = 0;
      s.n_iter = it;
    }
  });
}

// ctl[1] = active models; rms[j] = rms of model j's last gradient, -1 once
// the model has stopped
__global__ void __launch_bounds__(kBT, 4) kb_status(int k, const ColState* st, int* ctl, double* rms) {
  __shared__ int cnt[kBT];
  int n = 0;
  for (int j = threadIdx.x; j < k; j += kBT) {
    n += st[j].active;
    rms[j] = st[j].active ? st[j].rms_t : -1.0;
  }
  cnt[threadIdx.x] = n;
  __syncthreads();
  for (int s = kBT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) cnt[threadIdx.x] += cnt[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) ctl[1] = cnt[0];
}

// model-major [k][n] <-> column layout [n+1][k] (row n, the bias slot, is
// left untouched by the forward copy)
__global__ void kb_to_cols(const double* __restrict__ src, double* __restrict__ dst, i64 n, int k) {
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (i64)gridDim.x * blockDim.x) {
    const i64 i = e / k;
    const int j = (int)(e - i * k);
    dst[e] = src[(i64)j * n + i];
  }
}
__global__ void kb_from_cols(const double* __restrict__ src, double* __restrict__ dst, i64 n, int k) {
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (i64)gridDim.x * blockDim.x) {
    const int j = (int)(e / n);
    const i64 i = e - (i64)j * n;
    dst[e] = src[i * k + j];
  }
}

__global__ void kb_d2f(const double* __restrict__ s, float* __restrict__ d, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) d[i] = (float)s[i];
}

// ------------------------------------------------------------ host driver
struct BatchEval {
  fvg_ctx* c = nullptr;
  DevCRS* A = nullptr;
  DevCRS* AT = nullptr;
  i64 m = 0, n = 0;
  int k = 0, storage = FVG_F64, icpt = 0, master = FVG_F64;
  int loss = 0;      // GLM loss kind shared by the models
  double eps = 0.0;
  const double* label = nullptr;
  const double* sw = nullptr;
  DBuf label_f, sw_f, R, s1, s2;

  void init(fvg_ctx* c_, fvg_matrix* M, int storage_, int k_, const double* label_, const double* sw_, int icpt_) {
    c = c_;
    A = &M->A;
    AT = M->AT.get();
    master = M->master;
    m = A->m;
    n = A->n;
    k = k_;
    label = label_;
    sw = sw_;
    icpt = icpt_;
    label_f.alloc(sizeof(float) * std::max<i64>(m, 1), c->stream);
    convert_values(c, label, FVG_F64, label_f.p, FVG_F32, m);
    if (sw) {
      sw_f.alloc(sizeof(float) * std::max<i64>(m, 1), c->stream);
      convert_values(c, sw, FVG_F64, sw_f.p, FVG_F32, m);
    }
    set_storage(storage_);
  }
  void set_storage(int st) {
    storage = st;
    crs_ensure_plane(c, *A, storage, master);
    crs_ensure_plane(c, *AT, storage, master);
    R.alloc((size_t)(storage == FVG_F64 ? 8 : 4) * std::max<i64>(m * k, 1), c->stream);
    s1.alloc((size_t)spmm_scratch_bytes(c, *A, storage), c->stream);
    s2.alloc((size_t)spmm_scratch_bytes(c, *AT, storage), c->stream);
  }
  // x: weights [n][k] (FP64 for FP64 storage, FP32 otherwise); bias[k];
  // g[n+1][k]; ev[k][2] = loss, bias sum
  void eval(const void* x, const double* bias, double* g, double* ev) {
    const size_t xs = storage == FVG_F64 ? 8 : 4;
    for (int c0 = 0; c0 < k; c0 += 64) {
      const int kb = std::min(64, k - c0);
      {
        ProfScope ps(c, P_BATCH_PASS1);
        crs_spmm_logreg_block(c, *A, storage, (const char*)x + c0 * xs, k, kb, label, sw, label_f.as<float>(),
                              sw ? sw_f.as<float>() : nullptr, icpt, bias + c0, (char*)R.p + c0 * xs, k, ev + 2 * c0,
                              g + n * k + c0, s1.p, loss, eps);
      }
      ProfScope ps(c, P_BATCH_PASS2);
      crs_spmm_block(c, *AT, storage, (const char*)R.p + c0 * xs, k, kb, FVG_F64, g + c0, k, s2.p);
    }
  }
};

struct Pinned {
  void* p = nullptr;
  explicit Pinned(size_t b) { FVG_CUDA(cudaMallocHost(&p, b)); }
  ~Pinned() { if (p) cudaFreeHost(p); }
};

void lbfgs_batched_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                         const fvg_glm_params* p, i64 k, const double* lam_h, double* w_h, double* b_h,
                         i64* n_iter_h, double* loss_h) {
  check_common(p, M, label_h);
  if (k < 1 || k > kBMaxModels) fail(FVG_ERR_INVALID_ARG, "number of models must be in [1, 4096]");
  if (!lam_h) fail(FVG_ERR_INVALID_ARG, "null regularisation values");
  for (i64 j = 0; j < k; j++)
    if (!(lam_h[j] >= 0)) fail(FVG_ERR_INVALID_ARG, "checkAssumption failed: regParam >= 0");
  if (p->mat_type != FVG_CRS) fail(FVG_ERR_UNSUPPORTED, "batched training runs on the CRS format");
  if (p->num_partitions > 1 || p->row_splits) fail(FVG_ERR_INVALID_ARG, "batched training takes one partition");
  if (p->hist_size < 1 || p->hist_size > kBMaxHist)
    fail(FVG_ERR_INVALID_ARG, "hist_size must be in [1, " + std::to_string(kBMaxHist) + "]");
  const i64 m = M->A.m, n = M->A.n, n1 = n + 1;
  const int h = (int)p->hist_size;
  const int kk = (int)k;
  cudaStream_t s = c->stream;
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
  int storage = p->storage;
  if (storage == FVG_SPLIT) fail(FVG_ERR_UNSUPPORTED, "split storage is offered by the L-BFGS trainers, single evaluations and the products");
  const bool mixed = storage != FVG_F64;

  DBuf label, sw;
  label.alloc(sizeof(double) * m, s);
  FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  BatchEval ev;
  ev.init(c, M, storage, kk, label.as<double>(), sw_h ? sw.as<double>() : nullptr, p->intercept);
  ev.loss = p->loss;
  ev.eps = p->epsilon;

  const size_t vec = sizeof(double) * (size_t)n1 * kk;
  DBuf W, NW, G, NG, Q, Z, STEP, S, Y, WF, B, EV, ST, part, ctl;
  for (DBuf* b : {&W, &NW, &G, &NG, &Q, &Z, &STEP}) b->alloc(vec, s);
  S.alloc(vec * h, s);
  Y.alloc(vec * h, s);
  WF.alloc(sizeof(float) * (size_t)std::max<i64>(n * kk, 1), s);
  B.alloc(sizeof(double) * 2 * kk, s);
  EV.alloc(sizeof(double) * 2 * kk, s);
  ST.alloc(sizeof(ColState) * kk, s);
  int kp = 1;
  while (kp < kk && kp < kBT) kp <<= 1;
  if (kk > kBT) fail(FVG_ERR_INVALID_ARG, "at most 256 models per batch");
  const int rpb = kBT / kp;
  // one wave: the column kernels are built for 4 CTAs of 256 threads per SM
  const int vgrid = (int)std::max<i64>(1, std::min<i64>((n1 + rpb - 1) / rpb, 4 * (i64)c->num_sms));
  part.alloc(sizeof(double) * 2 * (size_t)vgrid * kk + 256, s);
  ctl.alloc(256 + sizeof(double) * kk, s);
  unsigned* ticket = (unsigned*)((char*)part.p + sizeof(double) * 2 * (size_t)vgrid * kk);
  FVG_CUDA(cudaMemsetAsync(ticket, 0, 256, s));
  int* ctl_i = ctl.as<int>();
  double* rms_d = (double*)((char*)ctl.p + 256);
  double* B0 = B.as<double>();
  double* B1 = B0 + kk;

  const unsigned dg = (unsigned)std::max<i64>(1, std::min<i64>((n * kk + 255) / 256, 4 * (i64)c->num_sms));
  // initial models: weight[j*n + i] -> W[i][j] (through NW as staging); per-model state
  {
    FVG_CUDA(cudaMemcpyAsync(NW.p, w_h, sizeof(double) * (size_t)n * kk, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemsetAsync(W.p, 0, vec, s));
    kb_to_cols<<<dg, 256, 0, s>>>(NW.as<double>(), W.as<double>(), n, kk);
    check_launch("kb_to_cols");
    count_launch(c);
    std::vector<ColState> cs((size_t)kk);
    for (int j = 0; j < kk; j++) {
      cs[j] = ColState{};
      cs[j].lambda = lam_h[j];
      cs[j].active = 1;
    }
    FVG_CUDA(cudaMemcpyAsync(ST.p, cs.data(), sizeof(ColState) * kk, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(B0, b_h, sizeof(double) * kk, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(B1, b_h, sizeof(double) * kk, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaStreamSynchronize(s));  // the host vectors above go out of scope
  }
  BArgs a{n, n1, kk, kp, rpb, h, part.as<double>(), ticket, ST.as<ColState>()};
  Pinned hp(256 + sizeof(double) * kk);
  int* hctl = (int*)hp.p;
  double* hrms = (double*)((char*)hp.p + 256);

  auto weights_for = [&](const double* w) -> const void* {
    if (!mixed) return w;
    kb_d2f<<<dg, 256, 0, s>>>(w, WF.as<float>(), n * kk);
    check_launch("kb_d2f");
    count_launch(c);
    return WF.p;
  };
  auto norms = [&](const double* g, int accepted) {
    ProfScope ps(c, P_LBFGS);
    kb_gmax<<<vgrid, kBT, 0, s>>>(g, a);
    kb_gnorm<<<vgrid, kBT, 0, s>>>(g, EV.as<double>(), accepted, a);
    check_launch("kb_gnorm");
    count_launch(c, 2);
  };

  ev.eval(weights_for(W.as<double>()), B0, G.as<double>(), EV.as<double>());
  norms(G.as<double>(), 1);

  const bool ell = false;
  int rear = 0, front = 0;
  std::vector<std::vector<double>> rms_hist((size_t)kk);
  i64 it = 1;
  for (; it <= p->num_iteration; it++) {
    const int kh = (int)std::min<i64>(it - 1, h);
    {
      ProfScope ps(c, P_LBFGS);
      for (int q = kh - 1; q >= 0; q--)
        kb_down<<<vgrid, kBT, 0, s>>>(q, kh, rear, G.as<double>(), Q.as<double>(), S.as<double>(), Y.as<double>(),
                                      a);
      for (int q = 0; q < kh; q++)
        kb_up<<<vgrid, kBT, 0, s>>>(q, kh, rear, Q.as<double>(), Z.as<double>(), S.as<double>(), Y.as<double>(), a);
      kb_step<<<vgrid, kBT, 0, s>>>(kh, rear, G.as<double>(), Z.as<double>(), STEP.as<double>(), S.as<double>(), a);
      kb_step_norm<<<vgrid, kBT, 0, s>>>(STEP.as<double>(), a);
      kb_begin_search<<<1, kBT, 0, s>>>(kk, a.st);
      check_launch("batched two-loop");
      count_launch(c, 2 * kh + 3);
    }
    for (int t = 1; t <= 10; t++) {
      {
        ProfScope ps(c, P_LBFGS);
        kb_trial<<<vgrid, kBT, 0, s>>>(t, W.as<double>(), STEP.as<double>(), NW.as<double>(),
                                       mixed ? WF.as<float>() : nullptr, B0, B1, p->reg_type, ell ? 1 : 0,
                                       p->l2_no_eta, a);
        check_launch("kb_trial");
        count_launch(c);
      }
      ev.eval(mixed ? WF.p : NW.p, B1, NG.as<double>(), EV.as<double>());
      norms(NG.as<double>(), 0);
      kb_decide<<<1, kBT, 0, s>>>(t, EV.as<double>(), kk, a.st, ctl_i);
      check_launch("kb_decide");
      count_launch(c);
      FVG_CUDA(cudaMemcpyAsync(hctl, ctl_i, sizeof(int), cudaMemcpyDeviceToHost, s));
      FVG_CUDA(cudaStreamSynchronize(s));
      if (hctl[0] == 0) break;
    }
    const int nf = (kh == 0) ? 0 : (front + 1) % h;
    {
      ProfScope ps(c, P_LBFGS);
      kb_accept<<<vgrid, kBT, 0, s>>>(nf, (int)it, p->convergence_tol, W.as<double>(), G.as<double>(),
                                      NW.as<double>(), NG.as<double>(), S.as<double>(), Y.as<double>(), B0, B1,
                                      EV.as<double>(), a);
      kb_status<<<1, kBT, 0, s>>>(kk, a.st, ctl_i, rms_d);
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
    FVG_CUDA(cudaMemcpyAsync(hctl, ctl_i, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaMemcpyAsync(hrms, rms_d, sizeof(double) * kk, cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    if (hctl[1] == 0) break;
    // refinement (see the single-model driver): leave BF16 values for FP32
    // once any model's gradient norm stalls
    if (mixed && storage == FVG_BF16 && p->refine) {
      bool stall = false;
      for (int j = 0; j < kk; j++) {
        if (hrms[j] < 0) continue;  // stopped
        auto& hh = rms_hist[j];
        hh.push_back(hrms[j]);
        if (hh.size() >= 4) {
          const double best = *std::min_element(hh.end() - 4, hh.end() - 1);
          if (hrms[j] > p->refine_stall * best) stall = true;
        }
      }
      if (stall) {
        storage = FVG_F32;
        ev.set_storage(storage);
        ev.eval(weights_for(W.as<double>()), B0, G.as<double>(), EV.as<double>());
        norms(G.as<double>(), 1);
      }
    }
  }
  // results: W[i][j] -> weight[j*n + i]
  kb_from_cols<<<dg, 256, 0, s>>>(W.as<double>(), NW.as<double>(), n, kk);
  check_launch("kb_from_cols");
  count_launch(c);
  std::vector<ColState> cs((size_t)kk);
  FVG_CUDA(cudaMemcpyAsync(w_h, NW.p, sizeof(double) * (size_t)n * kk, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(cs.data(), ST.p, sizeof(ColState) * kk, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(b_h, B0, sizeof(double) * kk, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  for (i64 j = 0; j < k; j++) {
    n_iter_h[j] = cs[j].active ? p->num_iteration : cs[j].n_iter;
    loss_h[j] = cs[j].loss;
  }
}

}  // namespace fvg
