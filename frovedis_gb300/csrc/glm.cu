// Logistic-regression drivers on the device.
//
// L-BFGS: lbfgs_parallelizer::do_train (ml/glm/lbfgs_parallelizer.hpp:
// 267-364 with the transposed copy, 366-462 for ELL) with lbfgs<T>::
// compute_hkgk / update_history (ml/glm/lbfgs.hpp:79-143) and the ring buffer
// of matrix/cir_array_list.hpp.  All model, gradient and history vectors stay
// on the device in FP64; every reduction is a fixed-order grid reduction (the
// last CTA to finish combines the per-CTA partials in CTA order), so runs are
// deterministic.  Element-wise updates use round-to-nearest intrinsics so no
// multiply-add is contracted where the reference rounds twice.  The host only
// reads three scalars per line-search trial (new loss, loss, rms) to take the
// accept decision the reference takes on rank 0.
//
// SGD: sgd_parallelizer::do_train_with_trans (ml/glm/sgd_parallelizer.hpp:
// 132-255) with gradient_descent::optimize / update_model (gradient_descent.hpp:
// 128-164, 242-259); P ranks are emulated as P row blocks whose model deltas
// are summed in rank order.
#include <algorithm>
#include <cmath>

#include "fvg_internal.cuh"

namespace fvg {

constexpr int kMaxHist = 64;
constexpr int kVecThreads = 256;

struct LbState {
  int k, rear, front, h;
  double rho[kMaxHist], yy[kMaxHist], al[kMaxHist], beta[kMaxHist];
  double factor[12];
  double dot_gs, smax, stepsize, flip, bstep;
  double loss;      // accepted loss
  double eval[2];   // last evaluation: loss, bias
  double b[2];      // [0] accepted intercept, [1] trial intercept
  double gmax, gnorm, rms;              // of the accepted gradient
  double gmax_t, gnorm_t, rms_t;        // of the last trial gradient
  double host[4];   // newloss, loss, rms_t, factor of the last trial (read back)
};

struct VecArgs {
  i64 n;   // weights
  i64 n1;  // n + 1
  int h;
  double* part;
  unsigned* ticket;
  LbState* st;
};

__device__ __forceinline__ int slot(const LbState* st, int i) { return (st->rear + i) % st->h; }

// Fixed-order grid reduction of NV values (sum or max per value); the last
// CTA calls fin(totals) with thread 0.
template <int NV, class Fin>
__device__ __forceinline__ void grid_reduce(double (&v)[NV], const bool (&is_max)[NV], double* part,
                                            unsigned* ticket, Fin fin) {
  __shared__ double sm[NV][kVecThreads];
  __shared__ bool last;
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int st = kVecThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
#pragma unroll
      for (int q = 0; q < NV; q++)
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + st])
                                       : sm[q][threadIdx.x] + sm[q][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) part[(i64)blockIdx.x * NV + q] = sm[q][0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  double t[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) t[q] = 0.0;
  for (i64 b = threadIdx.x; b < gridDim.x; b += kVecThreads)
#pragma unroll
    for (int q = 0; q < NV; q++) {
      double x = __ldcg(&part[b * NV + q]);
      t[q] = is_max[q] ? fmax(t[q], x) : t[q] + x;
    }
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = t[q];
  __syncthreads();
  for (int st = kVecThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
#pragma unroll
      for (int q = 0; q < NV; q++)
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + st])
                                       : sm[q][threadIdx.x] + sm[q][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double tot[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) tot[q] = sm[q][0];
    fin(tot);
    *ticket = 0u;
  }
}

#define VEC_LOOP(j, n) for (i64 j = (i64)blockIdx.x * kVecThreads + threadIdx.x; j < (n); j += (i64)gridDim.x * kVecThreads)

// ---------------------------------------------------- L-BFGS direction
// The whole direction in one cooperative launch: the two loops of
// compute_hkgk (lbfgs.hpp:79-112) —
//   first loop, i = k-1 .. 0:  al[i] = rho[i] * (s_i · q);  q -= y_i * al[i]
//   second loop, i = 0 .. k-1: beta = rho[i] * (y_i · z);  z += s_i * (al[i] - beta)
//   (z = q * H0 before it, H0 = (1/rho) / (y·y) of the newest pair)
// — then step = -z (or the no-history step z = -c * 0.1 * g with
// c = |g| <= 1 ? |g| : 1/|g|, lbfgs.hpp:86-91), g·step, max|step| and the
// max-scaled step norm (vector_operations.hpp:227-264) with the uphill flip,
// the 1e20 factor cap and the factors of the 10 trials.  Each update of q
// (z) is applied in the same pass as the next dot product.  Where a dot
// product must be complete the CTAs meet at a grid barrier; every CTA then
// adds all CTAs' partial sums in the same fixed order, so each holds the same
// value and no second barrier is needed.  Partial-sum slots alternate
// between two buffers: a CTA may write the next step's partials while slower
// CTAs still read this step's.  Each thread always handles the same elements,
// so the vectors it reads back were written by itself.
struct DirArgs {
  const double* G;
  double* Q;
  double* Z;
  double* STEP;
  const double* S;
  const double* Y;
  VecArgs a;
  double* part;              // [2][2 * gridDim.x]
  unsigned long long* bar;   // barrier arrivals, zeroed before the launch
  unsigned* err;
  unsigned limit;            // poll budget of each barrier wait
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier `b` of this launch.  The wait is bounded: a CTA that gives up
// sets the error word and stops waiting at later barriers (the results are
// then garbage and the call reports the error).
__device__ __forceinline__ void dir_sync(const DirArgs& d, int b, bool* dead) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(d.bar, 1ull);
    const unsigned long long target = (unsigned long long)gridDim.x * (unsigned long long)(b + 1);
    if (!*dead) {
      for (unsigned it = 0; ld_acquire_u64(d.bar) < target; it++) {
        if (it >= d.limit) {
          atomicOr(d.err, 4u);
          *dead = true;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

constexpr int kDirThreads = 256;  // (one CTA of 1024 per SM measured slower)
#define DIR_LOOP(j, n) for (i64 j = (i64)blockIdx.x * kDirThreads + threadIdx.x; j < (n); j += (i64)gridDim.x * kDirThreads)

// CTA partials of NV values (sum, or max where is_max) into slot[blockIdx.x * NV + q]
template <int NV>
__device__ __forceinline__ void dir_partial(double (&v)[NV], const bool (&is_max)[NV], double* slot,
                                            double (*sm)[kDirThreads]) {
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int st = kDirThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
#pragma unroll
      for (int q = 0; q < NV; q++)
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + st])
                                       : sm[q][threadIdx.x] + sm[q][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NV; q++) slot[(i64)blockIdx.x * NV + q] = sm[q][0];
}

// every CTA: the totals of all CTAs' partials, in a fixed order, into tot
template <int NV>
__device__ __forceinline__ void dir_total(const double* slot, const bool (&is_max)[NV], double (&tot)[NV],
                                          double (*sm)[kDirThreads]) {
  double t[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) t[q] = 0.0;
  for (i64 b = threadIdx.x; b < gridDim.x; b += kDirThreads)
#pragma unroll
    for (int q = 0; q < NV; q++) {
      const double x = __ldcg(&slot[b * NV + q]);
      t[q] = is_max[q] ? fmax(t[q], x) : t[q] + x;
    }
  __syncthreads();  // sm is free (the partial's reads are done)
#pragma unroll
  for (int q = 0; q < NV; q++) sm[q][threadIdx.x] = t[q];
  __syncthreads();
  for (int st = kDirThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
#pragma unroll
      for (int q = 0; q < NV; q++)
        sm[q][threadIdx.x] = is_max[q] ? fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + st])
                                       : sm[q][threadIdx.x] + sm[q][threadIdx.x + st];
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < NV; q++) tot[q] = sm[q][0];
  __syncthreads();
}

__global__ void __launch_bounds__(kDirThreads) k_direction(DirArgs d) {
  const VecArgs a = d.a;
  LbState* st = a.st;
  const int k = st->k;
  __shared__ double sm[2][kDirThreads];
  __shared__ double s_al[kMaxHist], s_beta[kMaxHist];
  __shared__ bool dead;
  if (threadIdx.x == 0) dead = false;
  const bool lead = (blockIdx.x == 0 && threadIdx.x == 0);
  const i64 G2 = 2 * (i64)gridDim.x;
  int b = 0;
  const bool sum1[1] = {false};
  // first loop
  for (int i = k - 1; i >= 0; i--, b++) {
    const bool first = (i == k - 1);
    const double* Si = d.S + (i64)slot(st, i) * a.n1;
    const double* Yp = first ? nullptr : d.Y + (i64)slot(st, i + 1) * a.n1;
    const double alp = first ? 0.0 : s_al[i + 1];
    double v[1] = {0.0};
    DIR_LOOP(j, a.n1) {
      double q = first ? d.G[j] : __dsub_rn(d.Q[j], __dmul_rn(Yp[j], alp));
      d.Q[j] = q;
      v[0] += Si[j] * q;
    }
    double* sl = d.part + (b & 1) * G2;
    dir_partial<1>(v, sum1, sl, sm);
    dir_sync(d, b, &dead);
    double t[1];
    dir_total<1>(sl, sum1, t, sm);
    const double al = st->rho[slot(st, i)] * t[0];
    if (threadIdx.x == 0) s_al[i] = al;
    if (lead) st->al[i] = al;
    __syncthreads();
  }
  // second loop
  for (int i = 0; i < k; i++, b++) {
    const double* Yi = d.Y + (i64)slot(st, i) * a.n1;
    double H0 = 0.0, f = 0.0, al0 = 0.0;
    const double* Sp = nullptr;
    if (i == 0) {
      const int sl0 = slot(st, k - 1);
      double yy = st->yy[sl0];
      if (yy == 0) yy = 1.0;
      const double ys = 1.0 / st->rho[sl0];
      H0 = ys / yy;
      al0 = s_al[0];
    } else {
      Sp = d.S + (i64)slot(st, i - 1) * a.n1;
      f = s_al[i - 1] - s_beta[i - 1];
    }
    double v[1] = {0.0};
    DIR_LOOP(j, a.n1) {
      double z = (i == 0) ? __dmul_rn(__dsub_rn(d.Q[j], __dmul_rn(Yi[j], al0)), H0)
                          : __dadd_rn(d.Z[j], __dmul_rn(Sp[j], f));
      d.Z[j] = z;
      v[0] += Yi[j] * z;
    }
    double* sl = d.part + (b & 1) * G2;
    dir_partial<1>(v, sum1, sl, sm);
    dir_sync(d, b, &dead);
    double t[1];
    dir_total<1>(sl, sum1, t, sm);
    const double be = st->rho[slot(st, i)] * t[0];
    if (threadIdx.x == 0) s_beta[i] = be;
    if (lead) st->beta[i] = be;
    __syncthreads();
  }
  // step = -z (finishing the second loop) or the no-history step
  double dot_gs, smax;
  {
    double c = 0.0, f = 0.0;
    const double* Sp = nullptr;
    if (k == 0) {
      double gn = st->gnorm;
      if (gn > 1) gn = 1.0 / gn;
      c = __dmul_rn(-gn, 0.1);
    } else {
      Sp = d.S + (i64)slot(st, k - 1) * a.n1;
      f = s_al[k - 1] - s_beta[k - 1];
    }
    double v[2] = {0.0, 0.0};
    DIR_LOOP(j, a.n1) {
      double z = (k == 0) ? __dmul_rn(c, d.G[j]) : __dadd_rn(d.Z[j], __dmul_rn(Sp[j], f));
      double s = -z;
      d.STEP[j] = s;
      v[0] += d.G[j] * s;
      v[1] = fmax(v[1], fabs(s));
    }
    const bool mx[2] = {false, true};
    double* sl = d.part + (b & 1) * G2;
    dir_partial<2>(v, mx, sl, sm);
    dir_sync(d, b, &dead);
    double t[2];
    dir_total<2>(sl, mx, t, sm);
    dot_gs = t[0];
    smax = t[1];
    b++;
  }
  // stepsize = max-scaled norm of the step; flip, factors, intercept step
  {
    const double inv = smax == 0 ? 0.0 : 1.0 / smax;
    double v[1] = {0.0};
    DIR_LOOP(j, a.n1) {
      double t = d.STEP[j] * inv;
      v[0] += t * t;
    }
    double* sl = d.part + (b & 1) * G2;
    dir_partial<1>(v, sum1, sl, sm);
    dir_sync(d, b, &dead);
    double t[1];
    dir_total<1>(sl, sum1, t, sm);
    if (lead) {
      st->dot_gs = dot_gs;
      st->smax = smax;
      double ss = (smax == 0) ? 0.0 : sqrt(t[0]) * smax;
      st->stepsize = ss;
      st->flip = (dot_gs > 0) ? -1.0 : 1.0;
      double fac = 1.0;
      if (fac * ss > 1e20) fac = 1e20 / ss;
      st->factor[1] = fac;
      for (int q = 2; q <= 10; q++) st->factor[q] = st->factor[q - 1] / 10.0;
      st->bstep = __ldcg(&d.STEP[a.n1 - 1]) * st->flip;
    }
  }
}

// trial model w' = w + factor*step, b' = b + factor*bstep, then the
// regulariser (regularizer.hpp:14-61; eta = factor, or 1 for ELL).
__global__ void __launch_bounds__(kVecThreads) k_trial(int j, const double* __restrict__ W,
                                                       const double* __restrict__ STEP, double* __restrict__ NW,
                                                       float* __restrict__ NWF, int rtype, double lambda, int eta_one,
                                                       int no_eta, VecArgs a) {
  LbState* st = a.st;
  const double f = st->factor[j], fl = st->flip;
  const double eta = eta_one ? 1.0 : f;
  const double scale = fmax(0.0, 1.0 - (lambda * eta));
  VEC_LOOP(i, a.n) {
    double w = __dadd_rn(W[i], __dmul_rn(f, __dmul_rn(STEP[i], fl)));
    if (rtype == FVG_REG_L2) {
      w = no_eta ? __dsub_rn(w, __dmul_rn(lambda, w)) : __dmul_rn(scale, w);
    } else if (rtype == FVG_REG_L1) {
      double sg = (double)((w >= 0) - (w < 0));
      w = __dsub_rn(w, __dmul_rn(lambda, sg));
    }
    NW[i] = w;
    if (NWF) NWF[i] = (float)w;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->b[1] = __dadd_rn(st->b[0], __dmul_rn(f, st->bstep));
}

// max |g| of a gradient, then its max-scaled norm and rms = |g| / sqrt(n+1)
__global__ void __launch_bounds__(kVecThreads) k_gmax(const double* __restrict__ G, VecArgs a) {
  LbState* st = a.st;
  double v[1] = {0.0};
  VEC_LOOP(j, a.n1) v[0] = fmax(v[0], fabs(G[j]));
  const bool mx[1] = {true};
  grid_reduce<1>(v, mx, a.part, a.ticket, [&](double* t) { st->gmax_t = t[0]; });
}

__global__ void __launch_bounds__(kVecThreads) k_gnorm(const double* __restrict__ G, VecArgs a, int accepted) {
  LbState* st = a.st;
  const double mxv = st->gmax_t;
  const double inv = mxv == 0 ? 0.0 : 1.0 / mxv;
  double v[1] = {0.0};
  VEC_LOOP(j, a.n1) {
    double t = G[j] * inv;
    v[0] += t * t;
  }
  const bool mx[1] = {false};
  grid_reduce<1>(v, mx, a.part, a.ticket, [&](double* t) {
    double nrm = (mxv == 0) ? 0.0 : sqrt(t[0]) * mxv;
    st->gnorm_t = nrm;
    st->rms_t = nrm / sqrt((double)a.n1);
    st->host[0] = st->eval[0];
    st->host[1] = st->loss;
    st->host[2] = st->rms_t;
    if (accepted) {  // initial evaluation
      st->gnorm = nrm;
      st->rms = st->rms_t;
      st->gmax = mxv;
      st->loss = st->eval[0];
    }
  });
}

// Accept the trial and push the (s, y) pair (lbfgs.hpp:114-143):
// s = [w',b'] - [w,b]; y = g' - g with |y_j| < 1e-10 → 0; rho = 1/(s·y)
// (s·y == 0 → 1); ring push; w ← w', g ← g', loss ← new loss.
__global__ void __launch_bounds__(kVecThreads) k_accept(double* __restrict__ W, double* __restrict__ G,
                                                        const double* __restrict__ NW,
                                                        const double* __restrict__ NG, double* __restrict__ S,
                                                        double* __restrict__ Y, VecArgs a) {
  LbState* st = a.st;
  const int k = st->k, h = st->h;
  int nf;
  if (k == 0) nf = 0;
  else nf = (st->front + 1) % h;
  double* Sn = S + (i64)nf * a.n1;
  double* Yn = Y + (i64)nf * a.n1;
  const double bn = st->b[1], bo = st->b[0];
  double v[2] = {0.0, 0.0};
  VEC_LOOP(j, a.n1) {
    double s = (j < a.n) ? __dsub_rn(NW[j], W[j]) : __dsub_rn(bn, bo);
    double y = __dsub_rn(NG[j], G[j]);
    if (fabs(y) < 1e-10) y = 0.0;
    Sn[j] = s;
    Yn[j] = y;
    if (j < a.n) W[j] = NW[j];
    G[j] = NG[j];
    v[0] += s * y;
    v[1] += y * y;
  }
  const bool mx[2] = {false, false};
  grid_reduce<2>(v, mx, a.part, a.ticket, [&](double* t) {
    double dv = t[0];
    if (dv == 0) dv = 1;
    st->rho[nf] = 1.0 / dv;
    st->yy[nf] = t[1];
    if (k == 0) { st->rear = 0; st->front = 0; }
    else if (k == h) { st->rear = (st->rear + 1) % h; st->front = nf; }
    else st->front = nf;
    st->k = k < h ? k + 1 : h;
    st->loss = st->eval[0];
    st->b[0] = st->b[1];
    st->gnorm = st->gnorm_t;
    st->rms = st->rms_t;
  });
}

__global__ void k_d2f(const double* __restrict__ s, float* __restrict__ d, i64 n) {
  VEC_LOOP(j, n) d[j] = (float)s[j];
}

// -------------------------------------------------------------- operand
// One local matrix in one format with what its forward (A x) and backward
// (A^T r) products need.  Forward/backward mirror compute_gradient's
// `data * w` and `trans * dloss` (gradient_descent.hpp:211) or
// `trans_mv(data, dloss)` (gradient_descent.hpp:183, ELL: done here as a
// gather over the transposed CRS copy).
struct Operand {
  int fmt = FVG_CRS;
  i64 m = 0, n = 0;
  DevCRS* A = nullptr;   // forward CRS (CRS format)
  DevCRS* AT = nullptr;  // backward CRS (CRS and ELL)
  DevHYB* H = nullptr;
  DevHYB* HT = nullptr;
  DevJDS* J = nullptr;
  DevJDS* JT = nullptr;
  DevELL* E = nullptr;
  int master = FVG_F64;
  fvg_matrix* M = nullptr;  // the whole matrix (row-panel backward product); null for row blocks
  // owned pieces (minibatches)
  std::unique_ptr<DevCRS> oA, oAT;
  std::unique_ptr<DevHYB> oH, oHT;
  std::unique_ptr<DevJDS> oJ, oJT;
  std::unique_ptr<DevELL> oE;
};

static void ensure_storage(fvg_ctx* c, Operand& o, int storage) {
  if (storage == FVG_SPLIT) {
    if (o.fmt != FVG_CRS) fail(FVG_ERR_UNSUPPORTED, "split storage runs on the CRS format");
    if (o.A) crs_ensure_split(c, *o.A, o.master);
    if (o.AT) crs_ensure_split(c, *o.AT, o.master);
    return;
  }
  if (o.A) crs_ensure_plane(c, *o.A, storage, o.master);
  if (o.AT) crs_ensure_plane(c, *o.AT, storage, o.master);
  if (o.H) {
    ensure_plane_generic(c, o.H->jds.val, o.H->jds.nnz, storage, o.master);
    crs_ensure_plane(c, o.H->crs, storage, o.master);
  }
  if (o.HT) {
    ensure_plane_generic(c, o.HT->jds.val, o.HT->jds.nnz, storage, o.master);
    crs_ensure_plane(c, o.HT->crs, storage, o.master);
  }
  if (o.J) ensure_plane_generic(c, o.J->val, o.J->nnz, storage, o.master);
  if (o.JT) ensure_plane_generic(c, o.JT->val, o.JT->nnz, storage, o.master);
  if (o.E) ensure_plane_generic(c, o.E->val, o.E->m * o.E->width, storage, o.master);
}

// Loss/gradient evaluation over an operand (compute_gradient with trans,
// gradient_descent.hpp:196-225).  w: FP64 weights or their FP32 copy,
// grad[n+1] FP64 (bias last), out[2] = {loss, bias} on the device.
struct Evaluator {
  fvg_ctx* c = nullptr;
  Operand* op = nullptr;
  int storage = FVG_F64;
  const double* label = nullptr;
  const double* sw = nullptr;
  int icpt = 0;
  int loss = 0;      // GLM loss kind (set after init; logistic by default)
  double eps = 0.0;  // epsilon of the eps-insensitive kinds
  DBuf r, z, s1, s2, label_f, sw_f;
  void init(fvg_ctx* c_, Operand* op_, int storage_, const double* label_, const double* sw_, int icpt_) {
    c = c_;
    op = op_;
    storage = storage_;
    label = label_;
    sw = sw_;
    icpt = icpt_;
    ensure_storage(c, *op, storage);
    if (storage == FVG_SPLIT) {
      init_split();
      return;
    }
    // FP32 copies of labels / weights for the FP32-arithmetic epilogue
    label_f.alloc(sizeof(float) * std::max<i64>(op->m, 1), c->stream);
    convert_values(c, label, FVG_F64, label_f.p, FVG_F32, op->m);
    if (sw) {
      sw_f.alloc(sizeof(float) * std::max<i64>(op->m, 1), c->stream);
      convert_values(c, sw, FVG_F64, sw_f.p, FVG_F32, op->m);
    }
    const int vdt = storage == FVG_F64 ? FVG_F64 : FVG_F32;
    r.alloc((size_t)dtype_size(vdt) * std::max<i64>(op->m, 1), c->stream);
    if (op->fmt != FVG_CRS) z.alloc((size_t)dtype_size(vdt) * std::max<i64>(op->m, 1), c->stream);
    if (op->fmt == FVG_CRS) {
      s1.alloc(crs_pass_scratch_bytes(c, *op->A, storage), c->stream);
      FVG_CUDA(cudaMemsetAsync(s1.p, 0, 256, c->stream));
    }
    if (op->AT) {
      s2.alloc(crs_pass_scratch_bytes(c, *op->AT, storage), c->stream);
      FVG_CUDA(cudaMemsetAsync(s2.p, 0, 256, c->stream));
    }
    use_panels();
  }
  // split storage: labels / weights as df pairs, the forward product per row
  // as df pairs, r = dloss * sw as df pairs, the row kernel's partial sums
  DBuf wtx2, gpart;
  void init_split() {
    const i64 m1 = std::max<i64>(op->m, 1);
    label_f.alloc(sizeof(float2) * m1, c->stream);
    split_vector(c, label, label_f.p, op->m);
    if (sw) {
      sw_f.alloc(sizeof(float2) * m1, c->stream);
      split_vector(c, sw, sw_f.p, op->m);
    }
    r.alloc(sizeof(float2) * m1, c->stream);
    wtx2.alloc(sizeof(float2) * m1, c->stream);
    const i64 g = glm_split_grid(c, op->m);
    gpart.alloc(sizeof(double) * 2 * g + 256, c->stream);
    FVG_CUDA(cudaMemsetAsync((char*)gpart.p + sizeof(double) * 2 * g, 0, 256, c->stream));
    // the row-panel layout (backward) and the forward head, when the matrix
    // has them; the whole CRS copies' schedules only for the passes without
    if (op->M && op->fmt == FVG_CRS) {
      PT = panels_for(c, op->M);
      if (PT) {
        panel_ensure_split(c, *PT);
        s3.alloc(panel_split_scratch_bytes(c, *PT, false), c->stream);
      }
      HD = head_for(c, op->M);
      if (HD) {
        panel_ensure_split(c, *HD);
        s4.alloc(panel_split_scratch_bytes(c, *HD, true), c->stream);
      }
    }
    if (!HD) s1.alloc(crs_split_scratch_bytes(c, *op->A, true), c->stream);
    if (!PT) s2.alloc(crs_split_scratch_bytes(c, *op->AT, false), c->stream);
  }
  void eval_split(const void* x, const double* b, double* grad, double* out) {
    const i64 g = glm_split_grid(c, op->m);
    {
      ProfScope ps(c, P_PASS1);
      if (HD) head_pass_split(c, *HD, x, wtx2.p, s4.p);
      else crs_pass_split(c, *op->A, x, true, wtx2.p, s1.p, P_NKEYS);
      GlmSplitArgs e;
      e.lab = label_f.p;
      e.sw = sw ? sw_f.p : nullptr;
      e.intercept = b;
      e.icpt = icpt;
      e.kind = loss;
      e.eps = eps;
      e.r = r.p;
      e.cta_part = gpart.as<double>();
      e.ticket = (unsigned*)((char*)gpart.p + sizeof(double) * 2 * g);
      e.out = out;
      e.grad_bias = grad + op->n;
      glm_split_rows(c, wtx2.p, HD ? HD->ypan2.p : nullptr, op->m, e);
    }
    if (PT) {
      ProfScope ps(c, P_PASS2);
      panel_trans_mv_split(c, *PT, r.p, grad, s3.p);
    } else {
      crs_pass_split(c, *op->AT, r.p, false, grad, s2.p, P_PASS2);
    }
  }
  // FP32 / BF16 values: the row-panel layout for the backward product when
  // the matrix has one (CRS and ELL operands share the transposed CRS), and
  // the forward head for the CRS forward product
  DevPanels* PT = nullptr;
  DevPanels* HD = nullptr;
  DBuf s3, s4;
  void use_panels() {
    if (storage == FVG_F64 || storage == FVG_SPLIT || !op->M) return;
    if (!PT && op->AT) {
      PT = panels_for(c, op->M);
      if (PT) {
        panel_ensure_plane(c, *PT, storage);
        s3.alloc(panel_scratch_bytes(c, *PT, storage), c->stream);
        FVG_CUDA(cudaMemsetAsync(s3.p, 0, 256, c->stream));
      }
    }
    if (!HD && op->fmt == FVG_CRS && op->A) {
      HD = head_for(c, op->M);
      if (HD) {
        head_ensure_plane(c, *HD, storage);
        s4.alloc(head_scratch_bytes(c, *HD, storage), c->stream);
        FVG_CUDA(cudaMemsetAsync(s4.p, 0, 256, c->stream));
      }
    }
  }
  void set_storage(int st) {
    storage = st;
    ensure_storage(c, *op, storage);
    use_panels();
    if (PT && storage != FVG_F64) panel_ensure_plane(c, *PT, storage);
    if (HD && storage != FVG_F64) head_ensure_plane(c, *HD, storage);
  }
  // x: weights (FP64 for FP64 storage, FP32 otherwise); b: device intercept
  void eval(const void* x, const double* b, double* grad, double* out) {
    const int vdt = storage == FVG_F64 ? FVG_F64 : FVG_F32;
    LogregEpi lr;
    lr.label = label;
    lr.sw = sw;
    lr.label_f = label_f.as<float>();
    lr.sw_f = sw ? sw_f.as<float>() : nullptr;
    lr.intercept = b;
    lr.icpt = icpt;
    lr.r = r.p;
    lr.r_dt = vdt;
    lr.out = out;
    lr.grad_bias = grad + op->n;
    lr.loss = loss;
    lr.eps = eps;
    if (op->m == 0) {  // compute_gradient: empty data → zero gradient, no loss
      FVG_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * (op->n + 1), c->stream));
      FVG_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 2, c->stream));
      return;
    }
    if (storage == FVG_SPLIT) {
      eval_split(x, b, grad, out);
      return;
    }
    const bool f32v = storage == FVG_F32;  // timed apart: the passes read 4-byte values
    if (op->fmt == FVG_CRS && HD && storage != FVG_F64) {
      head_logreg_pass(c, *HD, storage, (const float*)x, lr, s4.p, f32v ? P_PASS1_F32 : P_PASS1);
    } else if (op->fmt == FVG_CRS) {
      crs_pass(c, *op->A, storage, vdt, x, vdt, nullptr, EPI_LOGREG, &lr, s1.p, f32v ? P_PASS1_F32 : P_PASS1);
    } else {
      if (op->fmt == FVG_HYBRID) hyb_spmv(c, *op->H, storage, vdt, x, vdt, z.p);
      else if (op->fmt == FVG_JDS) jds_spmv(c, *op->J, storage, vdt, x, vdt, z.p, false);
      else ell_spmv(c, *op->E, storage, vdt, x, vdt, z.p);
      logreg_rows(c, z.p, vdt, op->m, lr);
    }
    // backward product into grad[0..n) (FP64 output)
    if (op->fmt == FVG_HYBRID) hyb_spmv(c, *op->HT, storage, vdt, r.p, FVG_F64, grad);
    else if (op->fmt == FVG_JDS) jds_spmv(c, *op->JT, storage, vdt, r.p, FVG_F64, grad, false);
    else if (PT && storage != FVG_F64)
      panel_trans_mv(c, *PT, storage, r.as<float>(), FVG_F64, grad, s3.p, f32v ? P_PASS2_F32 : P_PASS2);
    else crs_pass(c, *op->AT, storage, vdt, r.p, FVG_F64, grad, EPI_STORE, nullptr, s2.p,
                  f32v ? P_PASS2_F32 : P_PASS2);
  }
};

static void build_operand(fvg_ctx* c, fvg_matrix* M, int fmt, Operand& o) {
  o.fmt = fmt;
  o.M = M;
  o.m = M->A.m;
  o.n = M->A.n;
  o.master = M->master;
  if (fmt == FVG_CRS || fmt == FVG_ELL) {
    if (!M->AT) {
      M->AT.reset(new DevCRS());
      crs_build_transpose(c, M->A, *M->AT, M->master);
    }
    o.AT = M->AT.get();
  }
  if (fmt == FVG_CRS) o.A = &M->A;
  if (fmt == FVG_ELL) {
    if (!M->ell) {
      M->ell.reset(new DevELL());
      ell_build(c, M->A, *M->ell, M->master);
    }
    o.E = M->ell.get();
  }
  if (fmt == FVG_HYBRID) {
    if (!M->hyb) {
      M->hyb.reset(new DevHYB());
      hyb_build(c, M->A, *M->hyb, M->master, 256);
    }
    if (!M->thyb) {
      if (!M->AT) {
        M->AT.reset(new DevCRS());
        crs_build_transpose(c, M->A, *M->AT, M->master);
      }
      M->thyb.reset(new DevHYB());
      hyb_build(c, *M->AT, *M->thyb, M->master, 256);
    }
    o.H = M->hyb.get();
    o.HT = M->thyb.get();
  }
  if (fmt == FVG_JDS) {
    if (!M->jds) {
      M->jds.reset(new DevJDS());
      jds_build(c, M->A, *M->jds, M->master);
    }
    if (!M->tjds) {
      if (!M->AT) {
        M->AT.reset(new DevCRS());
        crs_build_transpose(c, M->A, *M->AT, M->master);
      }
      M->tjds.reset(new DevJDS());
      jds_build(c, *M->AT, *M->tjds, M->master);
    }
    o.J = M->jds.get();
    o.JT = M->tjds.get();
  }
}

// rows [r0, r1) of A as their own CRS matrix (a rank block or a minibatch:
// ml/glm/common.hpp:232-257)
__global__ void k_rebase(const i32* __restrict__ off, i64 r0, i64 cnt, i32* __restrict__ out) {
  VEC_LOOP(i, cnt + 1) out[i] = off[r0 + i] - off[r0];
}

static void crs_rows(fvg_ctx* c, const DevCRS& a, int master, i64 r0, i64 r1, DevCRS& b) {
  b.m = r1 - r0;
  b.n = a.n;
  i32 s = 0, e = 0;
  FVG_CUDA(cudaMemcpyAsync(&s, a.off.as<i32>() + r0, sizeof(i32), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaMemcpyAsync(&e, a.off.as<i32>() + r1, sizeof(i32), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  b.nnz = e - s;
  b.off.alloc(sizeof(i32) * (b.m + 1), c->stream);
  k_rebase<<<(unsigned)std::max<i64>(1, std::min<i64>((b.m + 256) / 256, 4096)), kVecThreads, 0, c->stream>>>(
      a.off.as<i32>(), r0, b.m, b.off.as<i32>());
  check_launch("rebase");
  count_launch(c);
  b.idx.alloc(sizeof(i32) * (b.nnz + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(b.idx.as<i32>() + b.nnz, 0, sizeof(i32) * kPad, c->stream));
  if (b.nnz) FVG_CUDA(cudaMemcpyAsync(b.idx.p, a.idx.as<i32>() + s, sizeof(i32) * b.nnz, cudaMemcpyDeviceToDevice,
                                      c->stream));
  const int sz = dtype_size(master);
  b.val[master].alloc((size_t)sz * (b.nnz + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync((char*)b.val[master].p + (size_t)sz * b.nnz, 0, (size_t)sz * kPad, c->stream));
  if (b.nnz) FVG_CUDA(cudaMemcpyAsync(b.val[master].p, (const char*)a.val[master].p + (size_t)sz * s,
                                      (size_t)sz * b.nnz, cudaMemcpyDeviceToDevice, c->stream));
  b.max_row = a.max_row;  // upper bound; only used for sizing
  // exact max row length of the block for the layouts that need it
  std::vector<i32> hoff(b.m + 1);
  FVG_CUDA(cudaMemcpyAsync(hoff.data(), b.off.p, sizeof(i32) * (b.m + 1), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  i64 mr = 0;
  for (i64 i = 0; i < b.m; i++) mr = std::max<i64>(mr, (i64)hoff[i + 1] - hoff[i]);
  b.max_row = mr;
}

static void build_block_operand(fvg_ctx* c, fvg_matrix* M, int fmt, i64 r0, i64 r1, Operand& o) {
  o.fmt = fmt;
  o.master = M->master;
  o.oA.reset(new DevCRS());
  crs_rows(c, M->A, M->master, r0, r1, *o.oA);
  o.m = o.oA->m;
  o.n = o.oA->n;
  auto trans = [&]() {
    o.oAT.reset(new DevCRS());
    crs_build_transpose(c, *o.oA, *o.oAT, o.master);
  };
  if (fmt == FVG_CRS) {
    trans();
    o.A = o.oA.get();
    o.AT = o.oAT.get();
  } else if (fmt == FVG_ELL) {
    trans();
    o.oE.reset(new DevELL());
    ell_build(c, *o.oA, *o.oE, o.master);
    o.E = o.oE.get();
    o.AT = o.oAT.get();
  } else if (fmt == FVG_HYBRID) {
    trans();
    o.oH.reset(new DevHYB());
    hyb_build(c, *o.oA, *o.oH, o.master, 256);
    o.oHT.reset(new DevHYB());
    hyb_build(c, *o.oAT, *o.oHT, o.master, 256);
    o.H = o.oH.get();
    o.HT = o.oHT.get();
  } else {
    trans();
    o.oJ.reset(new DevJDS());
    jds_build(c, *o.oA, *o.oJ, o.master);
    o.oJT.reset(new DevJDS());
    jds_build(c, *o.oAT, *o.oJT, o.master);
    o.J = o.oJ.get();
    o.JT = o.oJT.get();
  }
}

void check_common(const fvg_glm_params* p, fvg_matrix* M, const double* label) {
  if (!p) fail(FVG_ERR_INVALID_ARG, "null params");
  if (!(p->num_iteration > 0 && p->alpha > 0 && p->reg_param >= 0 && p->convergence_tol >= 0))
    fail(FVG_ERR_INVALID_ARG, "checkAssumption failed: numIteration > 0 && alpha > 0 && regParam >= 0 && "
                              "convergenceTol >= 0");
  if (M->A.n == 0 || M->A.m == 0) fail(FVG_ERR_INVALID_ARG, "Empty training data\n");
  if (!label) fail(FVG_ERR_INVALID_ARG, "Number of label and data are different\n");
  if (p->reg_type < 0 || p->reg_type > 2) fail(FVG_ERR_INVALID_ARG, "Unsupported regularizer!\n");
  if (p->storage < 0 || p->storage > FVG_SPLIT) fail(FVG_ERR_INVALID_ARG, "unknown storage precision");
  if (p->storage == FVG_F64 && M->master != FVG_F64)
    fail(FVG_ERR_INVALID_ARG, "FP64 storage needs FP64 input values");
  if (p->loss < FVG_LOSS_LOGISTIC || p->loss > FVG_LOSS_SQ_EPS_INSENSITIVE) fail(FVG_ERR_INVALID_ARG, "Unsupported loss kind!\n");
}

struct HostPinned {
  double* p = nullptr;
  explicit HostPinned(size_t n) { FVG_CUDA(cudaMallocHost(&p, sizeof(double) * n)); }
  ~HostPinned() { if (p) cudaFreeHost(p); }
};

// The device L-BFGS loop (lbfgs_parallelizer::do_train, lbfgs_parallelizer.hpp:
// 267-364, with lbfgs.hpp:79-143) over an evaluation (LbfgsEval).
void lbfgs_core(fvg_ctx* c, i64 n, const fvg_glm_params* p, int eta_one, LbfgsEval& ev, double* w_h,
                       double* b_h, i64* n_iter, double* loss_out) {
  const i64 n1 = n + 1;
  const int h = (int)p->hist_size;
  cudaStream_t s = c->stream;
  DBuf W, NW, G, NG, Q, Z, STEP, S, Y, part, stbuf;
  W.alloc(sizeof(double) * n1, s);
  NW.alloc(sizeof(double) * n1, s);
  G.alloc(sizeof(double) * n1, s);
  NG.alloc(sizeof(double) * n1, s);
  Q.alloc(sizeof(double) * n1, s);
  Z.alloc(sizeof(double) * n1, s);
  STEP.alloc(sizeof(double) * n1, s);
  S.alloc(sizeof(double) * n1 * h, s);
  Y.alloc(sizeof(double) * n1 * h, s);
  const int vgrid = (int)std::max<i64>(1, std::min<i64>((n1 + kVecThreads - 1) / kVecThreads, 6 * c->num_sms));
  part.alloc(sizeof(double) * 2 * vgrid + 256, s);
  stbuf.alloc(sizeof(LbState) + 256, s);
  unsigned* ticket = (unsigned*)((char*)part.p + sizeof(double) * 2 * vgrid);
  FVG_CUDA(cudaMemsetAsync(ticket, 0, 256, s));
  LbState init = {};
  init.h = h;
  init.b[0] = *b_h;
  LbState* st = stbuf.as<LbState>();
  FVG_CUDA(cudaMemcpyAsync(st, &init, sizeof(LbState), cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(W.p, w_h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  VecArgs va{n, n1, h, part.as<double>(), ticket, st};
  HostPinned hp(4);
  // the direction kernel: a cooperative grid (every CTA resident), its
  // partial sums and barrier counter
  const int dir_blocks = occupancy_blocks((const void*)k_direction, kDirThreads);
  const int dgrid = (int)std::max<i64>(1, std::min<i64>((n1 + kDirThreads - 1) / kDirThreads,
                                                        (i64)std::min(dir_blocks, 8) * c->num_sms));
  DBuf dpart, dbar;
  dpart.alloc(sizeof(double) * 4 * dgrid, s);
  dbar.alloc(sizeof(unsigned long long), s);
  DirArgs dargs{G.as<double>(), Q.as<double>(), Z.as<double>(), STEP.as<double>(), S.as<double>(), Y.as<double>(),
                va, dpart.as<double>(), dbar.as<unsigned long long>(), c->dev_err, barrier_polls(c)};

  auto evaluate = [&](const double* w64, const double* b, double* g, int accepted) {
    ev.eval(w64, b, g, st->eval);
    ProfScope ps(c, P_LBFGS);
    k_gmax<<<vgrid, kVecThreads, 0, s>>>(g, va);
    k_gnorm<<<vgrid, kVecThreads, 0, s>>>(g, va, accepted);
    check_launch("gnorm");
    count_launch(c, 2);
  };
  auto read_host = [&]() {
    FVG_CUDA(cudaMemcpyAsync(hp.p, st->host, sizeof(double) * 4, cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
  };

  // initial evaluation (lbfgs_parallelizer.hpp:286-295)
  evaluate(W.as<double>(), &st->b[0], G.as<double>(), 1);
  read_host();
  double loss = hp.p[0];

  i64 i = 1;
  for (; i <= p->num_iteration; i++) {
    {
      ProfScope ps(c, P_LBFGS);
      FVG_CUDA(cudaMemsetAsync(dbar.p, 0, sizeof(unsigned long long), s));
      void* args[] = {&dargs};
      FVG_CUDA(cudaLaunchCooperativeKernel((void*)k_direction, dgrid, kDirThreads, args, 0, s));
      check_launch("direction");
      count_launch(c);
    }
    int j = 1;
    double newloss = 0, rms_t = 0;
    for (; j <= 10; j++) {
      {
        ProfScope ps(c, P_LBFGS);
        k_trial<<<vgrid, kVecThreads, 0, s>>>(j, W.as<double>(), STEP.as<double>(), NW.as<double>(), nullptr,
                                              p->reg_type, p->reg_param, eta_one, p->l2_no_eta, va);
        check_launch("trial");
        count_launch(c);
      }
      evaluate(NW.as<double>(), &st->b[1], NG.as<double>(), 0);
      read_host();
      newloss = hp.p[0];
      rms_t = hp.p[2];
      if (newloss - loss < 1e-4) break;  // LBFGS_SEARCH_TOL (lbfgs_parallelizer.hpp:155, 329)
    }
    {
      ProfScope ps(c, P_LBFGS);
      k_accept<<<vgrid, kVecThreads, 0, s>>>(W.as<double>(), G.as<double>(), NW.as<double>(), NG.as<double>(),
                                             S.as<double>(), Y.as<double>(), va);
      check_launch("accept");
      count_launch(c);
    }
    loss = newloss;
    if (p->trace) {
      double fac = 0;
      FVG_CUDA(cudaMemcpyAsync(&fac, &st->factor[std::min(j, 10)], sizeof(double), cudaMemcpyDeviceToHost, s));
      FVG_CUDA(cudaStreamSynchronize(s));
      p->trace[4 * (i - 1) + 0] = loss;
      p->trace[4 * (i - 1) + 1] = (double)j;
      p->trace[4 * (i - 1) + 2] = rms_t;
      p->trace[4 * (i - 1) + 3] = fac;
    }
    if (rms_t <= p->convergence_tol) break;
    if (ev.refine(rms_t)) {
      // re-evaluate the accepted model with the new values
      evaluate(W.as<double>(), &st->b[0], G.as<double>(), 1);
      read_host();
      loss = hp.p[0];
    }
  }
  *n_iter = (i == p->num_iteration + 1) ? p->num_iteration : i;
  *loss_out = loss;
  FVG_CUDA(cudaMemcpyAsync(w_h, W.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(b_h, &st->b[0], sizeof(double), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
}

// ============================================================== L-BFGS
// The GLM evaluation of the loop: the model converted for the value storage
// (FP64 as is, an FP32 copy for FP32 / BF16 values, df pairs for split
// values), then the two fused passes (Evaluator::eval); BF16 runs leave for
// FP32 values once the gradient-norm decrease stalls (refinement).
struct GlmLbfgsEval : LbfgsEval {
  fvg_ctx* c = nullptr;
  Evaluator* ev = nullptr;
  const fvg_glm_params* p = nullptr;
  int storage = FVG_F64;
  i64 n = 0;
  DBuf x;  // the converted model
  std::vector<double> rms_hist;
  void eval(const double* w64, const double* b, double* g, double* out) override {
    const void* xp = w64;
    if (storage == FVG_SPLIT) {
      split_vector(c, w64, x.p, n);
      xp = x.p;
    } else if (storage != FVG_F64) {
      const int vg = (int)std::max<i64>(1, std::min<i64>((n + kVecThreads - 1) / kVecThreads, 6 * c->num_sms));
      k_d2f<<<vg, kVecThreads, 0, c->stream>>>(w64, x.as<float>(), n);
      check_launch("d2f");
      count_launch(c);
      xp = x.p;
    }
    ev->eval(xp, b, g, out);
  }
  bool refine(double rms_t) override {
    if (storage != FVG_BF16 || !p->refine) return false;
    rms_hist.push_back(rms_t);
    if (rms_hist.size() < 4) return false;
    const double best = *std::min_element(rms_hist.end() - 4, rms_hist.end() - 1);
    if (!(rms_t > p->refine_stall * best)) return false;
    storage = FVG_F32;
    ev->set_storage(storage);
    return true;
  }
};

void lbfgs_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h, const fvg_glm_params* p,
                 double* w_h, double* b_h, i64* n_iter, double* loss_out) {
  check_common(p, M, label_h);
  const int fmt = p->mat_type;
  if (fmt == FVG_JDS || fmt < 0 || fmt > 3) fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  if (p->hist_size < 1 || p->hist_size > kMaxHist)
    fail(FVG_ERR_INVALID_ARG, "hist_size must be in [1, " + std::to_string(kMaxHist) + "]");
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  Operand op;
  build_operand(c, M, fmt, op);
  DBuf label, sw;
  label.alloc(sizeof(double) * m, s);
  FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  Evaluator ev;
  ev.init(c, &op, p->storage, label.as<double>(), sw_h ? sw.as<double>() : nullptr, p->intercept);
  ev.loss = p->loss;
  ev.eps = p->epsilon;
  GlmLbfgsEval ge;
  ge.c = c;
  ge.ev = &ev;
  ge.p = p;
  ge.storage = p->storage;
  ge.n = n;
  if (p->storage != FVG_F64) ge.x.alloc(sizeof(float2) * (n + 1), s);
  // ELL: the no-trans driver regularises with eta = 1 (lbfgs_parallelizer.hpp:419)
  lbfgs_core(c, n, p, fmt == FVG_ELL ? 1 : 0, ge, w_h, b_h, n_iter, loss_out);
}

// ============================================================ SGD
struct SgdArgs {
  i64 n, n1;
  double* part;
  unsigned* ticket;
  double* scal;  // [0] rmse, [1] b (accepted), [2] lb (local), [3] tot_b, [4] loss sum, [5] prev b,
                 // [6] the current rank's running loss, [7] rank 0's intercept change
  // shrink variant (shrink_sgd_parallelizer.hpp): columns with a nonzero in
  // any rank's rows (used[j] != 0) and rank 0's count of its own columns
  const int* used;
  double n_used0;
};

// w -= ra * g; b -= ra * bias  (update_model, gradient_descent.hpp:242-259)
__global__ void k_sgd_update(double* __restrict__ LW, const double* __restrict__ G, double ra, int icpt, SgdArgs a) {
  VEC_LOOP(j, a.n) LW[j] = __dsub_rn(LW[j], __dmul_rn(ra, G[j]));
  if (icpt && blockIdx.x == 0 && threadIdx.x == 0) a.scal[2] = __dsub_rn(a.scal[2], __dmul_rn(ra, G[a.n]));
}

// rank delta LW - W accumulated into TOT in rank order (calc_diff_inplace +
// typed_allreduce, sgd_parallelizer.hpp:178-187); the rank's loss joins the
// loss sum in the same order (a rank without rows adds 0).
__global__ void k_sgd_delta(const double* __restrict__ LW, const double* __restrict__ W, double* __restrict__ TOT,
                            int first, int has_rows, SgdArgs a) {
  VEC_LOOP(j, a.n) {
    double d = __dsub_rn(LW[j], W[j]);
    TOT[j] = first ? d : __dadd_rn(TOT[j], d);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double db = __dsub_rn(a.scal[2], a.scal[1]);
    a.scal[3] = first ? db : __dadd_rn(a.scal[3], db);
    if (first) a.scal[7] = db;
    const double rl = has_rows ? a.scal[6] : 0.0;
    a.scal[4] = first ? rl : __dadd_rn(a.scal[4], rl);
  }
}

// w += Σdelta; b += Σdelta_b; regularize(w, alpha/sqrt(i)); RMSE of the
// change (sgd_parallelizer.hpp:189-217).  Shrink variant
// (update_model_local, shrink_sgd_parallelizer.hpp:99-151): only the used
// columns exist and are regularised (eta = 1); the RMSE is taken over the
// summed change before regularisation plus rank 0's own intercept change,
// divided by rank 0's column count + 1.
__global__ void __launch_bounds__(kVecThreads) k_sgd_apply(double* __restrict__ W, const double* __restrict__ TOT,
                                                           int rtype, double lambda, double eta, int no_eta,
                                                           int icpt, SgdArgs a) {
  const double scale = fmax(0.0, 1.0 - (lambda * eta));
  double v[1] = {0.0};
  VEC_LOOP(j, a.n) {
    if (a.used && !a.used[j]) continue;
    double prev = W[j];
    double w = __dadd_rn(prev, TOT[j]);
    if (rtype == FVG_REG_L2) w = no_eta ? __dsub_rn(w, __dmul_rn(lambda, w)) : __dmul_rn(scale, w);
    else if (rtype == FVG_REG_L1) w = __dsub_rn(w, __dmul_rn(lambda, (double)((w >= 0) - (w < 0))));
    W[j] = w;
    double df = a.used ? TOT[j] : prev - w;
    v[0] += df * df;
  }
  const bool mx[1] = {false};
  grid_reduce<1>(v, mx, a.part, a.ticket, [&](double* t) {
    double pb = a.scal[1];
    double nb = __dadd_rn(pb, a.scal[3]);
    a.scal[1] = nb;
    if (a.used) {
      double red = t[0] + (icpt ? a.scal[7] * a.scal[7] : 0.0);
      a.scal[0] = sqrt(red / (a.n_used0 + 1.0));
    } else {
      double red = t[0] + (pb - nb) * (pb - nb);
      a.scal[0] = sqrt(red / (double)(a.n + 1));
    }
  });
}

// shrink_column_local (matrix/shrink_matrix.hpp): marks the columns a block
// of nonzeros uses; the count of newly marked columns is added to *count.
__global__ void k_mark_used(const i32* __restrict__ idx, i64 nnz, int* __restrict__ used,
                            unsigned long long* __restrict__ count) {
  unsigned long long mine = 0;
  for (i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (i64)gridDim.x * blockDim.x)
    if (atomicExch(&used[idx[e]], 1) == 0) mine++;
  if (count && mine) atomicAdd(count, mine);
}

// shrink_vector_merge: columns no rank holds come back as 0.
__global__ void k_zero_unused(double* __restrict__ W, const int* __restrict__ used, i64 n) {
  for (i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (i64)gridDim.x * blockDim.x)
    if (!used[j]) W[j] = 0.0;
}

// One minibatch's loss into its rank's running loss (gradient_descent::
// optimize passes one loss variable through the rank's minibatches,
// gradient_descent.hpp:128-145).  The squared loss halves the whole running
// value after each batch (gradient.hpp:70-73); out[0] already holds the
// batch's halved sum, and halving commutes with rounding, so
// 0.5 * running + out[0] equals the reference's 0.5 * (running + sum).
__global__ void k_sgd_loss(const double* __restrict__ out, double* __restrict__ scal, int first, int halve) {
  const double prev = first ? 0.0 : scal[6];
  scal[6] = __dadd_rn(halve ? 0.5 * prev : prev, out[0]);
}

void sgd_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h, const fvg_glm_params* p,
               double* w_h, double* b_h, i64* n_iter, double* loss_out, bool shrink) {
  check_common(p, M, label_h);
  const int fmt = p->mat_type;
  if (fmt < 0 || fmt > 3) fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  if (!(p->mini_batch_fraction > 0.0 && p->mini_batch_fraction <= 1.0))
    fail(FVG_ERR_INVALID_ARG, "checkAssumption failed: miniBatchFraction > 0.0 && miniBatchFraction <= 1.0");
  const i64 m = M->A.m, n = M->A.n, n1 = n + 1;
  const int P = std::max(1, p->num_partitions);
  cudaStream_t s = c->stream;
  std::vector<i64> splits(P + 1);
  if (p->row_splits) {
    for (int r = 0; r <= P; r++) splits[r] = p->row_splits[r];
    if (splits[0] != 0 || splits[P] != m) fail(FVG_ERR_INVALID_ARG, "row_splits must run from 0 to num_row");
    for (int r = 0; r < P; r++)
      if (splits[r + 1] < splits[r]) fail(FVG_ERR_INVALID_ARG, "row_splits must be non-decreasing");
  } else {
    for (int r = 0; r <= P; r++) splits[r] = m * r / P;
  }
  DBuf label, sw;
  label.alloc(sizeof(double) * m, s);
  FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  // minibatches per rank (common.hpp:283-321: ceil(frac*rows) rounded up to 1024)
  struct Batch {
    Operand op;
    Evaluator ev;
    i64 r0;
  };
  std::vector<std::vector<std::unique_ptr<Batch>>> ranks(P);
  const int storage = p->storage;
  if (storage == FVG_SPLIT) fail(FVG_ERR_UNSUPPORTED, "split storage is offered by the L-BFGS trainers, single evaluations and the products");
  for (int r = 0; r < P; r++) {
    i64 ns = splits[r + 1] - splits[r];
    i64 tmp = (i64)std::ceil(ns * p->mini_batch_fraction);
    i64 t2 = (tmp == 0 ? 0 : (tmp - 1) / 1024 + 1) * 1024;
    i64 mbs = t2 < ns ? t2 : ns;
    i64 nb = (ns == 0) ? 0 : (ns - 1) / mbs + 1;
    for (i64 k = 0; k < nb; k++) {
      i64 r0 = splits[r] + k * mbs, r1 = std::min(splits[r] + (k + 1) * mbs, splits[r + 1]);
      auto b = std::make_unique<Batch>();
      b->r0 = r0;
      build_block_operand(c, M, fmt, r0, r1, b->op);
      b->ev.init(c, &b->op, storage, label.as<double>() + r0, sw_h ? sw.as<double>() + r0 : nullptr, p->intercept);
      b->ev.loss = p->loss;
      b->ev.eps = p->epsilon;
      ranks[r].push_back(std::move(b));
    }
  }
  DBuf W, LW, LWF, G, TOT, part, scal, out;
  W.alloc(sizeof(double) * n1, s);
  LW.alloc(sizeof(double) * n1, s);
  LWF.alloc(sizeof(float) * n1, s);
  G.alloc(sizeof(double) * n1, s);
  TOT.alloc(sizeof(double) * n1, s);
  const int vgrid = (int)std::max<i64>(1, std::min<i64>((n1 + kVecThreads - 1) / kVecThreads, 6 * c->num_sms));
  part.alloc(sizeof(double) * 2 * vgrid + 256, s);
  unsigned* ticket = (unsigned*)((char*)part.p + sizeof(double) * 2 * vgrid);
  FVG_CUDA(cudaMemsetAsync(ticket, 0, 256, s));
  scal.alloc(sizeof(double) * 8, s);
  out.alloc(sizeof(double) * 2, s);
  double hs[8] = {0, *b_h, *b_h, 0, 0, 0, 0, 0};
  FVG_CUDA(cudaMemcpyAsync(scal.p, hs, sizeof(hs), cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(W.p, w_h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  SgdArgs sa{n, n1, part.as<double>(), ticket, scal.as<double>(), nullptr, 0.0};
  DBuf used, used0;
  if (shrink) {
    // used columns over all ranks, and rank 0's own count (each rank's
    // shrink table covers all of its minibatches)
    used.alloc(sizeof(int) * std::max<i64>(n, 1), s);
    used0.alloc(sizeof(int) * std::max<i64>(n, 1) + 256, s);
    FVG_CUDA(cudaMemsetAsync(used.p, 0, sizeof(int) * std::max<i64>(n, 1), s));
    FVG_CUDA(cudaMemsetAsync(used0.p, 0, sizeof(int) * std::max<i64>(n, 1) + 256, s));
    unsigned long long* cnt0 = (unsigned long long*)((char*)used0.p + sizeof(int) * std::max<i64>(n, 1));
    for (int r = 0; r < P; r++)
      for (auto& b : ranks[r]) {
        const DevCRS& A = *b->op.oA;
        if (A.nnz == 0) continue;
        const int g = (int)std::max<i64>(1, std::min<i64>((A.nnz + 255) / 256, 4 * (i64)c->num_sms));
        k_mark_used<<<g, 256, 0, s>>>(A.idx.as<i32>(), A.nnz, used.as<int>(), nullptr);
        if (r == 0) k_mark_used<<<g, 256, 0, s>>>(A.idx.as<i32>(), A.nnz, used0.as<int>(), cnt0);
        check_launch("mark_used");
        count_launch(c, r == 0 ? 2 : 1);
      }
    unsigned long long n0 = 0;
    FVG_CUDA(cudaMemcpyAsync(&n0, cnt0, sizeof(n0), cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    sa.used = used.as<int>();
    sa.n_used0 = (double)n0;
  }
  HostPinned hp(8);
  i64 i;
  for (i = 1; i <= p->num_iteration; i++) {
    const double ra = p->alpha / std::sqrt((double)i);
    bool first_rank = true;
    for (int r = 0; r < P; r++) {
      bool first_loss = true;
      FVG_CUDA(cudaMemcpyAsync(LW.p, W.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      FVG_CUDA(cudaMemcpyAsync(scal.as<double>() + 2, scal.as<double>() + 1, sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
      for (auto& b : ranks[r]) {
        const void* x = LW.p;
        if (storage != FVG_F64) {
          k_d2f<<<vgrid, kVecThreads, 0, s>>>(LW.as<double>(), LWF.as<float>(), n);
          check_launch("d2f");
          count_launch(c);
          x = LWF.p;
        }
        b->ev.eval(x, scal.as<double>() + 2, G.as<double>(), out.as<double>());
        k_sgd_loss<<<1, 1, 0, s>>>(out.as<double>(), scal.as<double>(), first_loss ? 1 : 0,
                                   p->loss == FVG_LOSS_SQUARED ? 1 : 0);
        k_sgd_update<<<vgrid, kVecThreads, 0, s>>>(LW.as<double>(), G.as<double>(), ra, p->intercept, sa);
        check_launch("sgd_update");
        count_launch(c, 2);
        first_loss = false;
      }
      k_sgd_delta<<<vgrid, kVecThreads, 0, s>>>(LW.as<double>(), W.as<double>(), TOT.as<double>(), first_rank ? 1 : 0,
                                                ranks[r].empty() ? 0 : 1, sa);
      check_launch("sgd_delta");
      count_launch(c);
      first_rank = false;
    }
    // the shrink driver calls regularize(w) with its default eta = 1
    // (shrink_sgd_parallelizer.hpp:134; regularizer.hpp:43)
    k_sgd_apply<<<vgrid, kVecThreads, 0, s>>>(W.as<double>(), TOT.as<double>(), p->reg_type, p->reg_param,
                                              shrink ? 1.0 : p->alpha / std::sqrt((double)i), p->l2_no_eta,
                                              p->intercept, sa);
    check_launch("sgd_apply");
    count_launch(c);
    FVG_CUDA(cudaMemcpyAsync(hp.p, scal.p, sizeof(double) * 8, cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    if (hp.p[0] < p->convergence_tol) break;
  }
  *n_iter = (i == p->num_iteration + 1) ? p->num_iteration : i;
  // the shrink driver's no-trans (ELL) loop reports i as is: numIteration+1
  // when it ran out (shrink_sgd_parallelizer.hpp:315)
  if (shrink && fmt == FVG_ELL) *n_iter = i;
  if (shrink && n > 0) {
    k_zero_unused<<<vgrid, kVecThreads, 0, s>>>(W.as<double>(), used.as<int>(), n);
    check_launch("zero_unused");
    count_launch(c);
  }
  FVG_CUDA(cudaMemcpyAsync(hp.p, scal.p, sizeof(double) * 8, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(w_h, W.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  *b_h = hp.p[1];
  *loss_out = hp.p[4];
}

// ====================================================== single evaluation
void logreg_eval(fvg_ctx* c, fvg_matrix* M, int fmt, int storage, const double* label_h, const double* sw_h,
                 const double* w_h, double b, int icpt, double* grad_h, double* loss_h, int loss_kind, double eps) {
  if (loss_kind < FVG_LOSS_LOGISTIC || loss_kind > FVG_LOSS_SQ_EPS_INSENSITIVE) fail(FVG_ERR_INVALID_ARG, "Unsupported loss kind!\n");
  if (fmt < 0 || fmt > 3) fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  if (storage == FVG_F64 && M->master != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 storage needs FP64 values");
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  Operand op;
  build_operand(c, M, fmt, op);
  DBuf label, sw, w, wf, g, out, bd;
  label.alloc(sizeof(double) * std::max<i64>(m, 1), s);
  if (m) FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  w.alloc(sizeof(double) * (n + 1), s);
  wf.alloc(sizeof(float) * (n + 1), s);
  g.alloc(sizeof(double) * (n + 1), s);
  out.alloc(sizeof(double) * 2, s);
  bd.alloc(sizeof(double), s);
  FVG_CUDA(cudaMemcpyAsync(w.p, w_h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(bd.p, &b, sizeof(double), cudaMemcpyHostToDevice, s));
  Evaluator ev;
  ev.init(c, &op, storage, label.as<double>(), sw_h ? sw.as<double>() : nullptr, icpt);
  ev.loss = loss_kind;
  ev.eps = eps;
  const void* x = w.p;
  DBuf w2;
  if (storage == FVG_SPLIT) {
    w2.alloc(sizeof(float2) * (n + 1), s);
    split_vector(c, w.as<double>(), w2.p, n);
    x = w2.p;
  } else if (storage != FVG_F64) {
    k_d2f<<<256, kVecThreads, 0, s>>>(w.as<double>(), wf.as<float>(), n);
    check_launch("d2f");
    count_launch(c);
    x = wf.p;
  }
  ev.eval(x, bd.as<double>(), g.as<double>(), out.as<double>());
  double ho[2];
  FVG_CUDA(cudaMemcpyAsync(grad_h, g.p, sizeof(double) * (n + 1), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(ho, out.p, sizeof(ho), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  *loss_h = ho[0];
}

}  // namespace fvg

namespace fvg {

// ============================================================ autotuner
// The reference picks the product format by MatType (CRS on x86, HYBRID on
// VE: logistic_regression_with_lbfgs.hpp:280-285) and has no layout knobs.
// Here every candidate layout gives the same sums up to summation order, so
// the choice is a matter of speed: each candidate — format (CRS, and for
// FP32/BF16 values ELL when its padding stays within 4x the nonzeros, and
// the hybrid), the forward head on or off, the row panels off or on with a
// hot threshold of 1, 2 or 4 entries per panel — is timed over `reps` loss/
// gradient evaluations (CUDA events on the context stream, after one warm
// evaluation), and the fastest is left set on the matrix.
namespace {
void set_layout(fvg_ctx* c, fvg_matrix* M, int head, double panel_min) {
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  M->head.reset();
  M->head_tried = false;
  M->head_cols = head ? -1 : 0;
  M->pan.reset();
  M->pan_tried = false;
  M->panel_rows = panel_min > 0 ? -1 : 0;
  M->panel_min = panel_min > 0 ? panel_min : -1.0;
}
}  // namespace

void autotune(fvg_ctx* c, fvg_matrix* M, int storage, const double* label_h, int reps,
              std::vector<fvg_tune_choice>& tried, fvg_tune_choice& best) {
  if (storage < FVG_F64 || storage > FVG_SPLIT) fail(FVG_ERR_INVALID_ARG, "unknown storage dtype");
  if (storage == FVG_F64 && M->master != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 storage needs FP64 values");
  if (M->A.m == 0 || M->A.n == 0) fail(FVG_ERR_INVALID_ARG, "Empty training data\n");
  reps = std::max(1, reps);
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  DBuf label, w, wx, g, out, bd;
  label.alloc(sizeof(double) * m, s);
  if (label_h) {
    FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  } else {
    std::vector<double> ones((size_t)m, 1.0);
    FVG_CUDA(cudaMemcpyAsync(label.p, ones.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaStreamSynchronize(s));
  }
  w.alloc(sizeof(double) * (n + 1), s);
  FVG_CUDA(cudaMemsetAsync(w.p, 0, sizeof(double) * (n + 1), s));
  wx.alloc(sizeof(float2) * (n + 1), s);
  g.alloc(sizeof(double) * (n + 1), s);
  out.alloc(sizeof(double) * 2, s);
  bd.alloc(sizeof(double), s);
  FVG_CUDA(cudaMemsetAsync(bd.p, 0, sizeof(double), s));
  const void* x = w.p;
  if (storage == FVG_SPLIT) {
    split_vector(c, w.as<double>(), wx.p, n);
    x = wx.p;
  } else if (storage != FVG_F64) {
    FVG_CUDA(cudaMemsetAsync(wx.p, 0, sizeof(float) * (n + 1), s));
    x = wx.p;
  }
  // candidates
  std::vector<fvg_tune_choice> cand;
  const bool lowp = storage == FVG_F32 || storage == FVG_BF16;
  const bool layouts = storage != FVG_F64;  // the head and the panels exist for FP32 / BF16 / split values
  for (int head : {0, 1})
    for (double pm : {0.0, 1.0, 2.0, 4.0}) {
      if (!layouts && (head || pm > 0)) continue;
      cand.push_back({FVG_CRS, head, pm, 0.0});
    }
  if (lowp) {
    if (M->A.max_row * m <= 4 * M->A.nnz) cand.push_back({FVG_ELL, 0, 0.0, 0.0});
    cand.push_back({FVG_HYBRID, 0, 0.0, 0.0});
  }
  cudaEvent_t e0, e1;
  FVG_CUDA(cudaEventCreate(&e0));
  FVG_CUDA(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evs{e0, e1};
  best = {FVG_CRS, 0, 0.0, -1.0};
  for (auto ch : cand) {
    set_layout(c, M, ch.head, ch.panel_min);
    Operand op;
    build_operand(c, M, ch.format, op);
    Evaluator ev;
    ev.init(c, &op, storage, label.as<double>(), nullptr, 0);
    if ((ch.head && !ev.HD) || (ch.panel_min > 0 && !ev.PT)) continue;  // the layout does not apply
    ev.eval(x, bd.as<double>(), g.as<double>(), out.as<double>());
    FVG_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; r++) ev.eval(x, bd.as<double>(), g.as<double>(), out.as<double>());
    FVG_CUDA(cudaEventRecord(e1, s));
    FVG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    FVG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    ch.eval_ms = ms / reps;
    tried.push_back(ch);
    if (best.eval_ms < 0 || ch.eval_ms < best.eval_ms) best = ch;
  }
  if (best.eval_ms < 0) fail(FVG_ERR_INTERNAL, "no candidate layout could be timed");
  set_layout(c, M, best.head, best.panel_min);
  check_device_error(c);
}

}  // namespace fvg
