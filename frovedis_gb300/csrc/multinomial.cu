// Multinomial logistic regression on the device: softmax_parallelizer::
// do_train with the transposed copy (ml/glm/softmax_parallelizer.hpp:210-242)
// and softmax_gradient_descent::compute_gradient (ml/glm/
// softmax_gradient_descent.hpp:119-136).  Per iteration:
//  1. P = (softmax(X W + icpt) - onehot(label)) * sw: one multi-vector pass
//     over X with the softmax fused into its epilogue (<= 128 classes; more
//     classes: the product first, then a row-softmax kernel);
//  2. G = X^T P: a multi-vector pass over the transposed copy (FP64 output);
//  3. update_global_model (softmax_parallelizer.hpp:147-200): W = reg(W -
//     a_i G), intercept -= a_i * (column sums of G), a_i = alpha/sqrt(i), and
//     the RMS of the model change for the _CONV_RATE_CHECK_ stop
//     (ml/glm/common.hpp:21) — one fused pass over W and G plus a one-CTA
//     finish; the host reads the RMS (8 bytes) per iteration.
// W and G are row-major [n][K] FP64 (the reference's rowmajor_matrix_local
// weight); the FP32/BF16 paths gather an FP32 copy of W.  All reductions
// have a fixed order.
#include <algorithm>
#include <cmath>

#include "fvg_internal.cuh"

namespace fvg {

// Rows of P (the gathered matrix of the backward product A^T P) in one slab
// of the backward's slab-ordered pieces: 48 MiB of the gathered block.
static i64 backward_slab(int K, int storage) {
  const i64 w = std::min<i64>(K, 128) * (storage == FVG_F64 ? 8 : 4);
  return std::max<i64>(4096, (i64)(48ll << 20) / w);
}


constexpr int kMT = 256;

void crs_spmm_softmax(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int K, const double* label,
                      const double* sw, const float* label_f, const float* sw_f, int icpt, const double* icpt_v,
                      void* P, i64 ldp, void* scratch, double* loss_out = nullptr);

template <class T> __device__ __forceinline__ T exp_t(T x);
template <> __device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }

// Row softmax for more than 128 classes (a warp per row, in place over
// Z = X W): z += icpt, row max, exp(z - max), row sum, z * (1/sum), then the
// error term when labels are given.
template <class T>
__global__ void __launch_bounds__(kMT) km_softmax_rows(T* __restrict__ Z, i64 m, int K, const double* __restrict__ icpt,
                                                        int icpt_on, const T* __restrict__ label,
                                                        const T* __restrict__ sw) {
  const int lane = threadIdx.x & 31;
  for (i64 r = ((i64)blockIdx.x * kMT + threadIdx.x) >> 5; r < m; r += ((i64)gridDim.x * kMT) >> 5) {
    T* z = Z + r * K;
    T mx = -INFINITY;
    for (int j = lane; j < K; j += 32) {
      T v = z[j];
      if (icpt_on) v += (T)icpt[j];
      z[j] = v;
      mx = fmax(mx, v);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    T sum = 0;
    for (int j = lane; j < K; j += 32) {
      const T e = exp_t<T>(z[j] - mx);
      z[j] = e;
      sum += e;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const T inv = (T)1 / sum;
    const T lab = label ? label[r] : (T)0;
    const T w = (label && sw) ? sw[r] : (T)1;
    for (int j = lane; j < K; j += 32) {
      T pr = inv * z[j];
      if (label) {
        pr -= (lab == (T)j) ? (T)1 : (T)0;
        pr *= w;
      }
      z[j] = pr;
    }
  }
}

// W = reg(W - ra*G) (regularize with eta = 1, regularizer.hpp:14-61); per
// CTA: column sums of G (the intercept gradient, sum_of_rows) and the sum of
// squared weight changes.  Thread (column j, row lane rr) walks rows
// r0+rr, r0+rr+rpb, ... of the CTA's row range.
__global__ void __launch_bounds__(kMT) km_update(double* __restrict__ W, const double* __restrict__ G, i64 n, int K,
                                                 int kp, double ra, int rtype, double lambda,
                                                 double* __restrict__ colpart, double* __restrict__ sqpart) {
  __shared__ double sm[kMT];
  const int rpb = kMT / kp;
  const int jj = threadIdx.x % kp, rr = threadIdx.x / kp;
  const i64 rows = (n + gridDim.x - 1) / gridDim.x;
  const i64 r0 = (i64)blockIdx.x * rows, r1 = std::min<i64>(n, r0 + rows);
  const double scale = fmax(0.0, 1.0 - lambda);
  double sq = 0.0;
  for (int c0 = 0; c0 < K; c0 += kp) {
    const int j = c0 + jj;
    double cs = 0.0;
    if (j < K) {
      for (i64 r = r0 + rr; r < r1; r += rpb) {
        const i64 e = r * K + j;
        const double g = G[e], old = W[e];
        double w = __dsub_rn(old, __dmul_rn(ra, g));
        if (rtype == FVG_REG_L2) w = __dmul_rn(scale, w);
        else if (rtype == FVG_REG_L1) w = __dsub_rn(w, __dmul_rn(lambda, (double)((w >= 0) - (w < 0))));
        W[e] = w;
        cs += g;
        const double d = w - old;
        sq += d * d;
      }
    }
    sm[threadIdx.x] = cs;
    __syncthreads();
    for (int s = rpb / 2; s > 0; s >>= 1) {
      if (rr < s) sm[threadIdx.x] += sm[threadIdx.x + s * kp];
      __syncthreads();
    }
    if (rr == 0 && j < K) colpart[(i64)blockIdx.x * K + j] = sm[threadIdx.x];
    __syncthreads();
  }
  sm[threadIdx.x] = sq;
  __syncthreads();
  for (int s = kMT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) sqpart[blockIdx.x] = sm[0];
}

// intercept -= ra * (column sums of G); out[0] = RMS of the model change
// over (n [+1]) * K entries.
__global__ void __launch_bounds__(kMT) km_finish(const double* __restrict__ colpart, const double* __restrict__ sqpart,
                                                 int nblk, i64 n, int K, double ra, int icpt_on,
                                                 double* __restrict__ icpt, double* __restrict__ out) {
  __shared__ double sm[kMT];
  double isq = 0.0;
  for (int j = threadIdx.x; j < K; j += kMT) {
    double bias = 0.0;
    for (int b = 0; b < nblk; b++) bias += colpart[(i64)b * K + j];
    if (icpt_on) {
      const double old = icpt[j];
      const double nw = __dsub_rn(old, __dmul_rn(ra, bias));
      icpt[j] = nw;
      const double d = nw - old;
      isq += d * d;
    }
  }
  sm[threadIdx.x] = isq;
  __syncthreads();
  for (int s = kMT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double sq = 0.0;
    for (int b = 0; b < nblk; b++) sq += sqpart[b];
    sq += sm[0];
    const double nft = (double)(n + (icpt_on ? 1 : 0));
    out[0] = sqrt(sq / (nft * K));
  }
}

__global__ void km_d2f(const double* __restrict__ s, float* __restrict__ d, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) d[i] = (float)s[i];
}

struct Softmax {
  fvg_ctx* c;
  DevCRS* A;
  int storage;
  i64 m, n;
  int K;
  DBuf Z, scratch, label_f, sw_f;
  void init(fvg_ctx* c_, DevCRS* A_, int master, int storage_, int K_, const double* label, const double* sw) {
    c = c_;
    A = A_;
    storage = storage_;
    m = A->m;
    n = A->n;
    K = K_;
    crs_ensure_plane(c, *A, storage, master);
    Z.alloc((size_t)(storage == FVG_F64 ? 8 : 4) * std::max<i64>(m * K, 1), c->stream);
    scratch.alloc((size_t)spmm_scratch_bytes(c, *A, storage), c->stream);
    if (label) {
      label_f.alloc(sizeof(float) * std::max<i64>(m, 1), c->stream);
      convert_values(c, label, FVG_F64, label_f.p, FVG_F32, m);
    }
    if (sw) {
      sw_f.alloc(sizeof(float) * std::max<i64>(m, 1), c->stream);
      convert_values(c, sw, FVG_F64, sw_f.p, FVG_F32, m);
    }
  }
  // Z = softmax(X w + icpt) [- onehot(label)] [* sw]; w: [n][K] of the
  // accumulator type
  void forward(const void* w, const double* label, const double* sw, int icpt_on, const double* icpt) {
    ProfScope ps(c, P_BATCH_PASS1);
    const bool f64 = storage == FVG_F64;
    const float* lf = label ? label_f.as<float>() : nullptr;
    const float* sf = (label && sw) ? sw_f.as<float>() : nullptr;
    if (K <= 128) {
      crs_spmm_softmax(c, *A, storage, w, K, K, label, label ? sw : nullptr, lf, sf, icpt_on, icpt, Z.p, K,
                       scratch.p);
      return;
    }
    const size_t es = f64 ? 8 : 4;
    for (int c0 = 0; c0 < K; c0 += 128) {
      const int kb = std::min(128, K - c0);
      crs_spmm_block(c, *A, storage, (const char*)w + c0 * es, K, kb, f64 ? FVG_F64 : FVG_F32, (char*)Z.p + c0 * es,
                     K, scratch.p);
    }
    const unsigned g = (unsigned)std::max<i64>(1, std::min<i64>((m * 32 + kMT - 1) / kMT, 8 * (i64)c->num_sms));
    if (f64)
      km_softmax_rows<double><<<g, kMT, 0, c->stream>>>(Z.as<double>(), m, K, icpt, icpt_on, label,
                                                        label ? sw : nullptr);
    else
      km_softmax_rows<float><<<g, kMT, 0, c->stream>>>(Z.as<float>(), m, K, icpt, icpt_on, lf, sf);
    check_launch("km_softmax_rows");
    count_launch(c);
  }
};

void multinomial_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                       const fvg_glm_params* p, i64 K, double* w_h, double* b_h, i64* n_iter) {
  check_common(p, M, label_h);
  if (K < 1 || K > (1 << 20)) fail(FVG_ERR_INVALID_ARG, "number of classes must be in [1, 2^20]");
  if (p->mat_type != FVG_CRS && p->mat_type != FVG_HYBRID)
    fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
  const int storage = p->storage;
  if (storage == FVG_SPLIT) fail(FVG_ERR_UNSUPPORTED, "split storage is offered by the L-BFGS trainers, single evaluations and the products");
  const bool mixed = storage != FVG_F64;
  crs_ensure_plane(c, *M->AT, storage, M->master);

  DBuf label, sw, W, WF, G, ICPT, colpart, sqpart, out, s2;
  label.alloc(sizeof(double) * m, s);
  FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  Softmax sm;
  sm.init(c, &M->A, M->master, storage, (int)K, label.as<double>(), sw_h ? sw.as<double>() : nullptr);
  const size_t nk = (size_t)n * K;
  W.alloc(sizeof(double) * nk, s);
  G.alloc(sizeof(double) * nk, s);
  if (mixed) WF.alloc(sizeof(float) * nk, s);
  ICPT.alloc(sizeof(double) * K, s);
  FVG_CUDA(cudaMemcpyAsync(W.p, w_h, sizeof(double) * nk, cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(ICPT.p, b_h, sizeof(double) * K, cudaMemcpyHostToDevice, s));
  const i64 slab = backward_slab((int)K, storage);
  s2.alloc((size_t)spmm_scratch_bytes(c, *M->AT, storage, slab), s);
  int kp = 1;
  while (kp < K && kp < kMT) kp <<= 1;
  const int nblk = (int)std::max<i64>(1, std::min<i64>((n + 63) / 64, 4 * (i64)c->num_sms));
  colpart.alloc(sizeof(double) * (size_t)nblk * K, s);
  sqpart.alloc(sizeof(double) * nblk, s);
  out.alloc(256, s);
  double* hout = nullptr;
  FVG_CUDA(cudaMallocHost(&hout, sizeof(double)));
  struct Free {
    double* p;
    ~Free() { cudaFreeHost(p); }
  } free_h{hout};
  const unsigned dg = (unsigned)std::max<i64>(1, std::min<i64>(((i64)nk + 255) / 256, 4 * (i64)c->num_sms));
  const size_t es = mixed ? 4 : 8;

  i64 i;
  for (i = 1; i <= p->num_iteration; i++) {
    const void* wx = W.p;
    if (mixed) {
      km_d2f<<<dg, 256, 0, s>>>(W.as<double>(), WF.as<float>(), (i64)nk);
      check_launch("km_d2f");
      count_launch(c);
      wx = WF.p;
    }
    sm.forward(wx, label.as<double>(), sw_h ? sw.as<double>() : nullptr, p->intercept, ICPT.as<double>());
    {
      ProfScope ps(c, P_BATCH_PASS2);
      for (int c0 = 0; c0 < K; c0 += 128) {
        const int kb = (int)std::min<i64>(128, K - c0);
        crs_spmm_block(c, *M->AT, storage, (const char*)sm.Z.p + c0 * es, K, kb, FVG_F64, G.as<double>() + c0, K,
                       s2.p, nullptr, slab);
      }
    }
    const double ra = p->alpha / std::sqrt((double)i);
    {
      ProfScope ps(c, P_LBFGS);
      km_update<<<nblk, kMT, 0, s>>>(W.as<double>(), G.as<double>(), n, (int)K, kp, ra, p->reg_type, p->reg_param,
                                     colpart.as<double>(), sqpart.as<double>());
      km_finish<<<1, kMT, 0, s>>>(colpart.as<double>(), sqpart.as<double>(), nblk, n, (int)K, ra, p->intercept,
                                  ICPT.as<double>(), out.as<double>());
      check_launch("km_update");
      count_launch(c, 2);
    }
    FVG_CUDA(cudaMemcpyAsync(hout, out.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    if (*hout <= p->convergence_tol) break;
  }
  *n_iter = (i == p->num_iteration + 1) ? p->num_iteration : i;
  FVG_CUDA(cudaMemcpyAsync(w_h, W.p, sizeof(double) * nk, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(b_h, ICPT.p, sizeof(double) * K, cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
}

// Multinomial logistic regression by L-BFGS (no reference counterpart: the
// reference trains the softmax model by gradient descent only).  The
// gradient is the reference's, softmax_gradient_descent::compute_gradient
// with the transposed copy (softmax_gradient_descent.hpp:119-136); the loss
// the line search needs, which the reference's softmax path does not
// compute, is the cross-entropy sum_i -log p[i, label_i] (unweighted, as
// logistic_gradient's loss is), accumulated in the forward pass's softmax
// epilogue.  The device L-BFGS loop (lbfgs.hpp:79-143, lbfgs_parallelizer.hpp
// :267-364) runs on the weights W (num_col x K row-major, FP64) as one vector
// of num_col * K entries; no intercept.
struct SoftmaxLbfgsEval : LbfgsEval {
  fvg_ctx* c = nullptr;
  fvg_matrix* M = nullptr;
  Softmax sm;
  int storage = FVG_F64;
  i64 n = 0;
  int K = 0;
  const double* label = nullptr;
  const double* sw = nullptr;
  DBuf WF, s2, lossbuf;
  i64 slab = 0;
  void eval(const double* w64, const double* b, double* g, double* out) override {
    (void)b;
    const bool mixed = storage != FVG_F64;
    const void* wx = w64;
    const i64 nk = n * K;
    if (mixed) {
      const unsigned dg = (unsigned)std::max<i64>(1, std::min<i64>((nk + 255) / 256, 4 * (i64)c->num_sms));
      km_d2f<<<dg, 256, 0, c->stream>>>(w64, WF.as<float>(), nk);
      check_launch("km_d2f");
      count_launch(c);
      wx = WF.p;
    }
    {
      ProfScope ps(c, P_BATCH_PASS1);
      crs_spmm_softmax(c, *sm.A, storage, wx, K, K, label, sw, label ? sm.label_f.as<float>() : nullptr,
                       sw ? sm.sw_f.as<float>() : nullptr, 0, nullptr, sm.Z.p, K, sm.scratch.p, lossbuf.as<double>());
    }
    {
      ProfScope ps(c, P_BATCH_PASS2);
      crs_spmm_block(c, *M->AT, storage, sm.Z.p, K, K, FVG_F64, g, K, s2.p, nullptr, slab);
    }
    FVG_CUDA(cudaMemsetAsync(g + nk, 0, sizeof(double), c->stream));
    FVG_CUDA(cudaMemcpyAsync(out, lossbuf.p, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    FVG_CUDA(cudaMemsetAsync(out + 1, 0, sizeof(double), c->stream));
  }
};

void multinomial_lbfgs_train(fvg_ctx* c, fvg_matrix* M, const double* label_h, const double* sw_h,
                             const fvg_glm_params* p, i64 K, double* w_h, i64* n_iter, double* loss_out) {
  check_common(p, M, label_h);
  if (K < 2 || K > 128) fail(FVG_ERR_INVALID_ARG, "the L-BFGS multinomial solver takes 2 to 128 classes");
  if (p->intercept) fail(FVG_ERR_UNSUPPORTED, "the L-BFGS multinomial solver trains no intercept");
  if (p->mat_type != FVG_CRS && p->mat_type != FVG_HYBRID)
    fail(FVG_ERR_UNSUPPORTED, "Unsupported input matrix type!!\n");
  if (p->hist_size < 1 || p->hist_size > 32) fail(FVG_ERR_INVALID_ARG, "hist_size must be in [1, 32]");
  const int storage = p->storage;
  if (storage == FVG_SPLIT) fail(FVG_ERR_UNSUPPORTED, "split storage is offered by the binary L-BFGS trainers, single evaluations and the products");
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
  crs_ensure_plane(c, *M->AT, storage, M->master);
  DBuf label, sw;
  label.alloc(sizeof(double) * m, s);
  FVG_CUDA(cudaMemcpyAsync(label.p, label_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  if (sw_h) {
    sw.alloc(sizeof(double) * m, s);
    FVG_CUDA(cudaMemcpyAsync(sw.p, sw_h, sizeof(double) * m, cudaMemcpyHostToDevice, s));
  }
  SoftmaxLbfgsEval ev;
  ev.c = c;
  ev.M = M;
  ev.storage = storage;
  ev.n = n;
  ev.K = (int)K;
  ev.label = label.as<double>();
  ev.sw = sw_h ? sw.as<double>() : nullptr;
  ev.sm.init(c, &M->A, M->master, storage, (int)K, ev.label, ev.sw);
  if (storage != FVG_F64) ev.WF.alloc(sizeof(float) * (size_t)n * K, s);
  ev.slab = backward_slab((int)K, storage);
  ev.s2.alloc((size_t)spmm_scratch_bytes(c, *M->AT, storage, ev.slab), s);
  ev.lossbuf.alloc(sizeof(double) * 2 * 128, s);
  double b = 0.0;
  lbfgs_core(c, n * K, p, 0, ev, w_h, &b, n_iter, loss_out);
}

// multinomial_logistic_regression_model<T>::compute_probability_matrix
// (multinomial_logistic_regression_model.hpp:82-89), FP64.
void multinomial_probability(fvg_ctx* c, fvg_matrix* M, const double* w_h, const double* b_h, i64 K, int icpt_on,
                             double* prob_h) {
  if (K < 1 || K > (1 << 20)) fail(FVG_ERR_INVALID_ARG, "number of classes must be in [1, 2^20]");
  if (M->master != FVG_F64) fail(FVG_ERR_INVALID_ARG, "compute_probability_matrix needs FP64 values");
  const i64 m = M->A.m, n = M->A.n;
  cudaStream_t s = c->stream;
  DBuf W, ICPT;
  W.alloc(sizeof(double) * std::max<i64>(n * K, 1), s);
  ICPT.alloc(sizeof(double) * K, s);
  if (n) FVG_CUDA(cudaMemcpyAsync(W.p, w_h, sizeof(double) * n * K, cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(ICPT.p, b_h, sizeof(double) * K, cudaMemcpyHostToDevice, s));
  Softmax sm;
  sm.init(c, &M->A, M->master, FVG_F64, (int)K, nullptr, nullptr);
  if (m) {
    sm.forward(W.p, nullptr, nullptr, icpt_on, ICPT.as<double>());
    FVG_CUDA(cudaMemcpyAsync(prob_h, sm.Z.p, sizeof(double) * m * K, cudaMemcpyDeviceToHost, s));
  }
  FVG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace fvg
