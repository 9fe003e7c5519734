// Device helpers shared by the product kernels: fixed-order block sums,
// compensated accumulators, the per-row logistic loss/gradient and value
// widening.
#pragma once

#include "fvg_internal.cuh"

namespace fvg {

template <class T> __device__ __forceinline__ T block_sum256(T v) {
  __shared__ T red[8];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  T t = 0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < 8; q++) t += red[q];
  }
  return t;  // valid in thread 0
}

// ---------------------------------------------------- compensated sums
struct CSum {  // Neumaier, FP64 (the FP64 path)
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double v) {
    double t = s + v;
    if (fabs(s) >= fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ double total() const { return s + c; }
};
struct FSum {  // Kahan in FP32 (the FP32-arithmetic path keeps the FP64 unit idle)
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double total() const { return (double)s - (double)c; }
};
template <class AT> struct SumOf { using type = CSum; };
template <> struct SumOf<float> { using type = FSum; };

// Fixed-order block reduction of two compensated sums (256 threads).
__device__ __forceinline__ void block_csum2(double a, double b, double* out_a, double* out_b) {
  __shared__ double ra[256], rb[256];
  __syncthreads();
  ra[threadIdx.x] = a;
  rb[threadIdx.x] = b;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      ra[threadIdx.x] += ra[threadIdx.x + st];
      rb[threadIdx.x] += rb[threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out_a = ra[0];
    *out_b = rb[0];
  }
}

// ------------------------------------------------------- logistic math
// logistic_gradient<T>::compute_dloss for one row (gradient.hpp:24-50).
__device__ __forceinline__ void logistic_row(double wtx, double lab, double& loss, double& d) {
  double z = lab * wtx;
  double neg = lab * -1.0;
  if (z > 18.0) {
    double e = exp(-z);
    loss = e;
    d = e * neg;
  } else if (z < -18.0) {
    loss = -z;
    d = neg;
  } else {
    loss = log(1.0 + exp(-z));
    d = neg * (1.0 / (1.0 + exp(z)));
  }
  if (d > 1e12) d = 1e12;
  else if (d < -1e12) d = -1e12;
}
// FP32 variant for the BF16/FP32-storage path (log1p form keeps small
// losses that log(1+e) would round away in single precision).
__device__ __forceinline__ void logistic_row(float wtx, float lab, float& loss, float& d) {
  float z = lab * wtx;
  float neg = -lab;
  if (z > 18.0f) {
    float e = expf(-z);
    loss = e;
    d = e * neg;
  } else if (z < -18.0f) {
    loss = -z;
    d = neg;
  } else {
    loss = log1pf(expf(-z));
    d = neg / (1.0f + expf(z));
  }
  if (d > 1e12f) d = 1e12f;
  else if (d < -1e12f) d = -1e12f;
}

// The FP32 logistic row of the multi-model products with one exponential:
// e = exp(-|z|), 1 / (1 + exp(z)) = (z > 0 ? e : 1) / (1 + e) and
// log(1 + exp(-z)) = max(-z, 0) + log1p(e).  Every branch of
// gradient.hpp:24-50 is the same function: beyond |z| = 18 the reference's
// e and -z differ from these forms by less than e / 2 relative (below FP32
// resolution), so the result differs from logistic_row(float) by rounding.
__device__ __forceinline__ void logistic_row_1exp(float wtx, float lab, float& loss, float& d) {
  const float z = lab * wtx;
  const float e = expf(-fabsf(z));
  loss = fmaxf(-z, 0.0f) + log1pf(e);
  d = -lab * __fdividef(z > 0.0f ? e : 1.0f, 1.0f + e);
  if (d > 1e12f) d = 1e12f;
  else if (d < -1e12f) d = -1e12f;
}

// ------------------------------------------------------ GLM loss kinds
// compute_dloss of the GLM family for one row (ml/glm/gradient.hpp):
// 0 logistic_gradient, 1 linear_gradient (55-87), 2 hinge_gradient
// (89-121), 3 epsilon_insensitive (123-159), 4 squared_epsilon_insensitive
// (161-202).  MAX_LOSS / MIN_LOSS clip at ±1e12, HINGE_THRESHOLD = 1
// (gradient.hpp:8-10).  The squared loss comes back halved per row: the
// reference halves a rank's sum (70-73) and scaling by 0.5 is exact, so the
// halves add up to the same value.  The kind is uniform across a launch.
enum GlmLossKind { LOSS_LOGISTIC = 0, LOSS_SQUARED = 1, LOSS_HINGE = 2, LOSS_EPS = 3, LOSS_SQEPS = 4 };

template <class AT> __device__ __forceinline__ AT clip_dloss(AT d) {
  return d > (AT)1e12 ? (AT)1e12 : (d < (AT)-1e12 ? (AT)-1e12 : d);
}

template <class AT>
__device__ __forceinline__ void glm_row(int kind, AT eps, AT wtx, AT lab, AT& loss, AT& d) {
  if (kind == LOSS_LOGISTIC) {
    logistic_row(wtx, lab, loss, d);
  } else if (kind == LOSS_SQUARED) {
    const AT e = wtx - lab;
    loss = (AT)0.5 * (e * e);
    d = clip_dloss(e);
  } else if (kind == LOSS_HINGE) {
    const AT z = wtx * lab;
    const bool in = z <= (AT)1;
    loss = in ? (AT)1 - z : (AT)0;
    d = in ? -lab : (AT)0;
  } else {
    const AT z = lab - wtx;  // positive: the prediction is below the label
    const AT e = fabs(z) - eps;
    if (kind == LOSS_EPS) {
      loss = e > 0 ? e : (AT)0;
      d = z > eps ? (AT)-1 : ((wtx - lab) > eps ? (AT)1 : (AT)0);
    } else {
      loss = e > 0 ? e * e : (AT)0;
      d = z > eps ? (AT)-2 * (z - eps) : (z < -eps ? (AT)2 * (-z - eps) : (AT)0);
      d = clip_dloss(d);
    }
  }
}

template <class VT> __device__ __forceinline__ float to_f(VT v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<bf16>(bf16 v) { return __bfloat162float(v); }

template <class VT, class AT> __device__ __forceinline__ AT to_acc(VT v) { return (AT)to_f<VT>(v); }
template <> __device__ __forceinline__ double to_acc<double, double>(double v) { return v; }

// Streaming (evict-first) load of one value, widened to the accumulator.
template <class VT, class AT> __device__ __forceinline__ AT ld_val(const VT* q);
template <> __device__ __forceinline__ double ld_val<double, double>(const double* q) { return __ldcs(q); }
template <> __device__ __forceinline__ float ld_val<float, float>(const float* q) { return __ldcs(q); }
template <> __device__ __forceinline__ float ld_val<bf16, float>(const bf16* q) {
  return __uint_as_float((unsigned)__ldcs(reinterpret_cast<const unsigned short*>(q)) << 16);
}

}  // namespace fvg
