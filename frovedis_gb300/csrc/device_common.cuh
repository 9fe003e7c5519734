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
