// Double-FP32 ("df64") arithmetic for the split-value path.
//
// A number is an unevaluated sum h + l of two FP32 values with |l| <= ulp(h)
// (about 48 significant bits).  GB300 issues FP64 at a small fraction of its
// FP32 rate, so the split path keeps every per-nonzero and per-row operation
// on the FP32 pipe with error-free transformations:
//   * TwoSum (Knuth) and Fast2Sum (Dekker) give a + b exactly as s + e;
//   * an FMA gives a * b exactly as p + e (e = fma(a, b, -p)).
// Products, sums and the per-row loss/gradient of the GLM family reach about
// 1e-14 relative error; FP64 is used only for O(n) conversions.
//
// Every operation below is written with explicit round-to-nearest
// intrinsics, so the compiler neither contracts a multiply and an add into
// an FMA nor reorders the compensation terms.
#pragma once

#include "fvg_internal.cuh"

namespace fvg {

struct df {
  float h, l;
};

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float ap = __fsub_rn(s, bp);
  return {s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }
// a + b; error about 2^-46 of |a| + |b| (the "sloppy" double-word sum,
// enough for accumulations whose bound is the sum of magnitudes)
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.h, b.h);
  s.l = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return fast_two_sum(s.h, s.l);
}
// a + b with the low parts added through a second TwoSum: relative error
// about 2^-46 of |a + b| even under cancellation
__device__ __forceinline__ df df_add_acc(df a, df b) {
  df s = two_sum(a.h, b.h);
  const df t = two_sum(a.l, b.l);
  s.l = __fadd_rn(s.l, t.h);
  s = fast_two_sum(s.h, s.l);
  s.l = __fadd_rn(s.l, t.l);
  return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.h, b);
  s.l = __fadd_rn(s.l, a.l);
  return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return fast_two_sum(p, e);
}
// a / b: one reciprocal, one residual correction (relative error ~2^-46)
__device__ __forceinline__ df df_div(df a, df b) {
  const float rb = __frcp_rn(b.h);
  const float q1 = __fmul_rn(a.h, rb);
  const df r = df_add_acc(a, df_neg(df_mul_f(b, q1)));
  const float q2 = __fmul_rn(r.h, rb);
  return fast_two_sum(q1, q2);
}
// exact scaling by a power of two (no overflow / underflow in the callers)
__device__ __forceinline__ df df_scale(df a, float p2) { return {__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }

__device__ __forceinline__ df df_from_double(double d) {
  const float h = __double2float_rn(d);
  return {h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ float2 df_pack(df a) { return make_float2(a.h, a.l); }
__device__ __forceinline__ df df_unpack(float2 v) { return {v.x, v.y}; }

// Running sum of products p + t (p the rounded product, t its low part):
// TwoSum on the high parts, the errors and low parts added in s.l.
struct DfAcc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float p, float t) {
    const float sn = __fadd_rn(s, p);
    const float bp = __fsub_rn(sn, s);
    const float ap = __fsub_rn(sn, bp);
    const float err = __fadd_rn(__fsub_rn(s, ap), __fsub_rn(p, bp));
    c = __fadd_rn(c, __fadd_rn(err, t));
    s = sn;
  }
  __device__ __forceinline__ df get() const { return fast_two_sum(s, c); }
};

// Exact product of a split value (vh + vl) and a df vector entry, as p + t:
// vh*xh exactly via an FMA, the cross terms rounded once (about 2^-48 of
// the product; vl*xl is below that and dropped).
__device__ __forceinline__ void df_prod(float vh, float vl, float2 x, float& p, float& t) {
  p = __fmul_rn(vh, x.x);
  float e = __fmaf_rn(vh, x.x, -p);
  e = __fmaf_rn(vh, x.y, e);
  t = __fmaf_rn(vl, x.x, e);
}

// ------------------------------------------------------------ exp / log1p
// exp(x) by the table-driven method of P. T. P. Tang ("Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989), carried out in df64:
//   N = round(x * 64 / ln2), x = N * ln2/64 + r with |r| <= ln2/128,
//   exp(x) = 2^(N div 64) * 2^((N mod 64)/64) * exp(r),
//   exp(r) - 1 = r + r^2/2 + r^3/6 + r^4/24 + r^5/120 + r^6/720  (the next
//   term is below 3e-20).
// ln2/64 is split into c1 (12 significant bits, so N * c1 is exact for
// |N| < 2^12 ... and x - N*c1 is exact by Sterbenz' lemma), c2 and c3.
// The 64 table entries 2^(j/64) are df pairs filled from the host at
// context creation (df64_init in split.cu, the one translation unit that uses
// df_exp; the library is built without relocatable device code, so each unit
// including this header has its own copy).  Domain: x in [-87, 88]; below -87
// the result is 0 (the FP32 exponent range ends there).
static __device__ float2 g_exp2_tab[64];

__device__ __forceinline__ df df_exp(df x) {
  if (x.h < -87.f) return {0.f, 0.f};
  const float c1 = 0x1.62ep-7f, c2 = 0x1.0bfbe8p-21f, c3 = 0x1.cf79acp-46f;
  const float Nf = rintf(__fmul_rn(x.h, 0x1.715476p+6f));
  const int N = (int)Nf;
  const float a = __fmaf_rn(-Nf, c1, x.h);
  df r = two_sum(a, x.l);
  const float ph = __fmul_rn(Nf, c2);
  const float pl = __fmaf_rn(Nf, c2, -ph);
  r = df_add(r, {-ph, -pl});
  r = df_add_f(r, -__fmul_rn(Nf, c3));
  // tail r^3/6 + r^4/24 + r^5/120 + r^6/720 in FP32 (below 3e-8)
  const float rh = r.h;
  float q = __fmaf_rn(rh, 1.f / 720.f, 1.f / 120.f);
  q = __fmaf_rn(rh, q, 1.f / 24.f);
  q = __fmaf_rn(rh, q, 1.f / 6.f);
  q = __fmul_rn(__fmul_rn(__fmul_rn(rh, rh), rh), q);
  df s = df_add(r, df_scale(df_mul(r, r), 0.5f));
  s = df_add_f(s, q);
  const int j = N & 63;
  const int M = (N - j) / 64;
  const float2 t2 = g_exp2_tab[j];
  const df T = {t2.x, t2.y};
  df e = df_add(T, df_mul(T, s));
  return df_scale(e, __int_as_float((M + 127) << 23));
}

// log(1 + t) for t in [0, 1]: y0 = log1pf(t.h), then one Newton step on
// f(y) = exp(y) - (1 + t):  y1 = y0 - 1 + (1 + t) * exp(-y0).  The error of
// y0 (about 1e-7) becomes about 1e-14.  (Near t = 0 the absolute error stays
// at the df64 resolution of 1 + t, about 4e-15.)
__device__ __forceinline__ df df_log1p01(df t) {
  df u = two_sum(1.f, t.h);
  u.l = __fadd_rn(u.l, t.l);
  u = fast_two_sum(u.h, u.l);
  const float y0 = log1pf(t.h);
  const df E = df_exp({-y0, 0.f});
  const df P = df_mul(u, E);
  df c = two_sum(P.h, -1.f);
  c.l = __fadd_rn(c.l, P.l);
  return df_add_acc({y0, 0.f}, fast_two_sum(c.h, c.l));
}

// compare helpers on normalised pairs
__device__ __forceinline__ bool df_gt(df a, df b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ bool df_lt(df a, df b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ df df_abs(df a) { return (a.h < 0.f || (a.h == 0.f && a.l < 0.f)) ? df_neg(a) : a; }
__device__ __forceinline__ df df_clip(df d) {
  if (df_gt(d, {1e12f, 0.f})) return {1e12f, 0.f};
  if (df_lt(d, {-1e12f, 0.f})) return {-1e12f, 0.f};
  return d;
}

// compute_dloss of the GLM family for one row in df64 (gradient.hpp:15-202;
// kinds as GlmLossKind in device_common.cuh).  Logistic (gradient.hpp:24-50):
//   z = label * wtx;  z > 18: loss = e^-z, d = -label * e^-z;
//   z < -18: loss = -z, d = -label;  else loss = log(1 + e^-z),
//   d = -label / (1 + e^z);  d clipped to +-1e12.
// With t = e^-|z| the middle branch is log1p(t) (+ |z| when z < 0) and
// d = -label * t / (1 + t) (z >= 0) or -label / (1 + t) (z < 0): one exp.
__device__ __forceinline__ void glm_row_df(int kind, df eps, df wtx, df lab, df& loss, df& d) {
  if (kind == 0) {
    const df z = df_mul(lab, wtx);
    const df nl = df_neg(lab);
    if (z.h > 18.f || (z.h == 18.f && z.l > 0.f)) {
      const df e = df_exp(df_neg(z));
      loss = e;
      d = df_mul(e, nl);
    } else if (z.h < -18.f || (z.h == -18.f && z.l < 0.f)) {
      loss = df_neg(z);
      d = nl;
    } else {
      const bool neg = z.h < 0.f;
      const df az = neg ? df_neg(z) : z;
      const df t = df_exp(df_neg(az));
      const df u = df_add_f(t, 1.f);
      const df lp = df_log1p01(t);
      loss = neg ? df_add(lp, az) : lp;
      d = df_mul(nl, df_div(neg ? df{1.f, 0.f} : t, u));
    }
    d = df_clip(d);
  } else if (kind == 1) {  // linear_gradient: 0.5 * (wtx - label)^2
    const df e = df_add_acc(wtx, df_neg(lab));
    loss = df_scale(df_mul(e, e), 0.5f);
    d = df_clip(e);
  } else if (kind == 2) {  // hinge_gradient
    const df z = df_mul(wtx, lab);
    const bool in = !df_gt(z, {1.f, 0.f});
    loss = in ? df_add_acc({1.f, 0.f}, df_neg(z)) : df{0.f, 0.f};
    d = in ? df_neg(lab) : df{0.f, 0.f};
  } else {  // epsilon-insensitive (3) and its square (4)
    const df z = df_add_acc(lab, df_neg(wtx));
    const df e = df_add_acc(df_abs(z), df_neg(eps));
    const bool pos = df_gt(e, {0.f, 0.f});
    const df mz = df_neg(z);
    if (kind == 3) {
      loss = pos ? e : df{0.f, 0.f};
      d = df_gt(z, eps) ? df{-1.f, 0.f} : (df_gt(mz, eps) ? df{1.f, 0.f} : df{0.f, 0.f});
    } else {
      loss = pos ? df_mul(e, e) : df{0.f, 0.f};
      if (df_gt(z, eps)) d = df_scale(df_add_acc(z, df_neg(eps)), -2.f);
      else if (df_lt(z, df_neg(eps))) d = df_scale(df_add_acc(mz, df_neg(eps)), 2.f);
      else d = {0.f, 0.f};
      d = df_clip(d);
    }
  }
}

}  // namespace fvg

namespace fvg {

// ---------------------------------------------- chunked row segments
// One lane's chunk of C consecutive entries of a work item (products p + t,
// zero outside the lane's valid range), for the chunked split kernels.  B
// marks, relative to the chunk, every entry after the lane's first valid
// one at which a (non-empty) row starts.  The common case is branch-free:
// H = the entries before the first mark (the segment continuing the row open
// at the chunk's start), T = the entries from the last mark on (the segment
// of the row open at its end, or the whole chunk when nothing is marked).
template <int C>
__device__ __forceinline__ void chunk_segments(const float (&p)[C], const float (&t)[C], unsigned B, df& H, df& T) {
  const int fb = B ? __ffs(B) - 1 : C;   // first mark
  const int lb = B ? 31 - __clz(B) : -1;  // last mark
  DfAcc acc, head;
#pragma unroll
  for (int k = 0; k < C; k++) {
    const bool cap = k == fb, rst = k == lb;
    head.s = cap ? acc.s : head.s;
    head.c = cap ? acc.c : head.c;
    acc.s = rst ? 0.f : acc.s;
    acc.c = rst ? 0.f : acc.c;
    acc.add(p[k], t[k]);
  }
  H = B ? head.get() : df{0.f, 0.f};
  T = acc.get();
}

// chunk_segments that also records the rows starting and ending between two
// marks ("middle rows", for layouts whose rows are often shorter than a
// chunk): at every mark after the first, the sum since the previous mark is
// stored unnormalised as (s, c) at mid[pos0 + previous mark], one pass over
// the chunk instead of one chunk_range per middle row.
template <int C>
__device__ __forceinline__ void chunk_segments_mid(const float (&p)[C], const float (&t)[C], unsigned B, df& H,
                                                   df& T, float2* mid, int pos0) {
  const int fb = B ? __ffs(B) - 1 : C;  // first mark
  DfAcc acc, head;
  int prev = 0;  // the current segment's first entry (after the first mark)
#pragma unroll
  for (int k = 0; k < C; k++) {
    const bool mk = (B >> k) & 1u;
    const bool cap = k == fb;
    if (mk && !cap) mid[pos0 + prev] = make_float2(acc.s, acc.c);
    head.s = cap ? acc.s : head.s;
    head.c = cap ? acc.c : head.c;
    acc.s = mk ? 0.f : acc.s;
    acc.c = mk ? 0.f : acc.c;
    prev = mk ? k : prev;
    acc.add(p[k], t[k]);
  }
  H = B ? head.get() : df{0.f, 0.f};
  T = acc.get();
}

// Sum of the chunk's entries [a, b): rows that start and end between two
// marks (a second path, rarely taken where rows are longer than a chunk).
template <int C>
__device__ __forceinline__ df chunk_range(const float (&p)[C], const float (&t)[C], int a, int b) {
  DfAcc acc;
#pragma unroll
  for (int k = 0; k < C; k++) {
    const bool in = k >= a && k < b;
    acc.add(in ? p[k] : 0.f, in ? t[k] : 0.f);
  }
  return acc.get();
}

}  // namespace fvg
