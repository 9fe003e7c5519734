// Multi-vector CRS products: Y = A X for a block of up to 128 columns of a
// row-major X (crs_matrix_spmm_impl, crs_matrix.hpp:2036-2050), with
// optional fused epilogues:
//  * logistic (batched binary training): R = dloss(A W + b) * sw per (row,
//    model) and per-model loss / bias sums (gradient.hpp:15-53);
//  * softmax (multinomial training): P = (softmax(A W + b) - onehot(label))
//    * sw per row (softmax_gradient_descent.hpp:140-235).
//
// The kernel walks the same warp work items as the CRS SpMV (tiles of short
// rows, pieces of long rows, at most 512 nonzeros each).  For every nonzero
// the warp reads one row of X: lane L takes columns L, L+32, ... (CPL columns
// per lane), so a row of X is read with coalesced 128-byte accesses.  Column
// ids and values are loaded 32 at a time, one per lane, and broadcast with
// shuffles.  Pieces of long rows leave 32*CPL partial sums each; the
// finalize kernel adds them in piece order.  Loss and bias sums of the
// logistic epilogue are compensated per lane, then combined per CTA and
// across CTAs in a fixed order (deterministic).
#include "device_common.cuh"

namespace fvg {

constexpr int kSpmmMaxCols = 128;  // columns per launch (four per lane)
constexpr int EPI_SOFTMAX = 2;

struct SpmmK {
  const i32* off;
  const i32* idx;
  const void* val;
  const Item* items;
  i64 nitems;
  const void* X;  // first column of the block; row stride ldx
  i64 ldx;
  int kb;         // columns in this block
  void* Y;        // EPI_STORE output, row stride ldy
  i64 ldy;
  void* partials;  // [npieces][32*CPL] accumulator type
  // epilogues
  const double* label;  // logistic: +-1; softmax: class id
  const double* sw;
  const float* label_f;
  const float* sw_f;
  int icpt;
  const double* bias;  // [kb] intercepts
  void* R;             // epilogue output (accumulator type), row stride ldr
  i64 ldr;
  double* cta_part;  // logistic: [grid][64][2] loss, bias
  int loss;          // GLM loss kind of the per-model epilogue
  double eps;
  // Stacked datasets (logistic epilogue): rows [seg_row[d], seg_row[d+1])
  // belong to dataset d, whose intercepts sit at bias + d * ldb.  Every warp
  // leaves one loss / bias partial per dataset in seg_part[d][warp] (zero
  // for the datasets it saw no row of); nseg = 0: one dataset, per-CTA
  // partials in cta_part.
  const i32* seg_row;
  int nseg;
  i64 ldb;
  double* seg_part;
  const int* gate;  // the launch does nothing while *gate == 0 (null: always runs)
  // Column masks of stacked datasets (null: every column): bit c of
  // mask[d * mstride + mword] set = column c of dataset d is computed;
  // masked columns are neither gathered nor written (their outputs keep
  // what they held) and their loss / bias sums are left out.
  const unsigned long long* mask;
  i64 mstride;
  int mword;
};

__device__ __forceinline__ unsigned long long mask_of(const SpmmK& p, int d) {
  return p.mask ? __ldcg(p.mask + (i64)d * p.mstride + p.mword) : ~0ull;
}
// column c (< 64 whenever a mask is given) is computed under mask word mw;
// all-ones = no mask
__device__ __forceinline__ bool col_on(unsigned long long mw, int c) {
  return mw == ~0ull || (c < 64 && ((mw >> c) & 1ull));
}
// any of the n columns c .. c + n - 1
__device__ __forceinline__ bool cols_on(unsigned long long mw, int c, int n) {
  return mw == ~0ull || (c < 64 && ((mw >> c) & ((1ull << n) - 1)) != 0);
}

__device__ __forceinline__ bool gated_off(const int* gate) { return gate && __ldcg(gate) == 0; }

// Lane layouts of the block's columns.  Strided (VEC = false): lane L owns
// columns L, L+32, ...; every load is one element.  Packed (VEC = true):
// lane L owns columns CPL*L .. CPL*L+CPL-1 and reads / writes them with one
// vector access (needs ldx, the output stride and kb to be multiples of CPL
// and CPL-aligned bases).  Each column's sum runs over the nonzeros in the
// same order in both layouts; only the softmax denominator's lane partials
// group the classes differently.
template <bool VEC, int CPL> __device__ __forceinline__ int colof(int lane, int q) {
  return VEC ? lane * CPL + q : lane + 32 * q;
}

// CPL consecutive elements at an aligned address
template <class XT, int CPL> struct VecLd;
template <int CPL> struct VecLd<float, CPL> {
  static __device__ __forceinline__ void ld(const float* x, float (&o)[CPL]) {
    if constexpr (CPL == 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(x));
      o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    } else if constexpr (CPL == 2) {
      const float2 v = __ldg(reinterpret_cast<const float2*>(x));
      o[0] = v.x; o[1] = v.y;
    } else {
      o[0] = __ldg(x);
    }
  }
};
template <int CPL> struct VecLd<double, CPL> {
  static __device__ __forceinline__ void ld(const double* x, double (&o)[CPL]) {
#pragma unroll
    for (int h = 0; h < CPL; h += 2) {
      if constexpr (CPL >= 2) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(x + h));
        o[h] = v.x; o[h + 1] = v.y;
      } else {
        o[0] = __ldg(x);
      }
    }
  }
};

// CPL consecutive elements stored at an aligned address
template <class T, int CPL> __device__ __forceinline__ void vec_st(T* y, const T (&v)[CPL]) {
  if constexpr (sizeof(T) == 4 && CPL == 4) {
    *reinterpret_cast<float4*>(y) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (sizeof(T) == 4 && CPL == 2) {
    *reinterpret_cast<float2*>(y) = make_float2(v[0], v[1]);
  } else if constexpr (sizeof(T) == 8 && CPL >= 2) {
#pragma unroll
    for (int h = 0; h < CPL; h += 2) *reinterpret_cast<double2*>(y + h) = make_double2(v[h], v[h + 1]);
  } else {
#pragma unroll
    for (int q = 0; q < CPL; q++) y[q] = v[q];
  }
}

template <class VT, class XT, class AT, int CPL, bool VEC>
__device__ __forceinline__ void row_dot(const SpmmK& p, i32 e0, i32 e1, int lane, AT (&a)[CPL]) {
  const XT* X = (const XT*)p.X;
  const VT* val = (const VT*)p.val;
#pragma unroll
  for (int q = 0; q < CPL; q++) a[q] = 0;
  const bool mine = !VEC || lane * CPL < p.kb;
  for (i32 e = e0; e < e1; e += 32) {
    const int cnt = min(32, e1 - e);
    i32 mi = 0;
    AT mv = 0;
    if (lane < cnt) {
      mi = __ldcs(p.idx + e + lane);
      mv = ld_val<VT, AT>(val + e + lane);
    }
#pragma unroll 4
    for (int t = 0; t < cnt; t++) {
      const i32 col = __shfl_sync(0xffffffffu, mi, t);
      const AT v = __shfl_sync(0xffffffffu, mv, t);
      if constexpr (VEC) {
        if (mine) {
          XT x[CPL];
          VecLd<XT, CPL>::ld(X + (long long)col * (int)p.ldx + lane * CPL, x);
#pragma unroll
          for (int q = 0; q < CPL; q++) a[q] += v * (AT)x[q];
        }
      } else {
        const XT* xr = X + (long long)col * (int)p.ldx + lane;
#pragma unroll
        for (int q = 0; q < CPL; q++)
          if (lane + 32 * q < p.kb) a[q] += v * (AT)__ldg(xr + 32 * q);
      }
    }
  }
}

template <class AT> __device__ __forceinline__ AT exp_acc(AT x);
template <> __device__ __forceinline__ double exp_acc<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float exp_acc<float>(float x) { return expf(x); }
template <class AT> __device__ __forceinline__ AT log_acc(AT x);
template <> __device__ __forceinline__ double log_acc<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float log_acc<float>(float x) { return logf(x); }

template <class AT, class YT, int EPI, int CPL, bool VEC, class S>
__device__ __forceinline__ void spmm_epi(const SpmmK& p, i32 row, const AT (&a)[CPL], const AT (&b)[CPL], int lane,
                                         S (&ls)[CPL], S (&bs)[CPL], unsigned long long mw = ~0ull) {
#define ON(q) (colof<VEC, CPL>(lane, q) < p.kb && col_on(mw, colof<VEC, CPL>(lane, q)))
  if (EPI == EPI_STORE) {
    YT* y = (YT*)p.Y + (i64)row * p.ldy;
    if constexpr (VEC) {
      if (mw != ~0ull) {
#pragma unroll
        for (int q = 0; q < CPL; q++)
          if (ON(q)) y[colof<VEC, CPL>(lane, q)] = (YT)a[q];
      } else if (lane * CPL < p.kb) {
        YT o[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) o[q] = (YT)a[q];
        vec_st<YT, CPL>(y + lane * CPL, o);
      }
    } else {
#pragma unroll
      for (int q = 0; q < CPL; q++)
        if (ON(q)) y[colof<VEC, CPL>(lane, q)] = (YT)a[q];
    }
    return;
  }
  // softmax without labels: the probability matrix alone (compute_probability_matrix)
  const bool has_label = (sizeof(AT) == 8) ? p.label != nullptr : p.label_f != nullptr;
  AT lab = 0, w = 1;
  bool has_sw = false;
  if (has_label) {
    if constexpr (sizeof(AT) == 8) {
      lab = p.label[row];
      has_sw = p.sw != nullptr;
      if (has_sw) w = p.sw[row];
    } else {
      lab = p.label_f[row];
      has_sw = p.sw_f != nullptr;
      if (has_sw) w = p.sw_f[row];
    }
  }
  AT* r = (AT*)p.R + (i64)row * p.ldr;
  AT out[CPL];
  if (EPI == EPI_LOGREG) {
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      out[q] = 0;
      if (!ON(q)) continue;
      AT loss, d;
      glm_row<AT>(p.loss, (AT)p.eps, a[q] + b[q], lab, loss, d);
      if (has_sw) d = d * w;
      out[q] = d;
      ls[q].add(loss);
      bs[q].add(d);
    }
  } else {  // EPI_SOFTMAX: compute_exp_matrix, compute_softmax_probability, compute_error_inplace
    AT z[CPL], mx = -INFINITY;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      z[q] = a[q] + b[q];
      if (ON(q)) mx = fmax(mx, z[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    // the label's margin z_label - max, for the cross-entropy
    AT zy = 0;
    if (has_label)
#pragma unroll
      for (int q = 0; q < CPL; q++)
        if (ON(q) && lab == (AT)colof<VEC, CPL>(lane, q)) zy = z[q] - mx;
    AT sum = 0;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      z[q] = ON(q) ? exp_acc<AT>(z[q] - mx) : (AT)0;
      sum += z[q];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    // cross-entropy -log p[label] = log(sum) - (z_label - max), unweighted,
    // into lane 0's first partial (the L-BFGS line search's loss)
    if (has_label && p.cta_part) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) zy += __shfl_xor_sync(0xffffffffu, zy, o);
      if (lane == 0) ls[0].add(log_acc<AT>(sum) - zy);
    }
    const AT inv = (AT)1 / sum;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      AT pr = inv * z[q];
      if (has_label) {
        pr -= (lab == (AT)colof<VEC, CPL>(lane, q)) ? (AT)1 : (AT)0;
        if (has_sw) pr *= w;
      }
      out[q] = pr;
    }
  }
  if constexpr (VEC) {
    if (lane * CPL < p.kb) vec_st<AT, CPL>(r + lane * CPL, out);
  } else {
#pragma unroll
    for (int q = 0; q < CPL; q++)
      if (ON(q)) r[colof<VEC, CPL>(lane, q)] = out[q];
  }
#undef ON
}

template <class VT, class XT, class AT, class YT, int EPI, int CPL, bool VEC>
__global__ void __launch_bounds__(kThreads, 4) k_spmm(const SpmmK p) {
  using Sum = typename SumOf<AT>::type;
  constexpr int NC = 32 * CPL;
  if (gated_off(p.gate)) return;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const i64 gw = (i64)blockIdx.x * (kThreads / 32) + wib;
  const i64 nw = (i64)gridDim.x * (kThreads / 32);
  AT b[CPL];
#pragma unroll
  for (int q = 0; q < CPL; q++) {
    const int c = colof<VEC, CPL>(lane, q);
    b[q] = (EPI != EPI_STORE && p.icpt && c < p.kb) ? (AT)p.bias[c] : (AT)0;
  }
  Sum ls[CPL], bs[CPL];
  for (i64 it = gw; it < p.nitems; it += nw) {
    const Item item = p.items[it];
    AT a[CPL];
    if (item.r1 < 0) {  // piece of a long row
      row_dot<VT, XT, AT, CPL, VEC>(p, item.e0, item.e1, lane, a);
      AT* part = (AT*)p.partials + (i64)(-1 - item.r1) * NC;
#pragma unroll
      for (int q = 0; q < CPL; q++) part[colof<VEC, CPL>(lane, q)] = a[q];
    } else {
      for (i32 r = item.r0; r < item.r1; r++) {
        row_dot<VT, XT, AT, CPL, VEC>(p, __ldg(p.off + r), __ldg(p.off + r + 1), lane, a);
        spmm_epi<AT, YT, EPI, CPL, VEC>(p, r, a, b, lane, ls, bs);
      }
    }
  }
  if constexpr (EPI == EPI_LOGREG || EPI == EPI_SOFTMAX) if (EPI == EPI_LOGREG || p.cta_part) {
    __shared__ double red[kThreads / 32][NC][2];
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      red[wib][colof<VEC, CPL>(lane, q)][0] = ls[q].total();
      red[wib][colof<VEC, CPL>(lane, q)][1] = bs[q].total();
    }
    __syncthreads();
    if (threadIdx.x < 2 * NC) {
      const int col = threadIdx.x % NC, qq = threadIdx.x / NC;
      double t = 0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; w++) t += red[w][col][qq];
      p.cta_part[((i64)blockIdx.x * NC + col) * 2 + qq] = t;
    }
  }
}

struct SpmmFin {
  SpmmK k;
  const i32* long_rows;
  const i32* long_piece0;
  i64 nlong;
  i64 ncta;
  double* fin_part;  // [gridDim][NC][2]
  double* out;       // [kb][2]: loss, bias
  double* gbias;     // [kb] or null: where each column's bias lands
  unsigned* ticket;
  double* seg_fpart;  // stacked datasets: [nseg][warps][NC][2] of this kernel
};

// ------------------------------------------------ stacked-dataset partials
// A warp meets its rows in increasing order, so the datasets it visits come
// in order too: SegWalk keeps the current one, and when a row of a later
// dataset arrives it stores the warp's loss / bias sums of the current one
// in its slot, zeros in the slots of the datasets skipped, and loads the
// next dataset's intercepts.  finish() stores the last sums and zeros the
// remaining slots: every warp writes each of its nseg slots exactly once, so
// the reduction reads all of them in warp order without a memset.
template <class AT, int QN> struct SegWalk {
  using Sum = typename SumOf<AT>::type;
  int d = 0;
  i32 end = 0;
  double* slots;  // this warp's slot of dataset 0; slot d at + d * stride
  i64 stride;
  __device__ __forceinline__ SegWalk(const SpmmK& p, double* base, i64 warp, i64 nwarps, int nc)
      : end(p.nseg > 0 ? __ldg(p.seg_row + 1) : 0x7fffffff), slots(base ? base + warp * nc * 2 : nullptr),
        stride(nwarps * nc * 2) {}
  __device__ __forceinline__ void put(int dd, const int (&col)[QN], Sum (&ls)[QN], Sum (&bs)[QN]) {
    if (!slots) return;
    double* s = slots + dd * stride;
#pragma unroll
    for (int q = 0; q < QN; q++) {
      s[2 * col[q]] = ls[q].total();
      s[2 * col[q] + 1] = bs[q].total();
      ls[q] = Sum();
      bs[q] = Sum();
    }
  }
  __device__ __forceinline__ void zero(int dd, const int (&col)[QN]) {
    if (!slots) return;
    double* s = slots + dd * stride;
#pragma unroll
    for (int q = 0; q < QN; q++) {
      s[2 * col[q]] = 0.0;
      s[2 * col[q] + 1] = 0.0;
    }
  }
  // row r (warp-uniform) is next; true when the dataset changed
  __device__ __forceinline__ bool to_row(const SpmmK& p, i32 r, const int (&col)[QN], Sum (&ls)[QN], Sum (&bs)[QN]) {
    if (r < end) return false;
    put(d, col, ls, bs);
    d++;
    while (r >= __ldg(p.seg_row + d + 1)) zero(d++, col);
    end = __ldg(p.seg_row + d + 1);
    return true;
  }
  // the dataset of row r wherever it lies (schedules whose items are not in
  // row order; no sums are kept then)
  __device__ __forceinline__ void seek(const SpmmK& p, i32 r) {
    int lo = 0, hi = p.nseg - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(p.seg_row + mid) <= r) lo = mid;
      else hi = mid - 1;
    }
    d = lo;
    end = __ldg(p.seg_row + d + 1);
  }
  __device__ __forceinline__ void finish(const SpmmK& p, const int (&col)[QN], Sum (&ls)[QN], Sum (&bs)[QN]) {
    if (!slots) return;
    put(d, col, ls, bs);
    for (int dd = d + 1; dd < p.nseg; dd++) zero(dd, col);
  }
};

// Long rows (a warp each): add the pieces' partials in piece order, apply the
// epilogue; then (logistic) the last CTA reduces all loss / bias partials per
// column in a fixed order.
template <class AT, class YT, int EPI, int CPL, bool VEC>
__global__ void __launch_bounds__(kThreads) k_spmm_fin(const SpmmFin f) {
  using Sum = typename SumOf<AT>::type;
  constexpr int NC = 32 * CPL;
  const SpmmK& p = f.k;
  if (gated_off(p.gate)) return;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const bool track = p.nseg > 0;                  // stacked datasets
  const bool seg = EPI == EPI_LOGREG && track;    // per-dataset loss slots
  AT b[CPL];
  auto load_bias = [&](const double* bias) {
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      const int c = colof<VEC, CPL>(lane, q);
      b[q] = (EPI != EPI_STORE && p.icpt && c < p.kb) ? (AT)bias[c] : (AT)0;
    }
  };
  load_bias(p.bias);
  Sum ls[CPL], bs[CPL];
  int cols[CPL];
#pragma unroll
  for (int q = 0; q < CPL; q++) cols[q] = colof<VEC, CPL>(lane, q);
  const i64 gw = (i64)blockIdx.x * (kThreads / 32) + wib, nw = (i64)gridDim.x * (kThreads / 32);
  SegWalk<AT, CPL> sw(p, seg ? f.seg_fpart : nullptr, gw, nw, NC);
  unsigned long long mw = mask_of(p, 0);
  for (i64 i = gw; i < f.nlong; i += nw) {
    const i64 q0 = f.long_piece0[i], q1 = f.long_piece0[i + 1];
    const i32 row = f.long_rows[i];
    if (track && sw.to_row(p, row, cols, ls, bs)) {
      if (EPI == EPI_LOGREG) load_bias(p.bias + sw.d * p.ldb);
      mw = mask_of(p, sw.d);
    }
    if (mw == 0) continue;
    AT a[CPL];
#pragma unroll
    for (int q = 0; q < CPL; q++) a[q] = 0;
    for (i64 pc = q0; pc < q1; pc++) {
      const AT* part = (const AT*)p.partials + pc * NC;
#pragma unroll
      for (int q = 0; q < CPL; q++) a[q] += part[colof<VEC, CPL>(lane, q)];
    }
    spmm_epi<AT, YT, EPI, CPL, VEC>(p, row, a, b, lane, ls, bs, mw);
  }
  if (track && !seg) return;
  if (seg) {
    sw.finish(p, cols, ls, bs);
    return;
  }
  if constexpr (EPI == EPI_LOGREG || EPI == EPI_SOFTMAX) if (EPI == EPI_LOGREG || p.cta_part) {
    __shared__ double red[kThreads / 32][NC][2];
    __shared__ double half[2][2 * NC];
    __shared__ bool last;
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      red[wib][colof<VEC, CPL>(lane, q)][0] = ls[q].total();
      red[wib][colof<VEC, CPL>(lane, q)][1] = bs[q].total();
    }
    __syncthreads();
    if (threadIdx.x < 2 * NC) {
      const int col = threadIdx.x % NC, qq = threadIdx.x / NC;
      double t = 0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; w++) t += red[w][col][qq];
      f.fin_part[((i64)blockIdx.x * NC + col) * 2 + qq] = t;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(f.ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    if constexpr (EPI == EPI_SOFTMAX) {
      // the cross-entropy sits in column 0's loss partials: thread t adds
      // CTAs t, t + 256, ... of both kernels, then a fixed tree
      CSum t;
      for (i64 bb = threadIdx.x; bb < f.ncta; bb += kThreads) t.add(__ldcg(&p.cta_part[(bb * NC) * 2]));
      for (i64 bb = threadIdx.x; bb < gridDim.x; bb += kThreads) t.add(__ldcg(&f.fin_part[(bb * NC) * 2]));
      double tl = 0.0, tb = 0.0;
      block_csum2(t.total(), 0.0, &tl, &tb);
      if (threadIdx.x == 0) {
        f.out[0] = tl;
        f.out[1] = 0.0;
        *f.ticket = 0u;
      }
      return;
    } else {
    // (column, quantity) pairs over the threads, two halves of the partials
    // each; 2*NC pairs must fit in half the CTA
    static_assert(EPI != EPI_LOGREG || 4 * NC <= kThreads, "logistic epilogue: too many columns per launch");
    const int pair = threadIdx.x % (2 * NC), hf = threadIdx.x / (2 * NC);
    const int col = pair % NC, qq = pair / NC;
    CSum t;
    if (hf < 2) {
      for (i64 bb = hf; bb < f.ncta; bb += 2) t.add(__ldcg(&p.cta_part[(bb * NC + col) * 2 + qq]));
      for (i64 bb = hf; bb < gridDim.x; bb += 2) t.add(__ldcg(&f.fin_part[(bb * NC + col) * 2 + qq]));
      half[hf][pair] = t.total();
    }
    __syncthreads();
    if (threadIdx.x < 2 * NC && col < p.kb) {
      const double tot = half[0][pair] + half[1][pair];
      if (qq == 0) {
        f.out[2 * col] = tot;
      } else {
        f.out[2 * col + 1] = p.icpt ? tot : 0.0;
        if (f.gbias) f.gbias[col] = p.icpt ? tot : 0.0;
      }
    }
    if (threadIdx.x == 0) *f.ticket = 0u;
    }
  }
}

// ------------------------------------------------ grouped lane layout
// For the store, logistic and softmax epilogues with aligned rows of X: lane
// (group g, sub-lane s) of G groups of LPR = 32 / G lanes reads columns
// s*CPL .. s*CPL+CPL-1 of a row of X with one load (CPL = 8 FP32 values,
// 32 bytes, or 2 FP64 values, 16 bytes), and group g takes nonzeros g,
// g+G, g+2G, ... of every 32-entry chunk, so a warp gathers G rows of X per
// step.  FP32 products are accumulated with packed two-lane FMAs
// (fma.rn.f32x2: each half rounds like a scalar FMA).  At the end of a row
// the groups' sums meet in a fixed butterfly that leaves lane (g, s) with the
// QG = CPL / G columns s*CPL + g*QG ... of the row (reduce-scatter), which it
// runs the epilogue on.  A launch covers NC = LPR * CPL columns; pieces and
// the per-CTA partials use the column order of the finalize kernel with
// NC / 32 columns a lane.  Each column's sum is the group sums added in the
// butterfly's fixed order (deterministic; it differs from the
// one-nonzero-at-a-time order only by rounding).
template <class XT, int G> struct GLay {
  static constexpr int CPL = sizeof(XT) == 4 ? 8 : 2;
  static constexpr int LPR = 32 / G;
  static constexpr int NC = LPR * CPL;
  static constexpr int QG = CPL / G;
  static_assert(G >= 1 && G <= CPL && NC <= 128, "groups per warp");
};

__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// acc = v * x + acc on both FP32 halves
__device__ __forceinline__ void fma2(unsigned long long& acc, unsigned long long v, unsigned long long x) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(v), "l"(x));
}

// A chunk of 32 entries staged for the warp: the row offset of the gathered
// row of X (column id x stride) and the value, zero past the chunk's end.
template <class AT> struct alignas(16) StageE {
  long long off;
  AT v;
};

template <class VT, class XT, class AT, int G>
__device__ __forceinline__ void row_dot_g(const SpmmK& p, i32 e0, i32 e1, int lane, AT (&a)[GLay<XT, G>::CPL],
                                          StageE<AT>* st, bool lane_on = true) {
  using L = GLay<XT, G>;
  constexpr int CPL = L::CPL;
  constexpr bool PACK = sizeof(XT) == 4 && sizeof(AT) == 4;
  const int sub = lane % L::LPR, grp = lane / L::LPR;
  const XT* X = (const XT*)p.X + sub * CPL;
  const int ldx = (int)p.ldx;  // a row stride of X fits 32 bits
  const VT* val = (const VT*)p.val;
  const bool mine = lane_on && sub * CPL < p.kb;
  unsigned long long acc[CPL / 2];  // packed FP32 pairs
#pragma unroll
  for (int q = 0; q < CPL; q++) a[q] = 0;
#pragma unroll
  for (int q = 0; q < CPL / 2; q++) acc[q] = 0ull;
  for (i32 e = e0; e < e1; e += 32) {
    const int cnt = min(32, e1 - e);
    // stage the chunk (offsets computed once per entry); the padding
    // entries (offset 0, value 0) round the chunk up to whole steps
    StageE<AT> se;
    se.off = 0;
    se.v = 0;
    if (lane < cnt) {
      se.off = (long long)__ldcs(p.idx + e + lane) * ldx;
      se.v = ld_val<VT, AT>(val + e + lane);
    }
    __syncwarp();
    st[lane] = se;
    __syncwarp();
    // group grp takes entries grp, grp + G, ...; lanes whose columns are
    // not computed skip the chunk
    if (mine) {
      const int steps = (cnt + G - 1) / G;
#pragma unroll 4
      for (int k = 0; k < steps; k++) {
        const StageE<AT> t = st[k * G + grp];
        const XT* xp = X + t.off;
        if constexpr (PACK) {
          // the lane's 8 FP32 columns in one 32-byte load, as 4 packed pairs
          static_assert(CPL == 8, "one 32-byte load a lane");
          unsigned long long x0, x1, x2, x3;
          asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];"
              : "=l"(x0), "=l"(x1), "=l"(x2), "=l"(x3)
              : "l"(xp));
          const unsigned long long vv = pack2((float)t.v, (float)t.v);
          fma2(acc[0], vv, x0);
          fma2(acc[1], vv, x1);
          fma2(acc[2], vv, x2);
          fma2(acc[3], vv, x3);
        } else {
          XT x[CPL];
          VecLd<XT, CPL>::ld(xp, x);
#pragma unroll
          for (int q = 0; q < CPL; q++) a[q] += t.v * (AT)x[q];
        }
      }
    }
  }
  if constexpr (PACK) {
#pragma unroll
    for (int q = 0; q < CPL / 2; q++) {
      float lo, hi;
      unpack2(acc[q], lo, hi);
      a[2 * q] = lo;
      a[2 * q + 1] = hi;
    }
  }
  // reduce-scatter over the groups: at offset o the lane keeps the half of
  // its columns picked by bit o of its lane id and sends the other half
#pragma unroll
  for (int o = 16, h = CPL / 2; o >= L::LPR; o >>= 1, h >>= 1) {
    const bool hi = (lane & o) != 0;
#pragma unroll
    for (int q = 0; q < h; q++) {
      const AT keep = hi ? a[h + q] : a[q];
      const AT send = hi ? a[q] : a[h + q];
      a[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
}

template <class VT, class XT, class AT, class YT, int EPI, int G>
__global__ void __launch_bounds__(kThreads, 4) k_spmm_g(const SpmmK p) {
  using L = GLay<XT, G>;
  using Sum = typename SumOf<AT>::type;
  constexpr int CPL = L::CPL, NC = L::NC, QG = L::QG;
  if (gated_off(p.gate)) return;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int c0 = (lane % L::LPR) * CPL + (lane / L::LPR) * QG;  // first of the lane's epilogue columns
  const i64 gw = (i64)blockIdx.x * (kThreads / 32) + wib;
  const i64 nw = (i64)gridDim.x * (kThreads / 32);
  const bool track = p.nseg > 0;                // stacked datasets
  const bool seg = EPI == EPI_LOGREG && track;  // per-dataset loss slots
  int cols[QG];
#pragma unroll
  for (int q = 0; q < QG; q++) cols[q] = c0 + q;
  AT b[QG];
  auto load_bias = [&](const double* bias) {
#pragma unroll
    for (int q = 0; q < QG; q++) b[q] = (EPI != EPI_STORE && p.icpt && cols[q] < p.kb) ? (AT)bias[cols[q]] : (AT)0;
  };
  load_bias(p.bias);
  Sum ls[QG], bs[QG];
  SegWalk<AT, QG> walk(p, seg ? p.seg_part : nullptr, gw, nw, NC);
  const int lsh = (lane % L::LPR) * CPL;  // the lane's gathered columns: lsh .. lsh + CPL - 1
  __shared__ StageE<AT> stage[kThreads / 32][32];
  unsigned long long mw = mask_of(p, 0);
  AT lab = 0, w = 1;
  for (i64 it = gw; it < p.nitems; it += nw) {
    const Item item = p.items[it];
    AT a[CPL];
    // the store epilogue keeps no per-dataset sums, so its items may come in
    // any order (slab-ordered pieces): each item looks its dataset up
    if (EPI == EPI_STORE && track) {
      walk.seek(p, item.r0);
      mw = mask_of(p, walk.d);
    }
    if (item.r1 < 0) {  // piece of a long row (item.r0)
      if (EPI != EPI_STORE && track && walk.to_row(p, item.r0, cols, ls, bs)) {
        if (EPI == EPI_LOGREG) load_bias(p.bias + walk.d * p.ldb);
        mw = mask_of(p, walk.d);
      }
      if (mw == 0) continue;  // the finalize skips the row too
      row_dot_g<VT, XT, AT, G>(p, item.e0, item.e1, lane, a, stage[wib], cols_on(mw, lsh, CPL));
      AT* part = (AT*)p.partials + (i64)(-1 - item.r1) * NC;
#pragma unroll
      for (int q = 0; q < QG; q++) part[cols[q]] = a[q];
      continue;
    }
    for (i32 r = item.r0; r < item.r1; r++) {
      if (track && walk.to_row(p, r, cols, ls, bs)) {
        if (EPI == EPI_LOGREG) load_bias(p.bias + walk.d * p.ldb);
        mw = mask_of(p, walk.d);
      }
      if (mw == 0) continue;  // no column of this dataset is computed
      row_dot_g<VT, XT, AT, G>(p, __ldg(p.off + r), __ldg(p.off + r + 1), lane, a, stage[wib], cols_on(mw, lsh, CPL));
      if constexpr (EPI == EPI_STORE) {
        YT* y = (YT*)p.Y + (i64)r * p.ldy;
#pragma unroll
        for (int q = 0; q < QG; q++)
          if (cols[q] < p.kb && col_on(mw, cols[q])) y[cols[q]] = (YT)a[q];
      } else {
        // labels: always with the logistic epilogue; the softmax one runs
        // without them for the probability matrix alone
        const bool has_label = (sizeof(AT) == 8) ? p.label != nullptr : p.label_f != nullptr;
        bool has_sw = false;
        if (has_label) {
          if constexpr (sizeof(AT) == 8) {
            lab = p.label[r];
            has_sw = p.sw != nullptr;
            if (has_sw) w = p.sw[r];
          } else {
            lab = p.label_f[r];
            has_sw = p.sw_f != nullptr;
            if (has_sw) w = p.sw_f[r];
          }
        }
        AT* rr = (AT*)p.R + (i64)r * p.ldr;
        if constexpr (EPI == EPI_LOGREG) {
#pragma unroll
          for (int q = 0; q < QG; q++) {
            if (cols[q] >= p.kb || !col_on(mw, cols[q])) continue;
            AT loss, d;
            if constexpr (sizeof(AT) == 4) {
              if (p.loss == LOSS_LOGISTIC) logistic_row_1exp(a[q] + b[q], lab, loss, d);
              else glm_row<AT>(p.loss, (AT)p.eps, a[q] + b[q], lab, loss, d);
            } else {
              glm_row<AT>(p.loss, (AT)p.eps, a[q] + b[q], lab, loss, d);
            }
            if (has_sw) d = d * w;
            rr[cols[q]] = d;
            ls[q].add(loss);
            bs[q].add(d);
          }
        } else {  // softmax over the row's classes, every class held by one lane
          AT z[QG], mx = -INFINITY;
#pragma unroll
          for (int q = 0; q < QG; q++) {
            z[q] = a[q] + b[q];
            if (cols[q] < p.kb) mx = fmax(mx, z[q]);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
          AT zy = 0, sum = 0;
#pragma unroll
          for (int q = 0; q < QG; q++) {
            if (has_label && cols[q] < p.kb && lab == (AT)cols[q]) zy = z[q] - mx;
            z[q] = cols[q] < p.kb ? exp_acc<AT>(z[q] - mx) : (AT)0;
            sum += z[q];
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
          // cross-entropy -log p[label] = log(sum) - (z_label - max), unweighted
          if (has_label && p.cta_part) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) zy += __shfl_xor_sync(0xffffffffu, zy, o);
            if (lane == 0) ls[0].add(log_acc<AT>(sum) - zy);
          }
          const AT inv = (AT)1 / sum;
#pragma unroll
          for (int q = 0; q < QG; q++) {
            if (cols[q] >= p.kb) continue;
            AT pr = inv * z[q];
            if (has_label) {
              pr -= (lab == (AT)cols[q]) ? (AT)1 : (AT)0;
              if (has_sw) pr *= w;
            }
            rr[cols[q]] = pr;
          }
        }
      }
    }
  }
  if (track && !seg) return;
  if constexpr (EPI == EPI_LOGREG || EPI == EPI_SOFTMAX) {
    if (EPI == EPI_SOFTMAX && !p.cta_part) return;
    if (seg) {
      walk.finish(p, cols, ls, bs);
      return;
    }
    __shared__ double red[kThreads / 32][NC][2];
#pragma unroll
    for (int q = 0; q < QG; q++) {
      red[wib][cols[q]][0] = ls[q].total();
      red[wib][cols[q]][1] = bs[q].total();
    }
    __syncthreads();
    if (threadIdx.x < 2 * NC) {
      const int col = threadIdx.x % NC, qq = threadIdx.x / NC;
      double t = 0;
#pragma unroll
      for (int w8 = 0; w8 < kThreads / 32; w8++) t += red[w8][col][qq];
      p.cta_part[((i64)blockIdx.x * NC + col) * 2 + qq] = t;
    }
  }
}

// Stacked datasets: loss / bias sums of dataset blockIdx.x from the warp
// slots of the main kernel (nw1 warps) and the finalize kernel (nw2), each
// in warp order.  A CTA of 1024 threads takes 32 (column, quantity) pairs
// (blockIdx.y: which 32) x 32 stripes; stripe s adds warps s, s + 32, ...;
// the stripes are added in order.  out[2 * (d * ldo + col) + q]; the bias
// sums also go to gb[grow[d] * ldg + col].
template <int NC>
__global__ void __launch_bounds__(1024) k_spmm_seg_reduce(const double* __restrict__ s1, i64 nw1,
                                                          const double* __restrict__ s2, i64 nw2, int kout, int icpt,
                                                          double* __restrict__ out, i64 ldo, double* __restrict__ gb,
                                                          const i64* __restrict__ grow, i64 ldg, const int* gate,
                                                          const unsigned long long* mask, i64 mstride, int mword) {
  constexpr int P = 2 * NC, S = 32;
  static_assert(P % 32 == 0, "pairs per CTA");
  __shared__ double part[S][33];
  if (gated_off(gate)) return;
  const int d = blockIdx.x;
  const int pl = threadIdx.x & 31, st = threadIdx.x >> 5;
  const int pr = blockIdx.y * 32 + pl;
  CSum t;
  const double* b1 = s1 + (i64)d * nw1 * P;
  for (i64 w = st; w < nw1; w += S) t.add(__ldcg(b1 + w * P + pr));
  const double* b2 = s2 + (i64)d * nw2 * P;
  for (i64 w = st; w < nw2; w += S) t.add(__ldcg(b2 + w * P + pr));
  part[st][pl] = t.total();
  __syncthreads();
  if (st != 0) return;
  double tot = 0.0;
#pragma unroll
  for (int q = 0; q < S; q++) tot += part[q][pl];
  const int col = pr >> 1, qq = pr & 1;
  if (col >= kout) return;
  if (mask && !col_on(__ldcg(mask + (i64)d * mstride + mword), col)) return;  // not evaluated: keep
  if (qq == 0) {
    out[2 * ((i64)d * ldo + col)] = tot;
  } else {
    out[2 * ((i64)d * ldo + col) + 1] = icpt ? tot : 0.0;
    if (gb) gb[grow[d] * ldg + col] = icpt ? tot : 0.0;
  }
}

// ------------------------------------------------------------ host side
static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class VT, class XT, class AT, class YT, int EPI, int CPL, bool VEC>
static int spmm_grid(fvg_ctx* c) {
  return occupancy_blocks((const void*)k_spmm<VT, XT, AT, YT, EPI, CPL, VEC>, kThreads) * c->num_sms;
}

static int spmm_fin_grid(fvg_ctx* c, i64 nlong) {
  return (int)std::max<i64>(1, std::min<i64>((nlong + 7) / 8, 2 * c->num_sms));
}

// Scratch of one block pass (sized for 128 columns): ticket, per-CTA
// partials of the main and finalize kernels, long-row piece partials.
i64 spmm_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage, i64 slab) {
  const Sched& s = slab > 0 ? crs_sched_slabs(c, a, tile_for_storage(storage), slab)
                            : crs_sched(c, a, tile_for_storage(storage));
  const size_t at = storage == FVG_F64 ? 8 : 4;
  const i64 grid = 8 * (i64)c->num_sms;  // occupancy upper bound (8 CTAs of 256 threads per SM)
  return (i64)(al256(256) + al256(sizeof(double) * 2 * kSpmmMaxCols * grid) +
               al256(sizeof(double) * 2 * kSpmmMaxCols * spmm_fin_grid(c, s.nlong)) +
               al256(at * kSpmmMaxCols * std::max<i64>(s.npieces, 1)));
}

template <class VT, class XT, class AT, class YT, int EPI, int CPL, bool VEC>
static void launch_spmm_l(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, SpmmK p, double* out, double* gbias,
                          char* scratch) {
  const int grid =
      (int)std::max<i64>(1, std::min<i64>(spmm_grid<VT, XT, AT, YT, EPI, CPL, VEC>(c), (s.nitems + 7) / 8));
  const int fg = spmm_fin_grid(c, s.nlong);
  unsigned* ticket = (unsigned*)scratch;
  double* cta = (double*)(scratch + al256(256));
  double* fin = (double*)((char*)cta + al256(sizeof(double) * 2 * kSpmmMaxCols * 8 * (i64)c->num_sms));
  p.partials = (char*)fin + al256(sizeof(double) * 2 * kSpmmMaxCols * fg);
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.val = a.val[storage].p;
  p.items = s.items.as<Item>();
  p.nitems = s.nitems;
  // softmax: the cross-entropy is reduced only when the caller asks for it
  const bool reduce = EPI == EPI_LOGREG || (EPI == EPI_SOFTMAX && out);
  p.cta_part = reduce ? cta : nullptr;
  if (s.nitems > 0) {
    k_spmm<VT, XT, AT, YT, EPI, CPL, VEC><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_spmm");
    count_launch(c);
  }
  if (s.nlong > 0 || reduce) {
    SpmmFin f;
    f.k = p;
    f.long_rows = s.long_rows.as<i32>();
    f.long_piece0 = s.long_piece0.as<i32>();
    f.nlong = s.nlong;
    f.ncta = s.nitems > 0 ? grid : 0;
    f.fin_part = fin;
    f.out = out;
    f.gbias = gbias;
    f.ticket = ticket;
    k_spmm_fin<AT, YT, EPI, CPL, VEC><<<fg, kThreads, 0, c->stream>>>(f);
    check_launch("k_spmm_fin");
    count_launch(c);
  }
}

static bool aligned_to(const void* ptr, size_t b) { return ((uintptr_t)ptr % b) == 0; }

// Grouped layout launch: k_spmm_g and its finalize kernel (NC / 32
// columns a lane); for stacked datasets the slot reduction is left to
// crs_spmm_seg_finish.
template <class VT, class XT, class AT, class YT, int EPI, int G>
static void launch_grouped_l(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, SpmmK p, double* out,
                             double* gbias, char* scratch, SpmmSeg* sg) {
  using L = GLay<XT, G>;
  constexpr int NC = L::NC, CF = NC / 32;
  const int grid = (int)std::max<i64>(
      1, std::min<i64>(occupancy_blocks((const void*)k_spmm_g<VT, XT, AT, YT, EPI, G>, kThreads) * c->num_sms,
                       (s.nitems + 7) / 8));
  const int fg = spmm_fin_grid(c, s.nlong);
  unsigned* ticket = (unsigned*)scratch;
  double* cta = (double*)(scratch + al256(256));
  double* fin = (double*)((char*)cta + al256(sizeof(double) * 2 * kSpmmMaxCols * 8 * (i64)c->num_sms));
  p.partials = (char*)fin + al256(sizeof(double) * 2 * kSpmmMaxCols * fg);
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.val = a.val[storage].p;
  p.items = s.items.as<Item>();
  p.nitems = s.nitems;
  // softmax: the cross-entropy is reduced only when the caller asks for it
  const bool reduce = EPI == EPI_LOGREG || (EPI == EPI_SOFTMAX && out);
  p.cta_part = reduce ? cta : nullptr;
  const bool track = sg && sg->nseg > 0;
  const bool seg = EPI == EPI_LOGREG && track;
  const i64 nw1 = (i64)grid * (kThreads / 32), nw2 = (i64)fg * (kThreads / 32);
  if (track) {
    if (!sg->seg_row || (seg && !sg->slots) || sg->nseg > 65535)
      fail(FVG_ERR_INTERNAL, "stacked-dataset pass without its row bounds or slots");
    if (sg->mask && p.kb > 64) fail(FVG_ERR_INTERNAL, "column masks cover 64 columns");
    p.nseg = sg->nseg;
    p.seg_row = sg->seg_row;
    p.ldb = sg->ldb;
    p.seg_part = seg ? sg->slots : nullptr;
    p.gate = sg->gate;
    p.mask = sg->mask;
    p.mstride = sg->mstride;
    p.mword = sg->mword;
  }
  if (s.nitems > 0 || seg) {
    k_spmm_g<VT, XT, AT, YT, EPI, G><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_spmm_g");
    count_launch(c);
  }
  if (s.nlong > 0 || reduce) {
    SpmmFin f;
    f.k = p;
    f.long_rows = s.long_rows.as<i32>();
    f.long_piece0 = s.long_piece0.as<i32>();
    f.nlong = s.nlong;
    f.ncta = s.nitems > 0 ? grid : 0;
    f.fin_part = fin;
    f.out = out;
    f.gbias = gbias;
    f.ticket = ticket;
    f.seg_fpart = seg ? sg->slots + (i64)sg->nseg * nw1 * NC * 2 : nullptr;
    k_spmm_fin<AT, YT, EPI, CF, true><<<fg, kThreads, 0, c->stream>>>(f);
    check_launch("k_spmm_fin");
    count_launch(c);
  }
  if (seg) {
    sg->nw1 = nw1;
    sg->nw2 = nw2;
    sg->nc = NC;
    sg->icpt = p.icpt;
  }
}

// Grouped layout when its 16-byte accesses are aligned; false: not taken.
template <class VT, class XT, class AT, class YT, int EPI>
static bool launch_grouped(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, const SpmmK& p, double* out,
                           double* gbias, char* scratch, SpmmSeg* sg = nullptr) {
  // vector loads: column blocks and strides in whole vectors (the FP32
  // lanes read 8 columns, the FP64 ones 2), 16-byte aligned bases
  constexpr int VW = 16 / (int)sizeof(XT);
  bool ok = p.kb % VW == 0 && p.ldx % VW == 0 && aligned_to(p.X, 16);
  if (EPI == EPI_STORE) ok = ok && p.ldy % VW == 0 && aligned_to(p.Y, 16);
  else ok = ok && p.ldr % VW == 0 && aligned_to(p.R, 16);
  if (!ok) return false;
  if constexpr (sizeof(XT) == 4) {
    // FP32: 8 columns a lane read with one 32-byte load: whole 8-column
    // groups, 32-byte aligned rows
    if (p.kb % 8 != 0 || p.ldx % 8 != 0 || p.kb > 128 || !aligned_to(p.X, 32)) return false;
    if (p.kb <= 32) {
      launch_grouped_l<VT, XT, AT, YT, EPI, 8>(c, a, s, storage, p, out, gbias, scratch, sg);
      return true;
    }
    if (p.kb <= 64) {
      launch_grouped_l<VT, XT, AT, YT, EPI, 4>(c, a, s, storage, p, out, gbias, scratch, sg);
      return true;
    }
    // the logistic epilogue's finalize reduction takes at most 64 columns
    if constexpr (EPI != EPI_LOGREG) {
      launch_grouped_l<VT, XT, AT, YT, EPI, 2>(c, a, s, storage, p, out, gbias, scratch, sg);
      return true;
    }
    return false;
  } else {
    if (p.kb > 64) return false;
    if (p.kb <= 32) launch_grouped_l<VT, XT, AT, YT, EPI, 2>(c, a, s, storage, p, out, gbias, scratch, sg);
    else launch_grouped_l<VT, XT, AT, YT, EPI, 1>(c, a, s, storage, p, out, gbias, scratch, sg);
    return true;
  }
}

// Packed lane layout when every access it makes is aligned: the block's
// width and the strides of X and of the output are multiples of CPL and the
// bases are aligned to CPL elements.
template <class VT, class XT, class AT, class YT, int EPI, int CPL>
static void launch_spmm(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, SpmmK p, double* out, double* gbias,
                        char* scratch) {
  bool vec = CPL >= 2 && p.kb % CPL == 0 && p.ldx % CPL == 0 && aligned_to(p.X, CPL * sizeof(XT));
  if (EPI == EPI_STORE) vec = vec && p.ldy % CPL == 0 && aligned_to(p.Y, CPL * sizeof(YT));
  else vec = vec && p.ldr % CPL == 0 && aligned_to(p.R, CPL * sizeof(AT));
  if constexpr (CPL >= 2) {
    if (vec) {
      launch_spmm_l<VT, XT, AT, YT, EPI, CPL, true>(c, a, s, storage, p, out, gbias, scratch);
      return;
    }
  }
  launch_spmm_l<VT, XT, AT, YT, EPI, CPL, false>(c, a, s, storage, p, out, gbias, scratch);
}

template <class VT, class XT, class AT, class YT>
static void launch_store(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, const SpmmK& p, char* sc) {
  if (p.kb <= 32) launch_spmm<VT, XT, AT, YT, EPI_STORE, 1>(c, a, s, storage, p, nullptr, nullptr, sc);
  else if (p.kb <= 64) launch_spmm<VT, XT, AT, YT, EPI_STORE, 2>(c, a, s, storage, p, nullptr, nullptr, sc);
  else launch_spmm<VT, XT, AT, YT, EPI_STORE, 4>(c, a, s, storage, p, nullptr, nullptr, sc);
}

// Y[:, c0:c0+kb] = A X[:, c0:c0+kb] (X, Y pointers already offset to c0).
void crs_spmm_block(fvg_ctx* c, DevCRS& a, int storage, const void* X, i64 ldx, int kb, int y_dt, void* Y, i64 ldy,
                    void* scratch, const int* gate, i64 slab) {
  if (kb < 1 || kb > kSpmmMaxCols) fail(FVG_ERR_INTERNAL, "spmm block width out of range");
  if (!a.val[storage].p) fail(FVG_ERR_INTERNAL, "missing value plane for the requested storage");
  const Sched& s = slab > 0 ? crs_sched_slabs(c, a, tile_for_storage(storage), slab)
                            : crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = X;
  p.ldx = ldx;
  if (ldx > 0x7fffffffll) fail(FVG_ERR_INVALID_ARG, "dense operand row stride beyond 2^31 - 1");
  p.kb = kb;
  p.Y = Y;
  p.ldy = ldy;
  p.gate = gate;
  char* sc = (char*)scratch;
  if (storage == FVG_F64) {
    if (!launch_grouped<double, double, double, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc))
      launch_store<double, double, double, double>(c, a, s, storage, p, sc);
  } else if (storage == FVG_F32) {
    if (y_dt == FVG_F64) {
      if (!launch_grouped<float, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc))
        launch_store<float, float, float, double>(c, a, s, storage, p, sc);
    } else if (!launch_grouped<float, float, float, float, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc)) {
      launch_store<float, float, float, float>(c, a, s, storage, p, sc);
    }
  } else {
    if (y_dt == FVG_F64) {
      if (!launch_grouped<bf16, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc))
        launch_store<bf16, float, float, double>(c, a, s, storage, p, sc);
    } else if (!launch_grouped<bf16, float, float, float, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc)) {
      launch_store<bf16, float, float, float>(c, a, s, storage, p, sc);
    }
  }
}

// Y = A X over stacked datasets (rows [seg_row[d], seg_row[d+1]) of A belong
// to dataset d) with the column masks and the gate of sg; masked columns of
// Y keep what they held.  X, Y and their strides 16-byte aligned, kb a
// multiple of 8 (of 2 for FP64) and at most 64.
void crs_spmm_store_seg(fvg_ctx* c, DevCRS& a, int storage, const void* X, i64 ldx, int kb, void* Y, i64 ldy,
                        void* scratch, SpmmSeg& sg, i64 slab) {
  if (kb < 1 || kb > 64 || sg.nseg < 1) fail(FVG_ERR_INTERNAL, "stacked store: block width or datasets out of range");
  if (!a.val[storage].p) fail(FVG_ERR_INTERNAL, "missing value plane for the requested storage");
  const Sched& s = slab > 0 ? crs_sched_slabs(c, a, tile_for_storage(storage), slab)
                            : crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = X;
  p.ldx = ldx;
  if (ldx > 0x7fffffffll) fail(FVG_ERR_INVALID_ARG, "dense operand row stride beyond 2^31 - 1");
  p.kb = kb;
  p.Y = Y;
  p.ldy = ldy;
  char* sc = (char*)scratch;
  bool ok;
  if (storage == FVG_F64)
    ok = launch_grouped<double, double, double, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  else if (storage == FVG_F32)
    ok = launch_grouped<float, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  else
    ok = launch_grouped<bf16, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  if (!ok) fail(FVG_ERR_INTERNAL, "stacked store needs 16-byte aligned rows");
}

// Batched GLM forward pass over a block of kb <= 64 models: R = dloss(A W +
// b) * sw per (row, model) for the loss kind `loss`; out[2j] = loss of model
// j, out[2j+1] = its bias sum (0 without intercept), also written to gbias[j]
// when given.
void crs_spmm_logreg_block(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int kb, const double* label,
                           const double* sw, const float* label_f, const float* sw_f, int icpt, const double* bias,
                           void* R, i64 ldr, double* out, double* gbias, void* scratch, int loss, double eps) {
  if (kb < 1 || kb > 64) fail(FVG_ERR_INTERNAL, "spmm block width out of range");
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = W;
  p.ldx = ldw;
  if (ldw > 0x7fffffffll) fail(FVG_ERR_INVALID_ARG, "dense operand row stride beyond 2^31 - 1");
  p.kb = kb;
  p.label = label;
  p.sw = sw;
  p.label_f = label_f;
  p.sw_f = sw_f;
  p.icpt = icpt;
  p.bias = bias;
  p.R = R;
  p.ldr = ldr;
  p.loss = loss;
  p.eps = eps;
  char* sc = (char*)scratch;
  FVG_CUDA(cudaMemsetAsync(sc, 0, 256, c->stream));
  if (storage == FVG_F64) {
    if (!launch_grouped<double, double, double, double, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc))
      launch_spmm<double, double, double, double, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
  } else if (storage == FVG_F32) {
    if (!launch_grouped<float, float, float, float, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc))
      launch_spmm<float, float, float, float, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
  } else if (!launch_grouped<bf16, float, float, float, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc)) {
    launch_spmm<bf16, float, float, float, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
  }
}

// Warp slots of a stacked-dataset pass: main kernel (at most 8 CTAs an SM)
// and finalize kernel, NC = the launch's columns, two doubles each.
i64 spmm_seg_slot_bytes(fvg_ctx* c, int nseg, int kb) {
  const i64 nc = kb <= 32 ? 32 : (kb <= 64 ? 64 : 128);
  const i64 warps = (8 * (i64)c->num_sms + 2 * (i64)c->num_sms) * (kThreads / 32);
  return (i64)std::max(nseg, 1) * warps * nc * 2 * (i64)sizeof(double);
}

void crs_spmm_logreg_seg(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int kb, const double* label,
                         const double* sw, const float* label_f, const float* sw_f, int icpt, const double* bias,
                         void* R, i64 ldr, void* scratch, SpmmSeg& sg, int loss, double eps) {
  if (kb < 1 || kb > 64 || sg.nseg < 1) fail(FVG_ERR_INTERNAL, "stacked pass: block width or datasets out of range");
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = W;
  p.ldx = ldw;
  if (ldw > 0x7fffffffll) fail(FVG_ERR_INVALID_ARG, "dense operand row stride beyond 2^31 - 1");
  p.kb = kb;
  p.label = label;
  p.sw = sw;
  p.label_f = label_f;
  p.sw_f = sw_f;
  p.icpt = icpt;
  p.bias = bias;
  p.R = R;
  p.ldr = ldr;
  p.loss = loss;
  p.eps = eps;
  char* sc = (char*)scratch;
  bool ok;
  if (storage == FVG_F64)
    ok = launch_grouped<double, double, double, double, EPI_LOGREG>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  else if (storage == FVG_F32)
    ok = launch_grouped<float, float, float, float, EPI_LOGREG>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  else
    ok = launch_grouped<bf16, float, float, float, EPI_LOGREG>(c, a, s, storage, p, nullptr, nullptr, sc, &sg);
  if (!ok) fail(FVG_ERR_INTERNAL, "stacked pass needs 16-byte aligned rows");
}

// Per-dataset loss / bias sums of the last crs_spmm_logreg_seg pass (after
// the backward product, which writes the bias rows of the gradient as 0).
void crs_spmm_seg_finish(fvg_ctx* c, const SpmmSeg& sg) {
  if (sg.nw1 <= 0) fail(FVG_ERR_INTERNAL, "stacked-dataset reduction without its pass");
  const double* s2 = sg.slots + (i64)sg.nseg * sg.nw1 * sg.nc * 2;
  if (sg.nc == 32)
    k_spmm_seg_reduce<32><<<dim3(sg.nseg, 2), 1024, 0, c->stream>>>(sg.slots, sg.nw1, s2, sg.nw2, sg.kout, sg.icpt, sg.out,
                                                           sg.ldo, sg.gb, sg.grow, sg.ldg, sg.gate, sg.mask,
                                                           sg.mstride, sg.mword);
  else if (sg.nc == 64)
    k_spmm_seg_reduce<64><<<dim3(sg.nseg, 4), 1024, 0, c->stream>>>(sg.slots, sg.nw1, s2, sg.nw2, sg.kout, sg.icpt, sg.out,
                                                           sg.ldo, sg.gb, sg.grow, sg.ldg, sg.gate, sg.mask,
                                                           sg.mstride, sg.mword);
  else
    k_spmm_seg_reduce<128><<<dim3(sg.nseg, 8), 1024, 0, c->stream>>>(sg.slots, sg.nw1, s2, sg.nw2, sg.kout, sg.icpt, sg.out,
                                                            sg.ldo, sg.gb, sg.grow, sg.ldg, sg.gate, sg.mask,
                                                           sg.mstride, sg.mword);
  check_launch("k_spmm_seg_reduce");
  count_launch(c);
}

// Multinomial forward pass, K <= 128 classes: P = (softmax(A W + icpt) -
// onehot(label)) * sw, row-major [m][ldp] of the accumulator type; with
// loss_out (device, 2 * K doubles) also the cross-entropy sum in loss_out[0].
void crs_spmm_softmax(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int K, const double* label,
                      const double* sw, const float* label_f, const float* sw_f, int icpt, const double* icpt_v,
                      void* P, i64 ldp, void* scratch, double* loss_out) {
  if (K < 1 || K > kSpmmMaxCols) fail(FVG_ERR_INTERNAL, "softmax block width out of range");
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = W;
  p.ldx = ldw;
  if (ldw > 0x7fffffffll) fail(FVG_ERR_INVALID_ARG, "dense operand row stride beyond 2^31 - 1");
  p.kb = K;
  p.label = label;
  p.sw = sw;
  p.label_f = label_f;
  p.sw_f = sw_f;
  p.icpt = icpt;
  p.bias = icpt_v;
  p.R = P;
  p.ldr = ldp;
  char* sc = (char*)scratch;
  FVG_CUDA(cudaMemsetAsync(sc, 0, 256, c->stream));
  if (storage == FVG_F64) {
    if (!launch_grouped<double, double, double, double, EPI_SOFTMAX>(c, a, s, storage, p, loss_out, nullptr, sc))
      launch_spmm<double, double, double, double, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
  } else if (storage == FVG_F32) {
    if (!launch_grouped<float, float, float, float, EPI_SOFTMAX>(c, a, s, storage, p, loss_out, nullptr, sc))
      launch_spmm<float, float, float, float, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
  } else if (!launch_grouped<bf16, float, float, float, EPI_SOFTMAX>(c, a, s, storage, p, loss_out, nullptr, sc)) {
    launch_spmm<bf16, float, float, float, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
  }
}

// Y = A X, X row-major num_col x k, Y row-major num_row x k, in blocks of 128
// columns.
void crs_spmm(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* X, i64 k, void* Y) {
  ProfScope pr(c, P_SPMM);
  if (a.m == 0 || k == 0) return;
  if (storage == FVG_F64 && x_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
  DBuf sc;
  sc.alloc((size_t)spmm_scratch_bytes(c, a, storage), c->stream);
  const size_t es = (size_t)dtype_size(x_dt);
  for (i64 c0 = 0; c0 < k; c0 += kSpmmMaxCols) {
    const int kb = (int)std::min<i64>(kSpmmMaxCols, k - c0);
    crs_spmm_block(c, a, storage, (const char*)X + c0 * es, k, kb, x_dt, (char*)Y + c0 * es, k, sc.p);
  }
}

}  // namespace fvg
