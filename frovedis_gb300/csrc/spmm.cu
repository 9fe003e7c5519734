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
};

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
          VecLd<XT, CPL>::ld(X + (i64)col * p.ldx + lane * CPL, x);
#pragma unroll
          for (int q = 0; q < CPL; q++) a[q] += v * (AT)x[q];
        }
      } else {
        const XT* xr = X + (i64)col * p.ldx + lane;
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
                                         S (&ls)[CPL], S (&bs)[CPL]) {
#define ON(q) (colof<VEC, CPL>(lane, q) < p.kb)
  if (EPI == EPI_STORE) {
    YT* y = (YT*)p.Y + (i64)row * p.ldy;
    if constexpr (VEC) {
      if (lane * CPL < p.kb) {
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
};

// Long rows (a warp each): add the pieces' partials in piece order, apply the
// epilogue; then (logistic) the last CTA reduces all loss / bias partials per
// column in a fixed order.
template <class AT, class YT, int EPI, int CPL, bool VEC>
__global__ void __launch_bounds__(kThreads) k_spmm_fin(const SpmmFin f) {
  using Sum = typename SumOf<AT>::type;
  constexpr int NC = 32 * CPL;
  const SpmmK& p = f.k;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  AT b[CPL];
#pragma unroll
  for (int q = 0; q < CPL; q++) {
    const int c = colof<VEC, CPL>(lane, q);
    b[q] = (EPI != EPI_STORE && p.icpt && c < p.kb) ? (AT)p.bias[c] : (AT)0;
  }
  Sum ls[CPL], bs[CPL];
  for (i64 i = (i64)blockIdx.x * (kThreads / 32) + wib; i < f.nlong; i += (i64)gridDim.x * (kThreads / 32)) {
    const i64 q0 = f.long_piece0[i], q1 = f.long_piece0[i + 1];
    AT a[CPL];
#pragma unroll
    for (int q = 0; q < CPL; q++) a[q] = 0;
    for (i64 pc = q0; pc < q1; pc++) {
      const AT* part = (const AT*)p.partials + pc * NC;
#pragma unroll
      for (int q = 0; q < CPL; q++) a[q] += part[colof<VEC, CPL>(lane, q)];
    }
    spmm_epi<AT, YT, EPI, CPL, VEC>(p, f.long_rows[i], a, b, lane, ls, bs);
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
i64 spmm_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage) {
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
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
                    void* scratch) {
  if (kb < 1 || kb > kSpmmMaxCols) fail(FVG_ERR_INTERNAL, "spmm block width out of range");
  if (!a.val[storage].p) fail(FVG_ERR_INTERNAL, "missing value plane for the requested storage");
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  SpmmK p = {};
  p.X = X;
  p.ldx = ldx;
  p.kb = kb;
  p.Y = Y;
  p.ldy = ldy;
  char* sc = (char*)scratch;
  FVG_CUDA(cudaMemsetAsync(sc, 0, 256, c->stream));
  if (storage == FVG_F64) {
    launch_store<double, double, double, double>(c, a, s, storage, p, sc);
  } else if (storage == FVG_F32) {
    if (y_dt == FVG_F64) launch_store<float, float, float, double>(c, a, s, storage, p, sc);
    else launch_store<float, float, float, float>(c, a, s, storage, p, sc);
  } else {
    if (y_dt == FVG_F64) launch_store<bf16, float, float, double>(c, a, s, storage, p, sc);
    else launch_store<bf16, float, float, float>(c, a, s, storage, p, sc);
  }
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
  if (storage == FVG_F64)
    launch_spmm<double, double, double, double, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
  else if (storage == FVG_F32)
    launch_spmm<float, float, float, float, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
  else
    launch_spmm<bf16, float, float, float, EPI_LOGREG, 2>(c, a, s, storage, p, out, gbias, sc);
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
  if (storage == FVG_F64)
    launch_spmm<double, double, double, double, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
  else if (storage == FVG_F32)
    launch_spmm<float, float, float, float, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
  else
    launch_spmm<bf16, float, float, float, EPI_SOFTMAX, 4>(c, a, s, storage, p, loss_out, nullptr, sc);
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
