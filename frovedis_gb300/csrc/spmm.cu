// Multi-vector CRS products: Y = A X for a block of up to 64 columns of a
// row-major X (crs_matrix_spmm_impl, crs_matrix.hpp:2036-2050), and the
// batched logistic evaluation that trains several models on one matrix
// (one forward product A W for all models, the logistic epilogue per
// (row, model), one backward product A^T R).
//
// The kernel walks the same warp work items as the CRS SpMV (tiles of short
// rows, pieces of long rows, at most 512 nonzeros each).  For every nonzero
// the warp reads one row of X: lane L takes columns L and L+32, so a 64-column
// row is two coalesced 128-byte reads.  Column ids and values are loaded 32 at
// a time, one per lane, and broadcast with shuffles.  Pieces of long rows
// leave 64 partial sums each; the finalize kernel adds them in piece order.
// Loss and bias sums of the logistic epilogue are compensated per lane, then
// combined per CTA and across CTAs in a fixed order (deterministic).
#include "device_common.cuh"

namespace fvg {

constexpr int kSpmmCols = 64;  // columns per launch (two per lane)

struct SpmmK {
  const i32* off;
  const i32* idx;
  const void* val;
  const Item* items;
  i64 nitems;
  const void* X;  // first column of the block; row stride ldx
  i64 ldx;
  int kb;         // columns in this block (<= 64)
  void* Y;        // EPI_STORE output, row stride ldy
  i64 ldy;
  void* partials;  // [npieces][64] accumulator type
  // logistic epilogue (per column j < kb: intercept bias[j])
  const double* label;
  const double* sw;
  const float* label_f;
  const float* sw_f;
  int icpt;
  const double* bias;
  void* R;   // dloss*sw, accumulator type, row stride ldr
  i64 ldr;
  double* cta_part;  // [grid][64][2]: loss, bias
};

template <class VT, class XT, class AT>
__device__ __forceinline__ void row_dot(const SpmmK& p, i32 e0, i32 e1, int lane, bool c0, bool c1, AT& a0,
                                        AT& a1) {
  const XT* X = (const XT*)p.X;
  const VT* val = (const VT*)p.val;
  a0 = 0;
  a1 = 0;
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
      const XT* xr = X + (i64)col * p.ldx;
      if (c0) a0 += v * (AT)__ldg(xr + lane);
      if (c1) a1 += v * (AT)__ldg(xr + lane + 32);
    }
  }
}

template <class AT, class YT, int EPI, class S>
__device__ __forceinline__ void spmm_epi(const SpmmK& p, i32 row, AT a0, AT a1, AT b0, AT b1, int lane, bool c0,
                                         bool c1, S& l0, S& l1, S& s0, S& s1) {
  if (EPI == EPI_STORE) {
    YT* y = (YT*)p.Y + (i64)row * p.ldy;
    if (c0) y[lane] = (YT)a0;
    if (c1) y[lane + 32] = (YT)a1;
  } else {
    AT lab, w = 1;
    bool has_sw;
    if constexpr (sizeof(AT) == 8) {
      lab = p.label[row];
      has_sw = p.sw != nullptr;
      if (has_sw) w = p.sw[row];
    } else {
      lab = p.label_f[row];
      has_sw = p.sw_f != nullptr;
      if (has_sw) w = p.sw_f[row];
    }
    AT* r = (AT*)p.R + (i64)row * p.ldr;
    AT loss, d;
    if (c0) {
      logistic_row(a0 + b0, lab, loss, d);
      if (has_sw) d = d * w;
      r[lane] = d;
      l0.add(loss);
      s0.add(d);
    }
    if (c1) {
      logistic_row(a1 + b1, lab, loss, d);
      if (has_sw) d = d * w;
      r[lane + 32] = d;
      l1.add(loss);
      s1.add(d);
    }
  }
}

template <class VT, class XT, class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads) k_spmm(const SpmmK p) {
  using Sum = typename SumOf<AT>::type;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const i64 gw = (i64)blockIdx.x * (kThreads / 32) + wib;
  const i64 nw = (i64)gridDim.x * (kThreads / 32);
  const bool c0 = lane < p.kb, c1 = lane + 32 < p.kb;
  AT b0 = 0, b1 = 0;
  if (EPI == EPI_LOGREG && p.icpt) {
    if (c0) b0 = (AT)p.bias[lane];
    if (c1) b1 = (AT)p.bias[lane + 32];
  }
  Sum l0, l1, s0, s1;
  for (i64 it = gw; it < p.nitems; it += nw) {
    const Item item = p.items[it];
    AT a0, a1;
    if (item.r1 < 0) {  // piece of a long row
      row_dot<VT, XT, AT>(p, item.e0, item.e1, lane, c0, c1, a0, a1);
      AT* part = (AT*)p.partials + (i64)(-1 - item.r1) * kSpmmCols;
      part[lane] = a0;
      part[lane + 32] = a1;
    } else {
      for (i32 r = item.r0; r < item.r1; r++) {
        row_dot<VT, XT, AT>(p, __ldg(p.off + r), __ldg(p.off + r + 1), lane, c0, c1, a0, a1);
        spmm_epi<AT, YT, EPI>(p, r, a0, a1, b0, b1, lane, c0, c1, l0, l1, s0, s1);
      }
    }
  }
  if (EPI == EPI_LOGREG) {
    __shared__ double red[kThreads / 32][kSpmmCols][2];
    red[wib][lane][0] = l0.total();
    red[wib][lane][1] = s0.total();
    red[wib][lane + 32][0] = l1.total();
    red[wib][lane + 32][1] = s1.total();
    __syncthreads();
    if (threadIdx.x < 2 * kSpmmCols) {
      const int col = threadIdx.x & (kSpmmCols - 1), q = threadIdx.x / kSpmmCols;
      double t = 0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; w++) t += red[w][col][q];
      p.cta_part[((i64)blockIdx.x * kSpmmCols + col) * 2 + q] = t;
    }
  }
}

struct SpmmFin {
  SpmmK k;
  const i32* long_rows;
  const i32* long_piece0;
  i64 nlong;
  i64 ncta;
  double* fin_part;  // [gridDim][64][2]
  double* out;       // [kb][2]: loss, bias
  double* gbias;     // [kb] or null: where each column's bias lands
  unsigned* ticket;
};

// Long rows (a warp each): add the pieces' partials in piece order, apply the
// epilogue; then (logistic) the last CTA reduces all loss / bias partials per
// column in a fixed order.
template <class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads) k_spmm_fin(const SpmmFin f) {
  using Sum = typename SumOf<AT>::type;
  const SpmmK& p = f.k;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const bool c0 = lane < p.kb, c1 = lane + 32 < p.kb;
  AT b0 = 0, b1 = 0;
  if (EPI == EPI_LOGREG && p.icpt) {
    if (c0) b0 = (AT)p.bias[lane];
    if (c1) b1 = (AT)p.bias[lane + 32];
  }
  Sum l0, l1, s0, s1;
  for (i64 i = (i64)blockIdx.x * (kThreads / 32) + wib; i < f.nlong; i += (i64)gridDim.x * (kThreads / 32)) {
    const i64 q0 = f.long_piece0[i], q1 = f.long_piece0[i + 1];
    AT a0 = 0, a1 = 0;
    for (i64 q = q0; q < q1; q++) {
      const AT* part = (const AT*)p.partials + q * kSpmmCols;
      a0 += part[lane];
      a1 += part[lane + 32];
    }
    spmm_epi<AT, YT, EPI>(p, f.long_rows[i], a0, a1, b0, b1, lane, c0, c1, l0, l1, s0, s1);
  }
  if (EPI != EPI_LOGREG) return;
  __shared__ double red[kThreads / 32][kSpmmCols][2];
  __shared__ double half[2][2 * kSpmmCols];
  __shared__ bool last;
  red[wib][lane][0] = l0.total();
  red[wib][lane][1] = s0.total();
  red[wib][lane + 32][0] = l1.total();
  red[wib][lane + 32][1] = s1.total();
  __syncthreads();
  if (threadIdx.x < 2 * kSpmmCols) {
    const int col = threadIdx.x & (kSpmmCols - 1), q = threadIdx.x / kSpmmCols;
    double t = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; w++) t += red[w][col][q];
    f.fin_part[((i64)blockIdx.x * kSpmmCols + col) * 2 + q] = t;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(f.ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // thread t: column t % 64, quantity (t / 64) % 2, half t / 128 of the partials
  const int pair = threadIdx.x & (2 * kSpmmCols - 1), hf = threadIdx.x / (2 * kSpmmCols);
  const int col = pair & (kSpmmCols - 1), q = pair / kSpmmCols;
  CSum t;
  for (i64 b = hf; b < f.ncta; b += 2) t.add(__ldcg(&p.cta_part[(b * kSpmmCols + col) * 2 + q]));
  for (i64 b = hf; b < gridDim.x; b += 2) t.add(__ldcg(&f.fin_part[(b * kSpmmCols + col) * 2 + q]));
  half[hf][pair] = t.total();
  __syncthreads();
  if (threadIdx.x < 2 * kSpmmCols && col < p.kb) {
    const double tot = half[0][pair] + half[1][pair];
    if (q == 0) {
      f.out[2 * col] = tot;
    } else {
      f.out[2 * col + 1] = p.icpt ? tot : 0.0;
      if (f.gbias) f.gbias[col] = p.icpt ? tot : 0.0;
    }
  }
  if (threadIdx.x == 0) *f.ticket = 0u;
}

// ------------------------------------------------------------ host side
static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

template <class VT, class XT, class AT, class YT, int EPI>
static int spmm_grid(fvg_ctx* c) {
  static int blocks = -1;
  if (blocks < 0) {
    int nb = 0;
    FVG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_spmm<VT, XT, AT, YT, EPI>, kThreads, 0));
    blocks = std::max(1, nb);
  }
  return blocks * c->num_sms;
}

static int spmm_fin_grid(fvg_ctx* c, i64 nlong) {
  return (int)std::max<i64>(1, std::min<i64>((nlong + 7) / 8, 2 * c->num_sms));
}

// Scratch of one block pass: ticket, per-CTA partials of the main and
// finalize kernels, long-row piece partials.
i64 spmm_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage) {
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  const size_t at = storage == FVG_F64 ? 8 : 4;
  const i64 grid = 8 * (i64)c->num_sms;  // occupancy upper bound (8 CTAs of 256 threads per SM)
  return (i64)(al256(256) + al256(sizeof(double) * 2 * kSpmmCols * grid) +
               al256(sizeof(double) * 2 * kSpmmCols * spmm_fin_grid(c, s.nlong)) +
               al256(at * kSpmmCols * std::max<i64>(s.npieces, 1)));
}

template <class VT, class XT, class AT, class YT, int EPI>
static void launch_spmm(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, SpmmK p, double* out, double* gbias,
                        char* scratch) {
  const int grid = (int)std::max<i64>(1, std::min<i64>(spmm_grid<VT, XT, AT, YT, EPI>(c), (s.nitems + 7) / 8));
  const int fg = spmm_fin_grid(c, s.nlong);
  unsigned* ticket = (unsigned*)scratch;
  double* cta = (double*)(scratch + al256(256));
  double* fin = (double*)((char*)cta + al256(sizeof(double) * 2 * kSpmmCols * 8 * (i64)c->num_sms));
  p.partials = (char*)fin + al256(sizeof(double) * 2 * kSpmmCols * fg);
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.val = a.val[storage].p;
  p.items = s.items.as<Item>();
  p.nitems = s.nitems;
  p.cta_part = cta;
  if (s.nitems > 0) {
    k_spmm<VT, XT, AT, YT, EPI><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_spmm");
    count_launch(c);
  }
  if (s.nlong > 0 || EPI == EPI_LOGREG) {
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
    k_spmm_fin<AT, YT, EPI><<<fg, kThreads, 0, c->stream>>>(f);
    check_launch("k_spmm_fin");
    count_launch(c);
  }
}

// Y[:, c0:c0+kb] = A X[:, c0:c0+kb] (X, Y pointers already offset to c0).
void crs_spmm_block(fvg_ctx* c, DevCRS& a, int storage, const void* X, i64 ldx, int kb, int y_dt, void* Y, i64 ldy,
                    void* scratch) {
  if (kb < 1 || kb > kSpmmCols) fail(FVG_ERR_INTERNAL, "spmm block width out of range");
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
    launch_spmm<double, double, double, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc);
  } else if (storage == FVG_F32) {
    if (y_dt == FVG_F64) launch_spmm<float, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc);
    else launch_spmm<float, float, float, float, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc);
  } else {
    if (y_dt == FVG_F64) launch_spmm<bf16, float, float, double, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc);
    else launch_spmm<bf16, float, float, float, EPI_STORE>(c, a, s, storage, p, nullptr, nullptr, sc);
  }
}

// Batched logistic forward pass over a block of kb models: R = dloss(A W + b)
// * sw per (row, model); out[2j] = loss of model j, out[2j+1] = its bias sum
// (0 without intercept), also written to gbias[j] when given.
void crs_spmm_logreg_block(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int kb, const double* label,
                           const double* sw, const float* label_f, const float* sw_f, int icpt, const double* bias,
                           void* R, i64 ldr, double* out, double* gbias, void* scratch) {
  if (kb < 1 || kb > kSpmmCols) fail(FVG_ERR_INTERNAL, "spmm block width out of range");
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
  char* sc = (char*)scratch;
  FVG_CUDA(cudaMemsetAsync(sc, 0, 256, c->stream));
  if (storage == FVG_F64)
    launch_spmm<double, double, double, double, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc);
  else if (storage == FVG_F32)
    launch_spmm<float, float, float, float, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc);
  else
    launch_spmm<bf16, float, float, float, EPI_LOGREG>(c, a, s, storage, p, out, gbias, sc);
}

// Y = A X, X row-major num_col x k, Y row-major num_row x k, in blocks of 64
// columns.
void crs_spmm(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* X, i64 k, void* Y) {
  ProfScope pr(c, P_SPMM);
  if (a.m == 0 || k == 0) return;
  if (storage == FVG_F64 && x_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
  DBuf sc;
  sc.alloc((size_t)spmm_scratch_bytes(c, a, storage), c->stream);
  const size_t es = (size_t)dtype_size(x_dt);
  for (i64 c0 = 0; c0 < k; c0 += kSpmmCols) {
    const int kb = (int)std::min<i64>(kSpmmCols, k - c0);
    crs_spmm_block(c, a, storage, (const char*)X + c0 * es, k, kb, x_dt, (char*)Y + c0 * es, k, sc.p);
  }
}

}  // namespace fvg
