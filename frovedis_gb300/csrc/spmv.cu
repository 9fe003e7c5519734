// Sparse products on the device.
//
// CRS (crs_matrix_spmv_impl, crs_matrix.hpp:1505-1516): one persistent,
// row-binned kernel.  Rows are grouped by length (row bins, see build.cu);
// a row of bin b is read by 2^b lanes (b = 0..5), by a whole CTA (bin 6), or
// split into fixed chunks whose partial sums the finalize kernel adds in
// chunk order (bin 7).  Every lane streams 16-byte vectors of column ids and
// values (4 elements for FP64/FP32 values, 8 for BF16) with no-L1-allocate
// loads, and gathers x through the read-only path.  All reductions have a
// fixed order, so results are deterministic run to run.
//
// The optional logistic epilogue fuses compute_wtx + logistic_gradient::
// compute_dloss + `* sample_weight` + bias sum (gradient_descent.hpp:196-211,
// gradient.hpp:15-53) into the same pass: it writes dloss*sw per row and
// per-CTA compensated FP64 partial sums of the loss and of dloss*sw, which
// the finalize kernel reduces in a fixed order.
#include "fvg_internal.cuh"

namespace fvg {

// ---------------------------------------------------------------- loads
__device__ __forceinline__ void ld_idx4(const i32* p, int& a, int& b, int& c, int& d) {
  asm("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
      : "=r"(a), "=r"(b), "=r"(c), "=r"(d)
      : "l"(p));
}
__device__ __forceinline__ void ld_f64x2(const double* p, double& a, double& b) {
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];" : "=d"(a), "=d"(b) : "l"(p));
}
__device__ __forceinline__ void ld_f32x4(const float* p, float& a, float& b, float& c, float& d) {
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
      : "=f"(a), "=f"(b), "=f"(c), "=f"(d)
      : "l"(p));
}
__device__ __forceinline__ void ld_u32x4(const void* p, unsigned& a, unsigned& b, unsigned& c, unsigned& d) {
  asm("ld.global.nc.L1::no_allocate.v4.b32 {%0,%1,%2,%3}, [%4];"
      : "=r"(a), "=r"(b), "=r"(c), "=r"(d)
      : "l"(p));
}
__device__ __forceinline__ float bf_lo(unsigned u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf_hi(unsigned u) { return __uint_as_float(u & 0xffff0000u); }

template <class VT> struct VecTraits;
template <> struct VecTraits<double> { static constexpr int VE = 4; };
template <> struct VecTraits<float> { static constexpr int VE = 4; };
template <> struct VecTraits<bf16> { static constexpr int VE = 8; };

// Loads vector v (VE elements) of column ids and values, converted to AT.
template <class VT, class AT> struct VecLoad;
template <> struct VecLoad<double, double> {
  static __device__ __forceinline__ void load(const i32* idx, const double* val, i64 v, int* c, double* w) {
    ld_idx4(idx + 4 * v, c[0], c[1], c[2], c[3]);
    ld_f64x2(val + 4 * v, w[0], w[1]);
    ld_f64x2(val + 4 * v + 2, w[2], w[3]);
  }
};
template <> struct VecLoad<float, float> {
  static __device__ __forceinline__ void load(const i32* idx, const float* val, i64 v, int* c, float* w) {
    ld_idx4(idx + 4 * v, c[0], c[1], c[2], c[3]);
    ld_f32x4(val + 4 * v, w[0], w[1], w[2], w[3]);
  }
};
template <> struct VecLoad<bf16, float> {
  static __device__ __forceinline__ void load(const i32* idx, const bf16* val, i64 v, int* c, float* w) {
    ld_idx4(idx + 8 * v, c[0], c[1], c[2], c[3]);
    ld_idx4(idx + 8 * v + 4, c[4], c[5], c[6], c[7]);
    unsigned u0, u1, u2, u3;
    ld_u32x4(val + 8 * v, u0, u1, u2, u3);
    w[0] = bf_lo(u0); w[1] = bf_hi(u0); w[2] = bf_lo(u1); w[3] = bf_hi(u1);
    w[4] = bf_lo(u2); w[5] = bf_hi(u2); w[6] = bf_lo(u3); w[7] = bf_hi(u3);
  }
};

template <class XT> __device__ __forceinline__ XT ldx(const XT* x, int c) { return __ldg(x + c); }

// acc += Σ val*x over the elements of vector v that lie in [s, e)
template <class VT, class XT, class AT>
__device__ __forceinline__ void vec_accum(const i32* __restrict__ idx, const VT* __restrict__ val,
                                          const XT* __restrict__ x, i64 v, i64 s, i64 e, AT& acc) {
  constexpr int VE = VecTraits<VT>::VE;
  int c[VE];
  AT w[VE];
  VecLoad<VT, AT>::load(idx, val, v, c, w);
  const i64 base = v * VE;
  if (base >= s && base + VE <= e) {
#pragma unroll
    for (int j = 0; j < VE; j++) acc += w[j] * (AT)ldx(x, c[j]);
  } else {
#pragma unroll
    for (int j = 0; j < VE; j++)
      if (base + j >= s && base + j < e) acc += w[j] * (AT)ldx(x, c[j]);
  }
}

// Partial dot product of elements [s, e) handled by `lane` of an L-lane group.
template <int L, class VT, class XT, class AT>
__device__ __forceinline__ AT range_partial(const i32* __restrict__ idx, const VT* __restrict__ val,
                                            const XT* __restrict__ x, i64 s, i64 e, int lane) {
  constexpr int VE = VecTraits<VT>::VE;
  AT a0 = 0, a1 = 0;
  if (e > s) {
    const i64 v1 = (e - 1) / VE + 1;
    i64 v = s / VE + lane;
    for (; v + L < v1; v += 2 * L) {
      vec_accum<VT, XT, AT>(idx, val, x, v, s, e, a0);
      vec_accum<VT, XT, AT>(idx, val, x, v + L, s, e, a1);
    }
    if (v < v1) vec_accum<VT, XT, AT>(idx, val, x, v, s, e, a0);
  }
  return a0 + a1;
}

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
struct CSum {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double v) {  // Neumaier
    double t = s + v;
    if (fabs(s) >= fabs(v)) c += (s - t) + v;
    else c += (v - t) + s;
    s = t;
  }
  __device__ __forceinline__ double total() const { return s + c; }
};

// Fixed-order block reduction of two compensated sums (256 threads).
__device__ __forceinline__ void block_csum2(CSum a, CSum b, double* out_a, double* out_b) {
  __shared__ double ra[256], rb[256];
  __syncthreads();
  ra[threadIdx.x] = a.total();
  rb[threadIdx.x] = b.total();
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
__device__ __forceinline__ void logistic_row(float wtx, double lab, double& loss, float& d) {
  float z = (float)lab * wtx;
  float neg = -(float)lab;
  if (z > 18.0f) {
    float e = expf(-z);
    loss = (double)e;
    d = e * neg;
  } else if (z < -18.0f) {
    loss = (double)-z;
    d = neg;
  } else {
    loss = (double)log1pf(expf(-z));
    d = neg / (1.0f + expf(z));
  }
  if (d > 1e12f) d = 1e12f;
  else if (d < -1e12f) d = -1e12f;
}

// ------------------------------------------------------------ kernel args
struct CrsK {
  const i32* off;
  const i32* idx;
  const void* val;
  const void* x;
  const i32* rows;
  const i32* chunk_row;
  const i32* chunk_beg;
  i64 item_start[kBins + 1];
  i64 row_start[kBins + 1];
  void* y;
  void* partials;
  // logistic epilogue
  const double* label;
  const double* sw;
  const double* intercept;
  int icpt;
  void* r;
  double* cta_part;
};

template <class AT, class YT, int EPI>
__device__ __forceinline__ void epilogue(const CrsK& p, i32 row, AT acc, AT b, CSum& ls, CSum& bs) {
  if (EPI == EPI_STORE) {
    ((YT*)p.y)[row] = (YT)acc;
  } else {
    AT wtx = acc + b;
    double lab = p.label[row];
    double loss;
    AT d;
    logistic_row(wtx, lab, loss, d);
    if (p.sw) d = (AT)(d * (AT)p.sw[row]);
    ((YT*)p.r)[row] = (YT)d;
    ls.add(loss);
    bs.add((double)d);
  }
}

template <int LOG2L, class VT, class XT, class AT, class YT, int EPI>
__device__ __forceinline__ void do_lane_rows(const CrsK& p, int bin, i64 item, AT b, CSum& ls, CSum& bs) {
  constexpr int L = 1 << LOG2L;
  constexpr int RPI = kThreads / L;
  const int sub = threadIdx.x / L, lane = threadIdx.x % L;
  const i64 ri = (item - p.item_start[bin]) * RPI + sub;
  const bool has = ri < p.row_start[bin + 1] - p.row_start[bin];
  i32 row = has ? p.rows[p.row_start[bin] + ri] : 0;
  i64 s = has ? p.off[row] : 0, e = has ? p.off[row + 1] : 0;
  AT acc = range_partial<L, VT, XT, AT>(p.idx, (const VT*)p.val, (const XT*)p.x, s, e, lane);
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (has && lane == 0) epilogue<AT, YT, EPI>(p, row, acc, b, ls, bs);
}

template <class VT, class XT, class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads) k_crs(const CrsK p) {
  CSum ls, bs;
  const AT b = (EPI == EPI_LOGREG && p.icpt) ? (AT)*p.intercept : (AT)0;
  const i64 total = p.item_start[kBins];
  int bin = 0;
  for (i64 item = blockIdx.x; item < total; item += gridDim.x) {
    while (item >= p.item_start[bin + 1]) bin++;
    switch (bin) {
      case 0: do_lane_rows<0, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 1: do_lane_rows<1, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 2: do_lane_rows<2, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 3: do_lane_rows<3, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 4: do_lane_rows<4, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 5: do_lane_rows<5, VT, XT, AT, YT, EPI>(p, bin, item, b, ls, bs); break;
      case 6: {
        i32 row = p.rows[p.row_start[6] + (item - p.item_start[6])];
        AT acc = range_partial<kThreads, VT, XT, AT>(p.idx, (const VT*)p.val, (const XT*)p.x, p.off[row],
                                                     p.off[row + 1], threadIdx.x);
        acc = block_sum256(acc);
        if (threadIdx.x == 0) epilogue<AT, YT, EPI>(p, row, acc, b, ls, bs);
        break;
      }
      default: {
        i64 ci = item - p.item_start[7];
        i32 row = p.chunk_row[ci];
        i64 beg = p.chunk_beg[ci];
        i64 end = (beg & ~7ll) + kChunk;
        i64 re = p.off[row + 1];
        if (end > re) end = re;
        AT acc = range_partial<kThreads, VT, XT, AT>(p.idx, (const VT*)p.val, (const XT*)p.x, beg, end,
                                                     threadIdx.x);
        acc = block_sum256(acc);
        if (threadIdx.x == 0) ((AT*)p.partials)[ci] = acc;
        break;
      }
    }
  }
  if (EPI == EPI_LOGREG) block_csum2(ls, bs, &p.cta_part[2 * blockIdx.x], &p.cta_part[2 * blockIdx.x + 1]);
}

// ------------------------------------------------------------- finalize
struct FinK {
  const i32* long_rows;
  const i32* long_chunk0;
  i64 nlong;
  const void* partials;
  void* y;
  // logistic
  const double* label;
  const double* sw;
  const double* intercept;
  int icpt;
  void* r;
  const double* cta_part;
  i64 ncta;
  double* long_part;
  double* out;        // [loss, bias]
  double* grad_bias;  // optional
  unsigned* ticket;
};

template <class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads) k_finalize(const FinK f) {
  const AT b = (EPI == EPI_LOGREG && f.icpt) ? (AT)*f.intercept : (AT)0;
  for (i64 i = blockIdx.x; i < f.nlong; i += gridDim.x) {
    i64 c0 = f.long_chunk0[i], c1 = f.long_chunk0[i + 1];
    AT acc = 0;
    for (i64 j = c0 + threadIdx.x; j < c1; j += kThreads) acc += ((const AT*)f.partials)[j];
    acc = block_sum256(acc);
    if (threadIdx.x == 0) {
      i32 row = f.long_rows[i];
      if (EPI == EPI_STORE) {
        ((YT*)f.y)[row] = (YT)acc;
      } else {
        double loss;
        AT d;
        logistic_row((AT)(acc + b), f.label[row], loss, d);
        if (f.sw) d = (AT)(d * (AT)f.sw[row]);
        ((YT*)f.r)[row] = (YT)d;
        f.long_part[2 * i] = loss;
        f.long_part[2 * i + 1] = (double)d;
      }
    }
  }
  if (EPI != EPI_LOGREG) return;
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(f.ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  CSum ls, bs;
  for (i64 i = threadIdx.x; i < f.ncta; i += kThreads) {
    ls.add(__ldcg(&f.cta_part[2 * i]));
    bs.add(__ldcg(&f.cta_part[2 * i + 1]));
  }
  for (i64 i = threadIdx.x; i < f.nlong; i += kThreads) {
    ls.add(__ldcg(&f.long_part[2 * i]));
    bs.add(__ldcg(&f.long_part[2 * i + 1]));
  }
  double tl = 0, tb = 0;
  block_csum2(ls, bs, &tl, &tb);
  if (threadIdx.x == 0) {
    f.out[0] = tl;
    f.out[1] = f.icpt ? tb : 0.0;
    if (f.grad_bias) *f.grad_bias = f.icpt ? tb : 0.0;
    *f.ticket = 0u;
  }
}

// ------------------------------------------------------------- host side
static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct PassScratch {
  unsigned* ticket;
  double* out;
  double* cta_part;
  double* long_part;
  void* partials;
};

static size_t carve(char* base, const Sched& s, int grid, size_t at_size, PassScratch* ps) {
  size_t o = 0;
  auto take = [&](size_t b) { size_t r = o; o += align256(b); return base ? base + r : nullptr; };
  char* t = take(sizeof(unsigned) * 2);
  char* out = take(sizeof(double) * 2);
  char* cp = take(sizeof(double) * 2 * (size_t)grid);
  char* lp = take(sizeof(double) * 2 * (size_t)std::max<i64>(s.nlong, 1));
  char* pa = take(at_size * (size_t)std::max<i64>(s.nchunks, 1));
  if (ps) {
    ps->ticket = (unsigned*)t;
    ps->out = (double*)out;
    ps->cta_part = (double*)cp;
    ps->long_part = (double*)lp;
    ps->partials = pa;
  }
  return o;
}

i64 crs_pass_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage) {
  const Sched& s = crs_sched(c, a, storage == FVG_BF16 ? 8 : 4);
  return (i64)carve(nullptr, s, c->grid_spmv, 8, nullptr);
}

template <class VT, class XT, class AT, class YT, int EPI>
static void launch_crs(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, const void* x, void* y,
                       const LogregEpi* lr, const PassScratch& ps, int grid) {
  CrsK p;
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.val = a.val[storage].p;
  p.x = x;
  p.rows = s.rows.as<i32>();
  p.chunk_row = s.chunk_row.as<i32>();
  p.chunk_beg = s.chunk_beg.as<i32>();
  for (int b = 0; b <= kBins; b++) {
    p.item_start[b] = s.item_start[b];
    p.row_start[b] = s.row_start[b];
  }
  p.y = y;
  p.partials = ps.partials;
  p.label = lr ? lr->label : nullptr;
  p.sw = lr ? lr->sw : nullptr;
  p.intercept = lr ? lr->intercept : nullptr;
  p.icpt = lr ? lr->icpt : 0;
  p.r = lr ? lr->r : nullptr;
  p.cta_part = ps.cta_part;
  if (s.items() > 0) {
    k_crs<VT, XT, AT, YT, EPI><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_crs");
    count_launch(c);
  }
  if (s.nlong > 0 || EPI == EPI_LOGREG) {
    FinK f;
    f.long_rows = s.long_rows.as<i32>();
    f.long_chunk0 = s.long_chunk0.as<i32>();
    f.nlong = s.nlong;
    f.partials = ps.partials;
    f.y = y;
    f.label = p.label;
    f.sw = p.sw;
    f.intercept = p.intercept;
    f.icpt = p.icpt;
    f.r = p.r;
    f.cta_part = ps.cta_part;
    f.ncta = s.items() > 0 ? grid : 0;
    f.long_part = ps.long_part;
    f.out = (lr && lr->out) ? lr->out : ps.out;
    f.grad_bias = lr ? lr->grad_bias : nullptr;
    f.ticket = ps.ticket;
    int fg = (int)std::max<i64>(1, std::min<i64>(s.nlong, 4 * c->num_sms));
    ProfScope pf(c, P_FINALIZE);
    k_finalize<AT, YT, EPI><<<fg, kThreads, 0, c->stream>>>(f);
    check_launch("k_finalize");
    count_launch(c);
  }
}

void crs_pass(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* x, int y_dt, void* y, int epi,
              const LogregEpi* lr, void* scratch, int prof_key) {
  const int ve = storage == FVG_BF16 ? 8 : 4;
  const Sched& s = crs_sched(c, a, ve);
  if (!a.val[storage].p) fail(FVG_ERR_INTERNAL, "missing value plane for the requested storage");
  int grid = (int)std::max<i64>(1, std::min<i64>(c->grid_spmv, s.items()));
  const size_t at_size = (storage == FVG_F64) ? 8 : 4;
  DBuf tmp;
  PassScratch ps;
  if (!scratch) {
    size_t bytes = carve(nullptr, s, c->grid_spmv, at_size, nullptr);
    tmp.alloc(bytes, c->stream);
    FVG_CUDA(cudaMemsetAsync(tmp.p, 0, 256, c->stream));  // ticket
    scratch = tmp.p;
  }
  carve((char*)scratch, s, c->grid_spmv, at_size, &ps);
  ProfScope pr(c, prof_key);
  const int out_dt = (epi == EPI_LOGREG) ? (lr ? lr->r_dt : y_dt) : y_dt;
  if (storage == FVG_F64) {
    if (x_dt != FVG_F64 || out_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
    if (epi == EPI_STORE) launch_crs<double, double, double, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps, grid);
    else launch_crs<double, double, double, double, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps, grid);
  } else if (storage == FVG_F32) {
    if (x_dt != FVG_F32) fail(FVG_ERR_INVALID_ARG, "FP32 values need FP32 input vectors");
    if (epi == EPI_STORE && out_dt == FVG_F64)
      launch_crs<float, float, float, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps, grid);
    else if (epi == EPI_STORE)
      launch_crs<float, float, float, float, EPI_STORE>(c, a, s, storage, x, y, lr, ps, grid);
    else
      launch_crs<float, float, float, float, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps, grid);
  } else {
    if (x_dt != FVG_F32) fail(FVG_ERR_INVALID_ARG, "BF16 values need FP32 input vectors");
    if (epi == EPI_STORE && out_dt == FVG_F64)
      launch_crs<bf16, float, float, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps, grid);
    else if (epi == EPI_STORE)
      launch_crs<bf16, float, float, float, EPI_STORE>(c, a, s, storage, x, y, lr, ps, grid);
    else
      launch_crs<bf16, float, float, float, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps, grid);
  }
}

// ------------------------------------------------------------------- JDS
// Thread per permuted row; diagonal d of row p sits at off[d] + p, so a warp
// reads each diagonal contiguously.  Diagonal lengths never increase, so row
// p has exactly the diagonals d with off[d+1] - off[d] > p (binary search).
// part (hybrid) adds the CRS tail of the first npart permuted rows after the
// JDS sum, as jds_crs_hybrid_spmv_impl does (jds_crs_hybrid.hpp:198-211).
template <class VT, class XT, class AT, class YT>
__global__ void __launch_bounds__(256) k_jds(const i32* __restrict__ perm, const i64* __restrict__ off,
                                             const i32* __restrict__ idx, const VT* __restrict__ val,
                                             i64 m, i64 ndiag, const XT* __restrict__ x, YT* __restrict__ y,
                                             const AT* __restrict__ part, i64 npart) {
  for (i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += (i64)gridDim.x * blockDim.x) {
    i64 lo = 0, hi = ndiag;
    while (lo < hi) {
      i64 mid = (lo + hi) >> 1;
      if (off[mid + 1] - off[mid] > p) lo = mid + 1;
      else hi = mid;
    }
    const i64 len = lo;
    AT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    i64 d = 0;
    for (; d + 3 < len; d += 4) {
      i64 q0 = off[d] + p, q1 = off[d + 1] + p, q2 = off[d + 2] + p, q3 = off[d + 3] + p;
      a0 += (AT)val[q0] * (AT)__ldg(x + idx[q0]);
      a1 += (AT)val[q1] * (AT)__ldg(x + idx[q1]);
      a2 += (AT)val[q2] * (AT)__ldg(x + idx[q2]);
      a3 += (AT)val[q3] * (AT)__ldg(x + idx[q3]);
    }
    for (; d < len; d++) {
      i64 q = off[d] + p;
      a0 += (AT)val[q] * (AT)__ldg(x + idx[q]);
    }
    AT acc = (a0 + a1) + (a2 + a3);
    if (p < npart) acc = acc + part[p];
    y[perm[p]] = (YT)acc;
  }
}

template <class T> __global__ void k_zero(T* y, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) y[i] = (T)0;
}

static unsigned grid_rows(i64 n) {
  i64 g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)(g < 1 ? 1 : g);
}

template <class VT, class XT, class AT, class YT>
static void launch_jds(fvg_ctx* c, DevJDS& j, int storage, const void* x, void* y, const void* part, i64 npart) {
  if (j.m == 0) return;
  if (j.empty_perm) {
    k_zero<YT><<<grid_rows(j.m), 256, 0, c->stream>>>((YT*)y, j.m);
  } else {
    k_jds<VT, XT, AT, YT><<<grid_rows(j.m), 256, 0, c->stream>>>(
        j.perm.as<i32>(), j.off.as<i64>(), j.idx.as<i32>(), j.val[storage].as<VT>(), j.m, j.ndiag, (const XT*)x,
        (YT*)y, (const AT*)part, npart);
  }
  check_launch("k_jds");
  count_launch(c);
}

static void jds_dispatch(fvg_ctx* c, DevJDS& j, int storage, int x_dt, const void* x, int y_dt, void* y,
                         const void* part, i64 npart) {
  if (storage == FVG_F64) {
    if (x_dt != FVG_F64 || y_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
    launch_jds<double, double, double, double>(c, j, storage, x, y, part, npart);
  } else if (storage == FVG_F32) {
    if (y_dt == FVG_F64) launch_jds<float, float, float, double>(c, j, storage, x, y, part, npart);
    else launch_jds<float, float, float, float>(c, j, storage, x, y, part, npart);
  } else {
    if (y_dt == FVG_F64) launch_jds<bf16, float, float, double>(c, j, storage, x, y, part, npart);
    else launch_jds<bf16, float, float, float>(c, j, storage, x, y, part, npart);
  }
}

void jds_spmv(fvg_ctx* c, DevJDS& j, int storage, int x_dt, const void* x, int y_dt, void* y, bool) {
  ProfScope pr(c, P_SPMV_JDS);
  ensure_plane_generic(c, j.val, j.nnz, storage, FVG_F64);
  jds_dispatch(c, j, storage, x_dt, x, y_dt, y, nullptr, 0);
}

void hyb_spmv(fvg_ctx* c, DevHYB& h, int storage, int x_dt, const void* x, int y_dt, void* y) {
  ProfScope pr(c, P_SPMV_HYB);
  if (h.all_crs) {  // whole matrix in the CRS part, natural row order
    crs_pass(c, h.crs, storage, x_dt, x, y_dt, y, EPI_STORE, nullptr, nullptr, P_NKEYS);
    return;
  }
  DBuf part;
  const int at = (storage == FVG_F64) ? FVG_F64 : FVG_F32;
  if (h.crs_rows > 0) {
    part.alloc((size_t)dtype_size(at) * h.crs_rows, c->stream);
    crs_pass(c, h.crs, storage, x_dt, x, at, part.p, EPI_STORE, nullptr, nullptr, P_NKEYS);
  }
  jds_dispatch(c, h.jds, storage, x_dt, x, y_dt, y, part.p, h.crs_rows);
}

// ------------------------------------------------------------------- ELL
template <class VT, class XT, class AT, class YT>
__global__ void __launch_bounds__(256) k_ell(const i32* __restrict__ idx, const VT* __restrict__ val, i64 m,
                                             i64 width, const XT* __restrict__ x, YT* __restrict__ y) {
  for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (i64)gridDim.x * blockDim.x) {
    AT a0 = 0, a1 = 0;
    i64 k = 0;
    for (; k + 1 < width; k += 2) {
      i64 q0 = k * m + r, q1 = q0 + m;
      a0 += (AT)val[q0] * (AT)__ldg(x + idx[q0]);
      a1 += (AT)val[q1] * (AT)__ldg(x + idx[q1]);
    }
    if (k < width) a0 += (AT)val[k * m + r] * (AT)__ldg(x + idx[k * m + r]);
    y[r] = (YT)(a0 + a1);
  }
}

void ell_spmv(fvg_ctx* c, DevELL& e, int storage, int x_dt, const void* x, int y_dt, void* y) {
  ProfScope pr(c, P_SPMV_ELL);
  if (e.m == 0) return;
  ensure_plane_generic(c, e.val, e.m * e.width, storage, FVG_F64);
  unsigned g = grid_rows(e.m);
  if (storage == FVG_F64) {
    if (x_dt != FVG_F64 || y_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
    k_ell<double, double, double, double><<<g, 256, 0, c->stream>>>(e.idx.as<i32>(), e.val[storage].as<double>(),
                                                                    e.m, e.width, (const double*)x, (double*)y);
  } else if (storage == FVG_F32) {
    if (y_dt == FVG_F64)
      k_ell<float, float, float, double><<<g, 256, 0, c->stream>>>(e.idx.as<i32>(), e.val[storage].as<float>(), e.m,
                                                                   e.width, (const float*)x, (double*)y);
    else
      k_ell<float, float, float, float><<<g, 256, 0, c->stream>>>(e.idx.as<i32>(), e.val[storage].as<float>(), e.m,
                                                                  e.width, (const float*)x, (float*)y);
  } else {
    if (y_dt == FVG_F64)
      k_ell<bf16, float, float, double><<<g, 256, 0, c->stream>>>(e.idx.as<i32>(), e.val[storage].as<bf16>(), e.m,
                                                                  e.width, (const float*)x, (double*)y);
    else
      k_ell<bf16, float, float, float><<<g, 256, 0, c->stream>>>(e.idx.as<i32>(), e.val[storage].as<bf16>(), e.m,
                                                                 e.width, (const float*)x, (float*)y);
  }
  check_launch("k_ell");
  count_launch(c);
}

// ------------------------------------------------------------------ SpMM
// Y = A X (row-major, k columns): a warp per row, lanes across columns.
template <class VT, class XT, class AT>
__global__ void __launch_bounds__(256) k_spmm_crs(const i32* __restrict__ off, const i32* __restrict__ idx,
                                                  const VT* __restrict__ val, i64 m, const XT* __restrict__ X,
                                                  i64 k, XT* __restrict__ Y) {
  const int lane = threadIdx.x & 31;
  const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const i64 nwarps = ((i64)gridDim.x * blockDim.x) >> 5;
  for (i64 r = warp; r < m; r += nwarps) {
    i64 s = off[r], e = off[r + 1];
    for (i64 c0 = 0; c0 < k; c0 += 64) {
      AT a0 = 0, a1 = 0;
      i64 ca = c0 + lane, cb = c0 + 32 + lane;
      for (i64 q = s; q < e; q++) {
        AT v = (AT)val[q];
        const XT* xr = X + (i64)idx[q] * k;
        if (ca < k) a0 += v * (AT)__ldg(xr + ca);
        if (cb < k) a1 += v * (AT)__ldg(xr + cb);
      }
      if (ca < k) Y[r * k + ca] = (XT)a0;
      if (cb < k) Y[r * k + cb] = (XT)a1;
    }
  }
}

void crs_spmm(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* X, i64 k, void* Y) {
  ProfScope pr(c, P_SPMM);
  if (a.m == 0 || k == 0) return;
  i64 warps = std::min<i64>(a.m, (i64)c->num_sms * 64);
  unsigned g = (unsigned)((warps * 32 + 255) / 256);
  if (storage == FVG_F64) {
    if (x_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
    k_spmm_crs<double, double, double><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(),
                                                                  a.val[storage].as<double>(), a.m,
                                                                  (const double*)X, k, (double*)Y);
  } else if (storage == FVG_F32) {
    k_spmm_crs<float, float, float><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(),
                                                               a.val[storage].as<float>(), a.m, (const float*)X, k,
                                                               (float*)Y);
  } else {
    k_spmm_crs<bf16, float, float><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(),
                                                              a.val[storage].as<bf16>(), a.m, (const float*)X, k,
                                                              (float*)Y);
  }
  check_launch("k_spmm_crs");
  count_launch(c);
}

// Resident CTAs per SM of the heaviest CRS instantiation (sizes the
// persistent grid).
int crs_blocks_per_sm() {
  int a = 0, b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_crs<double, double, double, double, EPI_LOGREG>, kThreads, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_crs<bf16, float, float, float, EPI_LOGREG>, kThreads, 0);
  int r = std::min(a > 0 ? a : 8, b > 0 ? b : 8);
  return r < 1 ? 1 : r;
}

// logistic_regression_model<T>::predict_probability (ml/glm/linear_model.hpp:
// 376-392): v += intercept (when non-zero); exp argument above 709 → 0.
__global__ void k_sigmoid(double* v, i64 m, double b) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (i64)gridDim.x * blockDim.x) {
    double x = v[i];
    if (b != 0) x += b;
    double e = -1.0 * x;
    v[i] = (e > 709) ? 0.0 : 1.0 / (1.0 + exp(e));
  }
}

void sigmoid_probability(fvg_ctx* c, double* v, i64 m, double b) {
  if (m <= 0) return;
  k_sigmoid<<<grid_rows(m), 256, 0, c->stream>>>(v, m, b);
  check_launch("k_sigmoid");
  count_launch(c);
}

// ------------------------------------------------- per-row logistic pass
// For layouts whose product is computed first (ELL/JDS/hybrid): applies the
// logistic epilogue to z = A w already in memory.
template <class AT>
__global__ void __launch_bounds__(256) k_logreg_rows(const AT* __restrict__ wtx, i64 m, const CrsK p) {
  CSum ls, bs;
  const AT b = p.icpt ? (AT)*p.intercept : (AT)0;
  for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (i64)gridDim.x * blockDim.x)
    epilogue<AT, AT, EPI_LOGREG>(p, (i32)r, wtx[r], b, ls, bs);
  block_csum2(ls, bs, &p.cta_part[2 * blockIdx.x], &p.cta_part[2 * blockIdx.x + 1]);
}

void logreg_rows(fvg_ctx* c, const void* wtx, int wtx_dt, i64 m, const LogregEpi& lr) {
  int grid = (int)std::max<i64>(1, std::min<i64>(c->grid_spmv, (m + 255) / 256));
  DBuf tmp;
  size_t need = 256 * 3 + sizeof(double) * 2 * (size_t)grid;
  tmp.alloc(need, c->stream);
  FVG_CUDA(cudaMemsetAsync(tmp.p, 0, 256, c->stream));
  unsigned* ticket = (unsigned*)tmp.p;
  double* out = (double*)((char*)tmp.p + 256);
  double* cta = (double*)((char*)tmp.p + 512);
  CrsK p = {};
  p.label = lr.label;
  p.sw = lr.sw;
  p.intercept = lr.intercept;
  p.icpt = lr.icpt;
  p.r = lr.r;
  p.cta_part = cta;
  if (wtx_dt == FVG_F64) k_logreg_rows<double><<<grid, 256, 0, c->stream>>>((const double*)wtx, m, p);
  else k_logreg_rows<float><<<grid, 256, 0, c->stream>>>((const float*)wtx, m, p);
  check_launch("k_logreg_rows");
  count_launch(c);
  FinK f = {};
  f.nlong = 0;
  f.label = lr.label;
  f.sw = lr.sw;
  f.intercept = lr.intercept;
  f.icpt = lr.icpt;
  f.r = lr.r;
  f.cta_part = cta;
  f.ncta = grid;
  f.out = lr.out ? lr.out : out;
  f.grad_bias = lr.grad_bias;
  f.ticket = ticket;
  if (wtx_dt == FVG_F64) k_finalize<double, double, EPI_LOGREG><<<1, kThreads, 0, c->stream>>>(f);
  else k_finalize<float, float, EPI_LOGREG><<<1, kThreads, 0, c->stream>>>(f);
  check_launch("k_finalize_rows");
  count_launch(c);
}

}  // namespace fvg
