// Split-value storage: FP64-accurate products at FP32 speed.
//
// The reference multiplies FP64 values (crs_matrix_spmv_impl,
// crs_matrix.hpp:1505-1516) and evaluates the loss/gradient in FP64
// (gradient_descent.hpp:196-225, gradient.hpp:15-53).  On GB300 FP64 issues
// at a small fraction of the FP32 rate, and FP32 or BF16 values alone move the
// L-BFGS trajectory far from the FP64 one (their rounding, 2^-24 or 2^-9 per
// value, grows over the iterations).  Split storage keeps each value v as
//   hi = FP32(v)                 (the FP32 plane, shared with FP32 storage)
//   lo = BF16(v - hi)            (a 2-byte residual plane)
// so hi + lo is within 2^-33 of v, and multiplies in double-FP32 (df64.cuh):
// x arrives as (hi, lo) pairs, each product hi*x is made exact with an FMA,
// rows are summed with TwoSum, and the per-row GLM loss/gradient runs in df64
// (table-driven exp, Newton-corrected log1p).  FP64 appears only in O(rows)
// conversions of the results.
//
// Pass 1 (A w): k_crs_split over the CRS items writes each row's product as a
// df pair; k_fin_split adds long rows' pieces in order; k_glm_split applies
// the loss kind (compute_dloss * sample_weight), writes r = dloss * sw as df
// pairs and reduces loss and bias in a fixed order.  Pass 2 (A^T r) is
// k_crs_split over the transposed copy.  Every sum has a fixed order, so
// results are identical run to run.
#include <cmath>
#include <mutex>
#include <type_traits>

#include "device_common.cuh"
#include "df64.cuh"
#include "split_bits.h"

namespace fvg {

// 2^(j/64), j = 0..63, as df pairs, into the device table of df_exp.  The
// host's exp2 is accurate to an ulp of FP64, far below the df64 resolution.
void df64_init(fvg_ctx* c) {
  float2 tab[64];
  for (int j = 0; j < 64; j++) {
    const double v = std::exp2(j / 64.0);
    const float h = (float)v;
    tab[j] = make_float2(h, (float)(v - (double)h));
  }
  FVG_CUDA(cudaMemcpyToSymbol(g_exp2_tab, tab, sizeof(tab)));
}

namespace {

constexpr int kSplitThreads = 256;
// Entries per lane of the split CRS kernel and its work items' size (an item
// from its first entry rounded down to CH fits 32 lanes x CH).  The forward
// products (A's rows, the head's row tails: FP32-pair output) run 8 entries a
// lane at 3 CTAs per SM, the transposed ones (rare columns: FP64 output) 16
// at 2: the measured best of 8 / 16 entries and 2 / 3 / 4 CTAs for each.
constexpr int split_crs_ch(bool fwd) { return fwd ? 8 : 16; }
constexpr int split_crs_tile(bool fwd) { return 30 * split_crs_ch(fwd); }

unsigned grid_rows(fvg_ctx* c, i64 n, int per_sm = 8) {
  i64 g = (n + kSplitThreads - 1) / kSplitThreads;
  g = std::min<i64>(g, (i64)per_sm * c->num_sms);
  return (unsigned)std::max<i64>(g, 1);
}

// residual plane: lo = BF16(v - FP32(v)) (one-off per matrix); flags a value
// whose FP32 rounding overflows
// (the FP32 plane holds FP32(v), so the residual follows from v alone: by
// integer arithmetic on its bits, split_bits.h, where that applies)
__global__ void k_split_plane(const double* __restrict__ v, const float* __restrict__ hi, bf16* __restrict__ lo,
                              i64 n, unsigned* __restrict__ bad) {
  unsigned b = 0;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double x = v[i];
    uint32_t hb;
    uint16_t lb;
    if (split_bits((uint64_t)__double_as_longlong(x), &hb, &lb)) {
      if ((hb & 0x7fffffffu) == 0x7f800000u) b = 1;
      lo[i] = __ushort_as_bfloat16(lb);
    } else {
      const float h = hi[i];
      if (isinf(h) && !isinf(x)) b = 1;
      lo[i] = __double2bfloat16(isinf(h) ? 0.0 : x - (double)h);
    }
  }
  if (b) atomicOr(bad, 1u);
}

// Both planes from the FP64 values in one pass: hi = FP32(v), lo =
// BF16(v - hi) by integer arithmetic on the FP64 bits (split_bits.h), the
// FP64 conversions only for values outside its range.
__global__ void k_split_values(const double* __restrict__ v, float* __restrict__ hi, bf16* __restrict__ lo, i64 n,
                               unsigned* __restrict__ bad) {
  unsigned b = 0;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const double x = v[i];
    uint32_t hb;
    uint16_t lb;
    if (split_bits((uint64_t)__double_as_longlong(x), &hb, &lb)) {
      if ((hb & 0x7fffffffu) == 0x7f800000u) b = 1;
      hi[i] = __uint_as_float(hb);
      lo[i] = __ushort_as_bfloat16(lb);
    } else {
      const float h = __double2float_rn(x);
      if (isinf(h) && !isinf(x)) b = 1;
      hi[i] = h;
      lo[i] = __double2bfloat16(isinf(h) ? 0.0 : x - (double)h);
    }
  }
  if (b) atomicOr(bad, 1u);
}

__global__ void k_split_vec(const double* __restrict__ x, float2* __restrict__ y, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    y[i] = df_pack(df_from_double(x[i]));
}

// ------------------------------------------------------------- CRS pass
struct SplitK {
  const i32* off;
  const i32* idx;
  const float* vh;
  const unsigned short* vl;
  const float2* x;
  const Item* items;
  i64 nitems;
  void* y;           // double[rows] or float2[rows]
  float2* partials;  // long-row pieces
};

template <class YT> __device__ __forceinline__ void store_row(void* y, i64 row, df a);
template <> __device__ __forceinline__ void store_row<double>(void* y, i64 row, df a) {
  ((double*)y)[row] = df_to_double(a);
}
template <> __device__ __forceinline__ void store_row<float2>(void* y, i64 row, df a) {
  ((float2*)y)[row] = df_pack(a);
}

__device__ __forceinline__ df shfl_df(df a, int o) {
  return {__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}
__device__ __forceinline__ df shfl_up_df1(df a) {
  return {__shfl_up_sync(0xffffffffu, a.h, 1), __shfl_up_sync(0xffffffffu, a.l, 1)};
}

// Segmented inclusive scan over the warp's lanes, in lane order:
// S_L = v_L + (reset_L ? 0 : S_{L-1}).
__device__ __forceinline__ df seg_scan(df v, bool reset, int lane) {
  bool f = reset;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const df u = {__shfl_up_sync(0xffffffffu, v.h, o), __shfl_up_sync(0xffffffffu, v.l, o)};
    const bool fu = __shfl_up_sync(0xffffffffu, (int)f, o) != 0;
    if (lane >= o) {
      if (!f) v = df_add(u, v);
      f = f || fu;
    }
  }
  return v;
}

// Persistent kernel over CRS work items of at most split_crs_tile() entries
// (tiles of short rows, pieces of long rows; the packing of k_crs).  Lane L
// takes the CH entries q0 + CH*L .. q0 + CH*L + CH - 1 (q0 = the item's first
// entry rounded down to CH): column ids, FP32 values and BF16 residuals come in
// 128-bit loads, x's pairs are gathered, each product is made exact (p + t)
// and added to the lane's current row segment with TwoSum.  A row that
// starts and ends inside the chunk is written at once; the segments open at
// the chunk's two ends join the neighbouring lanes' through a segmented scan
// in lane order.  A piece of a long row is one warp reduction.  Every sum has
// a fixed order, so results are identical run to run.
template <class YT>
__global__ void __launch_bounds__(kThreads, std::is_same<YT, float2>::value ? 3 : 2) k_crs_split(const SplitK p) {
  constexpr int CH = split_crs_ch(std::is_same<YT, float2>::value);
  __shared__ int soffs[kThreads / 32][kTileRows + 1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int* soff = soffs[w];
  const i64 W = (i64)gridDim.x * (kThreads / 32);
  const i64 n = p.nitems;
  i64 t = (i64)blockIdx.x * (kThreads / 32) + w;
  Item nx = (t < n) ? p.items[t] : Item{0, 0, 0, 0};
  for (; t < n; t += W) {
    const Item it = nx;
    if (t + W < n) nx = p.items[t + W];
    const int q0 = it.e0 & ~(CH - 1);
    const bool tile = it.r1 >= 0;
    const int R = tile ? it.r1 - it.r0 : 0;
    if (tile)
      for (int k = lane; k <= R; k += 32) soff[k] = __ldg(p.off + it.r0 + k) - q0;
    const int lo_e = max(it.e0 - q0, lane * CH), hi_e = min(it.e1 - q0, lane * CH + CH);
    // the chunk (the arrays are padded past the last nonzero, and q0 + 16L
    // stays below it whenever the lane has entries)
    int c[CH];
    float hv[CH];
    unsigned lw[CH / 2];
    if (lo_e < hi_e) {
      const i64 b = (i64)q0 + lane * CH;
      const int4* ip = reinterpret_cast<const int4*>(p.idx + b);
      const float4* hp = reinterpret_cast<const float4*>(p.vh + b);
      const uint4* lp = reinterpret_cast<const uint4*>(p.vl + b);
#pragma unroll
      for (int q = 0; q < CH / 4; q++) {
        const int4 iv = __ldcs(ip + q);
        const float4 fv = __ldcs(hp + q);
        c[4 * q] = iv.x; c[4 * q + 1] = iv.y; c[4 * q + 2] = iv.z; c[4 * q + 3] = iv.w;
        hv[4 * q] = fv.x; hv[4 * q + 1] = fv.y; hv[4 * q + 2] = fv.z; hv[4 * q + 3] = fv.w;
      }
#pragma unroll
      for (int q = 0; q < CH / 8; q++) {
        const uint4 lv = __ldcs(lp + q);
        lw[4 * q] = lv.x; lw[4 * q + 1] = lv.y; lw[4 * q + 2] = lv.z; lw[4 * q + 3] = lv.w;
      }
    }
    float2 xv[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) {
      const int e = lane * CH + k;
      xv[k] = (e >= lo_e && e < hi_e) ? __ldg(p.x + c[k]) : make_float2(0.f, 0.f);
    }
    if (!tile) {
      DfAcc acc;
#pragma unroll
      for (int k = 0; k < CH; k++) {
        const int e = lane * CH + k;
        if (e >= lo_e && e < hi_e) {
          const float vl = __uint_as_float((k & 1) ? (lw[k >> 1] & 0xffff0000u) : (lw[k >> 1] << 16));
          float pp, tt;
          df_prod(hv[k], vl, xv[k], pp, tt);
          acc.add(pp, tt);
        }
      }
      df a = acc.get();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a = df_add(a, shfl_df(a, o));
      if (lane == 0) p.partials[-1 - it.r1] = df_pack(a);
    } else {
      __syncwarp();  // soff
      for (int j = lane; j < R; j += 32)
        if (soff[j] == soff[j + 1]) store_row<YT>(p.y, it.r0 + j, df{0.f, 0.f});  // empty rows
      // the lane's CH products (zero outside its valid range)
      float pp[CH], tt[CH];
#pragma unroll
      for (int k = 0; k < CH; k++) {
        const int e = lane * CH + k;
        const bool ok = e >= lo_e && e < hi_e;
        const float vl = __uint_as_float((k & 1) ? (lw[k >> 1] & 0xffff0000u) : (lw[k >> 1] << 16));
        float a, b;
        df_prod(hv[k], vl, xv[k], a, b);
        pp[k] = ok ? a : 0.f;
        tt[k] = ok ? b : 0.f;
      }
      // rows: j0 holds the first valid entry; B marks the rows starting after it
      unsigned B = 0;
      int j = 0, j0 = 0, nb = 0;
      bool starts = false;
      const bool any = lo_e < hi_e;
      if (any) {
        int a = 0, b = R;  // the last row starting at or before lo_e (the non-empty one holding it)
        while (b - a > 1) {
          const int mid = (a + b) >> 1;
          if (soff[mid] <= lo_e) a = mid;
          else b = mid;
        }
        j = j0 = a;
        starts = soff[j] == lo_e;
        nb = soff[j + 1];
        while (nb < hi_e) {
          B |= 1u << (nb - lane * CH);
          do {
            j++;
            nb = soff[j + 1];
          } while (nb == soff[j]);
        }
      }
      df H, T;
      chunk_segments<CH>(pp, tt, B, H, T);
      if (__popc(B) >= 2) {  // rows between two marks: started and ended in this chunk
        unsigned rest = B & (B - 1);
        int a = __ffs(B) - 1, jj = j0;
        do {
          jj++;
        } while (soff[jj + 1] == soff[jj]);
        while (rest) {
          const int b = __ffs(rest) - 1;
          rest &= rest - 1;
          store_row<YT>(p.y, it.r0 + jj, chunk_range<CH>(pp, tt, a, b));
          a = b;
          do {
            jj++;
          } while (soff[jj + 1] == soff[jj]);
        }
      }
      const df S = seg_scan(any ? T : df{0.f, 0.f}, any && (B != 0 || starts), lane);
      df carry = shfl_up_df1(S);
      if (lane == 0) carry = {0.f, 0.f};
      if (B) store_row<YT>(p.y, it.r0 + j0, starts ? H : df_add(carry, H));
      if (any && nb == hi_e) store_row<YT>(p.y, it.r0 + j, S);  // the tail row ends with this lane's range
    }
    __syncwarp();
  }
}

// long rows: a warp adds a row's pieces (lane L: pieces L, L+32, ...; then
// the butterfly), in the same order on every run
template <class YT>
__global__ void __launch_bounds__(kThreads) k_fin_split(const i32* __restrict__ long_rows,
                                                        const i32* __restrict__ long_piece0, i64 nlong,
                                                        const float2* __restrict__ partials, void* y) {
  const int lane = threadIdx.x & 31;
  for (i64 i = (i64)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); i < nlong;
       i += (i64)gridDim.x * (kThreads / 32)) {
    const i64 c0 = long_piece0[i], c1 = long_piece0[i + 1];
    df a = {0.f, 0.f};
    for (i64 j = c0 + lane; j < c1; j += 32) a = df_add(a, df_unpack(__ldcg(partials + j)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = df_add(a, shfl_df(a, o));
    if (lane == 0) store_row<YT>(y, long_rows[i], a);
  }
}

// ------------------------------------------------------------- GLM rows
struct GlmSplitK {
  const float2* wtx;
  const float2* head;  // optional second partial product per row
  i64 m;
  const float2* lab;
  const float2* sw;  // null: all ones
  const double* intercept;
  int icpt;
  int kind;
  double eps;
  float2* r;
  double* cta_part;  // [2 * gridDim.x]
  unsigned* ticket;
  double* out;        // [2]: loss, bias
  double* grad_bias;  // optional
};

__device__ __forceinline__ df block_df_sum(df a, df* red /* [8] */) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = df_add(a, shfl_df(a, o));
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = a;
  __syncthreads();
  df t = {0.f, 0.f};
  if (threadIdx.x == 0)
    for (int q = 0; q < kSplitThreads / 32; q++) t = df_add(t, red[q]);
  return t;  // thread 0
}

// compute_dloss * sample_weight per row (gradient_descent.hpp:196-211), the
// loss summed unweighted and the bias as the sum of dloss * sw; the CTAs'
// partial sums are added in CTA order by the last CTA (FP64, compensated).
__global__ void __launch_bounds__(kSplitThreads) k_glm_split(const GlmSplitK p) {
  __shared__ df red_l[kSplitThreads / 32], red_b[kSplitThreads / 32];
  const df b = p.icpt ? df_from_double(*p.intercept) : df{0.f, 0.f};
  const df eps = df_from_double(p.eps);
  df ls = {0.f, 0.f}, bs = {0.f, 0.f};
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < p.m; i += (i64)gridDim.x * blockDim.x) {
    df z = df_unpack(p.wtx[i]);
    if (p.head) z = df_add_acc(z, df_unpack(p.head[i]));
    z = df_add_acc(z, b);
    df loss, d;
    glm_row_df(p.kind, eps, z, df_unpack(p.lab[i]), loss, d);
    if (p.sw) d = df_mul(d, df_unpack(p.sw[i]));
    p.r[i] = df_pack(d);
    ls = df_add(ls, loss);
    bs = df_add(bs, d);
  }
  const df tl = block_df_sum(ls, red_l);
  const df tb = block_df_sum(bs, red_b);
  if (threadIdx.x == 0) {
    p.cta_part[2 * blockIdx.x] = df_to_double(tl);
    p.cta_part[2 * blockIdx.x + 1] = df_to_double(tb);
  }
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(p.ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA: thread t adds CTAs t, t + 256, ... (compensated), then a
  // fixed tree over the threads
  CSum l, s;
  for (unsigned q = threadIdx.x; q < gridDim.x; q += kSplitThreads) {
    l.add(__ldcg(&p.cta_part[2 * q]));
    s.add(__ldcg(&p.cta_part[2 * q + 1]));
  }
  double tl2 = 0.0, tb2 = 0.0;
  block_csum2(l.total(), s.total(), &tl2, &tb2);
  if (threadIdx.x == 0) {
    p.out[0] = tl2;
    p.out[1] = p.icpt ? tb2 : 0.0;
    if (p.grad_bias) *p.grad_bias = p.icpt ? tb2 : 0.0;
    *p.ticket = 0u;
  }
}

}  // namespace

// ------------------------------------------------------------------ host
void split_residual_plane(fvg_ctx* c, const DBuf* planes, i64 n, int master, DBuf& lo) {
  DBuf out;
  out.alloc(sizeof(bf16) * (size_t)(n + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(out.p, 0, sizeof(bf16) * (size_t)(n + kPad), c->stream));
  if (master == FVG_F64 && n > 0) {  // FP32 / BF16 uploads: the FP32 plane is exact, the residual 0
    DBuf bad;
    bad.alloc(sizeof(unsigned), c->stream);
    FVG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(unsigned), c->stream));
    k_split_plane<<<grid_rows(c, n, 16), kSplitThreads, 0, c->stream>>>(
        planes[FVG_F64].as<double>(), planes[FVG_F32].as<float>(), out.as<bf16>(), n, bad.as<unsigned>());
    check_launch("split_plane");
    count_launch(c);
    unsigned hb = 0;
    FVG_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
    if (hb) fail(FVG_ERR_INVALID_ARG, "split storage: a value lies outside the FP32 range");
  }
  lo = std::move(out);
}

// The FP32 and residual planes of a value set; from FP64 values with neither
// plane yet, both in one pass.
void ensure_split_planes(fvg_ctx* c, DBuf* planes, i64 n, int master, DBuf& lo) {
  if (master == FVG_F64 && !planes[FVG_F32].p && !lo.p && n > 0) {
    DBuf hi, out, bad;
    hi.alloc(sizeof(float) * (size_t)(n + kPad), c->stream);
    out.alloc(sizeof(bf16) * (size_t)(n + kPad), c->stream);
    FVG_CUDA(cudaMemsetAsync(hi.as<float>() + n, 0, sizeof(float) * kPad, c->stream));
    FVG_CUDA(cudaMemsetAsync(out.as<bf16>() + n, 0, sizeof(bf16) * kPad, c->stream));
    bad.alloc(sizeof(unsigned), c->stream);
    FVG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(unsigned), c->stream));
    k_split_values<<<grid_rows(c, n, 16), kSplitThreads, 0, c->stream>>>(planes[FVG_F64].as<double>(), hi.as<float>(),
                                                                         out.as<bf16>(), n, bad.as<unsigned>());
    check_launch("split_values");
    count_launch(c);
    unsigned hb = 0;
    FVG_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
    if (hb) fail(FVG_ERR_INVALID_ARG, "split storage: a value lies outside the FP32 range");
    planes[FVG_F32] = std::move(hi);
    lo = std::move(out);
    return;
  }
  ensure_plane_generic(c, planes, n, FVG_F32, master);
  if (!lo.p) split_residual_plane(c, planes, n, master, lo);
}

void crs_ensure_split(fvg_ctx* c, DevCRS& a, int master) { ensure_split_planes(c, a.val, a.nnz, master, a.lo); }

void split_vector(fvg_ctx* c, const double* x, void* y, i64 n) {
  if (n <= 0) return;
  k_split_vec<<<grid_rows(c, n), kSplitThreads, 0, c->stream>>>(x, (float2*)y, n);
  check_launch("split_vec");
  count_launch(c);
}

i64 crs_split_scratch_bytes(fvg_ctx* c, DevCRS& a, bool y_df) {
  const Sched& s = crs_sched(c, a, split_crs_tile(y_df));
  return (i64)sizeof(float2) * std::max<i64>(s.npieces, 1);
}

void crs_pass_split(fvg_ctx* c, DevCRS& a, const void* x, bool y_df, void* y, void* scratch, int prof_key) {
  const Sched& s = crs_sched(c, a, split_crs_tile(y_df));
  if (!a.val[FVG_F32].p || !a.lo.p) fail(FVG_ERR_INTERNAL, "split storage planes missing");
  DBuf tmp;
  if (!scratch) {
    tmp.alloc((size_t)crs_split_scratch_bytes(c, a, y_df), c->stream);
    scratch = tmp.p;
  }
  ProfScope pr(c, prof_key);
  SplitK p;
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.vh = a.val[FVG_F32].as<float>();
  p.vl = a.lo.as<unsigned short>();
  p.x = (const float2*)x;
  p.items = s.items.as<Item>();
  p.nitems = s.nitems;
  p.y = y;
  p.partials = (float2*)scratch;
  if (s.nitems > 0) {
    const void* kfn = y_df ? (const void*)k_crs_split<float2> : (const void*)k_crs_split<double>;
    int grid = occupancy_blocks(kfn, kThreads) * c->num_sms;
    grid = (int)std::max<i64>(1, std::min<i64>(grid, s.nitems));
    if (y_df) k_crs_split<float2><<<grid, kThreads, 0, c->stream>>>(p);
    else k_crs_split<double><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_crs_split");
    count_launch(c);
  }
  if (s.nlong > 0) {
    const int fg = (int)std::max<i64>(1, std::min<i64>((s.nlong + 7) / 8, 4 * c->num_sms));
    if (y_df)
      k_fin_split<float2><<<fg, kThreads, 0, c->stream>>>(s.long_rows.as<i32>(), s.long_piece0.as<i32>(), s.nlong,
                                                          (const float2*)scratch, y);
    else
      k_fin_split<double><<<fg, kThreads, 0, c->stream>>>(s.long_rows.as<i32>(), s.long_piece0.as<i32>(), s.nlong,
                                                          (const float2*)scratch, y);
    check_launch("k_fin_split");
    count_launch(c);
  }
}

int glm_split_grid(fvg_ctx* c, i64 m) { return (int)grid_rows(c, m, 4); }

void glm_split_rows(fvg_ctx* c, const void* wtx, const void* head, i64 m, const GlmSplitArgs& e) {
  GlmSplitK p;
  p.wtx = (const float2*)wtx;
  p.head = (const float2*)head;
  p.m = m;
  p.lab = (const float2*)e.lab;
  p.sw = (const float2*)e.sw;
  p.intercept = e.intercept;
  p.icpt = e.icpt;
  p.kind = e.kind;
  p.eps = e.eps;
  p.r = (float2*)e.r;
  p.cta_part = e.cta_part;
  p.ticket = e.ticket;
  p.out = e.out;
  p.grad_bias = e.grad_bias;
  k_glm_split<<<glm_split_grid(c, m), kSplitThreads, 0, c->stream>>>(p);
  check_launch("k_glm_split");
  count_launch(c);
}

}  // namespace fvg
