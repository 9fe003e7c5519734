// Sparse products on the device.
//
// CRS (crs_matrix_spmv_impl, crs_matrix.hpp:1505-1516): one persistent
// kernel walks the matrix in row order as warp work items of at most 512
// nonzeros, built once per matrix on the host from the row offsets.  An item
// is either a tile of consecutive short rows (up to 248 rows, a bounded
// number of products per lane) or a piece of a long row (the finalize kernel
// adds the pieces in order).  A warp streams the item's values and column ids
// with coalesced evict-first loads, gathers x through the read-only path,
// stages the products in its own shared-memory slice and sums each row with
// 1..32 lanes.  All reductions have a fixed order, so results are
// deterministic run to run.
//
// The optional logistic epilogue fuses compute_wtx + logistic_gradient::
// compute_dloss + `* sample_weight` + bias sum (gradient_descent.hpp:196-211,
// gradient.hpp:15-53) into the same pass: it writes dloss*sw per row and
// per-CTA compensated partial sums of the loss and of dloss*sw (FP32 Kahan
// sums on the FP32-arithmetic path, which keep GB300's narrow FP64 unit out of
// the per-row work; FP64 Neumaier sums on the FP64 path), which the finalize
// kernel reduces in FP64 in a fixed order.
#include "device_common.cuh"

namespace fvg {

// ------------------------------------------------------------ kernel args
struct CrsK {
  const i32* off;
  const i32* idx;
  const void* val;
  const void* x;
  const Item* items;
  i64 nitems;
  int tile;
  void* y;
  void* partials;
  // logistic epilogue
  const double* label;
  const double* sw;
  const float* label_f;
  const float* sw_f;
  const double* intercept;
  int icpt;
  void* r;
  double* cta_part;
  unsigned* err;
  int loss;    // GLM loss kind
  double eps;  // its epsilon
  const float* ybase;  // FP32 path: per-row partial sums from another pass, added before the epilogue
};

template <class AT, class YT, int EPI, class S>
__device__ __forceinline__ void epilogue(const CrsK& p, i32 row, AT acc, AT b, S& ls, S& bs) {
  if (EPI == EPI_STORE) {
    ((YT*)p.y)[row] = (YT)acc;
  } else {
    AT wtx = acc + b;
    if constexpr (sizeof(AT) == 4)
      if (p.ybase) wtx += p.ybase[row];
    AT loss, d;
    if constexpr (sizeof(AT) == 8) {
      glm_row<AT>(p.loss, (AT)p.eps, wtx, p.label[row], loss, d);
      if (p.sw) d = d * p.sw[row];
    } else {
      glm_row<AT>(p.loss, (AT)p.eps, wtx, p.label_f[row], loss, d);
      if (p.sw_f) d = d * p.sw_f[row];
    }
    ((YT*)p.r)[row] = (YT)d;
    ls.add(loss);
    bs.add(d);
  }
}

// ------------------------------------------------------------ warp tiles

// Persistent CRS kernel.  Warp g of the grid handles items g, g+W, g+2W, ...
// (W = warps in the grid).  Phase 1: the warp streams the item's nonzeros
// with coalesced loads (lane L: nonzeros L, L+32, ...; a group of rounds
// issued before any use), gathers x and writes the products to its own
// shared-memory slice.  Phase 2: rows of a tile are
// summed from shared memory by 1..32 lanes each (32 / rows, rounded to a
// power of two), the lanes of a row combined by shuffles; a piece is summed
// by the whole warp.  No CTA-wide barrier inside the loop.
template <class VT, class XT, class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads, FVG_CRS_MIN_BLOCKS) k_crs(const CrsK p) {
  constexpr int SPAN = kWarpTile;        // products slice per warp
  constexpr int NR = SPAN / 32;          // element rounds per lane
  constexpr int RG = sizeof(VT) == 8 ? (FVG_CRS_ROUNDS + 1) / 2 : FVG_CRS_ROUNDS;  // rounds in flight together
  // FP64: GB300 issues FP64 at a small fraction of the FP32 rate, so phase 1
  // only gathers x and phase 2 does one fused multiply-add per nonzero
  // (instead of a multiply here and an add there) with the value re-read
  // (the warp streamed it just before: L1/L2)
  constexpr bool kFmaRows = sizeof(AT) == 8;
  __shared__ AT sprod[kThreads / 32][SPAN];
  __shared__ int soffs[kThreads / 32][kTileRows + 1];
  using Sum = typename SumOf<AT>::type;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  AT* prod = sprod[w];
  int* soff = soffs[w];
  const i64 W = (i64)gridDim.x * (kThreads / 32);
  const i64 n = p.nitems;
  const XT* __restrict__ x = (const XT*)p.x;
  const VT* __restrict__ val = (const VT*)p.val;
  Sum ls, bs;
  const AT bias = (EPI == EPI_LOGREG && p.icpt) ? (AT)*p.intercept : (AT)0;
  i64 t = (i64)blockIdx.x * (kThreads / 32) + w;
  Item nx = (t < n) ? p.items[t] : Item{0, 0, 0, 0};
  for (; t < n; t += W) {
    const Item it = nx;
    if (t + W < n) nx = p.items[t + W];  // prefetch the next descriptor
    const int a0 = it.e0;
    const int span = it.e1 - a0;
    // row boundaries of a tile into the warp's offsets slice
    if (it.r1 >= 0)
      for (int k = lane; k <= it.r1 - it.r0; k += 32) soff[k] = __ldg(p.off + it.r0 + k);
    // phase 1: lane L takes nonzeros L, L+32, ... so one gather instruction
    // covers 32 consecutive nonzeros (neighbouring columns / rows share
    // sectors); RG rounds of loads are issued before their gathers.
#pragma unroll
    for (int g = 0; g < NR; g += RG) {
      int c[RG];
      AT v[RG];
#pragma unroll
      for (int q = 0; q < RG; q++) {
        const int k = (g + q) * 32 + lane;
        if (g + q < NR && k < span) {
          c[q] = __ldcs(p.idx + a0 + k);
          if constexpr (!kFmaRows) v[q] = ld_val<VT, AT>(val + a0 + k);
        }
      }
#pragma unroll
      for (int q = 0; q < RG; q++) {
        const int k = (g + q) * 32 + lane;
        if (g + q < NR && k < span) {
          if constexpr (kFmaRows) prod[k] = (AT)__ldg(x + c[q]);  // the value joins in phase 2
          else prod[k] = v[q] * (AT)__ldg(x + c[q]);
        }
      }
    }
    __syncwarp();
    // phase 2
    if (it.r1 >= 0) {
      // Gl lanes per row: 32 / R rounded to a power of two; tiles of 32 or
      // more (short) rows take rounds of 32 rows, one lane each
      const int R = it.r1 - it.r0;
      const int Gl = lanes_per_row(R);  // the packer keeps a lane's share <= kLaneWork
      const int per_round = 32 / Gl;
      for (int rb = 0; rb < R; rb += per_round) {
        const int j = rb + lane / Gl, sub = lane % Gl;
        AT acc = 0;
        if (j < R) {
          const int s = soff[j] - a0, e = soff[j + 1] - a0;
          int k = s + sub;
          if constexpr (kFmaRows) {
            const VT* vr = val + a0;
            if (e - s > 4 * Gl) {
              AT a1 = 0, a2 = 0, a3 = 0;
              for (; k + 3 * Gl < e; k += 4 * Gl) {
                acc = fma((AT)vr[k], prod[k], acc);
                a1 = fma((AT)vr[k + Gl], prod[k + Gl], a1);
                a2 = fma((AT)vr[k + 2 * Gl], prod[k + 2 * Gl], a2);
                a3 = fma((AT)vr[k + 3 * Gl], prod[k + 3 * Gl], a3);
              }
              for (; k < e; k += Gl) acc = fma((AT)vr[k], prod[k], acc);
              acc = (acc + a1) + (a2 + a3);
            } else {
              for (; k < e; k += Gl) acc = fma((AT)vr[k], prod[k], acc);
            }
          } else {
            AT a1 = 0, a2 = 0, a3 = 0;
            for (; k + 3 * Gl < e; k += 4 * Gl) {
              acc += prod[k];
              a1 += prod[k + Gl];
              a2 += prod[k + 2 * Gl];
              a3 += prod[k + 3 * Gl];
            }
            for (; k < e; k += Gl) acc += prod[k];
            acc = (acc + a1) + (a2 + a3);
          }
        }
        for (int o = Gl >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (j < R && sub == 0) epilogue<AT, YT, EPI>(p, it.r0 + j, acc, bias, ls, bs);
      }
    } else {
      AT acc = 0;
      if constexpr (kFmaRows) {
        for (int k = it.e0 - a0 + lane; k < span; k += 32) acc = fma((AT)val[a0 + k], prod[k], acc);
      } else {
        for (int k = it.e0 - a0 + lane; k < span; k += 32) acc += prod[k];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) ((AT*)p.partials)[-1 - it.r1] = acc;
    }
    __syncwarp();
  }
  if (EPI == EPI_LOGREG) block_csum2(ls.total(), bs.total(), &p.cta_part[2 * blockIdx.x], &p.cta_part[2 * blockIdx.x + 1]);
}

// ------------------------------------------------------------- finalize
struct FinK {
  const i32* long_rows;
  const i32* long_piece0;
  i64 nlong;
  const void* partials;
  void* y;
  // logistic
  const double* label;
  const double* sw;
  const float* label_f;
  const float* sw_f;
  const double* intercept;
  int icpt;
  void* r;
  const double* cta_part;
  i64 ncta;
  double* long_part;
  double* out;        // [loss, bias]
  double* grad_bias;  // optional
  unsigned* ticket;
  int loss;
  double eps;
  const float* ybase;
};

// Long rows: sum the pieces' partials in piece order and apply the
// epilogue; then (logistic) the last CTA reduces every partial loss / bias
// in a fixed order.
template <class AT, class YT, int EPI>
__global__ void __launch_bounds__(kThreads) k_finalize(const FinK f) {
  const AT b = (EPI == EPI_LOGREG && f.icpt) ? (AT)*f.intercept : (AT)0;
  const int lane = threadIdx.x & 31;
  // a warp per long row: lane L adds pieces L, L+32, ..., then the warp's tree
  for (i64 i = (i64)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); i < f.nlong;
       i += (i64)gridDim.x * (kThreads / 32)) {
    i64 c0 = f.long_piece0[i], c1 = f.long_piece0[i + 1];
    AT acc = 0;
    for (i64 j = c0 + lane; j < c1; j += 32) acc += ((const AT*)f.partials)[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      i32 row = f.long_rows[i];
      if (EPI == EPI_STORE) {
        ((YT*)f.y)[row] = (YT)acc;
      } else {
        AT loss, d, wtx = acc + b;
        if constexpr (sizeof(AT) == 4)
          if (f.ybase) wtx += f.ybase[row];
        if constexpr (sizeof(AT) == 8) {
          glm_row<AT>(f.loss, (AT)f.eps, wtx, f.label[row], loss, d);
          if (f.sw) d = d * f.sw[row];
        } else {
          glm_row<AT>(f.loss, (AT)f.eps, wtx, f.label_f[row], loss, d);
          if (f.sw_f) d = d * f.sw_f[row];
        }
        ((YT*)f.r)[row] = (YT)d;
        f.long_part[2 * i] = (double)loss;
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
  block_csum2(ls.total(), bs.total(), &tl, &tb);
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
  char* pa = take(at_size * (size_t)std::max<i64>(s.npieces, 1));
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
  // pieces depend only on the item size, which FP32 and BF16 share
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  return (i64)carve(nullptr, s, c->grid_spmv, 8, nullptr);
}

template <class VT, class XT, class AT, class YT, int EPI>
static int crs_grid(fvg_ctx* c, int tile) {
  (void)tile;
  return occupancy_blocks((const void*)k_crs<VT, XT, AT, YT, EPI>, kThreads) * c->num_sms;
}

template <class VT, class XT, class AT, class YT, int EPI>
static void launch_crs(fvg_ctx* c, DevCRS& a, const Sched& s, int storage, const void* x, void* y,
                       const LogregEpi* lr, const PassScratch& ps, bool timed = true) {
  CrsK p;
  p.off = a.off.as<i32>();
  p.idx = a.idx.as<i32>();
  p.val = a.val[storage].p;
  p.x = x;
  p.items = s.items.as<Item>();
  p.nitems = s.nitems;
  p.tile = s.tile;
  p.y = y;
  p.partials = ps.partials;
  p.label = lr ? lr->label : nullptr;
  p.sw = lr ? lr->sw : nullptr;
  p.label_f = lr ? lr->label_f : nullptr;
  p.sw_f = lr ? lr->sw_f : nullptr;
  p.intercept = lr ? lr->intercept : nullptr;
  p.icpt = lr ? lr->icpt : 0;
  p.r = lr ? lr->r : nullptr;
  p.ybase = lr ? lr->ybase : nullptr;
  p.cta_part = ps.cta_part;
  p.err = c->dev_err;
  p.loss = lr ? lr->loss : 0;
  p.eps = lr ? lr->eps : 0.0;
  int grid = (int)std::max<i64>(1, std::min<i64>(crs_grid<VT, XT, AT, YT, EPI>(c, s.tile), s.nitems));
  grid = std::min(grid, c->grid_spmv);
  if (s.nitems > 0) {
    k_crs<VT, XT, AT, YT, EPI><<<grid, kThreads, 0, c->stream>>>(p);
    check_launch("k_crs");
    count_launch(c);
  }
  if (s.nlong > 0 || EPI == EPI_LOGREG) {
    FinK f;
    f.long_rows = s.long_rows.as<i32>();
    f.long_piece0 = s.long_piece0.as<i32>();
    f.nlong = s.nlong;
    f.partials = ps.partials;
    f.y = y;
    f.label = p.label;
    f.sw = p.sw;
    f.label_f = p.label_f;
    f.sw_f = p.sw_f;
    f.intercept = p.intercept;
    f.icpt = p.icpt;
    f.r = p.r;
    f.ybase = p.ybase;
    f.cta_part = ps.cta_part;
    f.ncta = s.nitems > 0 ? grid : 0;
    f.long_part = ps.long_part;
    f.out = (lr && lr->out) ? lr->out : ps.out;
    f.grad_bias = lr ? lr->grad_bias : nullptr;
    f.ticket = ps.ticket;
    f.loss = p.loss;
    f.eps = p.eps;
    int fg = (int)std::max<i64>(1, std::min<i64>((s.nlong + 7) / 8, 4 * c->num_sms));  // a warp per long row
    ProfScope pf(c, timed ? P_FINALIZE : P_NKEYS);
    k_finalize<AT, YT, EPI><<<fg, kThreads, 0, c->stream>>>(f);
    check_launch("k_finalize");
    count_launch(c);
  }
}

void crs_pass(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* x, int y_dt, void* y, int epi,
              const LogregEpi* lr, void* scratch, int prof_key) {
  const Sched& s = crs_sched(c, a, tile_for_storage(storage));
  if (!a.val[storage].p) fail(FVG_ERR_INTERNAL, "missing value plane for the requested storage");
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
  if (epi == EPI_LOGREG && storage != FVG_F64 && !(lr && lr->label_f))
    fail(FVG_ERR_INTERNAL, "FP32 logistic pass needs FP32 labels");
  ProfScope pr(c, prof_key);
  const int out_dt = (epi == EPI_LOGREG) ? (lr ? lr->r_dt : y_dt) : y_dt;
  if (storage == FVG_F64) {
    if (x_dt != FVG_F64 || out_dt != FVG_F64) fail(FVG_ERR_INVALID_ARG, "FP64 values need FP64 vectors");
    if (epi == EPI_STORE) launch_crs<double, double, double, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps);
    else launch_crs<double, double, double, double, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps);
  } else if (storage == FVG_F32) {
    if (x_dt != FVG_F32) fail(FVG_ERR_INVALID_ARG, "FP32 values need FP32 input vectors");
    if (epi == EPI_STORE && out_dt == FVG_F64)
      launch_crs<float, float, float, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps);
    else if (epi == EPI_STORE)
      launch_crs<float, float, float, float, EPI_STORE>(c, a, s, storage, x, y, lr, ps);
    else
      launch_crs<float, float, float, float, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps);
  } else {
    if (x_dt != FVG_F32) fail(FVG_ERR_INVALID_ARG, "BF16 values need FP32 input vectors");
    if (epi == EPI_STORE && out_dt == FVG_F64)
      launch_crs<bf16, float, float, double, EPI_STORE>(c, a, s, storage, x, y, lr, ps);
    else if (epi == EPI_STORE)
      launch_crs<bf16, float, float, float, EPI_STORE>(c, a, s, storage, x, y, lr, ps);
    else
      launch_crs<bf16, float, float, float, EPI_LOGREG>(c, a, s, storage, x, y, lr, ps);
  }
}

// y = A x over a CRS layout whose work schedule already exists, with the
// caller's scratch (piece partial sums only) and no allocation of any kind.
// Returns the scratch bytes the pass needs when scratch is null.
size_t crs_spmv_no_alloc(fvg_ctx* c, DevCRS& a, int storage, const void* x, void* y, void* scratch,
                         size_t scratch_bytes) {
  const Sched* s = a.sched[0].get();
  if (!s) fail(FVG_ERR_INVALID_ARG, "matrix not prepared: call fvg_matrix_prepare(ctx, mat, FVG_CRS, ...) first");
  if (!a.val[storage].p) fail(FVG_ERR_INVALID_ARG, "value plane missing: call fvg_matrix_add_storage first");
  const size_t at_size = (storage == FVG_F64) ? 8 : 4;
  const size_t need = at_size * (size_t)std::max<i64>(s->npieces, 1);
  if (!scratch) return need;
  if (need > scratch_bytes) fail(FVG_ERR_INVALID_ARG, "matrix needs more scratch than the allocation-free entry point has");
  PassScratch ps = {};
  ps.partials = scratch;
  if (storage == FVG_F64)
    launch_crs<double, double, double, double, EPI_STORE>(c, a, *s, storage, x, y, nullptr, ps, false);
  else if (storage == FVG_F32)
    launch_crs<float, float, float, float, EPI_STORE>(c, a, *s, storage, x, y, nullptr, ps, false);
  else
    launch_crs<bf16, float, float, float, EPI_STORE>(c, a, *s, storage, x, y, nullptr, ps, false);
  return need;
}

// ------------------------------------------------------------------- JDS
// Work items (JdsItem): a warp per block of 32 consecutive permuted rows
// (lane = row) and at most kJdsSeg of the block's diagonals.  Diagonal d of
// row p sits at off[d] + p, so the warp reads each diagonal's 32 entries
// with one coalesced access; row p has diagonal d iff the diagonal's length
// off[d+1] - off[d] exceeds p.  Four diagonals are summed into four
// accumulators, added as (a0 + a1) + (a2 + a3) at the item's end.  A block
// with more diagonals than one item holds leaves per-row partials, which
// k_jds_split adds in diagonal order.  part (hybrid) adds the CRS tail of
// the first npart permuted rows after the JDS sum, as
// jds_crs_hybrid_spmv_impl does (jds_crs_hybrid.hpp:198-211).
template <class VT, class XT, class AT>
__device__ __forceinline__ AT jds_term(const VT* __restrict__ val, const i32* __restrict__ idx,
                                       const XT* __restrict__ x, i64 q) {
  return (AT)val[q] * (AT)__ldg(x + __ldg(idx + q));
}

template <class VT, class XT, class AT, class YT>
__global__ void __launch_bounds__(256) k_jds(const JdsItem* __restrict__ items, i64 nitems,
                                             const i32* __restrict__ perm, const i64* __restrict__ off,
                                             const i32* __restrict__ idx, const VT* __restrict__ val, i64 m,
                                             const XT* __restrict__ x, YT* __restrict__ y,
                                             const AT* __restrict__ part, i64 npart, AT* __restrict__ partials) {
  const int lane = threadIdx.x & 31;
  const i64 nw = ((i64)gridDim.x * blockDim.x) >> 5;
  for (i64 it = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < nitems; it += nw) {
    const JdsItem t = items[it];
    const i64 p = (i64)t.b * 32 + lane;
    AT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    i64 d = t.d0;
    i64 o = __ldg(off + d);
    for (; d + 3 < t.d1; d += 4) {
      const i64 o1 = __ldg(off + d + 1), o2 = __ldg(off + d + 2), o3 = __ldg(off + d + 3), o4 = __ldg(off + d + 4);
      if (p < o1 - o) a0 += jds_term<VT, XT, AT>(val, idx, x, o + p);
      if (p < o2 - o1) a1 += jds_term<VT, XT, AT>(val, idx, x, o1 + p);
      if (p < o3 - o2) a2 += jds_term<VT, XT, AT>(val, idx, x, o2 + p);
      if (p < o4 - o3) a3 += jds_term<VT, XT, AT>(val, idx, x, o3 + p);
      o = o4;
    }
    for (; d < t.d1; d++) {
      const i64 o1 = __ldg(off + d + 1);
      if (p < o1 - o) a0 += jds_term<VT, XT, AT>(val, idx, x, o + p);
      o = o1;
    }
    AT acc = (a0 + a1) + (a2 + a3);
    if (t.slot >= 0) {
      partials[(i64)t.slot * 32 + lane] = acc;
    } else if (p < m) {
      if (p < npart) acc = acc + part[p];
      y[perm[p]] = (YT)acc;
    }
  }
}

// blocks cut into several items: their partials in diagonal order
template <class AT, class YT>
__global__ void __launch_bounds__(256) k_jds_split(const JdsSplit* __restrict__ sp, i64 nsplits,
                                                   const i32* __restrict__ perm, i64 m, YT* __restrict__ y,
                                                   const AT* __restrict__ part, i64 npart,
                                                   const AT* __restrict__ partials) {
  const int lane = threadIdx.x & 31;
  const i64 nw = ((i64)gridDim.x * blockDim.x) >> 5;
  for (i64 i = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nsplits; i += nw) {
    const JdsSplit s = sp[i];
    const i64 p = (i64)s.b * 32 + lane;
    AT acc = 0;
    for (int q = 0; q < s.nslot; q++) acc += partials[(i64)(s.slot0 + q) * 32 + lane];
    if (p < m) {
      if (p < npart) acc = acc + part[p];
      y[perm[p]] = (YT)acc;
    }
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
    DBuf partials;
    if (j.nslots > 0) partials.alloc(sizeof(AT) * 32 * (size_t)j.nslots, c->stream);
    k_jds<VT, XT, AT, YT><<<grid_rows(j.nitems * 32), 256, 0, c->stream>>>(
        j.items.as<JdsItem>(), j.nitems, j.perm.as<i32>(), j.off.as<i64>(), j.idx.as<i32>(), j.val[storage].as<VT>(),
        j.m, (const XT*)x, (YT*)y, (const AT*)part, npart, partials.as<AT>());
    if (j.nsplits > 0) {
      check_launch("k_jds");
      count_launch(c);
      k_jds_split<AT, YT><<<grid_rows(j.nsplits * 32), 256, 0, c->stream>>>(
          j.splits.as<JdsSplit>(), j.nsplits, j.perm.as<i32>(), j.m, (YT*)y, (const AT*)part, npart,
          partials.as<AT>());
    }
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

// Resident CTAs per SM of the heaviest CRS instantiation (sizes the
// persistent grid).
// Upper bound of resident 256-thread CTAs per SM; sizes the per-CTA partial
// buffers (the launch itself uses the occupancy of each instantiation).
int crs_blocks_per_sm() { return 2048 / kThreads; }

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
  typename SumOf<AT>::type ls, bs;
  const AT b = p.icpt ? (AT)*p.intercept : (AT)0;
  for (i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x; r < m; r += (i64)gridDim.x * blockDim.x)
    epilogue<AT, AT, EPI_LOGREG>(p, (i32)r, wtx[r], b, ls, bs);
  block_csum2(ls.total(), bs.total(), &p.cta_part[2 * blockIdx.x], &p.cta_part[2 * blockIdx.x + 1]);
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
  p.label_f = lr.label_f;
  p.sw_f = lr.sw_f;
  p.intercept = lr.intercept;
  p.icpt = lr.icpt;
  p.r = lr.r;
  p.cta_part = cta;
  p.loss = lr.loss;
  p.eps = lr.eps;
  if (wtx_dt == FVG_F64) k_logreg_rows<double><<<grid, 256, 0, c->stream>>>((const double*)wtx, m, p);
  else k_logreg_rows<float><<<grid, 256, 0, c->stream>>>((const float*)wtx, m, p);
  check_launch("k_logreg_rows");
  count_launch(c);
  FinK f = {};
  f.nlong = 0;
  f.label = lr.label;
  f.sw = lr.sw;
  f.label_f = lr.label_f;
  f.sw_f = lr.sw_f;
  f.intercept = lr.intercept;
  f.icpt = lr.icpt;
  f.r = lr.r;
  f.cta_part = cta;
  f.ncta = grid;
  f.out = lr.out ? lr.out : out;
  f.grad_bias = lr.grad_bias;
  f.ticket = ticket;
  f.loss = lr.loss;
  f.eps = lr.eps;
  if (wtx_dt == FVG_F64) k_finalize<double, double, EPI_LOGREG><<<1, kThreads, 0, c->stream>>>(f);
  else k_finalize<float, float, EPI_LOGREG><<<1, kThreads, 0, c->stream>>>(f);
  check_launch("k_finalize_rows");
  count_launch(c);
}

}  // namespace fvg
