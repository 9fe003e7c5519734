// Shared-memory gathers for the FP32-arithmetic passes, and the device
// packing of every work-item schedule.
//
// Backward product g = A^T r (row panels).  The reference multiplies its
// transposed copy (crs_matrix.hpp:356-412 builds it, gradient_descent.hpp:211
// multiplies it with dloss), and so does the plain path here: every nonzero
// of A^T gathers r[source row].  With millions of rows r sits in L2 and each
// gather of a sparsely used column fetches a 32-byte sector for 4 useful
// bytes, so that pass is bound by L2-to-SM traffic, far below HBM speed.
// The row-panel layout regroups the columns that occur in most stretches of
// rows.  A's rows are cut into panels of `rows` consecutive rows.  A CTA
// copies one panel's slice of r into shared memory and walks the panel's
// entries of the hot columns in (column, row) order, gathering from shared
// memory; each (panel, hot column) pair gives one FP32 partial sum ("panel
// row" q = panel * nhot + h).  g[hot column] is the compensated sum of its
// partials in a fixed order.  Columns with fewer entries keep their rows in
// a transposed CRS of their own (the hot rows emptied), multiplied by the
// plain CRS kernel first.
//
// Forward product A w (forward head).  The entries of A's most frequent
// columns form a CRS of their own with 2-byte column slots; every CTA stages
// w at those columns once and sums its share of the rows' head entries with
// the same kernel; the rest of each row goes through the plain CRS kernel,
// whose logistic epilogue adds the head partial (crs_matrix.hpp:1505-1516 is
// the product, gradient_descent.hpp:227-240 and gradient.hpp:15-53 the
// epilogue).
//
// Every sum has a fixed order, so results are the same on every run.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "bulk_copy.cuh"
#include "device_common.cuh"
#include "df64.cuh"

namespace fvg {

namespace {

unsigned grid_n(i64 n, int threads = 256) {
  i64 g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}
#define PGRID_STRIDE(i, n) for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (i64)gridDim.x * blockDim.x)
#define PWARP_STRIDE(q, n)                                                              \
  for (i64 q = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < (n);             \
       q += ((i64)gridDim.x * blockDim.x) >> 5)

constexpr int kPanelWarps = 32;          // one CTA of 32 warps per SM
constexpr i64 kPanelRowsAuto = 1 << 30;  // auto: the tallest panels shared memory holds
constexpr double kPanelMinAuto = 2.0;    // hot: >= this many entries per panel on average

// ------------------------------------------------------------------ build
__global__ void k_hot_flags(const i32* __restrict__ toff, i64 n, i64 thresh, i64* __restrict__ flag) {
  PGRID_STRIDE(c, n) flag[c] = ((i64)toff[c + 1] - toff[c] >= thresh) ? 1 : 0;
}

__global__ void k_hot_list(const i64* __restrict__ flag, const i64* __restrict__ pos, i64 n, i32* __restrict__ hot) {
  PGRID_STRIDE(c, n) if (flag[c]) hot[pos[c]] = (i32)c;
}

// B[h*(np+1) + p]: position in A^T of the first entry of hot column h whose
// source row is >= p*rows (the column's source rows ascend).
__global__ void k_panel_bounds(const i32* __restrict__ toff, const i32* __restrict__ tidx, const i32* __restrict__ hot,
                               i64 nhot, i64 np, i64 rows, i32* __restrict__ B) {
  PGRID_STRIDE(i, nhot * (np + 1)) {
    const i64 h = i / (np + 1), p = i - h * (np + 1);
    const i32 c = hot[h];
    i64 lo = toff[c], hi = toff[c + 1];
    const i64 target = p * rows;
    while (lo < hi) {
      const i64 mid = (lo + hi) >> 1;
      if ((i64)tidx[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    B[i] = (i32)lo;
  }
}

__global__ void k_panel_lens(const i32* __restrict__ B, i64 nhot, i64 np, i64* __restrict__ len) {
  PGRID_STRIDE(q, np * nhot) {
    const i64 p = q / nhot, h = q - p * nhot;
    len[q] = (i64)B[h * (np + 1) + p + 1] - B[h * (np + 1) + p];
  }
}

__global__ void k_i64_to_i32(const i64* __restrict__ s, i32* __restrict__ d, i64 n) {
  PGRID_STRIDE(i, n) d[i] = (i32)s[i];
}

// The source's other value planes (FP32, BF16, split residual) that a fill
// copies beside the master plane, so that a layout built from a matrix that
// already holds them needs no conversion afterwards; null where absent.
struct SidePlanes {
  const float* s32 = nullptr;
  float* d32 = nullptr;
  const bf16* s16 = nullptr;
  bf16* d16 = nullptr;
  const bf16* slo = nullptr;
  bf16* dlo = nullptr;
  __device__ __forceinline__ void copy(i64 from, i64 to) const {
    if (s32) d32[to] = s32[from];
    if (s16) d16[to] = s16[from];
    if (slo) dlo[to] = slo[from];
  }
};

// a warp per panel row: its entries copied with the row made panel-local
template <class T>
__global__ void k_panel_fill(const i32* __restrict__ B, const i64* __restrict__ poff, const i32* __restrict__ tidx,
                             const T* __restrict__ tval, i64 nhot, i64 np, i64 rows, uint16_t* __restrict__ prow,
                             T* __restrict__ pval, const SidePlanes sp) {
  const int lane = threadIdx.x & 31;
  PWARP_STRIDE(q, np * nhot) {
    const i64 p = q / nhot, h = q - p * nhot;
    const i64 s = B[h * (np + 1) + p], e = B[h * (np + 1) + p + 1], d = poff[q];
    const i64 r0 = p * rows;
    for (i64 k = lane; k < e - s; k += 32) {
      prow[d + k] = (uint16_t)(tidx[s + k] - r0);
      pval[d + k] = tval[s + k];
      sp.copy(s + k, d + k);
    }
  }
}

__global__ void k_cold_lens(const i32* __restrict__ toff, const i64* __restrict__ flag, i64 n, i64* __restrict__ len) {
  PGRID_STRIDE(c, n) len[c] = flag[c] ? 0 : (i64)toff[c + 1] - toff[c];
}

template <class T>
__global__ void k_cold_fill(const i32* __restrict__ toff, const i64* __restrict__ flag, const i64* __restrict__ coff,
                            i64 n, const i32* __restrict__ tidx, const T* __restrict__ tval, i32* __restrict__ cidx,
                            T* __restrict__ cval, const SidePlanes sp) {
  const int lane = threadIdx.x & 31;
  PWARP_STRIDE(c, n) {
    if (flag[c]) continue;
    const i64 s = toff[c], e = toff[c + 1], d = coff[c];
    for (i64 k = lane; k < e - s; k += 32) {
      cidx[d + k] = tidx[s + k];
      cval[d + k] = tval[s + k];
      sp.copy(s + k, d + k);
    }
  }
}

// Work items of a CRS, one thread per chunk of rows (chunk p: piece p % sub
// of the stretch of nhot rows p / sub), with the CRS schedule's packing rules
// (tiles of short rows within `tile` entries, kTileRows rows and kLaneWork
// products per lane; longer rows in pieces cut at 8-element boundaries).  The
// greedy packing is sequential within a chunk; a thread walks its chunk's
// offsets in order, loading them 8 at a time.  Pass 0 counts each chunk's items, long rows and pieces;
// pass 1 writes them at the scanned offsets `base` (chunk-major: a chunk's
// items, long rows and pieces are contiguous and numbered globally).
__global__ void k_panel_pack(const i32* __restrict__ off, i64 nrows, i64 nhot, i64 sub, i64 np, int tile, int write,
                             i32* __restrict__ cnt, const i32* __restrict__ base, Item* __restrict__ items,
                             i32* __restrict__ lrows, i32* __restrict__ lpiece0, i32* __restrict__ lfirst) {
  const i64 step = (nhot + sub - 1) / sub;
  for (i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += (i64)gridDim.x * blockDim.x) {
    const i64 s0 = (p / sub) * nhot, s1 = min(s0 + nhot, nrows), j = p % sub;
    const i64 r0 = min(s0 + j * step, s1), r1 = min(r0 + step, s1);
    const i32 bi = write ? base[p] : 0, bl = write ? base[(np + 1) + p] : 0, bp = write ? base[2 * (np + 1) + p] : 0;
    i32 ni = 0, nl = 0, npc = 0;
    i64 t0 = r0, tnnz = 0, tmax = 0;
    i32 o_cur = off[r0], o_t0 = o_cur;  // off[r], off[t0]
    auto row = [&](i64 r, i32 o_next) {
      const i64 len = (i64)o_next - o_cur;
      if (len > tile) {
        if (r > t0) {
          if (write) items[bi + ni] = Item{(int32_t)t0, (int32_t)r, o_t0, o_cur};
          ni++;
        }
        const i64 st = o_cur, en = o_next, b8 = st & ~7ll;
        const i64 npr = (en - b8 + tile - 1) / tile;  // pieces: b8 + k*tile < en
        if (write) {  // its pieces' items: k_long_pieces
          lrows[bl + nl] = (i32)r;
          lpiece0[bl + nl] = bp + npc;
          lfirst[bl + nl] = bi + ni;
        }
        nl++;
        ni += (i32)npr;
        npc += (i32)npr;
        t0 = r + 1;
        o_t0 = o_next;
        tnnz = 0;
        tmax = 0;
      } else {
        if (r > t0) {
          const i64 R = r - t0 + 1, mx = max(tmax, len);
          if (tnnz + len > tile || R > kTileRows || mx > (i64)kLaneWork * lanes_per_row((int)R)) {
            if (write) items[bi + ni] = Item{(int32_t)t0, (int32_t)r, o_t0, o_cur};
            ni++;
            t0 = r;
            o_t0 = o_cur;
            tnnz = 0;
            tmax = 0;
          }
        }
        tnnz += len;
        tmax = max(tmax, len);
      }
      o_cur = o_next;
    };
    // the offsets of 8 rows are loaded together, then the rows walked in order
    i64 r = r0;
    for (; r + 8 <= r1; r += 8) {
      i32 o[8];
#pragma unroll
      for (int q = 0; q < 8; q++) o[q] = off[r + 1 + q];
#pragma unroll
      for (int q = 0; q < 8; q++) row(r + q, o[q]);
    }
    for (; r < r1; r++) row(r, off[r + 1]);
    if (r1 > t0) {
      if (write) items[bi + ni] = Item{(int32_t)t0, (int32_t)r1, o_t0, o_cur};
      ni++;
    }
    if (!write) {
      cnt[p] = ni;
      cnt[np + p] = nl;
      cnt[2 * np + p] = npc;
    }
  }
}

// The items of the long rows' pieces (piece k of a row starting at st:
// [st, b8 + tile) for k = 0, then [b8 + k*tile, b8 + (k+1)*tile) cut at the
// row's end, b8 = st rounded down to 8), a warp per long row.
__global__ void k_long_pieces(const i32* __restrict__ off, const i32* __restrict__ lrows,
                              const i32* __restrict__ lpiece0, const i32* __restrict__ lfirst, i64 nlong, int tile,
                              Item* __restrict__ items) {
  const int lane = threadIdx.x & 31;
  PWARP_STRIDE(L, nlong) {
    const i32 r = lrows[L];
    const i64 st = off[r], en = off[r + 1], b8 = st & ~7ll;
    const i64 npr = (en - b8 + tile - 1) / tile;
    const i64 it0 = lfirst[L], pc0 = lpiece0[L];
    for (i64 k = lane; k < npr; k += 32) {
      const i64 e0 = (k == 0) ? st : b8 + k * tile, e1 = min(en, b8 + (k + 1) * tile);
      items[it0 + k] = Item{(int32_t)r, (int32_t)(-1 - (pc0 + k)), (int32_t)e0, (int32_t)e1};
    }
  }
}

// ---------------------------------------------------------- forward head
// The forward product y = A w gathers w[col] for every nonzero; the
// frequent columns' part of it takes the same route as the panels: A's
// entries in the H most frequent columns ("head") form their own CRS with
// uint16 column slots, and every CTA stages w at those columns in shared
// memory once.  The rows are cut into one stretch per CTA ("virtual
// panels" of the panel kernel); the rest of each row ("tail") stays a CRS
// with int32 column ids whose pass adds the head partial before the
// logistic epilogue.

// sort keys of the head selection: decreasing count (31-bit), the column
__global__ void k_head_keys(const i32* __restrict__ toff, i64 n, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ cols) {
  PGRID_STRIDE(j, n) {
    keys[j] = 0x7fffffffu - (uint32_t)(toff[j + 1] - toff[j]);
    cols[j] = (uint32_t)j;
  }
}

__global__ void k_head_slots(const uint32_t* __restrict__ cols, i64 H, i32* __restrict__ slot) {
  PGRID_STRIDE(i, H) slot[cols[i]] = (i32)i;
}

// per row: entries in head columns (slot >= 0) and in the tail
__global__ void k_head_counts(const i32* __restrict__ off, const i32* __restrict__ idx, i64 m,
                              const i32* __restrict__ slot, i64* __restrict__ hcnt, i64* __restrict__ tcnt) {
  const int lane = threadIdx.x & 31;
  PWARP_STRIDE(r, m) {
    const i64 s0 = off[r], e0 = off[r + 1];
    int h = 0;
    for (i64 e = s0 + lane; e < e0; e += 32) h += slot[idx[e]] >= 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if (lane == 0) {
      hcnt[r] = h;
      tcnt[r] = (e0 - s0) - h;
    }
  }
}

// head offsets padded to Q rows (rows past m are empty)
__global__ void k_head_off(const i64* __restrict__ hoff, i64 m, i64 Q, i32* __restrict__ poff) {
  PGRID_STRIDE(q, Q + 1) poff[q] = (i32)hoff[q < m ? q : m];
}

// a warp per row: head entries (slot, value) and tail entries (column,
// value), each in the row's order
template <class T>
__global__ void k_head_fill(const i32* __restrict__ off, const i32* __restrict__ idx, const T* __restrict__ val,
                            i64 m, const i32* __restrict__ slot, const i64* __restrict__ hoff,
                            const i64* __restrict__ toff, uint16_t* __restrict__ hslot, T* __restrict__ hval,
                            i32* __restrict__ tidx, T* __restrict__ tval, const SidePlanes sph,
                            const SidePlanes spt) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  PWARP_STRIDE(r, m) {
    const i64 s0 = off[r], e0 = off[r + 1];
    i64 hp = hoff[r], tp = toff[r];
    for (i64 b = s0; b < e0; b += 32) {
      const i64 e = b + lane;
      const bool ok = e < e0;
      const i32 col = ok ? idx[e] : 0;
      const i32 sl = ok ? slot[col] : -1;
      const bool head = ok && sl >= 0;
      const unsigned hb = __ballot_sync(0xffffffffu, head);
      const unsigned tb = __ballot_sync(0xffffffffu, ok && !head);
      if (head) {
        const i64 q = hp + __popc(hb & lt);
        hslot[q] = (uint16_t)sl;
        hval[q] = val[e];
        sph.copy(e, q);
      } else if (ok) {
        const i64 q = tp + __popc(tb & lt);
        tidx[q] = col;
        tval[q] = val[e];
        spt.copy(e, q);
      }
      hp += __popc(hb);
      tp += __popc(tb);
    }
  }
}

// ---------------------------------------------------------------- product
struct PanK {
  const i32* poff;
  const uint16_t* prow;
  const void* val;
  const float* r;
  i64 m, rows, npanels;
  const Item* items;
  const i32* pitem0;
  const i32* long_rows;
  const i32* plong0;
  const i32* long_piece0;
  float* partials;
  float* ypan;
  unsigned* err;
  unsigned wait_limit;  // poll budget of the copy waits
  int aligned;  // r is 16-byte aligned: the slice is staged with 16-byte loads
  // forward head: every CTA stages the same slice r[xmap[0..rows)] once
  // (the frequent columns of w), panels are stretches of A's rows
  const i32* xmap;
  i64 group;  // consecutive panels a CTA takes at a time
};


// Shared memory of one CTA: per warp one staging buffer for a work item's
// entries (panel rows as uint16, then the values; the item's products are
// later written over it) with its mbarrier and the tile's row offsets; then
// the panel's slice of r.
template <class VT> struct PanelSmem {
  static constexpr int kCap = kWarpTile + 16;  // entries of one copy: 16-byte aligned ends
  static constexpr int kIdxB = kCap * 2;
  static constexpr int kStageB = kIdxB + kCap * (int)sizeof(VT);  // >= kCap * 4: room for the products
  static constexpr int kSoffB = ((kTileRows + 1) * 2 + 15) / 16 * 16;
  static constexpr int kWarpB = kStageB + kSoffB;
  static constexpr int kStatic = 16 * kPanelWarps + kPanelWarps * kWarpB;  // mbarriers, then the warps' areas
};

// One CTA of kPanelWarps warps per SM takes units of `group` consecutive
// panels: b, b+G, ...  Per unit: the vector's slice into shared memory (row
// panels: r's rows of the panel; forward head: w at the head columns, staged
// once); then the warps walk the unit's work items (tiles of short rows,
// pieces of long ones; warp w takes items w, w+W, ...).  Per item a bulk copy
// stages the entries in the warp's buffer (the copies of the other 31 warps
// cover its latency); the products with the vector gathered from shared
// memory overwrite the staged entries, and each row is added by 1..32 lanes
// in a fixed order.  After a barrier the pieces of long rows are added in
// piece order.  (Measured on GB300 against a double-buffered variant with 16
// warps and a separate product buffer: this one is 10% faster on the 10M x 1M
// benchmark matrix.)
template <class VT>
__global__ void __launch_bounds__(kPanelWarps * 32, 1) k_panel(const PanK p) {
  using SM = PanelSmem<VT>;
  constexpr int NW = kPanelWarps;
  constexpr int NR2 = (kWarpTile + 16 + 63) / 64;  // pair rounds of a staged copy (<= 520 entries)
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + 2 * w;
  unsigned char* area = smem + 16 * NW + w * SM::kWarpB;
  unsigned short* soff = reinterpret_cast<unsigned short*>(area + SM::kStageB);
  float* prod = reinterpret_cast<float*>(area);
  float2* prod2 = reinterpret_cast<float2*>(area);
  float* xs = reinterpret_cast<float*>(smem + SM::kStatic);
  const VT* __restrict__ val = (const VT*)p.val;
  if (lane == 0) mbar_init(bar, 1);
  fence_mbar_init();
  __syncthreads();
  const uint64_t pol = policy_evict_first();
  unsigned parity = 0;
  bool pend = false, dead = false;
  const bool shared = p.xmap != nullptr;
  // a CTA takes `group` consecutive panels at a time (their items and long
  // rows are contiguous): one per step for row panels, a whole share of the
  // rows at once for the forward head (one barrier per CTA)
  const int nunits = (int)((p.npanels + p.group - 1) / p.group);
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
    const int pn = u * (int)p.group, pe = (int)min((i64)pn + p.group, p.npanels);
    const i64 base = shared ? 0 : (i64)pn * p.rows;
    const int nr = shared ? (int)p.rows : (int)min(p.rows, p.m - base);
    __syncthreads();
    if (shared) {
      if (u == blockIdx.x)
        for (int i = threadIdx.x; i < nr; i += NW * 32) xs[i] = __ldg(p.r + p.xmap[i]);
    } else {
      const int n4 = p.aligned ? nr >> 2 : 0;
      const float4* src = reinterpret_cast<const float4*>(p.r + base);
      float4* dst = reinterpret_cast<float4*>(xs);
      int i = threadIdx.x;
      for (; i + 3 * NW * 32 < n4; i += 4 * NW * 32) {
        const float4 a0 = src[i], a1 = src[i + NW * 32], a2 = src[i + 2 * NW * 32], a3 = src[i + 3 * NW * 32];
        dst[i] = a0;
        dst[i + NW * 32] = a1;
        dst[i + 2 * NW * 32] = a2;
        dst[i + 3 * NW * 32] = a3;
      }
      for (; i < n4; i += NW * 32) dst[i] = src[i];
      for (i = (n4 << 2) + threadIdx.x; i < nr; i += NW * 32) xs[i] = p.r[base + i];
    }
    __syncthreads();
    const int t1 = p.pitem0[pe];
    int t = p.pitem0[pn] + w;
    Item nx = (t < t1) ? p.items[t] : Item{0, 0, 0, 0};
    for (; t < t1 && !dead; t += NW) {
      const Item it = nx;
      if (t + NW < t1) nx = p.items[t + NW];
      const int q0 = it.e0 & ~7, q1 = (it.e1 + 7) & ~7;
      const unsigned n = (unsigned)(q1 - q0);
      if (lane == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, n * 2u + n * (unsigned)sizeof(VT));
        if (n > 0) {
          bulk_g2s(area, p.prow + q0, n * 2u, bar, pol);
          bulk_g2s(area + SM::kIdxB, val + q0, n * (unsigned)sizeof(VT), bar, pol);
        }
      }
      pend = true;
      if (it.r1 >= 0)
        for (int k = lane; k <= it.r1 - it.r0; k += 32) soff[k] = (unsigned short)(__ldg(p.poff + it.r0 + k) - q0);
      if (!mbar_wait_bounded(bar, parity, p.err, p.wait_limit)) {
        dead = true;
        break;
      }
      parity ^= 1u;
      pend = false;
      __syncwarp();
      {
        // every staged pair into registers first: the products overwrite them
        const unsigned* sidx2 = reinterpret_cast<const unsigned*>(area);
        const VT* sval = reinterpret_cast<const VT*>(area + SM::kIdxB);
        const int n2 = (int)(n >> 1);
        unsigned c[NR2];
        float v0[NR2], v1[NR2];
#pragma unroll
        for (int q = 0; q < NR2; q++) {
          const int k2 = q * 32 + lane;
          if (k2 < n2) {
            c[q] = sidx2[k2];
            v0[q] = (float)sval[2 * k2];
            v1[q] = (float)sval[2 * k2 + 1];
          }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < NR2; q++) {
          const int k2 = q * 32 + lane;
          if (k2 < n2) prod2[k2] = make_float2(v0[q] * xs[c[q] & 0xffffu], v1[q] * xs[c[q] >> 16]);
        }
      }
      __syncwarp();
      if (it.r1 >= 0) {
        const int R = it.r1 - it.r0;
        const int Gl = lanes_per_row(R);
        const int per_round = 32 / Gl;
        for (int rb = 0; rb < R; rb += per_round) {
          const int j = rb + lane / Gl, sub = lane % Gl;
          float acc = 0.f;
          if (j < R) {
            const int s = soff[j], e = soff[j + 1];
            float a1 = 0.f, a2 = 0.f, a3 = 0.f;
            int k = s + sub;
            for (; k + 3 * Gl < e; k += 4 * Gl) {
              acc += prod[k];
              a1 += prod[k + Gl];
              a2 += prod[k + 2 * Gl];
              a3 += prod[k + 3 * Gl];
            }
            for (; k < e; k += Gl) acc += prod[k];
            acc = (acc + a1) + (a2 + a3);
          }
          for (int o = Gl >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (j < R && sub == 0) p.ypan[it.r0 + j] = acc;
        }
      } else {
        float acc = 0.f;
        const int e = it.e1 - q0;
        for (int k = it.e0 - q0 + lane; k < e; k += 32) acc += prod[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) p.partials[-1 - it.r1] = acc;
      }
      __syncwarp();
    }
    __syncthreads();
    const int l1 = p.plong0[pe];
    for (int L = p.plong0[pn] + w; L < l1; L += NW) {
      const int c0 = p.long_piece0[L], c1 = p.long_piece0[L + 1];
      float acc = 0.f;
      for (int j = c0 + lane; j < c1; j += 32) acc += __ldcg(p.partials + j);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) p.ypan[p.long_rows[L]] = acc;
    }
  }
  // a warp that gave up still drains its copy in flight (default budget)
  // before the CTA's shared memory is released
  if (pend) mbar_wait_bounded(bar, parity, nullptr, kCopyPolls);
}

// g[hot[h]] = sum over panels of ypan[panel*nhot + h] in a fixed order:
// 32 columns per CTA of 1024 threads; warp w adds panels w, w+32, ... in two
// compensated FP32 sums (GB300's FP64 unit is too narrow for one FP64 add per
// partial), then warp 0 adds the 32 warp sums in FP64, in order.
template <class YT>
__global__ void __launch_bounds__(1024) k_panel_colsum(const float* __restrict__ ypan, const i32* __restrict__ hot,
                                                       i64 nhot, i64 np, YT* __restrict__ y) {
  __shared__ double part[32][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (i64 h0 = (i64)blockIdx.x * 32; h0 < nhot; h0 += (i64)gridDim.x * 32) {
    const i64 h = h0 + lane;
    FSum a, b;
    if (h < nhot) {
      i64 pn = w;
      for (; pn + 32 < np; pn += 64) {
        a.add(__ldcs(ypan + pn * nhot + h));
        b.add(__ldcs(ypan + (pn + 32) * nhot + h));
      }
      if (pn < np) a.add(__ldcs(ypan + pn * nhot + h));
    }
    part[w][lane] = a.total() + b.total();
    __syncthreads();
    if (w == 0 && h < nhot) {
      double s = 0.0;
#pragma unroll 8
      for (int q = 0; q < 32; q++) s += part[q][lane];
      y[hot[h]] = (YT)s;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------ split storage
// The row-panel / forward-head kernel for split values (FP32 value + BF16
// residual per entry, df64 products: df64.cuh).  Same layout as k_panel; the
// staged entry is 8 bytes (uint16 slot, FP32 value, BF16 residual) and the
// vector slice keeps both FP32 words of each df pair (8 bytes a row: rounding
// the slice's low word would add noise that changes from one evaluation to
// the next and, unlike the fixed rounding of the values, does not cancel in
// the L-BFGS gradient differences).  To fit a panel beside the staging
// buffers, one CTA of kSplitWarps warps per SM walks its own work items of at
// most kSplitTile entries, so that one item is one pass of 32 lanes x
// kSplitChunk entries: no products are staged and no second pass re-reads
// them.
#ifndef FVG_SPLIT_WARPS
#define FVG_SPLIT_WARPS 28
#endif
constexpr int kSplitWarps = FVG_SPLIT_WARPS;  // one CTA per SM (its shared slice fills the SM)
constexpr int kSplitTile = 480;  // an item's staged copy (8-aligned ends) fits 32 lanes x 16 entries
constexpr int kSplitChunk = 16;  // entries per lane
struct SplitSmem {
  static constexpr int kCap = 32 * kSplitChunk;        // entries of one copy
  static constexpr int kHiB = kCap * 2;                // offset of the FP32 values
  static constexpr int kLoB = kHiB + kCap * 4;         // offset of the BF16 residuals
  static constexpr int kStageB = kLoB + kCap * 2;      // = kCap * 8
  static constexpr int kSoffB = ((kTileRows + 1) * 2 + 15) / 16 * 16;
  static constexpr int kWarpB = kStageB + kSoffB;
  static constexpr int kStatic = 16 * kSplitWarps + kSplitWarps * kWarpB;
};

struct PanSK {
  const i32* poff;
  const uint16_t* prow;
  const float* vh;
  const unsigned short* vl;
  const float2* x;  // df pairs: r (row panels) or w (forward head)
  i64 m, rows, npanels;
  const Item* items;
  const i32* pitem0;
  const i32* long_rows;
  const i32* plong0;
  const i32* long_piece0;
  float2* partials;
  float2* ypan;
  unsigned* err;
  unsigned wait_limit;
  const i32* xmap;  // forward head: the slice is x[xmap[0..rows)], staged once
  i64 group;
};

__device__ __forceinline__ df shfl_xor_df(df a, int o) {
  return {__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}
__device__ __forceinline__ df shfl_up_df(df a, int o) {
  return {__shfl_up_sync(0xffffffffu, a.h, o), __shfl_up_sync(0xffffffffu, a.l, o)};
}

// Segmented inclusive scan over the warp's lanes, in lane order:
// S_L = v_L + (reset_L ? 0 : S_{L-1}) (Hillis-Steele; a lane stops adding
// once a reset lies between it and the lane it reads).
__device__ __forceinline__ df seg_scan_df(df v, bool reset, int lane) {
  bool f = reset;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const df u = shfl_up_df(v, o);
    const bool fu = __shfl_up_sync(0xffffffffu, (int)f, o) != 0;
    if (lane >= o) {
      if (!f) v = df_add(u, v);
      f = f || fu;
    }
  }
  return v;
}

// One CTA of kSplitWarps warps per SM takes units of `group` consecutive
// panels (as k_panel).  Per work item (at most kSplitTile entries) a bulk
// copy stages the entries (uint16 slots, FP32 values, BF16 residuals); lane L
// then takes the kSplitChunk staged entries from kSplitChunk*L on (16-byte
// shared loads), makes each
// product exact (p + t), and adds its row segments in registers with TwoSum:
// a row that ends inside the chunk is written at once when it also started
// there; the row that was open at the chunk's start and the one open at its
// end join the neighbouring lanes' segments through a segmented scan in lane
// order.  Pieces of long rows: a warp reduction, added after the CTA barrier
// in piece order.  Every sum has a fixed order.
// MID (the row panels, whose rows are often shorter than a lane's chunk): the
// rows that start and end inside one lane's chunk are summed in the chunk's
// single pass, parked in the warp's staging area (free once the entries are
// in registers) and written after it; without MID (the forward head, rows
// longer than a chunk) each such row is re-summed over the chunk.
template <bool MID>
__global__ void __launch_bounds__(kSplitWarps * 32, 1) k_panel_split(const PanSK p) {
  using SM = SplitSmem;
  constexpr int NW = kSplitWarps;
  constexpr int CH = kSplitChunk;
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem) + 2 * w;
  unsigned char* area = smem + 16 * NW + w * SM::kWarpB;
  unsigned short* soff = reinterpret_cast<unsigned short*>(area + SM::kStageB);
  float2* xs = reinterpret_cast<float2*>(smem + SM::kStatic);  // df pairs: one 8-byte load a gather
  if (lane == 0) mbar_init(bar, 1);
  fence_mbar_init();
  __syncthreads();
  const uint64_t pol = policy_evict_first();
  unsigned parity = 0;
  bool pend = false, dead = false;
  const bool shared = p.xmap != nullptr;
  const int nunits = (int)((p.npanels + p.group - 1) / p.group);
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
    const int pn = u * (int)p.group, pe = (int)min((i64)pn + p.group, p.npanels);
    const i64 base = shared ? 0 : (i64)pn * p.rows;
    const int nr = shared ? (int)p.rows : (int)min(p.rows, p.m - base);
    __syncthreads();
    if (!shared || u == blockIdx.x)
      for (int i = threadIdx.x; i < nr; i += NW * 32) {
        const float2 v = __ldg(p.x + (shared ? (i64)p.xmap[i] : base + i));
        xs[i] = v;
      }
    __syncthreads();
    const int t1 = p.pitem0[pe];
    int t = p.pitem0[pn] + w;
    Item nx = (t < t1) ? p.items[t] : Item{0, 0, 0, 0};
    for (; t < t1 && !dead; t += NW) {
      const Item it = nx;
      if (t + NW < t1) nx = p.items[t + NW];
      const int q0 = it.e0 & ~7, q1 = (it.e1 + 7) & ~7;
      const unsigned n = (unsigned)(q1 - q0);
      if (lane == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, n * 8u);
        if (n > 0) {
          bulk_g2s(area, p.prow + q0, n * 2u, bar, pol);
          bulk_g2s(area + SM::kHiB, p.vh + q0, n * 4u, bar, pol);
          bulk_g2s(area + SM::kLoB, p.vl + q0, n * 2u, bar, pol);
        }
      }
      pend = true;
      const bool tile = it.r1 >= 0;
      const int R = tile ? it.r1 - it.r0 : 0;
      if (tile)
        for (int k = lane; k <= R; k += 32) soff[k] = (unsigned short)(__ldg(p.poff + it.r0 + k) - q0);
      if (!mbar_wait_bounded(bar, parity, p.err, p.wait_limit)) {
        dead = true;
        break;
      }
      parity ^= 1u;
      pend = false;
      __syncwarp();
      // The copy's padding entries (before e0, and from e1 to the end of the
      // lane chunk holding it: at most 7 and 15) become slot 0, value 0, so
      // that their products are exact zeros and no entry needs a range test.
      {
        const int lead = it.e0 - q0, tz = it.e1 - q0;
        const int tend = min((tz + CH - 1) / CH * CH, SM::kCap);
        unsigned short* ss = reinterpret_cast<unsigned short*>(area);
        float* sh = reinterpret_cast<float*>(area + SM::kHiB);
        unsigned short* sl = reinterpret_cast<unsigned short*>(area + SM::kLoB);
        if (lane < lead) {
          ss[lane] = 0;
          sh[lane] = 0.f;
          sl[lane] = 0;
        }
        if (lane < tend - tz) {
          ss[tz + lane] = 0;
          sh[tz + lane] = 0.f;
          sl[tz + lane] = 0;
        }
        __syncwarp();
      }
      // this lane's CH staged entries (16-byte shared loads)
      unsigned sw[CH / 2], lw[CH / 2];
      float hv[CH];
#pragma unroll
      for (int q = 0; q < CH / 8; q++) {
        const uint4 s4 = reinterpret_cast<const uint4*>(area)[lane * (CH / 8) + q];
        const uint4 l4 = reinterpret_cast<const uint4*>(area + SM::kLoB)[lane * (CH / 8) + q];
        sw[4 * q] = s4.x; sw[4 * q + 1] = s4.y; sw[4 * q + 2] = s4.z; sw[4 * q + 3] = s4.w;
        lw[4 * q] = l4.x; lw[4 * q + 1] = l4.y; lw[4 * q + 2] = l4.z; lw[4 * q + 3] = l4.w;
      }
#pragma unroll
      for (int q = 0; q < CH / 4; q++) {
        const float4 h = reinterpret_cast<const float4*>(area + SM::kHiB)[lane * (CH / 4) + q];
        hv[4 * q] = h.x; hv[4 * q + 1] = h.y; hv[4 * q + 2] = h.z; hv[4 * q + 3] = h.w;
      }
      const int lo_e = max(it.e0 - q0, lane * CH), hi_e = min(it.e1 - q0, lane * CH + CH);
      const bool any = lo_e < hi_e;
      // a lane past the item's end reads stale (or never written) slots: slot 0
#pragma unroll
      for (int q = 0; q < CH / 2; q++) sw[q] = any ? sw[q] : 0u;
      if (!tile) {
        DfAcc acc;
#pragma unroll
        for (int k = 0; k < CH; k++) {
          const unsigned c = (sw[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
          const float vl = __uint_as_float((k & 1) ? (lw[k >> 1] & 0xffff0000u) : (lw[k >> 1] << 16));
          float pp, tt;
          df_prod(hv[k], vl, xs[c], pp, tt);
          acc.add(pp, tt);
        }
        if (!any) acc = DfAcc{};
        df a = acc.get();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = df_add(a, shfl_xor_df(a, o));
        if (lane == 0) p.partials[-1 - it.r1] = df_pack(a);
      } else {
        __syncwarp();  // soff
        for (int j = lane; j < R; j += 32)
          if (soff[j] == soff[j + 1]) p.ypan[it.r0 + j] = make_float2(0.f, 0.f);  // empty rows
        // the lane's CH products (padding entries give exact zeros; a lane
        // past the item's end has any == false and its sums are dropped)
        float pp[CH], tt[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) {
          const unsigned c = (sw[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
          const float vl = __uint_as_float((k & 1) ? (lw[k >> 1] & 0xffff0000u) : (lw[k >> 1] << 16));
          df_prod(hv[k], vl, xs[c], pp[k], tt[k]);
        }
        // rows: j0 holds the first valid entry; B marks the rows starting after it
        unsigned B = 0;
        int j = 0, j0 = 0, nb = 0;
        bool starts = false;
        if (any) {
          int a = 0, b = R;  // the last row starting at or before lo_e (the non-empty one holding it)
          while (b - a > 1) {
            const int mid = (a + b) >> 1;
            if ((int)soff[mid] <= lo_e) a = mid;
            else b = mid;
          }
          j = j0 = a;
          starts = (int)soff[j] == lo_e;
          nb = soff[j + 1];
          while (nb < hi_e) {
            B |= 1u << (nb - lane * CH);
            do {
              j++;
              nb = soff[j + 1];
            } while (nb == (int)soff[j]);
          }
        }
        df H, T;
        float2* mid = reinterpret_cast<float2*>(area);  // kCap pairs: the staging area's 8 bytes an entry
        if constexpr (MID) {
          chunk_segments_mid<CH>(pp, tt, B, H, T, mid, lane * CH);
        } else {
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
              p.ypan[it.r0 + jj] = df_pack(chunk_range<CH>(pp, tt, a, b));
              a = b;
              do {
                jj++;
              } while (soff[jj + 1] == soff[jj]);
            }
          }
        }
        // the tail segment starts inside this lane when a row starts here
        const df S = seg_scan_df(any ? T : df{0.f, 0.f}, any && (B != 0 || starts), lane);
        df carry = shfl_up_df(S, 1);
        if (lane == 0) carry = {0.f, 0.f};
        if (B) p.ypan[it.r0 + j0] = df_pack(starts ? H : df_add(carry, H));
        if (any && nb == hi_e) p.ypan[it.r0 + j] = df_pack(S);  // the tail row ends with this lane's range
        if constexpr (MID) {
          // the middle rows: non-empty rows whose start and end are both marks
          // of one lane (start after the lane's first entry, end before its
          // range ends)
          __syncwarp();
          const int ie0 = it.e0 - q0, ie1 = it.e1 - q0;
          for (int jr = lane; jr < R; jr += 32) {
            const int s0 = soff[jr], s1 = soff[jr + 1];
            if (s1 == s0) continue;
            const int L = s0 / CH;
            if (s0 > max(ie0, L * CH) && s1 < min(ie1, L * CH + CH)) {
              const float2 v = mid[s0];
              p.ypan[it.r0 + jr] = df_pack(fast_two_sum(v.x, v.y));
            }
          }
        }
      }
      fence_proxy_async();  // the padding stores, before the next copy into the area
      __syncwarp();
    }
    __syncthreads();
    const int l1 = p.plong0[pe];
    for (int L = p.plong0[pn] + w; L < l1; L += NW) {
      const int c0 = p.long_piece0[L], c1 = p.long_piece0[L + 1];
      df a = {0.f, 0.f};
      for (int jj = c0 + lane; jj < c1; jj += 32) a = df_add(a, df_unpack(__ldcg(p.partials + jj)));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a = df_add(a, shfl_xor_df(a, o));
      if (lane == 0) p.ypan[p.long_rows[L]] = df_pack(a);
    }
  }
  // a warp that gave up still drains its copy in flight (default budget)
  if (pend) mbar_wait_bounded(bar, parity, nullptr, kCopyPolls);
}

// g[hot[h]] = sum over panels of the df partials ypan[panel*nhot + h]:
// 32 columns per CTA of 1024 threads, warp w adds panels w, w+32, ...; warp
// 0 adds the 32 warp sums in order; FP64 result.
__global__ void __launch_bounds__(1024) k_panel_colsum_split(const float2* __restrict__ ypan,
                                                             const i32* __restrict__ hot, i64 nhot, i64 np,
                                                             double* __restrict__ y) {
  __shared__ float2 part[32][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (i64 h0 = (i64)blockIdx.x * 32; h0 < nhot; h0 += (i64)gridDim.x * 32) {
    const i64 h = h0 + lane;
    df a = {0.f, 0.f};
    if (h < nhot)
      for (i64 pn = w; pn < np; pn += 32) a = df_add(a, df_unpack(__ldcs(ypan + pn * nhot + h)));
    part[w][lane] = df_pack(a);
    __syncthreads();
    if (w == 0 && h < nhot) {
      df s = {0.f, 0.f};
#pragma unroll 8
      for (int q = 0; q < 32; q++) s = df_add(s, df_unpack(part[q][lane]));
      y[hot[h]] = df_to_double(s);
    }
    __syncthreads();
  }
}

int panel_split_smem_bytes(i64 rows) { return SplitSmem::kStatic + (int)(rows * 8); }

template <class VT> int panel_smem_bytes(i64 rows) { return PanelSmem<VT>::kStatic + (int)(rows * 4); }

// Tallest panel (or head) one CTA can stage beside the staging buffers, for
// the FP32 / BF16 kernel and the split kernel alike.
i64 panel_rows_cap(fvg_ctx* c) {
  int per_sm = 0, reserved = 0, optin = 0;
  FVG_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device));
  FVG_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, c->device));
  FVG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
  const i64 per_cta = std::min<i64>((i64)per_sm - (i64)reserved, (i64)optin);
  // the FP32 kernel stages 4 bytes a row, the split kernel 8 (beside
  // smaller staging buffers): a layout serves both
  i64 cap = std::min<i64>((per_cta - PanelSmem<float>::kStatic) / 4, (per_cta - SplitSmem::kStatic) / 8);
  cap = std::min<i64>(cap, 65536);  // panel-local rows are uint16
  return cap & ~3ll;
}

void alloc_padded(fvg_ctx* c, DBuf& b, i64 n, int elem) {
  b.alloc((size_t)(n + kPad) * elem, c->stream);
  FVG_CUDA(cudaMemsetAsync((char*)b.p + (size_t)n * elem, 0, (size_t)kPad * elem, c->stream));
}

// Allocates, for n entries, the planes of `dst` / `dlo` that the source holds
// besides its master plane and returns the copy pointers.
SidePlanes side_planes(fvg_ctx* c, const DBuf* src, const DBuf& slo, int master, DBuf* dst, DBuf& dlo, i64 n) {
  SidePlanes sp;
  if (master != FVG_F32 && src[FVG_F32].p) {
    alloc_padded(c, dst[FVG_F32], n, 4);
    sp.s32 = src[FVG_F32].as<float>();
    sp.d32 = dst[FVG_F32].as<float>();
  }
  if (master != FVG_BF16 && src[FVG_BF16].p) {
    alloc_padded(c, dst[FVG_BF16], n, 2);
    sp.s16 = src[FVG_BF16].as<bf16>();
    sp.d16 = dst[FVG_BF16].as<bf16>();
  }
  if (slo.p) {
    alloc_padded(c, dlo, n, 2);
    sp.slo = slo.as<bf16>();
    sp.dlo = dlo.as<bf16>();
  }
  return sp;
}

template <class T>
void fill_planes(fvg_ctx* c, const DevCRS& at, DevPanels& pn, const i32* B, const i64* poff64, const i64* flag,
                 const i64* coff) {
  const T* tv = at.val[pn.master].as<T>();
  const SidePlanes spp = side_planes(c, at.val, at.lo, pn.master, pn.val, pn.lo, pn.E);
  const SidePlanes spc = side_planes(c, at.val, at.lo, pn.master, pn.cold.val, pn.cold.lo, pn.cold.nnz);
  k_panel_fill<T><<<grid_n(32 * pn.npanels * pn.nhot), 256, 0, c->stream>>>(
      B, poff64, at.idx.as<i32>(), tv, pn.nhot, pn.npanels, pn.rows, pn.prow.as<uint16_t>(), pn.val[pn.master].as<T>(),
      spp);
  check_launch("panel_fill");
  k_cold_fill<T><<<grid_n(32 * pn.n), 256, 0, c->stream>>>(at.off.as<i32>(), flag, coff, pn.n, at.idx.as<i32>(), tv,
                                                           pn.cold.idx.as<i32>(), pn.cold.val[pn.master].as<T>(), spc);
  check_launch("cold_fill");
  count_launch(c, 2);
}

}  // namespace

// Work items of a CRS cut into chunks of `chunk` rows (a chunk's items, long
// rows and pieces are contiguous, numbered globally), packed on the device:
// counts, their exclusive scans (a few thousand numbers, on the host), then
// the items.
void device_pack(fvg_ctx* c, const i32* off, i64 nrows, i64 chunk, i64 nchunks, int tile, PackOut& o, i64 sub) {
  const i64 np = std::max<i64>(nchunks, 1) * sub;
  DBuf cnt, basev;
  cnt.alloc(sizeof(i32) * 3 * np, c->stream);
  // a thread per chunk
  const unsigned pg = (unsigned)std::min<i64>((np + 255) / 256, 1 << 20);
  k_panel_pack<<<pg, 256, 0, c->stream>>>(off, nrows, chunk, sub, np, tile, 0, cnt.as<i32>(), nullptr, nullptr,
                                          nullptr, nullptr, nullptr);
  check_launch("pack");
  count_launch(c);
  std::vector<i32> hc((size_t)(3 * np));
  o.base.assign((size_t)(3 * (np + 1)), 0);
  FVG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(i32) * 3 * np, cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  i64 tot[3] = {0, 0, 0};
  for (int kind = 0; kind < 3; kind++) {
    for (i64 p = 0; p < np; p++) {
      o.base[(size_t)(kind * (np + 1) + p)] = (i32)tot[kind];
      tot[kind] += hc[(size_t)(kind * np + p)];
    }
    o.base[(size_t)(kind * (np + 1) + np)] = (i32)tot[kind];
  }
  if (tot[0] >= (1ll << 31) - 1 || tot[2] >= (1ll << 31) - 1) fail(FVG_ERR_INTERNAL, "work schedule too large");
  o.nitems = tot[0];
  o.nlong = tot[1];
  o.npieces = tot[2];
  basev.alloc(sizeof(i32) * 3 * (np + 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(basev.p, o.base.data(), sizeof(i32) * 3 * (np + 1), cudaMemcpyHostToDevice, c->stream));
  o.items.alloc(sizeof(Item) * std::max<i64>(o.nitems, 1), c->stream);
  o.long_rows.alloc(sizeof(i32) * std::max<i64>(o.nlong, 1), c->stream);
  o.long_piece0.alloc(sizeof(i32) * (o.nlong + 1), c->stream);
  DBuf lfirst;
  lfirst.alloc(sizeof(i32) * std::max<i64>(o.nlong, 1), c->stream);
  k_panel_pack<<<pg, 256, 0, c->stream>>>(off, nrows, chunk, sub, np, tile, 1, nullptr, basev.as<i32>(),
                                          o.items.as<Item>(), o.long_rows.as<i32>(), o.long_piece0.as<i32>(),
                                          lfirst.as<i32>());
  check_launch("pack");
  count_launch(c);
  if (o.nlong > 0) {
    const unsigned lg = (unsigned)std::min<i64>((o.nlong + 7) / 8, 1 << 20);
    k_long_pieces<<<lg, 256, 0, c->stream>>>(off, o.long_rows.as<i32>(), o.long_piece0.as<i32>(), lfirst.as<i32>(),
                                             o.nlong, tile, o.items.as<Item>());
    check_launch("long_pieces");
    count_launch(c);
  }
  const i32 npc = (i32)o.npieces;
  FVG_CUDA(cudaMemcpyAsync(o.long_piece0.as<i32>() + o.nlong, &npc, sizeof(i32), cudaMemcpyHostToDevice, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host values go out of scope
}

namespace {

// The split kernel's work items: the same packing with kSplitTile-entry items
void pack_split_items(fvg_ctx* c, DevPanels& pn) {
  const i64 nhot = pn.nhot, np = pn.npanels;
  PackOut o;
  const i64 sub = std::max<i64>(1, (nhot + kPanelPackRows - 1) / kPanelPackRows);
  device_pack(c, pn.poff.as<i32>(), np * nhot, nhot, np, kSplitTile, o, sub);
  auto it = std::make_unique<PanelItems>();
  it->tile = kSplitTile;
  it->nitems = o.nitems;
  it->nlong = o.nlong;
  it->npieces = o.npieces;
  it->items = std::move(o.items);
  it->long_rows = std::move(o.long_rows);
  it->long_piece0 = std::move(o.long_piece0);
  const i64 nc = np * sub;
  std::vector<i32> pi((size_t)np + 1), pl((size_t)np + 1);
  for (i64 q = 0; q <= np; q++) {
    pi[(size_t)q] = o.base[(size_t)(q * sub)];
    pl[(size_t)q] = o.base[(size_t)((nc + 1) + q * sub)];
  }
  it->pitem0.alloc(sizeof(i32) * (np + 1), c->stream);
  it->plong0.alloc(sizeof(i32) * (np + 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(it->pitem0.p, pi.data(), sizeof(i32) * (np + 1), cudaMemcpyHostToDevice, c->stream));
  FVG_CUDA(cudaMemcpyAsync(it->plong0.p, pl.data(), sizeof(i32) * (np + 1), cudaMemcpyHostToDevice, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host arrays go out of scope
  pn.split_items = std::move(it);
}

void pack_panels(fvg_ctx* c, DevPanels& pn, i64 nhot, i64 np) {
  PackOut o;
  // each panel's rows in pieces of ~kPanelPackRows rows, a packing thread each
  const i64 sub = std::max<i64>(1, (nhot + kPanelPackRows - 1) / kPanelPackRows);
  device_pack(c, pn.poff.as<i32>(), np * nhot, nhot, np, kWarpTile, o, sub);
  pn.nitems = o.nitems;
  pn.nlong = o.nlong;
  pn.npieces = o.npieces;
  pn.items = std::move(o.items);
  pn.long_rows = std::move(o.long_rows);
  pn.long_piece0 = std::move(o.long_piece0);
  // a panel's items and long rows: from its first piece's on
  const i64 nc = np * sub;
  std::vector<i32> pi((size_t)np + 1), pl((size_t)np + 1);
  for (i64 q = 0; q <= np; q++) {
    pi[(size_t)q] = o.base[(size_t)(q * sub)];
    pl[(size_t)q] = o.base[(size_t)((nc + 1) + q * sub)];
  }
  pn.pitem0.alloc(sizeof(i32) * (np + 1), c->stream);
  pn.plong0.alloc(sizeof(i32) * (np + 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(pn.pitem0.p, pi.data(), sizeof(i32) * (np + 1), cudaMemcpyHostToDevice, c->stream));
  FVG_CUDA(cudaMemcpyAsync(pn.plong0.p, pl.data(), sizeof(i32) * (np + 1), cudaMemcpyHostToDevice, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host arrays go out of scope
}

// Builds the layout from the transposed CRS; null when it would not pay
// (too few panels or too little of the matrix in hot columns) or does not fit
// its index types.
std::unique_ptr<DevPanels> panel_build(fvg_ctx* c, const DevCRS& at, int master, i64 force_rows, double min_pp) {
  ProfScope ps(c, P_PANEL_BUILD);
  const i64 m = at.n, n = at.m, nnz = at.nnz;
  const bool forced = force_rows > 0;
  if (m <= 0 || n <= 0 || nnz <= 0) return nullptr;
  const i64 cap = panel_rows_cap(c);
  i64 rows;
  if (forced) {
    if (force_rows % 4 != 0 || force_rows > cap)
      fail(FVG_ERR_INVALID_ARG, "panel rows must be a multiple of 4 and at most " + std::to_string(cap));
    rows = force_rows;
  } else {
    const i64 target = std::min<i64>(kPanelRowsAuto, cap);
    const i64 grid = c->num_sms;  // one CTA per SM
    const i64 np0 = (m + target - 1) / target;
    if (np0 < 8) return nullptr;  // too few panels to pay for the split
    if (np0 >= grid) {
      // the fewest whole rounds over the persistent grid whose panels fit in
      // shared memory (the tallest panels: the most columns count as hot)
      const i64 rounds = (m + cap * grid - 1) / (cap * grid);
      rows = ((m + rounds * grid - 1) / (rounds * grid) + 3) & ~3ll;
    } else {
      rows = target;
    }
  }
  const double mpp = min_pp > 0 ? min_pp : kPanelMinAuto;
  auto pn = std::make_unique<DevPanels>();
  pn->m = m;
  pn->n = n;
  pn->rows = rows;
  pn->npanels = (m + rows - 1) / rows;
  pn->min_per_panel = mpp;
  pn->master = master;
  const i64 np = pn->npanels;
  const i64 thresh = std::max<i64>(1, (i64)std::ceil(mpp * (double)np));
  // hot columns
  DBuf flag, pos;
  flag.alloc(sizeof(i64) * n, c->stream);
  pos.alloc(sizeof(i64) * (n + 1), c->stream);
  k_hot_flags<<<grid_n(n), 256, 0, c->stream>>>(at.off.as<i32>(), n, thresh, flag.as<i64>());
  check_launch("hot_flags");
  count_launch(c);
  scan_i64(c, flag.as<i64>(), pos.as<i64>(), n);
  i64 nhot = 0;
  FVG_CUDA(cudaMemcpyAsync(&nhot, pos.as<i64>() + n, sizeof(i64), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  if (nhot == 0 || np * nhot >= (1ll << 31) - 1) return nullptr;
  pn->nhot = nhot;
  pn->hot_cols.alloc(sizeof(i32) * nhot, c->stream);
  k_hot_list<<<grid_n(n), 256, 0, c->stream>>>(flag.as<i64>(), pos.as<i64>(), n, pn->hot_cols.as<i32>());
  check_launch("hot_list");
  count_launch(c);
  // per (panel, hot column) ranges and their offsets
  DBuf B, len, poff64;
  B.alloc(sizeof(i32) * nhot * (np + 1), c->stream);
  k_panel_bounds<<<grid_n(nhot * (np + 1)), 256, 0, c->stream>>>(at.off.as<i32>(), at.idx.as<i32>(),
                                                                  pn->hot_cols.as<i32>(), nhot, np, rows, B.as<i32>());
  check_launch("panel_bounds");
  const i64 Q = np * nhot;
  len.alloc(sizeof(i64) * Q, c->stream);
  poff64.alloc(sizeof(i64) * (Q + 1), c->stream);
  k_panel_lens<<<grid_n(Q), 256, 0, c->stream>>>(B.as<i32>(), nhot, np, len.as<i64>());
  check_launch("panel_lens");
  count_launch(c, 2);
  scan_i64(c, len.as<i64>(), poff64.as<i64>(), Q);
  i64 E = 0;
  FVG_CUDA(cudaMemcpyAsync(&E, poff64.as<i64>() + Q, sizeof(i64), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  if (!forced && (double)E < 0.25 * (double)nnz) return nullptr;  // mostly cold: the plain path
  pn->E = E;
  pn->poff.alloc(sizeof(i32) * (Q + 1), c->stream);
  k_i64_to_i32<<<grid_n(Q + 1), 256, 0, c->stream>>>(poff64.as<i64>(), pn->poff.as<i32>(), Q + 1);
  check_launch("poff");
  count_launch(c);
  alloc_padded(c, pn->prow, E, 2);
  alloc_padded(c, pn->val[master], E, dtype_size(master));
  // cold columns: A^T with the hot rows emptied
  DevCRS& cold = pn->cold;
  cold.m = n;
  cold.n = m;
  DBuf clen, coff64;
  clen.alloc(sizeof(i64) * n, c->stream);
  coff64.alloc(sizeof(i64) * (n + 1), c->stream);
  k_cold_lens<<<grid_n(n), 256, 0, c->stream>>>(at.off.as<i32>(), flag.as<i64>(), n, clen.as<i64>());
  check_launch("cold_lens");
  count_launch(c);
  scan_i64(c, clen.as<i64>(), coff64.as<i64>(), n);
  FVG_CUDA(cudaMemcpyAsync(&cold.nnz, coff64.as<i64>() + n, sizeof(i64), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  cold.off.alloc(sizeof(i32) * (n + 1), c->stream);
  k_i64_to_i32<<<grid_n(n + 1), 256, 0, c->stream>>>(coff64.as<i64>(), cold.off.as<i32>(), n + 1);
  check_launch("cold_off");
  count_launch(c);
  alloc_padded(c, cold.idx, cold.nnz, 4);
  alloc_padded(c, cold.val[master], cold.nnz, dtype_size(master));
  if (master == FVG_F64) fill_planes<double>(c, at, *pn, B.as<i32>(), poff64.as<i64>(), flag.as<i64>(), coff64.as<i64>());
  else if (master == FVG_F32) fill_planes<float>(c, at, *pn, B.as<i32>(), poff64.as<i64>(), flag.as<i64>(), coff64.as<i64>());
  else fill_planes<bf16>(c, at, *pn, B.as<i32>(), poff64.as<i64>(), flag.as<i64>(), coff64.as<i64>());
  cold.max_row = 0;  // not used by the product
  pack_panels(c, *pn, nhot, np);
  const i64 pieces = pn->npieces;
  crs_sched(c, pn->cold, kWarpTile);  // the cold product's work items
  pn->ypan.alloc(sizeof(float) * Q, c->stream);
  pn->partials.alloc(sizeof(float) * std::max<i64>(pieces, 1), c->stream);
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
  return pn;
}

template <class VT>
void launch_panel(fvg_ctx* c, const PanK& k, i64 rows) {
  constexpr int threads = kPanelWarps * 32;
  auto kfn = k_panel<VT>;
  // the attribute once per device, at the device's limit (row panels and
  // the forward head ask for different sizes call after call); resident
  // CTAs per SM for the (device, size) pairs seen so far
  static std::mutex mu;  // contexts of different host threads launch concurrently
  static std::vector<int> attr_set;
  static std::vector<std::pair<long long, int>> blocks_for;
  const int smem = panel_smem_bytes<VT>(rows);
  std::unique_lock<std::mutex> lock(mu);
  if (std::find(attr_set.begin(), attr_set.end(), c->device) == attr_set.end()) {
    int optin = 0;
    FVG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    FVG_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    attr_set.push_back(c->device);
  }
  const long long key = ((long long)c->device << 32) | (unsigned)smem;
  int blocks = 0;
  for (auto& e : blocks_for)
    if (e.first == key) blocks = e.second;
  if (!blocks) {
    int nb = 0;
    FVG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kfn, threads, smem));
    blocks = std::max(1, nb);
    blocks_for.push_back({key, blocks});
  }
  lock.unlock();
  const i64 nunits = (k.npanels + k.group - 1) / k.group;
  const int grid = (int)std::max<i64>(1, std::min<i64>(nunits, (i64)blocks * c->num_sms));
  kfn<<<grid, threads, smem, c->stream>>>(k);
  check_launch("k_panel");
  count_launch(c);
}


// The forward head of A: the H most frequent columns (ties: lower column
// first), H at most what one CTA stages beside the staging buffers.  Null
// when it would not pay (small matrices, or the head holding less than half
// of the entries) unless forced (force_cols > 0).
std::unique_ptr<DevPanels> head_build(fvg_ctx* c, const DevCRS& a, const DevCRS& at, int master, i64 force_cols) {
  ProfScope ps(c, P_HEAD_BUILD);
  const i64 m = a.m, n = a.n, nnz = a.nnz;
  const bool forced = force_cols > 0;
  if (m <= 0 || n <= 0 || nnz <= 0) return nullptr;
  const i64 cap = panel_rows_cap(c);
  if (forced && force_cols > cap)
    fail(FVG_ERR_INVALID_ARG, "head columns must be at most " + std::to_string(cap));
  const i64 grid = c->num_sms;  // one CTA (one stretch of rows) per SM
  if (!forced && m < 64 * grid * kPanelWarps) return nullptr;
  const i64 H = std::min<i64>(n, forced ? force_cols : cap);
  // the H largest column counts (from the transposed offsets), on the
  // device: a stable sort of the columns by decreasing count (ties keep
  // column order), the first H take slots 0..H-1
  DBuf keys, cols, dslot;
  keys.alloc(sizeof(uint32_t) * n, c->stream);
  cols.alloc(sizeof(uint32_t) * n, c->stream);
  dslot.alloc(sizeof(i32) * n, c->stream);
  k_head_keys<<<grid_n(n), 256, 0, c->stream>>>(at.off.as<i32>(), n, keys.as<uint32_t>(), cols.as<uint32_t>());
  check_launch("head_keys");
  count_launch(c);
  radix_sort_pairs(c, keys.as<uint32_t>(), cols.as<uint32_t>(), n, 31);
  fill_i32(c, dslot.as<i32>(), -1, n);
  k_head_slots<<<grid_n(H), 256, 0, c->stream>>>(cols.as<uint32_t>(), H, dslot.as<i32>());
  check_launch("head_slots");
  count_launch(c);
  auto hd = std::make_unique<DevPanels>();
  hd->shared = true;
  hd->master = master;
  hd->m = H;  // the staged slice: w at the head columns (slot order)
  hd->n = n;
  hd->rows = H;
  // stretches of at most ~4096 rows, a whole number of them per CTA: the
  // device packer takes one warp per stretch
  const i64 per_cta = std::max<i64>(1, (m + grid * 4096 - 1) / (grid * 4096));
  hd->nhot = (m + grid * per_cta - 1) / (grid * per_cta);  // rows per stretch
  hd->npanels = (m + hd->nhot - 1) / hd->nhot;
  const i64 np = hd->npanels, chunk = hd->nhot, Q = np * chunk;
  hd->hot_cols.alloc(sizeof(i32) * std::max<i64>(H, 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(hd->hot_cols.p, cols.p, sizeof(i32) * H, cudaMemcpyDeviceToDevice, c->stream));
  DBuf hcnt, tcnt, hoff, tof;
  hcnt.alloc(sizeof(i64) * m, c->stream);
  tcnt.alloc(sizeof(i64) * m, c->stream);
  hoff.alloc(sizeof(i64) * (m + 1), c->stream);
  tof.alloc(sizeof(i64) * (m + 1), c->stream);
  k_head_counts<<<grid_n(32 * m), 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), m, dslot.as<i32>(),
                                                       hcnt.as<i64>(), tcnt.as<i64>());
  check_launch("head_counts");
  count_launch(c);
  scan_i64(c, hcnt.as<i64>(), hoff.as<i64>(), m);
  scan_i64(c, tcnt.as<i64>(), tof.as<i64>(), m);
  i64 tot[2];
  FVG_CUDA(cudaMemcpyAsync(&tot[0], hoff.as<i64>() + m, sizeof(i64), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaMemcpyAsync(&tot[1], tof.as<i64>() + m, sizeof(i64), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  if (!forced && (double)tot[0] < 0.5 * (double)nnz) return nullptr;  // most entries outside the head
  hd->E = tot[0];
  hd->poff.alloc(sizeof(i32) * (Q + 1), c->stream);
  k_head_off<<<grid_n(Q + 1), 256, 0, c->stream>>>(hoff.as<i64>(), m, Q, hd->poff.as<i32>());
  check_launch("head_off");
  count_launch(c);
  alloc_padded(c, hd->prow, hd->E, 2);
  alloc_padded(c, hd->val[master], hd->E, dtype_size(master));
  DevCRS& tail = hd->cold;
  tail.m = m;
  tail.n = n;
  tail.nnz = tot[1];
  tail.off.alloc(sizeof(i32) * (m + 1), c->stream);
  k_i64_to_i32<<<grid_n(m + 1), 256, 0, c->stream>>>(tof.as<i64>(), tail.off.as<i32>(), m + 1);
  check_launch("tail_off");
  count_launch(c);
  alloc_padded(c, tail.idx, tail.nnz, 4);
  alloc_padded(c, tail.val[master], tail.nnz, dtype_size(master));
  const SidePlanes sph = side_planes(c, a.val, a.lo, master, hd->val, hd->lo, hd->E);
  const SidePlanes spt = side_planes(c, a.val, a.lo, master, tail.val, tail.lo, tail.nnz);
  auto fill = [&](auto tag) {
    using T = decltype(tag);
    k_head_fill<T><<<grid_n(32 * m), 256, 0, c->stream>>>(
        a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<T>(), m, dslot.as<i32>(), hoff.as<i64>(), tof.as<i64>(),
        hd->prow.as<uint16_t>(), hd->val[master].as<T>(), tail.idx.as<i32>(), tail.val[master].as<T>(), sph, spt);
    check_launch("head_fill");
    count_launch(c);
  };
  if (master == FVG_F64) fill(double{});
  else if (master == FVG_F32) fill(float{});
  else fill(bf16{});
  tail.max_row = 0;
  pack_panels(c, *hd, chunk, np);
  crs_sched(c, tail, kWarpTile);
  hd->ypan.alloc(sizeof(float) * Q, c->stream);
  hd->partials.alloc(sizeof(float) * std::max<i64>(hd->npieces, 1), c->stream);
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
  return hd;
}

}  // namespace

DevPanels* panels_for(fvg_ctx* c, fvg_matrix* M) {
  if (M->panel_rows == 0) return nullptr;
  if (M->pan) return M->pan.get();
  if (M->pan_tried) return nullptr;
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
  // a forced layout that cannot be built throws here, on every call
  std::unique_ptr<DevPanels> pn = panel_build(c, *M->AT, M->master, M->panel_rows, M->panel_min);
  M->pan_tried = true;
  M->pan = std::move(pn);
  return M->pan.get();
}

void panel_ensure_plane(fvg_ctx* c, DevPanels& pn, int dt) {
  ensure_plane_generic(c, pn.val, pn.E, dt, pn.master);
  crs_ensure_plane(c, pn.cold, dt, pn.master);
}

i64 panel_scratch_bytes(fvg_ctx* c, DevPanels& pn, int storage) { return crs_pass_scratch_bytes(c, pn.cold, storage); }

void panel_trans_mv(fvg_ctx* c, DevPanels& pn, int storage, const float* r, int y_dt, void* y, void* scratch,
                    int prof_key) {
  if (storage == FVG_F64) fail(FVG_ERR_INTERNAL, "the panel product runs on FP32 or BF16 values");
  if (y_dt != FVG_F64 && y_dt != FVG_F32) fail(FVG_ERR_INTERNAL, "panel product output must be FP64 or FP32");
  panel_ensure_plane(c, pn, storage);
  ProfScope pr(c, prof_key);
  // cold columns (and zeros for the hot ones) by the transposed CRS kernel
  crs_pass(c, pn.cold, storage, FVG_F32, r, y_dt, y, EPI_STORE, nullptr, scratch, P_NKEYS);
  PanK k;
  k.poff = pn.poff.as<i32>();
  k.prow = pn.prow.as<uint16_t>();
  k.val = pn.val[storage].p;
  k.r = r;
  k.m = pn.m;
  k.rows = pn.rows;
  k.npanels = pn.npanels;
  k.items = pn.items.as<Item>();
  k.pitem0 = pn.pitem0.as<i32>();
  k.long_rows = pn.long_rows.as<i32>();
  k.plong0 = pn.plong0.as<i32>();
  k.long_piece0 = pn.long_piece0.as<i32>();
  k.partials = pn.partials.as<float>();
  k.ypan = pn.ypan.as<float>();
  k.err = c->dev_err;
  k.wait_limit = copy_polls(c);
  k.aligned = ((reinterpret_cast<uintptr_t>(r) & 15) == 0) ? 1 : 0;
  k.xmap = nullptr;
  k.group = 1;
  if (storage == FVG_F32) launch_panel<float>(c, k, pn.rows);
  else launch_panel<bf16>(c, k, pn.rows);
  const unsigned cg = (unsigned)std::max<i64>(1, std::min<i64>((pn.nhot + 31) / 32, 2 * c->num_sms));
  if (y_dt == FVG_F64)
    k_panel_colsum<double><<<cg, 1024, 0, c->stream>>>(pn.ypan.as<float>(), pn.hot_cols.as<i32>(), pn.nhot,
                                                        pn.npanels, (double*)y);
  else
    k_panel_colsum<float><<<cg, 1024, 0, c->stream>>>(pn.ypan.as<float>(), pn.hot_cols.as<i32>(), pn.nhot,
                                                       pn.npanels, (float*)y);
  check_launch("k_panel_colsum");
  count_launch(c);
}

}  // namespace fvg

namespace fvg {

DevPanels* head_for(fvg_ctx* c, fvg_matrix* M) {
  if (M->head_cols == 0) return nullptr;
  if (M->head) return M->head.get();
  if (M->head_tried) return nullptr;
  if (!M->AT) {
    M->AT.reset(new DevCRS());
    crs_build_transpose(c, M->A, *M->AT, M->master);
  }
  std::unique_ptr<DevPanels> hd = head_build(c, M->A, *M->AT, M->master, M->head_cols);
  M->head_tried = true;
  M->head = std::move(hd);
  return M->head.get();
}

void head_ensure_plane(fvg_ctx* c, DevPanels& hd, int dt) {
  ensure_plane_generic(c, hd.val, hd.E, dt, hd.master);
  crs_ensure_plane(c, hd.cold, dt, hd.master);
}

i64 head_scratch_bytes(fvg_ctx* c, DevPanels& hd, int storage) { return crs_pass_scratch_bytes(c, hd.cold, storage); }

void head_logreg_pass(fvg_ctx* c, DevPanels& hd, int storage, const float* w, const LogregEpi& lr, void* scratch,
                      int prof_key) {
  if (storage == FVG_F64) fail(FVG_ERR_INTERNAL, "the head pass runs on FP32 or BF16 values");
  head_ensure_plane(c, hd, storage);
  ProfScope pr(c, prof_key);
  PanK k;
  k.poff = hd.poff.as<i32>();
  k.prow = hd.prow.as<uint16_t>();
  k.val = hd.val[storage].p;
  k.r = w;
  k.m = hd.m;
  k.rows = hd.rows;
  k.npanels = hd.npanels;
  k.items = hd.items.as<Item>();
  k.pitem0 = hd.pitem0.as<i32>();
  k.long_rows = hd.long_rows.as<i32>();
  k.plong0 = hd.plong0.as<i32>();
  k.long_piece0 = hd.long_piece0.as<i32>();
  k.partials = hd.partials.as<float>();
  k.ypan = hd.ypan.as<float>();
  k.err = c->dev_err;
  k.wait_limit = copy_polls(c);
  k.aligned = 0;
  k.xmap = hd.hot_cols.as<i32>();
  k.group = (hd.npanels + c->num_sms - 1) / c->num_sms;  // a CTA's whole share of the stretches
  if (storage == FVG_F32) launch_panel<float>(c, k, hd.rows);
  else launch_panel<bf16>(c, k, hd.rows);
  LogregEpi t = lr;
  t.ybase = hd.ypan.as<float>();
  crs_pass(c, hd.cold, storage, FVG_F32, w, FVG_F32, nullptr, EPI_LOGREG, &t, scratch, P_NKEYS);
}

}  // namespace fvg

// ------------------------------------------------------------ split storage
namespace fvg {

namespace {
void launch_panel_split(fvg_ctx* c, const PanSK& k, i64 rows) {
  constexpr int threads = kSplitWarps * 32;
  static std::mutex mu;  // contexts of different host threads launch concurrently
  static std::vector<int> attr_set;
  const int smem = panel_split_smem_bytes(rows);
  {
    std::lock_guard<std::mutex> lock(mu);
    if (std::find(attr_set.begin(), attr_set.end(), c->device) == attr_set.end()) {
      int optin = 0;
      FVG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
      FVG_CUDA(cudaFuncSetAttribute(k_panel_split<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
      FVG_CUDA(cudaFuncSetAttribute(k_panel_split<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
      attr_set.push_back(c->device);
    }
  }
  // the row panels (no shared slice map) take the middle-row pass
  const bool panels = k.xmap == nullptr;
  const void* kfn = panels ? (const void*)k_panel_split<true> : (const void*)k_panel_split<false>;
  const int blocks = occupancy_blocks(kfn, threads, (size_t)smem);
  const i64 nunits = (k.npanels + k.group - 1) / k.group;
  const int grid = (int)std::max<i64>(1, std::min<i64>(nunits, (i64)blocks * c->num_sms));
  if (panels) k_panel_split<true><<<grid, threads, smem, c->stream>>>(k);
  else k_panel_split<false><<<grid, threads, smem, c->stream>>>(k);
  check_launch("k_panel_split");
  count_launch(c);
}

PanSK split_args(fvg_ctx* c, DevPanels& pn, const void* x) {
  PanSK k;
  k.poff = pn.poff.as<i32>();
  k.prow = pn.prow.as<uint16_t>();
  k.vh = pn.val[FVG_F32].as<float>();
  k.vl = pn.lo.as<unsigned short>();
  k.x = (const float2*)x;
  k.m = pn.m;
  k.rows = pn.rows;
  k.npanels = pn.npanels;
  const PanelItems& si = *pn.split_items;
  k.items = si.items.as<Item>();
  k.pitem0 = si.pitem0.as<i32>();
  k.long_rows = si.long_rows.as<i32>();
  k.plong0 = si.plong0.as<i32>();
  k.long_piece0 = si.long_piece0.as<i32>();
  k.partials = pn.partials2.as<float2>();
  k.ypan = pn.ypan2.as<float2>();
  k.err = c->dev_err;
  k.wait_limit = copy_polls(c);
  k.xmap = nullptr;
  k.group = 1;
  return k;
}
}  // namespace

void panel_ensure_split(fvg_ctx* c, DevPanels& pn) {
  if (pn.rows > panel_rows_cap(c))
    fail(FVG_ERR_INTERNAL, "panel layout too tall for the split kernel");
  ensure_split_planes(c, pn.val, pn.E, pn.master, pn.lo);
  crs_ensure_split(c, pn.cold, pn.master);
  if (!pn.split_items) pack_split_items(c, pn);
  if (!pn.ypan2.p) {
    pn.ypan2.alloc(sizeof(float2) * std::max<i64>(pn.npanels * pn.nhot, 1), c->stream);
    pn.partials2.alloc(sizeof(float2) * std::max<i64>(pn.split_items->npieces, 1), c->stream);
  }
}

i64 panel_split_scratch_bytes(fvg_ctx* c, DevPanels& pn, bool y_df) {
  return crs_split_scratch_bytes(c, pn.cold, y_df);
}

void panel_trans_mv_split(fvg_ctx* c, DevPanels& pn, const void* r, double* y, void* scratch) {
  panel_ensure_split(c, pn);
  // cold columns (and zeros for the hot ones) by the transposed CRS kernel
  crs_pass_split(c, pn.cold, r, false, y, scratch, P_NKEYS);
  launch_panel_split(c, split_args(c, pn, r), pn.rows);
  const unsigned cg = (unsigned)std::max<i64>(1, std::min<i64>((pn.nhot + 31) / 32, 2 * c->num_sms));
  k_panel_colsum_split<<<cg, 1024, 0, c->stream>>>(pn.ypan2.as<float2>(), pn.hot_cols.as<i32>(), pn.nhot,
                                                    pn.npanels, y);
  check_launch("k_panel_colsum_split");
  count_launch(c);
}

void head_pass_split(fvg_ctx* c, DevPanels& hd, const void* w, void* wtx, void* scratch) {
  panel_ensure_split(c, hd);
  PanSK k = split_args(c, hd, w);
  k.xmap = hd.hot_cols.as<i32>();
  k.group = (hd.npanels + c->num_sms - 1) / c->num_sms;  // a CTA's whole share of the stretches
  launch_panel_split(c, k, hd.rows);
  crs_pass_split(c, hd.cold, w, true, wtx, scratch, P_NKEYS);
}

}  // namespace fvg
