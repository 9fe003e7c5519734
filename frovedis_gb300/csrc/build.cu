// Device-side builders: CRS upload and checks, the transposed CRS copy
// (crs_matrix.hpp:356-412), the work-item schedule of the CRS kernel, and the
// ELL / JDS / JDS-CRS-hybrid layouts (ell_matrix.hpp:63-95,
// jds_matrix.hpp:81-146, jds_crs_hybrid.hpp:38-153).
#include <algorithm>
#include <vector>

#include "fvg_internal.cuh"

namespace fvg {

static unsigned grid_n(i64 n, int threads = 256) {
  i64 g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}
#define GRID_STRIDE(i, n) for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (i64)gridDim.x * blockDim.x)

static int bits_for(i64 maxval) {  // bits needed to represent values in [0, maxval]
  int b = 0;
  while (b < 62 && (1ll << b) <= maxval) b++;
  return b;
}

static void alloc_plane(fvg_ctx* c, DBuf& b, i64 n, int dt) {
  b.alloc((size_t)(n + kPad) * dtype_size(dt), c->stream);
  FVG_CUDA(cudaMemsetAsync((char*)b.p + (size_t)n * dtype_size(dt), 0, (size_t)kPad * dtype_size(dt), c->stream));
}

void ensure_plane_generic(fvg_ctx* c, DBuf* planes, i64 n, int dt, int master) {
  if (planes[dt].p) return;
  if (!planes[master].p) fail(FVG_ERR_INTERNAL, "value plane missing");
  if (dt == FVG_F64 && master != FVG_F64)
    fail(FVG_ERR_INVALID_ARG, "FP64 storage requested for a matrix uploaded with lower-precision values");
  alloc_plane(c, planes[dt], n, dt);
  convert_values(c, planes[master].p, master, planes[dt].p, dt, n);
}

void crs_ensure_plane(fvg_ctx* c, DevCRS& a, int dt, int master) { ensure_plane_generic(c, a.val, a.nnz, dt, master); }

// ------------------------------------------------------------------ upload
// Counts and the longest row are combined per warp first: one atomic per
// warp instead of one per row on a single address.
__global__ void k_check_crs(const i32* __restrict__ off, const i32* __restrict__ idx, i64 m, i64 n, i64 nnz,
                            unsigned long long* __restrict__ flags /* [0]=bad off, [1]=bad idx, [2]=max len */) {
  unsigned bad_off = 0, bad_idx = 0, mx = 0;
  GRID_STRIDE(r, m) {
    i32 s = off[r], e = off[r + 1];
    if (e < s || s < 0 || e > nnz) bad_off++;
    else mx = max(mx, (unsigned)(e - s));
  }
  GRID_STRIDE(p, nnz) {
    i32 c = idx[p];
    if (c < 0 || c >= n) bad_idx++;
  }
  bad_off = __reduce_add_sync(0xffffffffu, bad_off);
  bad_idx = __reduce_add_sync(0xffffffffu, bad_idx);
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0) {
    if (bad_off) atomicAdd(&flags[0], (unsigned long long)bad_off);
    if (bad_idx) atomicAdd(&flags[1], (unsigned long long)bad_idx);
    if (mx) atomicMax(&flags[2], (unsigned long long)mx);
  }
}

void crs_upload(fvg_ctx* c, DevCRS& a, i64 m, i64 n, const i32* off, const i32* idx, const void* val, int dt,
                bool on_device) {
  if (m < 0 || n < 0) fail(FVG_ERR_INVALID_ARG, "negative matrix dimension");
  if (!off) fail(FVG_ERR_INVALID_ARG, "null row offsets");
  i32 first = 0, last = 0;
  cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (on_device) {
    FVG_CUDA(cudaMemcpyAsync(&first, off, sizeof(i32), cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaMemcpyAsync(&last, off + m, sizeof(i32), cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
  } else {
    first = off[0];
    last = off[m];
  }
  if (first != 0) fail(FVG_ERR_INVALID_ARG, "row offsets must start at 0");
  if (last < 0) fail(FVG_ERR_INVALID_ARG, "negative nnz");
  i64 nnz = last;
  if (nnz > 0 && (!idx || !val)) fail(FVG_ERR_INVALID_ARG, "null idx/val");
  a.m = m;
  a.n = n;
  a.nnz = nnz;
  a.off.alloc(sizeof(i32) * (m + 1), c->stream);
  a.idx.alloc(sizeof(i32) * (nnz + kPad), c->stream);
  FVG_CUDA(cudaMemcpyAsync(a.off.p, off, sizeof(i32) * (m + 1), kind, c->stream));
  FVG_CUDA(cudaMemsetAsync(a.idx.as<i32>() + nnz, 0, sizeof(i32) * kPad, c->stream));
  if (nnz) FVG_CUDA(cudaMemcpyAsync(a.idx.p, idx, sizeof(i32) * nnz, kind, c->stream));
  alloc_plane(c, a.val[dt], nnz, dt);
  if (nnz) FVG_CUDA(cudaMemcpyAsync(a.val[dt].p, val, (size_t)dtype_size(dt) * nnz, kind, c->stream));
  DBuf flags;
  flags.alloc(sizeof(unsigned long long) * 3, c->stream);
  FVG_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(unsigned long long) * 3, c->stream));
  k_check_crs<<<grid_n(std::max(m, nnz)), 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), m, n, nnz,
                                                                flags.as<unsigned long long>());
  check_launch("check_crs");
  count_launch(c);
  unsigned long long h[3];
  FVG_CUDA(cudaMemcpyAsync(h, flags.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  if (h[0]) fail(FVG_ERR_INVALID_ARG, "row offsets are not non-decreasing within [0, nnz]");
  if (h[1]) fail(FVG_ERR_INVALID_ARG, "column index out of range [0, num_col)");
  a.max_row = (i64)h[2];
}

__global__ void k_max_row(const i32* __restrict__ off, i64 m, unsigned long long* __restrict__ mx) {
  unsigned v = 0;
  GRID_STRIDE(r, m) v = max(v, (unsigned)(off[r + 1] - off[r]));
  v = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && v) atomicMax(mx, (unsigned long long)v);
}

static i64 max_row_len(fvg_ctx* c, const i32* off, i64 m) {
  if (m <= 0) return 0;
  DBuf mx;
  mx.alloc(sizeof(unsigned long long), c->stream);
  FVG_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), c->stream));
  k_max_row<<<grid_n(m), 256, 0, c->stream>>>(off, m, mx.as<unsigned long long>());
  check_launch("max_row");
  count_launch(c);
  unsigned long long h = 0;
  FVG_CUDA(cudaMemcpyAsync(&h, mx.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  return (i64)h;
}

// --------------------------------------------------------------- transpose
__global__ void k_iota_u32(uint32_t* p, i64 n) { GRID_STRIDE(i, n) p[i] = (uint32_t)i; }

// toff[c] = first sorted position whose column is >= c
__global__ void k_boundaries(const uint32_t* __restrict__ keys, i64 nnz, i64 ncols, i32* __restrict__ toff) {
  GRID_STRIDE(i, nnz + 1) {
    i64 prev = (i == 0) ? -1 : (i64)keys[i - 1];
    i64 cur = (i == nnz) ? ncols : (i64)keys[i];
    for (i64 c = prev + 1; c <= cur; c++) toff[c] = (i32)i;
  }
}

// Row id of every nonzero in A's order: a warp per row, lanes write
// consecutive entries.
__global__ void k_expand_rows(const i32* __restrict__ off, i64 m, uint32_t* __restrict__ rows) {
  const int lane = threadIdx.x & 31;
  const i64 w = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const i64 nw = ((i64)gridDim.x * blockDim.x) >> 5;
  for (i64 r = w; r < m; r += nw)
    for (i64 e = (i64)off[r] + lane; e < off[r + 1]; e += 32) rows[e] = (uint32_t)r;
}

void crs_build_transpose(fvg_ctx* c, const DevCRS& a, DevCRS& t, int master) {
  ProfScope ps(c, P_TRANSPOSE);
  t.m = a.n;
  t.n = a.m;
  t.nnz = a.nnz;
  t.off.alloc(sizeof(i32) * (t.m + 1), c->stream);
  t.idx.alloc(sizeof(i32) * (t.nnz + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(t.idx.as<i32>() + t.nnz, 0, sizeof(i32) * kPad, c->stream));
  alloc_plane(c, t.val[master], t.nnz, master);
  if (a.nnz == 0) {
    fill_i32(c, t.off.as<i32>(), 0, t.m + 1);
    t.max_row = 0;
    return;
  }
  // A stable sort of the nonzeros by column (stable = in row order within a
  // column) that carries each one's row and value, so the sorted rows and
  // values are the transposed copy's column ids and values.
  DBuf rows, keys;
  rows.alloc(sizeof(uint32_t) * (a.nnz + kRsPad), c->stream);
  keys.alloc(sizeof(uint32_t) * (a.nnz + kRsPad), c->stream);
  k_expand_rows<<<grid_n(32 * a.m), 256, 0, c->stream>>>(a.off.as<i32>(), a.m, rows.as<uint32_t>());
  check_launch("expand_rows");
  count_launch(c);
  const uint32_t* kin = reinterpret_cast<const uint32_t*>(a.idx.as<i32>());  // ids are in [0, n)
  uint32_t* tidx = reinterpret_cast<uint32_t*>(t.idx.as<i32>());
  const int bits = bits_for(a.n - 1);
  if (master == FVG_F64)
    radix_sort_rowval<double>(c, kin, rows.as<uint32_t>(), a.val[master].as<double>(), keys.as<uint32_t>(), tidx,
                              t.val[master].as<double>(), a.nnz, bits);
  else if (master == FVG_F32)
    radix_sort_rowval<float>(c, kin, rows.as<uint32_t>(), a.val[master].as<float>(), keys.as<uint32_t>(), tidx,
                             t.val[master].as<float>(), a.nnz, bits);
  else
    radix_sort_rowval<bf16>(c, kin, rows.as<uint32_t>(), a.val[master].as<bf16>(), keys.as<uint32_t>(), tidx,
                            t.val[master].as<bf16>(), a.nnz, bits);
  rows.release();
  k_boundaries<<<grid_n(a.nnz + 1), 256, 0, c->stream>>>(keys.as<uint32_t>(), a.nnz, a.n, t.off.as<i32>());
  check_launch("boundaries");
  count_launch(c);
  keys.release();
  t.max_row = max_row_len(c, t.off.as<i32>(), t.m);
  check_device_error(c);  // the sort's bounded copy waits
}

// ---------------------------------------------------------------- schedule
// Packs rows, in row order, into work items (see Sched): consecutive short
// rows share a row tile while the tile stays within `tile` nonzeros,
// kTileRows rows and kLaneWork products per lane; a long row becomes its own
// pieces of at most `tile` nonzeros, cut at 8-element boundaries.  Built on
// the device once per matrix, in chunks of kSchedChunk rows packed by one
// thread each (a tile never spans two chunks).
constexpr i64 kSchedChunk = kPackRows;

const Sched& crs_sched(fvg_ctx* c, DevCRS& a, int tile) {
  // slot 0: the CRS kernel's items (kWarpTile); slot 1: another item size
  // (the split kernel's), built on its first use
  const int slot = tile == kWarpTile ? 0 : 1;
  if (a.sched[slot]) {
    if (a.sched[slot]->tile != tile) fail(FVG_ERR_INTERNAL, "a second work-item size for one matrix");
    return *a.sched[slot];
  }
  ProfScope ps(c, P_SCHED);
  auto s = std::make_unique<Sched>();
  s->tile = tile;
  const i64 m = a.m;
  const i64 nchunks = std::max<i64>(1, (m + kSchedChunk - 1) / kSchedChunk);
  PackOut o;
  device_pack(c, a.off.as<i32>(), m, kSchedChunk, nchunks, tile, o);
  s->nitems = o.nitems;
  s->nlong = o.nlong;
  s->npieces = o.npieces;
  s->items = std::move(o.items);
  s->long_rows = std::move(o.long_rows);
  s->long_piece0 = std::move(o.long_piece0);
  a.sched[slot] = std::move(s);
  return *a.sched[slot];
}

// ------------------------------------------------------ slab-ordered pieces
// Work items of a transposed product whose gathered vector rows are larger
// than L2 (the batched and multinomial backward products, A^T R with R's
// rows 256-512 bytes): the rows longer than a tile are cut into pieces at
// every slab boundary of their column ids (slab = `slab` consecutive rows
// of R) as well as every `tile` entries, and those pieces are listed slab by
// slab, so that the warps sweeping the item list gather from one slab of R
// at a time (an L2-sized slab stays in L2).  Short rows stay in their tiles
// (after the pieces).  Pieces of a row keep consecutive numbers in slab
// order, so the finalize kernel adds them in a fixed order.
__device__ __forceinline__ i64 first_at_least(const i32* __restrict__ idx, i64 lo, i64 hi, i64 v) {
  while (lo < hi) {
    const i64 mid = (lo + hi) >> 1;
    if ((i64)idx[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_slab_pieces(const i32* __restrict__ long_rows, i64 nlong, const i32* __restrict__ off,
                              const i32* __restrict__ idx, int tile, i64 slab, const i32* __restrict__ piece0,
                              i32* __restrict__ cnt, Item* __restrict__ items, uint32_t* __restrict__ keys) {
  GRID_STRIDE(i, nlong) {
    const i32 r = long_rows[i];
    i64 e = off[r];
    const i64 end = off[r + 1];
    i64 q = piece0 ? piece0[i] : 0;
    i32 n = 0;
    while (e < end) {
      const i64 b = (i64)idx[e] / slab;
      const i64 be = first_at_least(idx, e, end, (b + 1) * slab);
      for (i64 s = e; s < be; s += tile) {
        const i64 t = s + tile < be ? s + tile : be;
        if (items) {
          items[q] = Item{r, (i32)(-1 - q), (i32)s, (i32)t};
          keys[q] = (uint32_t)b;
        }
        q++;
        n++;
      }
      e = be;
    }
    if (cnt) cnt[i] = n;
  }
}

__global__ void k_gather_items(const Item* __restrict__ src, const uint32_t* __restrict__ order, i64 n,
                               Item* __restrict__ dst) {
  GRID_STRIDE(i, n) dst[i] = src[order[i]];
}

const Sched& crs_sched_slabs(fvg_ctx* c, DevCRS& a, int tile, i64 slab) {
  if (a.slab_sched && a.slab_rows == slab && a.slab_sched->tile == tile) return *a.slab_sched;
  const Sched& s0 = crs_sched(c, a, tile);
  ProfScope ps(c, P_SCHED);
  auto s = std::make_unique<Sched>();
  s->tile = tile;
  s->nlong = s0.nlong;
  cudaStream_t st = c->stream;
  // tiles of the plain schedule (its items whose r1 >= 0)
  std::vector<Item> h0((size_t)s0.nitems);
  if (s0.nitems)
    FVG_CUDA(cudaMemcpyAsync(h0.data(), s0.items.p, sizeof(Item) * s0.nitems, cudaMemcpyDeviceToHost, st));
  DBuf cnt;
  cnt.alloc(sizeof(i32) * std::max<i64>(s0.nlong, 1), st);
  if (s0.nlong) {
    k_slab_pieces<<<grid_n(s0.nlong), 256, 0, st>>>(s0.long_rows.as<i32>(), s0.nlong, a.off.as<i32>(),
                                                     a.idx.as<i32>(), tile, slab, nullptr, cnt.as<i32>(), nullptr,
                                                     nullptr);
    check_launch("slab piece count");
    count_launch(c);
  }
  std::vector<i32> hc((size_t)s0.nlong);
  if (s0.nlong) FVG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(i32) * s0.nlong, cudaMemcpyDeviceToHost, st));
  FVG_CUDA(cudaStreamSynchronize(st));
  std::vector<i32> p0((size_t)s0.nlong + 1, 0);
  i64 np = 0;
  for (i64 i = 0; i < s0.nlong; i++) {
    p0[(size_t)i] = (i32)np;
    np += hc[(size_t)i];
  }
  if (np >= (1ll << 31) - 1) fail(FVG_ERR_INTERNAL, "slab schedule too large");
  p0[(size_t)s0.nlong] = (i32)np;
  i64 ntiles = 0;
  for (const Item& it : h0) ntiles += it.r1 >= 0;
  s->npieces = np;
  s->nitems = np + ntiles;
  s->long_rows.alloc(sizeof(i32) * std::max<i64>(s0.nlong, 1), st);
  s->long_piece0.alloc(sizeof(i32) * (s0.nlong + 1), st);
  s->items.alloc(sizeof(Item) * std::max<i64>(s->nitems, 1), st);
  if (s0.nlong)
    FVG_CUDA(cudaMemcpyAsync(s->long_rows.p, s0.long_rows.p, sizeof(i32) * s0.nlong, cudaMemcpyDeviceToDevice, st));
  FVG_CUDA(cudaMemcpyAsync(s->long_piece0.p, p0.data(), sizeof(i32) * (s0.nlong + 1), cudaMemcpyHostToDevice, st));
  if (np) {
    DBuf tmp, keys, order;
    tmp.alloc(sizeof(Item) * np, st);
    keys.alloc(sizeof(uint32_t) * np, st);
    order.alloc(sizeof(uint32_t) * np, st);
    k_slab_pieces<<<grid_n(s0.nlong), 256, 0, st>>>(s0.long_rows.as<i32>(), s0.nlong, a.off.as<i32>(),
                                                     a.idx.as<i32>(), tile, slab, s->long_piece0.as<i32>(), nullptr,
                                                     tmp.as<Item>(), keys.as<uint32_t>());
    k_iota_u32<<<grid_n(np), 256, 0, st>>>(order.as<uint32_t>(), np);
    check_launch("slab pieces");
    count_launch(c, 2);
    // stable by slab: within a slab the pieces keep row order
    radix_sort_pairs(c, keys.as<uint32_t>(), order.as<uint32_t>(), np, bits_for((a.n - 1) / slab));
    k_gather_items<<<grid_n(np), 256, 0, st>>>(tmp.as<Item>(), order.as<uint32_t>(), np, s->items.as<Item>());
    check_launch("slab order");
    count_launch(c);
  }
  std::vector<Item> ht;
  ht.reserve((size_t)ntiles);
  for (const Item& it : h0)
    if (it.r1 >= 0) ht.push_back(it);
  if (ntiles)
    FVG_CUDA(cudaMemcpyAsync(s->items.as<Item>() + np, ht.data(), sizeof(Item) * ntiles, cudaMemcpyHostToDevice, st));
  FVG_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
  a.slab_sched = std::move(s);
  a.slab_rows = slab;
  return *a.slab_sched;
}

// --------------------------------------------------------------------- ELL
template <class T>
__global__ void k_ell_fill(const i32* __restrict__ off, const i32* __restrict__ idx, const T* __restrict__ val,
                           i64 m, i32* __restrict__ eidx, T* __restrict__ eval) {
  GRID_STRIDE(r, m) {
    i64 s = off[r], e = off[r + 1];
    for (i64 k = 0; k < e - s; k++) {
      eidx[m * k + r] = idx[s + k];
      eval[m * k + r] = val[s + k];
    }
  }
}

void ell_build(fvg_ctx* c, const DevCRS& a, DevELL& e, int master) {
  e.m = a.m;
  e.n = a.n;
  e.width = (a.m == 0) ? 0 : a.max_row;
  double bytes = (double)a.m * (double)e.width * (4.0 + dtype_size(master));
  size_t freeb = 0, totb = 0;
  cudaMemGetInfo(&freeb, &totb);
  if (bytes > 0.6 * (double)freeb)
    fail(FVG_ERR_OUT_OF_MEMORY, "ELL layout needs " + std::to_string(bytes / 1e9) + " GB (num_row x longest row)");
  i64 cells = a.m * e.width;
  e.idx.alloc(sizeof(i32) * (cells + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(e.idx.p, 0, sizeof(i32) * (cells + kPad), c->stream));
  e.val[master].alloc((size_t)dtype_size(master) * (cells + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(e.val[master].p, 0, (size_t)dtype_size(master) * (cells + kPad), c->stream));
  if (cells == 0) return;
  unsigned g = grid_n(a.m);
  if (master == FVG_F64)
    k_ell_fill<double><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<double>(), a.m,
                                                 e.idx.as<i32>(), e.val[master].as<double>());
  else if (master == FVG_F32)
    k_ell_fill<float><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<float>(), a.m,
                                                e.idx.as<i32>(), e.val[master].as<float>());
  else
    k_ell_fill<bf16><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<bf16>(), a.m,
                                               e.idx.as<i32>(), e.val[master].as<bf16>());
  check_launch("ell_fill");
  count_launch(c);
}

// --------------------------------------------------------------------- JDS
__global__ void k_jds_keys(const i32* __restrict__ off, i64 m, i64 maxlen, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals, i64* __restrict__ lenhist) {
  GRID_STRIDE(i, m) {
    i64 r = m - 1 - i;  // rows listed in descending order: ties end up larger row first
    i64 len = (i64)off[r + 1] - off[r];
    keys[i] = (uint32_t)(maxlen - len);
    vals[i] = (uint32_t)r;
    atomicAdd((unsigned long long*)&lenhist[len], 1ull);
  }
}

// count_gt[d] = number of rows longer than d = m - (rows with len <= d)
__global__ void k_count_gt(const i64* __restrict__ ex, i64 m, i64 ndiag, i64* __restrict__ cgt) {
  GRID_STRIDE(d, ndiag) cgt[d] = m - ex[d + 1];
}

template <class T>
__global__ void k_jds_fill(const i32* __restrict__ off, const i32* __restrict__ idx, const T* __restrict__ val,
                           const i32* __restrict__ perm, i64 m, const i64* __restrict__ joff, i64 cap,
                           i32* __restrict__ jidx, T* __restrict__ jval) {
  GRID_STRIDE(p, m) {
    i32 r = perm[p];
    i64 s = off[r], len = (i64)off[r + 1] - s;
    if (len > cap) len = cap;
    for (i64 d = 0; d < len; d++) {
      i64 q = joff[d] + p;
      jidx[q] = idx[s + d];
      jval[q] = val[s + d];
    }
  }
}

static void jds_order(fvg_ctx* c, const DevCRS& a, DBuf& perm, i64 ndiag, DBuf& joff) {
  i64 m = a.m;
  DBuf keys, hist, ex, cgt;
  perm.alloc(sizeof(i32) * std::max<i64>(m, 1), c->stream);
  keys.alloc(sizeof(uint32_t) * std::max<i64>(m, 1), c->stream);
  hist.alloc(sizeof(i64) * (a.max_row + 1), c->stream);
  ex.alloc(sizeof(i64) * (a.max_row + 2), c->stream);
  FVG_CUDA(cudaMemsetAsync(hist.p, 0, sizeof(i64) * (a.max_row + 1), c->stream));
  k_jds_keys<<<grid_n(m), 256, 0, c->stream>>>(a.off.as<i32>(), m, a.max_row, keys.as<uint32_t>(),
                                                perm.as<uint32_t>(), hist.as<i64>());
  check_launch("jds_keys");
  count_launch(c);
  radix_sort_pairs(c, keys.as<uint32_t>(), perm.as<uint32_t>(), m, bits_for(a.max_row));
  scan_i64(c, hist.as<i64>(), ex.as<i64>(), a.max_row + 1);
  cgt.alloc(sizeof(i64) * std::max<i64>(ndiag, 1), c->stream);
  joff.alloc(sizeof(i64) * (ndiag + 1), c->stream);
  if (ndiag > 0) {
    k_count_gt<<<grid_n(ndiag), 256, 0, c->stream>>>(ex.as<i64>(), m, ndiag, cgt.as<i64>());
    check_launch("count_gt");
    count_launch(c);
  }
  scan_i64(c, cgt.as<i64>(), joff.as<i64>(), ndiag);
}

template <class T>
static void launch_jds_fill(fvg_ctx* c, const DevCRS& a, int master, const i32* perm, i64 rows, const i64* joff,
                            i64 cap, i32* jidx, void* jval) {
  if (rows <= 0) return;
  k_jds_fill<T><<<grid_n(rows), 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<T>(), perm,
                                                      rows, joff, cap, jidx, (T*)jval);
  check_launch("jds_fill");
  count_launch(c);
}

static void jds_fill(fvg_ctx* c, const DevCRS& a, int master, const i32* perm, i64 rows, const i64* joff, i64 cap,
                     i32* jidx, void* jval) {
  if (master == FVG_F64) launch_jds_fill<double>(c, a, master, perm, rows, joff, cap, jidx, jval);
  else if (master == FVG_F32) launch_jds_fill<float>(c, a, master, perm, rows, joff, cap, jidx, jval);
  else launch_jds_fill<bf16>(c, a, master, perm, rows, joff, cap, jidx, jval);
}

// Work items of the JDS product from the diagonal lengths (off is
// non-increasing in length): row block b has len(32b) diagonals, cut into
// kJdsSeg-diagonal items; the blocks cut in several get partial slots.
static void jds_items(fvg_ctx* c, DevJDS& j) {
  const i64 nb = (j.m + 31) / 32;
  std::vector<i64> off((size_t)j.ndiag + 1);
  FVG_CUDA(cudaMemcpyAsync(off.data(), j.off.p, sizeof(i64) * (j.ndiag + 1), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<JdsItem> items;
  std::vector<JdsSplit> splits;
  items.reserve((size_t)nb + 16);
  i32 slots = 0;
  for (i64 b = 0; b < nb; b++) {
    const i64 p0 = 32 * b;
    // diagonals longer than p0: the first d with length <= p0
    i64 lo = 0, hi = j.ndiag;
    while (lo < hi) {
      const i64 mid = (lo + hi) >> 1;
      if (off[mid + 1] - off[mid] > p0) lo = mid + 1;
      else hi = mid;
    }
    const i64 D = lo;
    if (D <= kJdsSeg) {
      items.push_back(JdsItem{(i32)b, 0, (i32)D, -1});
      continue;
    }
    const i32 ns = (i32)((D + kJdsSeg - 1) / kJdsSeg);
    splits.push_back(JdsSplit{(i32)b, slots, ns, 0});
    for (i32 q = 0; q < ns; q++)
      items.push_back(JdsItem{(i32)b, (i32)(q * kJdsSeg), (i32)std::min<i64>(D, (q + 1) * kJdsSeg), slots + q});
    slots += ns;
  }
  j.nitems = (i64)items.size();
  j.nsplits = (i64)splits.size();
  j.nslots = slots;
  j.items.alloc(sizeof(JdsItem) * std::max<size_t>(items.size(), 1), c->stream);
  j.splits.alloc(sizeof(JdsSplit) * std::max<size_t>(splits.size(), 1), c->stream);
  if (!items.empty())
    FVG_CUDA(cudaMemcpyAsync(j.items.p, items.data(), sizeof(JdsItem) * items.size(), cudaMemcpyHostToDevice,
                             c->stream));
  if (!splits.empty())
    FVG_CUDA(cudaMemcpyAsync(j.splits.p, splits.data(), sizeof(JdsSplit) * splits.size(), cudaMemcpyHostToDevice,
                             c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
}

void jds_build(fvg_ctx* c, const DevCRS& a, DevJDS& j, int master) {
  j.m = a.m;
  j.n = a.n;
  j.nnz = a.nnz;
  if (a.nnz == 0) {  // jds_matrix.hpp:87-90: empty perm, off = {0}
    j.ndiag = 0;
    j.empty_perm = true;
    j.off.alloc(sizeof(i64), c->stream);
    FVG_CUDA(cudaMemsetAsync(j.off.p, 0, sizeof(i64), c->stream));
    j.perm.alloc(sizeof(i32), c->stream);
    j.idx.alloc(sizeof(i32) * kPad, c->stream);
    alloc_plane(c, j.val[master], 0, master);
    return;
  }
  j.ndiag = a.max_row;
  jds_order(c, a, j.perm, j.ndiag, j.off);
  j.idx.alloc(sizeof(i32) * (a.nnz + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(j.idx.as<i32>() + a.nnz, 0, sizeof(i32) * kPad, c->stream));
  alloc_plane(c, j.val[master], a.nnz, master);
  jds_fill(c, a, master, j.perm.as<i32>(), a.m, j.off.as<i64>(), j.ndiag, j.idx.as<i32>(), j.val[master].p);
  jds_items(c, j);
}

// ------------------------------------------------------------------ hybrid
template <class T>
__global__ void k_hyb_tail(const i32* __restrict__ off, const i32* __restrict__ idx, const T* __restrict__ val,
                           const i32* __restrict__ perm, i64 rows, i64 start, const i32* __restrict__ coff,
                           i32* __restrict__ cidx, T* __restrict__ cval) {
  for (i64 i = blockIdx.x; i < rows; i += gridDim.x) {
    i32 r = perm[i];
    i64 s = (i64)off[r] + start, e = off[r + 1];
    i64 o = coff[i];
    for (i64 k = s + threadIdx.x; k < e; k += blockDim.x) {
      cidx[o + (k - s)] = idx[k];
      cval[o + (k - s)] = val[k];
    }
  }
}

__global__ void k_sorted_lens(const i32* __restrict__ off, const i32* __restrict__ perm, i64 cnt,
                              i64* __restrict__ lens) {
  GRID_STRIDE(i, cnt) lens[i] = (i64)off[perm[i] + 1] - off[perm[i]];
}

__global__ void k_iota_i32(i32* p, i64 n) { GRID_STRIDE(i, n) p[i] = (i32)i; }

void hyb_build(fvg_ctx* c, const DevCRS& a, DevHYB& h, int master, i64 thr) {
  h.m = a.m;
  h.n = a.n;
  h.jds.m = a.m;
  h.jds.n = a.n;
  auto copy_crs = [&](DevCRS& dst) {
    dst.m = a.m; dst.n = a.n; dst.nnz = a.nnz; dst.max_row = a.max_row;
    dst.off.alloc(sizeof(i32) * (a.m + 1), c->stream);
    FVG_CUDA(cudaMemcpyAsync(dst.off.p, a.off.p, sizeof(i32) * (a.m + 1), cudaMemcpyDeviceToDevice, c->stream));
    dst.idx.alloc(sizeof(i32) * (a.nnz + kPad), c->stream);
    FVG_CUDA(cudaMemcpyAsync(dst.idx.p, a.idx.p, sizeof(i32) * (a.nnz + kPad), cudaMemcpyDeviceToDevice, c->stream));
    alloc_plane(c, dst.val[master], a.nnz, master);
    FVG_CUDA(cudaMemcpyAsync(dst.val[master].p, a.val[master].p, (size_t)dtype_size(master) * a.nnz,
                             cudaMemcpyDeviceToDevice, c->stream));
  };
  auto empty_jds = [&](bool identity) {
    h.jds.ndiag = 0;
    h.jds.nnz = 0;
    h.jds.off.alloc(sizeof(i64), c->stream);
    FVG_CUDA(cudaMemsetAsync(h.jds.off.p, 0, sizeof(i64), c->stream));
    h.jds.idx.alloc(sizeof(i32) * kPad, c->stream);
    alloc_plane(c, h.jds.val[master], 0, master);
    h.jds.perm.alloc(sizeof(i32) * std::max<i64>(a.m, 1), c->stream);
    if (identity) {
      k_iota_i32<<<grid_n(a.m), 256, 0, c->stream>>>(h.jds.perm.as<i32>(), a.m);
      check_launch("iota");
      count_launch(c);
    }
    h.jds.empty_perm = !identity;
  };
  if (a.nnz == 0) {  // jds_crs_hybrid.hpp:47-49
    copy_crs(h.crs);
    empty_jds(false);
    h.crs_rows = a.m;
    h.all_crs = true;
    return;
  }
  if (a.m <= thr) {  // 50-56: CRS part is the whole matrix, perm = identity
    copy_crs(h.crs);
    empty_jds(true);
    h.crs_rows = a.m;
    h.all_crs = true;
    return;
  }
  if (thr == 0) {  // 57-61
    jds_build(c, a, h.jds, master);
    h.crs_rows = 0;
    h.crs.m = 0; h.crs.n = a.n; h.crs.nnz = 0;
    h.crs.off.alloc(sizeof(i32), c->stream);
    FVG_CUDA(cudaMemsetAsync(h.crs.off.p, 0, sizeof(i32), c->stream));
    h.crs.idx.alloc(sizeof(i32) * kPad, c->stream);
    alloc_plane(c, h.crs.val[master], 0, master);
    return;
  }
  // 86-153: full JDS order, JDS width = length at sorted position thr
  DBuf joff_full;
  jds_order(c, a, h.jds.perm, a.max_row, joff_full);
  std::vector<i64> lens(thr + 1);
  {
    DBuf dl;
    dl.alloc(sizeof(i64) * (thr + 1), c->stream);
    k_sorted_lens<<<grid_n(thr + 1), 256, 0, c->stream>>>(a.off.as<i32>(), h.jds.perm.as<i32>(), thr + 1,
                                                           dl.as<i64>());
    check_launch("sorted_lens");
    count_launch(c);
    FVG_CUDA(cudaMemcpyAsync(lens.data(), dl.p, sizeof(i64) * (thr + 1), cudaMemcpyDeviceToHost, c->stream));
    FVG_CUDA(cudaStreamSynchronize(c->stream));
  }
  i64 start = lens[thr];
  i64 crs_rows = thr;
  for (; crs_rows != 0; crs_rows--)
    if (lens[crs_rows - 1] != start) break;
  std::vector<i32> hcoff(crs_rows + 1, 0);
  for (i64 i = 0; i < crs_rows; i++) hcoff[i + 1] = hcoff[i] + (i32)(lens[i] - start);
  i64 crs_size = hcoff[crs_rows];
  h.crs_rows = crs_rows;
  h.all_crs = false;
  // JDS part: first `start` elements of every row
  h.jds.ndiag = start;
  h.jds.nnz = a.nnz - crs_size;
  h.jds.off.alloc(sizeof(i64) * (start + 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(h.jds.off.p, joff_full.p, sizeof(i64) * (start + 1), cudaMemcpyDeviceToDevice,
                           c->stream));
  h.jds.idx.alloc(sizeof(i32) * (h.jds.nnz + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(h.jds.idx.as<i32>() + h.jds.nnz, 0, sizeof(i32) * kPad, c->stream));
  alloc_plane(c, h.jds.val[master], h.jds.nnz, master);
  jds_fill(c, a, master, h.jds.perm.as<i32>(), a.m, h.jds.off.as<i64>(), start, h.jds.idx.as<i32>(),
           h.jds.val[master].p);
  jds_items(c, h.jds);
  // CRS tail of the crs_rows longest rows, in sorted order
  h.crs.m = crs_rows;
  h.crs.n = a.n;
  h.crs.nnz = crs_size;
  h.crs.max_row = crs_rows ? lens[0] - start : 0;
  h.crs.off.alloc(sizeof(i32) * (crs_rows + 1), c->stream);
  FVG_CUDA(cudaMemcpyAsync(h.crs.off.p, hcoff.data(), sizeof(i32) * (crs_rows + 1), cudaMemcpyHostToDevice,
                           c->stream));
  h.crs.idx.alloc(sizeof(i32) * (crs_size + kPad), c->stream);
  FVG_CUDA(cudaMemsetAsync(h.crs.idx.as<i32>() + crs_size, 0, sizeof(i32) * kPad, c->stream));
  alloc_plane(c, h.crs.val[master], crs_size, master);
  if (crs_rows > 0) {
    unsigned g = (unsigned)std::min<i64>(crs_rows, 4096);
    if (master == FVG_F64)
      k_hyb_tail<double><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<double>(),
                                                   h.jds.perm.as<i32>(), crs_rows, start, h.crs.off.as<i32>(),
                                                   h.crs.idx.as<i32>(), h.crs.val[master].as<double>());
    else if (master == FVG_F32)
      k_hyb_tail<float><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<float>(),
                                                  h.jds.perm.as<i32>(), crs_rows, start, h.crs.off.as<i32>(),
                                                  h.crs.idx.as<i32>(), h.crs.val[master].as<float>());
    else
      k_hyb_tail<bf16><<<g, 256, 0, c->stream>>>(a.off.as<i32>(), a.idx.as<i32>(), a.val[master].as<bf16>(),
                                                 h.jds.perm.as<i32>(), crs_rows, start, h.crs.off.as<i32>(),
                                                 h.crs.idx.as<i32>(), h.crs.val[master].as<bf16>());
    check_launch("hyb_tail");
    count_launch(c);
  }
  FVG_CUDA(cudaStreamSynchronize(c->stream));  // hcoff host buffer
}

}  // namespace fvg
