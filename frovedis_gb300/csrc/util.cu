// Device utilities: buffers, error plumbing, profiler, exclusive scan,
// stable LSD radix sort, value conversion and gathers.
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "bulk_copy.cuh"
#include "fvg_internal.cuh"

namespace fvg {

void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
  fail(e == cudaErrorMemoryAllocation ? FVG_ERR_OUT_OF_MEMORY : FVG_ERR_CUDA, buf);
}

void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw_cuda(e, what, __FILE__, __LINE__);
}

void check_device_error(fvg_ctx* c) {
  unsigned h = 0;
  FVG_CUDA(cudaMemcpyAsync(&h, c->dev_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  FVG_CUDA(cudaStreamSynchronize(c->stream));
  if (h) {
    FVG_CUDA(cudaMemsetAsync(c->dev_err, 0, sizeof(unsigned), c->stream));
    std::string what;
    if (h & 2u) what += " a bulk copy did not complete in its poll budget;";
    if (h & 4u) what += " a grid barrier was not reached in its poll budget;";
    fail(FVG_ERR_INTERNAL, "a device-side bounded wait gave up:" + what + " results are invalid");
  }
}

// Testing aid: the `after`-th next device allocation fails as if the device
// were out of memory (< 0: off).
static std::atomic<long long> g_alloc_fail_after{-1};
void inject_alloc_failure(long long after) { g_alloc_fail_after.store(after); }

void DBuf::alloc(size_t nbytes, cudaStream_t s) {
  release();
  stream = s;
  bytes = nbytes;
  if (nbytes == 0) return;
  if (g_alloc_fail_after.load() >= 0 && g_alloc_fail_after.fetch_sub(1) == 0)
    throw_cuda(cudaErrorMemoryAllocation, "cudaMallocAsync (injected failure)", __FILE__, __LINE__);
  FVG_CUDA(cudaMallocAsync(&p, nbytes, s));
  // the SpMV kernels issue 16-byte vector loads from the start of every
  // index/value array
  if (reinterpret_cast<uintptr_t>(p) & 255u) fail(FVG_ERR_INTERNAL, "device allocation is not 256-byte aligned");
}

void DBuf::release() {
  if (p) cudaFreeAsync(p, stream);
  p = nullptr;
  bytes = 0;
}

int dtype_size(int dt) { return dt == FVG_F64 ? 8 : dt == FVG_F32 ? 4 : 2; }

// Resident CTAs per SM of a kernel on the current device, computed once per
// (device, kernel, block size, dynamic shared memory) under a mutex: the
// library may be driven from several host threads, each with its own context.
int occupancy_blocks(const void* kernel, int threads, size_t dyn_smem) {
  static std::mutex mu;
  static std::map<std::pair<std::pair<int, const void*>, std::pair<int, size_t>>, int> cache;
  int dev = 0;
  FVG_CUDA(cudaGetDevice(&dev));
  const auto key = std::make_pair(std::make_pair(dev, kernel), std::make_pair(threads, dyn_smem));
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int nb = 0;
  FVG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, dyn_smem));
  nb = nb < 1 ? 1 : nb;
  cache.emplace(key, nb);
  return nb;
}

// ------------------------------------------------------------- profiler
// Event pairs are recorded around the timed launches without synchronising;
// elapsed times are collected when the totals are read.
struct Profiler {
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[P_NKEYS];
  cudaEvent_t open_ev[P_NKEYS] = {};
  double total_ms[P_NKEYS] = {};
  int64_t count[P_NKEYS] = {};
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    FVG_CUDA(cudaEventCreate(&e));
    return e;
  }
  void collect() {
    for (int k = 0; k < P_NKEYS; k++) {
      for (auto& pr : pending[k]) {
        FVG_CUDA(cudaEventSynchronize(pr.second));
        float ms = 0;
        FVG_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
        total_ms[k] += ms;
        count[k] += 1;
        pool.push_back(pr.first);
        pool.push_back(pr.second);
      }
      pending[k].clear();
    }
  }
  ~Profiler() {
    for (int k = 0; k < P_NKEYS; k++)
      for (auto& pr : pending[k]) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    for (auto e : pool) cudaEventDestroy(e);
    for (auto e : open_ev) if (e) cudaEventDestroy(e);
  }
};

void prof_begin(fvg_ctx* c, int key) {
  if (!c->profiling || key < 0 || key >= P_NKEYS) return;
  Profiler& p = *c->prof;
  if (p.open_ev[key]) return;  // nested use of the same key: outer scope wins
  cudaEvent_t e = p.get();
  FVG_CUDA(cudaEventRecord(e, c->stream));
  p.open_ev[key] = e;
}

void prof_end(fvg_ctx* c, int key) {
  if (!c->profiling || key < 0 || key >= P_NKEYS) return;
  Profiler& p = *c->prof;
  if (!p.open_ev[key]) return;
  cudaEvent_t e = p.get();
  cudaEventRecord(e, c->stream);
  p.pending[key].push_back({p.open_ev[key], e});
  p.open_ev[key] = nullptr;
}

void prof_collect(fvg_ctx* c, int key, double* ms, int64_t* n) {
  if (!c->prof) { *ms = 0; *n = 0; return; }
  c->prof->collect();
  *ms = c->prof->total_ms[key];
  *n = c->prof->count[key];
}

void prof_reset(fvg_ctx* c) {
  if (!c->prof) return;
  c->prof->collect();
  for (int k = 0; k < P_NKEYS; k++) { c->prof->total_ms[k] = 0; c->prof->count[k] = 0; }
}

void prof_create(fvg_ctx* c) { c->prof = new Profiler(); }
void prof_destroy(fvg_ctx* c) {
  delete c->prof;
  c->prof = nullptr;
}

// ------------------------------------------------------------------ scan
constexpr int kScanThreads = 256, kScanItems = 16, kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ i64 warp_incl_scan(i64 v) {
  int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    i64 t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the block total too.
__device__ __forceinline__ i64 block_excl_scan(i64 v, i64* total) {
  __shared__ i64 wsum[kScanThreads / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  i64 inc = warp_incl_scan(v);
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    i64 s = (lane < kScanThreads / 32) ? wsum[lane] : 0;
    i64 si = warp_incl_scan(s);
    if (lane < kScanThreads / 32) wsum[lane] = si - s;
    if (lane == kScanThreads / 32 - 1) *total = si;
  }
  __syncthreads();
  i64 r = inc - v + wsum[w];
  __syncthreads();
  return r;
}

__global__ void k_scan_reduce(const i64* __restrict__ in, i64 n, i64* __restrict__ sums) {
  i64 base = (i64)blockIdx.x * kScanTile;
  i64 s = 0;
  for (int k = 0; k < kScanItems; k++) {
    i64 i = base + (i64)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  __shared__ i64 tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_down(const i64* in, i64 n, const i64* __restrict__ block_off, i64* out) {
  i64 base = (i64)blockIdx.x * kScanTile + (i64)threadIdx.x * kScanItems;
  i64 v[kScanItems];
  i64 s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    i64 i = base + k;
    v[k] = (i < n) ? in[i] : 0;
    s += v[k];
  }
  __shared__ i64 tot;
  i64 ex = block_excl_scan(s, &tot) + block_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    i64 i = base + k;
    if (i < n) out[i] = ex;
    ex += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) out[n] = ex;
}

void scan_i64(fvg_ctx* c, const i64* in, i64* out, i64 n) {
  if (n <= 0) {
    FVG_CUDA(cudaMemsetAsync(out, 0, sizeof(i64), c->stream));
    return;
  }
  i64 nb = (n + kScanTile - 1) / kScanTile;
  DBuf sums, offs;
  sums.alloc(sizeof(i64) * nb, c->stream);
  offs.alloc(sizeof(i64) * (nb + 1), c->stream);
  k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, c->stream>>>(in, n, sums.as<i64>());
  check_launch("scan_reduce");
  count_launch(c);
  if (nb == 1) {
    FVG_CUDA(cudaMemsetAsync(offs.p, 0, sizeof(i64), c->stream));
  } else {
    scan_i64(c, sums.as<i64>(), offs.as<i64>(), nb);
  }
  k_scan_down<<<(unsigned)nb, kScanThreads, 0, c->stream>>>(in, n, offs.as<i64>(), out);
  check_launch("scan_down");
  count_launch(c);
}

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort, 8-bit digits.  A tile of 4096 keys per CTA; warp w
// of the CTA owns keys [w*512, w*512+512) of the tile and ranks them in 16
// rounds of 32 consecutive keys with __match_any_sync, so the rank order is
// the input order (stability).
constexpr int kRsThreads = 256, kRsWarps = 8, kRsRounds = 16, kRsTile = kRsThreads * kRsRounds;
constexpr int kRsRoundsRv = 12, kRsTileRv = kRsThreads * kRsRoundsRv;  // the payload-carrying sort

template <int R>
__global__ void k_rs_upsweep(const uint32_t* __restrict__ keys, i64 n, int shift, i64 nblocks,
                             i64* __restrict__ hist) {
  __shared__ int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  i64 base = (i64)blockIdx.x * (kRsThreads * R);
  for (int k = 0; k < R; k++) {
    i64 i = base + (i64)k * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1);
  }
  __syncthreads();
  hist[(i64)threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of 256 ints in shared memory by a 256-thread CTA.
__device__ __forceinline__ void scan256_exclusive(int* v) {
  __shared__ int wsum[kRsWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int x = v[threadIdx.x];
  int inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  int before = 0;
  for (int q = 0; q < w; q++) before += wsum[q];
  v[threadIdx.x] = before + inc - x;
}

// Ranks of a tile's keys (warp w: keys [w*512, w*512+512) of the tile in 16
// rounds of 32; key i at kin[i - key_base]) and the digit bookkeeping of the
// downsweeps: on return
// wcnt[w][d] is warp w's first slot within digit d's run of the tile,
// dstart[d] the run's first tile slot, rank[r] the key's rank among the
// warp's keys of its digit (-1 past n).  Ranks follow the input order.
template <int R>
__device__ __forceinline__ void rs_rank_tile(const uint32_t* __restrict__ kin, i64 key_base, i64 n, int shift,
                                             uint32_t (&key)[R], int (&rank)[R], int (*wcnt)[256], int* dstart) {
  for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const i64 base = (i64)blockIdx.x * (kRsThreads * R) + (i64)w * (R * 32);
#pragma unroll
  for (int r = 0; r < R; r++) {
    i64 i = base + r * 32 + lane;
    bool ok = i < n;
    key[r] = ok ? kin[i - key_base] : 0u;
    int d = ok ? (int)((key[r] >> shift) & 255u) : 256 + lane;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    int before = __popc(peers & lt);
    int cur = ok ? wcnt[w][d] : 0;
    __syncwarp();
    if (ok && before == 0) wcnt[w][d] = cur + __popc(peers);
    __syncwarp();
    rank[r] = ok ? cur + before : -1;
  }
  __syncthreads();
  {  // exclusive prefix over warps for digit = threadIdx.x; the digit's tile total
    int d = threadIdx.x, acc = 0;
    for (int q = 0; q < kRsWarps; q++) {
      int t = wcnt[q][d];
      wcnt[q][d] = acc;
      acc += t;
    }
    dstart[d] = acc;
  }
  __syncthreads();
  scan256_exclusive(dstart);  // first tile slot of each digit
  __syncthreads();
}

// Downsweep: ranks as above, then the tile is sorted by digit in shared
// memory (digit-major, input order within a digit) and written back in that
// order, so consecutive threads store consecutive positions of a digit's run.
__global__ void k_rs_downsweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                               uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, i64 n, int shift,
                               i64 nblocks, const i64* __restrict__ goff) {
  __shared__ int wcnt[kRsWarps][256];
  __shared__ int dstart[256];
  __shared__ uint32_t skey[kRsTile], sval[kRsTile];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t key[kRsRounds];
  int rank[kRsRounds];
  rs_rank_tile<kRsRounds>(kin, 0, n, shift, key, rank, wcnt, dstart);
  const i64 base = (i64)blockIdx.x * kRsTile + (i64)w * (kRsRounds * 32);
#pragma unroll
  for (int r = 0; r < kRsRounds; r++) {
    if (rank[r] < 0) continue;
    const int d = (int)((key[r] >> shift) & 255u);
    const int lp = dstart[d] + wcnt[w][d] + rank[r];
    skey[lp] = key[r];
    sval[lp] = vin[base + r * 32 + lane];
  }
  __syncthreads();
  const i64 t0 = (i64)blockIdx.x * kRsTile;
  const int cnt = (int)(n - t0 < kRsTile ? n - t0 : kRsTile);
  for (int i = threadIdx.x; i < cnt; i += kRsThreads) {
    const uint32_t k = skey[i];
    const int d = (int)((k >> shift) & 255u);
    const i64 pos = goff[(i64)d * nblocks + blockIdx.x] + (i - dstart[d]);
    kout[pos] = k;
    vout[pos] = sval[i];
  }
}

// Downsweep carrying a (row, value) payload.  Thread 0 stages the tile's keys,
// rows and values in shared memory with three bulk copies on one mbarrier
// (the copies' sizes rounded up to 16 bytes: the arrays are padded past n);
// the warps rank the staged keys, the ranked keys go to their tile slots (over
// the staged keys, which the ranking no longer needs) with their input
// position, and the write-back reads each slot's row and value from the
// staged copy.  Tiles of kRsTileRv entries (12 rounds: three CTAs per SM with
// FP64 values); dynamic shared memory: kRsTileRv keys and rows (uint32) and
// kRsTileRv values.  A copy wait that runs out of polls sets bit 2 of *err
// and the CTA returns without writing.
template <class T>
__global__ void __launch_bounds__(kRsThreads) k_rs_downsweep_rv(const uint32_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ rin,
                                                                const T* __restrict__ vin, uint32_t* __restrict__ kout,
                                                                uint32_t* __restrict__ rout, T* __restrict__ vout,
                                                                i64 n, int shift, i64 nblocks,
                                                                const i64* __restrict__ goff, unsigned* err,
                                                                unsigned limit) {
  constexpr int R = kRsRoundsRv, TILE = kRsTileRv;
  __shared__ int wcnt[kRsWarps][256];
  __shared__ int dstart[256];
  __shared__ uint16_t spos[TILE];
  __shared__ __align__(8) uint64_t bar;
  extern __shared__ __align__(16) unsigned char rs_dyn[];
  uint32_t* kst = reinterpret_cast<uint32_t*>(rs_dyn);  // staged keys, then the tile's sorted keys
  uint32_t* srow = kst + TILE;
  T* sv = reinterpret_cast<T*>(srow + TILE);
  const i64 t0 = (i64)blockIdx.x * TILE;
  const int cnt = (int)(n - t0 < TILE ? n - t0 : TILE);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned b4 = (unsigned)((cnt * 4 + 15) & ~15), bv = (unsigned)((cnt * (int)sizeof(T) + 15) & ~15);
    const uint64_t pol = policy_evict_first();
    mbar_arrive_expect_tx(&bar, 2 * b4 + bv);
    bulk_g2s(kst, kin + t0, b4, &bar, pol);
    bulk_g2s(srow, rin + t0, b4, &bar, pol);
    bulk_g2s(sv, vin + t0, bv, &bar, pol);
  }
  const bool ok = mbar_wait_bounded(&bar, 0, err, limit);
  if (!__syncthreads_and(ok)) {
    if (ok) return;  // another warp gave up: its error bit is set
    mbar_wait_bounded(&bar, 0, nullptr, kCopyPolls);  // drain the copies in flight
    return;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t key[R];
  int rank[R];
  rs_rank_tile<R>(kst, t0, n, shift, key, rank, wcnt, dstart);  // ends with a barrier: kst is free
#pragma unroll
  for (int r = 0; r < R; r++) {
    if (rank[r] < 0) continue;
    const int d = (int)((key[r] >> shift) & 255u);
    const int lp = dstart[d] + wcnt[w][d] + rank[r];
    kst[lp] = key[r];
    spos[lp] = (uint16_t)(w * (R * 32) + r * 32 + lane);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += kRsThreads) {
    const uint32_t k = kst[i];
    const int s = spos[i];
    const int d = (int)((k >> shift) & 255u);
    const i64 pos = goff[(i64)d * nblocks + blockIdx.x] + (i - dstart[d]);
    kout[pos] = k;
    rout[pos] = srow[s];
    vout[pos] = sv[s];
  }
}

void radix_sort_pairs(fvg_ctx* c, uint32_t* keys, uint32_t* vals, i64 n, int bits) {
  if (n <= 1 || bits <= 0) return;
  i64 nb = (n + kRsTile - 1) / kRsTile;
  DBuf k2, v2, hist, goff;
  k2.alloc(sizeof(uint32_t) * n, c->stream);
  v2.alloc(sizeof(uint32_t) * n, c->stream);
  hist.alloc(sizeof(i64) * 256 * nb, c->stream);
  goff.alloc(sizeof(i64) * (256 * nb + 1), c->stream);
  uint32_t *ka = keys, *va = vals, *kb = k2.as<uint32_t>(), *vb = v2.as<uint32_t>();
  int passes = 0;
  for (int shift = 0; shift < bits; shift += 8, passes++) {
    k_rs_upsweep<kRsRounds><<<(unsigned)nb, kRsThreads, 0, c->stream>>>(ka, n, shift, nb, hist.as<i64>());
    check_launch("rs_upsweep");
    scan_i64(c, hist.as<i64>(), goff.as<i64>(), 256 * nb);
    k_rs_downsweep<<<(unsigned)nb, kRsThreads, 0, c->stream>>>(ka, va, kb, vb, n, shift, nb, goff.as<i64>());
    check_launch("rs_downsweep");
    count_launch(c, 2);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (passes & 1) {
    FVG_CUDA(cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
    FVG_CUDA(cudaMemcpyAsync(vals, va, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, c->stream));
  }
}

// Stable sort of (key, row, value) triples by the low `bits` bits of the
// key, from (kin, rin, vin) into (kout, rout, vout); the inputs are not
// changed.  All six arrays hold kRsPad elements past n (the tiles are staged
// with 16-byte bulk copies).  Passes alternate between the outputs and one set of temporaries,
// starting on the side that makes the last pass write the outputs.
template <class T>
void radix_sort_rowval(fvg_ctx* c, const uint32_t* kin, const uint32_t* rin, const T* vin, uint32_t* kout,
                       uint32_t* rout, T* vout, i64 n, int bits) {
  if (n <= 0) return;
  // the tiles are staged by bulk copies, which need 16-byte aligned sources
  // (tile starts are multiples of 16 bytes from each array's base)
  if (((uintptr_t)kin | (uintptr_t)rin | (uintptr_t)vin | (uintptr_t)kout | (uintptr_t)rout | (uintptr_t)vout) & 15u)
    fail(FVG_ERR_INTERNAL, "radix sort arrays must be 16-byte aligned");
  const int passes = std::max(1, (bits + 7) / 8);
  const i64 nb = (n + kRsTileRv - 1) / kRsTileRv;
  const int dyn = (int)((2 * sizeof(uint32_t) + sizeof(T)) * kRsTileRv);
  FVG_CUDA(cudaFuncSetAttribute(k_rs_downsweep_rv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  DBuf kt, rt, vt, hist, goff;
  if (passes > 1) {  // padded: the staging copies read up to 15 bytes past n
    kt.alloc(sizeof(uint32_t) * (n + kRsPad), c->stream);
    rt.alloc(sizeof(uint32_t) * (n + kRsPad), c->stream);
    vt.alloc(sizeof(T) * (n + kRsPad), c->stream);
  }
  hist.alloc(sizeof(i64) * 256 * nb, c->stream);
  goff.alloc(sizeof(i64) * (256 * nb + 1), c->stream);
  const uint32_t *ks = kin, *rs = rin;
  const T* vs = vin;
  for (int p = 0; p < passes; p++) {
    const bool to_out = ((passes - 1 - p) & 1) == 0;
    uint32_t* kd = to_out ? kout : kt.as<uint32_t>();
    uint32_t* rd = to_out ? rout : rt.as<uint32_t>();
    T* vd = to_out ? vout : vt.as<T>();
    const int shift = 8 * p;
    k_rs_upsweep<kRsRoundsRv><<<(unsigned)nb, kRsThreads, 0, c->stream>>>(ks, n, shift, nb, hist.as<i64>());
    check_launch("rs_upsweep");
    scan_i64(c, hist.as<i64>(), goff.as<i64>(), 256 * nb);
    k_rs_downsweep_rv<T><<<(unsigned)nb, kRsThreads, dyn, c->stream>>>(ks, rs, vs, kd, rd, vd, n, shift, nb,
                                                                      goff.as<i64>(), c->dev_err, copy_polls(c));
    check_launch("rs_downsweep_rv");
    count_launch(c, 2);
    ks = kd;
    rs = rd;
    vs = vd;
  }
}
template void radix_sort_rowval<double>(fvg_ctx*, const uint32_t*, const uint32_t*, const double*, uint32_t*,
                                        uint32_t*, double*, i64, int);
template void radix_sort_rowval<float>(fvg_ctx*, const uint32_t*, const uint32_t*, const float*, uint32_t*,
                                       uint32_t*, float*, i64, int);
template void radix_sort_rowval<bf16>(fvg_ctx*, const uint32_t*, const uint32_t*, const bf16*, uint32_t*,
                                      uint32_t*, bf16*, i64, int);

// ------------------------------------------------------- element kernels
__global__ void k_fill_i32(i32* p, i32 v, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) p[i] = v;
}

static unsigned grid_for(i64 n, int threads = 256) {
  i64 g = (n + threads - 1) / threads;
  if (g > 152 * 32) g = 152 * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

void fill_i32(fvg_ctx* c, i32* p, i32 v, i64 n) {
  if (n <= 0) return;
  k_fill_i32<<<grid_for(n), 256, 0, c->stream>>>(p, v, n);
  check_launch("fill_i32");
  count_launch(c);
}

template <class S, class D> __device__ __forceinline__ D cvt(S s);
template <> __device__ __forceinline__ double cvt<double, double>(double s) { return s; }
template <> __device__ __forceinline__ float cvt<double, float>(double s) { return (float)s; }
template <> __device__ __forceinline__ bf16 cvt<double, bf16>(double s) { return __double2bfloat16(s); }
template <> __device__ __forceinline__ double cvt<float, double>(float s) { return (double)s; }
template <> __device__ __forceinline__ float cvt<float, float>(float s) { return s; }
template <> __device__ __forceinline__ bf16 cvt<float, bf16>(float s) { return __float2bfloat16_rn(s); }
template <> __device__ __forceinline__ double cvt<bf16, double>(bf16 s) { return (double)__bfloat162float(s); }
template <> __device__ __forceinline__ float cvt<bf16, float>(bf16 s) { return __bfloat162float(s); }
template <> __device__ __forceinline__ bf16 cvt<bf16, bf16>(bf16 s) { return s; }

template <class S, class D> __global__ void k_convert(const S* __restrict__ s, D* __restrict__ d, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    d[i] = cvt<S, D>(s[i]);
}

template <class S> static void convert_from(fvg_ctx* c, const S* s, void* d, int ddt, i64 n) {
  unsigned g = grid_for(n);
  if (ddt == FVG_F64) k_convert<S, double><<<g, 256, 0, c->stream>>>(s, (double*)d, n);
  else if (ddt == FVG_F32) k_convert<S, float><<<g, 256, 0, c->stream>>>(s, (float*)d, n);
  else k_convert<S, bf16><<<g, 256, 0, c->stream>>>(s, (bf16*)d, n);
}

void convert_values(fvg_ctx* c, const void* src, int sdt, void* dst, int ddt, i64 n) {
  if (n <= 0) return;
  if (sdt == FVG_F64) convert_from(c, (const double*)src, dst, ddt, n);
  else if (sdt == FVG_F32) convert_from(c, (const float*)src, dst, ddt, n);
  else convert_from(c, (const bf16*)src, dst, ddt, n);
  check_launch("convert_values");
  count_launch(c);
}

template <class T>
__global__ void k_gather(const T* __restrict__ s, const uint32_t* __restrict__ perm, T* __restrict__ d, i64 n) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
    d[i] = s[perm[i]];
}

void gather_values(fvg_ctx* c, const void* src, const uint32_t* perm, void* dst, int dt, i64 n) {
  if (n <= 0) return;
  unsigned g = grid_for(n);
  if (dt == FVG_F64) k_gather<double><<<g, 256, 0, c->stream>>>((const double*)src, perm, (double*)dst, n);
  else if (dt == FVG_F32) k_gather<float><<<g, 256, 0, c->stream>>>((const float*)src, perm, (float*)dst, n);
  else k_gather<bf16><<<g, 256, 0, c->stream>>>((const bf16*)src, perm, (bf16*)dst, n);
  check_launch("gather_values");
  count_launch(c);
}

}  // namespace fvg
