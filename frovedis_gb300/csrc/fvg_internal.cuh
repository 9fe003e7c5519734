// Internal declarations shared by the CUDA translation units of libfvg.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fvg.h"

namespace fvg {

using i64 = int64_t;
using i32 = int32_t;
using bf16 = __nv_bfloat16;

// ------------------------------------------------------------------ errors
struct Error {
  fvg_status code;
  std::string msg;
};
[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);
[[noreturn]] inline void fail(fvg_status code, const std::string& msg) { throw Error{code, msg}; }
#define FVG_CUDA(x)                                                  \
  do {                                                               \
    cudaError_t e__ = (x);                                           \
    if (e__ != cudaSuccess) ::fvg::throw_cuda(e__, #x, __FILE__, __LINE__); \
  } while (0)

// ---------------------------------------------------------- device buffers
// Owning device allocation, stream-ordered free.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept { *this = std::move(o); }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; bytes = o.bytes; stream = o.stream;
      o.p = nullptr; o.bytes = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t nbytes, cudaStream_t s);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Elements of padding after every value/index array, so that 16-byte vector
// loads of the last partial vector stay inside the allocation.
constexpr i64 kPad = 32;

// ---------------------------------------------------------- CRS schedule
// The CRS kernel walks the matrix in row order as a list of warp work items
// of at most `tile` nonzeros each:
//  * a row tile: consecutive short rows (each <= tile nonzeros, at most
//    kTileRows rows), and
//  * a piece of a long row (> tile nonzeros): rows are split into pieces at
//    8-element boundaries; the finalize kernel adds the pieces' partial sums
//    in piece order.
// An item's nonzeros are contiguous, so a warp reads them with coalesced
// 16-byte vector loads.
constexpr int kThreads = 256;
constexpr int kTileRows = 248;  // rows per tile (their offsets are staged in shared memory)
constexpr int kLaneWork = 32;   // products one lane may sum for one row in a tile
// Rows one thread of the work-item packer walks in order (a tile never spans
// two such chunks): short enough that the packers' sequential walks take a
// fraction of a millisecond, long enough to fill kTileRows-row tiles.  The
// panel and head layouts' rows are shorter (their items hold more rows), so
// they are packed in longer chunks.
constexpr i64 kPackRows = 256;
constexpr i64 kPanelPackRows = 1024;
// Lanes per row when a warp sums a tile of R rows: 32 / R rounded to a power
// of two; tiles of 32 or more rows take rounds of 32 rows, one lane each.
__host__ __device__ __forceinline__ int lanes_per_row(int R) {
  if (R >= 32) return 1;
  int p2 = 1;
  while (p2 < R) p2 <<= 1;
  return 32 / p2;
}
struct Item {
  int32_t r0;  // first row (tile) or the long row (piece)
  int32_t r1;  // one past the last row (tile), or -1 - piece index (piece)
  int32_t e0;  // first nonzero
  int32_t e1;  // one past the last nonzero
};
struct Sched {
  int tile = 0;                // nonzeros per item
  i64 nitems = 0;
  DBuf items;                  // Item[nitems] in row order
  i64 nlong = 0, npieces = 0;
  DBuf long_rows;              // int32 [nlong]
  DBuf long_piece0;            // int32 [nlong+1] first piece of each long row
};
// Tuning knobs of the CRS kernel (compile-time; defaults from measurements
// on GB300): nonzeros per warp item, resident CTAs per SM the register
// budget targets, element rounds whose loads are issued together.
#ifndef FVG_WARP_TILE
#define FVG_WARP_TILE 512
#endif
#ifndef FVG_CRS_MIN_BLOCKS
#define FVG_CRS_MIN_BLOCKS 4
#endif
#ifndef FVG_CRS_ROUNDS
#define FVG_CRS_ROUNDS 8
#endif
constexpr int kWarpTile = FVG_WARP_TILE;  // nonzeros per warp item
inline int tile_for_storage(int) { return kWarpTile; }

// Device CRS matrix with up to three value planes.
struct DevCRS {
  i64 m = 0, n = 0, nnz = 0;
  DBuf off, idx;  // int32
  DBuf val[3];    // indexed by fvg_dtype
  DBuf lo;        // bf16 [nnz+kPad]: value - FP32 value (split storage; with val[FVG_F32])
  std::unique_ptr<Sched> sched[2];  // work items: slot 0 kWarpTile, slot 1 the split kernel's size
  std::unique_ptr<Sched> slab_sched;  // long rows in slab-ordered pieces (crs_sched_slabs)
  i64 slab_rows = 0;
  i64 max_row = 0;
};

struct DevELL {  // column-major m x width, zero padded (ell_matrix.hpp:63-95)
  i64 m = 0, n = 0, width = 0;
  DBuf idx;
  DBuf val[3];
};

struct DevJDS {  // jds_matrix_local (jds_matrix.hpp:15-146)
  i64 m = 0, n = 0, ndiag = 0, nnz = 0;
  DBuf perm;     // int32 [m]
  DBuf off;      // int64 [ndiag+1]
  DBuf idx;      // int32 [nnz]
  DBuf val[3];
  bool empty_perm = false;  // all-zero matrix: the reference leaves perm empty
  // Work items of the product (JdsItem): a warp per block of 32 permuted rows
  // and at most kJdsSeg diagonals; blocks with more diagonals are cut into
  // several items whose per-row partials (nslots x 32 accumulators) are added
  // in diagonal order by the split blocks' finalize (JdsSplit).
  DBuf items, splits;
  i64 nitems = 0, nsplits = 0, nslots = 0;
};
constexpr i64 kJdsSeg = 128;
struct JdsItem {
  int32_t b;     // row block: permuted rows 32b .. 32b+31
  int32_t d0;    // diagonals [d0, d1)
  int32_t d1;
  int32_t slot;  // partial slot, -1: the item covers the whole block
};
struct JdsSplit {
  int32_t b, slot0, nslot, pad;
};

struct DevHYB {  // jds_crs_hybrid_local (jds_crs_hybrid.hpp:8-153)
  i64 m = 0, n = 0, crs_rows = 0;
  DevJDS jds;
  DevCRS crs;  // tail rows, in permuted order (row i ↔ jds.perm[i])
  bool all_crs = false;  // m <= threshold: the whole matrix is the CRS part
};

// Work items over a panel layout's rows, panel by panel (Item as in Sched):
// a panel's items start at pitem0[panel], its long rows at plong0[panel].
struct PanelItems {
  int tile = 0;
  i64 nitems = 0, nlong = 0, npieces = 0;
  DBuf items, pitem0, long_rows, plong0, long_piece0;
};

// Row-panel layout of the backward product g = A^T r (FP32 arithmetic).
// A's rows are cut into panels of `rows` consecutive rows; a CTA stages one
// panel's slice of r in shared memory and sums, for every hot column h, the
// products of the column's entries that fall in the panel ("panel row"
// q = panel * nhot + h, local row ids as uint16).  Hot columns are those with
// at least `min_per_panel` entries per panel on average; the other columns
// keep their rows in `cold`, the transposed CRS with the hot rows emptied,
// whose product gathers r from L2 as before.  g[hot] is the fixed-order sum
// of the panels' partial sums.
struct DevPanels {
  i64 m = 0, n = 0;                 // A: m rows (cut into panels), n columns
  i64 rows = 0, npanels = 0, nhot = 0, E = 0;
  double min_per_panel = 0.0;
  int master = FVG_F64;
  DBuf hot_cols;                    // int32 [nhot], ascending
  DBuf poff;                        // int32 [npanels*nhot + 1]
  DBuf prow;                        // uint16 [E + kPad]: row within the panel
  DBuf val[3];                      // [E + kPad] per dtype
  DBuf lo;                          // bf16 [E + kPad]: residual of the FP32 values (split storage)
  DevCRS cold;                      // n rows, hot rows empty
  // work items over the panel rows, panel by panel (Item as in Sched)
  i64 nitems = 0, nlong = 0, npieces = 0;
  DBuf items, pitem0, long_rows, plong0, long_piece0;
  DBuf ypan;                        // float [npanels*nhot]
  DBuf partials;                    // float [npieces]
  // split storage: its own work items (smaller staging buffers) and df-pair
  // partial sums (float2)
  std::unique_ptr<PanelItems> split_items;
  DBuf ypan2, partials2;
  // forward head (shared = true): every CTA stages w at the columns
  // hot_cols[0..rows) once; panels are stretches of nhot rows of A; `cold`
  // holds the rest of each row (m rows, int32 column ids)
  bool shared = false;
};
// Work items of a CRS packed on the device, in chunks of `chunk` rows
// (items never span chunks): counts per chunk, their exclusive scans
// (`base`: items, long rows, pieces, each np+1 entries), the items, the long
// rows and the first piece of each long row (nlong+1 entries).
struct PackOut {
  i64 nitems = 0, nlong = 0, npieces = 0;
  DBuf items, long_rows, long_piece0;
  std::vector<i32> base;
};
// Each chunk may itself be packed in `sub` pieces (a warp each; items never
// span two pieces); base then has nchunks*sub+1 entries per kind.
void device_pack(fvg_ctx* c, const i32* off, i64 nrows, i64 chunk, i64 nchunks, int tile, PackOut& o, i64 sub = 1);

struct Profiler;

}  // namespace fvg

struct fvg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  int num_sms = 0;
  int grid_spmv = 0;    // persistent grid of the CRS kernel
  int64_t launches = 0;
  bool profiling = false;
  fvg::Profiler* prof = nullptr;  // owned; prof_create / prof_destroy
  // live matrices: destroying the context releases their device memory
  std::vector<fvg_matrix*> matrices;
  // device error word: a kernel that must give up (a bounded wait that ran
  // out) sets a bit here instead of trapping; read after each call
  unsigned* dev_err = nullptr;
  // poll budget of the bounded device-side waits (< 0: the defaults below)
  int64_t wait_limit = -1;
  // batched trainers: evaluations run (the line-search trials that had a
  // model searching, initial and precision-switch evaluations) and the
  // (dataset, model) evaluations inside them, since the context was made
  int64_t batch_evals = 0, batch_model_evals = 0;
};

struct fvg_matrix {
  fvg_ctx* ctx = nullptr;
  int master = FVG_F64;           // dtype of the uploaded values
  fvg::DevCRS A;
  std::unique_ptr<fvg::DevCRS> AT;
  std::unique_ptr<fvg::DevELL> ell;
  std::unique_ptr<fvg::DevJDS> jds, tjds;
  std::unique_ptr<fvg::DevHYB> hyb, thyb;
  std::vector<double> labels;  // libsvm loads: one label per row
  bool has_labels = false;
  // row-panel layout of A^T r: built on demand; panel_rows < 0 picks the
  // layout from the matrix, 0 turns it off, > 0 forces that panel height
  std::unique_ptr<fvg::DevPanels> pan;
  bool pan_tried = false;
  int64_t panel_rows = -1;
  double panel_min = -1.0;
  // forward head of A (frequent columns staged in shared memory): built on
  // demand; head_cols < 0 picks it from the matrix, 0 turns it off, > 0
  // forces that many columns
  std::unique_ptr<fvg::DevPanels> head;
  bool head_tried = false;
  int64_t head_cols = -1;
};

namespace fvg {

// ------------------------------------------------------------ profiling
enum ProfKey { P_SPMV_CRS = 0, P_PASS1, P_PASS2, P_FINALIZE, P_LBFGS, P_TRANSPOSE, P_SPMV_ELL, P_SPMV_JDS,
               P_SPMV_HYB, P_SPMM, P_PASS1_F32, P_PASS2_F32, P_BATCH_PASS1, P_BATCH_PASS2, P_PANEL_BUILD,
               P_HEAD_BUILD, P_SCHED, P_NKEYS };
void prof_begin(fvg_ctx* c, int key);
void prof_end(fvg_ctx* c, int key);
void prof_collect(fvg_ctx* c, int key, double* ms, int64_t* n);
void prof_reset(fvg_ctx* c);
void prof_create(fvg_ctx* c);
void prof_destroy(fvg_ctx* c);
struct ProfScope {
  fvg_ctx* c;
  int k;
  ProfScope(fvg_ctx* c_, int k_) : c(c_), k(k_) { prof_begin(c, k); }
  ~ProfScope() { prof_end(c, k); }
};
inline void count_launch(fvg_ctx* c, int n = 1) { c->launches += n; }
void check_launch(const char* what);
// Default poll budgets of the bounded device-side waits: the L-BFGS
// direction's grid barriers (2^24 polls of ~32 ns) and the panel kernels'
// bulk-copy waits (2^16 polls, each a sleep of at most 20 us in the
// barrier: ~1.3 s); a context may lower them for testing.
constexpr unsigned kBarrierPolls = 1u << 24;
constexpr unsigned kCopyPolls = 1u << 16;
inline unsigned barrier_polls(const fvg_ctx* c) { return c->wait_limit < 0 ? kBarrierPolls : (unsigned)c->wait_limit; }
inline unsigned copy_polls(const fvg_ctx* c) { return c->wait_limit < 0 ? kCopyPolls : (unsigned)c->wait_limit; }
// Reads (and clears) the device error word; fails when a kernel reported one.
void check_device_error(fvg_ctx* c);

// ------------------------------------------------------------ utilities
int dtype_size(int dt);
void inject_alloc_failure(long long after);
// resident CTAs per SM of `kernel` on the current device (cached per device)
int occupancy_blocks(const void* kernel, int threads, size_t dyn_smem = 0);
// exclusive scan of n int64 values in place (out has n+1 entries: out[n]=total)
void scan_i64(fvg_ctx* c, const i64* in, i64* out, i64 n);
// stable LSD radix sort of (key,val) u32 pairs by the low `bits` bits of key
void radix_sort_pairs(fvg_ctx* c, uint32_t* keys, uint32_t* vals, i64 n, int bits);
// stable sort of (key, row, value) by key; every array padded by kRsPad elements
constexpr i64 kRsPad = 16;
static_assert(kPad >= kRsPad, "CRS arrays carry the sort's padding");
template <class T>
void radix_sort_rowval(fvg_ctx* c, const uint32_t* kin, const uint32_t* rin, const T* vin, uint32_t* kout,
                       uint32_t* rout, T* vout, i64 n, int bits);
void fill_i32(fvg_ctx* c, i32* p, i32 v, i64 n);
void convert_values(fvg_ctx* c, const void* src, int sdt, void* dst, int ddt, i64 n);
void gather_values(fvg_ctx* c, const void* src, const uint32_t* perm, void* dst, int dt, i64 n);

// ------------------------------------------------------------ builders
void crs_upload(fvg_ctx* c, DevCRS& a, i64 m, i64 n, const i32* off, const i32* idx, const void* val, int dt,
                bool on_device);
void crs_ensure_plane(fvg_ctx* c, DevCRS& a, int dt, int master);
void crs_build_transpose(fvg_ctx* c, const DevCRS& a, DevCRS& t, int master);
const Sched& crs_sched(fvg_ctx* c, DevCRS& a, int tile);
// The rows longer than a tile cut into pieces also at every slab of `slab`
// column ids, the pieces listed slab by slab before the tiles (cached).
const Sched& crs_sched_slabs(fvg_ctx* c, DevCRS& a, int tile, i64 slab);
void ell_build(fvg_ctx* c, const DevCRS& a, DevELL& e, int master);
void jds_build(fvg_ctx* c, const DevCRS& a, DevJDS& j, int master);
void hyb_build(fvg_ctx* c, const DevCRS& a, DevHYB& h, int master, i64 threshold);
void ensure_plane_generic(fvg_ctx* c, DBuf* planes, i64 n, int dt, int master);

// ------------------------------------------------------------ products
// Epilogue of a CRS pass.
enum EpiKind { EPI_STORE = 0, EPI_LOGREG = 1 };
struct LogregEpi {
  const double* label = nullptr;
  const double* sw = nullptr;       // nullptr: all ones
  const float* label_f = nullptr;   // FP32 copies used by the FP32-arithmetic path
  const float* sw_f = nullptr;
  const double* intercept = nullptr;  // device scalar
  int icpt = 0;
  void* r = nullptr;                // dloss*sw, dtype r_dt
  int r_dt = FVG_F64;
  double* cta_part = nullptr;       // [2*grid]: loss, bias per CTA
  double* long_part = nullptr;      // [2*nlong]
  double* out = nullptr;            // [2]: loss, bias  (written by finalize)
  double* grad_bias = nullptr;      // where the bias lands (grad[n]); may be null
  unsigned* ticket = nullptr;
  int loss = 0;                     // GLM loss kind (0 logistic .. 4 squared eps-insensitive)
  double eps = 0.0;                 // epsilon of the eps-insensitive kinds
  const float* ybase = nullptr;     // FP32 path: per-row partial products added before the epilogue
};
// y = A x over the CRS layout (any plane), optional logistic epilogue.
void crs_pass(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* x, int y_dt, void* y, int epi,
              const LogregEpi* lr, void* scratch_partials, int prof_key);
i64 crs_pass_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage);
void ell_spmv(fvg_ctx* c, DevELL& e, int storage, int x_dt, const void* x, int y_dt, void* y);
void jds_spmv(fvg_ctx* c, DevJDS& j, int storage, int x_dt, const void* x, int y_dt, void* y, bool accumulate_perm);
void hyb_spmv(fvg_ctx* c, DevHYB& h, int storage, int x_dt, const void* x, int y_dt, void* y);
void crs_spmm(fvg_ctx* c, DevCRS& a, int storage, int x_dt, const void* X, i64 k, void* Y);
// One block of at most 64 columns (X, Y already offset to the block's first
// column; ldx / ldy row strides); scratch of spmm_scratch_bytes().
// slab > 0: the schedule of crs_sched_slabs (long rows in pieces listed by
// slabs of `slab` rows of X, for X larger than L2); the scratch must be sized
// with the same slab.
i64 spmm_scratch_bytes(fvg_ctx* c, DevCRS& a, int storage, i64 slab = 0);
void crs_spmm_block(fvg_ctx* c, DevCRS& a, int storage, const void* X, i64 ldx, int kb, int y_dt, void* Y, i64 ldy,
                    void* scratch, const int* gate = nullptr, i64 slab = 0);
void crs_spmm_logreg_block(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int kb, const double* label,
                           const double* sw, const float* label_f, const float* sw_f, int icpt, const double* bias,
                           void* R, i64 ldr, double* out, double* gbias, void* scratch, int loss = 0,
                           double eps = 0.0);
// Logistic forward pass over datasets stacked block-diagonally in one CRS
// (rows of dataset d: [seg_row[d], seg_row[d+1])): per-dataset intercepts
// (bias + d * ldb) and loss / bias sums, out[2 * (d * ldo + j)] and
// out[2 * (d * ldo + j) + 1]; the bias sums also land in gb[grow[d] * ldg +
// j] (crs_spmm_seg_finish).  W (32-byte aligned for FP32) and R 16-byte
// aligned, kb and the strides multiples of 8.  The whole pass does nothing while *gate == 0
// (gate may be null).
struct SpmmSeg {
  int nseg = 0;
  const i32* seg_row = nullptr;  // device [nseg + 1]
  i64 ldb = 0;
  double* slots = nullptr;       // device scratch, spmm_seg_slot_bytes()
  int kout = 0;                  // models of this block with results
  double* out = nullptr;
  i64 ldo = 0;
  double* gb = nullptr;
  const i64* grow = nullptr;     // device [nseg]
  i64 ldg = 0;
  const int* gate = nullptr;
  // column masks (null: all): bit j of mask[d * mstride + mword] set =
  // column j of the block is computed for dataset d; masked outputs keep
  // their contents (kb <= 64)
  const unsigned long long* mask = nullptr;
  i64 mstride = 0;
  int mword = 0;
  // set by the pass for crs_spmm_seg_finish
  i64 nw1 = 0, nw2 = 0;
  int nc = 0, icpt = 0;
};
i64 spmm_seg_slot_bytes(fvg_ctx* c, int nseg, int kb);
void crs_spmm_logreg_seg(fvg_ctx* c, DevCRS& a, int storage, const void* W, i64 ldw, int kb, const double* label,
                         const double* sw, const float* label_f, const float* sw_f, int icpt, const double* bias,
                         void* R, i64 ldr, void* scratch, SpmmSeg& sg, int loss = 0, double eps = 0.0);
// The per-dataset sums of the pass (launch after the backward product).
void crs_spmm_seg_finish(fvg_ctx* c, const SpmmSeg& sg);
// Y = A X (FP64 Y) over stacked datasets with sg's row bounds, masks, gate
// (the same alignment as crs_spmm_logreg_seg).
void crs_spmm_store_seg(fvg_ctx* c, DevCRS& a, int storage, const void* X, i64 ldx, int kb, void* Y, i64 ldy,
                        void* scratch, SpmmSeg& sg, i64 slab = 0);

// Row-panel backward product (FP32/BF16 storage): builds the layout when the
// matrix's column counts make it pay (or as forced); returns null when the
// plain transposed CRS is used.
DevPanels* panels_for(fvg_ctx* c, fvg_matrix* M);
void panel_ensure_plane(fvg_ctx* c, DevPanels& pn, int dt);
i64 panel_scratch_bytes(fvg_ctx* c, DevPanels& pn, int storage);
// y[0..n) = A^T r for FP32 r; y FP64 or FP32.
void panel_trans_mv(fvg_ctx* c, DevPanels& pn, int storage, const float* r, int y_dt, void* y, void* scratch,
                    int prof_key);
// Forward head of A for the FP32/BF16 pass 1 (null when the plain CRS pass
// is used), and that pass: head partials, then the tail's CRS pass with the
// logistic epilogue over head + tail.
DevPanels* head_for(fvg_ctx* c, fvg_matrix* M);
void head_ensure_plane(fvg_ctx* c, DevPanels& hd, int dt);
i64 head_scratch_bytes(fvg_ctx* c, DevPanels& hd, int storage);
void head_logreg_pass(fvg_ctx* c, DevPanels& hd, int storage, const float* w, const LogregEpi& lr, void* scratch,
                      int prof_key);
// Split storage on the same layouts: g = A^T r (r df pairs, g FP64: hot
// columns from the panels, the rest from the cold CRS); the forward head's
// partial per row into hd.ypan2 and the tail's product into wtx (df pairs).
void panel_ensure_split(fvg_ctx* c, DevPanels& pn);
i64 panel_split_scratch_bytes(fvg_ctx* c, DevPanels& pn, bool y_df);
void panel_trans_mv_split(fvg_ctx* c, DevPanels& pn, const void* r, double* y, void* scratch);
void head_pass_split(fvg_ctx* c, DevPanels& hd, const void* w, void* wtx, void* scratch);

// ------------------------------------------------------- split storage
// FP64 values kept as an FP32 plane plus a BF16 residual plane, multiplied
// in double-FP32 arithmetic (split.cu).  Vectors are df pairs (float2).
void df64_init(fvg_ctx* c);  // the exp table of the df64 math, once per device
void crs_ensure_split(fvg_ctx* c, DevCRS& a, int master);
// lo = BF16(v - FP32 plane) for n values of planes[] (the FP64 and FP32 planes)
void split_residual_plane(fvg_ctx* c, const DBuf* planes, i64 n, int master, DBuf& lo);
void ensure_split_planes(fvg_ctx* c, DBuf* planes, i64 n, int master, DBuf& lo);
void split_vector(fvg_ctx* c, const double* x, void* y, i64 n);  // y: float2[n]
i64 crs_split_scratch_bytes(fvg_ctx* c, DevCRS& a, bool y_df);  // y_df: FP32-pair output (forward)
// y = A x, x float2 pairs; y FP64 (y_df false) or float2 pairs
void crs_pass_split(fvg_ctx* c, DevCRS& a, const void* x, bool y_df, void* y, void* scratch, int prof_key);
struct GlmSplitArgs {
  const void* lab = nullptr;  // float2[m]
  const void* sw = nullptr;   // float2[m] or null
  const double* intercept = nullptr;
  int icpt = 0;
  int kind = 0;
  double eps = 0.0;
  void* r = nullptr;          // float2[m]: dloss * sw
  double* cta_part = nullptr; // [2 * glm_split_grid(m)]
  unsigned* ticket = nullptr; // zero on entry, left zero
  double* out = nullptr;      // [2]: loss, bias
  double* grad_bias = nullptr;
};
int glm_split_grid(fvg_ctx* c, i64 m);
// per-row loss/gradient over z = wtx (+ head) + intercept (float2 pairs)
void glm_split_rows(fvg_ctx* c, const void* wtx, const void* head, i64 m, const GlmSplitArgs& e);

// The device L-BFGS loop over an evaluation: eval() evaluates the model whose
// n weights are w64 (device FP64) and whose intercept is *b (device) into the
// gradient g[0..n] (bias last) and out[0] = loss, out[1] = bias sum;
// refine() may switch the value precision after an iteration (the accepted
// model is then evaluated again).  eta_one: regularise with eta = 1 (ELL).
struct LbfgsEval {
  virtual void eval(const double* w64, const double* b, double* g, double* out) = 0;
  virtual bool refine(double rms) {
    (void)rms;
    return false;
  }
  virtual ~LbfgsEval() = default;
};
void lbfgs_core(fvg_ctx* c, i64 n, const fvg_glm_params* p, int eta_one, LbfgsEval& ev, double* w_h, double* b_h,
                i64* n_iter, double* loss_out);

// Times the candidate training layouts of a matrix and leaves the fastest set.
void autotune(fvg_ctx* c, fvg_matrix* M, int storage, const double* label_h, int reps,
              std::vector<fvg_tune_choice>& tried, fvg_tune_choice& best);

// Argument checks shared by the trainers (lbfgs_parallelizer.hpp:536-552).
void check_common(const fvg_glm_params* p, fvg_matrix* M, const double* label);

// Per-row logistic epilogue applied to a finished product z = A w (used by
// the non-CRS formats): r, loss/bias partial sums; then finalize_logreg.
void logreg_rows(fvg_ctx* c, const void* wtx, int wtx_dt, i64 m, const LogregEpi& lr);

}  // namespace fvg
