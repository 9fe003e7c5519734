// Loaders of the reference's on-disk CRS formats, parsed on the device.
//
//  * binary directory (make_crs_matrix_local_loadbinary, crs_matrix.hpp:
//    565-603): nums ("num_row num_col"), an optional type file ("valtype
//    idxtype offtype", checked against the requested types like
//    confirm_given_type_against_expected, core/utility.hpp:101-113), and the
//    val / idx / off arrays in native byte order.  The arrays are uploaded as
//    they are and the index / offset types converted on the device.
//  * text CRS (make_crs_matrix_local_load, crs_matrix.hpp:665-775): one row
//    per line, "col:value" pairs separated by white space, 0-based columns.
//  * libsvm (make_crs_matrix_local_loadlibsvm, crs_matrix.hpp:863-899): a
//    label, then "col:value" pairs; the column count is the largest id + 1
//    taken before the index-origin adjustment (AUTO: ids shift down by one
//    when the smallest is positive).
//
// Text parsing: the file's bytes are copied to the device once.  The
// newline and colon positions are compacted in order (per-chunk counts, a
// scan, per-chunk writes); each colon is one entry: its column id is read
// backwards from the colon and its value forwards.  Values use the exact
// fast path of decimal conversion (Clinger 1990): a significand below 2^53
// (2^24 for FP32) scaled by 10^e with |e| <= 22 (10) is one correctly
// rounded multiplication or division of exactly representable operands, so
// it equals strtod (strtof).  Other values (long significands, large
// exponents, inf/nan, hex) are listed and converted on the host with
// strtod / strtof, so every value is bit-identical to the reference's
// parse.  Lines must be well formed (only white space between tokens); any
// other character is an error instead of the reference's silent stop.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "fvg_internal.cuh"

namespace fvg {

constexpr int kLT = 256;         // threads per CTA
constexpr int kChunk = 16;       // bytes per thread in the compaction passes
constexpr int kBlockBytes = kLT * kChunk;

__device__ const double kPow10d[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                       1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
__device__ const float kPow10f[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};

__device__ __forceinline__ bool blank(char ch) {
  return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f';
}
__device__ __forceinline__ bool digit(char ch) { return ch >= '0' && ch <= '9'; }

// ---------------------------------------------------- position compaction
// counts of newlines and colons per CTA-sized chunk of the file
__global__ void __launch_bounds__(kLT) k_count_marks(const char* __restrict__ buf, i64 n, i64* __restrict__ nl_cnt,
                                                     i64* __restrict__ co_cnt) {
  __shared__ int snl[kLT], sco[kLT];
  const i64 base = (i64)blockIdx.x * kBlockBytes + (i64)threadIdx.x * kChunk;
  int a = 0, b = 0;
  for (int k = 0; k < kChunk; k++) {
    const i64 i = base + k;
    if (i < n) {
      const char ch = buf[i];
      a += ch == '\n';
      b += ch == ':';
    }
  }
  snl[threadIdx.x] = a;
  sco[threadIdx.x] = b;
  __syncthreads();
  for (int s = kLT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      snl[threadIdx.x] += snl[threadIdx.x + s];
      sco[threadIdx.x] += sco[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    nl_cnt[blockIdx.x] = snl[0];
    co_cnt[blockIdx.x] = sco[0];
  }
}

// positions of newlines and colons, in file order
__global__ void __launch_bounds__(kLT) k_write_marks(const char* __restrict__ buf, i64 n,
                                                     const i64* __restrict__ nl_base,
                                                     const i64* __restrict__ co_base, i64* __restrict__ nl_pos,
                                                     i64* __restrict__ co_pos) {
  __shared__ int snl[kLT], sco[kLT];
  const i64 base = (i64)blockIdx.x * kBlockBytes + (i64)threadIdx.x * kChunk;
  int a = 0, b = 0;
  for (int k = 0; k < kChunk; k++) {
    const i64 i = base + k;
    if (i < n) {
      const char ch = buf[i];
      a += ch == '\n';
      b += ch == ':';
    }
  }
  snl[threadIdx.x] = a;
  sco[threadIdx.x] = b;
  __syncthreads();
  // exclusive scan of the per-thread counts (Hillis-Steele on 256 values)
  for (int s = 1; s < kLT; s <<= 1) {
    const int x = threadIdx.x >= s ? snl[threadIdx.x - s] : 0;
    const int y = threadIdx.x >= s ? sco[threadIdx.x - s] : 0;
    __syncthreads();
    snl[threadIdx.x] += x;
    sco[threadIdx.x] += y;
    __syncthreads();
  }
  i64 pa = nl_base[blockIdx.x] + snl[threadIdx.x] - a;
  i64 pb = co_base[blockIdx.x] + sco[threadIdx.x] - b;
  for (int k = 0; k < kChunk; k++) {
    const i64 i = base + k;
    if (i < n) {
      const char ch = buf[i];
      if (ch == '\n') nl_pos[pa++] = i;
      if (ch == ':') co_pos[pb++] = i;
    }
  }
}

// ---------------------------------------------------------------- numbers
struct Num {
  double d;
  float f;
  int status;  // 0: parsed, 1: convert on the host, 2: malformed
  i64 start;   // first character of the number (after blanks)
  i64 end;     // one past the token
};

// A strtod / strtof token starting at or after `i` (leading blanks skipped),
// ending before `lim`.
__device__ Num parse_number(const char* __restrict__ buf, i64 i, i64 lim, bool want_float) {
  Num r{0.0, 0.0f, 2, i, i};
  while (i < lim && blank(buf[i])) i++;
  const i64 start = i;
  r.start = start;
  bool neg = false;
  if (i < lim && (buf[i] == '+' || buf[i] == '-')) {
    neg = buf[i] == '-';
    i++;
  }
  if (i < lim && !digit(buf[i]) && buf[i] != '.') {
    // inf / nan / anything strtod may still take: decided on the host
    i64 j = i;
    while (j < lim && !blank(buf[j]) && buf[j] != '\n') j++;
    r.status = (j > i) ? 1 : 2;
    r.end = j;
    return r;
  }
  if (i + 1 < lim && buf[i] == '0' && (buf[i + 1] == 'x' || buf[i + 1] == 'X')) {  // hex float: host
    i64 j = i;
    while (j < lim && !blank(buf[j]) && buf[j] != '\n') j++;
    r.status = 1;
    r.end = j;
    return r;
  }
  unsigned long long w = 0;
  int nd = 0, e10 = 0;
  bool any = false, truncated = false;
  for (; i < lim && digit(buf[i]); i++) {
    any = true;
    const int dv = buf[i] - '0';
    if (w == 0 && dv == 0) continue;
    if (nd < 19) {
      w = w * 10 + dv;
      nd++;
    } else {
      e10++;
      truncated |= dv != 0;
    }
  }
  if (i < lim && buf[i] == '.') {
    i++;
    for (; i < lim && digit(buf[i]); i++) {
      any = true;
      const int dv = buf[i] - '0';
      if (w == 0 && dv == 0) {
        e10--;
        continue;
      }
      if (nd < 19) {
        w = w * 10 + dv;
        nd++;
        e10--;
      } else {
        truncated |= dv != 0;
      }
    }
  }
  if (any && i < lim && (buf[i] == 'e' || buf[i] == 'E')) {
    i64 j = i + 1;
    bool eneg = false;
    if (j < lim && (buf[j] == '+' || buf[j] == '-')) {
      eneg = buf[j] == '-';
      j++;
    }
    if (j < lim && digit(buf[j])) {
      int ex = 0;
      for (; j < lim && digit(buf[j]); j++) ex = min(ex * 10 + (buf[j] - '0'), 100000);
      e10 += eneg ? -ex : ex;
      i = j;
    }
  }
  r.end = i;
  if (!any) return r;  // malformed
  if (truncated) {
    r.status = 1;
    return r;
  }
  r.status = 0;
  if (w == 0) {
    r.d = neg ? -0.0 : 0.0;
    r.f = neg ? -0.0f : 0.0f;
    return r;
  }
  if (want_float) {
    if (w <= (1ull << 24) && e10 >= -10 && e10 <= 10) {
      float v = (float)w;
      v = e10 >= 0 ? __fmul_rn(v, kPow10f[e10]) : __fdiv_rn(v, kPow10f[-e10]);
      r.f = neg ? -v : v;
      return r;
    }
  } else if (w <= (1ull << 53) && e10 >= -22 && e10 <= 22) {
    double v = (double)w;
    v = e10 >= 0 ? __dmul_rn(v, kPow10d[e10]) : __ddiv_rn(v, kPow10d[-e10]);
    r.d = neg ? -v : v;
    return r;
  }
  r.status = 1;
  return r;
}

struct LineInfo {
  const i64* nl_pos;
  i64 nnl;
  i64 nbytes;
  __device__ __forceinline__ i64 start(i64 r) const { return r == 0 ? 0 : nl_pos[r - 1] + 1; }
  __device__ __forceinline__ i64 end(i64 r) const { return r < nnl ? nl_pos[r] : nbytes; }
  // line holding byte position p: number of newlines before p
  __device__ __forceinline__ i64 line_of(i64 p) const {
    i64 lo = 0, hi = nnl;  // first newline position >= p
    while (lo < hi) {
      const i64 mid = (lo + hi) >> 1;
      if (nl_pos[mid] < p) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  }
};

struct EntryOut {
  i64* row;          // line of each entry
  int64_t* col;      // column id as written
  void* val;         // FP64 or FP32
  int want_float;
  unsigned char* covered;
  unsigned* nslow;   // entries / labels converted on the host
  i64* slow;         // (entry or -1 - line, token start, token end)
  i64 slow_cap;
  unsigned* bad;     // malformed token seen
};

__device__ __forceinline__ void put_slow(const EntryOut& o, i64 who, i64 start, i64 end) {
  const unsigned k = atomicAdd(o.nslow, 1u);
  if ((i64)k < o.slow_cap) {
    o.slow[3 * k] = who;
    o.slow[3 * k + 1] = start;
    o.slow[3 * k + 2] = end;
  }
}

__device__ __forceinline__ void cover(const EntryOut& o, i64 a, i64 b) {
  for (i64 i = a; i < b; i++) o.covered[i] = 1;
}

// one entry per colon: "col:value"
__global__ void __launch_bounds__(kLT) k_parse_entries(const char* __restrict__ buf, LineInfo L,
                                                       const i64* __restrict__ co_pos, i64 ne, EntryOut o) {
  for (i64 e = (i64)blockIdx.x * kLT + threadIdx.x; e < ne; e += (i64)gridDim.x * kLT) {
    const i64 p = co_pos[e];
    const i64 r = L.line_of(p);
    const i64 ls = L.start(r), le = L.end(r);
    o.row[e] = r;
    // column id: digits right before the colon, an optional sign, then a
    // blank or the line start
    i64 b = p;
    while (b > ls && digit(buf[b - 1])) b--;
    bool ok = b < p;
    long long col = 0;
    for (i64 i = b; i < p && ok; i++) col = min(col * 10 + (buf[i] - '0'), 1ll << 40);
    if (b > ls && (buf[b - 1] == '+' || buf[b - 1] == '-')) {
      if (buf[b - 1] == '-') col = -col;
      b--;
    }
    if (b > ls && !blank(buf[b - 1])) ok = false;
    o.col[e] = col;
    const Num v = parse_number(buf, p + 1, le, o.want_float != 0);
    if (v.status == 2 || (v.end < le && !blank(buf[v.end]))) ok = false;
    if (!ok) {
      atomicOr(o.bad, 1u);
      continue;
    }
    if (v.status == 1) put_slow(o, e, v.start, v.end);
    else if (o.want_float) ((float*)o.val)[e] = v.f;
    else ((double*)o.val)[e] = v.d;
    cover(o, b, v.end);
  }
}

// libsvm: the label at the start of each line (strtox on the line; an empty
// line gives 0)
__global__ void __launch_bounds__(kLT) k_parse_labels(const char* __restrict__ buf, LineInfo L, i64 nlines,
                                                      double* __restrict__ label, EntryOut o) {
  for (i64 r = (i64)blockIdx.x * kLT + threadIdx.x; r < nlines; r += (i64)gridDim.x * kLT) {
    const i64 ls = L.start(r), le = L.end(r);
    i64 i = ls;
    while (i < le && blank(buf[i])) i++;
    if (i == le) {
      label[r] = 0.0;
      continue;
    }
    const Num v = parse_number(buf, i, le, false);
    if (v.status == 2 || (v.end < le && !blank(buf[v.end]))) {
      atomicOr(o.bad, 1u);
      continue;
    }
    if (v.status == 1) put_slow(o, -1 - r, v.start, v.end);
    else label[r] = v.d;
    cover(o, i, v.end);
  }
}

// every byte is white space, a newline or part of a parsed token
__global__ void k_check_cover(const char* __restrict__ buf, i64 n, const unsigned char* __restrict__ covered,
                              unsigned* bad) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    const char ch = buf[i];
    if (!covered[i] && !blank(ch) && ch != '\n' && ch != '\0') atomicOr(bad, 2u);
  }
}

// off[r] = first entry of line r (entries are in line order)
__global__ void k_row_bounds(const i64* __restrict__ row, i64 ne, i64 nlines, i32* __restrict__ off) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i <= ne; i += (i64)gridDim.x * blockDim.x) {
    const i64 prev = (i == 0) ? -1 : row[i - 1];
    const i64 cur = (i == ne) ? nlines : row[i];
    for (i64 r = prev + 1; r <= cur; r++) off[r] = (i32)i;
  }
}

// min / max column id, then the int32 ids (shifted by `shift`)
__global__ void k_col_range(const int64_t* __restrict__ col, i64 ne, long long* mn, long long* mx) {
  long long a = (1ll << 62), b = -(1ll << 62);
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += (i64)gridDim.x * blockDim.x) {
    a = min(a, (long long)col[i]);
    b = max(b, (long long)col[i]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {  // one atomic per warp
    a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mn, a);
    atomicMax(mx, b);
  }
}
__global__ void k_col_narrow(const int64_t* __restrict__ col, i64 ne, long long shift, i32* __restrict__ out) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += (i64)gridDim.x * blockDim.x)
    out[i] = (i32)(col[i] - shift);
}

// values converted on the host: entry e (>= 0) or the label of line -1 - who
__global__ void k_scatter_slow(const i64* __restrict__ who, const double* __restrict__ v, i64 k, void* val,
                               int as_float, double* __restrict__ label) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (i64)gridDim.x * blockDim.x) {
    const i64 w = who[i];
    if (w >= 0) {
      if (as_float) ((float*)val)[w] = (float)v[i];
      else ((double*)val)[w] = v[i];
    } else {
      label[-1 - w] = v[i];
    }
  }
}

static unsigned grid_for(fvg_ctx* c, i64 n) {
  return (unsigned)std::max<i64>(1, std::min<i64>((n + kLT - 1) / kLT, 16 * (i64)c->num_sms));
}

static std::vector<char> read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail(FVG_ERR_INVALID_ARG, "cannot open " + path + ": " + std::strerror(errno));
  f.seekg(0, std::ios::end);
  const std::streamoff sz = f.tellg();
  f.seekg(0, std::ios::beg);
  std::vector<char> buf((size_t)std::max<std::streamoff>(sz, 0) + 1, '\0');
  if (sz > 0 && !f.read(buf.data(), sz)) fail(FVG_ERR_INVALID_ARG, "cannot read " + path);
  buf.resize((size_t)sz);
  return buf;
}

struct Parsed {
  i64 m = 0, n = 0, nnz = 0;
  DBuf off, idx, val;  // int32, int32, value dtype
  std::vector<double> label;
};

// Parses a text CRS / libsvm file (the host copy stays for the fallback
// conversions).
static void parse_text(fvg_ctx* c, const std::string& path, int dt, bool libsvm, int origin, i64 num_col,
                       Parsed& P) {
  cudaStream_t s = c->stream;
  std::vector<char> host = read_file(path);
  const i64 nbytes = (i64)host.size();
  DBuf buf;
  buf.alloc((size_t)nbytes + 16, s);
  FVG_CUDA(cudaMemsetAsync(buf.p, 0, (size_t)nbytes + 16, s));
  if (nbytes) FVG_CUDA(cudaMemcpyAsync(buf.p, host.data(), (size_t)nbytes, cudaMemcpyHostToDevice, s));
  const char* b = buf.as<char>();
  // newline and colon positions
  const i64 nblk = std::max<i64>(1, (nbytes + kBlockBytes - 1) / kBlockBytes);
  DBuf nlc, coc, nlb, cob;
  nlc.alloc(sizeof(i64) * nblk, s);
  coc.alloc(sizeof(i64) * nblk, s);
  nlb.alloc(sizeof(i64) * (nblk + 1), s);
  cob.alloc(sizeof(i64) * (nblk + 1), s);
  k_count_marks<<<(unsigned)nblk, kLT, 0, s>>>(b, nbytes, nlc.as<i64>(), coc.as<i64>());
  check_launch("k_count_marks");
  count_launch(c);
  scan_i64(c, nlc.as<i64>(), nlb.as<i64>(), nblk);
  scan_i64(c, coc.as<i64>(), cob.as<i64>(), nblk);
  i64 tot[2] = {0, 0};
  FVG_CUDA(cudaMemcpyAsync(&tot[0], nlb.as<i64>() + nblk, sizeof(i64), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaMemcpyAsync(&tot[1], cob.as<i64>() + nblk, sizeof(i64), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  const i64 nnl = tot[0], ne = tot[1];
  if (ne >= (1ll << 31)) fail(FVG_ERR_INVALID_ARG, "more than 2^31 - 1 nonzeros");
  const i64 nlines = nnl + ((nbytes > 0 && host[nbytes - 1] != '\n') ? 1 : 0);  // std::getline rows
  if (nlines >= (1ll << 31)) fail(FVG_ERR_INVALID_ARG, "more than 2^31 - 1 rows");
  DBuf nl_pos, co_pos;
  nl_pos.alloc(sizeof(i64) * std::max<i64>(nnl, 1), s);
  co_pos.alloc(sizeof(i64) * std::max<i64>(ne, 1), s);
  k_write_marks<<<(unsigned)nblk, kLT, 0, s>>>(b, nbytes, nlb.as<i64>(), cob.as<i64>(), nl_pos.as<i64>(),
                                               co_pos.as<i64>());
  check_launch("k_write_marks");
  count_launch(c);
  // entries
  const int es = dt == FVG_F32 ? 4 : 8;
  DBuf row, col, val, covered, flags, slow, lab;
  row.alloc(sizeof(i64) * std::max<i64>(ne, 1), s);
  col.alloc(sizeof(int64_t) * std::max<i64>(ne, 1), s);
  val.alloc((size_t)es * std::max<i64>(ne, 1), s);
  covered.alloc((size_t)std::max<i64>(nbytes, 1), s);
  FVG_CUDA(cudaMemsetAsync(covered.p, 0, (size_t)std::max<i64>(nbytes, 1), s));
  flags.alloc(256, s);
  FVG_CUDA(cudaMemsetAsync(flags.p, 0, 256, s));
  const i64 slow_cap = std::max<i64>(ne + nlines, 1);
  slow.alloc(sizeof(i64) * 3 * slow_cap, s);
  lab.alloc(sizeof(double) * std::max<i64>(nlines, 1), s);
  EntryOut o;
  o.row = row.as<i64>();
  o.col = col.as<int64_t>();
  o.val = val.p;
  o.want_float = dt == FVG_F32;
  o.covered = covered.as<unsigned char>();
  o.bad = flags.as<unsigned>();
  o.nslow = flags.as<unsigned>() + 1;
  o.slow = slow.as<i64>();
  o.slow_cap = slow_cap;
  LineInfo L{nl_pos.as<i64>(), nnl, nbytes};
  if (ne) {
    k_parse_entries<<<grid_for(c, ne), kLT, 0, s>>>(b, L, co_pos.as<i64>(), ne, o);
    check_launch("k_parse_entries");
    count_launch(c);
  }
  if (libsvm && nlines) {
    k_parse_labels<<<grid_for(c, nlines), kLT, 0, s>>>(b, L, nlines, lab.as<double>(), o);
    check_launch("k_parse_labels");
    count_launch(c);
  }
  if (nbytes) {
    k_check_cover<<<grid_for(c, nbytes), kLT, 0, s>>>(b, nbytes, covered.as<unsigned char>(), o.bad);
    check_launch("k_check_cover");
    count_launch(c);
  }
  unsigned hf[2] = {0, 0};
  FVG_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  if (hf[0]) fail(FVG_ERR_INVALID_ARG, "malformed line in " + path + ": expected \"col:value\" tokens");
  // host conversion of the values outside the exact fast path, scattered
  // back on the device
  if (hf[1]) {
    std::vector<i64> hs(3 * (size_t)hf[1]);
    FVG_CUDA(cudaMemcpyAsync(hs.data(), slow.p, sizeof(i64) * hs.size(), cudaMemcpyDeviceToHost, s));
    FVG_CUDA(cudaStreamSynchronize(s));
    std::vector<i64> at;
    std::vector<double> vd;
    for (size_t k = 0; k < hf[1]; k++) {
      const i64 who = hs[3 * k], st = hs[3 * k + 1], en = hs[3 * k + 2];
      char* endp = nullptr;
      double v;
      if (who >= 0 && dt == FVG_F32) v = (double)std::strtof(host.data() + st, &endp);  // exact in double
      else v = std::strtod(host.data() + st, &endp);
      if (endp != host.data() + en) fail(FVG_ERR_INVALID_ARG, "malformed number in " + path);
      at.push_back(who);
      vd.push_back(v);
    }
    DBuf dat, dv;
    dat.alloc(sizeof(i64) * at.size(), s);
    dv.alloc(sizeof(double) * vd.size(), s);
    FVG_CUDA(cudaMemcpyAsync(dat.p, at.data(), sizeof(i64) * at.size(), cudaMemcpyHostToDevice, s));
    FVG_CUDA(cudaMemcpyAsync(dv.p, vd.data(), sizeof(double) * vd.size(), cudaMemcpyHostToDevice, s));
    k_scatter_slow<<<grid_for(c, (i64)at.size()), kLT, 0, s>>>(dat.as<i64>(), dv.as<double>(), (i64)at.size(),
                                                               val.p, dt == FVG_F32, lab.as<double>());
    check_launch("k_scatter_slow");
    count_launch(c);
    FVG_CUDA(cudaStreamSynchronize(s));
  }
  // column range, origin, int32 ids
  long long range[2] = {(1ll << 62), -(1ll << 62)};
  DBuf rg;
  rg.alloc(sizeof(range), s);
  FVG_CUDA(cudaMemcpyAsync(rg.p, range, sizeof(range), cudaMemcpyHostToDevice, s));
  if (ne) {
    k_col_range<<<grid_for(c, ne), kLT, 0, s>>>(col.as<int64_t>(), ne, rg.as<long long>(), rg.as<long long>() + 1);
    check_launch("k_col_range");
    count_launch(c);
  }
  FVG_CUDA(cudaMemcpyAsync(range, rg.p, sizeof(range), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  long long shift = 0;
  i64 ncol = num_col;
  if (ne) {
    if (ncol < 0) ncol = range[1] + 1;  // largest id + 1, before the origin shift
    if (libsvm && (origin == 2 || (origin == 0 && range[0] > 0))) shift = 1;
    if (range[0] - shift < 0) fail(FVG_ERR_INVALID_ARG, "negative column index in " + path);
    if (range[1] - shift >= ncol || ncol >= (1ll << 31))
      fail(FVG_ERR_INVALID_ARG, "column index out of range in " + path);
  } else if (ncol < 0) {
    ncol = 0;
  }
  P.m = nlines;
  P.n = ncol;
  P.nnz = ne;
  P.off.alloc(sizeof(i32) * (nlines + 1), s);
  P.idx.alloc(sizeof(i32) * std::max<i64>(ne, 1), s);
  if (nlines + 1 > 0) {
    k_row_bounds<<<grid_for(c, ne + 1), kLT, 0, s>>>(row.as<i64>(), ne, nlines, P.off.as<i32>());
    check_launch("k_row_bounds");
    count_launch(c);
  }
  if (ne) {
    k_col_narrow<<<grid_for(c, ne), kLT, 0, s>>>(col.as<int64_t>(), ne, shift, P.idx.as<i32>());
    check_launch("k_col_narrow");
    count_launch(c);
  }
  P.val = std::move(val);
  if (libsvm) {
    P.label.resize((size_t)nlines);
    if (nlines)
      FVG_CUDA(cudaMemcpyAsync(P.label.data(), lab.p, sizeof(double) * nlines, cudaMemcpyDeviceToHost, s));
  }
  FVG_CUDA(cudaStreamSynchronize(s));
}

// ------------------------------------------------------------------ binary
__global__ void k_narrow_any(const void* __restrict__ src, int bytes, int is_signed, i64 n, i32* __restrict__ out,
                             unsigned* bad) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    long long v;
    if (bytes == 8) v = ((const long long*)src)[i];
    else if (is_signed) v = ((const int*)src)[i];
    else v = (long long)((const unsigned*)src)[i];
    if (bytes == 8 && !is_signed && v < 0) v = -1;  // above 2^63
    if (v < 0 || v >= (1ll << 31)) atomicOr(bad, 1u);
    out[i] = (i32)v;
  }
}

static int type_bytes(const std::string& t, bool* is_signed) {
  *is_signed = t[0] == 'i';
  if (t == "int32_t" || t == "uint32_t") return 4;
  if (t == "int64_t" || t == "uint64_t") return 8;
  fail(FVG_ERR_INVALID_ARG, "unsupported index type " + t + " (int32_t, uint32_t, int64_t, uint64_t)");
}

static void load_binary(fvg_ctx* c, const std::string& dir, int dt, const std::string& idx_type,
                        const std::string& off_type, Parsed& P) {
  cudaStream_t s = c->stream;
  std::ifstream nums(dir + "/nums");
  i64 m = -1, n = -1;
  if (!(nums >> m >> n)) fail(FVG_ERR_INVALID_ARG, "cannot read " + dir + "/nums");
  const std::string vtype = dt == FVG_F32 ? "float" : "double";
  struct stat sb;
  if (stat((dir + "/type").c_str(), &sb) == 0) {
    std::ifstream ty(dir + "/type");
    std::string a, b2, c2;
    ty >> a >> b2 >> c2;
    const char* fn = "make_crs_matrix_local_loadbinary";
    auto check = [&](const std::string& expect, const std::string& given, const char* what) {
      if (expect != given)
        fail(FVG_ERR_INVALID_ARG, std::string(fn) + ": " + what + " type mismatch detected! expected type: " +
                                      expect + "; given type: " + given + "\n");
    };
    check(a, vtype, "val");
    check(b2, idx_type, "idx");
    check(c2, off_type, "off");
  }
  bool isg = false, osg = false;
  const int ib = type_bytes(idx_type, &isg), ob = type_bytes(off_type, &osg);
  const int vb = dt == FVG_F32 ? 4 : 8;
  std::vector<char> hv = read_file(dir + "/val"), hi = read_file(dir + "/idx"), ho = read_file(dir + "/off");
  if (hv.size() % vb || hi.size() % ib || ho.size() % ob)
    fail(FVG_ERR_INVALID_ARG, "make_dvector_loadbinary: incorrect filesize");
  const i64 nnz = (i64)(hv.size() / vb);
  if ((i64)(hi.size() / ib) != nnz || (i64)(ho.size() / ob) != m + 1)
    fail(FVG_ERR_INVALID_ARG, "binary CRS arrays do not match nums (" + std::to_string(m) + " rows)");
  if (nnz >= (1ll << 31) || m >= (1ll << 31) || n >= (1ll << 31))
    fail(FVG_ERR_INVALID_ARG, "matrix too large for int32 indices");
  DBuf rawi, rawo, flags;
  rawi.alloc(std::max<size_t>(hi.size(), 8), s);
  rawo.alloc(std::max<size_t>(ho.size(), 8), s);
  flags.alloc(256, s);
  FVG_CUDA(cudaMemsetAsync(flags.p, 0, 256, s));
  if (!hi.empty()) FVG_CUDA(cudaMemcpyAsync(rawi.p, hi.data(), hi.size(), cudaMemcpyHostToDevice, s));
  FVG_CUDA(cudaMemcpyAsync(rawo.p, ho.data(), ho.size(), cudaMemcpyHostToDevice, s));
  P.m = m;
  P.n = n;
  P.nnz = nnz;
  P.off.alloc(sizeof(i32) * (m + 1), s);
  P.idx.alloc(sizeof(i32) * std::max<i64>(nnz, 1), s);
  P.val.alloc((size_t)vb * std::max<i64>(nnz, 1), s);
  if (nnz) {
    FVG_CUDA(cudaMemcpyAsync(P.val.p, hv.data(), hv.size(), cudaMemcpyHostToDevice, s));
    k_narrow_any<<<grid_for(c, nnz), kLT, 0, s>>>(rawi.p, ib, isg, nnz, P.idx.as<i32>(), flags.as<unsigned>());
    check_launch("k_narrow_any");
    count_launch(c);
  }
  k_narrow_any<<<grid_for(c, m + 1), kLT, 0, s>>>(rawo.p, ob, osg, m + 1, P.off.as<i32>(), flags.as<unsigned>());
  check_launch("k_narrow_any");
  count_launch(c);
  unsigned hb = 0;
  FVG_CUDA(cudaMemcpyAsync(&hb, flags.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  FVG_CUDA(cudaStreamSynchronize(s));
  if (hb) fail(FVG_ERR_INVALID_ARG, "index or offset outside [0, 2^31)");
}

void matrix_from_parsed(fvg_ctx* c, Parsed& P, int dt, DevCRS& A) {
  crs_upload(c, A, P.m, P.n, P.off.as<i32>(), P.idx.as<i32>(), P.val.p, dt, true);
}

void load_text_matrix(fvg_ctx* c, const char* path, int dt, i64 num_col, DevCRS& A) {
  Parsed P;
  parse_text(c, path, dt, false, 0, num_col, P);
  matrix_from_parsed(c, P, dt, A);
}

void load_libsvm_matrix(fvg_ctx* c, const char* path, int dt, int origin, DevCRS& A, std::vector<double>& label) {
  Parsed P;
  parse_text(c, path, dt, true, origin, -1, P);
  matrix_from_parsed(c, P, dt, A);
  label.swap(P.label);
}

void load_binary_matrix(fvg_ctx* c, const char* dir, int dt, const char* idx_type, const char* off_type,
                        DevCRS& A) {
  Parsed P;
  load_binary(c, dir, dt, idx_type, off_type, P);
  matrix_from_parsed(c, P, dt, A);
}

}  // namespace fvg
